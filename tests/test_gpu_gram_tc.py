"""tcgen05 split-BF16 Gram against a float64 Gram (mixed-precision bound 1e-4)."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def cs_err(got, x1, x2):
    """max |got - x1 x2^T/D| / sqrt(q11 q22): error relative to the Cauchy-Schwarz scale."""
    d = x1.shape[1]
    exact = x1.astype(np.float64) @ x2.astype(np.float64).T / d
    q1 = np.sum(x1.astype(np.float64) ** 2, 1) / d
    q2 = np.sum(x2.astype(np.float64) ** 2, 1) / d
    return float(np.max(np.abs(got - exact) / np.sqrt(np.outer(q1, q2))))


@pytest.mark.parametrize('n1,n2,d', [(128, 128, 64), (256, 256, 784), (300, 130, 100),
                                     (1000, 700, 3072)])
def test_tc_gram_matches_float64(nt, n1, n2, d):
    from nt_gb300 import _ops as O
    rng = np.random.default_rng(n1 + d)
    x1 = rng.standard_normal((n1, d)).astype(np.float32)
    x2 = rng.standard_normal((n2, d)).astype(np.float32)
    got = O.gram(torch.from_numpy(x1).cuda(), torch.from_numpy(x2).cuda(), 1).cpu().numpy()
    assert cs_err(got, x1, x2) < 1e-5
    ref = O.gram(torch.from_numpy(x1).cuda(), torch.from_numpy(x2).cuda(), 0).cpu().numpy()
    assert cs_err(ref, x1, x2) < 1e-6


def test_fcn_mixed_precision_vs_oracle(nt):
    from oracle import nt_oracle as o
    rng = np.random.default_rng(0)
    x = rng.standard_normal((192, 784))
    x = x / np.linalg.norm(x, axis=1, keepdims=True) * math.sqrt(784)
    lay = lambda m: [m.Dense(512, W_std=1.5, b_std=0.05), m.Relu(),
                     m.Dense(512, W_std=1.5, b_std=0.05), m.Relu(), m.Dense(1, W_std=1.5, b_std=0.05)]
    got = nt.stax.serial(*lay(nt.stax))[2](x[:128], x[128:], ('nngp', 'ntk'), precision='mixed')
    want = o.serial(*lay(o))(x[:128], x[128:], ('nngp', 'ntk'))
    for g, w in zip(got, want):
        assert np.max(np.abs(g.cpu().numpy() - w) / np.abs(w)) < 1e-4


@pytest.mark.parametrize('n,d', [(128, 64), (300, 99), (1000, 3072), (129, 784)])
def test_tc_gram_symmetric_inputs(nt, n, d):
    """x1 is x2: the lower triangle of tiles, each off-diagonal tile mirrored. The result is
    exactly symmetric, within the mixed-precision bound of float64 and no less accurate than
    the general path on two copies of x (d = 99: rows not 16-byte aligned, the split's scalar
    path). On the diagonal every partial sum is positive, so the tensor cores' FP32
    accumulation error grows with d there (about 2e-5 at d = 3072) in both paths."""
    from nt_gb300 import _ops as O
    rng = np.random.default_rng(n + d)
    x = rng.standard_normal((n, d)).astype(np.float32)
    t = torch.from_numpy(x).cuda()
    got = O.gram(t, t, 1).cpu().numpy()
    assert np.array_equal(got, got.T)
    assert cs_err(got, x, x) < 1e-4
    other = O.gram(t, t.clone(), 1).cpu().numpy()
    assert cs_err(got, x, x) <= cs_err(other, x, x) + 1e-7


@pytest.mark.parametrize('n,d', [(128, 64), (300, 99), (1000, 3072), (130, 784)])
def test_fp32_gram_symmetric_inputs_bit_identical(nt, n, d):
    """The FP32 Gram (precision 0) for x1 is x2 computes the lower triangle of tiles and
    mirrors it: bit for bit the general path's result (every entry a fmaf chain in ascending
    d, fmaf commutative in its product), and within float32 accuracy of float64 (the
    diagonal's sums of squares carry the sequential sum's rounding, ~2.5e-6 at d = 3072)."""
    from nt_gb300 import _ops as O
    rng = np.random.default_rng(n * d)
    x = rng.standard_normal((n, d)).astype(np.float32)
    t = torch.from_numpy(x).cuda()
    got = O.gram(t, t, 0).cpu().numpy()
    assert np.array_equal(got, got.T)
    assert np.array_equal(got, O.gram(t, t.clone(), 0).cpu().numpy())
    assert cs_err(got, x, x) < 1e-5
