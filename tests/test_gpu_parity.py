"""GPU parity: the sm_103a kernels against the float64 oracle on the same inputs.

Tolerance: the plain-FP32 path must match the float64 oracle within a
relative error of 1e-5 on readout kernels ([N1, N2] outputs) and within
1e-5 of the largest entry on full spatial kernels.
"""
import math

import numpy as np
import pytest
import torch

from oracle import nt_oracle as o

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def elem_rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-30)))


def cpu(t):
    return t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)


def both(nt, layers_fn, x1, x2, get=('nngp', 'ntk', 'cov1', 'cov2'), **kw):
    s = nt.stax
    _, _, kf = s.serial(*layers_fn(s))
    ko = o.serial(*layers_fn(o))
    got = kf(x1, x2, get, **kw)
    want = ko(x1, x2, get)
    return [cpu(g) for g in got], list(want)


def fcn_layers(m):
    return [m.Dense(512, W_std=1.5, b_std=0.05), m.Relu(), m.Dense(512, W_std=1.5, b_std=0.05),
            m.Relu(), m.Dense(1, W_std=1.5, b_std=0.05)]


def normalized_rows(rng, n, d):
    x = rng.standard_normal((n, d)).astype(np.float32)
    return (x / np.linalg.norm(x, axis=1, keepdims=True) * math.sqrt(d)).astype(np.float32)


def test_fcn_config(nt):
    rng0, rng1 = np.random.default_rng(0), np.random.default_rng(1)
    x1, x2 = normalized_rows(rng0, 64, 784), normalized_rows(rng1, 48, 784)
    got, want = both(nt, fcn_layers, x1, x2)
    for g, w in zip(got, want):
        assert elem_rel_err(g, w) < RTOL


def test_fcn_erf_and_abrelu(nt):
    rng = np.random.default_rng(2)
    x1, x2 = rng.standard_normal((16, 20)), rng.standard_normal((12, 20))
    lay = lambda m: [m.Dense(3, 1.3, 0.2), m.Erf(0.7, 1.2, 0.1), m.Dense(3, 0.9, 0.3),
                     m.ABRelu(-0.3, 1.1), m.Dense(1, 1.1)]
    got, want = both(nt, lay, x1, x2)
    for g, w in zip(got, want):
        assert elem_rel_err(g, w) < RTOL
    got, want = both(nt, lay, x1, None, get=('nngp', 'ntk', 'cov1'))
    for g, w in zip(got, want):
        assert elem_rel_err(g, w) < RTOL



@pytest.mark.parametrize('same_inputs', [True, False])
@pytest.mark.parametrize('do_stabilize', [True, False])
def test_abrelu_family_identities(nt, same_inputs, do_stabilize):
    """tests/stax/elementwise_test.py:541-636 on the CUDA path: ABRelu(0, 1), (0, -1),
    (-1, 0) and (1, 0) all give ReLU's kernels; ABRelu(a, a) is a times the identity;
    LeakyRelu(a) is ABRelu(a, 1) and Abs is ABRelu(-1, 1); every kernel also against the
    float64 oracle."""
    rng = np.random.default_rng(1)
    x1 = rng.standard_normal((3, 2))
    x2 = None if same_inputs else rng.standard_normal((4, 2))
    fc = lambda m: m.Dense(5, 1., 0.)

    def k(layers_fn, a=x1, b=x2, get=('nngp', 'ntk')):
        got, want = both(nt, layers_fn, a, b, get)
        for g, w in zip(got, want):
            assert rel_err(g, w) < RTOL
        return got

    relu = k(lambda m: [fc(m), m.Relu(do_stabilize)])
    for a, b in [(0, 1), (0, -1), (-1, 0), (1, 0)]:
        got = k(lambda m: [fc(m), m.ABRelu(a, b, do_stabilize)])
        for g, w in zip(got, relu):
            assert rel_err(g, w) < RTOL, (a, b)
    for a in [-5, -1, -0.5, 0.5, 1, 5]:
        kid = k(lambda m: [fc(m), m.Identity()], x1 * a, None if x2 is None else x2 * a,
                ('nngp', 'ntk', 'cov1'))
        kab = k(lambda m: [fc(m), m.ABRelu(a, a, do_stabilize)], get=('nngp', 'ntk', 'cov1'))
        for g, w in zip(kab, kid):
            assert rel_err(g, w) < RTOL, a
    for a in [-2, -1, 0, 1, 2]:
        kl = k(lambda m: [fc(m), m.LeakyRelu(a, do_stabilize)])
        ka = k(lambda m: [fc(m), m.ABRelu(a, 1, do_stabilize)])
        for g, w in zip(kl, ka):
            assert np.array_equal(g, w), a
    kabs = k(lambda m: [fc(m), m.Abs(do_stabilize)])
    kab = k(lambda m: [fc(m), m.ABRelu(-1, 1, do_stabilize)])
    for g, w in zip(kabs, kab):
        assert np.array_equal(g, w)


@pytest.mark.parametrize('avg_pool', [True, False])
@pytest.mark.parametrize('same_inputs', [True, False])
def test_serial_composition_through_a_kernel(nt, avg_pool, same_inputs):
    """tests/stax/stax_test.py:636-687 on the CUDA path: serial(block, readout) equals the
    readout's kernel_fn applied to the Kernel the block's kernel_fn returns (full spatial),
    and the composed kernels match the float64 oracle."""
    s = nt.stax
    rng = np.random.default_rng(11)
    x1 = rng.standard_normal((3, 5, 5, 3))
    x2 = None if same_inputs else rng.standard_normal((4, 5, 5, 3))
    block = lambda m: [m.Conv(1, (3, 3)), m.Relu()]
    readout = lambda m: ([m.Conv(1, (3, 3)), m.GlobalAvgPool(), m.Dense(1)] if avg_pool
                         else [m.Flatten(), m.Dense(1)])
    composed = s.serial(*block(s), *readout(s))[2](x1, x2, ('nngp', 'ntk'))
    bk = s.serial(*block(s))[2](x1, x2, diagonal_spatial=False)
    via = s.serial(*readout(s))[2](bk, None, ('nngp', 'ntk'))
    want = o.serial(*block(o), *readout(o))(x1, x2, ('nngp', 'ntk'))
    for g, c, w in zip(via, composed, want):
        assert rel_err(cpu(g), cpu(c)) < 1e-6
        assert elem_rel_err(cpu(c), w) < RTOL


@pytest.mark.parametrize('act', ['relu', 'relu_stab', 'erf'])
def test_zero_inputs_give_finite_kernels(nt, act):
    """tests/stax/stax_test.py:587-634 (sparse inputs): rows of zeros have zero variance
    at every layer; the activation rules must return finite kernels (no 0/0) equal to the
    float64 oracle's."""
    rng = np.random.default_rng(1)
    x = rng.standard_normal((4, 3))
    x[:2] = 0.
    for get in ('nngp', 'ntk'):
        lay = lambda m: [m.Dense(1024), m.Relu(act == 'relu_stab') if act != 'erf' else m.Erf(),
                         m.Dense(1 if get == 'ntk' else 1024)]
        got = cpu(nt.stax.serial(*lay(nt.stax))[2](x, None, get))
        want = o.serial(*lay(o))(x, None, get)
        assert np.all(np.isfinite(got)), get
        assert rel_err(got, want) < RTOL, get


@pytest.mark.parametrize('normalize_edges', [False, True])
def test_avg_pool_all_ones_kat(nt, normalize_edges):
    """tests/stax/stax_test.py:494-551 on the CUDA path: AvgPool((2, 2), (1, 1), 'SAME') of
    all-ones inputs. With normalize_edges every kernel entry is 1; without, the window
    averages are out_unnorm = [[1, 1, 0.5], [0.5, 0.5, 0.25]] and the kernels their outer
    products in the zipped layout."""
    X1, X2 = np.ones((4, 2, 3, 2)), np.ones((3, 2, 3, 2))
    k = nt.stax.AvgPool((2, 2), (1, 1), 'SAME', normalize_edges=normalize_edges)[2](X1, X2)
    nngp, cov1, cov2 = cpu(k.nngp), cpu(k.cov1), cpu(k.cov2)
    if normalize_edges:
        want = np.ones((2, 2, 3, 3))
    else:
        out_unnorm = np.array([[1., 1., 0.5], [0.5, 0.5, 0.25]])
        want = np.transpose(np.outer(out_unnorm, out_unnorm).reshape(2, 3, 2, 3), (0, 2, 1, 3))
    assert nngp.shape == (4, 3, 2, 2, 3, 3) and cov1.shape == (4, 2, 2, 3, 3)
    np.testing.assert_allclose(nngp, np.broadcast_to(want, nngp.shape), rtol=1e-6)
    np.testing.assert_allclose(cov1, np.broadcast_to(want, cov1.shape), rtol=1e-6)
    np.testing.assert_allclose(cov2, np.broadcast_to(want, cov2.shape), rtol=1e-6)


@pytest.mark.parametrize('same_inputs', [True, False])
def test_flatten_at_the_bottom_equals_dense_on_flattened_inputs(nt, same_inputs):
    """tests/stax/linear_test.py:53-100 on the CUDA path: serial(Flatten, Dense, Erf, Dense)
    on images equals serial(Dense, Erf, Dense) on the flattened images, and the float64
    oracle's kernels (relative to the largest entry: the Erf kernel changes sign, and
    entries near zero carry no relative accuracy)."""
    rng = np.random.default_rng(13)
    x1 = rng.standard_normal((4, 4, 3, 2))
    x2 = None if same_inputs else rng.standard_normal((2, 4, 3, 2))
    flat = lambda x: None if x is None else x.reshape(x.shape[0], -1)
    top = lambda m: [m.Dense(512, 1.7, 0.1), m.Erf(), m.Dense(512, 1.7, 0.1)]
    k = nt.stax.serial(*top(nt.stax))[2](flat(x1), flat(x2), ('nngp', 'ntk'))
    got, want = both(nt, lambda m: [m.Flatten()] + top(m), x1, x2, ('nngp', 'ntk'))
    for g, a, w in zip(got, k, want):
        assert rel_err(g, cpu(a)) < 1e-6
        assert rel_err(g, w) < RTOL

CONV_CASES = [
    dict(filter_shape=(3, 3), padding='SAME'),
    dict(filter_shape=(3, 3), padding='VALID'),
    dict(filter_shape=(2, 3), strides=(2, 1), padding='SAME'),
    dict(filter_shape=(3, 2), padding='CIRCULAR'),
]


@pytest.mark.parametrize('case', CONV_CASES)
def test_conv_relu_full_spatial(nt, case):
    rng = np.random.default_rng(3)
    x1, x2 = rng.standard_normal((2, 8, 8, 3)), rng.standard_normal((3, 8, 8, 3))
    lay = lambda m: [m.Conv(4, W_std=1.4, b_std=0.1, **case), m.Relu(),
                     m.Conv(4, W_std=1.2, b_std=0.05, **case)]
    got, want = both(nt, lay, x1, x2)
    for g, w in zip(got, want):
        assert g.shape == w.shape
        assert rel_err(g, w) < RTOL


def test_conv_nonsquare_reversal_layout(nt):
    rng = np.random.default_rng(4)
    x1, x2 = rng.standard_normal((2, 6, 4, 2)), rng.standard_normal((2, 6, 4, 2))
    lay = lambda m: [m.Conv(2, (3, 3), padding='SAME', W_std=1.1), m.Relu()]
    s = nt.stax
    k = s.serial(*lay(s))[2](x1, x2)
    ko = o.serial(*lay(o))(x1, x2)
    assert k.is_reversed == ko.is_reversed is True
    assert tuple(k.nngp.shape) == ko.nngp.shape == (2, 2, 4, 4, 6, 6)
    assert rel_err(cpu(k.nngp), ko.nngp) < RTOL


@pytest.mark.parametrize('pool', ['avg_same_norm', 'avg_same', 'sum_valid', 'avg_valid'])
def test_pools(nt, pool):
    rng = np.random.default_rng(5)
    x1, x2 = rng.standard_normal((2, 7, 6, 2)), rng.standard_normal((2, 7, 6, 2))
    mk = {
        'avg_same_norm': lambda m: m.AvgPool((2, 3), (1, 2), 'SAME', normalize_edges=True),
        'avg_same': lambda m: m.AvgPool((2, 2), (2, 2), 'SAME'),
        'sum_valid': lambda m: m.SumPool((2, 2), (1, 1), 'VALID'),
        'avg_valid': lambda m: m.AvgPool((3, 2), (2, 2), 'VALID'),
    }[pool]
    lay = lambda m: [m.Conv(2, (3, 3), padding='SAME', W_std=1.2, b_std=0.1), m.Relu(), mk(m),
                     m.Conv(2, (3, 3), padding='SAME', W_std=1.1)]
    got, want = both(nt, lay, x1, x2)
    for g, w in zip(got, want):
        assert rel_err(g, w) < RTOL


@pytest.mark.parametrize('readout', ['flatten', 'gap', 'gsp'])
def test_readouts(nt, readout):
    rng = np.random.default_rng(6)
    x1, x2 = rng.standard_normal((3, 6, 6, 3)), rng.standard_normal((2, 6, 6, 3))
    ro = {'flatten': lambda m: m.Flatten(), 'gap': lambda m: m.GlobalAvgPool(),
          'gsp': lambda m: m.GlobalSumPool()}[readout]
    lay = lambda m: [m.Conv(2, (3, 3), padding='SAME', W_std=1.3, b_std=0.2), m.Relu(), ro(m),
                     m.Dense(1, 1.1, 0.1)]
    got, want = both(nt, lay, x1, x2)
    for g, w in zip(got, want):
        assert elem_rel_err(g, w) < RTOL


def test_diagonal_spatial_network(nt):
    rng = np.random.default_rng(7)
    x1, x2 = rng.standard_normal((3, 6, 5, 2)), rng.standard_normal((2, 6, 5, 2))
    lay = lambda m: [m.Conv(2, (3, 3), padding='SAME', W_std=1.3, b_std=0.2), m.Erf(),
                     m.Conv(2, (3, 3), padding='SAME', W_std=1.1), m.Relu(), m.Flatten(),
                     m.Dense(1, 1.2)]
    s = nt.stax
    assert bool(s.serial(*lay(s))[2].diagonal)
    got, want = both(nt, lay, x1, x2)
    for g, w in zip(got, want):
        assert elem_rel_err(g, w) < RTOL


def test_one_spatial_dim(nt):
    rng = np.random.default_rng(8)
    x1, x2 = rng.standard_normal((2, 9, 3)), rng.standard_normal((3, 9, 3))
    lay = lambda m: [m.Conv(2, (3,), padding='SAME', W_std=1.3, b_std=0.2), m.Relu(),
                     m.AvgPool((2,), (2,)), m.Conv(2, (2,), padding='VALID', W_std=1.1)]
    got, want = both(nt, lay, x1, x2)
    for g, w in zip(got, want):
        assert rel_err(g, w) < RTOL


def myrtle(m, depth, readout='flatten'):
    f = {5: [2, 1, 1], 7: [2, 2, 2], 10: [3, 3, 3]}[depth]
    conv = lambda: m.Conv(1, (3, 3), padding='SAME', W_std=math.sqrt(2.), b_std=0.)
    L = []
    for _ in range(f[0]):
        L += [conv(), m.Relu()]
    L += [m.AvgPool((2, 2), (2, 2))]
    for _ in range(f[1]):
        L += [conv(), m.Relu()]
    L += [m.AvgPool((2, 2), (2, 2))]
    for _ in range(f[2]):
        L += [conv(), m.Relu()]
    if readout == 'flatten':
        L += [m.AvgPool((2, 2), (2, 2))] * 3 + [m.Flatten(), m.Dense(10, math.sqrt(2.), 0.)]
    else:
        L += [m.GlobalAvgPool(), m.Dense(10, math.sqrt(2.), 0.)]
    return L


@pytest.fixture(scope='module')
def cifar_like():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((5, 32, 32, 3)).astype(np.float32)
    x = (x - x.mean(axis=(0, 1, 2))) / x.std(axis=(0, 1, 2))
    return x[:3], x[3:]


def test_myrtle5_fused_chain_vs_oracle(nt, cifar_like):
    x1, x2 = cifar_like
    got, want = both(nt, lambda m: myrtle(m, 5), x1, x2)
    for g, w in zip(got, want):
        assert elem_rel_err(g, w) < RTOL


def test_myrtle5_symmetric_call(nt, cifar_like):
    x1, _ = cifar_like
    got, want = both(nt, lambda m: myrtle(m, 5), x1, None, get=('nngp', 'ntk', 'cov1'))
    for g, w in zip(got, want):
        assert elem_rel_err(g, w) < RTOL
    np.testing.assert_allclose(np.diag(got[0]), got[2], rtol=2e-6)


def test_fused_chain_matches_layer_by_layer(nt, cifar_like):
    """The fused kernel and the materialised per-layer kernels agree."""
    from nt_gb300 import _chain
    x1, x2 = cifar_like
    s = nt.stax
    _, _, kf = s.serial(*myrtle(s, 10, 'gap'))
    fused = kf(x1, x2, ('nngp', 'ntk'))
    assert _chain.plan_chain(kf.specs, x1.shape, False) is not None
    from nt_gb300.stax import _Ctx, _input_kernel, _as_input
    ctx = _Ctx('fp32')
    k = _input_kernel(_as_input(x1), _as_input(x2), False, True, False, ctx)
    k = kf.apply_kernel(k, ctx)
    assert rel_err(cpu(fused.nngp), cpu(k.nngp)) < 2e-6
    assert rel_err(cpu(fused.ntk), cpu(k.ntk)) < 2e-6


def test_batch_ragged_equals_unbatched(nt, cifar_like):
    x1, x2 = cifar_like
    xa = np.concatenate([x1, x2])
    s = nt.stax
    _, _, kf = s.serial(s.Conv(1, (3, 3), padding='SAME', W_std=1.5), s.Relu(), s.Flatten(),
                        s.Dense(1, 1.2, 0.1))
    full = kf(xa, xa[:4], ('nngp', 'ntk'))
    bt = nt.batch(kf, batch_size=2)(xa, xa[:4], ('nngp', 'ntk'))
    np.testing.assert_allclose(cpu(bt.nngp), cpu(full.nngp), rtol=1e-6)
    np.testing.assert_allclose(cpu(bt.ntk), cpu(full.ntk), rtol=1e-6)
    _, _, km = s.serial(*myrtle(s, 5))
    a = km(xa, None, 'ntk')
    b = nt.batch(km, batch_size=2)(xa, None, 'ntk')
    np.testing.assert_allclose(cpu(b), cpu(a), rtol=1e-6)


def test_activation_needs_gaussian_input(nt):
    s = nt.stax
    _, _, kf = s.serial(s.Relu())
    with pytest.raises(ValueError, match='Gaussian'):
        kf(np.ones((2, 3)), None)


@pytest.mark.parametrize('depth,readout', [(10, 'gap'), (7, 'flatten')])
def test_myrtle_deeper_fused_chain_vs_oracle(nt, cifar_like, depth, readout):
    """Myrtle-10 ([3, 3, 3] + GlobalAvgPool) and Myrtle-7 on the fused kernel against the
    float64 oracle: plain FP32 within 1e-5, the mixed form within 1e-4."""
    x1, x2 = cifar_like
    s = nt.stax
    _, _, kf = s.serial(*myrtle(s, depth, readout))
    want = o.serial(*myrtle(o, depth, readout))(x1[:2], x2, ('nngp', 'ntk'))
    plain = kf(x1[:2], x2, ('nngp', 'ntk'))
    mixed = kf(x1[:2], x2, ('nngp', 'ntk'), precision='mixed')
    for g, w in zip(plain, want):
        assert elem_rel_err(cpu(g), w) < RTOL
    for g, w in zip(mixed, want):
        assert elem_rel_err(cpu(g), w) < 1e-4


def test_myrtle5_mixed_vs_oracle(nt, cifar_like):
    x1, x2 = cifar_like
    got, want = both(nt, lambda m: myrtle(m, 5), x1, x2, get=('nngp', 'ntk'), precision='mixed')
    for g, w in zip(got, want):
        assert elem_rel_err(g, w) < 1e-4


def test_symmetric_grid_is_mirrored_triangle(nt):
    """kernel_fn(x, None) on the fused path evaluates the pairs i <= j once and mirrors
    them: the result is exactly symmetric and matches kernel_fn(x, x) (every pair
    evaluated) to float32 rounding."""
    rng = np.random.default_rng(5)
    x = rng.standard_normal((7, 32, 32, 3)).astype(np.float32)
    s = nt.stax
    _, _, kf = s.serial(*myrtle(s, 5))
    sym = kf(x, None, ('nngp', 'ntk'))
    full = kf(x, x.copy(), ('nngp', 'ntk'))
    for a, b in zip(sym, full):
        a, b = cpu(a), cpu(b)
        assert np.array_equal(a, a.T)
        assert rel_err(a, b) < 2e-6


@pytest.mark.parametrize('with_x2', [True, False])
def test_captured_batch_replays_eager_results(nt, with_x2):
    """CapturedBatch: one CUDA-graph capture of the fused batch, replayed on new inputs,
    gives the eager nt.batch results bit for bit."""
    rng = np.random.default_rng(12)
    s = nt.stax
    _, _, kf = s.serial(*myrtle(s, 5))
    shape1, shape2 = (6, 32, 32, 3), (5, 32, 32, 3)
    cap = nt.CapturedBatch(kf, shape1, shape2 if with_x2 else None, ('nngp', 'ntk'),
                           batch_size=4)
    for seed in range(2):
        x1 = torch.tensor(rng.standard_normal(shape1), dtype=torch.float32, device='cuda')
        x2 = torch.tensor(rng.standard_normal(shape2), dtype=torch.float32, device='cuda')
        got = cap(x1, x2 if with_x2 else None)
        want = nt.batch(kf, batch_size=4)(x1, x2 if with_x2 else None, ('nngp', 'ntk'))
        for g, w in zip(got, want):
            assert torch.equal(g, w)


def test_edge_batches(nt):
    """Empty batches return empty kernels of the right shape; one-sample batches, x2=None with
    one sample, batch_size larger than N and batch_size = 1 agree with the oracle."""
    rng = np.random.default_rng(8)
    s = nt.stax
    _, _, kf = s.serial(*myrtle(s, 5))
    x = rng.standard_normal((3, 32, 32, 3)).astype(np.float32)
    ko = o.serial(*myrtle(o, 5))
    e = kf(x[:0], x, ('nngp', 'ntk'))
    assert tuple(e.nngp.shape) == (0, 3) and tuple(e.ntk.shape) == (0, 3)
    e = kf(x, x[:0], 'nngp')
    assert tuple(e.shape) == (3, 0)
    e = kf(x[:0], None, 'ntk')
    assert tuple(e.shape) == (0, 0)
    want = ko(x[:1], x[1:], ('nngp', 'ntk'))
    got = kf(x[:1], x[1:], ('nngp', 'ntk'))
    for g, w in zip(got, want):
        assert elem_rel_err(cpu(g), w) < RTOL
    one = kf(x[:1], None, 'ntk')
    assert elem_rel_err(cpu(one), ko(x[:1], None, 'ntk')) < RTOL
    for bs in (1, 10):
        b = nt.batch(kf, batch_size=bs)(x, None, 'ntk')
        assert elem_rel_err(cpu(b), ko(x, None, 'ntk')) < RTOL


@pytest.mark.parametrize('act', ['gelu', 'sin', 'cos', 'rbf'])
def test_more_dual_activations_vs_oracle(nt, act, cifar_like):
    """Gelu, Sin, Cos and Rbf (elementwise.py:195-400) as epilogues of the Dense rule (flat
    inputs), of the materialised conv rule (6x6 images) and of the fused whole-network kernel
    (32x32 images; checked against the oracle and against the per-layer kernels)."""
    def mk(m):
        return {'gelu': m.Gelu(), 'sin': m.Sin(1.2, 0.8, 0.3), 'cos': m.Cos(0.9, 1.1, -0.2),
                'rbf': m.Rbf(0.4)}[act]

    rng = np.random.default_rng(33)
    xf1, xf2 = rng.standard_normal((6, 20)), rng.standard_normal((5, 20))
    got, want = both(nt, lambda m: [m.Dense(8, 1.3, 0.1), mk(m), m.Dense(1, 1.1, 0.05)],
                     xf1, xf2)
    for g, w in zip(got, want):
        assert elem_rel_err(g, w) < RTOL
    xc1, xc2 = rng.standard_normal((2, 6, 6, 2)), rng.standard_normal((3, 6, 6, 2))
    got, want = both(nt, lambda m: [m.Conv(2, (3, 3), padding='SAME', W_std=1.2, b_std=0.1),
                                    mk(m), m.GlobalAvgPool(), m.Dense(1, 1.1, 0.)], xc1, xc2)
    for g, w in zip(got, want):
        assert rel_err(g, w) < RTOL
    x1, x2 = cifar_like
    lay = lambda m: [m.Conv(1, (3, 3), padding='SAME', W_std=1.3), mk(m),
                     m.AvgPool((2, 2), (2, 2)), m.Conv(1, (3, 3), padding='SAME', W_std=1.2),
                     mk(m), m.GlobalAvgPool(), m.Dense(1, 1.0, 0.)]
    from nt_gb300 import _chain
    from nt_gb300.stax import _Ctx, _input_kernel, _as_input
    kf = nt.stax.serial(*lay(nt.stax))[2]
    assert _chain.plan_chain(kf.specs, x1.shape, False) is not None
    got, want = both(nt, lay, x1[:2], x2, get=('nngp', 'ntk'))
    for g, w in zip(got, want):
        assert elem_rel_err(g, w) < RTOL
    ctx = _Ctx('fp32')
    k = _input_kernel(_as_input(x1[:2]), _as_input(x2), False, True, False, ctx)
    k = kf.apply_kernel(k, ctx)
    assert rel_err(got[0], cpu(k.nngp)) < 2e-6
    assert rel_err(got[1], cpu(k.ntk)) < 2e-6


def test_argument_swap_symmetry(nt, cifar_like):
    """elementwise_test.py:639-732 (argument-swap symmetry): K(x2, x1) is K(x1, x2) transposed,
    on the fused whole-network kernel and on the layer-by-layer kernels (an Erf network)."""
    x1, x2 = cifar_like
    s = nt.stax
    kf = s.serial(*myrtle(s, 5))[2]
    a = kf(x1, x2, ('nngp', 'ntk'))
    b = kf(x2, x1, ('nngp', 'ntk'))
    for u, v in zip(a, b):
        np.testing.assert_allclose(cpu(u), cpu(v).T, rtol=2e-6)
    ke = s.serial(s.Conv(2, (3, 3), padding='SAME', W_std=1.3, b_std=0.1), s.Erf(),
                  s.Conv(2, (2, 2), padding='VALID', W_std=1.2), s.Relu(), s.GlobalAvgPool(),
                  s.Dense(1, 1.1, 0.))[2]
    rng = np.random.default_rng(9)
    y1, y2 = rng.standard_normal((3, 7, 6, 2)), rng.standard_normal((2, 7, 6, 2))
    a = ke(y1, y2, ('nngp', 'ntk'))
    b = ke(y2, y1, ('nngp', 'ntk'))
    for u, v in zip(a, b):
        np.testing.assert_allclose(cpu(u), cpu(v).T, rtol=2e-6)
