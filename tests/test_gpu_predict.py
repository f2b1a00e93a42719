"""GPU parity of predict.gradient_descent_mse (Cholesky + FP64 refinement)."""
import math

import numpy as np
import pytest
import scipy.linalg as sla
import torch

from oracle import nt_oracle as o

pytestmark = pytest.mark.gpu


def fcn(m):
    return [m.Dense(512, W_std=1.5, b_std=0.05), m.Relu(), m.Dense(512, W_std=1.5, b_std=0.05),
            m.Relu(), m.Dense(1, W_std=1.5, b_std=0.05)]


def rows(seed, n, d):
    x = np.random.default_rng(seed).standard_normal((n, d))
    return x / np.linalg.norm(x, axis=1, keepdims=True) * math.sqrt(d)


def onehot(seed, n, k=10):
    lab = np.random.default_rng(seed).integers(0, k, n)
    return np.eye(k)[lab]


def test_fcn_config_end_to_end(nt):
    """The CPU-runnable FCN configuration: 256 x 784 inputs, diag_reg=1e-4, t=None."""
    x1, x2, y = rows(0, 256, 784), rows(1, 256, 784), onehot(2, 256)
    kf = nt.stax.serial(*fcn(nt.stax))[2]
    ktt = kf(x1, None, 'ntk')
    kts = kf(x2, x1, 'ntk')
    pred = nt.predict.gradient_descent_mse(ktt, y, diag_reg=1e-4)
    fx_train, fx_test = pred(None, 0., 0., kts)
    ko = o.serial(*fcn(o))
    want = o.gradient_descent_mse(ko(x1, None, 'ntk'), y, diag_reg=1e-4)(None, 0., 0.,
                                                                            ko(x2, x1, 'ntk'))
    np.testing.assert_allclose(fx_train.cpu().numpy(), want[0], rtol=1e-6)
    got = fx_test.cpu().numpy()
    assert np.max(np.abs(got - want[1])) / np.max(np.abs(want[1])) < 1e-4
    # the refined solve on the same float32 kernel, followed by the float32
    # k_test_train product, matches a float64 solve to ~1e-5
    k64 = ktt.double().cpu().numpy()
    a = k64 + 1e-4 * np.trace(k64) / 256 * np.eye(256)
    exact = kts.double().cpu().numpy() @ sla.cho_solve(sla.cho_factor(a), y)
    assert np.max(np.abs(got - exact)) / np.max(np.abs(exact)) < 1e-5


def test_cholesky_equals_eigh_at_infinite_time(nt):
    """tests/predict_test.py:396-428."""
    x1, x2 = rows(3, 64, 20), rows(4, 16, 20)
    y = np.random.default_rng(5).standard_normal((64, 3))
    kf = nt.stax.serial(*fcn(nt.stax))[2]
    ktt, kts = kf(x1, None, 'ntk'), kf(x2, x1, 'ntk')
    pred = nt.predict.gradient_descent_mse(ktt, y, diag_reg=1e-2)
    a = pred(None, 0., 0., kts)[1].cpu().numpy()
    b = pred(np.inf, 0., 0., kts)[1].cpu().numpy()
    np.testing.assert_allclose(a, b, rtol=2e-4, atol=2e-5)


@pytest.mark.parametrize('n,m', [(33, 1), (100, 10), (1000, 7), (2048, 10), (300, 2500), (517, 129)])
def test_solve_sizes_and_refinement(nt, n, m):
    rng = np.random.default_rng(n)
    g = rng.standard_normal((n, n + 5)).astype(np.float32)
    k = (g @ g.T / n).astype(np.float32)
    b = rng.standard_normal((n, m)).astype(np.float32)
    s = nt.predict.CholeskySolver(torch.from_numpy(k).cuda(), 1e-3, False, refine_iters=2)
    x = s.solve(torch.from_numpy(b).cuda()).double().cpu().numpy()
    a = k.astype(np.float64) + 1e-3 * np.trace(k.astype(np.float64)) / n * np.eye(n)
    exact = np.linalg.solve(a, b.astype(np.float64))
    assert np.max(np.abs(x - exact)) / np.max(np.abs(exact)) < 1e-6
    s0 = nt.predict.CholeskySolver(torch.from_numpy(k).cuda(), 1e-3, False, refine_iters=0)
    x0 = s0.solve(torch.from_numpy(b).cuda()).double().cpu().numpy()
    assert np.max(np.abs(x - exact)) <= np.max(np.abs(x0 - exact)) + 1e-12


def test_not_positive_definite_gives_nan(nt):
    k = -np.eye(8, dtype=np.float32)
    pred = nt.predict.gradient_descent_mse(k, np.ones((8, 2)), diag_reg=0.)
    with pytest.warns(UserWarning, match='positive definite'):
        _, fx = pred(None, 0., 0., np.eye(8))
    assert torch.isnan(fx).all()


def test_finite_time_matches_oracle(nt):
    x = rows(6, 40, 12)
    y = np.random.default_rng(7).standard_normal((40, 2))
    kf = nt.stax.serial(*fcn(nt.stax))[2]
    ktt = kf(x, None, 'ntk')
    pred = nt.predict.gradient_descent_mse(ktt, y, diag_reg=1e-3)
    got = pred(2.5, 0., 0., ktt)
    want = o.gradient_descent_mse(ktt.double().cpu().numpy(), y, diag_reg=1e-3)(
        2.5, 0., 0., ktt.double().cpu().numpy())
    for g, w in zip(got, want):
        np.testing.assert_allclose(g.cpu().numpy(), w, rtol=1e-4, atol=1e-6)
