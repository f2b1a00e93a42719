"""GPU parity of predict.gradient_descent_mse, gp_inference and the ensemble (tensor-core Cholesky with
double-float refinement at t = None / inf, the library's eigensolver at finite t)."""
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
    # a time far past every eigenvalue's decay takes the eigenbasis path and meets the limit
    c = pred(1e12, 0., 0., kts)[1].cpu().numpy()
    np.testing.assert_allclose(c, a, rtol=2e-4, atol=2e-5)


def test_scalar_infinite_time_takes_the_cholesky_path(nt, monkeypatch):
    """A scalar t = inf is served by the Cholesky kernels (the limit t=None computes); an
    array of times containing inf keeps the eigenbasis path, where expm1(-inf) = -1."""
    x1, x2 = rows(6, 48, 20), rows(7, 8, 20)
    y = onehot(8, 48)
    kf = nt.stax.serial(*fcn(nt.stax))[2]
    ktt, kts = kf(x1, None, 'ntk'), kf(x2, x1, 'ntk')
    calls = []
    real = nt.predict.CholeskySolver.solve
    monkeypatch.setattr(nt.predict.CholeskySolver, 'solve',
                        lambda self, *a, **k: calls.append(1) or real(self, *a, **k))
    pred = nt.predict.gradient_descent_mse(ktt, y, diag_reg=1e-3)
    fx_train, fx_test = pred(np.inf, 0., 0., kts)
    assert calls, 'scalar t = inf did not reach the Cholesky solve'
    torch.testing.assert_close(fx_train, torch.tensor(y, dtype=torch.float32).cuda())
    want = pred(None, 0., 0., kts)[1]
    torch.testing.assert_close(fx_test, want, rtol=0, atol=0)
    both = pred(np.array([1., np.inf]), 0., 0., kts)[1]
    assert both.shape == (2, 8, 10)
    np.testing.assert_allclose(both[1].cpu().numpy(), want.cpu().numpy(), rtol=2e-4, atol=2e-5)


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


def test_finite_time_array_of_times_matches_oracle(nt):
    """predict_test.py:135-160 (_test_multi_step): t of shape (2, 1, 3) gives outputs of
    shape t.shape + fx.shape, each slice the prediction at that time; against the float64
    oracle, with nonzero initial outputs and held-out test inputs."""
    rng = np.random.default_rng(8)
    x, xt = rows(6, 40, 12), rows(9, 15, 12)
    y = rng.standard_normal((40, 2))
    f0, g0 = rng.standard_normal((40, 2)) * 0.3, rng.standard_normal((15, 2)) * 0.3
    kf = nt.stax.serial(*fcn(nt.stax))[2]
    kdd, ktd = kf(x, None, 'ntk'), kf(xt, x, 'ntk')
    ts = np.arange(6.).reshape(2, 1, 3) * 0.8
    got = nt.predict.gradient_descent_mse(kdd, y, learning_rate=1.5, diag_reg=1e-3)(
        ts, f0, g0, ktd)
    want = o.gradient_descent_mse(kdd.double().cpu().numpy(), y, learning_rate=1.5,
                                  diag_reg=1e-3)(ts, f0, g0, ktd.double().cpu().numpy())
    assert tuple(got[0].shape) == (2, 1, 3, 40, 2) and tuple(got[1].shape) == (2, 1, 3, 15, 2)
    for g, w in zip(got, want):
        np.testing.assert_allclose(g.cpu().numpy(), w, rtol=1e-4, atol=1e-6)


def _leaves(x):
    if isinstance(x, tuple):
        return [a for v in x for a in _leaves(v)]
    if isinstance(x, torch.Tensor):
        return [x.detach().double().cpu().numpy()]
    return [np.asarray(x, np.float64)]


def _ens_setup(nt):
    rng = np.random.default_rng(31)
    x_train = rng.standard_normal((40, 12))
    x_test = rng.standard_normal((15, 12))
    y_train = rng.standard_normal((40, 3))
    lay = lambda m: [m.Dense(64, 1.5, 0.2), m.Erf(), m.Dense(64, 1.3, 0.1), m.Relu(),
                     m.Dense(3, 1.2, 0.1)]
    return (nt.stax.serial(*lay(nt.stax))[2], o.serial(*lay(o)), x_train, x_test, y_train)


@pytest.mark.parametrize('get', ['nngp', 'ntk', ('ntk', 'nngp'), None])
@pytest.mark.parametrize('compute_cov', [False, True])
def test_gradient_descent_mse_ensemble_vs_oracle(nt, get, compute_cov):
    """predict.gradient_descent_mse_ensemble at t = None (Cholesky kernels) and at finite and
    infinite t (eigendecomposition) against the float64 oracle, on the train and a test set."""
    kf, ko, x_train, x_test, y_train = _ens_setup(nt)
    pred = nt.predict.gradient_descent_mse_ensemble(kf, x_train, y_train, diag_reg=1e-3)
    want_pred = o.gradient_descent_mse_ensemble(ko, x_train, y_train, diag_reg=1e-3)
    for x in (None, x_test):
        for t in (None, 0.5, np.array([1., 10.]), np.inf):
            got = _leaves(pred(t, x, get, compute_cov))
            want = _leaves(want_pred(t, x, get, compute_cov))
            assert len(got) == len(want)
            for g, w in zip(got, want):
                assert g.shape == w.shape
                scale = max(np.abs(w).max(), 1e-12)
                assert np.abs(g - w).max() / scale < 1e-4, (x is None, t)


def test_gp_inference_ntkgp_and_errors(nt):
    """predict.gp_inference: the NNGP / NTK / NTKGP posteriors against the oracle, and the
    reference's ValueError for an NTK covariance without the NNGP kernels."""
    kf, ko, x_train, x_test, y_train = _ens_setup(nt)
    k_dd = kf(x_train, None, ('nngp', 'ntk'))
    k_td = kf(x_test, x_train, ('nngp', 'ntk'))
    k_tt = kf(x_test, None, ('nngp', 'ntk'))
    ok_dd = dict(zip(('nngp', 'ntk'), ko(x_train, None, ('nngp', 'ntk'))))
    ok_td = dict(zip(('nngp', 'ntk'), ko(x_test, x_train, ('nngp', 'ntk'))))
    ok_tt = dict(zip(('nngp', 'ntk'), ko(x_test, None, ('nngp', 'ntk'))))
    gp = nt.predict.gp_inference(k_dd, y_train, diag_reg=1e-3)
    want = o.gp_inference(ok_dd, y_train, diag_reg=1e-3)
    for get in (('nngp', 'ntk', 'ntkgp'), 'ntkgp'):
        for g, w in zip(_leaves(gp(get, k_td, k_tt)), _leaves(want(get, ok_td, ok_tt))):
            assert np.abs(g - w).max() / max(np.abs(w).max(), 1e-12) < 1e-4
    with pytest.raises(ValueError):
        nt.predict.gp_inference({'ntk': k_dd.ntk}, y_train)(get='ntk',
                                                           k_test_train={'ntk': k_td.ntk},
                                                           k_test_test=k_tt.nngp)


def _power_law_features(seed, n, d=256, p=1.5):
    """Rows with a power-law feature spectrum: their Gram matrix is ill-conditioned like a
    deep-network NTK (eigenvalues ~ i^-2p)."""
    rng = np.random.default_rng(seed)
    scale = np.arange(1, d + 1, dtype=np.float64) ** -p
    return rng.standard_normal((n, d)) * scale


def test_infinite_time_mean_is_float64_accurate_on_an_ill_conditioned_kernel(nt):
    """predict.py:236-276 at t=None: k_test_train (K + lambda I)^{-1} y cancels when K is
    ill-conditioned (here cond ~ 7e4); the mean is formed from the FP64 solution in
    double-float, so it matches float64 to FP32 rounding rather than losing cond-many
    digits in an FP32 product. gp_inference's mean takes the same path."""
    feats = _power_law_features(7, 900)
    xtr, xte = feats[:800], feats[800:]
    k = (xtr @ xtr.T).astype(np.float32)
    kts = (xte @ xtr.T).astype(np.float32)
    y = onehot(3, 800)
    reg = 1e-2
    a = k.astype(np.float64) + reg * np.trace(k.astype(np.float64)) / 800 * np.eye(800)
    assert np.linalg.cond(a) > 1e4
    want = kts.astype(np.float64) @ sla.cho_solve(sla.cho_factor(a), y)
    scale = np.max(np.abs(want))
    fx = nt.predict.gradient_descent_mse(k, y, diag_reg=reg)(None, 0., 0., kts)[1]
    assert np.max(np.abs(fx.cpu().numpy() - want)) / scale < 1e-5
    mean = nt.predict.gp_inference(k, y, diag_reg=reg)(get='nngp', k_test_train=kts)
    assert np.max(np.abs(mean.cpu().numpy() - want)) / scale < 1e-5


def test_gemm_df_keeps_a_cancelling_product(nt):
    """ntg_gemm_df: A X with X = X1 + 1e6 X2, A X2 ~ 0 (X2 in A's null space): an FP32
    product would lose ~6 digits; double-float keeps the result to FP32 rounding."""
    from nt_gb300 import predict
    rng = np.random.default_rng(4)
    rows_, n, m = 37, 1000, 3
    a = rng.standard_normal((rows_, n)).astype(np.float32)
    a64 = a.astype(np.float64)
    null = sla.null_space(a64)[:, :m]
    x = rng.standard_normal((n, m)) + 1e6 * null
    want = a64 @ x
    got = predict._gemm_df(torch.from_numpy(a).cuda(), torch.from_numpy(x).cuda())
    got = got.cpu().numpy().astype(np.float64)
    assert np.max(np.abs(got - want) / np.abs(want)) < 1e-6
    # the FP32 product of the same operands, for scale: far off
    assert np.max(np.abs(a @ x.astype(np.float32) - want) / np.abs(want)) > 1e-4


def test_kernel_ridge_predict_and_its_gradients_vs_float64(nt):
    """kernel_ridge_predict (the t=None mean of predict.py:236-276 as a differentiable op) on
    an ill-conditioned kernel: forward and d/d(K_td, K, y) of <w, pred> against the float64
    closed forms gK_td = w alpha^T, gY = A^-1 K_td^T w, gK = -gY alpha^T - (r/n) <gY, alpha> I."""
    feats = _power_law_features(11, 136, d=96)
    xtr, xte = feats[:96], feats[96:]
    k = (xtr @ xtr.T).astype(np.float32)
    kts = (xte @ xtr.T).astype(np.float32)
    y = np.random.default_rng(5).standard_normal((96, 3)).astype(np.float32)
    w = np.random.default_rng(6).standard_normal((40, 3))
    reg = 1e-3
    k64 = k.astype(np.float64)
    a = k64 + reg * np.trace(k64) / 96 * np.eye(96)
    assert np.linalg.cond(a) > 1e3
    alpha = np.linalg.solve(a, y.astype(np.float64))
    want = kts.astype(np.float64) @ alpha
    gy_want = np.linalg.solve(a, kts.astype(np.float64).T @ w)
    gk_want = -gy_want @ alpha.T - reg / 96 * np.sum(gy_want * alpha) * np.eye(96)
    gkt_want = w @ alpha.T
    tk = torch.from_numpy(k).cuda().requires_grad_(True)
    tkt = torch.from_numpy(kts).cuda().requires_grad_(True)
    ty = torch.from_numpy(y).cuda().requires_grad_(True)
    pred = nt.predict.kernel_ridge_predict(tkt, tk, ty, diag_reg=reg)
    (pred.double() * torch.from_numpy(w).cuda()).sum().backward()

    def rel(got, ref):
        return np.max(np.abs(got.detach().cpu().numpy().astype(np.float64) - ref)) / np.max(np.abs(ref))
    assert rel(pred, want) < 1e-6
    assert rel(tkt.grad, gkt_want) < 1e-5
    assert rel(ty.grad, gy_want) < 1e-5
    assert rel(tk.grad, gk_want) < 1e-5
    # gradient_descent_mse's t=None test prediction is the same differentiable op
    tkt2 = torch.from_numpy(kts).cuda().requires_grad_(True)
    fx = nt.predict.gradient_descent_mse(k, y, diag_reg=reg)(None, 0., 0., tkt2)[1]
    assert rel(fx, want) < 1e-6
    (fx.double() * torch.from_numpy(w).cuda()).sum().backward()
    assert rel(tkt2.grad, gkt_want) < 1e-5
