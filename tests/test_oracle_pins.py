"""Pins the CPU oracle to the reference's own known-answer and identity tests.

The reference (neural-tangents 0.6.6) ships no golden vectors; its tests pin
the analytic kernels by closed forms and identities. Each test below re-runs
one of them against the oracle, citing the reference test it restates, plus
closed forms derived from the mathematics.
"""
import math

import numpy as np
import pytest

from oracle import nt_oracle as o


def test_avg_pool_all_ones_kat():
    """tests/stax/stax_test.py:494-539."""
    X1, X2 = np.ones((4, 2, 3, 2)), np.ones((3, 2, 3, 2))
    ker = o.serial(o.AvgPool((2, 2), (1, 1), 'SAME', normalize_edges=False))(X1, X2)
    kn = o.serial(o.AvgPool((2, 2), (1, 1), 'SAME', normalize_edges=True))(X1, X2)
    np.testing.assert_allclose(kn.nngp, np.ones_like(kn.nngp))
    np.testing.assert_allclose(kn.cov1, np.ones_like(kn.cov1))
    np.testing.assert_allclose(kn.cov2, np.ones_like(kn.cov2))
    out_unnorm = np.array([[1., 1., 0.5], [0.5, 0.5, 0.25]])
    ku = np.transpose(np.outer(out_unnorm, out_unnorm).reshape(2, 3, 2, 3), (0, 2, 1, 3))
    np.testing.assert_allclose(ker.nngp, np.broadcast_to(ku[None, None], ker.nngp.shape))
    np.testing.assert_allclose(ker.cov1, np.broadcast_to(ku[None], ker.cov1.shape))
    np.testing.assert_allclose(ker.cov2, np.broadcast_to(ku[None], ker.cov2.shape))


@pytest.mark.parametrize('same_inputs', [True, False])
@pytest.mark.parametrize('do_stabilize', [True, False])
def test_ab_relu_identities(same_inputs, do_stabilize):
    """tests/stax/elementwise_test.py:541-636."""
    rng = np.random.default_rng(1)
    X0_1 = rng.standard_normal((3, 2))
    X0_2 = None if same_inputs else rng.standard_normal((4, 2))
    fc = o.Dense(5, 1, 0)
    relu = o.serial(fc, o.Relu())(X0_1, X0_2)
    for a, b in [(0, 1), (0, -1), (-1, 0), (1, 0)]:
        k = o.serial(fc, o.ABRelu(a, b, do_stabilize))(X0_1, X0_2)
        np.testing.assert_allclose(k.nngp, relu.nngp, rtol=1e-12)
        np.testing.assert_allclose(k.ntk, relu.ntk, rtol=1e-12)
    for a in [-5, -1, -0.5, 0, 0.5, 1, 5]:
        kid = o.serial(fc, o.Identity())(X0_1 * a, None if X0_2 is None else X0_2 * a)
        kab = o.serial(fc, o.ABRelu(a, a, do_stabilize))(X0_1, X0_2)
        np.testing.assert_allclose(kab.nngp, kid.nngp, rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(kab.cov1, kid.cov1, rtol=1e-10, atol=1e-12)
    for a in [-2, -1, 0, 1, 2]:
        kl = o.serial(fc, o.LeakyRelu(a, do_stabilize))(X0_1, X0_2)
        ka = o.serial(fc, o.ABRelu(a, 1))(X0_1, X0_2)
        np.testing.assert_allclose(kl.nngp, ka.nngp, rtol=1e-10)
    np.testing.assert_allclose(o.serial(fc, o.Abs())(X0_1, X0_2).ntk,
                               o.serial(fc, o.ABRelu(-1, 1))(X0_1, X0_2).ntk, rtol=1e-12)


def test_relu_arccos_closed_form():
    """Cho & Saul degree-1 arc-cosine kernel for Dense(W=1) -> Relu."""
    rng = np.random.default_rng(3)
    x1, x2 = rng.standard_normal((5, 7)), rng.standard_normal((4, 7))
    k = o.serial(o.Dense(3, 1., None), o.Relu())(x1, x2)
    q11 = np.sum(x1 ** 2, 1) / 7
    q22 = np.sum(x2 ** 2, 1) / 7
    q12 = x1 @ x2.T / 7
    norm = np.sqrt(np.outer(q11, q22))
    th = np.arccos(np.clip(q12 / norm, -1, 1))
    nngp = norm / (2 * np.pi) * (np.sin(th) + (np.pi - th) * np.cos(th))
    np.testing.assert_allclose(k.nngp, nngp, rtol=1e-12)
    np.testing.assert_allclose(k.ntk, q12 * (np.pi - th) / (2 * np.pi), rtol=1e-12)
    np.testing.assert_allclose(k.cov1, q11 / 2, rtol=1e-12)


def test_erf_arcsine_closed_form():
    """Williams' arcsine kernel for Dense(W=1) -> Erf."""
    rng = np.random.default_rng(4)
    x1, x2 = rng.standard_normal((5, 6)), rng.standard_normal((3, 6))
    k = o.serial(o.Dense(3, 1., None), o.Erf())(x1, x2)
    q11 = np.sum(x1 ** 2, 1) / 6
    q22 = np.sum(x2 ** 2, 1) / 6
    q12 = x1 @ x2.T / 6
    nngp = 2 / np.pi * np.arcsin(2 * q12 / np.sqrt(np.outer(1 + 2 * q11, 1 + 2 * q22)))
    np.testing.assert_allclose(k.nngp, nngp, rtol=1e-12)


def test_serial_composition():
    """tests/stax/stax_test.py:636-687: serial(B, B) == B o B."""
    rng = np.random.default_rng(5)
    x1, x2 = rng.standard_normal((2, 8, 8, 3)), rng.standard_normal((3, 8, 8, 3))
    B = [o.Conv(1, (3, 3), padding='SAME', W_std=1.3, b_std=0.2), o.Relu()]
    kbb = o.serial(*B, *B)(x1, x2)
    kb = o.serial(*B)(x1, x2)
    kb2 = o.serial(*B).apply_to_kernel(kb)
    np.testing.assert_allclose(kbb.nngp, kb2.nngp, rtol=1e-12)
    np.testing.assert_allclose(kbb.ntk, kb2.ntk, rtol=1e-12)


@pytest.mark.parametrize('avg_pool', [True, False])
@pytest.mark.parametrize('same_inputs', [True, False])
def test_serial_composition_conv_readouts(avg_pool, same_inputs):
    """tests/stax/stax_test.py:654-685: a conv block followed by a readout. Composed ==
    readout o block with the block's kernel full-spatial or by default; a diagonal-spatial
    block kernel is enough for Flatten, and a ValueError for a Conv + GlobalAvgPool readout,
    which needs the full spatial covariance (requirements.py:100-112)."""
    rng = np.random.default_rng(11)
    x1 = rng.standard_normal((3, 5, 5, 3))
    x2 = None if same_inputs else rng.standard_normal((4, 5, 5, 3))
    block = [o.Conv(1, (3, 3)), o.Relu()]
    readout = ([o.Conv(1, (3, 3)), o.GlobalAvgPool(), o.Dense(1)] if avg_pool
               else [o.Flatten(), o.Dense(1)])
    composed = o.serial(*block, *readout)(x1, x2)
    rf, bf = o.serial(*readout), o.serial(*block)
    # the default block kernel is diagonal-spatial for the Flatten readout: its Relu runs on the
    # diagonal entries alone, where correlations near 1 make the arc-cosine lose ~1e-10
    tol = 1e-12 if avg_pool else 1e-8
    for k in (rf.apply_to_kernel(bf(x1, x2, diagonal_spatial=False)),
              rf.apply_to_kernel(bf(x1, x2))):
        np.testing.assert_allclose(k.nngp, composed.nngp, rtol=tol)
        np.testing.assert_allclose(k.ntk, composed.ntk, rtol=tol)
    if avg_pool:
        with pytest.raises(ValueError):
            rf.apply_to_kernel(bf(x1, x2, diagonal_spatial=True))
        with pytest.raises(ValueError):
            o.serial(*block, *readout)(x1, x2, diagonal_spatial=True)
    else:
        k = rf.apply_to_kernel(bf(x1, x2, diagonal_spatial=True))
        np.testing.assert_allclose(k.nngp, composed.nngp, rtol=1e-8)
        np.testing.assert_allclose(k.ntk, composed.ntk, rtol=1e-8)


def _conv_expectation(x1, x2, W_std, b_std, fs=3):
    """E[f(x1)[h,w] f(x2)[h',w']] of one SAME conv layer, written out directly."""
    n1, H, W, C = x1.shape
    n2 = x2.shape[0]
    p = fs // 2
    X1 = np.pad(x1, ((0, 0), (p, p), (p, p), (0, 0)))
    X2 = np.pad(x2, ((0, 0), (p, p), (p, p), (0, 0)))
    out = np.zeros((n1, n2, H, H, W, W))
    for h in range(H):
        for hp in range(H):
            for w in range(W):
                for wp in range(W):
                    acc = 0.
                    for d in range(fs):
                        for e in range(fs):
                            acc = acc + np.einsum('ac,bc->ab', X1[:, h + d, w + e],
                                                  X2[:, hp + d, wp + e])
                    out[:, :, h, hp, w, wp] = W_std ** 2 * acc / (C * fs * fs) + b_std ** 2
    return out


def test_conv_rule_is_the_exact_covariance_of_a_conv_layer():
    """Conv full-spatial rule (linear.py:1321-1424) == direct expectation; layout is
    reversed after one Conv (is_reversed, linear.py:1344-1349)."""
    rng = np.random.default_rng(6)
    x1, x2 = rng.standard_normal((2, 5, 4, 3)), rng.standard_normal((2, 5, 4, 3))
    k = o.serial(o.Conv(7, (3, 3), padding='SAME', W_std=1.7, b_std=0.3))(x1, x2)
    assert k.is_reversed
    direct = _conv_expectation(x1, x2, 1.7, 0.3)
    np.testing.assert_allclose(o.reverse_zipped(k.nngp, 2), direct, rtol=1e-12)
    np.testing.assert_allclose(k.ntk, k.nngp, rtol=1e-12)


def test_relu_conv_monte_carlo():
    """Analytic Conv->Relu->Conv kernel vs a width-4096 finite network (MC)."""
    rng = np.random.default_rng(7)
    x = rng.standard_normal((2, 4, 4, 2))
    k = o.serial(o.Conv(1, (3, 3), padding='SAME', W_std=1.5, b_std=0.1), o.Relu(),
                 o.Conv(1, (3, 3), padding='SAME', W_std=1.2, b_std=0.2))(x, None)
    width = 4096
    H = W = 4

    def conv(z, cin, cout, W_std, b_std):
        Wt = rng.standard_normal((3, 3, cin, cout)) * W_std / math.sqrt(cin * 9)
        b = rng.standard_normal(cout) * b_std
        zp = np.pad(z, ((0, 0), (1, 1), (1, 1), (0, 0)))
        out = np.zeros(z.shape[:3] + (cout,))
        for d in range(3):
            for e in range(3):
                out += zp[:, d:d + H, e:e + W] @ Wt[d, e]
        return out + b

    y = conv(np.maximum(conv(x, 2, width, 1.5, 0.1), 0), width, width, 1.2, 0.2)
    emp = np.einsum('ahwc,bgvc->abhgwv', y, y) / width
    ana = k.nngp if not k.is_reversed else o.reverse_zipped(k.nngp, 2)
    assert np.abs(emp - ana).max() < 0.15 * np.abs(ana).max()


def test_flatten_vs_global_avg_pool():
    """Flatten averages the spatial diagonal, GlobalAvgPool all entries (linear.py:1777-1882)."""
    rng = np.random.default_rng(8)
    x = rng.standard_normal((2, 4, 4, 3))
    base = [o.Conv(1, (3, 3), padding='SAME', W_std=1.1), o.Relu()]
    kf = o.serial(*base, o.Flatten())(x, None)
    kg = o.serial(*base, o.GlobalAvgPool())(x, None)
    kc = o.serial(*base)(x, None)
    full = kc.nngp
    np.testing.assert_allclose(kg.nngp, full.mean(axis=(2, 3, 4, 5)), rtol=1e-12)
    diag = np.einsum('abhhww->abhw', full).mean(axis=(2, 3))
    np.testing.assert_allclose(kf.nngp, diag, rtol=1e-12)


def test_cholesky_equals_eigh_infinite_time():
    """tests/predict_test.py:396-428."""
    rng = np.random.default_rng(9)
    x = rng.standard_normal((20, 5))
    xt = rng.standard_normal((7, 5))
    kf = o.serial(o.Dense(1, 1.5, 0.1), o.Relu(), o.Dense(1, 1.5, 0.1))
    ktt = kf(x, None, 'ntk')
    kts = kf(xt, x, 'ntk')
    y = rng.standard_normal((20, 3))
    pf = o.gradient_descent_mse(ktt, y, diag_reg=1e-3)
    a = pf(None, 0., 0., kts)
    b = pf(np.inf, 0., 0., kts)
    np.testing.assert_allclose(a[1], b[1], rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(a[0], y)


def test_myrtle5_readout_flatten_equals_mean_after_pools():
    """AvgPool(2,2) down to 1x1 followed by Flatten is the mean of the 8^4 entries."""
    rng = np.random.default_rng(10)
    x = rng.standard_normal((1, 8, 8, 3))
    base = [o.Conv(1, (3, 3), padding='SAME', W_std=1.4), o.Relu()]
    k1 = o.serial(*base, *[o.AvgPool((2, 2), (2, 2))] * 3, o.Flatten())(x, None)
    k2 = o.serial(*base, o.GlobalAvgPool())(x, None)
    np.testing.assert_allclose(k1.nngp, k2.nngp, rtol=1e-12)


# ---------------------------------------------------------------------------
# gp_inference / gradient_descent_mse_ensemble pins (tests/predict_test.py)
# ---------------------------------------------------------------------------
def _leaves(x):
    if isinstance(x, tuple):
        return [a for v in x for a in _leaves(v)]
    return [np.asarray(x, np.float64)]


def _fcn_ens_setup():
    rng = np.random.default_rng(21)
    x_train = rng.standard_normal((10, 5))
    x_test = rng.standard_normal((6, 5))
    y_train = rng.standard_normal((10, 3))
    kf = o.serial(o.Dense(16, 1.5, 0.2), o.Erf(), o.Dense(3, 1.2, 0.1))
    return kf, x_train, x_test, y_train


@pytest.mark.parametrize('get', ['nngp', 'ntk', ('nngp', 'ntk')])
def test_ensemble_infinite_time_agreement(get):
    """predict_test.py:396-428: t = inf (eigh) equals t = None (Cholesky), with covariance."""
    kf, x_train, x_test, y_train = _fcn_ens_setup()
    pred = o.gradient_descent_mse_ensemble(kf, x_train, y_train, diag_reg=1e-6)
    for x in (None, x_test):
        fin = pred(t=np.inf, x_test=x, get=get, compute_cov=True)
        inf = pred(t=None, x_test=x, get=get, compute_cov=True)
        for a, b in zip(_leaves(fin), _leaves(inf)):
            np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-6)


def test_ensemble_zero_time_agreement():
    """predict_test.py:437-491: at t = 0 the mean is 0 and the covariance the prior NNGP."""
    kf, x_train, x_test, y_train = _fcn_ens_setup()
    pred = o.gradient_descent_mse_ensemble(kf, x_train, y_train, diag_reg=1e-7)
    for x in (None, x_test):
        out = pred(t=0., x_test=x, get=('ntk', 'nngp'), compute_cov=True)
        prior = kf(x_train if x is None else x, None, 'nngp')
        for g in out:
            np.testing.assert_allclose(g.mean, 0., atol=1e-12)
            # the regularised train-train matrix enters the NNGP train-set covariance: diag_reg
            # (1e-7 of the mean trace) is the only difference
            np.testing.assert_allclose(g.covariance, prior, rtol=1e-6, atol=1e-6)


def test_ensemble_covariance_symmetric_psd():
    """predict_test.py:586-620: posterior covariances are symmetric positive semi-definite."""
    kf, x_train, x_test, y_train = _fcn_ens_setup()
    pred = o.gradient_descent_mse_ensemble(kf, x_train, y_train)
    ts = np.logspace(-3, 3, 5)
    for get in ('nngp', 'ntk'):
        for x in (None, x_test):
            for t in (None, ts):
                cov = pred(t=t, x_test=x, get=get, compute_cov=True).covariance
                np.testing.assert_allclose(cov, np.swapaxes(cov, -1, -2), atol=1e-10)
                assert np.min(np.linalg.eigvalsh(cov)) > -1e-4


def test_gp_inference_matches_ensemble_and_ntkgp_is_nngp_with_ntk():
    """predict_test.py:704-824: gp_inference equals the ensemble at t = None, and NTKGP is the
    NNGP posterior computed with the NTK in place of the NNGP."""
    kf, x_train, x_test, y_train = _fcn_ens_setup()
    k_dd = dict(zip(('nngp', 'ntk'), kf(x_train, None, ('nngp', 'ntk'))))
    k_td = dict(zip(('nngp', 'ntk'), kf(x_test, x_train, ('nngp', 'ntk'))))
    k_tt = dict(zip(('nngp', 'ntk'), kf(x_test, None, ('nngp', 'ntk'))))
    gp = o.gp_inference(k_dd, y_train, diag_reg=1e-5)
    ens = o.gradient_descent_mse_ensemble(kf, x_train, y_train, diag_reg=1e-5)
    a = gp(get=('nngp', 'ntk'), k_test_train=k_td, k_test_test=k_tt['nngp'])
    b = ens(None, x_test, ('nngp', 'ntk'), True)
    for ga, gb in zip(a, b):
        np.testing.assert_allclose(ga.mean, gb.mean, rtol=1e-10)
        np.testing.assert_allclose(ga.covariance, gb.covariance, rtol=1e-9, atol=1e-12)
    ntkgp = gp(get='ntkgp', k_test_train=k_td, k_test_test=k_tt)
    only_ntk = o.gp_inference({'nngp': k_dd['ntk']}, y_train, diag_reg=1e-5)(
        get='nngp', k_test_train={'nngp': k_td['ntk']}, k_test_test=k_tt['ntk'])
    np.testing.assert_allclose(ntkgp.mean, only_ntk.mean, rtol=1e-12)
    np.testing.assert_allclose(ntkgp.covariance, only_ntk.covariance, rtol=1e-12)
    with pytest.raises(ValueError):
        o.gp_inference({'ntk': k_dd['ntk']}, y_train)(get='ntk', k_test_train={'ntk': k_td['ntk']},
                                                      k_test_test=k_tt['nngp'])


# ---------------------------------------------------------------------------
# Gelu / Sin / Cos / Rbf (elementwise.py:195-400): Gaussian expectations by Monte Carlo,
# the check of the reference's elementwise tests (tests/stax/elementwise_test.py)
# ---------------------------------------------------------------------------
def _phi_pairs():
    from scipy.special import ndtr
    r2 = np.sqrt(2.)
    return [
        (o.Sin(1.3, 0.7, 0.2), lambda x: 1.3 * np.sin(0.7 * x + 0.2),
         lambda x: 1.3 * 0.7 * np.cos(0.7 * x + 0.2)),
        (o.Cos(0.9, 1.1, -0.3), lambda x: 0.9 * np.cos(1.1 * x - 0.3),
         lambda x: -0.9 * 1.1 * np.sin(1.1 * x - 0.3)),
        (o.Rbf(0.6), lambda x: r2 * np.sin(np.sqrt(1.2) * x + np.pi / 4),
         lambda x: r2 * np.sqrt(1.2) * np.cos(np.sqrt(1.2) * x + np.pi / 4)),
        (o.Gelu(), lambda x: x * ndtr(x),
         lambda x: ndtr(x) + x * np.exp(-x * x / 2) / np.sqrt(2 * np.pi)),
    ]


@pytest.mark.parametrize('case', range(4))
def test_dual_activations_match_gaussian_expectations(case):
    layer, phi, dphi = _phi_pairs()[case]
    rng = np.random.default_rng(40 + case)
    x = rng.standard_normal((2, 6))
    kf = o.serial(o.Dense(1, 1.1, 0.3), layer)
    q, t = kf(x[:1], x[1:], ('nngp', 'ntk'))
    c1, c2 = kf(x[:1], None, 'nngp'), kf(x[1:], None, 'nngp')
    pre = o.serial(o.Dense(1, 1.1, 0.3))
    v1 = float(pre(x[:1], None, 'nngp')[0, 0])
    v2 = float(pre(x[1:], None, 'nngp')[0, 0])
    qq = float(pre(x[:1], x[1:], 'nngp')[0, 0])
    tt = float(pre(x[:1], x[1:], 'ntk')[0, 0])
    n = 4_000_000
    z = rng.standard_normal((n, 2))
    l = np.linalg.cholesky(np.array([[v1, qq], [qq, v2]]))
    u = z @ l.T
    for got, samples in ((q[0, 0], phi(u[:, 0]) * phi(u[:, 1])),
                         (t[0, 0], tt * dphi(u[:, 0]) * dphi(u[:, 1])),
                         (c1[0, 0], phi(np.sqrt(v1) * z[:, 0]) ** 2),
                         (c2[0, 0], phi(np.sqrt(v2) * z[:, 1]) ** 2)):
        mean, err = samples.mean(), samples.std() / np.sqrt(n)
        assert abs(got - mean) < 6 * err + 1e-12, (got, mean, err)


@pytest.mark.parametrize('act', ['relu', 'erf', 'gelu', 'sin', 'rbf'])
def test_diagonal_spatial_is_the_diagonal_of_the_full_kernel(act):
    """requirements_test.py:55-137 (diagonal_batch / diagonal_spatial consistency): for a CNN
    without pooling the diagonal-spatial kernels equal the (h, h, w, w) entries of the
    full-spatial ones, nngp, ntk and the per-sample covariances alike."""
    mk = {'relu': lambda: o.Relu(), 'erf': lambda: o.Erf(), 'gelu': lambda: o.Gelu(),
          'sin': lambda: o.Sin(1.1, 0.9, 0.3), 'rbf': lambda: o.Rbf(0.4)}[act]
    kf = o.serial(o.Conv(2, (3, 3), padding='SAME', W_std=1.3, b_std=0.2), mk(),
                  o.Conv(2, (2, 3), strides=(1, 2), padding='VALID', W_std=1.1, b_std=0.1), mk())
    rng = np.random.default_rng(12)
    x1, x2 = rng.standard_normal((2, 6, 7, 3)), rng.standard_normal((3, 6, 7, 3))
    full = kf(x1, x2, None, diagonal_spatial=False)
    diag = kf(x1, x2, None, diagonal_spatial=True)
    assert not full.is_reversed and full.nngp.ndim == 6 and diag.nngp.ndim == 4
    pick2 = lambda k: np.einsum('abhhww->abhw', k)
    pick1 = lambda k: np.einsum('ahhww->ahw', k)
    np.testing.assert_allclose(diag.nngp, pick2(full.nngp), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(diag.ntk, pick2(full.ntk), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(diag.cov1, pick1(full.cov1), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(diag.cov2, pick1(full.cov2), rtol=1e-12, atol=1e-12)


# ---------------------------------------------------------------------------
# The same rules against a deterministic quadrature: the check of the reference's
# ElementwiseNumericalTest (tests/stax/elementwise_test.py:480-538), which compares each
# closed-form rule with its Gauss-Hermite rule (ElementwiseNumerical,
# elementwise.py:1134-1247). For the smooth activations a 120-point tensor rule is
# exact to ~1e-12 at these variances, so the closed forms are pinned far tighter than
# by sampling.
# ---------------------------------------------------------------------------
def _gauss_hermite_2d(f, v1, v2, q, deg=120):
    """E[f(u, v)] for (u, v) ~ N(0, [[v1, q], [q, v2]]): probabilists' Gauss-Hermite
    nodes in each of two independent standard normals, u = a z1, v = b z1 + c z2."""
    z, w = np.polynomial.hermite_e.hermegauss(deg)
    w = w / math.sqrt(2 * math.pi)
    a = math.sqrt(v1)
    b = q / a
    c = math.sqrt(max(v2 - b * b, 0.))
    u = a * z[:, None] + 0. * z[None, :]
    v = b * z[:, None] + c * z[None, :]
    return float(np.sum(w[:, None] * w[None, :] * f(u, v)))


def _smooth_cases():
    from scipy.special import erf
    erf_case = (o.Erf(), lambda x: erf(x), lambda x: 2 / math.sqrt(math.pi) * np.exp(-x * x))
    return _phi_pairs() + [erf_case]


@pytest.mark.parametrize('case', range(5))
def test_dual_activations_match_gauss_hermite_quadrature(case):
    """Second layer of Dense -> phi -> Dense -> phi: nngp, ntk and both per-sample
    variances of the rule equal the quadrature of phi(u) phi(v) (and ntk_in E[phi'(u)
    phi'(v)]) over the first three layers' kernel, as the reference's numerical test
    composes them (depth 2, W_std 1, b_std 0.01 there; other scales here)."""
    layer, phi, dphi = _smooth_cases()[case]
    rng = np.random.default_rng(60 + case)
    x1, x2 = rng.standard_normal((3, 7)), rng.standard_normal((2, 7))
    body = [o.Dense(1, 1.2, 0.1), layer, o.Dense(1, 0.9, 0.2)]
    kin = o.serial(*body)(x1, x2)
    kout = o.serial(*body, layer)(x1, x2)
    pp = lambda u, v: phi(u) * phi(v)
    dd = lambda u, v: dphi(u) * dphi(v)
    for i in range(3):
        v1 = float(kin.cov1[i])
        np.testing.assert_allclose(kout.cov1[i], _gauss_hermite_2d(pp, v1, v1, v1),
                                   rtol=1e-10, atol=1e-13)
        for j in range(2):
            v2, q, t = float(kin.cov2[j]), float(kin.nngp[i, j]), float(kin.ntk[i, j])
            np.testing.assert_allclose(kout.nngp[i, j], _gauss_hermite_2d(pp, v1, v2, q),
                                       rtol=1e-10, atol=1e-13)
            np.testing.assert_allclose(kout.ntk[i, j], t * _gauss_hermite_2d(dd, v1, v2, q),
                                       rtol=1e-10, atol=1e-13)
    for j in range(2):
        v2 = float(kin.cov2[j])
        np.testing.assert_allclose(kout.cov2[j], _gauss_hermite_2d(pp, v2, v2, v2),
                                   rtol=1e-10, atol=1e-13)


def test_sin_closed_form():
    """tests/stax/elementwise_test.py:428-437: Sin with its default a = b = 1, c = 0 has
    nngp = (exp(-(v1 + v2) / 2 + q) - exp(-(v1 + v2) / 2 - q)) / 2."""
    rng = np.random.default_rng(61)
    x1, x2 = rng.standard_normal((4, 5)), rng.standard_normal((3, 5))
    pre = o.serial(o.Dense(1, 1.1, 0.2))
    kin = pre(x1, x2)
    k = o.serial(o.Dense(1, 1.1, 0.2), o.Sin())(x1, x2)
    s = -0.5 * (kin.cov1[:, None] + kin.cov2[None, :])
    want = (np.exp(s + kin.nngp) - np.exp(s - kin.nngp)) / 2
    np.testing.assert_allclose(k.nngp, want, rtol=1e-12)


# ---------------------------------------------------------------------------
# gradient_descent_mse in time (tests/predict_test.py:108-160, 192-273)
# ---------------------------------------------------------------------------
def _linear_model(n=12, m=5, p=30, k=3, seed=70):
    """A network that is its own linearisation: f(x) = phi(x) w with fixed features, so
    its NTK is phi phi^T exactly and gradient flow on the MSE loss is a linear ODE."""
    rng = np.random.default_rng(seed)
    ph, pt = rng.standard_normal((n, p)), rng.standard_normal((m, p))
    w0 = rng.standard_normal((p, k)) * 0.3
    y = rng.standard_normal((n, k))
    return ph, pt, w0, y


def test_gd_mse_zero_multi_and_infinite_time():
    """predict_test.py:108-160: t = 0 returns the initial outputs; an array of times equals
    the stacked single-time predictions, shape t.shape + fx.shape; t = inf on the train set
    returns y and equals the t = None (Cholesky) predictions."""
    ph, pt, w0, y = _linear_model()
    k_dd, k_td = ph @ ph.T, pt @ ph.T
    f0, g0 = ph @ w0, pt @ w0
    pred = o.gradient_descent_mse(k_dd, y, learning_rate=0.7)
    a, b = pred(0., f0, g0, k_td)
    np.testing.assert_allclose(a, f0, rtol=0, atol=1e-13)
    np.testing.assert_allclose(b, g0, rtol=0, atol=1e-13)
    np.testing.assert_allclose(pred(0., f0), f0, rtol=0, atol=1e-13)
    ts = np.arange(6.).reshape(2, 1, 3) * 40.
    a, b = pred(ts, f0, g0, k_td)
    assert a.shape == ts.shape + f0.shape and b.shape == ts.shape + g0.shape
    for idx in np.ndindex(ts.shape):
        sa, sb = pred(ts[idx], f0, g0, k_td)
        np.testing.assert_allclose(a[idx], sa, rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(b[idx], sb, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(pred(np.inf, f0), y, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(pred(np.inf, f0), pred(None, f0, None, None), rtol=1e-10)
    for u, v in zip(pred(np.inf, f0, g0, k_td), pred(None, f0, g0, k_td)):
        np.testing.assert_allclose(u, v, rtol=1e-9, atol=1e-11)


def test_gd_mse_equals_gradient_flow_of_a_linearised_network():
    """predict_test.py:192-273 (testNTKGDPrediction, loss 'mse_analytic'): the analytic
    predictions at time t equal the network trained by gradient descent for time t on
    0.5 mean((f - y)^2). Here the network is exactly linear in its parameters, and its
    gradient flow dw/dt = -lr phi^T (phi w - y) / y.size is integrated in parameter space
    by the exponential of the augmented [[A, b], [0, 0]] matrix, independently of the
    eigenbasis in function space that the predictor uses."""
    import scipy.linalg as sla
    ph, pt, w0, y = _linear_model()
    lr, T = 0.7, 35.
    n, k = y.shape
    p = ph.shape[1]
    A = -lr * ph.T @ ph / y.size
    wT = np.empty_like(w0)
    for c in range(k):
        M = np.zeros((p + 1, p + 1))
        M[:p, :p] = A
        M[:p, p] = lr * ph.T @ y[:, c] / y.size
        wT[:, c] = (sla.expm(T * M) @ np.append(w0[:, c], 1.))[:p]
    pred = o.gradient_descent_mse(ph @ ph.T, y, learning_rate=lr)
    ftr, fte = pred(T, ph @ w0, pt @ w0, pt @ ph.T)
    np.testing.assert_allclose(ftr, ph @ wT, rtol=1e-9, atol=1e-11)
    np.testing.assert_allclose(fte, pt @ wT, rtol=1e-9, atol=1e-11)
    # and the trajectory moved: the initial outputs are far from the trained ones
    assert np.abs(ftr - ph @ w0).max() > 0.1


@pytest.mark.parametrize('same_inputs', [True, False])
def test_flatten_at_the_bottom_equals_dense_on_flattened_inputs(same_inputs):
    """tests/stax/linear_test.py:53-100: serial(Flatten, Dense, Erf, Dense) on images equals
    serial(Dense, Erf, Dense) on the flattened images, nngp and ntk."""
    rng = np.random.default_rng(13)
    x1 = rng.standard_normal((4, 4, 3, 2))
    x2 = None if same_inputs else rng.standard_normal((2, 4, 3, 2))
    flat = lambda x: None if x is None else x.reshape(x.shape[0], -1)
    dense = lambda: o.Dense(512, 1.7, 0.1)
    k = o.serial(dense(), o.Erf(), dense())(flat(x1), flat(x2), ('nngp', 'ntk'))
    kb = o.serial(o.Flatten(), dense(), o.Erf(), dense())(x1, x2, ('nngp', 'ntk'))
    for a, b in zip(kb, k):
        np.testing.assert_allclose(a, b, rtol=1e-12)


@pytest.mark.parametrize('with_t', [False, True])
@pytest.mark.parametrize('with_x', [False, True])
def test_ensemble_ntk_nngp_agreement(with_t, with_x):
    """predict_test.py:493-584 (testNTK_NTKNNGPAgreement): an array of times equals the
    stacked single-time predictions; the NTK mean equals the NNGP equations run on a kernel
    function that always returns the NTK; and the NNGP covariance equals the NTK equations
    run on one that always returns the NNGP (the reference checks this one roughly:
    ~5e-7 here at diag_reg 1e-7)."""
    rng = np.random.default_rng(80)
    x_train, x_test = rng.standard_normal((8, 6)), rng.standard_normal((4, 6))
    y = (rng.random((8, 2)) > 0.5).astype(np.float64)
    kf = o.serial(o.Dense(64, W_std=1.2, b_std=0.05), o.Erf(), o.Dense(2, W_std=1.2, b_std=0.05))
    reg = 1e-7
    ts = np.logspace(-2, 8, 10).reshape(5, 2) if with_t else None
    x = x_test if with_x else None
    pred = o.gradient_descent_mse_ensemble(kf, x_train, y, diag_reg=reg)
    ntk = np.asarray(pred(t=ts, get='ntk', x_test=x))
    if ts is not None:
        each = np.array([pred(t=t, get='ntk', x_test=x) for t in ts.ravel()])
        np.testing.assert_allclose(each.reshape(ts.shape + ntk.shape[2:]), ntk, rtol=1e-12,
                                   atol=1e-14)
    always_ntk = lambda a, b, get: kf(a, b, 'ntk')
    always_nngp = lambda a, b, get: kf(a, b, 'nngp')
    ntk_nngp = o.gradient_descent_mse_ensemble(always_ntk, x_train, y, diag_reg=reg)(
        t=ts, get='nngp', x_test=x)
    np.testing.assert_allclose(np.asarray(ntk_nngp), ntk, rtol=1e-10, atol=1e-12)
    nngp_cov = pred(t=ts, get='nngp', x_test=x, compute_cov=True).covariance
    ntk_cov = o.gradient_descent_mse_ensemble(always_nngp, x_train, y, diag_reg=reg)(
        t=ts, get='ntk', x_test=x, compute_cov=True).covariance
    assert ntk_cov.shape == nngp_cov.shape
    np.testing.assert_allclose(ntk_cov, nngp_cov, rtol=0,
                               atol=5e-6 * max(np.abs(nngp_cov).max(), 1e-3))


@pytest.mark.parametrize('get', ['ntk', 'nngp'])
def test_ensemble_mean_and_covariance_of_an_exactly_linear_network(get):
    """predict_test.py:622-686 (testTrainedEnsemblePredCov) made exact: an ensemble of
    networks f(x) = phi(x) w / sqrt(p), w0 ~ N(0, I), is its own linearisation with
    NNGP = NTK = phi phi^T / p. Gradient flow on 0.5 mean((f - y)^2) maps w0 to
    w(T) = E w0 + c (E, c from the exponential of the augmented parameter-space system), so
    the ensemble of outputs at time T has mean phi c / sqrt(p) and covariance
    phi E E^T phi^T / p, independently of the function-space equations of
    gradient_descent_mse_ensemble, on the training and the test inputs."""
    import scipy.linalg as sla
    rng = np.random.default_rng(90)
    n, m, p, k = 10, 4, 25, 2
    ph, pt = rng.standard_normal((n, p)), rng.standard_normal((m, p))
    y = rng.standard_normal((n, k))
    feats = np.concatenate([ph, pt])

    def kf(a, b, get):  # inputs are row indices into the feature table
        fa = feats[np.asarray(a, int)]
        fb = fa if b is None else feats[np.asarray(b, int)]
        return fa @ fb.T / p

    lr, T = 0.9, 40.
    A = -lr * ph.T @ ph / (y.size * p)
    E = sla.expm(T * A)
    c = np.empty((p, k))
    for j in range(k):
        M = np.zeros((p + 1, p + 1))
        M[:p, :p] = A
        M[:p, p] = lr * ph.T @ y[:, j] / (y.size * math.sqrt(p))
        c[:, j] = (sla.expm(T * M) @ np.append(np.zeros(p), 1.))[:p]
    pred = o.gradient_descent_mse_ensemble(kf, np.arange(n), y, learning_rate=lr)
    for x, f in ((np.arange(n, n + m), pt), (None, ph)):
        r = pred(t=T, x_test=x, get=get, compute_cov=True)
        np.testing.assert_allclose(r.mean, f @ c / math.sqrt(p), rtol=1e-10, atol=1e-13)
        np.testing.assert_allclose(r.covariance, f @ E @ E.T @ f.T / p, rtol=1e-10, atol=1e-13)
    assert np.abs(f @ c).max() > 0.1  # the ensemble has moved towards y
