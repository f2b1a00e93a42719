"""The tensor-core GEMM (3xTF32 tcgen05) and the blocked Cholesky built on it,
against float64 (scipy) on the same inputs: predict.py:1224-1258's cho_factor /
cho_solve, which the reference leaves to cuSOLVER."""
import numpy as np
import pytest
import scipy.linalg as sla
import torch

pytestmark = pytest.mark.gpu


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


@pytest.mark.parametrize('m,n,k,alpha,beta', [(128, 128, 32, 1., 0.), (300, 130, 100, -1., 1.),
                                              (1000, 700, 515, 0.5, 2.), (7, 5, 3, 1., 0.)])
def test_gemm_tc_matches_float64(nt, m, n, k, alpha, beta):
    from nt_gb300 import _lib as L
    rng = np.random.default_rng(m + n + k)
    kp = (k + 3) // 4 * 4  # row pitch: a multiple of 4 floats
    a = np.zeros((m, kp), np.float32)
    b = np.zeros((n, kp), np.float32)
    a[:, :k] = rng.standard_normal((m, k))
    b[:, :k] = rng.standard_normal((n, k))
    c0 = rng.standard_normal((m, n)).astype(np.float32)
    ta, tb, tc = _t(a), _t(b), _t(c0)
    L.call('ntg_gemm_tc', L.stream(), ta.data_ptr(), kp, tb.data_ptr(), kp, tc.data_ptr(), n, m,
           n, k, alpha, beta, 0)
    got = tc.cpu().numpy().astype(np.float64)
    a64, b64 = a[:, :k].astype(np.float64), b[:, :k].astype(np.float64)
    want = alpha * a64 @ b64.T + beta * c0
    scale = abs(alpha) * np.abs(a64) @ np.abs(b64).T + abs(beta) * np.abs(c0)
    assert np.max(np.abs(got - want) / scale) < 2e-6


def test_gemm_tc_lower_triangle_only(nt):
    from nt_gb300 import _lib as L
    rng = np.random.default_rng(3)
    n, k = 260, 128
    p = rng.standard_normal((n, k)).astype(np.float32)
    c0 = rng.standard_normal((n, n)).astype(np.float32)
    tp, tc = _t(p), _t(c0)
    L.call('ntg_gemm_tc', L.stream(), tp.data_ptr(), k, tp.data_ptr(), k, tc.data_ptr(), n, n, n,
           k, -1., 1., 1)
    got = tc.cpu().numpy()
    p64 = p.astype(np.float64)
    want = c0 - p64 @ p64.T
    low = np.tril(np.ones((n, n), bool))
    scale = np.abs(p64) @ np.abs(p64).T + np.abs(c0)
    assert np.max(np.abs(got - want)[low] / scale[low]) < 2e-6
    np.testing.assert_array_equal(got[~low], c0[~low])  # the upper triangle is untouched


def _spd(n, seed, cond_reg=1e-3):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, n + 7))
    k = g @ g.T / n
    return k.astype(np.float32)


def _factor(nt, k, diag_reg):
    from nt_gb300 import predict
    return predict.CholeskySolver(_t(k), diag_reg, False)


@pytest.mark.parametrize('n', [64, 128, 300, 1000])
def test_factor_matches_float64(nt, n):
    k = _spd(n, n)
    s = _factor(nt, k, 1e-3)
    assert s.info == 0
    lf = s.L.cpu().numpy().astype(np.float64)
    assert np.all(np.triu(lf, 1) == 0)
    a = k.astype(np.float64) + 1e-3 * np.trace(k.astype(np.float64)) / n * np.eye(n)
    # backward error of the FP32 factorisation
    assert np.max(np.abs(lf @ lf.T - a)) / np.max(np.abs(a)) < 1e-5
    want = np.linalg.cholesky(a)
    assert np.max(np.abs(lf - want)) / np.max(np.abs(want)) < 1e-4


@pytest.mark.parametrize('n,m', [(300, 1), (1000, 10), (777, 16), (513, 40), (1000, 300)])
def test_solve_matches_float64(nt, n, m):
    k = _spd(n, n + m)
    s = _factor(nt, k, 1e-4)
    rng = np.random.default_rng(m)
    b = rng.standard_normal((n, m)).astype(np.float32)
    a = k.astype(np.float64) + 1e-4 * np.trace(k.astype(np.float64)) / n * np.eye(n)
    want = sla.cho_solve(sla.cho_factor(a), b.astype(np.float64))
    got = s.solve(_t(b)).cpu().numpy()
    assert np.max(np.abs(got - want)) / np.max(np.abs(want)) < 1e-6
    plain = s.solve(_t(b), refine_iters=0, residual=False).cpu().numpy()
    # the unrefined FP32 solve is within the conditioning of the problem (kappa ~ 4e4)
    assert np.max(np.abs(plain - want)) / np.max(np.abs(want)) < 5e-2
    assert float(s.residual.item()) < 1e-4 * np.max(np.abs(b))


def test_not_positive_definite_reports_the_pivot(nt):
    k = np.eye(200, dtype=np.float32)
    k[150, 150] = -1.
    with pytest.warns(UserWarning, match='not positive definite'):
        s = _factor(nt, k, 0.)
    assert s.info == 151


def test_logdet_matches_float64(nt):
    k = _spd(400, 9)
    s = _factor(nt, k, 1e-3)
    a = k.astype(np.float64) + 1e-3 * np.trace(k.astype(np.float64)) / 400 * np.eye(400)
    want = np.linalg.slogdet(a)[1]
    # each pivot carries the float32 factor's rounding (cond ~ 1e3 here)
    assert abs(float(s.logdet().item()) - want) < 5e-5 * abs(want)


def test_concurrent_factorisations_on_two_streams(nt):
    """Two host threads, each on its own stream, factorise different matrices at once: the
    library's per-device streams and events are taken by one factorisation at a time, so
    each factor is that of its own matrix."""
    import threading
    from nt_gb300 import predict
    ks = [_spd(700, 41 + i) for i in range(2)]
    out, errs = [None, None], []

    def work(i):
        try:
            st = torch.cuda.Stream()
            with torch.cuda.stream(st):
                for _ in range(3):
                    s = predict.CholeskySolver(_t(ks[i]), 1e-3, False)
                    out[i] = s.L.clone()
            st.synchronize()
        except Exception as e:  # reported below
            errs.append(e)
    threads = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errs
    for i in range(2):
        a = ks[i].astype(np.float64)
        a = a + 1e-3 * np.trace(a) / 700 * np.eye(700)
        lf = out[i].cpu().numpy().astype(np.float64)
        assert np.max(np.abs(lf @ lf.T - a)) / np.max(np.abs(a)) < 1e-5
