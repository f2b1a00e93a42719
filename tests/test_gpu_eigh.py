"""The block-Jacobi eigensolver (ntg_eigh) and the spectral-weight kernel behind the
finite-time predictions (predict.py:185-229, 1180-1294, where the reference calls eigh),
against float64 numpy on the same matrices."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _sym(n, seed, kind):
    rng = np.random.default_rng(seed)
    if kind == 'psd':  # a kernel-like matrix: fast-decaying spectrum, clustered tail
        g = rng.standard_normal((n, max(4, n // 4)))
        a = g @ g.T / g.shape[1] + 1e-3 * np.eye(n)
    else:  # indefinite
        g = rng.standard_normal((n, n))
        a = (g + g.T) / 2
    return a.astype(np.float32)


@pytest.mark.parametrize('n', [1, 5, 40, 64, 100, 257, 1000])
@pytest.mark.parametrize('kind', ['psd', 'indefinite'])
def test_eigh_matches_float64(nt, n, kind):
    from nt_gb300 import predict
    a = _sym(n, n, kind)
    evals, evecs = predict._eigh(torch.from_numpy(a).cuda(), 0.)
    w = evals.double().cpu().numpy()
    v = evecs.double().cpu().numpy()
    a64 = a.astype(np.float64)
    scale = np.linalg.norm(a64, 2)
    # residual of every pair, orthogonality, eigenvalues against numpy's
    assert np.max(np.abs(a64 @ v - v * w[None])) / scale < 2e-5
    assert np.max(np.abs(v.T @ v - np.eye(n))) < 2e-5
    want = np.linalg.eigvalsh(a64)
    assert np.max(np.abs(np.sort(w) - want)) / scale < 1e-5


def test_eigh_shift(nt):
    from nt_gb300 import predict
    a = _sym(80, 3, 'psd')
    e0, _ = predict._eigh(torch.from_numpy(a).cuda(), 0.)
    e1, _ = predict._eigh(torch.from_numpy(a).cuda(), 0.25)
    np.testing.assert_allclose(np.sort(e1.cpu().numpy()), np.sort(e0.cpu().numpy()) + 0.25,
                               atol=2e-5)


@pytest.mark.parametrize('kind', range(7))
def test_spectral_weights(nt, kind):
    from nt_gb300 import predict
    rng = np.random.default_rng(kind)
    lam = np.concatenate([rng.uniform(1e-3, 5., 30), [-1e-4, 2e-6]]).astype(np.float32)
    x = rng.standard_normal((32, 3)).astype(np.float32)
    ts = np.array([0.3, 2., 50.])
    got = predict._spectral(torch.from_numpy(lam).cuda(), torch.from_numpy(ts).cuda(), kind,
                            7., torch.from_numpy(x).cuda()).cpu().numpy()
    l64 = lam.astype(np.float64)[:, None]
    pos = np.maximum(l64, 0.)
    for j, t in enumerate(ts):
        e = pos * t / 7.
        w = [np.expm1(-e), np.expm1(-e) / np.abs(l64), pos * np.exp(-2 * e), np.exp(-e),
             -np.expm1(-2 * e) / np.abs(l64), -np.expm1(-e), -np.expm1(-e) / np.abs(l64)][kind]
        np.testing.assert_allclose(got[:, j, :], w * x, rtol=1e-6, atol=1e-30)
