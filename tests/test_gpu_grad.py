"""Gradients of kernel_fn (hand-written adjoints) against central finite
differences of the float64 oracle (h = 1e-3, Richardson-extrapolated: the
difference quotient is then accurate to ~1e-10 relative, far below the float32
rounding of the GPU gradient), the check of the reference's own autodiff tests
(tests/stax/elementwise_test.py:639-732, 782-934). Both the plain float32 and
the mixed form are held to 1e-4 of the largest gradient component."""
import os

import numpy as np
import pytest
import torch

from oracle import nt_oracle as o

pytestmark = pytest.mark.gpu
H = 1e-3


TOL = 1e-4  # of the largest gradient component; the float64 differences are ~1e-10


def fd1(f, x, idx, h):
    xp, xm = x.copy(), x.copy()
    xp[idx] += h
    xm[idx] -= h
    return (f(xp) - f(xm)) / (2 * h)


def fd(f, x, idx, h=H):
    """Central difference with one Richardson step: (4 D(h/2) - D(h)) / 3, error O(h^4)."""
    return (4 * fd1(f, x, idx, h / 2) - fd1(f, x, idx, h)) / 3


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
def test_fcn_hyper_gradients(nt, precision):
    rng = np.random.default_rng(0)
    x = rng.standard_normal((12, 30))
    wq, wt = rng.standard_normal((12, 12)), rng.standard_normal((12, 12))
    hp = np.array([1.3, 0.1, 1.6, 0.15, 1.1, 0.05])  # (W, b) of three Dense layers

    def layers(m, h):
        return [m.Dense(8, h[0], h[1]), m.Relu(), m.Dense(8, h[2], h[3]), m.Erf(),
                m.Dense(1, h[4], h[5])]

    def loss_oracle(h):
        q, t = o.serial(*layers(o, h))(x, None, ('nngp', 'ntk'))
        return float(np.sum(wq * q) + np.sum(wt * t))

    ht = [torch.tensor(v, device='cuda', requires_grad=True) for v in hp]
    q, t = nt.stax.serial(*layers(nt.stax, ht))[2](x, None, ('nngp', 'ntk'),
                                                   precision=precision)
    loss = (torch.from_numpy(wq).float().cuda() * q).sum() + \
        (torch.from_numpy(wt).float().cuda() * t).sum()
    loss.backward()
    got = np.array([v.grad.item() for v in ht])
    want = np.array([fd(loss_oracle, hp, i) for i in range(len(hp))])
    np.testing.assert_allclose(got, want, rtol=TOL, atol=TOL * np.abs(want).max())


@pytest.mark.parametrize('readout', ['flatten', 'gap'])
def test_conv_input_gradients(nt, readout):
    rng = np.random.default_rng(1)
    x1 = rng.standard_normal((2, 6, 6, 2))
    x2 = rng.standard_normal((3, 6, 6, 2))
    wq, wt = rng.standard_normal((2, 3)), rng.standard_normal((2, 3))

    def layers(m):
        ro = m.Flatten() if readout == 'flatten' else m.GlobalAvgPool()
        return [m.Conv(2, (3, 3), padding='SAME', W_std=1.4, b_std=0.1), m.Relu(),
                m.AvgPool((2, 2), (2, 2)), m.Conv(2, (2, 2), padding='SAME', W_std=1.2, b_std=0.2),
                m.Erf(), ro, m.Dense(1, 1.1, 0.05)]

    def loss_oracle(a, b):
        q, t = o.serial(*layers(o))(a, b, ('nngp', 'ntk'))
        return float(np.sum(wq * q) + np.sum(wt * t))

    t1 = torch.tensor(x1, dtype=torch.float32, device='cuda', requires_grad=True)
    t2 = torch.tensor(x2, dtype=torch.float32, device='cuda', requires_grad=True)
    q, t = nt.stax.serial(*layers(nt.stax))[2](t1, t2, ('nngp', 'ntk'))
    loss = (torch.from_numpy(wq).float().cuda() * q).sum() + \
        (torch.from_numpy(wt).float().cuda() * t).sum()
    loss.backward()
    g1, g2 = t1.grad.cpu().numpy(), t2.grad.cpu().numpy()
    scale = max(np.abs(g1).max(), np.abs(g2).max())
    for idx in [(0, 0, 0, 0), (1, 3, 2, 1), (0, 5, 5, 1), (1, 2, 4, 0)]:
        want = fd(lambda a: loss_oracle(a, x2), x1, idx)
        assert abs(g1[idx] - want) < TOL * scale, (idx, g1[idx], want)
    for idx in [(0, 1, 1, 0), (2, 4, 0, 1), (1, 5, 3, 0)]:
        want = fd(lambda b: loss_oracle(x1, b), x2, idx)
        assert abs(g2[idx] - want) < TOL * scale, (idx, g2[idx], want)


def test_symmetric_call_gradient(nt):
    """x2 = None: both factors of every covariance depend on x1."""
    rng = np.random.default_rng(2)
    x = rng.standard_normal((3, 5, 5, 2))
    w = rng.standard_normal((3, 3))

    def layers(m):
        return [m.Conv(1, (3, 3), padding='SAME', W_std=1.3, b_std=0.1), m.Relu(),
                m.GlobalAvgPool(), m.Dense(1, 1.2, 0.1)]

    def loss_oracle(a):
        return float(np.sum(w * o.serial(*layers(o))(a, None, 'ntk')))

    tx = torch.tensor(x, dtype=torch.float32, device='cuda', requires_grad=True)
    k = nt.stax.serial(*layers(nt.stax))[2](tx, None, 'ntk')
    (torch.from_numpy(w).float().cuda() * k).sum().backward()
    g = tx.grad.cpu().numpy()
    for idx in [(0, 0, 0, 0), (1, 2, 3, 1), (2, 4, 4, 0)]:
        want = fd(loss_oracle, x, idx)
        assert abs(g[idx] - want) < TOL * np.abs(g).max(), (idx, g[idx], want)


@pytest.mark.parametrize('arch', ['dense', 'conv'])
@pytest.mark.parametrize('get', ['nngp', 'ntk'])
def test_zero_input_gradient_is_finite(nt, arch, get):
    """tests/stax/elementwise_test.py:949-1036 (issue 123): zero inputs give a finite kernel
    and a zero gradient, for a Dense + Relu network and for the issue's Conv(1, (3, 3)) +
    Relu + Flatten on [1, 8, 8, 3] zeros (the full-spatial rules and their adjoints)."""
    s = nt.stax
    if arch == 'dense':
        x = torch.zeros((2, 4), device='cuda', requires_grad=True)
        kf = s.serial(s.Dense(3, 1., 0.), s.Relu(), s.Dense(1))[2]
    else:
        x = torch.zeros((1, 8, 8, 3), device='cuda', requires_grad=True)
        kf = s.serial(s.Conv(1, (3, 3)), s.Relu(), s.Flatten())[2]
    k = kf(x, x, get)
    assert torch.isfinite(k).all()
    k[0, 0].backward()
    assert torch.isfinite(x.grad).all()
    assert (x.grad == 0).all()


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
def test_nll_hyper_gradients_through_cholesky(nt, precision):
    """NNGP negative log-likelihood of a depth-3 FCN: d/d(W_std, b_std) through the
    layer adjoints and the Cholesky adjoint, against float64 finite differences."""
    import scipy.linalg as sla
    rng = np.random.default_rng(3)
    x = rng.standard_normal((40, 24))
    y = rng.standard_normal((40, 3))
    hp = np.array([1.4, 0.1, 1.6, 0.12, 1.2, 0.08])

    def layers(m, h):
        return [m.Dense(8, h[0], h[1]), m.Relu(), m.Dense(8, h[2], h[3]), m.Relu(),
                m.Dense(1, h[4], h[5])]

    def nll_oracle(h):
        k = o.serial(*layers(o, h))(x, None, 'nngp')
        a = k + 1e-2 * np.trace(k) / 40 * np.eye(40)
        c = sla.cho_factor(a)
        alpha = sla.cho_solve(c, y)
        return 0.5 * np.sum(y * alpha) + 1.5 * 2 * np.sum(np.log(np.diag(c[0]))) + \
            0.5 * 40 * 3 * np.log(2 * np.pi)

    ht = [torch.tensor(v, device='cuda', requires_grad=True) for v in hp]
    k = nt.stax.serial(*layers(nt.stax, ht))[2](x, None, 'nngp', precision=precision)
    nll = nt.predict.negative_log_likelihood(k, y, diag_reg=1e-2)
    assert abs(nll.item() - nll_oracle(hp)) < 1e-5 * abs(nll_oracle(hp))
    nll.backward()
    got = np.array([v.grad.item() for v in ht])
    want = np.array([fd(nll_oracle, hp, i) for i in range(6)])
    np.testing.assert_allclose(got, want, rtol=TOL, atol=TOL * np.abs(want).max())


def test_batched_checkpointed_backward_equals_unbatched(nt):
    """nt.batch with inputs that need grad: per-tile recompute in the backward
    gives the same input gradients as one untiled differentiable evaluation."""
    rng = np.random.default_rng(4)
    xs = torch.tensor(rng.standard_normal((5, 8, 8, 3)), dtype=torch.float32, device='cuda')
    xt = torch.tensor(rng.standard_normal((3, 8, 8, 3)), dtype=torch.float32, device='cuda')
    w = torch.tensor(rng.standard_normal((3, 5)), dtype=torch.float32, device='cuda')
    s = nt.stax
    kf = s.serial(s.Conv(1, (3, 3), padding='SAME', W_std=1.4, b_std=0.), s.Relu(),
                  s.AvgPool((2, 2), (2, 2)), s.Conv(1, (3, 3), padding='SAME', W_std=1.4),
                  s.Relu(), s.GlobalAvgPool(), s.Dense(1, 1.3, 0.))[2]
    a = xs.clone().requires_grad_(True)
    (w * kf(xt, a, 'ntk')).sum().backward()
    b = xs.clone().requires_grad_(True)
    (w * nt.batch(kf, batch_size=2)(xt, b, 'ntk')).sum().backward()
    torch.testing.assert_close(b.grad, a.grad, rtol=1e-4, atol=1e-6)


def test_conv_input_gradients_power_of_two_planes(nt):
    """8 x 8 images: the vectorised activation VJP (C a power of two), the block
    pooling transpose and the stencil-as-its-own-transpose path."""
    rng = np.random.default_rng(4)
    x1 = rng.standard_normal((2, 8, 8, 3))
    x2 = rng.standard_normal((2, 8, 8, 3))
    wq, wt = rng.standard_normal((2, 2)), rng.standard_normal((2, 2))

    def layers(m):
        return [m.Conv(2, (3, 3), padding='SAME', W_std=1.4, b_std=0.1), m.Relu(),
                m.Conv(2, (3, 3), padding='SAME', W_std=1.3, b_std=0.0), m.Relu(),
                m.AvgPool((2, 2), (2, 2)), m.Conv(2, (3, 3), padding='SAME', W_std=1.2, b_std=0.2),
                m.Erf(), m.GlobalAvgPool(), m.Dense(1, 1.1, 0.05)]

    def loss_oracle(a, b):
        q, t = o.serial(*layers(o))(a, b, ('nngp', 'ntk'))
        return float(np.sum(wq * q) + np.sum(wt * t))

    t1 = torch.tensor(x1, dtype=torch.float32, device='cuda', requires_grad=True)
    t2 = torch.tensor(x2, dtype=torch.float32, device='cuda', requires_grad=True)
    q, t = nt.stax.serial(*layers(nt.stax))[2](t1, t2, ('nngp', 'ntk'))
    loss = (torch.from_numpy(wq).float().cuda() * q).sum() + \
        (torch.from_numpy(wt).float().cuda() * t).sum()
    loss.backward()
    g1, g2 = t1.grad.cpu().numpy(), t2.grad.cpu().numpy()
    scale = max(np.abs(g1).max(), np.abs(g2).max())
    for idx in [(0, 0, 0, 0), (1, 3, 2, 1), (0, 7, 7, 2), (1, 4, 5, 0)]:
        want = fd(lambda a: loss_oracle(a, x2), x1, idx)
        assert abs(g1[idx] - want) < TOL * scale, (idx, g1[idx], want)
    for idx in [(0, 1, 1, 0), (1, 6, 0, 2)]:
        want = fd(lambda b: loss_oracle(x1, b), x2, idx)
        assert abs(g2[idx] - want) < TOL * scale, (idx, g2[idx], want)


@pytest.mark.parametrize('kind', ['relu', 'erf', 'sin', 'rbf', 'gelu'])
def test_vectorised_activation_vjp_matches_elementwise_kernel(nt, kind):
    """ntg_act_bwd on 16-byte aligned buffers (chunked kernel with reduced variance
    cotangents) against the same call on buffers offset by one float (the
    elementwise kernel with one atomic per entry)."""
    from nt_gb300 import _lib as L
    g = torch.Generator(device='cuda').manual_seed(11)
    n1, n2, A, C = 2, 3, 8, 8
    shp = (n1 * n2, A, A, C, C)
    cov = torch.rand((n1 + n2, A, A, C, C), device='cuda', generator=g) * 0.2
    # positive diagonal (variances) well above the cross terms
    for a in range(A):
        for c in range(C):
            cov[:, a, a, c, c] += 2.
    v1 = L.Var(cov[:n1].data_ptr(), A * A * C * C, A * C * C + C * C, C + 1)
    v2 = L.Var(cov[n1:].data_ptr(), A * A * C * C, A * C * C + C * C, C + 1)
    act = {'relu': L.Act(L.NTG_ACT_ABRELU, 0., 1., 0., 0, 0.),
           'erf': L.Act(L.NTG_ACT_ERF, 1., 1., 0., 0, 0.),
           'sin': L.Act(L.NTG_ACT_SIN, 1.2, 0.8, float(np.cos(0.6)), 0, 0.),
           'rbf': L.Act(L.NTG_ACT_RBF, 0.7, 0., 0., 0, 0.),
           'gelu': L.Act(L.NTG_ACT_GELU, 0., 0., 0., 0, 0.)}[kind]
    ins = [torch.rand(shp, device='cuda', generator=g) * 2 - 1 for _ in range(4)]

    def run(offset):
        bufs = []
        for x in ins + [None, None]:
            raw = torch.empty(x.numel() + 1 if x is not None else ins[0].numel() + 1, device='cuda')
            v = raw[offset:offset + ins[0].numel()].view(shp)
            if x is not None:
                v.copy_(x)
            bufs.append(v)
        gd1 = torch.zeros((n1, A, C), device='cuda')
        gd2 = torch.zeros((n2, A, C), device='cuda')
        L.call('ntg_act_bwd', L.stream(), L.ptr(bufs[0]), L.ptr(bufs[1]), L.ptr(bufs[2]),
               L.ptr(bufs[3]), L.ptr(bufs[4]), L.ptr(bufs[5]), n1 * n2, n2, A, C, 0, act, v1, v2,
               gd1.data_ptr(), gd2.data_ptr())
        torch.cuda.synchronize()
        return bufs[4].clone(), bufs[5].clone(), gd1, gd2

    fast, slow = run(0), run(1)
    for a, b in zip(fast, slow):
        err = float((a - b).abs().max() / b.abs().max())
        assert err < 2e-5, err


@pytest.mark.parametrize('pairs', [True, False])
def test_input_covariance_adjoint_single_pass(nt, pairs):
    """ntg_input_fs_bwd2 on 32 x 32 planes (one pass over G for both image
    cotangents) against the same call with G offset by one float (the per-side
    kernels), and against a float64 torch contraction."""
    from nt_gb300 import _lib as L
    g = torch.Generator(device='cuda').manual_seed(17)
    n1, n2, A, C, K = 3, 2, 32, 32, 3
    x1 = torch.randn((n1, A, C, K), device='cuda', generator=g)
    x2 = torch.randn((n2, A, C, K), device='cuda', generator=g)
    shp = (n1, n2, A, A, C, C) if pairs else (n1, A, A, C, C)
    G = torch.randn(shp, device='cuda', generator=g)

    def run(offset):
        raw = torch.empty(G.numel() + 1, device='cuda')
        gv = raw[offset:offset + G.numel()].view(shp)
        gv.copy_(G)
        gx1 = torch.zeros_like(x1)
        gx2 = torch.zeros_like(x2)
        L.call('ntg_input_fs_bwd2', L.stream(), L.ptr(gv), L.ptr(x1),
               L.ptr(x2) if pairs else None, L.ptr(gx1), L.ptr(gx2) if pairs else None, n1,
               n2 if pairs else 0, A, C, K)
        torch.cuda.synchronize()
        return gx1, gx2

    fast, slow = run(0), run(1)
    Gd, a, b = G.double(), x1.double(), x2.double()
    if pairs:
        want1 = torch.einsum('ijhHwW,jHWk->ihwk', Gd, b) / K
        want2 = torch.einsum('ijhHwW,ihwk->jHWk', Gd, a) / K
    else:
        want1 = (torch.einsum('ihHwW,iHWk->ihwk', Gd, a) + torch.einsum('ihHwW,ihwk->iHWk', Gd, a)) / K
        want2 = torch.zeros_like(b)
    for got, ref, want in ((fast[0], slow[0], want1), (fast[1], slow[1], want2)):
        scale = float(want.abs().max()) if float(want.abs().max()) > 0 else 1.
        assert float((got.double() - want).abs().max()) / scale < 1e-5
        assert float((got - ref).abs().max()) / scale < 1e-5


def test_batched_symmetric_backward_equals_unbatched(nt):
    """nt.batch(x, None) recomputes each off-diagonal pair of tiles once, with the
    cotangents of both; the input gradient equals one untiled evaluation."""
    rng = np.random.default_rng(6)
    xs = torch.tensor(rng.standard_normal((5, 8, 8, 3)), dtype=torch.float32, device='cuda')
    w = torch.tensor(rng.standard_normal((5, 5)), dtype=torch.float32, device='cuda')
    s = nt.stax
    kf = s.serial(s.Conv(1, (3, 3), padding='SAME', W_std=1.4, b_std=0.1), s.Relu(),
                  s.AvgPool((2, 2), (2, 2)), s.Conv(1, (3, 3), padding='SAME', W_std=1.4),
                  s.Relu(), s.GlobalAvgPool(), s.Dense(1, 1.3, 0.))[2]
    for precision in ('fp32', 'mixed'):
        a = xs.clone().requires_grad_(True)
        (w * kf(a, None, 'ntk', precision=precision)).sum().backward()
        b = xs.clone().requires_grad_(True)
        (w * nt.batch(kf, batch_size=2)(b, None, 'ntk', precision=precision)).sum().backward()
        torch.testing.assert_close(b.grad, a.grad, rtol=1e-4, atol=1e-6)


def test_kernel_ridge_solve_gradients(nt):
    """predict.kernel_ridge_solve (Cholesky kernels, relative diag_reg) and
    predict.matmul: gradients with respect to K, y and the test kernel against
    float64 torch autograd of the same expressions."""
    rng = np.random.default_rng(8)
    n, m, nt_ = 40, 3, 25
    f = rng.standard_normal((n, 60))
    k = torch.tensor(f @ f.T / 60, device='cuda')
    y = torch.tensor(rng.standard_normal((n, m)), device='cuda')
    kt = torch.tensor(rng.standard_normal((nt_, n)), device='cuda')
    yt = torch.tensor(rng.standard_normal((nt_, m)), device='cuda')

    def loss64(kk, yy, ktt):
        a = kk + 1e-2 * torch.trace(kk) / n * torch.eye(n, device='cuda', dtype=kk.dtype)
        alpha = torch.linalg.solve(a, yy)
        return ((yt.double() - ktt @ alpha) ** 2).sum()

    leaves64 = [v.double().clone().requires_grad_(True) for v in (k, y, kt)]
    loss64(*leaves64).backward()
    leaves = [v.float().clone().requires_grad_(True) for v in (k, y, kt)]
    alpha = nt.predict.kernel_ridge_solve(leaves[0], leaves[1], diag_reg=1e-2)
    loss = ((yt.float() - nt.predict.matmul(leaves[2], alpha)) ** 2).sum()
    loss.backward()
    for got, want in zip(leaves, leaves64):
        err = float((got.grad.double() - want.grad).abs().max() / want.grad.abs().max())
        assert err < 1e-4, err


def test_autotuned_recompute_tile(nt, tmp_path, monkeypatch):
    """tune.recompute_tile picks one of its candidates from timed probes, caches it,
    and the batched backward with the tuned tile equals one with an explicit tile."""
    import importlib
    monkeypatch.setenv('NT_GB300_TUNE_CACHE', str(tmp_path / 'tune.json'))
    tune = importlib.reload(nt.tune)
    s = nt.stax
    kf = s.serial(s.Conv(1, (3, 3), padding='SAME', W_std=1.4), s.Relu(),
                  s.AvgPool((2, 2), (2, 2)), s.Conv(1, (3, 3), padding='SAME', W_std=1.4),
                  s.Relu(), s.GlobalAvgPool(), s.Dense(1, 1.3, 0.))[2]
    t = tune.recompute_tile(kf, (1, 8, 8, 3), 'fp32', candidates=(2, 4, 8))
    assert t in (2, 4, 8)
    assert os.path.exists(tmp_path / 'tune.json')
    assert tune.recompute_tile(kf, (1, 8, 8, 3), 'fp32', candidates=(2, 4, 8)) == t
    rng = np.random.default_rng(9)
    xs = torch.tensor(rng.standard_normal((9, 8, 8, 3)), dtype=torch.float32, device='cuda')
    xt = torch.tensor(rng.standard_normal((5, 8, 8, 3)), dtype=torch.float32, device='cuda')
    grads = []
    for tile in (None, 3):
        a = xs.clone().requires_grad_(True)
        nt.batch(kf, batch_size=8, recompute_tile=tile)(xt, a, 'ntk').sum().backward()
        grads.append(a.grad)
    torch.testing.assert_close(grads[0], grads[1], rtol=1e-4, atol=1e-6)
    tune.clear()


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
def test_conv_act_pool_fused_gradients_32x32(nt, precision):
    """32 x 32 images: conv + ReLU (+ AvgPool) fused in one pass (ConvActFn with
    ntg_conv_act_fs and ntg_act_pool_bwd) against central finite differences of the
    float64 oracle."""
    rng = np.random.default_rng(14)
    x1 = rng.standard_normal((1, 32, 32, 2))
    x2 = rng.standard_normal((2, 32, 32, 2))
    wq, wt = rng.standard_normal((1, 2)), rng.standard_normal((1, 2))

    def layers(m):
        return [m.Conv(1, (3, 3), padding='SAME', W_std=1.4, b_std=0.1), m.Relu(),
                m.Conv(1, (3, 3), padding='SAME', W_std=1.3, b_std=0.0), m.Relu(),
                m.AvgPool((2, 2), (2, 2)), m.Conv(1, (3, 3), padding='SAME', W_std=1.2),
                m.Erf(), m.GlobalAvgPool(), m.Dense(1, 1.1, 0.05)]

    def loss_oracle(a, b):
        q, t = o.serial(*layers(o))(a, b, ('nngp', 'ntk'))
        return float(np.sum(wq * q) + np.sum(wt * t))

    t1 = torch.tensor(x1, dtype=torch.float32, device='cuda', requires_grad=True)
    t2 = torch.tensor(x2, dtype=torch.float32, device='cuda', requires_grad=True)
    q, t = nt.stax.serial(*layers(nt.stax))[2](t1, t2, ('nngp', 'ntk'), precision=precision)
    loss = (torch.from_numpy(wq).float().cuda() * q).sum() + \
        (torch.from_numpy(wt).float().cuda() * t).sum()
    loss.backward()
    g1, g2 = t1.grad.cpu().numpy(), t2.grad.cpu().numpy()
    scale = max(np.abs(g1).max(), np.abs(g2).max())
    for idx in [(0, 0, 0, 0), (0, 13, 21, 1), (0, 31, 31, 0)]:
        want = fd(lambda a: loss_oracle(a, x2), x1, idx)
        assert abs(g1[idx] - want) < TOL * scale, (idx, g1[idx], want)
    for idx in [(1, 7, 30, 1)]:
        want = fd(lambda b: loss_oracle(x1, b), x2, idx)
        assert abs(g2[idx] - want) < TOL * scale, (idx, g2[idx], want)


def _rare(m, kind):
    return {'sin': lambda: m.Sin(1.2, 0.8, 0.3), 'cos': lambda: m.Cos(1.0, 1.1, 0.2),
            'rbf': lambda: m.Rbf(0.7), 'gelu': lambda: m.Gelu()}[kind]()


@pytest.mark.parametrize('kind', ['sin', 'cos', 'rbf', 'gelu'])
def test_rare_activation_fcn_gradients(nt, kind):
    """Sin / Cos / Rbf / Gelu adjoints (elementwise kernel) in a Dense network:
    d/d(W_std, b_std) and d/dx against central finite differences of the oracle."""
    rng = np.random.default_rng(21)
    x = rng.standard_normal((5, 12)) * 0.8
    wq, wt = rng.standard_normal((5, 5)), rng.standard_normal((5, 5))
    hp = np.array([1.2, 0.1, 0.9, 0.2, 1.1, 0.05])

    def layers(m, h):
        return [m.Dense(8, h[0], h[1]), _rare(m, kind), m.Dense(8, h[2], h[3]), _rare(m, kind),
                m.Dense(1, h[4], h[5])]

    def loss_oracle(h, xx):
        q, t = o.serial(*layers(o, h))(xx, None, ('nngp', 'ntk'))
        return float(np.sum(wq * q) + np.sum(wt * t))

    ht = [torch.tensor(v, device='cuda', requires_grad=True) for v in hp]
    xt = torch.tensor(x, dtype=torch.float32, device='cuda', requires_grad=True)
    q, t = nt.stax.serial(*layers(nt.stax, ht))[2](xt, None, ('nngp', 'ntk'))
    loss = (torch.from_numpy(wq).float().cuda() * q).sum() + \
        (torch.from_numpy(wt).float().cuda() * t).sum()
    loss.backward()
    got = np.array([v.grad.item() for v in ht])
    want = np.array([fd(lambda h: loss_oracle(h, x), hp, i) for i in range(len(hp))])
    np.testing.assert_allclose(got, want, rtol=TOL, atol=TOL * np.abs(want).max())
    gx = xt.grad.cpu().numpy()
    scale = np.abs(gx).max()
    for idx in [(0, 0), (2, 7), (4, 11)]:
        wx = fd(lambda xx: loss_oracle(hp, xx), x, idx)
        assert abs(gx[idx] - wx) < TOL * scale, (idx, gx[idx], wx)


@pytest.mark.parametrize('kind', ['sin', 'rbf', 'gelu'])
def test_rare_activation_conv_gradients(nt, kind):
    """8 x 8 images: the chunked activation VJP with the rare rules compiled in, its
    AvgPool-composed form and, at 4 x 4, the elementwise kernel."""
    rng = np.random.default_rng(22)
    x1 = rng.standard_normal((2, 8, 8, 2)) * 0.7
    x2 = rng.standard_normal((1, 8, 8, 2)) * 0.7
    wq, wt = rng.standard_normal((2, 1)), rng.standard_normal((2, 1))

    def layers(m):
        return [m.Conv(2, (3, 3), padding='SAME', W_std=1.2, b_std=0.1), _rare(m, kind),
                m.Conv(2, (3, 3), padding='SAME', W_std=1.1, b_std=0.0), _rare(m, kind),
                m.AvgPool((2, 2), (2, 2)), m.Conv(2, (3, 3), padding='SAME', W_std=1.0, b_std=0.2),
                _rare(m, kind), m.GlobalAvgPool(), m.Dense(1, 1.1, 0.05)]

    def loss_oracle(a, b):
        q, t = o.serial(*layers(o))(a, b, ('nngp', 'ntk'))
        return float(np.sum(wq * q) + np.sum(wt * t))

    t1 = torch.tensor(x1, dtype=torch.float32, device='cuda', requires_grad=True)
    t2 = torch.tensor(x2, dtype=torch.float32, device='cuda', requires_grad=True)
    q, t = nt.stax.serial(*layers(nt.stax))[2](t1, t2, ('nngp', 'ntk'))
    loss = (torch.from_numpy(wq).float().cuda() * q).sum() + \
        (torch.from_numpy(wt).float().cuda() * t).sum()
    loss.backward()
    g1, g2 = t1.grad.cpu().numpy(), t2.grad.cpu().numpy()
    scale = max(np.abs(g1).max(), np.abs(g2).max())
    for idx in [(0, 0, 0, 0), (1, 3, 2, 1), (0, 7, 7, 1)]:
        want = fd(lambda a: loss_oracle(a, x2), x1, idx)
        assert abs(g1[idx] - want) < TOL * scale, (idx, g1[idx], want)
    for idx in [(0, 4, 5, 0)]:
        want = fd(lambda b: loss_oracle(x1, b), x2, idx)
        assert abs(g2[idx] - want) < TOL * scale, (idx, g2[idx], want)


def test_diagonal_spatial_gradients(nt):
    """A CNN without pooling (Flatten readout) runs on diagonal-spatial kernels; its
    gradients (input covariance, conv and activation adjoints in the diagonal layout) match
    central finite differences of the oracle and the full-spatial gradients."""
    rng = np.random.default_rng(23)
    x1 = rng.standard_normal((2, 6, 5, 2))
    x2 = rng.standard_normal((3, 6, 5, 2))
    wq, wt = rng.standard_normal((2, 3)), rng.standard_normal((2, 3))

    def layers(m, w=1.3):
        return [m.Conv(2, (3, 3), padding='SAME', W_std=w, b_std=0.2), m.Erf(),
                m.Conv(2, (2, 2), padding='VALID', W_std=1.1, b_std=0.1), m.Relu(),
                m.Conv(2, (3, 3), strides=(2, 1), padding='SAME', W_std=1.2), m.Gelu(),
                m.Flatten(), m.Dense(1, 1.2, 0.05)]

    kf = nt.stax.serial(*layers(nt.stax))[2]
    assert bool(kf.diagonal)

    def loss_oracle(a, b):
        q, t = o.serial(*layers(o))(a, b, ('nngp', 'ntk'))
        return float(np.sum(wq * q) + np.sum(wt * t))

    def grads(ds):
        w = torch.tensor(1.3, device='cuda', requires_grad=True)
        t1 = torch.tensor(x1, dtype=torch.float32, device='cuda', requires_grad=True)
        t2 = torch.tensor(x2, dtype=torch.float32, device='cuda', requires_grad=True)
        f = nt.stax.serial(*layers(nt.stax, w))[2]
        q, t = f(t1, t2, ('nngp', 'ntk'), diagonal_spatial=ds)
        loss = (torch.from_numpy(wq).float().cuda() * q).sum() + \
            (torch.from_numpy(wt).float().cuda() * t).sum()
        loss.backward()
        return t1.grad.cpu().numpy(), t2.grad.cpu().numpy(), w.grad.item()

    g1, g2, gw = grads(None)
    f1, f2, fw = grads(False)
    scale = max(np.abs(g1).max(), np.abs(g2).max())
    np.testing.assert_allclose(g1, f1, rtol=0, atol=2e-5 * scale)
    np.testing.assert_allclose(g2, f2, rtol=0, atol=2e-5 * scale)
    assert abs(gw - fw) < 2e-5 * abs(fw)
    for idx in [(0, 0, 0, 0), (1, 3, 2, 1), (0, 5, 4, 1)]:
        want = fd(lambda a: loss_oracle(a, x2), x1, idx)
        assert abs(g1[idx] - want) < TOL * scale, (idx, g1[idx], want)
    for idx in [(2, 4, 1, 0)]:
        want = fd(lambda b: loss_oracle(x1, b), x2, idx)
        assert abs(g2[idx] - want) < TOL * scale, (idx, g2[idx], want)


def test_diagonal_spatial_output_gradients(nt):
    """kernel_fn(..., diagonal_spatial=True) without a readout returns [N1, N2, H, W]
    kernels; their gradients equal those of the diagonal of the full-spatial kernels, and
    the symmetric call differentiates through the shared input."""
    rng = np.random.default_rng(24)
    x = rng.standard_normal((3, 5, 4, 3))
    w = rng.standard_normal((3, 3, 5, 4))
    s = nt.stax
    kf = s.serial(s.Conv(2, (3, 3), padding='SAME', W_std=1.4, b_std=0.1), s.Relu(),
                  s.Conv(2, (3, 3), padding='SAME', W_std=1.2), s.Sin(1.1, 0.9, 0.2))[2]
    wt = torch.from_numpy(w).float().cuda()

    def grad(ds):
        t = torch.tensor(x, dtype=torch.float32, device='cuda', requires_grad=True)
        q, n = kf(t, None, ('nngp', 'ntk'), diagonal_spatial=ds)
        if not ds:  # [N1, N2, H, H, W, W] -> its (h, h, w, w) entries
            q = torch.einsum('abhhww->abhw', q)
            n = torch.einsum('abhhww->abhw', n)
        assert q.shape == (3, 3, 5, 4)
        ((wt * q).sum() + (wt * n).sum()).backward()
        return t.grad.cpu().numpy()

    gd, gf = grad(True), grad(False)
    np.testing.assert_allclose(gd, gf, rtol=0, atol=2e-5 * np.abs(gf).max())


@pytest.mark.parametrize('pooled', [False, True])
@pytest.mark.parametrize('zero_t', [False, True])
def test_fused_conv_act_backward_matches_two_kernels(nt, pooled, zero_t):
    """ntg_conv_act_bwd (activation VJP fused into the conv transpose) against the
    activation VJP kernel followed by the transposed stencil: the image-side cotangents are
    bit-identical, the variance cotangents equal up to the order of their sums."""
    from nt_gb300 import _lib as L, _ops as O
    g = torch.Generator(device='cuda').manual_seed(5)
    n1, n2, A = 2, 3, 32
    shp = (n1 * n2, A, A, A, A)
    cov = torch.rand((n1 + n2, A, A, A, A), device='cuda', generator=g) * 0.2
    for a in range(A):
        cov[:, a, a, :, :].diagonal(dim1=-2, dim2=-1).add_(2.)
    sa = A * A * A + A * A
    v1 = L.Var(cov[:n1].data_ptr(), A ** 4, sa, A + 1)
    v2 = L.Var(cov[n1:].data_ptr(), A ** 4, sa, A + 1)
    act = L.Act(L.NTG_ACT_ABRELU, 0., 1., 0., 0, 0.)
    pre_q = torch.rand(shp, device='cuda', generator=g) * 2 - 1
    pre_t = torch.rand(shp, device='cuda', generator=g)
    gshape = (n1 * n2, 16, 16, 16, 16) if pooled else shp
    gq = torch.rand(gshape, device='cuda', generator=g) - 0.5
    gt = torch.rand(gshape, device='cuda', generator=g) - 0.5
    w2 = 2.0
    gin_q = torch.empty(shp, device='cuda')
    gin_t = None if zero_t else torch.empty(shp, device='cuda')
    gd1, gd2 = torch.zeros((n1, A, A), device='cuda'), torch.zeros((n2, A, A), device='cuda')
    L.call('ntg_conv_act_bwd', L.stream(), L.ptr(pre_q), L.ptr(pre_t), L.ptr(gq), L.ptr(gt),
           int(pooled), L.ptr(gin_q), None if gin_t is None else L.ptr(gin_t), n1 * n2, n2, A,
           w2, act, v1, v2, gd1.data_ptr(), gd2.data_ptr())
    oq, ot = torch.empty(shp, device='cuda'), torch.empty(shp, device='cuda')
    hd1, hd2 = torch.zeros((n1, A, A), device='cuda'), torch.zeros((n2, A, A), device='cuda')
    if pooled:
        L.call('ntg_act_pool_bwd', L.stream(), L.ptr(pre_q), L.ptr(pre_t), L.ptr(gq), L.ptr(gt),
               L.ptr(oq), L.ptr(ot), n1 * n2, n2, A, A, act, v1, v2, hd1.data_ptr(),
               hd2.data_ptr())
    else:
        L.call('ntg_act_bwd', L.stream(), L.ptr(pre_q), L.ptr(pre_t), L.ptr(gq), L.ptr(gt),
               L.ptr(oq), L.ptr(ot), n1 * n2, n2, A, A, 0, act, v1, v2, hd1.data_ptr(),
               hd2.data_ptr())
    six = (n1, n2, A, A, A, A)
    want_t, want_q = O.conv_fs(ot.view(six), oq.view(six), n1 * n2, n2, A, A, 3, 3, 1, 1, 1, 1,
                               A, A, False, O.affine(w2, 0., w2, w2, 0., False), O.NO_ACT,
                               O.NO_VAR, O.NO_VAR, True, (n1, n2))
    torch.cuda.synchronize()
    L.check_device('ntg_conv_act_bwd')  # no bounded wait of the bulk-copy ring ran out
    assert torch.equal(gin_q, want_q.reshape(shp))
    if gin_t is not None:
        assert torch.equal(gin_t, want_t.reshape(shp))
    for a, b in ((gd1, hd1), (gd2, hd2)):
        assert float((a - b).abs().max() / b.abs().max()) < 1e-5


def test_fused_conv_act_backward_in_network(nt):
    """A 32 x 32 conv net's input gradients through the fused backward (W_std plain floats)
    equal those through the unfused rules (W_std tensors that need gradients)."""
    rng = np.random.default_rng(25)
    x1 = rng.standard_normal((2, 32, 32, 3))
    x2 = rng.standard_normal((2, 32, 32, 3))
    wq, wt = rng.standard_normal((2, 2)), rng.standard_normal((2, 2))
    s = nt.stax

    def grads(hyper):
        ws = [torch.tensor(v, device='cuda', requires_grad=True) if hyper else v
              for v in (1.4, 1.3, 1.2)]
        net = s.serial(s.Conv(1, (3, 3), padding='SAME', W_std=ws[0], b_std=0.1), s.Relu(),
                       s.Conv(1, (3, 3), padding='SAME', W_std=ws[1]), s.Relu(),
                       s.AvgPool((2, 2), (2, 2)), s.Conv(1, (3, 3), padding='SAME', W_std=ws[2]),
                       s.Relu(), s.GlobalAvgPool(), s.Dense(1, 1.1, 0.05))[2]
        t1 = torch.tensor(x1, dtype=torch.float32, device='cuda', requires_grad=True)
        t2 = torch.tensor(x2, dtype=torch.float32, device='cuda', requires_grad=True)
        q, t = net(t1, t2, ('nngp', 'ntk'))
        ((torch.from_numpy(wq).float().cuda() * q).sum() +
         (torch.from_numpy(wt).float().cuda() * t).sum()).backward()
        return t1.grad.cpu().numpy(), t2.grad.cpu().numpy()

    f1, f2 = grads(False)
    u1, u2 = grads(True)
    scale = max(np.abs(u1).max(), np.abs(u2).max())
    np.testing.assert_allclose(f1, u1, rtol=0, atol=1e-5 * scale)
    np.testing.assert_allclose(f2, u2, rtol=0, atol=1e-5 * scale)


def test_input_conv_act_fused_forward_and_backward(nt):
    """The first conv + ReLU of a 32 x 32 net computed from the images (ntg_input_conv_act_fs)
    gives the layer-by-layer kernels bit for bit, and its gradients equal those of the unfused
    rules (W_std a tensor that needs a gradient) and central differences of the oracle."""
    from nt_gb300 import _lib as L, _ops as O, stax
    rng = np.random.default_rng(26)
    x1 = rng.standard_normal((2, 32, 32, 3)).astype(np.float32)
    x2 = rng.standard_normal((3, 32, 32, 3)).astype(np.float32)
    t1, t2 = torch.from_numpy(x1).cuda(), torch.from_numpy(x2).cuda()
    aff = O.affine(2.0, 0.01, 2.0)
    act = L.Act(L.NTG_ACT_ABRELU, 0., 1., 0., 0, 0.)
    cv1 = O.conv_fs(O.input_fs(t1, None), None, 2, 0, 32, 32, 3, 3, 1, 1, 1, 1, 32, 32, False, aff,
                    O.NO_ACT, O.NO_VAR, O.NO_VAR, False, (2,))[0]
    cv2 = O.conv_fs(O.input_fs(t2, None), None, 3, 0, 32, 32, 3, 3, 1, 1, 1, 1, 32, 32, False, aff,
                    O.NO_ACT, O.NO_VAR, O.NO_VAR, False, (3,))[0]
    v1, v2 = O.var_view(cv1, False), O.var_view(cv2, False)
    shape = (2, 3, 32, 32, 32, 32)
    qa, ta, pre = (torch.empty(shape, device='cuda') for _ in range(3))
    L.call('ntg_input_conv_act_fs', L.stream(), L.ptr(t1), L.ptr(t2), 2, 3, 3, L.ptr(qa),
           L.ptr(ta), L.ptr(pre), aff, act, v1, v2)
    g = O.input_fs(t1, t2)
    wq, wt, pq, pt = (torch.empty(shape, device='cuda') for _ in range(4))
    L.call('ntg_conv_act_fs', L.stream(), L.ptr(g), None, L.ptr(wq), L.ptr(wt), L.ptr(pq),
           L.ptr(pt), 6, 3, 32, 32, aff, act, v1, v2)
    torch.cuda.synchronize()
    assert torch.equal(qa, wq) and torch.equal(ta, wt)
    assert torch.equal(pre, pq) and torch.equal(pre, pt)

    wq_, wt_ = rng.standard_normal((2, 3)), rng.standard_normal((2, 3))

    def layers(m, w):
        return [m.Conv(1, (3, 3), padding='SAME', W_std=w, b_std=0.1), m.Relu(),
                m.AvgPool((2, 2), (2, 2)), m.Conv(1, (3, 3), padding='SAME', W_std=1.2),
                m.Relu(), m.GlobalAvgPool(), m.Dense(1, 1.1, 0.)]

    def grads(hyper):
        w = torch.tensor(1.4, device='cuda', requires_grad=True) if hyper else 1.4
        a = torch.tensor(x1, device='cuda', requires_grad=True)
        b = torch.tensor(x2, device='cuda', requires_grad=True)
        q, t = stax.serial(*layers(stax, w))[2](a, b, ('nngp', 'ntk'))
        ((torch.from_numpy(wq_).float().cuda() * q).sum() +
         (torch.from_numpy(wt_).float().cuda() * t).sum()).backward()
        return a.grad.cpu().numpy(), b.grad.cpu().numpy(), q.detach().cpu().numpy()

    f1, f2, fq = grads(False)
    u1, u2, uq = grads(True)
    # W_std given as a float is squared in double, as a tensor in float32: W^2 may differ by an ulp
    np.testing.assert_allclose(fq, uq, rtol=1e-6)
    scale = max(np.abs(u1).max(), np.abs(u2).max())
    np.testing.assert_allclose(f1, u1, rtol=0, atol=1e-5 * scale)
    np.testing.assert_allclose(f2, u2, rtol=0, atol=1e-5 * scale)
    x1d, x2d = x1.astype(np.float64), x2.astype(np.float64)

    def loss_oracle(a, b):
        q, t = o.serial(*layers(o, 1.4))(a, b, ('nngp', 'ntk'))
        return float(np.sum(wq_ * q) + np.sum(wt_ * t))

    for idx in [(0, 0, 0, 0), (1, 17, 9, 2)]:
        want = fd(lambda a: loss_oracle(a, x2d), x1d, idx)
        assert abs(f1[idx] - want) < TOL * scale, (idx, f1[idx], want)


@pytest.mark.parametrize('has_t', [False, True])
def test_conv_act_pool_forward_matches_two_kernels(nt, has_t):
    """ntg_conv_act_pool_fs (conv + ReLU with the pool's window sums taken in the kernel)
    equals ntg_conv_act_fs followed by ntg_pool bit for bit, pre-activations included."""
    from nt_gb300 import _lib as L, _ops as O
    g = torch.Generator(device='cuda').manual_seed(6)
    n1, n2, A = 2, 2, 32
    shp = (n1 * n2, A, A, A, A)
    cov = torch.rand((n1 + n2, A, A, A, A), device='cuda', generator=g) * 0.2
    for a in range(A):
        cov[:, a, a, :, :].diagonal(dim1=-2, dim2=-1).add_(2.)
    sa = A * A * A + A * A
    v1 = L.Var(cov[:n1].data_ptr(), A ** 4, sa, A + 1)
    v2 = L.Var(cov[n1:].data_ptr(), A ** 4, sa, A + 1)
    act = L.Act(L.NTG_ACT_ABRELU, 0., 1., 0., 0, 0.)
    aff = O.affine(2.0, 0.05, 2.0)
    q = torch.rand(shp, device='cuda', generator=g) * 2 - 1
    t = torch.rand(shp, device='cuda', generator=g) if has_t else None
    pshape = (n1 * n2, 16, 16, 16, 16)
    oq, ot = torch.empty(pshape, device='cuda'), torch.empty(pshape, device='cuda')
    pq, pt = torch.empty(shp, device='cuda'), torch.empty(shp, device='cuda')
    hq = torch.empty((n1 * n2, A, A, 16, 16), device='cuda')
    ht = torch.empty_like(hq)
    L.call('ntg_conv_act_pool_fs', L.stream(), L.ptr(q), None if t is None else L.ptr(t),
           L.ptr(oq), L.ptr(ot), L.ptr(pq), L.ptr(pt), L.ptr(hq), L.ptr(ht), n1 * n2, n2, A, aff,
           act, v1, v2)
    aq, at = torch.empty(shp, device='cuda'), torch.empty(shp, device='cuda')
    rq, rt = torch.empty(shp, device='cuda'), torch.empty(shp, device='cuda')
    L.call('ntg_conv_act_fs', L.stream(), L.ptr(q), None if t is None else L.ptr(t), L.ptr(aq),
           L.ptr(at), L.ptr(rq), L.ptr(rt), n1 * n2, n2, A, A, aff, act, v1, v2)
    want_q = O.pool(aq, n1 * n2, A, A, 2, 2, 2, 2, 0, 0, 16, 16, False, False, True, False, pshape)
    want_t = O.pool(at, n1 * n2, A, A, 2, 2, 2, 2, 0, 0, 16, 16, False, False, True, False, pshape)
    torch.cuda.synchronize()
    assert torch.equal(pq, rq) and torch.equal(pt, rt)
    assert torch.equal(oq, want_q) and torch.equal(ot, want_t)


def test_nll_hyper_gradients_ill_conditioned(nt):
    """The NLL gradient of the FCN configuration (x [256, 784] on the sphere of radius sqrt(784),
    diag_reg 1e-4): the self pairs sit at correlation 1, where the activation VJP must see
    var1 var2 - q^2 == 0 exactly (the _sqrt convention cuts the singular term); a rounding
    residue there is amplified by the ill-conditioned solve."""
    import scipy.linalg as sla
    rng = np.random.default_rng(4)
    x = rng.standard_normal((256, 784))
    x *= np.sqrt(784) / np.linalg.norm(x, axis=1, keepdims=True)
    y = np.eye(10)[rng.integers(0, 10, 256)]
    hp = np.array([1.5, 0.05])

    def layers(m, w, b):
        return [m.Dense(512, w, b), m.Relu(), m.Dense(512, w, b), m.Relu(), m.Dense(1, w, b)]

    def nll_oracle(h):
        k = o.serial(*layers(o, h[0], h[1]))(x, None, 'nngp')
        a = k + 1e-4 * np.trace(k) / 256 * np.eye(256)
        c = sla.cho_factor(a)
        alpha = sla.cho_solve(c, y)
        # 0.5 y^T A^-1 y + (10 / 2) log det A, log det A = 2 sum log diag(L)
        return 0.5 * np.sum(y * alpha) + 10 * np.sum(np.log(np.diag(c[0]))) + \
            0.5 * 256 * 10 * np.log(2 * np.pi)

    w = torch.tensor(hp[0], device='cuda', requires_grad=True)
    b = torch.tensor(hp[1], device='cuda', requires_grad=True)
    k = nt.stax.serial(*layers(nt.stax, w, b))[2](x, None, 'nngp')
    nt.predict.negative_log_likelihood(k, y, diag_reg=1e-4).backward()
    got = np.array([w.grad.item(), b.grad.item()])
    want = np.array([fd(nll_oracle, hp, i, h=1e-4) for i in range(2)])
    np.testing.assert_allclose(got, want, rtol=2e-2, atol=2e-2 * np.abs(want).max())


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
def test_kernel_ridge_input_gradients_myrtle5_vs_float64(nt, precision):
    """The support-set gradient of the Myrtle-5 kernel-ridge loss (configuration 5 at
    x_s [2], x_t [3]): ||y_t - K_ts (K_ss + 1e-6 tr(K_ss)/n I)^-1 y_s||^2 through nt.batch's
    checkpointed tiles, the fused 32 x 32 adjoints and the solve adjoint, against float64
    finite differences of the oracle."""
    rng = np.random.default_rng(21)
    xs = rng.standard_normal((2, 32, 32, 3))
    xt = rng.standard_normal((3, 32, 32, 3))
    ys = np.eye(10)[rng.integers(0, 10, 2)]
    yt = np.eye(10)[rng.integers(0, 10, 3)]

    def layers(m):
        conv = lambda: m.Conv(1, (3, 3), padding='SAME', W_std=2 ** .5, b_std=0.)
        return [conv(), m.Relu(), conv(), m.Relu(), m.AvgPool((2, 2), (2, 2)), conv(), m.Relu(),
                m.AvgPool((2, 2), (2, 2)), conv(), m.Relu()] + \
            [m.AvgPool((2, 2), (2, 2))] * 3 + [m.Flatten(), m.Dense(10, 2 ** .5, 0.)]

    kfo = o.serial(*layers(o))

    def loss_oracle(a):
        kss = kfo(a, None, 'ntk')
        kts = kfo(xt, a, 'ntk')
        lam = 1e-6 * np.trace(kss) / kss.shape[0]
        alpha = np.linalg.solve(kss + lam * np.eye(kss.shape[0]), ys)
        return float(np.sum((yt - kts @ alpha) ** 2))

    kf = nt.stax.serial(*layers(nt.stax))[2]
    a = torch.tensor(xs, dtype=torch.float32, device='cuda', requires_grad=True)
    tt = torch.tensor(xt, dtype=torch.float32, device='cuda')
    batched = nt.batch(kf, batch_size=2)
    kss = batched(a, None, 'ntk', precision=precision)
    kts = batched(tt, a, 'ntk', precision=precision)
    alpha = nt.predict.kernel_ridge_solve(kss, torch.tensor(ys, dtype=torch.float32).cuda(),
                                          diag_reg=1e-6)
    ytt = torch.tensor(yt, dtype=torch.float32).cuda()
    loss = ((ytt - nt.predict.matmul(kts, alpha)) ** 2).sum()
    assert abs(loss.item() - loss_oracle(xs)) < 1e-5 * abs(loss_oracle(xs))
    loss.backward()
    g = a.grad.cpu().numpy()
    scale = np.abs(g).max()
    for idx in [(0, 0, 0, 0), (1, 17, 9, 2)]:
        want = fd(loss_oracle, xs, idx)
        assert abs(g[idx] - want) < TOL * scale, (idx, g[idx], want)
