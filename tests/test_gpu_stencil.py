"""The materialised 3x3 full-spatial stencil (conv + affine + ABRelu epilogue)
on 32 x 32 planes against a float64 torch statement of the same rule
(linear.py:3341-3378 stencil, linear.py:1394-1398 affine, elementwise.py:447-455
ABRelu), at every ring depth of the streamed kernel.

Tolerance: 1e-5 of the largest entry (plain FP32 against float64); the ring depth
only changes the launch, so results for different depths are bit-identical.
"""
import math

import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def stencil64(x):
    """(1/9) sum_{d,e in -1..1} x[b, h+d, h'+d, w+e, w'+e], zero outside (SAME)."""
    b, a, _, c, _ = x.shape
    p = torch.nn.functional.pad(x, (1, 1, 1, 1, 1, 1, 1, 1))
    out = torch.zeros_like(x)
    for d in (-1, 0, 1):
        for e in (-1, 0, 1):
            out += p[:, 1 + d:1 + d + a, 1 + d:1 + d + a, 1 + e:1 + e + c, 1 + e:1 + e + c]
    return out / 9.


def reference(q, t, var, w2, b2, relu):
    q, t, var = q.double(), (None if t is None else t.double()), var.double()
    sq = stencil64(q)
    qn = w2 * sq + b2
    tn = qn if t is None else w2 * stencil64(t) + qn
    if not relu:
        return qn, tn
    v1 = var[:, :, None, :, None]          # (h, w) of sample i1 = b
    v2 = var[0][None, None, :, None, :]    # (h', w') of sample i2 = 0 (n2 = 1)
    s = torch.sqrt(torch.clamp(v1 * v2 - qn * qn, min=0.))
    th = torch.atan2(s, qn)
    dot = (math.pi - th) / (2 * math.pi)
    return s / (2 * math.pi) + dot * qn, tn * dot


def run(nt, q, t, var, w2, b2, relu, want_t=True):
    from nt_gb300 import _lib as L, _ops as O
    B = q.shape[0]
    v = L.Var(var.data_ptr(), 32 * 32, 32, 1)
    act = L.Act(L.NTG_ACT_ABRELU if relu else L.NTG_ACT_NONE, 0., 1., 0., 0, 0.)
    outs = O.conv_fs(q, t, B, 1, 32, 32, 3, 3, 1, 1, 1, 1, 32, 32, False, O.affine(w2, b2, w2),
                     act, v, v, want_t, (B,))
    torch.cuda.synchronize()
    assert L.load().ntg_device_status() == 0
    return outs


@pytest.mark.parametrize('has_t', [True, False])
@pytest.mark.parametrize('relu', [True, False])
def test_stencil32_matches_float64(nt, has_t, relu):
    g = torch.Generator(device='cuda').manual_seed(3)
    B = 3
    q = torch.rand((B, 32, 32, 32, 32), device='cuda', generator=g)
    t = torch.rand_like(q) if has_t else None
    var = torch.rand((B, 32, 32), device='cuda', generator=g) + 2.
    oq, ot = run(nt, q, t, var, 1.3, 0.05, relu)
    wq, wt = reference(q, t, var, 1.3, 0.05, relu)
    for got, want in ((oq, wq), (ot, wt)):
        err = (got.double() - want).abs().max() / want.abs().max()
        assert float(err) < RTOL


def test_stencil32_ring_depths_bit_identical(nt):
    from nt_gb300 import _lib as L
    lib = L.load()
    g = torch.Generator(device='cuda').manual_seed(5)
    B = 4
    q = torch.rand((B, 32, 32, 32, 32), device='cuda', generator=g)
    t = torch.rand_like(q)
    var = torch.rand((B, 32, 32), device='cuda', generator=g) + 2.
    base = None
    try:
        for ring in (2, 3, 4, 6):
            assert lib.ntg_tune_set(L.NTG_TUNE_STENCIL_RING, ring) == 0
            oq, ot = run(nt, q, t, var, 2., 0., True)
            if base is None:
                base = (oq, ot)
            else:
                assert torch.equal(oq, base[0]) and torch.equal(ot, base[1])
    finally:
        lib.ntg_tune_set(L.NTG_TUNE_STENCIL_RING, 4)


def test_stencil32_nngp_only(nt):
    g = torch.Generator(device='cuda').manual_seed(7)
    q = torch.rand((2, 32, 32, 32, 32), device='cuda', generator=g)
    var = torch.rand((2, 32, 32), device='cuda', generator=g) + 2.
    oq, ot = run(nt, q, None, var, 2., 0.1, True, want_t=False)
    assert ot is None
    wq, _ = reference(q, None, var, 2., 0.1, True)
    assert float((oq.double() - wq).abs().max() / wq.abs().max()) < RTOL


@pytest.mark.parametrize('kind', ['relu', 'erf', 'none'])
def test_affine_act_vectorised_matches_elementwise(nt, kind):
    """ntg_affine_act on 16-byte aligned full-spatial buffers (chunked kernel with
    staged variances) and on buffers offset by one float (the elementwise kernel):
    the same operations per entry, so the results are bit-identical."""
    from nt_gb300 import _lib as L, _ops as O
    g = torch.Generator(device='cuda').manual_seed(13)
    n1, n2, A, C = 2, 3, 8, 16
    shp = (n1 * n2, A, A, C, C)
    cov = torch.rand((n1 + n2, A, A, C, C), device='cuda', generator=g) * 0.2 + 1.
    v1 = L.Var(cov[:n1].data_ptr(), A * A * C * C, A * C * C + C * C, C + 1)
    v2 = L.Var(cov[n1:].data_ptr(), A * A * C * C, A * C * C + C * C, C + 1)
    act = {'relu': L.Act(L.NTG_ACT_ABRELU, 0., 1., 0., 0, 0.),
           'erf': L.Act(L.NTG_ACT_ERF, 1., 1., 0., 0, 0.),
           'none': L.Act(L.NTG_ACT_NONE, 0., 0., 0., 0, 0.)}[kind]
    q = torch.rand(shp, device='cuda', generator=g) * 2 - 1
    t = torch.rand(shp, device='cuda', generator=g)
    aff = O.affine(1.7, 0.1, 1.7)

    def run(offset):
        bufs = []
        for x in (q, t, None, None):
            raw = torch.empty(q.numel() + 1, device='cuda')
            v = raw[offset:offset + q.numel()].view(shp)
            if x is not None:
                v.copy_(x)
            bufs.append(v)
        L.call('ntg_affine_act', L.stream(), L.ptr(bufs[0]), L.ptr(bufs[1]), L.ptr(bufs[2]),
               L.ptr(bufs[3]), n1 * n2, n2, A, C, 0, 1, aff, act, v1, v2)
        torch.cuda.synchronize()
        return bufs[2].clone(), bufs[3].clone()

    fast, slow = run(0), run(1)
    assert torch.equal(fast[0], slow[0]) and torch.equal(fast[1], slow[1])


@pytest.mark.parametrize('pairs', [True, False])
def test_input_covariance_vectorised_matches_elementwise(nt, pairs):
    """ntg_input_fs with a 16-byte aligned output (staged, vectorised kernel) and
    with the output offset by one float (one thread per entry): bit-identical."""
    from nt_gb300 import _lib as L
    g = torch.Generator(device='cuda').manual_seed(19)
    n1, n2, A, C, K = 3, 2, 32, 32, 3
    x1 = torch.randn((n1, A, C, K), device='cuda', generator=g)
    x2 = torch.randn((n2, A, C, K), device='cuda', generator=g)
    shp = (n1, n2, A, A, C, C) if pairs else (n1, A, A, C, C)
    numel = int(torch.tensor(shp).prod())

    def run(offset):
        raw = torch.empty(numel + 1, device='cuda')
        out = raw[offset:offset + numel].view(shp)
        L.call('ntg_input_fs', L.stream(), L.ptr(x1), L.ptr(x2) if pairs else None, n1,
               n2 if pairs else 0, A, C, K, int(pairs), L.ptr(out))
        torch.cuda.synchronize()
        return out.clone()

    fast, slow = run(0), run(1)
    assert torch.equal(fast, slow)
    want = (torch.einsum('ihwk,jHWk->ijhHwW', x1.double(), x2.double()) if pairs else
            torch.einsum('ihwk,iHWk->ihHwW', x1.double(), x1.double())) / K
    assert float((fast.double() - want).abs().max() / want.abs().max()) < 1e-6


def test_pool_transpose_block_matches_general(nt):
    """ntg_pool_bwd for AvgPool(2, 2) on full-spatial kernels: the block kernel
    (aligned output) against the general transpose (output offset by one float)."""
    from nt_gb300 import _lib as L
    g = torch.Generator(device='cuda').manual_seed(23)
    B, A, C = 5, 16, 16
    gout = torch.randn((B, A // 2, A // 2, C // 2, C // 2), device='cuda', generator=g)
    numel = B * A * A * C * C

    def run(offset):
        raw = torch.empty(numel + 1, device='cuda')
        gin = raw[offset:offset + numel].view(B, A, A, C, C)
        L.call('ntg_pool_bwd', L.stream(), L.ptr(gout), L.ptr(gin), B, A, C, 2, 2, 2, 2, 0, 0,
               A // 2, C // 2, 0, 0, 1, 0)
        torch.cuda.synchronize()
        return gin.clone()

    fast, slow = run(0), run(1)
    assert torch.equal(fast, slow)
