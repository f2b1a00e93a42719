"""Tensor-level wrappers over the C ABI (one function per entry point).

Each wrapper takes and returns contiguous float32 CUDA tensors, enqueues on
the current torch stream and raises NtgError when the library reports one.
"""
from __future__ import annotations

import math
from typing import Optional

import torch

from . import _lib as L


def affine(w2: float, b2: float, ntk_w2: float, ntk_nn: float = 1., ntk_c: float = 0.,
           nn_scaled: bool = True) -> L.Affine:
    return L.Affine(w2, b2, ntk_w2, ntk_nn, ntk_c, int(nn_scaled))


IDENTITY_AFFINE = affine(1., 0., 1., 0., 0., True)
NO_ACT = L.Act(L.NTG_ACT_NONE, 0., 0., 0., 0, 0.)
NO_VAR = L.Var(None, 0, 0, 0)


def var_view(cov: Optional[torch.Tensor], diag: bool) -> L.Var:
    """Strided view of the variances (diagonal) of a per-sample kernel."""
    if cov is None:
        return NO_VAR
    n = cov.shape[0]
    if cov.ndim == 1:
        return L.Var(L.ptr(cov), 1, 0, 0)
    if diag:
        a = cov.shape[1]
        c = cov.shape[2] if cov.ndim == 3 else 1
        return L.Var(L.ptr(cov), a * c, c, 1)
    a = cov.shape[1]
    c = cov.shape[3] if cov.ndim == 5 else 1
    del n
    return L.Var(L.ptr(cov), a * a * c * c, a * c * c + c * c, c + 1)


def spatial_ac(t: torch.Tensor, bnd: int, diag: bool) -> tuple[int, int]:
    """(A, C): spatial sizes of the first / second spatial axis (1 if absent)."""
    sp = t.shape[bnd:]
    if diag:
        if len(sp) == 0:
            return 1, 1
        if len(sp) == 1:
            return sp[0], 1
        if len(sp) == 2:
            return sp[0], sp[1]
    else:
        if len(sp) == 0:
            return 1, 1
        if len(sp) == 2:
            return sp[0], 1
        if len(sp) == 4:
            return sp[0], sp[2]
    raise NotImplementedError('nt_gb300 kernels support at most two spatial dimensions')


def gram(x1: torch.Tensor, x2: torch.Tensor, precision: int = 0) -> torch.Tensor:
    """x1 x2^T / D; precision 1 runs the split-BF16 tcgen05 tensor-core kernel."""
    n1, n2, d = x1.shape[0], x2.shape[0], x1.shape[1]
    out = torch.empty((n1, n2), device=x1.device, dtype=torch.float32)
    ws, nbytes = None, 0
    if precision == 1:
        nbytes = int(L.load().ntg_gram_workspace_bytes(n1, n2, d))
        ws = torch.empty((nbytes,), device=x1.device, dtype=torch.uint8)
    # a tensor-core pipeline wait that runs out raises the library's device error word,
    # which the public call around this one reads (L.boundary)
    L.call('ntg_gram', L.stream(), L.ptr(x1), L.ptr(x2), n1, n2, d, L.ptr(out), precision,
           None if ws is None else ws.data_ptr(), nbytes)
    return out


def cov_diag(x: torch.Tensor) -> torch.Tensor:
    out = torch.empty((x.shape[0],), device=x.device, dtype=torch.float32)
    L.call('ntg_cov_diag', L.stream(), L.ptr(x), x.shape[0], x.shape[1], L.ptr(out))
    return out


def input_ds(x1: torch.Tensor, x2: Optional[torch.Tensor]) -> torch.Tensor:
    """x [N, *spatial, K] -> [N1, N2, *spatial] (pairs) or [N, *spatial] (x2 None): the
    diagonal-spatial input covariances."""
    sp = tuple(x1.shape[1:-1])
    p, k = int(math.prod(sp)), x1.shape[-1]
    x1 = x1.contiguous()
    if x2 is None:
        out = torch.empty((x1.shape[0],) + sp, device=x1.device, dtype=torch.float32)
        L.call('ntg_input_ds', L.stream(), L.ptr(x1), None, x1.shape[0], 0, p, k, L.ptr(out))
    else:
        x2 = x2.contiguous()
        out = torch.empty((x1.shape[0], x2.shape[0]) + sp, device=x1.device, dtype=torch.float32)
        L.call('ntg_input_ds', L.stream(), L.ptr(x1), L.ptr(x2), x1.shape[0], x2.shape[0], p, k,
               L.ptr(out))
    return out


def input_fs(x1: torch.Tensor, x2: Optional[torch.Tensor]) -> torch.Tensor:
    """x [N, A, C, K] -> [N1, N2, A, A, C, C] (pairs) or [N, A, A, C, C] (x2 None)."""
    n1, a, c, k = x1.shape
    if x2 is None:
        out = torch.empty((n1, a, a, c, c), device=x1.device, dtype=torch.float32)
        L.call('ntg_input_fs', L.stream(), L.ptr(x1), None, n1, 0, a, c, k, 0, L.ptr(out))
    else:
        n2 = x2.shape[0]
        out = torch.empty((n1, n2, a, a, c, c), device=x1.device, dtype=torch.float32)
        L.call('ntg_input_fs', L.stream(), L.ptr(x1), L.ptr(x2), n1, n2, a, c, k, 1, L.ptr(out))
    return out


def conv_fs(q, t, batch, n2, a, c, fh, fw, sh, sw, ph, pw, ao, co, circular, aff, act, var1,
            var2, want_t, lead):
    out_q = torch.empty(lead + (ao, ao, co, co), device=q.device, dtype=torch.float32)
    out_t = torch.empty_like(out_q) if want_t else None
    L.call('ntg_conv_fs', L.stream(), L.ptr(q), L.ptr(t), L.ptr(out_q), L.ptr(out_t), batch, n2,
           a, c, fh, fw, sh, sw, ph, pw, ao, co, int(circular), aff, act, var1, var2)
    return out_q, out_t


def conv_ds(q, t, batch, a, c, fh, fw, sh, sw, ph, pw, ao, co, circular, aff, want_t, lead,
            has_c):
    shape = lead + ((ao, co) if has_c else (ao,))
    out_q = torch.empty(shape, device=q.device, dtype=torch.float32)
    out_t = torch.empty_like(out_q) if want_t else None
    L.call('ntg_conv_ds', L.stream(), L.ptr(q), L.ptr(t), L.ptr(out_q), L.ptr(out_t), batch, a, c,
           fh, fw, sh, sw, ph, pw, ao, co, int(circular), aff)
    return out_q, out_t


def affine_act(q, t, batch, n2, a, c, diag, has_affine, aff, act, var1, var2, want_t):
    out_q = torch.empty_like(q)
    out_t = torch.empty_like(q) if want_t else None
    L.call('ntg_affine_act', L.stream(), L.ptr(q), L.ptr(t), L.ptr(out_q), L.ptr(out_t), batch,
           n2, a, c, int(diag), int(has_affine), aff, act, var1, var2)
    return out_q, out_t


def max_abs(x: torch.Tensor) -> float:
    out = torch.empty((1,), device=x.device, dtype=torch.float32)
    L.call('ntg_max_abs', L.stream(), L.ptr(x), x.numel(), L.ptr(out))
    return float(out.item())


def pool(x, batch, a, c, wa, wc, sa, sc, pa, pc, ao, co, circular, diag, average,
         normalize_edges, out_shape):
    out = torch.empty(out_shape, device=x.device, dtype=torch.float32)
    L.call('ntg_pool', L.stream(), L.ptr(x), L.ptr(out), batch, a, c, wa, wc, sa, sc, pa, pc, ao,
           co, int(circular), int(diag), int(average), int(normalize_edges))
    return out


def global_pool(x: torch.Tensor, bnd: int, average: bool, post_scale: float = 1.) -> torch.Tensor:
    lead = tuple(x.shape[:bnd])
    batch = 1
    for d in lead:
        batch *= d
    m = x.numel() // max(batch, 1)
    out = torch.empty(lead, device=x.device, dtype=torch.float32)
    L.call('ntg_global_pool', L.stream(), L.ptr(x), L.ptr(out), batch, m, int(average), post_scale)
    return out


def flatten_fs(x: torch.Tensor, bnd: int, a: int, c: int) -> torch.Tensor:
    lead = tuple(x.shape[:bnd])
    batch = 1
    for d in lead:
        batch *= d
    out = torch.empty(lead, device=x.device, dtype=torch.float32)
    L.call('ntg_flatten_fs', L.stream(), L.ptr(x), L.ptr(out), batch, a, c)
    return out


def chain_fwd(prog: L.Chain, x1, x2, r0, n1, c0, n2, var1, var2, out_q, out_t, ld_out):
    import ctypes
    L.call('ntg_chain_fwd', L.stream(), ctypes.byref(prog), L.ptr(x1), L.ptr(x2), r0, n1, c0, n2,
           L.ptr(var1), L.ptr(var2), out_q.data_ptr(), None if out_t is None else out_t.data_ptr(),
           ld_out)


def chain_fwd_sym(prog: L.Chain, x, r0, n1, c0, n2, var, out_q, out_t, ld_out):
    """Pairs (r0.., c0..) of x with itself, each written at (i, j) and (j, i) of the
    whole kernel out [., ld_out]; the tile is diagonal (only i <= j evaluated) or
    has disjoint row and column ranges."""
    import ctypes
    L.call('ntg_chain_fwd_sym', L.stream(), ctypes.byref(prog), L.ptr(x), r0, n1, c0, n2,
           L.ptr(var), out_q.data_ptr(), None if out_t is None else out_t.data_ptr(), ld_out)
