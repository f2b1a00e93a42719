"""Reverse-mode differentiation of kernel_fn: one torch.autograd.Function per
layer rule, the counterpart of a ``jax.custom_vjp`` pair. Each forward calls
the layer's sm_103a kernels, each backward its hand-written adjoint kernels
(csrc/ntg_bwd.cu); gradients flow to the inputs x1, x2 and to W_std / b_std
given as tensors. Scope: full-spatial, diagonal-spatial (``ds``: kernels
[N1, N2, *spatial] holding only the (h, h, w, w) entries) or flat kernels, NTK
parameterisation.
"""
from __future__ import annotations

import math
from typing import Optional

import torch

from . import _lib as L
from . import _ops as O
from .kernel import Kernel, from_physical, to_physical


def _e(dev) -> torch.Tensor:
    return torch.empty(0, device=dev)


def _opt(t: Optional[torch.Tensor]) -> Optional[torch.Tensor]:
    return None if t is None or t.numel() == 0 else t


def _zero_ntk(t: Optional[torch.Tensor]) -> bool:
    return t is not None and t.ndim == 0


def _ac(x: torch.Tensor, bnd: int) -> tuple[int, int]:
    sp = x.shape[bnd:]
    if len(sp) == 0:
        return 1, 1
    if len(sp) == 2:
        return sp[0], 1
    return sp[0], sp[2]


def _as4(x: Optional[torch.Tensor], bnd: int):
    """View a kernel as [lead, A, A, C, C] (C = 1 for one spatial dimension)."""
    if x is None:
        return None
    a, c = _ac(x, bnd)
    return x.reshape(tuple(x.shape[:bnd]) + (a, a, c, c))


def _batch(x: torch.Tensor, bnd: int) -> int:
    return int(math.prod(x.shape[:bnd]))


def _positions(x: torch.Tensor, bnd: int) -> int:
    """Spatial positions of a diagonal-spatial kernel."""
    return int(math.prod(x.shape[bnd:]))


def _ds_var(cov: torch.Tensor) -> L.Var:
    """The variances of a diagonal-spatial per-sample kernel [N, *spatial]: the kernel itself,
    viewed as [N, P, 1]."""
    return L.Var(L.ptr(cov), _positions(cov, 1), 1, 0)


def _f(x) -> float:
    return float(x.item()) if isinstance(x, torch.Tensor) else float(x)


# ---------------------------------------------------------------------------
class InputFn(torch.autograd.Function):
    """requirements.py:641-830: inputs -> (nngp, cov1, cov2)."""

    @staticmethod
    def forward(ctx, x1, x2, gram_precision=0, ds=False):
        x2o = _opt(x2)
        xb = x1 if x2o is None else x2o
        ctx.ds = ds and x1.ndim > 2
        if ctx.ds:
            nngp = O.input_ds(x1, xb)
            cov1 = O.input_ds(x1, None)
            cov2 = _e(x1.device) if x2o is None else O.input_ds(x2o, None)
        elif x1.ndim == 2:
            nngp = O.gram(x1, xb, gram_precision)
            cov1 = torch.diagonal(nngp).contiguous() if x2o is None else O.cov_diag(x1)
            cov2 = _e(x1.device) if x2o is None else O.cov_diag(x2o)
        else:
            y1 = x1 if x1.ndim == 4 else x1.unsqueeze(2)
            yb = xb if xb.ndim == 4 else xb.unsqueeze(2)
            nngp = O.input_fs(y1, yb)
            cov1 = O.input_fs(y1, None)
            cov2 = _e(x1.device) if x2o is None else O.input_fs(yb, None)
            if x1.ndim == 3:
                a = x1.shape[1]
                nngp = nngp.reshape(nngp.shape[0], nngp.shape[1], a, a)
                cov1 = cov1.reshape(cov1.shape[0], a, a)
                if x2o is not None:
                    cov2 = cov2.reshape(cov2.shape[0], a, a)
        ctx.save_for_backward(x1, x2)
        return nngp, cov1, cov2

    @staticmethod
    def backward(ctx, gn, gc1, gc2):
        # the input rule's backward runs last in a network's backward pass
        with L.boundary('kernel_fn backward'):
            return InputFn._backward(ctx, gn, gc1, gc2)

    @staticmethod
    def _backward(ctx, gn, gc1, gc2):
        x1, x2 = ctx.saved_tensors
        x2o = _opt(x2)
        s = L.stream()
        gx1 = torch.zeros_like(x1)
        gx2 = None if x2o is None else torch.zeros_like(x2o)
        gn = gn.contiguous()
        if ctx.ds:
            n1, k = x1.shape[0], x1.shape[-1]
            p = int(math.prod(x1.shape[1:-1]))
            xb = x1 if x2o is None else x2o
            L.call('ntg_input_ds_bwd', s, L.ptr(gn), L.ptr(x1), L.ptr(xb), L.ptr(gx1),
                   L.ptr(gx1 if x2o is None else gx2), n1, xb.shape[0], p, k)
            for gcv, xx, gg in ((gc1, x1, gx1), (gc2, x2o, gx2)):
                if xx is None or gcv is None:
                    continue
                L.call('ntg_input_ds_bwd', s, L.ptr(gcv.contiguous()), L.ptr(xx), None,
                       L.ptr(gg), None, xx.shape[0], 0, p, k)
            return gx1, gx2, None, None
        if x1.ndim == 2:
            n1, d = x1.shape
            xb = x1 if x2o is None else x2o
            n2 = xb.shape[0]
            L.call('ntg_gemm_ex', s, L.ptr(gn), L.ptr(xb), L.ptr(gx1), n1, d, n2, 0, 1. / d, 1)
            L.call('ntg_gemm_ex', s, L.ptr(gn), L.ptr(x1),
                   L.ptr(gx1 if x2o is None else gx2), n2, d, n1, 1, 1. / d, 1)
            L.call('ntg_cov_diag_bwd', s, L.ptr(gc1.contiguous()), L.ptr(x1), L.ptr(gx1), n1, d)
            if x2o is not None:
                L.call('ntg_cov_diag_bwd', s, L.ptr(gc2.contiguous()), L.ptr(x2o), L.ptr(gx2),
                       n2, d)
            return gx1, gx2, None, None
        y1 = x1 if x1.ndim == 4 else x1.unsqueeze(2)
        yb = None if x2o is None else (x2o if x2o.ndim == 4 else x2o.unsqueeze(2))
        gy1 = gx1 if x1.ndim == 4 else gx1.unsqueeze(2)
        gyb = None if gx2 is None else (gx2 if x2o.ndim == 4 else gx2.unsqueeze(2))
        n1, a, c, k = y1.shape
        other = y1 if yb is None else yb
        n2 = other.shape[0]
        L.call('ntg_input_fs_bwd2', s, L.ptr(gn), L.ptr(y1), L.ptr(other), L.ptr(gy1),
               L.ptr(gy1 if yb is None else gyb), n1, n2, a, c, k)
        for gcv, yy, gg in ((gc1, y1, gy1), (gc2, yb, gyb)):
            if yy is None:
                continue
            L.call('ntg_input_fs_bwd2', s, L.ptr(gcv.contiguous()), L.ptr(yy), None, L.ptr(gg),
                   None, yy.shape[0], 0, a, c, k)
        return gx1, gx2, None, None


# ---------------------------------------------------------------------------
def _hyper(outs, grads, w2, b2, dev):
    acc = torch.zeros(2, device=dev, dtype=torch.float64)
    s = L.stream()
    for (q, t), (gq, gt) in zip(outs, grads):
        if q is None or gq is None:
            continue
        L.call('ntg_affine_hyper_bwd', s, L.ptr(q), None if t is None else L.ptr(t),
               L.ptr(gq.contiguous()), None if gt is None else L.ptr(gt.contiguous()),
               q.numel(), w2, b2, acc.data_ptr())
    return acc


class AffineFn(torch.autograd.Function):
    """Dense rule (linear.py:899-926) on all four tensors, NTK parameterisation."""

    @staticmethod
    def forward(ctx, w2t, b2t, q, t, c1, c2, ds=False):
        w2, b2 = _f(w2t), _f(b2t)
        aff = O.affine(w2, b2, w2)
        zero_t = _zero_ntk(t)
        c2o = _opt(c2)

        def aa(x, xt, want_t, bnd):
            if ds:  # elementwise: the entries as [batch, P] diagonal-spatial kernels
                return O.affine_act(x.contiguous(), xt, _batch(x, bnd), 0, _positions(x, bnd), 1,
                                    True, True, aff, O.NO_ACT, O.NO_VAR, O.NO_VAR, want_t)
            a, c = _ac(x, bnd)
            return O.affine_act(x.contiguous(), xt, _batch(x, bnd), 0, a, c, False, True, aff,
                                O.NO_ACT, O.NO_VAR, O.NO_VAR, want_t)

        qn, tn = aa(q, None if zero_t else t.contiguous(), True, 2)
        c1n, _ = aa(c1, None, False, 1)
        c2n = _e(q.device) if c2o is None else aa(c2o, None, False, 1)[0]
        ctx.save_for_backward(qn, tn, c1n, c2n)
        ctx.w2, ctx.b2, ctx.zero_t = w2, b2, zero_t
        return qn, tn, c1n, c2n

    @staticmethod
    def backward(ctx, gq, gt, gc1, gc2):
        qn, tn, c1n, c2n = ctx.saved_tensors
        w2, b2 = ctx.w2, ctx.b2
        aff = O.affine(w2, b2, w2)
        s = L.stream()

        def bwd(g, gtt, n):
            gu = torch.empty(n, device=qn.device)
            gut = torch.empty(n, device=qn.device) if gtt is not None else None
            L.call('ntg_affine_bwd', s, None if g is None else L.ptr(g.contiguous()),
                   None if gtt is None else L.ptr(gtt.contiguous()), L.ptr(gu),
                   None if gut is None else L.ptr(gut), n, aff, 1.)
            return gu, gut

        gu, gut = bwd(gq, gt, qn.numel())
        gc1i = bwd(gc1, None, c1n.numel())[0].reshape(c1n.shape)
        gc2i = None if c2n.numel() == 0 else bwd(gc2, None, c2n.numel())[0].reshape(c2n.shape)
        if ctx.needs_input_grad[0] or ctx.needs_input_grad[1]:
            acc = _hyper([(qn, tn), (c1n, None), (_opt(c2n), None)], [(gq, gt), (gc1, None),
                         (gc2 if c2n.numel() else None, None)], w2, b2, qn.device)
            gw2, gb2 = acc[0].float(), acc[1].float()
        else:
            gw2 = gb2 = None
        return (gw2, gb2, gu.reshape(qn.shape), None if ctx.zero_t else gut.reshape(qn.shape),
                gc1i, gc2i, None)


class ConvFn(torch.autograd.Function):
    """Full-spatial Conv rule (linear.py:1321-1424), NTK parameterisation."""

    @staticmethod
    def forward(ctx, w2t, b2t, q, t, c1, c2, geom, ds=False):
        w2, b2 = _f(w2t), _f(b2t)
        aff = O.affine(w2, b2, w2)
        fh, fw, sh, sw, ph, pw, ao, co, circ, nsp = geom
        zero_t = _zero_ntk(t)
        c2o = _opt(c2)
        ctx.ds = ds

        def conv(x, xt, want_t, bnd):
            if ds:  # linear.py:3381-3437
                lead = tuple(x.shape[:bnd])
                a = x.shape[bnd]
                c = x.shape[bnd + 1] if nsp == 2 else 1
                return O.conv_ds(x.contiguous(), None if xt is None else xt.contiguous(),
                                 _batch(x, bnd), a, c, fh, fw, sh, sw, ph, pw, ao, co, circ, aff,
                                 want_t, lead, nsp == 2)
            x4 = _as4(x.contiguous(), bnd)
            a, c = _ac(x, bnd)
            n2 = 0 if bnd == 1 else x.shape[1]
            lead = tuple(x.shape[:bnd])
            r = O.conv_fs(x4, None if xt is None else _as4(xt.contiguous(), bnd),
                          _batch(x, bnd), n2, a, c, fh, fw, sh, sw, ph, pw, ao, co, circ, aff,
                          O.NO_ACT, O.NO_VAR, O.NO_VAR, want_t, lead)
            if nsp == 1:
                r = tuple(None if y is None else y.reshape(lead + (ao, ao)) for y in r)
            return r

        qn, tn = conv(q, None if zero_t else t, True, 2)
        c1n = conv(c1, None, False, 1)[0]
        c2n = _e(q.device) if c2o is None else conv(c2o, None, False, 1)[0]
        ctx.save_for_backward(qn, tn, c1n, c2n)
        ctx.meta = (w2, b2, zero_t, geom, tuple(q.shape), tuple(c1.shape),
                    None if c2o is None else tuple(c2o.shape))
        return qn, tn, c1n, c2n

    @staticmethod
    def backward(ctx, gq, gt, gc1, gc2):
        qn, tn, c1n, c2n = ctx.saved_tensors
        w2, b2, zero_t, geom, qs, c1s, c2s = ctx.meta
        fh, fw, sh, sw, ph, pw, ao, co, circ, nsp = geom
        aff = O.affine(w2, b2, w2)
        scale = 1. / (fh * fw)
        s = L.stream()
        dev = qn.device

        ds = getattr(ctx, 'ds', False)

        def back(g, gtt, in_shape, bnd, want_t_in=True):
            n = int(math.prod(g.shape)) if g is not None else int(math.prod(gtt.shape))
            gu = torch.empty(n, device=dev)
            gut = torch.empty(n, device=dev) if (gtt is not None and want_t_in) else None
            L.call('ntg_affine_bwd', s, None if g is None else L.ptr(g.contiguous()),
                   None if gtt is None else L.ptr(gtt.contiguous()), L.ptr(gu),
                   None if gut is None else L.ptr(gut), n, aff, scale)
            lead = in_shape[:bnd]
            a = in_shape[bnd]
            c = (in_shape[bnd + 1] if ds else in_shape[bnd + 2]) if nsp == 2 else 1
            batch = int(math.prod(lead))
            outs = []
            for gg in (gu, gut):
                if gg is None:
                    outs.append(None)
                    continue
                gin = torch.empty(in_shape, device=dev)
                L.call('ntg_stencil_bwd', s, L.ptr(gg), L.ptr(gin), batch, a, c, fh, fw, sh, sw,
                       ph, pw, ao, co, int(circ), int(ds))
                outs.append(gin)
            return outs

        def back_symmetric(g, gtt, in_shape, bnd):
            # A stride-1 window centred on its output (odd filter, padding (f - 1) / 2, same
            # size) is its own transpose, so the adjoint is the forward stencil kernel with
            # the roles of the two tensors exchanged:
            #   g_nngp_in = s (W^2 Sum g + W^2 Sum g_ntk),  g_ntk_in = s W^2 Sum g_ntk.
            lead = tuple(in_shape[:bnd])
            a = in_shape[bnd]
            c = in_shape[bnd + 2] if nsp == 2 else 1
            n2 = 0 if bnd == 1 else in_shape[1]
            batch = int(math.prod(lead))

            def four(x):
                return None if x is None else _as4(x.contiguous(), bnd)

            if gtt is None:
                oq, _ = O.conv_fs(four(g), None, batch, n2, a, c, fh, fw, sh, sw, ph, pw, ao, co,
                                  circ, O.affine(w2, 0., 0., 0., 0., False), O.NO_ACT, O.NO_VAR,
                                  O.NO_VAR, False, lead)
                return [oq.reshape(in_shape), None]
            gti_, gqi_ = O.conv_fs(four(gtt), four(g), batch, n2, a, c, fh, fw, sh, sw, ph, pw, ao,
                                   co, circ, O.affine(w2, 0., w2, w2, 0., False), O.NO_ACT,
                                   O.NO_VAR, O.NO_VAR, True, lead)
            return [gqi_.reshape(in_shape), gti_.reshape(in_shape)]

        symmetric = (not ds and sh == 1 and sw == 1 and fh % 2 == 1 and fw % 2 == 1 and
                     2 * ph + 1 == fh and 2 * pw + 1 == fw and ao == qs[2] and
                     (nsp == 1 or co == qs[4]))
        # the output NTK's cotangent reaches the input nngp through ntk_out = nngp_out + ...
        # even when the input NTK is the scalar zero of an input kernel
        if symmetric and (gq is not None or gt is not None):
            gqi, gti = back_symmetric(gq if gq is not None else torch.zeros_like(gt), gt, qs, 2)
            gti = None if zero_t else gti
        else:
            gqi, gti = back(gq, gt, qs, 2, not zero_t)
        if symmetric and gc1 is not None:
            gc1i = back_symmetric(gc1, None, c1s, 1)[0]
        else:
            gc1i = back(gc1, None, c1s, 1)[0]
        if c2s is None:
            gc2i = None
        elif symmetric and gc2 is not None:
            gc2i = back_symmetric(gc2, None, c2s, 1)[0]
        else:
            gc2i = back(gc2, None, c2s, 1)[0]
        if ctx.needs_input_grad[0] or ctx.needs_input_grad[1]:
            acc = _hyper([(qn, tn), (c1n, None), (_opt(c2n), None)], [(gq, gt), (gc1, None),
                         (gc2 if c2s is not None else None, None)], w2, b2, dev)
            gw2, gb2 = acc[0].float(), acc[1].float()
        else:
            gw2 = gb2 = None
        return gw2, gb2, gqi, gti, gc1i, gc2i, None, None


# ---------------------------------------------------------------------------
def _diag_view(cov: torch.Tensor) -> L.Var:
    return O.var_view(_as4(cov, 1) if cov.ndim > 1 else cov, False)


class ActFn(torch.autograd.Function):
    """Activation rule (elementwise.py:423-477 ABRelu, :67-112 Erf) on all four tensors."""

    @staticmethod
    def forward(ctx, q, t, c1, c2, act, ds=False):
        c2o = _opt(c2)
        zero_t = _zero_ntk(t)
        ctx.ds = ds
        if ds:
            return ActFn._forward_ds(ctx, q, t, c1, c2o, act, zero_t)
        a, c = _ac(q, 2)
        q4, c14 = _as4(q.contiguous(), 2), _as4(c1.contiguous(), 1)
        c24 = None if c2o is None else _as4(c2o.contiguous(), 1)
        v1 = _diag_view(c14)
        v2 = _diag_view(c24 if c24 is not None else c14)
        n1, n2 = q.shape[0], q.shape[1]
        t4 = None if zero_t else _as4(t.contiguous(), 2)
        qn, tn = O.affine_act(q4, t4, n1 * n2, n2, a, c, False, False, O.IDENTITY_AFFINE, act, v1,
                              v2, not zero_t)

        def self_act(cv):
            vv = _diag_view(cv)
            return O.affine_act(cv, None, cv.shape[0], 0, a, c, False, False, O.IDENTITY_AFFINE,
                                act, vv, vv, False)[0]

        c1n = self_act(c14)
        c2n = _e(q.device) if c24 is None else self_act(c24)
        ctx.save_for_backward(q, t if not zero_t else _e(q.device), c1, c2)
        ctx.act, ctx.zero_t = act, zero_t
        tout = t.clone() if zero_t else tn.reshape(q.shape)
        return (qn.reshape(q.shape), tout, c1n.reshape(c1.shape),
                c2n if c2o is None else c2n.reshape(c2o.shape))

    @staticmethod
    def _forward_ds(ctx, q, t, c1, c2o, act, zero_t):
        """The activation rule on diagonal-spatial kernels [N1, N2, *spatial]: the variances
        of a position are the per-sample kernels themselves."""
        p = _positions(q, 2)
        n1, n2 = q.shape[0], q.shape[1]
        q, c1 = q.contiguous(), c1.contiguous()
        c2o = None if c2o is None else c2o.contiguous()
        v1 = _ds_var(c1)
        v2 = _ds_var(c2o if c2o is not None else c1)
        qn, tn = O.affine_act(q, None if zero_t else t.contiguous(), n1 * n2, n2, p, 1, True,
                              False, O.IDENTITY_AFFINE, act, v1, v2, not zero_t)

        def self_act(cv):
            vv = _ds_var(cv)
            return O.affine_act(cv, None, cv.shape[0], 0, p, 1, True, False, O.IDENTITY_AFFINE,
                                act, vv, vv, False)[0]

        c1n = self_act(c1)
        c2n = _e(q.device) if c2o is None else self_act(c2o)
        ctx.save_for_backward(q, t if not zero_t else _e(q.device), c1,
                              _e(q.device) if c2o is None else c2o)
        ctx.act, ctx.zero_t = act, zero_t
        return qn, t.clone() if zero_t else tn, c1n, c2n

    @staticmethod
    def _backward_ds(ctx, gq, gt, gc1, gc2):
        q, t, c1, c2 = ctx.saved_tensors
        act, zero_t = ctx.act, ctx.zero_t
        c2o = _opt(c2)
        s = L.stream()
        p = _positions(q, 2)
        n1, n2 = q.shape[0], q.shape[1]
        v1 = _ds_var(c1)
        v2 = _ds_var(c2o if c2o is not None else c1)
        gd1 = torch.zeros((n1, p), device=q.device)
        gd2 = gd1 if c2o is None else torch.zeros((c2o.shape[0], p), device=q.device)
        gqi = torch.empty_like(q)
        gti = None if zero_t else torch.empty_like(q)
        L.call('ntg_act_bwd', s, L.ptr(q), None if zero_t else L.ptr(t),
               None if gq is None else L.ptr(gq.contiguous()),
               None if (gt is None or zero_t) else L.ptr(gt.contiguous()), L.ptr(gqi),
               None if gti is None else L.ptr(gti), n1 * n2, n2, p, 1, 1, act, v1, v2,
               gd1.data_ptr(), gd2.data_ptr())

        def self_back(cv, gcv, gd):
            vv = _ds_var(cv)
            out = torch.empty_like(cv)
            L.call('ntg_act_bwd', s, L.ptr(cv), None,
                   None if gcv is None else L.ptr(gcv.contiguous()), None, L.ptr(out), None,
                   cv.shape[0], 0, p, 1, 1, act, vv, vv, gd.data_ptr(), gd.data_ptr())
            # every entry of a diagonal-spatial per-sample kernel is a variance
            L.call('ntg_diag_add', s, gd.data_ptr(), L.ptr(out), cv.shape[0], p, 1, p, 1, 0)
            return out

        gc1i = self_back(c1, gc1, gd1)
        gc2i = None if c2o is None else self_back(c2o, gc2, gd2)
        return gqi, None if zero_t else gti, gc1i, gc2i, None, None

    @staticmethod
    def backward(ctx, gq, gt, gc1, gc2):
        if getattr(ctx, 'ds', False):
            return ActFn._backward_ds(ctx, gq, gt, gc1, gc2)
        q, t, c1, c2 = ctx.saved_tensors
        act, zero_t = ctx.act, ctx.zero_t
        c2o = _opt(c2)
        s = L.stream()
        a, c = _ac(q, 2)
        n1, n2 = q.shape[0], q.shape[1]
        q4, c14 = _as4(q.contiguous(), 2), _as4(c1.contiguous(), 1)
        c24 = None if c2o is None else _as4(c2o.contiguous(), 1)
        v1 = _diag_view(c14)
        v2 = _diag_view(c24 if c24 is not None else c14)
        gd1 = torch.zeros((n1, a, c), device=q.device)
        gd2 = gd1 if c24 is None else torch.zeros((c24.shape[0], a, c), device=q.device)
        gqi = torch.empty_like(q4)
        gti = None if zero_t else torch.empty_like(q4)
        t4 = None if zero_t else _as4(t.contiguous(), 2)
        L.call('ntg_act_bwd', s, L.ptr(q4), None if t4 is None else L.ptr(t4),
               None if gq is None else L.ptr(_as4(gq.contiguous(), 2)),
               None if (gt is None or zero_t) else L.ptr(_as4(gt.contiguous(), 2)),
               L.ptr(gqi), None if gti is None else L.ptr(gti), n1 * n2, n2, a, c, 0, act, v1, v2,
               gd1.data_ptr(), gd2.data_ptr())

        def self_back(cv, gcv, gd):
            vv = _diag_view(cv)
            out = torch.empty_like(cv)
            L.call('ntg_act_bwd', s, L.ptr(cv), None,
                   None if gcv is None else L.ptr(_as4(gcv.contiguous(), 1) if cv.ndim > 1 else
                                                  gcv.contiguous()),
                   None, L.ptr(out), None, cv.shape[0], 0, a, c, 0, act, vv, vv,
                   gd.data_ptr(), gd.data_ptr())
            L.call('ntg_diag_add', s, gd.data_ptr(), L.ptr(out), cv.shape[0], a, c, vv.s_n, vv.s_a,
                   vv.s_c)
            return out

        # The pair VJP has already added its variance cotangents into gd1/gd2;
        # each self VJP adds its own and folds the total into its diagonal.
        gc1i = self_back(c14, gc1, gd1).reshape(c1.shape)
        gc2i = None if c24 is None else self_back(c24, gc2, gd2).reshape(c2o.shape)
        return (gqi.reshape(q.shape), None if zero_t else gti.reshape(q.shape), gc1i, gc2i, None,
                None)


class ActPoolFn(torch.autograd.Function):
    """Activation followed by AvgPool((2, 2), (2, 2)) on full-spatial kernels: the forward
    is the two rules; the backward applies the activation VJP to the pooled cotangents
    directly (ntg_act_pool_bwd), so the unpooled cotangent is never written."""

    @staticmethod
    def forward(ctx, q, t, c1, c2, act, pool_geom):
        qa, ta, c1a, c2a = ActFn.forward(ctx, q, t, c1, c2, act)
        ctx.pool_geom = pool_geom
        ctx.pool_shapes = [None if x is None else tuple(x.shape) for x in (qa, ta, c1a, c2a)]

        def run(x, bnd):
            if x is None or x.ndim == 0 or x.numel() == 0:
                return x
            a, c, wa, wc, sa, sc, pa, pc, ao, co, circ, avg, ne, two_d = pool_geom
            lead = tuple(x.shape[:bnd])
            return O.pool(x.contiguous(), int(math.prod(lead)), a, c, wa, wc, sa, sc, pa, pc, ao,
                          co, circ, False, avg, ne, lead + (ao, ao, co, co))

        return run(qa, 2), run(ta, 2), run(c1a, 1), run(c2a, 1)

    @staticmethod
    def backward(ctx, gq, gt, gc1, gc2):
        q, t, c1, c2 = ctx.saved_tensors
        act, zero_t = ctx.act, ctx.zero_t
        c2o = _opt(c2)
        s = L.stream()
        a, c = _ac(q, 2)
        n1, n2 = q.shape[0], q.shape[1]
        q4, c14 = _as4(q.contiguous(), 2), _as4(c1.contiguous(), 1)
        c24 = None if c2o is None else _as4(c2o.contiguous(), 1)
        v1 = _diag_view(c14)
        v2 = _diag_view(c24 if c24 is not None else c14)
        gd1 = torch.zeros((n1, a, c), device=q.device)
        gd2 = gd1 if c24 is None else torch.zeros((c24.shape[0], a, c), device=q.device)
        gqi = torch.empty_like(q4)
        gti = None if zero_t else torch.empty_like(q4)
        t4 = None if zero_t else _as4(t.contiguous(), 2)
        L.call('ntg_act_pool_bwd', s, L.ptr(q4), None if t4 is None else L.ptr(t4),
               None if gq is None else L.ptr(gq.contiguous()),
               None if (gt is None or zero_t) else L.ptr(gt.contiguous()),
               L.ptr(gqi), None if gti is None else L.ptr(gti), n1 * n2, n2, a, c, act, v1, v2,
               gd1.data_ptr(), gd2.data_ptr())

        def self_back(cv, gcv, gd):
            vv = _diag_view(cv)
            out = torch.empty_like(cv)
            L.call('ntg_act_pool_bwd', s, L.ptr(cv), None,
                   None if gcv is None else L.ptr(gcv.contiguous()), None, L.ptr(out), None,
                   cv.shape[0], 0, a, c, act, vv, vv, gd.data_ptr(), gd.data_ptr())
            L.call('ntg_diag_add', s, gd.data_ptr(), L.ptr(out), cv.shape[0], a, c, vv.s_n,
                   vv.s_a, vv.s_c)
            return out

        gc1i = self_back(c14, gc1, gd1).reshape(c1.shape)
        gc2i = None if c24 is None else self_back(c24, gc2, gd2).reshape(c2o.shape)
        return (gqi.reshape(q.shape), None if zero_t else gti.reshape(q.shape), gc1i, gc2i, None,
                None)


class _SubCtx:
    """The ctx fields another Function's backward reads, for composing rules."""

    def __init__(self, saved, **fields):
        self.saved_tensors = saved
        self.__dict__.update(fields)


def _conv_act_self_back(cv, gcv, gd, act, pooled, w2):
    """Backward of a 3x3 SAME conv + activation (+ AvgPool(2, 2)) on a per-sample kernel
    cv [n, A, A, C, C] (the conv output): the activation VJP, whose variance cotangents join
    the pair's already in gd and fold into the kernel's diagonal, then the conv's transpose
    (the stride-1 centred stencil is its own transpose)."""
    s = L.stream()
    n, a, c = cv.shape[0], cv.shape[1], cv.shape[3]
    vv = _diag_view(cv)
    out = torch.empty_like(cv)
    g = None if gcv is None else L.ptr(gcv.contiguous())
    if pooled:
        L.call('ntg_act_pool_bwd', s, L.ptr(cv), None, g, None, L.ptr(out), None, n, 0, a, c, act,
               vv, vv, gd.data_ptr(), gd.data_ptr())
    else:
        L.call('ntg_act_bwd', s, L.ptr(cv), None, g, None, L.ptr(out), None, n, 0, a, c, 0, act,
               vv, vv, gd.data_ptr(), gd.data_ptr())
    L.call('ntg_diag_add', s, gd.data_ptr(), L.ptr(out), n, a, c, vv.s_n, vv.s_a, vv.s_c)
    gin, _ = O.conv_fs(out, None, n, 0, a, c, 3, 3, 1, 1, 1, 1, a, c, False,
                       O.affine(w2, 0., 0., 0., 0., False), O.NO_ACT, O.NO_VAR, O.NO_VAR, False,
                       (n,))
    return gin


class InputConvActFn(torch.autograd.Function):
    """Input covariances, a 3x3 / stride 1 / SAME conv (NTK parameterisation) and an ABRelu
    on 32 x 32 images: the pair kernels take one pass from the images (ntg_input_conv_act_fs,
    the covariances never written) and one fused backward (ntg_conv_act_bwd with the conv
    output as both pre-activation tensors: the input NTK is zero, so the conv's NTK equals
    its NNGP); the per-sample kernels take the layer rules one by one."""

    @staticmethod
    def forward(ctx, x1, x2, w2t, b2t, act):
        w2, b2 = _f(w2t), _f(b2t)
        aff = O.affine(w2, b2, w2)
        x2o = _opt(x2)
        xb = x1 if x2o is None else x2o
        dev = x1.device
        n1, n2, k = x1.shape[0], xb.shape[0], x1.shape[3]
        a = c = 32

        def conv_self(cv):
            return O.conv_fs(cv, None, cv.shape[0], 0, a, c, 3, 3, 1, 1, 1, 1, a, c, False, aff,
                             O.NO_ACT, O.NO_VAR, O.NO_VAR, False, (cv.shape[0],))[0]

        def act_self(cv):
            vv = _diag_view(cv)
            return O.affine_act(cv, None, cv.shape[0], 0, a, c, False, False, O.IDENTITY_AFFINE,
                                act, vv, vv, False)[0]

        c1p = conv_self(O.input_fs(x1, None))
        c2p = None if x2o is None else conv_self(O.input_fs(x2o, None))
        v1 = _diag_view(c1p)
        v2 = _diag_view(c2p if c2p is not None else c1p)
        shape = (n1, n2, a, a, c, c)
        qa, ta = torch.empty(shape, device=dev), torch.empty(shape, device=dev)
        pre = torch.empty(shape, device=dev)
        L.call('ntg_input_conv_act_fs', L.stream(), L.ptr(x1), L.ptr(xb), n1, n2, k, L.ptr(qa),
               L.ptr(ta), L.ptr(pre), aff, act, v1, v2)
        c1a = act_self(c1p)
        c2a = _e(dev) if c2p is None else act_self(c2p)
        ctx.save_for_backward(x1, x2, pre, c1p, _e(dev) if c2p is None else c2p)
        ctx.w2, ctx.act = w2, act
        return qa, ta, c1a, c2a

    @staticmethod
    def backward(ctx, gq, gt, gc1, gc2):
        # the first layers' backward runs last in a network's backward pass
        with L.boundary('kernel_fn backward'):
            return InputConvActFn._backward(ctx, gq, gt, gc1, gc2)

    @staticmethod
    def _backward(ctx, gq, gt, gc1, gc2):
        x1, x2, pre, c1p, c2p = ctx.saved_tensors
        x2o, c2o = _opt(x2), _opt(c2p)
        w2, act = ctx.w2, ctx.act
        s = L.stream()
        dev = x1.device
        n1, n2 = pre.shape[0], pre.shape[1]
        a, c, k = 32, 32, x1.shape[3]
        v1 = _diag_view(c1p)
        v2 = _diag_view(c2o if c2o is not None else c1p)
        gd1 = torch.zeros((n1, a, c), device=dev)
        gd2 = gd1 if c2o is None else torch.zeros((n2, a, c), device=dev)
        gin = torch.empty_like(pre)
        L.call('ntg_conv_act_bwd', s, L.ptr(pre), L.ptr(pre),
               None if gq is None else L.ptr(gq.contiguous()),
               None if gt is None else L.ptr(gt.contiguous()), 0, L.ptr(gin), None, n1 * n2, n2,
               a, w2, act, v1, v2, gd1.data_ptr(), gd2.data_ptr())
        gc1i = _conv_act_self_back(c1p, gc1, gd1, act, False, w2)
        gc2i = None if c2o is None else _conv_act_self_back(c2o, gc2, gd2, act, False, w2)
        # input covariance adjoint (requirements.py:641-830): the pairs, then each image's own
        gx1 = torch.zeros_like(x1)
        gx2 = None if x2o is None else torch.zeros_like(x2o)
        other = x1 if x2o is None else x2o
        L.call('ntg_input_fs_bwd2', s, L.ptr(gin), L.ptr(x1), L.ptr(other), L.ptr(gx1),
               L.ptr(gx1 if x2o is None else gx2), n1, n2, a, c, k)
        for gcv, xx, gg in ((gc1i, x1, gx1), (gc2i, x2o, gx2)):
            if xx is None:
                continue
            L.call('ntg_input_fs_bwd2', s, L.ptr(gcv), L.ptr(xx), None, L.ptr(gg), None,
                   xx.shape[0], 0, a, c, k)
        return gx1, gx2, None, None, None


def input_conv_act_fusable(x1: torch.Tensor, specs, ds: bool) -> bool:
    """Whether the first two layers take InputConvActFn: 32 x 32 NHWC images with 1-4
    channels, a 3x3 / stride 1 / SAME zero-padded conv in the NTK parameterisation whose
    W_std / b_std need no gradient, then an ABRelu without do_stabilize."""
    from .stax import Padding
    if ds or x1.ndim != 4 or tuple(x1.shape[1:3]) != (32, 32) or not 1 <= x1.shape[3] <= 4:
        return False
    if len(specs) < 2 or specs[0].kind != 'conv' or specs[1].kind != 'act':
        return False
    p, q = specs[0].params, specs[1].params
    if (p['parameterization'] != 'ntk' or tuple(p['filter_shape']) != (3, 3)
            or tuple(p['strides']) != (1, 1) or p['padding'] != Padding.SAME):
        return False
    if any(isinstance(p[key], torch.Tensor) and p[key].requires_grad for key in ('W_std', 'b_std')):
        return False
    return q['fn'] == 'abrelu' and not q.get('do_stabilize')


class ConvActFn(torch.autograd.Function):
    """Conv (3x3, stride 1, SAME, 32 x 32 planes) followed by an activation, and optionally by
    AvgPool((2, 2), (2, 2)): the pair kernels take one pass (ntg_conv_act_fs writes the
    activated kernels and the conv output the activation's VJP needs); the per-sample
    kernels take the conv, then the activation with their own variances. The backward is
    the activation VJP (pooled cotangent read directly when the pool is fused) followed by
    the conv's."""

    @staticmethod
    def forward(ctx, w2t, b2t, q, t, c1, c2, geom, act, pool_geom):
        w2, b2 = _f(w2t), _f(b2t)
        aff = O.affine(w2, b2, w2)
        fh, fw, sh, sw, ph, pw, ao, co, circ, nsp = geom
        zero_t = _zero_ntk(t)
        c2o = _opt(c2)
        dev = q.device

        def conv_self(x):
            x4 = _as4(x.contiguous(), 1)
            a, c = _ac(x, 1)
            return O.conv_fs(x4, None, x.shape[0], 0, a, c, fh, fw, sh, sw, ph, pw, ao, co, circ,
                             aff, O.NO_ACT, O.NO_VAR, O.NO_VAR, False, (x.shape[0],))[0]

        c1p = conv_self(c1)
        c2p = _e(dev) if c2o is None else conv_self(c2o)
        v1 = _diag_view(c1p)
        v2 = _diag_view(c2p if c2o is not None else c1p)
        n1, n2, a = q.shape[0], q.shape[1], q.shape[2]
        c = q.shape[4]
        q4 = _as4(q.contiguous(), 2)
        t4 = None if zero_t else _as4(t.contiguous(), 2)
        shape = (n1, n2, a, a, c, c)
        qp, tp = torch.empty(shape, device=dev), torch.empty(shape, device=dev)
        if pool_geom is not None:
            # the activated pair kernels go straight into the pool (ntg_conv_act_pool_fs):
            # only their window sums along w are written, then added plane by plane
            pshape = (n1, n2, pool_geom[8], pool_geom[8], pool_geom[9], pool_geom[9])
            qa, ta = torch.empty(pshape, device=dev), torch.empty(pshape, device=dev)
            hq = torch.empty((n1 * n2, a, a, c // 2, c // 2), device=dev)
            ht = torch.empty_like(hq)
            L.call('ntg_conv_act_pool_fs', L.stream(), L.ptr(q4),
                   None if t4 is None else L.ptr(t4), L.ptr(qa), L.ptr(ta), L.ptr(qp), L.ptr(tp),
                   L.ptr(hq), L.ptr(ht), n1 * n2, n2, a, aff, act, v1, v2)
            del hq, ht
        else:
            qa, ta = torch.empty(shape, device=dev), torch.empty(shape, device=dev)
            L.call('ntg_conv_act_fs', L.stream(), L.ptr(q4), None if t4 is None else L.ptr(t4),
                   L.ptr(qa), L.ptr(ta), L.ptr(qp), L.ptr(tp), n1 * n2, n2, a, c, aff, act, v1,
                   v2)

        def act_self(cv):
            vv = _diag_view(cv)
            return O.affine_act(cv, None, cv.shape[0], 0, a, c, False, False, O.IDENTITY_AFFINE,
                                act, vv, vv, False)[0]

        c1a = act_self(c1p)
        c2a = _e(dev) if c2o is None else act_self(c2p)
        ctx.save_for_backward(qp, tp, c1p, c2p)
        ctx.conv_meta = (w2, b2, zero_t, geom, tuple(q.shape), tuple(c1.shape),
                         None if c2o is None else tuple(c2o.shape))
        ctx.act, ctx.pool_geom = act, pool_geom
        outs = [qa, ta, c1a, c2a]
        if pool_geom is not None:
            pa_, pc_ = pool_geom[6], pool_geom[7]
            ao2, co2 = pool_geom[8], pool_geom[9]

            def pool(x, bnd):
                if x.numel() == 0:
                    return x
                lead = tuple(x.shape[:bnd])
                return O.pool(x.contiguous(), int(math.prod(lead)), a, c, 2, 2, 2, 2, pa_, pc_,
                              ao2, co2, False, False, True, False, lead + (ao2, ao2, co2, co2))

            outs = [outs[0], outs[1], pool(outs[2], 1), pool(outs[3], 1)]
        return tuple(outs)

    @staticmethod
    def _backward_fused(ctx, gq, gt, gc1, gc2):
        """The pair kernels' activation VJP and conv transpose in one pass
        (ntg_conv_act_bwd); the per-sample kernels take the two rules separately."""
        qp, tp, c1p, c2p = ctx.saved_tensors
        w2, b2, zero_t, geom, qs, c1s, c2s = ctx.conv_meta
        act, pooled = ctx.act, ctx.pool_geom is not None
        s = L.stream()
        dev = qp.device
        n1, n2, a, c = qp.shape[0], qp.shape[1], qp.shape[2], qp.shape[4]
        c2o = _opt(c2p)
        v1 = _diag_view(c1p)
        v2 = _diag_view(c2o if c2o is not None else c1p)
        gd1 = torch.zeros((n1, a, c), device=dev)
        gd2 = gd1 if c2o is None else torch.zeros((c2o.shape[0], a, c), device=dev)
        gqi = torch.empty(qs, device=dev)
        gti = None if zero_t else torch.empty(qs, device=dev)
        L.call('ntg_conv_act_bwd', s, L.ptr(qp), L.ptr(tp),
               None if gq is None else L.ptr(gq.contiguous()),
               None if gt is None else L.ptr(gt.contiguous()), int(pooled), L.ptr(gqi),
               None if gti is None else L.ptr(gti), n1 * n2, n2, a, w2, act, v1, v2,
               gd1.data_ptr(), gd2.data_ptr())
        gc1i = _conv_act_self_back(c1p, gc1, gd1, act, pooled, w2).reshape(c1s)
        gc2i = (None if c2s is None else
                _conv_act_self_back(c2o, gc2, gd2, act, pooled, w2).reshape(c2s))
        return None, None, gqi, gti, gc1i, gc2i, None, None, None

    @staticmethod
    def backward(ctx, gq, gt, gc1, gc2):
        qp, tp, c1p, c2p = ctx.saved_tensors
        if (ctx.act.kind == L.NTG_ACT_ABRELU and ctx.act.stabilize <= 0.
                and not (ctx.needs_input_grad[0] or ctx.needs_input_grad[1])
                and (gq is not None or gt is not None)):
            return ConvActFn._backward_fused(ctx, gq, gt, gc1, gc2)
        act_ctx = _SubCtx((qp, tp, c1p, c2p), act=ctx.act, zero_t=False)
        if ctx.pool_geom is not None:
            g = ActPoolFn.backward(act_ctx, gq, gt, gc1, gc2)
        else:
            g = ActFn.backward(act_ctx, gq, gt, gc1, gc2)
        conv_ctx = _SubCtx((qp, tp, c1p, c2p), meta=ctx.conv_meta,
                           needs_input_grad=ctx.needs_input_grad[:2] + (True,) * 5)
        r = ConvFn.backward(conv_ctx, g[0], g[1], g[2], g[3])
        return r[0], r[1], r[2], r[3], r[4], r[5], None, None, None


def conv_act_fusable(q: torch.Tensor, geom) -> bool:
    """Whether ConvActFn applies: pair kernels [N1, N2, 32, 32, 32, 32] and a 3x3 / stride 1 /
    SAME / zero-padded conv."""
    fh, fw, sh, sw, ph, pw, ao, co, circ, nsp = geom
    return (q.ndim == 6 and nsp == 2 and q.shape[2] == 32 and q.shape[4] == 32 and
            (fh, fw, sh, sw, ph, pw) == (3, 3, 1, 1, 1, 1) and ao == 32 and co == 32 and not circ)


def act_pool_fusable(q: torch.Tensor, pool_geom) -> bool:
    """Whether ActPoolFn's fused backward applies: full-spatial [N1, N2, A, A, C, C] with C a
    power of two in [4, 32], AvgPool((2, 2), (2, 2)) without padding."""
    if q.ndim != 6:
        return False
    a, c, wa, wc, sa, sc, pa, pc, ao, co, circ, avg, ne, two_d = pool_geom
    return (two_d and avg and not ne and (wa, wc, sa, sc, pa, pc) == (2, 2, 2, 2, 0, 0) and
            a % 2 == 0 and c in (4, 8, 16, 32) and (a * a * c * c) % 1024 == 0 and
            ao == a // 2 and co == c // 2)


# ---------------------------------------------------------------------------
class PoolFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q, t, c1, c2, geom, ds=False):
        a, c, wa, wc, sa, sc, pa, pc, ao, co, circ, avg, ne, two_d = geom

        def run(x, bnd):
            if x is None or x.ndim == 0 or x.numel() == 0:
                return x
            lead = tuple(x.shape[:bnd])
            if ds:
                shape = lead + ((ao, co) if two_d else (ao,))
            else:
                shape = lead + ((ao, ao, co, co) if two_d else (ao, ao))
            return O.pool(x.contiguous(), int(math.prod(lead)), a, c, wa, wc, sa, sc, pa, pc, ao,
                          co, circ, ds, avg, ne, shape)

        ctx.geom, ctx.ds = geom, ds
        ctx.shapes = [None if x is None else tuple(x.shape) for x in (q, t, c1, c2)]
        return run(q, 2), run(t, 2), run(c1, 1), run(c2, 1)

    @staticmethod
    def backward(ctx, gq, gt, gc1, gc2):
        a, c, wa, wc, sa, sc, pa, pc, ao, co, circ, avg, ne, two_d = ctx.geom
        s = L.stream()
        outs = []
        for g, shp, bnd in zip((gq, gt, gc1, gc2), ctx.shapes, (2, 2, 1, 1)):
            if g is None or shp is None or len(shp) == 0 or int(math.prod(shp)) == 0:
                outs.append(None)
                continue
            gin = torch.empty(shp, device=g.device)
            L.call('ntg_pool_bwd', s, L.ptr(g.contiguous()), L.ptr(gin),
                   int(math.prod(shp[:bnd])), a, c, wa, wc, sa, sc, pa, pc, ao, co, int(circ),
                   int(ctx.ds), int(avg), int(ne))
            outs.append(gin)
        return (*outs, None, None)


class ReadoutFn(torch.autograd.Function):
    """GlobalAvgPool / GlobalSumPool (linear.py:1771-1801) and Flatten (:1865-1899)."""

    @staticmethod
    def forward(ctx, q, t, c1, c2, kind, ds=False):
        def run(x, bnd):
            if x is None or x.ndim <= bnd or x.numel() == 0:
                return x
            if ds:  # the mean of the positions; GlobalAvgPool scales it by 1 / P once more
                post = 1. / _positions(x, bnd) if kind == 'avg' else 1.
                return O.global_pool(x.contiguous(), bnd, kind != 'sum', post)
            if kind == 'flatten':
                a, c = _ac(x, bnd)
                return O.flatten_fs(_as4(x.contiguous(), bnd), bnd, a, c)
            return O.global_pool(x.contiguous(), bnd, kind == 'avg', 1.)

        ctx.kind, ctx.ds = kind, ds
        ctx.shapes = [None if x is None else tuple(x.shape) for x in (q, t, c1, c2)]
        return run(q, 2), run(t, 2), run(c1, 1), run(c2, 1)

    @staticmethod
    def backward(ctx, gq, gt, gc1, gc2):
        s = L.stream()
        outs = []
        for g, shp, bnd in zip((gq, gt, gc1, gc2), ctx.shapes, (2, 2, 1, 1)):
            if g is None or shp is None or len(shp) <= bnd or int(math.prod(shp)) == 0:
                outs.append(g if (shp is not None and len(shp) <= bnd) else None)
                continue
            m = int(math.prod(shp[bnd:]))
            a = shp[bnd]
            c = shp[bnd + 2] if len(shp) == bnd + 4 else 1
            gin = torch.empty(shp, device=g.device)
            if ctx.ds:
                sc = (1. / m if ctx.kind != 'sum' else 1.) * (1. / m if ctx.kind == 'avg' else 1.)
                L.call('ntg_readout_bwd', s, L.ptr(g.contiguous()), L.ptr(gin),
                       int(math.prod(shp[:bnd])), m, 1, 0, m, sc)
            elif ctx.kind == 'flatten':
                L.call('ntg_readout_bwd', s, L.ptr(g.contiguous()), L.ptr(gin),
                       int(math.prod(shp[:bnd])), a, c, 1, m, 1. / (a * c))
            else:
                L.call('ntg_readout_bwd', s, L.ptr(g.contiguous()), L.ptr(gin),
                       int(math.prod(shp[:bnd])), a, c, 0, m, 1. / m if ctx.kind == 'avg' else 1.)
            outs.append(gin)
        return (*outs, None, None)


# ---------------------------------------------------------------------------
def needs_grad(specs, *xs) -> bool:
    if not torch.is_grad_enabled():
        return False
    if any(isinstance(x, torch.Tensor) and x.requires_grad for x in xs):
        return True
    for sp in specs:
        for key in ('W_std', 'b_std'):
            v = sp.params.get(key)
            if isinstance(v, torch.Tensor) and v.requires_grad:
                return True
    return False


def _sq(v, dev):
    if v is None:
        return torch.zeros((), device=dev)
    if isinstance(v, torch.Tensor):
        return (v.to(dev, torch.float32) ** 2).reshape(())
    return torch.tensor(float(v) ** 2, device=dev)


def _ds_ac(q: torch.Tensor) -> tuple[int, int]:
    """Spatial sizes (A, C) of a diagonal-spatial pair kernel [N1, N2, A(, C)]."""
    return q.shape[2], (q.shape[3] if q.ndim > 3 else 1)


def _pool_geom(q: torch.Tensor, sp):
    """(a, c, windows, strides, pads, output sizes, circular, average, normalize_edges, two_d)
    of a pooling layer applied to the pair kernel q."""
    a, c = _ac(q, 2)
    return _pool_geom_sizes(a, c, sp)


def _pool_geom_sizes(a: int, c: int, sp):
    from .stax import Padding, _pads
    p = sp.params
    ws, st = p['window_shape'], p['strides']
    two_d = len(ws) == 2
    wa, sa = ws[0], st[0]
    wc, sc = (ws[1], st[1]) if two_d else (1, 1)
    pa, ao = _pads(a, wa, sa, p['padding'])
    pc, co = _pads(c, wc, sc, p['padding']) if two_d else (0, 1)
    ne = bool(p['normalize_edges']) and p['padding'] == Padding.SAME
    return (a, c, wa, wc, sa, sc, pa, pc, ao, co, p['padding'] == Padding.CIRCULAR,
            p['pool'] == 'avg', ne, two_d)


def run_ad(specs, x1: torch.Tensor, x2: Optional[torch.Tensor], compute_ntk: bool,
           precision: str = 'fp32', diagonal_spatial: bool = False) -> Kernel:
    """kernel_fn(x1, x2) through the differentiable layer Functions ('mixed': the
    compensated var1 var2 - q^2 in the activation rules and their VJPs;
    diagonal_spatial: the kernels keep only the (h, h, w, w) entries)."""
    from .stax import Padding, _act_struct, _Ctx, _pads
    dev = x1.device
    ctx = _Ctx(precision)
    if x1.ndim > 4:
        raise NotImplementedError('nt_gb300 supports at most two spatial dimensions')
    if specs and specs[0].channel_axis_none and x1.ndim > 2:
        x1 = x1.reshape(x1.shape[0], -1)
        x2 = None if x2 is None else x2.reshape(x2.shape[0], -1)
    shape1 = tuple(x1.shape)
    shape2 = shape1 if x2 is None else tuple(x2.shape)
    ds = bool(diagonal_spatial) and x1.ndim > 2
    is_gaussian, is_reversed = False, False
    skip_next = 0
    if compute_ntk and input_conv_act_fusable(x1, specs, ds):
        # input covariances, first conv and its activation from the images in one pass
        p0 = specs[0].params
        q, t, c1, c2 = InputConvActFn.apply(
            x1.contiguous(), _e(dev) if x2 is None else x2.contiguous(), _sq(p0['W_std'], dev),
            _sq(p0['b_std'], dev), _act_struct(specs[1].params, ctx))
        skip_next = 2
        is_reversed = True
    else:
        q, c1, c2 = InputFn.apply(x1, _e(dev) if x2 is None else x2, ctx.gram_precision, ds)
        t = torch.zeros((), device=dev) if compute_ntk else None
    for idx, sp in enumerate(specs):
        p = sp.params
        if skip_next:  # layers folded into the rule before them
            skip_next -= 1
        elif sp.kind == 'identity':
            pass
        elif sp.kind in ('dense', 'conv'):
            if p['parameterization'] != 'ntk':
                raise NotImplementedError('gradients need the NTK parameterisation')
            w2, b2 = _sq(p['W_std'], dev), _sq(p['b_std'], dev)
            tt = t if t is not None else torch.zeros((), device=dev)
            if sp.kind == 'dense':
                q, tt, c1, c2 = AffineFn.apply(w2, b2, q, tt, c1, c2, ds)
            else:
                nsp = len(p['filter_shape'])
                if nsp > 2:
                    raise NotImplementedError('Conv with 1 or 2 spatial dimensions')
                a, c = _ds_ac(q) if ds else _ac(q, 2)
                fh, sh = p['filter_shape'][0], p['strides'][0]
                fw, sw = (p['filter_shape'][1], p['strides'][1]) if nsp == 2 else (1, 1)
                ph, ao = _pads(a, fh, sh, p['padding'])
                pw, co = _pads(c, fw, sw, p['padding']) if nsp == 2 else (0, 1)
                geom = (fh, fw, sh, sw, ph, pw, ao, co, p['padding'] == Padding.CIRCULAR, nsp)
                nxt = specs[idx + 1] if idx + 1 < len(specs) else None
                nxt2 = specs[idx + 2] if idx + 2 < len(specs) else None
                if (nxt is not None and nxt.kind == 'act' and not nxt.params.get('do_stabilize')
                        and conv_act_fusable(q, geom)):
                    pool_geom = None
                    if nxt2 is not None and nxt2.kind == 'pool':
                        pg = _pool_geom_sizes(32, 32, nxt2)
                        if act_pool_fusable(q, pg):
                            pool_geom = pg
                    q, tt, c1, c2 = ConvActFn.apply(w2, b2, q, tt, c1, c2, geom,
                                                    _act_struct(nxt.params, ctx), pool_geom)
                    skip_next = 2 if pool_geom is not None else 1
                    is_gaussian = False
                    shape1, shape2 = sp.shape_fn(shape1), sp.shape_fn(shape2)
                    is_reversed = not is_reversed
                    t = tt if t is not None else None
                    continue
                q, tt, c1, c2 = ConvFn.apply(w2, b2, q, tt, c1, c2, geom, ds)
                is_reversed = not is_reversed
            t = tt if t is not None else None
            is_gaussian = True
        elif sp.kind == 'act':
            if not is_gaussian:
                raise ValueError('The input to the activation function must be Gaussian, '
                                 'i.e. a random affine transform is required before the '
                                 'activation function.')
            if p.get('do_stabilize'):
                raise NotImplementedError('do_stabilize is not differentiable here')
            tt = t if t is not None else torch.zeros((), device=dev)
            nxt = specs[idx + 1] if idx + 1 < len(specs) else None
            geom = _pool_geom(q, nxt) if (nxt is not None and nxt.kind == 'pool') else None
            if geom is not None and act_pool_fusable(q, geom) and t is not None and tt.ndim > 0:
                q, tt, c1, c2 = ActPoolFn.apply(q, tt, c1, c2, _act_struct(p, ctx), geom)
                skip_next = 1
            else:
                q, tt, c1, c2 = ActFn.apply(q, tt, c1, c2, _act_struct(p, ctx), ds)
            t = tt if t is not None else None
            is_gaussian = False
        elif sp.kind == 'pool':
            geom = _pool_geom_sizes(*_ds_ac(q), sp) if ds else _pool_geom(q, sp)
            tt = t if (t is not None and t.ndim > 0) else None
            q, tt2, c1, c2 = PoolFn.apply(q, tt, c1, c2, geom, ds)
            t = tt2 if tt is not None else t
        elif sp.kind in ('gpool', 'flatten'):
            kind = 'flatten' if sp.kind == 'flatten' else p['pool']
            tt = t if (t is not None and t.ndim > 0) else None
            q, tt2, c1, c2 = ReadoutFn.apply(q, tt, c1, c2, kind, ds)
            t = tt2 if tt is not None else t
            is_reversed = False
            ds = False
            if sp.kind == 'flatten':
                is_gaussian = False
        else:
            raise NotImplementedError(sp.kind)
        shape1, shape2 = sp.shape_fn(shape1), sp.shape_fn(shape2)
    c2o = _opt(c2)
    return Kernel(nngp=from_physical(q, 2, is_reversed, ds),
                  ntk=from_physical(t, 2, is_reversed, ds) if compute_ntk else None,
                  cov1=from_physical(c1, 1, is_reversed, ds),
                  cov2=None if c2o is None else from_physical(c2o, 1, is_reversed, ds),
                  x1_is_x2=x2 is None, is_gaussian=is_gaussian, is_reversed=is_reversed,
                  is_input=False, diagonal_batch=True, diagonal_spatial=ds, shape1=shape1,
                  shape2=shape2)
