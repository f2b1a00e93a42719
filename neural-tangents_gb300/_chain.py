"""Planner and driver of the fused whole-network kernel (ntg_chain_fwd).

A ``serial`` network whose spatial part is a Myrtle-style chain

    [Conv(3x3, SAME, stride 1) + activation?] x n0, AvgPool(2, 2),
    [Conv + activation?] x n1, AvgPool(2, 2), ..., readout

on 32x32 inputs with at most 4 channels is evaluated per (x1[i], x2[j]) pair
in one CTA with nothing but the readout written to HBM. The readout is
GlobalAvgPool (after any number of AvgPool(2, 2)), AvgPool(2, 2) down to 1x1
followed by Flatten, or Flatten right after the last segment. The activation
rules need the per-sample pre-activation variances of every conv layer; those
come from the per-sample chain, run with the materialised layer kernels
(N samples instead of N1*N2 pairs). Layers after the readout run through the
ordinary layer rules on [N1, N2] kernels. Anything else falls back to the
layer-by-layer path.
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import torch

from . import _lib as L
from . import _ops as O
from .kernel import Kernel
from .stax import Padding, _Ctx, _act_struct, _affine_struct

S0 = 32
SELF_CHUNK = 128


@dataclasses.dataclass
class ChainPlan:
    nseg: int
    nconv: list          # conv layers per segment
    convs: list          # (conv params, act params | None, input channels)
    readout: int         # 0 = mean of all entries, 1 = mean of the spatial diagonal
    n_rpools: int        # AvgPools between the last segment and the readout
    readout_kind: str    # 'gpool' | 'flatten'
    post: list           # LayerSpecs after the readout
    spatial: list        # LayerSpecs up to and including the readout
    is_gaussian: bool


def _is_pool2(s) -> bool:
    p = s.params
    return (s.kind == 'pool' and p['pool'] == 'avg' and tuple(p['window_shape']) == (2, 2)
            and tuple(p['strides']) == (2, 2) and p['padding'] in (Padding.VALID, Padding.SAME))


def plan_chain(specs, x_shape, diagonal_spatial: bool) -> Optional[ChainPlan]:
    if diagonal_spatial or len(x_shape) != 4 or tuple(x_shape[1:3]) != (S0, S0):
        return None
    if not 1 <= x_shape[3] <= 4:
        return None
    specs = [s for s in specs if s.kind != 'identity']
    ridx = next((i for i, s in enumerate(specs) if s.kind in ('gpool', 'flatten')), None)
    if ridx is None:
        return None
    spatial, post = specs[:ridx], specs[ridx + 1:]
    readout_spec = specs[ridx]
    if any(s.kind not in ('dense', 'act') for s in post):
        return None
    last_conv = max((i for i, s in enumerate(spatial) if s.kind == 'conv'), default=None)
    if last_conv is None or spatial[0].kind != 'conv':
        return None
    nconv, convs = [0], []
    shape = tuple(x_shape)
    i = 0
    is_gaussian = False
    while i < len(spatial):
        s = spatial[i]
        if s.kind == 'conv':
            p = s.params
            if (tuple(p['filter_shape']) != (3, 3) or tuple(p['strides']) != (1, 1)
                    or p['padding'] != Padding.SAME or nconv[-1] == 3):
                return None
            act = None
            cin = shape[-1]
            shape = s.shape_fn(shape)
            is_gaussian = True
            if i + 1 < len(spatial) and spatial[i + 1].kind == 'act':
                act = spatial[i + 1].params
                if act.get('do_stabilize'):
                    return None  # the stabilised ABRelu rescales by the pre-activation maximum
                is_gaussian = False
                i += 1
            convs.append((p, act, cin))
            nconv[-1] += 1
        elif _is_pool2(s):
            if i < last_conv:
                nconv.append(0)
                if len(nconv) > 3:
                    return None
            else:
                break
            shape = s.shape_fn(shape)
        else:
            return None
        i += 1
    rpools = spatial[i:]
    if not all(_is_pool2(s) for s in rpools):
        return None
    nseg = len(nconv)
    s_last = S0 >> (nseg - 1)
    n_rp = len(rpools)
    if s_last >> n_rp < 1 or (s_last % (1 << n_rp)) != 0:
        return None
    if readout_spec.kind == 'gpool':
        if readout_spec.params['pool'] != 'avg':
            return None
        readout = 0
    else:
        if n_rp == 0:
            readout = 1
        elif s_last >> n_rp == 1:
            readout = 0
        else:
            return None
        is_gaussian = False
    return ChainPlan(nseg=nseg, nconv=nconv, convs=convs, readout=readout, n_rpools=n_rp,
                     readout_kind=readout_spec.kind, post=post, spatial=specs[:ridx + 1],
                     is_gaussian=is_gaussian)


def _program(plan: ChainPlan, channels: int, ctx: _Ctx) -> L.Chain:
    pg = L.Chain()
    pg.nseg = plan.nseg
    pg.s0 = S0
    pg.channels = channels
    pg.readout = plan.readout
    for sgi in range(plan.nseg):
        pg.nconv[sgi] = plan.nconv[sgi]
    off = 0
    li = 0
    for sgi in range(plan.nseg):
        S = S0 >> sgi
        for _ in range(plan.nconv[sgi]):
            p, act, cin = plan.convs[li]
            fan = cin * 9 / p['s'][0] if p['parameterization'] == 'standard' else None
            pg.aff[li] = _affine_struct(p['W_std'], p['b_std'], p['parameterization'], fan)
            pg.act[li] = O.NO_ACT if act is None else _act_struct(act, ctx)
            pg.var_off[li] = off
            off += S * S
            li += 1
    pg.var_stride = off
    return pg


def self_chain(x: torch.Tensor, plan: ChainPlan, ctx: _Ctx):
    """Per-sample kernels through the chain: (variance maps [N, total], readout cov [N])."""
    n = x.shape[0]
    total = sum((S0 >> sgi) ** 2 * plan.nconv[sgi] for sgi in range(plan.nseg))
    var = torch.empty((n, max(total, 1)), device=x.device, dtype=torch.float32)
    covr = torch.empty((n,), device=x.device, dtype=torch.float32)
    for c0 in range(0, n, SELF_CHUNK):
        xc = x[c0:c0 + SELF_CHUNK].contiguous()
        m = xc.shape[0]
        cov = O.input_fs(xc, None)
        off = 0
        li = 0
        S = S0
        for sgi in range(plan.nseg):
            for _ in range(plan.nconv[sgi]):
                p, act, cin = plan.convs[li]
                fan = cin * 9 / p['s'][0] if p['parameterization'] == 'standard' else None
                aff = _affine_struct(p['W_std'], p['b_std'], p['parameterization'], fan)
                pre, _ = O.conv_fs(cov, None, m, 0, S, S, 3, 3, 1, 1, 1, 1, S, S, False, aff,
                                   O.NO_ACT, O.NO_VAR, O.NO_VAR, False, (m,))
                d = torch.diagonal(torch.diagonal(pre, dim1=1, dim2=2), dim1=1, dim2=2)
                var[c0:c0 + m, off:off + S * S].copy_(d.reshape(m, S * S))
                if act is not None:
                    v = O.var_view(pre, False)
                    cov, _ = O.affine_act(pre, None, m, 0, S, S, False, False, O.IDENTITY_AFFINE,
                                          _act_struct(act, ctx), v, v, False)
                else:
                    cov = pre
                off += S * S
                li += 1
            if sgi < plan.nseg - 1:
                cov = O.pool(cov, m, S, S, 2, 2, 2, 2, 0, 0, S // 2, S // 2, False, False, True,
                             False, (m, S // 2, S // 2, S // 2, S // 2))
                S //= 2
        if plan.readout == 0:
            covr[c0:c0 + m] = O.global_pool(cov, 1, True, 1.)
        else:
            covr[c0:c0 + m] = O.flatten_fs(cov, 1, S, S)
    return var, covr


def try_fused(kfn, x1: torch.Tensor, x2: Optional[torch.Tensor], diagonal_spatial: bool,
              compute_ntk: bool, ctx: _Ctx) -> Optional[Kernel]:
    plan = plan_chain(kfn.specs, tuple(x1.shape), diagonal_spatial)
    if plan is None or (x2 is not None and tuple(x2.shape[1:]) != tuple(x1.shape[1:])):
        return None
    k = run_fused(plan, x1, x2, ctx)
    k = kfn.apply_kernel(k, ctx, specs=plan.post)
    if not compute_ntk:
        k = k.replace(ntk=None)
    return k


def run_fused(plan: ChainPlan, x1: torch.Tensor, x2: Optional[torch.Tensor], ctx: _Ctx,
              out: Optional[tuple] = None, rows=None, cols=None, selfs=None,
              x1_is_x2: Optional[bool] = None) -> Kernel:
    """Readout Kernel of the chain for all pairs of x1 x x2 (x2 None: x1 x x1).

    ``x1_is_x2`` given skips the element-wise comparison of x1 and x2 (a host
    synchronisation, not allowed while a CUDA graph is being captured)."""
    pg = _program(plan, x1.shape[-1], ctx)
    if selfs is None:
        var1, cov1 = self_chain(x1, plan, ctx)
        var2, cov2 = (var1, None) if x2 is None else self_chain(x2, plan, ctx)
    else:
        var1, cov1, var2, cov2 = selfs
    xb = x1 if x2 is None else x2
    n1, n2 = x1.shape[0], xb.shape[0]
    if out is None:
        out_q = torch.empty((n1, n2), device=x1.device, dtype=torch.float32)
        out_t = torch.empty((n1, n2), device=x1.device, dtype=torch.float32)
    else:
        out_q, out_t = out
    if x2 is None:
        # K(x, x): the pairs i <= j once, mirrored (one launch over the triangle)
        O.chain_fwd_sym(pg, x1, 0, n1, 0, n1, var1, out_q, out_t, n2)
    else:
        O.chain_fwd(pg, x1, xb, 0, n1, 0, n2, var1, var2, out_q, out_t, n2)
    shape1 = tuple(x1.shape)
    shape2 = tuple(xb.shape)
    for s in plan.spatial:
        shape1, shape2 = s.shape_fn(shape1), s.shape_fn(shape2)
    return Kernel(nngp=out_q, ntk=out_t, cov1=cov1, cov2=cov2,
                  x1_is_x2=(x2 is None or bool(torch.equal(x1, x2))) if x1_is_x2 is None
                  else bool(x1_is_x2), is_gaussian=plan.is_gaussian,
                  is_reversed=False, is_input=False, diagonal_batch=True, diagonal_spatial=False,
                  shape1=shape1, shape2=shape2)
