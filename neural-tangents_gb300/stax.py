"""nt_gb300.stax -- the analytic-kernel layer API of ``neural_tangents.stax``.

Every layer returns the reference's ``(init_fn, apply_fn, kernel_fn)`` triple
(neural_tangents/_src/stax/requirements.py:50-78). ``kernel_fn`` keeps the
reference signature ``kernel_fn(x1_or_kernel, x2=None, get=None, *,
diagonal_batch=None, diagonal_spatial=None, **kwargs)`` (requirements.py:955-1054)
and returns a ``Kernel``, one array (``get`` a string) or an ``AnalyticKernel``
namedtuple (``get`` a tuple).  All kernel arithmetic runs in the sm_103a
kernels of libntgb300.so; inputs may be numpy arrays or torch tensors and are
moved to the current CUDA device.

Extra keyword (not in the reference): ``precision='fp32' | 'mixed'``.
'fp32' follows the reference's float32 arithmetic; 'mixed' evaluates
var1*var2 - q^2 compensated and the flat first-layer Gram on the tensor cores
with split BF16 products.
"""
from __future__ import annotations

import dataclasses
import enum
import math
from typing import Any, Callable, Optional, Sequence

import numpy as np
import torch

from . import _lib as L
from . import _ops as O
from .kernel import Kernel, analytic_kernel, from_physical, to_physical

# ---------------------------------------------------------------------------
# Requirement algebra (requirements.py:401-515)
# ---------------------------------------------------------------------------


class Bool(enum.IntEnum):
    """Three-valued requirement flag; `&` is the smaller of the two (requirements.py)."""
    NO = 0
    MAYBE = 1
    YES = 2

    def __and__(self, other: 'Bool') -> 'Bool':
        return Bool(min(int(self), int(other)))

    __rand__ = __and__


@dataclasses.dataclass(frozen=True)
class Diagonal:
    """Whether a layer accepts, and keeps, diagonal-only kernels: `a >> b` (and `b << a`) is
    the requirement of b applied after a, `a & b` that of parallel branches."""
    input: Bool = Bool.YES
    output: Bool = Bool.NO

    def __rshift__(self, other: 'Diagonal') -> 'Diagonal':
        if self.output == Bool.YES:
            return self
        if self.output > Bool.NO and other.input > Bool.NO:
            inp = self.input
        elif self.output == Bool.NO and other.input < Bool.YES:
            inp = Bool.NO
        else:
            inp = min(self.input, other.input)
        return Diagonal(input=inp, output=other.output)

    def __lshift__(self, other: 'Diagonal') -> 'Diagonal':
        return other >> self

    def __and__(self, other: 'Diagonal') -> 'Diagonal':
        return Diagonal(input=Bool(self.input) & Bool(other.input),
                        output=Bool(self.output) & Bool(other.output))

    __rand__ = __and__

    def __bool__(self) -> bool:
        return self.input == Bool.YES and self.output > Bool.NO


class Padding(enum.Enum):
    CIRCULAR = 'CIRCULAR'
    SAME = 'SAME'
    VALID = 'VALID'


# ---------------------------------------------------------------------------
# Layer descriptions
# ---------------------------------------------------------------------------


@dataclasses.dataclass
class LayerSpec:
    """What a layer is, for the kernel rules and the fused-chain planner."""
    kind: str                      # dense | conv | act | pool | gpool | flatten | identity
    diag: Diagonal
    params: dict
    shape_fn: Callable[[tuple], tuple]
    channel_axis_none: bool = False


class _Ctx:
    """Per-call options threaded through the layer rules."""

    def __init__(self, precision: str = 'fp32'):
        if precision not in ('fp32', 'mixed'):
            raise ValueError(f'precision must be "fp32" or "mixed", got {precision!r}')
        self.precision = precision

    @property
    def compensated(self) -> int:
        return 1 if self.precision == 'mixed' else 0

    @property
    def gram_precision(self) -> int:
        """ntg_gram precision: 1 (split-BF16 tcgen05) for the mixed form."""
        return 1 if self.precision == 'mixed' else 0


def _act_struct(p: dict, ctx: _Ctx, stabilize: float = 0.) -> L.Act:
    if p['fn'] == 'abrelu':
        return L.Act(L.NTG_ACT_ABRELU, p['a'], p['b'], 0., ctx.compensated, stabilize)
    if p['fn'] == 'erf':
        return L.Act(L.NTG_ACT_ERF, p['a'], p['b'], p['c'], ctx.compensated, 0.)
    if p['fn'] == 'sin':  # the kernels take cos(2 c), computed here in double precision
        return L.Act(L.NTG_ACT_SIN, p['a'], p['b'], math.cos(2. * p['c']), 0, 0.)
    if p['fn'] == 'rbf':
        return L.Act(L.NTG_ACT_RBF, p['gamma'], 0., 0., 0, 0.)
    if p['fn'] == 'gelu':
        return L.Act(L.NTG_ACT_GELU, 0., 0., 0., 0, 0.)
    raise ValueError(p['fn'])


def _affine_struct(W_std, b_std, parameterization, fan_in_over_s0=None) -> L.Affine:
    w2 = float(W_std) ** 2
    b2 = 0. if b_std is None else float(b_std) ** 2
    if parameterization == 'ntk':
        return O.affine(w2, b2, w2, 1., 0., True)
    if parameterization == 'standard':
        return O.affine(w2, b2, w2, float(fan_in_over_s0), 1. if b_std is not None else 0., False)
    raise ValueError(f'Parameterization not supported: {parameterization}')


def _pads(n: int, f: int, s: int, padding: Padding) -> tuple[int, int]:
    """lax.padtype_to_pads: (low pad, output size)."""
    if padding == Padding.VALID:
        return 0, (n - f) // s + 1
    out = -(-n // s)
    total = max((out - 1) * s + f - n, 0)
    return total // 2, out


# ---------------------------------------------------------------------------
# Layer rules on Kernels (the product path)
# ---------------------------------------------------------------------------


def _tensors(k: Kernel):
    """Physical (un-reversed, contiguous) nngp, ntk, cov1, cov2 of a Kernel."""
    ds, rv = k.diagonal_spatial, k.is_reversed
    ntk = k.ntk
    if ntk is not None and ntk.ndim == 0:
        ntk = None
    return (to_physical(k.nngp, 2, rv, ds), to_physical(ntk, 2, rv, ds),
            to_physical(k.cov1, 1, rv, ds), to_physical(k.cov2, 1, rv, ds))


def _has_ntk(k: Kernel) -> bool:
    return k.ntk is not None


def _zero_ntk(k: Kernel) -> bool:
    return k.ntk is not None and k.ntk.ndim == 0


def _finish(k: Kernel, nngp, ntk, cov1, cov2, **kw) -> Kernel:
    if ntk is None and _zero_ntk(k):
        ntk = k.ntk  # the scalar-zero NTK of an input kernel passes through unchanged
    rv = kw.get('is_reversed', k.is_reversed)
    ds = kw.get('diagonal_spatial', k.diagonal_spatial)
    return k.replace(nngp=from_physical(nngp, 2, rv, ds), ntk=from_physical(ntk, 2, rv, ds),
                     cov1=from_physical(cov1, 1, rv, ds), cov2=from_physical(cov2, 1, rv, ds),
                     **kw)


def _dense_rule(k: Kernel, p: dict, ctx: _Ctx, act: Optional[dict] = None) -> Kernel:
    """linear.py:899-926 (+ an activation rule fused after it)."""
    q, t, c1, c2 = _tensors(k)
    ds = k.diagonal_spatial
    input_width = k.shape1[-1] / p['s'][0] if p['parameterization'] == 'standard' else None
    aff = _affine_struct(p['W_std'], p['b_std'], p['parameterization'], input_width)
    a, c = O.spatial_ac(q, 2, ds)
    n1, n2 = q.shape[0], q.shape[1]

    def cov_affine(cv):
        if cv is None:
            return None
        out, _ = O.affine_act(cv, None, cv.shape[0], 0, a, c, ds, True, aff, O.NO_ACT, O.NO_VAR,
                              O.NO_VAR, False)
        return out

    c1n, c2n = cov_affine(c1), cov_affine(c2)
    want_t = _has_ntk(k)
    if act is None:
        qn, tn = O.affine_act(q, t, n1 * n2, n2, a, c, ds, True, aff, O.NO_ACT, O.NO_VAR,
                              O.NO_VAR, want_t)
        return _finish(k, qn, tn, c1n, c2n, is_gaussian=True, is_input=False)
    st = _stabilizer(act, ctx, None)
    ast = _act_struct(act, ctx, st)
    v1 = O.var_view(c1n, ds)
    v2 = O.var_view(c2n if c2n is not None else c1n, ds)
    qn, tn = O.affine_act(q, t, n1 * n2, n2, a, c, ds, True, aff, ast, v1, v2, want_t)
    c1o, c2o = _act_cov(c1n, ast, ds, a, c), _act_cov(c2n, ast, ds, a, c)
    return _finish(k, qn, tn, c1o, c2o, is_gaussian=False, is_input=False)


def _stabilizer(act: dict, ctx: _Ctx, nngp: Optional[torch.Tensor]) -> float:
    if act['fn'] != 'abrelu' or not act.get('do_stabilize'):
        return 0.
    if nngp is None:
        raise NotImplementedError('do_stabilize needs the pre-activation nngp')
    return max(O.max_abs(nngp), 1e-12)


def _act_cov(cv, ast, ds, a, c):
    """Activation rule on a per-sample kernel, using its own diagonal."""
    if cv is None:
        return None
    v = O.var_view(cv, ds)
    out, _ = O.affine_act(cv, None, cv.shape[0], 0, a, c, ds, False, O.IDENTITY_AFFINE, ast, v, v,
                          False)
    return out


def _act_rule(k: Kernel, p: dict, ctx: _Ctx) -> Kernel:
    """elementwise.py:1250-1275 + ABRelu :423-477 / Erf :67-112."""
    if not k.is_gaussian:
        raise ValueError('The input to the activation function must be Gaussian, '
                         'i.e. a random affine transform is required before the '
                         'activation function.')
    q, t, c1, c2 = _tensors(k)
    ds = k.diagonal_spatial
    a, c = O.spatial_ac(q, 2, ds)
    ast = _act_struct(p, ctx, _stabilizer(p, ctx, q))
    v1 = O.var_view(c1, ds)
    v2 = O.var_view(c2 if c2 is not None else c1, ds)
    n1, n2 = q.shape[0], q.shape[1]
    if _zero_ntk(k):
        t_out_zero = True
    else:
        t_out_zero = False
    qn, tn = O.affine_act(q, t, n1 * n2, n2, a, c, ds, False, O.IDENTITY_AFFINE, ast, v1, v2,
                          t is not None)
    ntk = tn
    if t_out_zero:
        ntk = k.ntk  # scalar zero stays zero
    return _finish(k, qn, ntk, _act_cov(c1, ast, ds, a, c), _act_cov(c2, ast, ds, a, c),
                   is_gaussian=False)


def _conv_geometry(p: dict, a: int, c: int, two_d: bool):
    fs, st = p['filter_shape'], p['strides']
    fh, sh = fs[0], st[0]
    fw, sw = (fs[1], st[1]) if two_d else (1, 1)
    ph, ao = _pads(a, fh, sh, p['padding'])
    if two_d:
        pw, co = _pads(c, fw, sw, p['padding'])
    else:
        pw, co = 0, 1
    return fh, fw, sh, sw, ph, pw, ao, co


def _conv_rule(k: Kernel, p: dict, ctx: _Ctx, act: Optional[dict] = None) -> Kernel:
    """linear.py:1321-1424 with the full-spatial loop :3115-3207/:3341-3378 or the
    diagonal-spatial rule :3381-3437 (+ an activation rule fused after it)."""
    q, t, c1, c2 = _tensors(k)
    ds = k.diagonal_spatial
    nsp = len(p['filter_shape'])
    if nsp > 2:
        raise NotImplementedError('nt_gb300 supports Conv with 1 or 2 spatial dimensions')
    a, c = O.spatial_ac(q, 2, ds)
    fh, fw, sh, sw, ph, pw, ao, co = _conv_geometry(p, a, c, nsp == 2)
    circular = p['padding'] == Padding.CIRCULAR
    fan = None
    if p['parameterization'] == 'standard':
        fan = k.shape1[-1] * int(np.prod(p['filter_shape'])) / p['s'][0]
    aff = _affine_struct(p['W_std'], p['b_std'], p['parameterization'], fan)
    n1, n2 = q.shape[0], q.shape[1]
    want_t = _has_ntk(k)
    if ds:
        has_c = q.ndim == 4

        def cds(x, xt, batch, lead, wt):
            return O.conv_ds(x, xt, batch, a, c, fh, fw, sh, sw, ph, pw, ao, co, circular, aff, wt,
                             lead, has_c)
        c1n = cds(c1, None, c1.shape[0], (c1.shape[0],), False)[0]
        c2n = None if c2 is None else cds(c2, None, c2.shape[0], (c2.shape[0],), False)[0]
        qn, tn = cds(q, t, n1 * n2, (n1, n2), want_t)
        out = _finish(k, qn, tn, c1n, c2n, is_gaussian=True, is_input=False)
        return out if act is None else _act_rule(out, act, ctx)

    def cfs(x, xt, batch, nn2, lead, wt, ast=O.NO_ACT, v1=O.NO_VAR, v2=O.NO_VAR):
        r = O.conv_fs(x, xt, batch, nn2, a, c, fh, fw, sh, sw, ph, pw, ao, co, circular, aff, ast,
                      v1, v2, wt, lead)
        if nsp == 1:
            r = tuple(None if y is None else y.reshape(lead + (ao, ao)) for y in r)
        return r

    def to4(x, bnd):  # view 1-D spatial kernels as [.., A, A, 1, 1]
        if x is None or nsp == 2:
            return x
        return x.reshape(tuple(x.shape[:bnd]) + (a, a, 1, 1))

    q4, t4, c14, c24 = to4(q, 2), to4(t, 2), to4(c1, 1), to4(c2, 1)
    c1n = cfs(c14, None, c1.shape[0], 0, (c1.shape[0],), False)[0]
    c2n = None if c2 is None else cfs(c24, None, c2.shape[0], 0, (c2.shape[0],), False)[0]
    rev = not k.is_reversed
    if act is None or act['fn'] == 'abrelu' and act.get('do_stabilize'):
        qn, tn = cfs(q4, t4, n1 * n2, n2, (n1, n2), want_t)
        out = _finish(k, qn, tn, c1n, c2n, is_gaussian=True, is_input=False, is_reversed=rev)
        return out if act is None else _act_rule(out, act, ctx)
    ast = _act_struct(act, ctx)
    c1v = to4(c1n, 1)
    c2v = to4(c2n, 1)
    v1 = O.var_view(c1v, False)
    v2 = O.var_view(c2v if c2v is not None else c1v, False)
    qn, tn = cfs(q4, t4, n1 * n2, n2, (n1, n2), want_t, ast, v1, v2)
    aa, cc = (ao, co)
    c1o = _act_cov(c1v, ast, False, aa, cc)
    c2o = None if c2v is None else _act_cov(c2v, ast, False, aa, cc)
    if nsp == 1:
        c1o = c1o.reshape(c1n.shape)
        c2o = None if c2o is None else c2o.reshape(c2n.shape)
    return _finish(k, qn, tn, c1o, c2o, is_gaussian=False, is_input=False, is_reversed=rev)


def _pool_rule(k: Kernel, p: dict, ctx: _Ctx) -> Kernel:
    """linear.py:1631-1664 / _pool_kernel :3499-3572."""
    q, t, c1, c2 = _tensors(k)
    ds = k.diagonal_spatial
    a, c = O.spatial_ac(q, 2, ds)
    ws, st = p['window_shape'], p['strides']
    two_d = len(ws) == 2
    if len(ws) > 2:
        raise NotImplementedError('nt_gb300 supports pooling over 1 or 2 spatial dimensions')
    wa, sa = ws[0], st[0]
    wc, sc = (ws[1], st[1]) if two_d else (1, 1)
    pa, ao = _pads(a, wa, sa, p['padding'])
    pc, co = _pads(c, wc, sc, p['padding']) if two_d else (0, 1)
    circular = p['padding'] == Padding.CIRCULAR
    avg = p['pool'] == 'avg'
    ne = bool(p['normalize_edges']) and p['padding'] == Padding.SAME

    def run(x, bnd):
        if x is None:
            return None
        lead = tuple(x.shape[:bnd])
        batch = int(np.prod(lead))
        if ds:
            shape = lead + ((ao, co) if two_d else (ao,))
        else:
            shape = lead + ((ao, ao, co, co) if two_d else (ao, ao))
        return O.pool(x, batch, a, c, wa, wc, sa, sc, pa, pc, ao, co, circular, ds, avg, ne, shape)

    return _finish(k, run(q, 2), run(t, 2), run(c1, 1), run(c2, 1))


def _gpool_rule(k: Kernel, p: dict, ctx: _Ctx) -> Kernel:
    """linear.py:1771-1801."""
    q, t, c1, c2 = _tensors(k)
    avg = p['pool'] == 'avg'

    def run(x, bnd):
        if x is None:
            return None
        if x.ndim == bnd:
            return x
        scale = 1.
        if k.diagonal_spatial and avg:
            scale = 1. / float(np.prod(x.shape[bnd:]))
        return O.global_pool(x, bnd, avg, scale)

    return _finish(k, run(q, 2), run(t, 2), run(c1, 1), run(c2, 1), is_reversed=False)


def _flatten_rule(k: Kernel, p: dict, ctx: _Ctx) -> Kernel:
    """linear.py:1865-1899."""
    q, t, c1, c2 = _tensors(k)
    ds = k.diagonal_spatial

    def run(x, bnd):
        if x is None or x.ndim == bnd:
            return x
        if ds:
            return O.global_pool(x, bnd, True, 1.)
        a, c = O.spatial_ac(x, bnd, False)
        if x.ndim == bnd + 2:
            x = x.reshape(tuple(x.shape[:bnd]) + (a, a, 1, 1))
        return O.flatten_fs(x, bnd, a, c)

    return _finish(k, run(q, 2), run(t, 2), run(c1, 1), run(c2, 1), is_gaussian=False,
                   is_reversed=False, diagonal_spatial=False)


RULES = {'dense': _dense_rule, 'conv': _conv_rule, 'act': _act_rule, 'pool': _pool_rule,
         'gpool': _gpool_rule, 'flatten': _flatten_rule}

# ---------------------------------------------------------------------------
# Finite-width functions (init_fn / apply_fn) -- torch, for shape inference and
# Monte-Carlo checks of the analytic kernels.
# ---------------------------------------------------------------------------


def _gen(rng) -> torch.Generator:
    g = torch.Generator(device='cpu')
    g.manual_seed(int(rng) if not hasattr(rng, 'shape') else int(np.asarray(rng).ravel()[-1]))
    return g


def _apply_spec(spec: LayerSpec, params, x: torch.Tensor) -> torch.Tensor:
    p = spec.params
    if spec.kind == 'identity':
        return x
    if spec.kind == 'dense':
        W, b = params
        n = x.shape[-1]
        if p['parameterization'] == 'ntk':
            out = p['W_std'] / math.sqrt(n) * (x @ W)
            return out if b is None else out + p['b_std'] * b
        out = (x @ W) / math.sqrt(p['s'][0])
        return out if b is None else out + b
    if spec.kind == 'conv':
        W, b = params
        nsp = len(p['filter_shape'])
        xc = torch.movedim(x, -1, 1)
        if p['padding'] == Padding.CIRCULAR:
            pads = []
            for d in reversed(range(nsp)):
                lo, _ = _pads(xc.shape[2 + d], p['filter_shape'][d], p['strides'][d], Padding.SAME)
                out_n = -(-xc.shape[2 + d] // p['strides'][d])
                tot = max((out_n - 1) * p['strides'][d] + p['filter_shape'][d] - xc.shape[2 + d], 0)
                pads += [lo, tot - lo]
            xc = torch.nn.functional.pad(xc, pads, mode='circular')
            padding = 0
        elif p['padding'] == Padding.SAME:
            pads = []
            for d in reversed(range(nsp)):
                out_n = -(-xc.shape[2 + d] // p['strides'][d])
                tot = max((out_n - 1) * p['strides'][d] + p['filter_shape'][d] - xc.shape[2 + d], 0)
                pads += [tot // 2, tot - tot // 2]
            xc = torch.nn.functional.pad(xc, pads)
            padding = 0
        else:
            padding = 0
        conv = torch.nn.functional.conv2d if nsp == 2 else torch.nn.functional.conv1d
        fan_in = x.shape[-1] * int(np.prod(p['filter_shape']))
        norm = p['W_std'] / math.sqrt(fan_in) if p['parameterization'] == 'ntk' else \
            1. / math.sqrt(p['s'][0])
        out = norm * conv(xc, W, stride=tuple(p['strides']), padding=padding)
        out = torch.movedim(out, 1, -1)
        if b is not None:
            out = out + (p['b_std'] if p['parameterization'] == 'ntk' else 1.) * b
        return out
    if spec.kind == 'act':
        if p['fn'] == 'abrelu':
            return p['a'] * torch.clamp(x, max=0) + p['b'] * torch.clamp(x, min=0)
        if p['fn'] == 'sin':
            return p['a'] * torch.sin(p['b'] * x + p['c'])
        if p['fn'] == 'rbf':
            return math.sqrt(2.) * torch.sin(math.sqrt(2. * p['gamma']) * x + math.pi / 4)
        if p['fn'] == 'gelu':
            return torch.nn.functional.gelu(x, approximate='tanh' if p['approximate'] else 'none')
        return p['a'] * torch.erf(p['b'] * x) + p['c']
    if spec.kind == 'pool':
        nsp = len(p['window_shape'])
        xc = torch.movedim(x, -1, 1)
        if p['padding'] != Padding.VALID:
            pads = []
            for d in reversed(range(nsp)):
                out_n = -(-xc.shape[2 + d] // p['strides'][d])
                tot = max((out_n - 1) * p['strides'][d] + p['window_shape'][d] - xc.shape[2 + d], 0)
                pads += [tot // 2, tot - tot // 2]
            mode = 'circular' if p['padding'] == Padding.CIRCULAR else 'constant'
            xc = torch.nn.functional.pad(xc, pads, mode=mode)
        pool = torch.nn.functional.avg_pool2d if nsp == 2 else torch.nn.functional.avg_pool1d
        out = pool(xc, tuple(p['window_shape']), tuple(p['strides']))
        if p['pool'] == 'sum':
            out = out * float(np.prod(p['window_shape']))
        return torch.movedim(out, 1, -1)
    if spec.kind == 'gpool':
        axes = tuple(range(1, x.ndim - 1))
        return x.mean(axes) if p['pool'] == 'avg' else x.sum(axes)
    if spec.kind == 'flatten':
        return x.reshape(x.shape[0], -1)
    raise NotImplementedError(spec.kind)


def _init_spec(spec: LayerSpec, g: torch.Generator, input_shape: tuple):
    p = spec.params
    out_shape = spec.shape_fn(tuple(input_shape))
    if spec.kind == 'dense':
        n = input_shape[-1]
        W = torch.randn((n, out_shape[-1]), generator=g)
        b = None if p['b_std'] is None else torch.randn((out_shape[-1],), generator=g)
        if p['parameterization'] == 'standard':
            W = W * p['W_std'] / math.sqrt(n / p['s'][0])
            b = None if b is None else b * p['b_std']
        return out_shape, (W, b)
    if spec.kind == 'conv':
        cin = input_shape[-1]
        W = torch.randn((out_shape[-1], cin) + tuple(p['filter_shape']), generator=g)
        b = None if p['b_std'] is None else torch.randn((out_shape[-1],), generator=g)
        if p['parameterization'] == 'standard':
            fan = cin * int(np.prod(p['filter_shape']))
            W = W * p['W_std'] / math.sqrt(fan / p['s'][0])
            b = None if b is None else b * p['b_std']
        return out_shape, (W, b)
    return out_shape, ()


# ---------------------------------------------------------------------------
# kernel_fn objects
# ---------------------------------------------------------------------------


def _as_input(x) -> torch.Tensor:
    dev = L.require_cuda()
    if isinstance(x, torch.Tensor):
        return x.to(device=dev, dtype=torch.float32).contiguous()
    return torch.as_tensor(np.asarray(x), dtype=torch.float32, device=dev).contiguous()


def _normalize_get(get):
    if get is None:
        return None, None
    if isinstance(get, str):
        return (get,), get
    return tuple(get), None


def _input_kernel(x1: torch.Tensor, x2: Optional[torch.Tensor], diagonal_spatial: bool,
                  compute_ntk: bool, channel_axis_none: bool, ctx: _Ctx) -> Kernel:
    """requirements.py:641-830 (batch axis 0, channel axis -1)."""
    shape1 = tuple(x1.shape)
    shape2 = shape1 if x2 is None else tuple(x2.shape)
    if x1.ndim < 2:
        raise ValueError(f'Inputs must be at least 2D (a batch dimension and a '
                         f'channel/feature dimension), got {x1.ndim}.')
    if channel_axis_none:
        x1 = x1.reshape(x1.shape[0], -1)
        x2 = None if x2 is None else x2.reshape(x2.shape[0], -1)
    if x1.ndim == 2:
        diagonal_spatial = False
    prec = 1 if ctx.precision == 'mixed' else 0
    xb = x1 if x2 is None else x2
    if x1.ndim == 2:
        nngp = O.gram(x1, xb, prec)
        if x2 is None:
            # the self covariances are the Gram diagonal itself, so that a self
            # pair has var1 * var2 - nngp^2 == 0 exactly
            cov1 = torch.diagonal(nngp).contiguous()
        else:
            cov1 = O.cov_diag(x1)
        cov2 = None if x2 is None else O.cov_diag(x2)
    elif diagonal_spatial:
        # per-position channel dot products [N1, N2, *spatial]
        nngp = O.input_ds(x1, xb)
        cov1 = O.input_ds(x1, None)
        cov2 = None if x2 is None else O.input_ds(x2, None)
    else:
        if x1.ndim > 4:
            raise NotImplementedError('nt_gb300 supports at most two spatial dimensions')
        y1 = x1 if x1.ndim == 4 else x1.unsqueeze(2)
        yb = xb if xb.ndim == 4 else xb.unsqueeze(2)
        nngp = O.input_fs(y1, yb)
        cov1 = O.input_fs(y1, None)
        cov2 = None if x2 is None else O.input_fs(yb, None)
        if x1.ndim == 3:
            a = x1.shape[1]
            nngp = nngp.reshape(nngp.shape[0], nngp.shape[1], a, a)
            cov1 = cov1.reshape(cov1.shape[0], a, a)
            cov2 = None if cov2 is None else cov2.reshape(cov2.shape[0], a, a)
    ntk = torch.zeros((), device=x1.device) if compute_ntk else None
    x1_is_x2 = x2 is None or (x1.shape == x2.shape and bool(torch.equal(x1, x2)))
    return Kernel(nngp=nngp, ntk=ntk, cov1=cov1, cov2=cov2, x1_is_x2=x1_is_x2,
                  is_gaussian=False, is_reversed=False, is_input=False, diagonal_batch=True,
                  diagonal_spatial=bool(diagonal_spatial), shape1=shape1, shape2=shape2)


class KernelFn:
    """An analytic ``kernel_fn`` (requirements.py:912-1054) over a layer list."""

    def __init__(self, specs: Sequence[LayerSpec], name: str):
        self.specs = list(specs)
        self.__name__ = name
        req = None
        for s in self.specs:
            req = s.diag if req is None else (req >> s.diag)
        self.diagonal = Diagonal() if req is None else req
        self.input_req = {'diagonal_batch': True, 'diagonal_spatial': self.diagonal,
                          'batch_axis': 0, 'channel_axis': -1}

    # -- Kernel -> Kernel ---------------------------------------------------
    def apply_kernel(self, k: Kernel, ctx: _Ctx, specs=None) -> Kernel:
        specs = self.specs if specs is None else specs
        i = 0
        while i < len(specs):
            s = specs[i]
            nxt = specs[i + 1] if i + 1 < len(specs) else None
            if s.kind in ('dense', 'conv') and nxt is not None and nxt.kind == 'act' \
                    and not nxt.params.get('do_stabilize'):
                k = RULES[s.kind](k, s.params, ctx, act=nxt.params)
                k = k.replace(shape1=nxt.shape_fn(s.shape_fn(k.shape1)),
                              shape2=nxt.shape_fn(s.shape_fn(k.shape2)))
                i += 2
                continue
            if s.kind != 'identity':
                k = RULES[s.kind](k, s.params, ctx)
            k = k.replace(shape1=s.shape_fn(k.shape1), shape2=s.shape_fn(k.shape2))
            i += 1
        return k

    def _empty(self, x1, x2, get, precision, diagonal_spatial):
        """Kernels of an empty batch: evaluated on one stand-in input per empty side, then
        sliced to zero rows/columns, so that shapes and dtypes are those of the rule."""
        n1 = x1.shape[0]
        n2 = n1 if x2 is None else x2.shape[0]
        p1 = x1 if n1 else torch.zeros((1,) + tuple(x1.shape[1:]), device=x1.device)
        p2 = None if x2 is None else (x2 if n2 else torch.zeros((1,) + tuple(x2.shape[1:]),
                                                              device=x2.device))
        out = self(p1, p2, get, precision=precision, diagonal_spatial=diagonal_spatial)

        def cut(name, v):
            if not isinstance(v, torch.Tensor) or v.ndim == 0:
                return v
            if name == 'cov1':
                return v[:n1]
            if name == 'cov2':
                return v[:n2]
            return v[:n1, :n2] if v.ndim >= 2 else v[:n1]

        if isinstance(out, torch.Tensor):
            return cut(get, out)
        if isinstance(out, Kernel):
            return out.replace(nngp=cut('nngp', out.nngp), ntk=cut('ntk', out.ntk),
                               cov1=cut('cov1', out.cov1), cov2=cut('cov2', out.cov2))
        return type(out)(*[cut(n, v) for n, v in zip(out._fields, out)])

    def __call__(self, x1_or_kernel, x2=None, get=None, *, pattern=None, mask_constant=None,
                 diagonal_batch=None, diagonal_spatial=None, precision='fp32', **kwargs):
        with L.boundary('kernel_fn'):
            return self._call(x1_or_kernel, x2, get, pattern=pattern,
                              mask_constant=mask_constant, diagonal_batch=diagonal_batch,
                              diagonal_spatial=diagonal_spatial, precision=precision, **kwargs)

    def _call(self, x1_or_kernel, x2=None, get=None, *, pattern=None, mask_constant=None,
              diagonal_batch=None, diagonal_spatial=None, precision='fp32', **kwargs):
        if mask_constant is not None:
            raise NotImplementedError('masked inputs are not supported by nt_gb300')
        if diagonal_batch is False:
            raise NotImplementedError('nt_gb300 computes diagonal_batch=True kernels')
        ctx = _Ctx(precision)
        names, single = _normalize_get(get)
        if isinstance(x1_or_kernel, Kernel) and x2 is None:
            k = self.apply_kernel(x1_or_kernel, ctx)
        else:
            ds = bool(self.diagonal) if diagonal_spatial is None else bool(diagonal_spatial)
            if diagonal_spatial is True and self.diagonal.input == Bool.NO:
                raise ValueError(f'Asked to compute `kernel_fn` output with `diagonal_spatial == '
                                 f'True`, while `kernel_fn` requires `diagonal_spatial == '
                                 f'{self.diagonal}`.')
            compute_ntk = names is None or 'ntk' in names
            x1 = _as_input(x1_or_kernel)
            x2t = None if x2 is None else _as_input(x2)
            if x1.shape[0] == 0 or (x2t is not None and x2t.shape[0] == 0):
                return self._empty(x1, x2t, get, precision, diagonal_spatial)
            from . import _autograd, _chain
            if _autograd.needs_grad(self.specs, x1, x2t):
                k = _autograd.run_ad(self.specs, x1, x2t, compute_ntk, precision, ds)
                if names is None:
                    return k
                vals = tuple(getattr(k, n) for n in names)
                return vals[0] if single is not None else analytic_kernel(names, vals)
            k = _chain.try_fused(self, x1, x2t, ds, compute_ntk, ctx)
            if k is None:
                cnone = bool(self.specs) and self.specs[0].channel_axis_none
                k = _input_kernel(x1, x2t, ds, compute_ntk, cnone, ctx)
                k = self.apply_kernel(k, ctx)
        if names is None:
            return k
        vals = tuple(getattr(k, n) for n in names)
        return vals[0] if single is not None else analytic_kernel(names, vals)


def _make_layer(spec: LayerSpec, name: str):
    kernel_fn = KernelFn([spec], name)

    def init_fn(rng, input_shape):
        return _init_spec(spec, _gen(rng), tuple(input_shape))

    def apply_fn(params, inputs, **kwargs):
        x = inputs if isinstance(inputs, torch.Tensor) else torch.as_tensor(np.asarray(inputs))
        dev = params[0].device if isinstance(params, tuple) and params and \
            isinstance(params[0], torch.Tensor) else x.device
        ps = tuple(None if p is None else p.to(x.device) for p in params) if params else params
        del dev
        return _apply_spec(spec, ps, x.float())

    init_fn.__name__ = apply_fn.__name__ = name
    return init_fn, apply_fn, kernel_fn


# ---------------------------------------------------------------------------
# Public layers
# ---------------------------------------------------------------------------


def Dense(out_dim: int, W_std: float = 1., b_std: Optional[float] = None, batch_axis: int = 0,
          channel_axis: int = -1, parameterization: str = 'ntk', s=(1, 1)):
    """linear.py:760-931."""
    _check_axes(batch_axis, channel_axis)
    parameterization = parameterization.lower()
    if parameterization not in ('ntk', 'standard'):
        raise ValueError(f'Parameterization not supported: {parameterization}')
    width = out_dim if parameterization == 'ntk' else out_dim * s[1]
    spec = LayerSpec('dense', Diagonal(), dict(out_dim=out_dim, W_std=W_std, b_std=b_std,
                                               parameterization=parameterization, s=tuple(s)),
                     lambda sh: tuple(sh[:-1]) + (width,))
    return _make_layer(spec, 'Dense')


def Conv(out_chan: int, filter_shape: Sequence[int], strides: Optional[Sequence[int]] = None,
         padding: str = 'VALID', W_std: float = 1., b_std: Optional[float] = None,
         dimension_numbers=None, parameterization: str = 'ntk', s=(1, 1)):
    """linear.py:934-991 -> _Conv :1116-1454 (shared weights, NHWC)."""
    if dimension_numbers is not None:
        raise NotImplementedError('nt_gb300 supports the default NHWC dimension numbers')
    filter_shape = tuple(filter_shape)
    strides = tuple(strides) if strides else (1,) * len(filter_shape)
    padding = Padding(padding)
    parameterization = parameterization.lower()
    if parameterization not in ('ntk', 'standard'):
        raise ValueError(parameterization)
    width = out_chan if parameterization == 'ntk' else out_chan * s[1]

    def shape_fn(sh):
        out = [_pads(n, f, st, padding)[1] for n, f, st in zip(sh[1:-1], filter_shape, strides)]
        return (sh[0],) + tuple(out) + (width,)

    spec = LayerSpec('conv', Diagonal(output=Bool.NO),
                     dict(out_chan=out_chan, filter_shape=filter_shape, strides=strides,
                          padding=padding, W_std=W_std, b_std=b_std,
                          parameterization=parameterization, s=tuple(s)), shape_fn)
    return _make_layer(spec, 'Conv')


def ABRelu(a: float, b: float, do_stabilize: bool = False):
    """elementwise.py:403-477."""
    spec = LayerSpec('act', Diagonal(), dict(fn='abrelu', a=float(a), b=float(b),
                                             do_stabilize=bool(do_stabilize)), lambda sh: sh)
    return _make_layer(spec, f'ABReLU({a}, {b})')


def Relu(do_stabilize: bool = False):
    return ABRelu(0, 1, do_stabilize)


def LeakyRelu(alpha: float, do_stabilize: bool = False):
    return ABRelu(alpha, 1, do_stabilize)


def Abs(do_stabilize: bool = False):
    return ABRelu(-1, 1, do_stabilize)


def Erf(a: float = 1., b: float = 1., c: float = 0.):
    """elementwise.py:47-114."""
    spec = LayerSpec('act', Diagonal(), dict(fn='erf', a=float(a), b=float(b), c=float(c)),
                     lambda sh: sh)
    return _make_layer(spec, f'Erf({a}, {b}, {c})')


def Sin(a: float = 1., b: float = 1., c: float = 0.):
    """elementwise.py:275-328: a sin(b x + c)."""
    spec = LayerSpec('act', Diagonal(), dict(fn='sin', a=float(a), b=float(b), c=float(c)),
                     lambda sh: sh)
    return _make_layer(spec, f'Sin({a}, {b}, {c})')


def Cos(a: float = 1., b: float = 1., c: float = 0.):
    """elementwise.py:331-345: Sin with the phase shifted by pi / 2."""
    return Sin(a=a, b=b, c=c + math.pi / 2)


def Rbf(gamma: float = 1.0):
    """elementwise.py:348-400: sqrt(2) sin(sqrt(2 gamma) x + pi / 4)."""
    spec = LayerSpec('act', Diagonal(), dict(fn='rbf', gamma=float(gamma)), lambda sh: sh)
    return _make_layer(spec, f'Rbf({gamma})')


def Gelu(approximate: bool = False):
    """elementwise.py:195-272 (the kernel does not depend on `approximate`)."""
    spec = LayerSpec('act', Diagonal(), dict(fn='gelu', approximate=bool(approximate)),
                     lambda sh: sh)
    return _make_layer(spec, 'Gelu')


def _pool(kind, window_shape, strides, padding, normalize_edges, batch_axis, channel_axis):
    _check_axes(batch_axis, channel_axis)
    window_shape = tuple(window_shape)
    strides = tuple(strides) if strides else (1,) * len(window_shape)
    padding = Padding(padding)

    def shape_fn(sh):
        out = [_pads(n, w, st, padding)[1] for n, w, st in zip(sh[1:-1], window_shape, strides)]
        return (sh[0],) + tuple(out) + (sh[-1],)

    spec = LayerSpec('pool', Diagonal(input=Bool.MAYBE),
                     dict(pool=kind, window_shape=window_shape, strides=strides, padding=padding,
                          normalize_edges=normalize_edges), shape_fn)
    return _make_layer(spec, 'AvgPool' if kind == 'avg' else 'SumPool')


def AvgPool(window_shape, strides=None, padding='VALID', normalize_edges=False, batch_axis=0,
            channel_axis=-1):
    """linear.py:1457-1495."""
    return _pool('avg', window_shape, strides, padding, normalize_edges, batch_axis, channel_axis)


def SumPool(window_shape, strides=None, padding='VALID', batch_axis=0, channel_axis=-1):
    return _pool('sum', window_shape, strides, padding, False, batch_axis, channel_axis)


def _gpool(kind, batch_axis, channel_axis):
    _check_axes(batch_axis, channel_axis)
    spec = LayerSpec('gpool', Diagonal(input=Bool.MAYBE, output=Bool.YES), dict(pool=kind),
                     lambda sh: (sh[0], sh[-1]))
    return _make_layer(spec, 'GlobalAvgPool' if kind == 'avg' else 'GlobalSumPool')


def GlobalAvgPool(batch_axis=0, channel_axis=-1):
    """linear.py:1699-1810."""
    return _gpool('avg', batch_axis, channel_axis)


def GlobalSumPool(batch_axis=0, channel_axis=-1):
    return _gpool('sum', batch_axis, channel_axis)


def Flatten(batch_axis=0, batch_axis_out=0):
    """linear.py:1813-1906."""
    if batch_axis != 0 or batch_axis_out not in (0, -2):
        raise NotImplementedError('nt_gb300 supports Flatten(batch_axis=0, batch_axis_out=0)')
    spec = LayerSpec('flatten', Diagonal(output=Bool.YES), {},
                     lambda sh: (sh[0], int(np.prod(sh[1:]))), channel_axis_none=True)
    return _make_layer(spec, 'Flatten')


def Identity():
    spec = LayerSpec('identity', Diagonal(), {}, lambda sh: sh)
    return _make_layer(spec, 'Identity')


def _check_axes(batch_axis, channel_axis):
    if batch_axis != 0 or channel_axis not in (-1,):
        raise NotImplementedError('nt_gb300 supports batch_axis=0, channel_axis=-1')


def serial(*layers):
    """combinators.py:40-68."""
    specs = []
    init_fns, apply_fns = [], []
    for init_fn, apply_fn, kernel_fn in layers:
        if not isinstance(kernel_fn, KernelFn):
            raise TypeError('serial() takes nt_gb300.stax layers')
        specs += kernel_fn.specs
        init_fns.append(init_fn)
        apply_fns.append(apply_fn)

    def init_fn(rng, input_shape):
        params = []
        shape = tuple(input_shape)
        g = _gen(rng)
        for idx, f in enumerate(init_fns):
            shape, p = f(int(torch.randint(0, 2 ** 31 - 1, (1,), generator=g)) + idx, shape)
            params.append(p)
        return shape, tuple(params)

    def apply_fn(params, inputs, **kwargs):
        x = inputs
        for f, p in zip(apply_fns, params):
            x = f(p, x, **kwargs)
        return x

    return init_fn, apply_fn, KernelFn(specs, 'serial')
