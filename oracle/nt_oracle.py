"""CPU restatement (numpy, float64 by default) of the analytic NNGP/NTK layer rules.

TEST INFRASTRUCTURE. This module is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import it.
The product path (the CUDA library behind ``include/nt_gb300.h`` and the host
package) never calls it.

What it restates (paths are inside the neural-tangents 0.6.6 project):

* ``neural_tangents/_src/stax/requirements.py:518-638`` -- input covariances
  (``_cov_*``), ``:641-830`` ``_inputs_to_kernel``, ``:401-515`` the
  ``Diagonal`` requirement algebra, ``:1057-1117`` ``get_diagonal`` /
  ``get_diagonal_outer_prods``.
* ``neural_tangents/_src/stax/linear.py:899-926`` Dense, ``:1321-1424`` Conv,
  ``:2938-2971`` ``_affine``, ``:3115-3207`` / ``:3341-3378`` the full-spatial
  convolution loop, ``:3381-3437`` the diagonal-spatial convolution,
  ``:1631-1664`` / ``:3499-3572`` pooling, ``:1771-1801`` global pooling,
  ``:1865-1899`` Flatten.
* ``neural_tangents/_src/stax/elementwise.py:67-112`` Erf, ``:423-477`` ABRelu,
  ``:195-272`` Gelu, ``:275-345`` Sin / Cos, ``:348-400`` Rbf,
  ``:1250-1310`` ``_elementwise`` / ``_sqrt`` / ``_arctan2``.
* ``neural_tangents/_src/utils/kernel.py:426-441`` Kernel scalar algebra.
* ``neural_tangents/_src/predict.py:71-278`` ``gradient_descent_mse``,
  ``:566-745`` ``gp_inference``, ``:753-1005`` ``gradient_descent_mse_ensemble``,
  ``:1180-1294`` eigen / Cholesky / expm1 helpers.

Parity pinning. The reference ships no stored golden vectors, and JAX is not
installed here. Its own stax / predict code is run on a numpy stand-in for the
JAX primitives it calls (``oracle/jax_stand_in``) by
``tests/golden/make_reference_golden.py``; this restatement reproduces those
outputs to 1e-12 (``tests/test_golden.py``). It is also pinned by the
reference's own known-answer and identity tests, re-run here by
``tests/test_oracle_pins.py``: the AvgPool all-ones closed form
(``tests/stax/stax_test.py:494-539``), the ABRelu identities
(``tests/stax/elementwise_test.py:541-636``), ``serial(B, B) == B o B``
(``tests/stax/stax_test.py:636-687``), Cholesky ``t=None`` equals eigh
``t=inf`` (``tests/predict_test.py:396-428``), the zero / multi / infinite time
predictions and the agreement with a trained (here exactly linear) network
(``tests/predict_test.py:108-160, 192-273``), the ensemble's NTK / NNGP agreement
and its mean and covariance against an exactly linear network ensemble
(``tests/predict_test.py:493-584, 622-686``), the dual activations against
Gauss-Hermite quadrature (``tests/stax/elementwise_test.py:480-538``), plus
closed forms derived from the mathematics (the arc-cosine kernel of Cho & Saul,
the arcsine kernel of Williams) and brute-force finite-width Monte Carlo checks.
(Batched equals unbatched, ``tests/batching_test.py:139-360``, is a property of
the product's tiling and is checked on its GPU path, not here.) The golden
fixtures under ``tests/golden/`` are outputs of this restatement, regenerated by
``tests/golden/make_golden.py``.
"""
from __future__ import annotations

import collections
import dataclasses
import enum
import math
from typing import Callable, Optional, Sequence

import numpy as np

# ---------------------------------------------------------------------------
# Requirement algebra (requirements.py:401-515, combinators.py:204-268)
# ---------------------------------------------------------------------------


class Bool(enum.IntEnum):
    NO = 0
    MAYBE = 1
    YES = 2


@dataclasses.dataclass(frozen=True)
class Diagonal:
    input: Bool = Bool.YES
    output: Bool = Bool.NO

    def __rshift__(self, other: "Diagonal") -> "Diagonal":
        # requirements.py:466-485
        if self.output == Bool.YES:
            return self
        if self.output > Bool.NO and other.input > Bool.NO:
            inp = self.input
        elif self.output == Bool.NO and other.input < Bool.YES:
            inp = Bool.NO
        else:
            inp = min(self.input, other.input)
        return Diagonal(input=inp, output=other.output)

    def __bool__(self) -> bool:
        return self.input == Bool.YES and self.output > Bool.NO


# ---------------------------------------------------------------------------
# Kernel container (kernel.py:27-149) -- numpy arrays, full-spatial layout
# [N1, N2, S1, S1', S2, S2', ...] ("zipped"), diagonal batch.
# ---------------------------------------------------------------------------


@dataclasses.dataclass
class Kernel:
    nngp: np.ndarray
    ntk: Optional[np.ndarray]
    cov1: np.ndarray
    cov2: Optional[np.ndarray]
    x1_is_x2: bool
    is_gaussian: bool
    is_reversed: bool
    is_input: bool
    diagonal_batch: bool
    diagonal_spatial: bool
    shape1: tuple
    shape2: tuple
    batch_axis: int = 0
    channel_axis: int = -1

    def replace(self, **kw) -> "Kernel":
        return dataclasses.replace(self, **kw)

    # kernel.py:426-441
    def mul(self, c: float) -> "Kernel":
        v = c ** 2
        return self.replace(
            cov1=v * self.cov1, nngp=v * self.nngp,
            cov2=None if self.cov2 is None else v * self.cov2,
            ntk=None if self.ntk is None else v * self.ntk)

    def add(self, c: float) -> "Kernel":
        v = c ** 2
        return self.replace(
            cov1=v + self.cov1, nngp=v + self.nngp,
            cov2=None if self.cov2 is None else v + self.cov2)


# ---------------------------------------------------------------------------
# Axis helpers (utils.py:324-553)
# ---------------------------------------------------------------------------


def zip_axes(x: np.ndarray, start: int) -> np.ndarray:
    """[..., X, Y, ..., X', Y'] -> [..., X, X', Y, Y'] from ``start``."""
    half = (x.ndim - start) // 2
    last = list(range(x.ndim - half, x.ndim))
    odd = list(range(start + 1, x.ndim, 2))
    return np.moveaxis(x, last, odd)


def unzip_axes(x: np.ndarray, start: int) -> np.ndarray:
    half = (x.ndim - start) // 2
    last = list(range(x.ndim - half, x.ndim))
    odd = list(range(start + 1, x.ndim, 2))
    return np.moveaxis(x, odd, last)


def diagonal_between(x: np.ndarray, start: int) -> np.ndarray:
    """Diagonal over zipped spatial pairs: [B.., S1,S1',S2,S2'] -> [B.., S1,S2]."""
    half = (x.ndim - start) // 2
    if half == 0:
        return x
    x = unzip_axes(x, start)
    side = x.shape[start:start + half]
    n = int(np.prod(side))
    x = x.reshape(x.shape[:start] + (n, n))
    x = np.diagonal(x, axis1=start, axis2=start + 1)
    return x.reshape(x.shape[:start] + side)


def outer_prod(x: np.ndarray, y: np.ndarray, start: int, op=np.multiply) -> np.ndarray:
    """utils.py:448-453: interleaved outer product from ``start``."""
    xs = x.shape[:start] + tuple(s for d in x.shape[start:] for s in (d, 1))
    ys = y.shape[:start] + tuple(s for d in y.shape[start:] for s in (1, d))
    return op(x.reshape(xs), y.reshape(ys))


def reverse_zipped(x: Optional[np.ndarray], start: int) -> Optional[np.ndarray]:
    """utils.py:465-480: reverse the order of zipped spatial pairs."""
    if x is None or x.ndim == 0:
        return x
    src = [j for i in range(x.ndim - 2, start - 1, -2) for j in (i, i + 1)]
    return np.moveaxis(x, src, list(range(start, x.ndim)))


# ---------------------------------------------------------------------------
# Inputs -> Kernel (requirements.py:518-830)
# ---------------------------------------------------------------------------


def _cov(x1: np.ndarray, x2: np.ndarray, diagonal_spatial: bool) -> np.ndarray:
    c = x1.shape[-1]
    if x1.ndim == 2:
        return x1 @ x2.T / c
    if diagonal_spatial:
        # requirements.py:556-569 -> [N1, N2, S1, S2, ...]
        return np.einsum('a...c,b...c->ab...', x1, x2) / c
    # requirements.py:542-553 -> [N1, S.., N2, S..] -> [N1, N2, S1, S1', ...]
    r = np.tensordot(x1, x2, axes=(-1, -1))
    nsp = x1.ndim - 2
    r = np.moveaxis(r, nsp + 1, 1)
    return zip_axes(r, 2) / c


def _cov_diag_batch(x: np.ndarray, diagonal_spatial: bool) -> np.ndarray:
    c = x.shape[-1]
    if x.ndim == 2 or diagonal_spatial:
        return np.sum(x * x, axis=-1) / c
    # requirements.py:529-539: dot_general with batch dim -> [N, S.., S..]
    r = np.einsum('n...c,nzc->n...z', x.reshape(x.shape[0], -1, c), x.reshape(x.shape[0], -1, c))
    sp = x.shape[1:-1]
    r = r.reshape((x.shape[0],) + sp + sp)
    return zip_axes(r, 1) / c


def inputs_to_kernel(x1, x2=None, *, diagonal_spatial=False, compute_ntk=True,
                     dtype=np.float64, channel_axis_none=False) -> Kernel:
    x1 = np.asarray(x1, dtype=dtype)
    x2n = None if x2 is None else np.asarray(x2, dtype=dtype)
    shape1, shape2 = x1.shape, (x1.shape if x2n is None else x2n.shape)
    if channel_axis_none:
        x1 = x1.reshape(x1.shape[0], -1)
        x2n = None if x2n is None else x2n.reshape(x2n.shape[0], -1)
        diagonal_spatial = False
    if x1.ndim == 2:
        diagonal_spatial = False
    cov1 = _cov_diag_batch(x1, diagonal_spatial)
    cov2 = None if x2n is None else _cov_diag_batch(x2n, diagonal_spatial)
    nngp = _cov(x1, x1 if x2n is None else x2n, diagonal_spatial)
    ntk = np.zeros((), dtype) if compute_ntk else None
    x1_is_x2 = x2n is None or (x1.shape == x2n.shape and bool(np.all(np.abs(x1 - x2n) < 1e-12)))
    return Kernel(nngp=nngp, ntk=ntk, cov1=cov1, cov2=cov2, x1_is_x2=x1_is_x2,
                  is_gaussian=False, is_reversed=False, is_input=False,
                  diagonal_batch=True, diagonal_spatial=bool(diagonal_spatial),
                  shape1=shape1, shape2=shape2)


# ---------------------------------------------------------------------------
# Padding helpers (lax.padtype_to_pads semantics)
# ---------------------------------------------------------------------------


def _pads(n: int, w: int, s: int, padding: str) -> tuple[int, int]:
    if padding == 'VALID':
        return 0, 0
    if padding in ('SAME', 'CIRCULAR'):
        out = -(-n // s)
        total = max((out - 1) * s + w - n, 0)
        return total // 2, total - total // 2
    raise ValueError(padding)


def _pad_axes(x, axes, windows, strides, padding):
    """Zero (SAME) or wrap (CIRCULAR, linear.py:2974-3019) padding on axes."""
    pads = [(0, 0)] * x.ndim
    for a, w, s in zip(axes, windows, strides):
        pads[a] = _pads(x.shape[a], w, s, padding)
    mode = 'wrap' if padding == 'CIRCULAR' else 'constant'
    return np.pad(x, pads, mode=mode)


def _reduce_window_sum(x, windows, strides, padding):
    """lax.reduce_window(add) over the trailing len(windows) axes."""
    axes = list(range(x.ndim - len(windows), x.ndim))
    if padding == 'SAME':
        x = _pad_axes(x, axes, windows, strides, 'SAME')
    out = x
    for a, w, s in zip(axes, windows, strides):
        n = out.shape[a]
        m = (n - w) // s + 1
        acc = 0
        for k in range(w):
            sl = [slice(None)] * out.ndim
            sl[a] = slice(k, k + (m - 1) * s + 1, s)
            acc = acc + out[tuple(sl)]
        out = acc
    return out


# ---------------------------------------------------------------------------
# Convolution rules (linear.py:3115-3437)
# ---------------------------------------------------------------------------


def _conv2d_diag_filter(lhs: np.ndarray, fs: int, st: int, padding: str) -> np.ndarray:
    """Depthwise conv of the trailing (S, S') plane with diag(1/fs) filter.

    ``linear.py:3352-3376``: out[a, b] = sum_k (1/fs) * pad(in)[a*st+k, b*st+k].
    """
    if padding == 'SAME':
        lhs = _pad_axes(lhs, [lhs.ndim - 2, lhs.ndim - 1], [fs, fs], [st, st], 'SAME')
    n0, n1 = lhs.shape[-2], lhs.shape[-1]
    m0, m1 = (n0 - fs) // st + 1, (n1 - fs) // st + 1
    acc = 0
    for k in range(fs):
        acc = acc + lhs[..., k:k + (m0 - 1) * st + 1:st, k:k + (m1 - 1) * st + 1:st]
    return acc / fs


def conv_full_spatial(lhs, filter_shape, strides, padding, batch_ndim):
    """linear.py:3115-3207 + 3341-3378 (shared weights, full spatial)."""
    if lhs is None or lhs.ndim == 0:
        return lhs
    if padding == 'CIRCULAR':
        axes = list(range(batch_ndim, lhs.ndim))
        fs2 = [f for f in filter_shape for _ in (0, 1)]
        st2 = [s for s in strides for _ in (0, 1)]
        lhs = _pad_axes(lhs, axes, fs2, st2, 'CIRCULAR')
        padding = 'VALID'
    for i in range(lhs.ndim - 1, batch_ndim, -2):
        sp = (i - batch_ndim) // 2
        lhs = np.moveaxis(lhs, (i - 1, i), (-2, -1))
        lhs = _conv2d_diag_filter(lhs, filter_shape[sp], strides[sp], padding)
    return lhs


def conv_diagonal_spatial(lhs, filter_shape, strides, padding, batch_ndim):
    """linear.py:3381-3437."""
    if lhs is None or lhs.ndim == 0:
        return lhs
    if padding == 'CIRCULAR':
        axes = list(range(batch_ndim, lhs.ndim))
        lhs = _pad_axes(lhs, axes, filter_shape, strides, 'CIRCULAR')
        padding = 'VALID'
    out = _reduce_window_sum(lhs, filter_shape, strides, padding)
    return out / float(np.prod(filter_shape))


# ---------------------------------------------------------------------------
# Layers. Each returns (name, kernel_fn, Diagonal requirement, shape_fn).
# ---------------------------------------------------------------------------


@dataclasses.dataclass
class Layer:
    name: str
    kernel_fn: Callable[[Kernel], Kernel]
    diag: Diagonal
    shape_fn: Callable[[tuple], tuple]


def _affine(mat, W_std, b_std):
    """linear.py:2938-2971."""
    if mat is None:
        return mat
    mat = mat * W_std ** 2
    if b_std is not None:
        mat = mat + b_std ** 2
    return mat


def Dense(out_dim, W_std=1., b_std=None, parameterization='ntk', s=(1, 1)):
    """linear.py:760-931 (kernel_fn :899-926)."""
    def kernel_fn(k: Kernel) -> Kernel:
        cov1, nngp, cov2, ntk = k.cov1, k.nngp, k.cov2, k.ntk
        fc = lambda x: _affine(x, W_std, b_std)
        if parameterization == 'ntk':
            cov1, nngp, cov2 = fc(cov1), fc(nngp), fc(cov2)
            if ntk is not None:
                ntk = nngp + W_std ** 2 * ntk
        elif parameterization == 'standard':
            input_width = k.shape1[-1] / s[0]
            if ntk is not None:
                ntk = input_width * nngp + W_std ** 2 * ntk
                if b_std is not None:
                    ntk = ntk + 1.
            cov1, nngp, cov2 = fc(cov1), fc(nngp), fc(cov2)
        else:
            raise ValueError(parameterization)
        return k.replace(cov1=cov1, nngp=nngp, cov2=cov2, ntk=ntk,
                         is_gaussian=True, is_input=False)

    width = out_dim if parameterization == 'ntk' else out_dim * s[1]
    return Layer('Dense', kernel_fn, Diagonal(),
                 lambda sh: sh[:-1] + (width,))


def Conv(out_chan, filter_shape, strides=None, padding='VALID', W_std=1.,
         b_std=None, parameterization='ntk', s=(1, 1)):
    """linear.py:934-991 -> _Conv 1116-1454 (kernel_fn :1321-1424)."""
    filter_shape = tuple(filter_shape)
    strides = tuple(strides) if strides else (1,) * len(filter_shape)

    def kernel_fn(k: Kernel) -> Kernel:
        cov1, nngp, cov2, ntk, is_reversed = k.cov1, k.nngp, k.cov2, k.ntk, k.is_reversed
        fsk, stk = filter_shape, strides
        if k.diagonal_spatial:
            conv_kernel = conv_diagonal_spatial
        else:
            if is_reversed:
                fsk, stk = fsk[::-1], stk[::-1]
            is_reversed = not is_reversed
            conv_kernel = conv_full_spatial

        def conv_unscaled(lhs, bnd):
            return conv_kernel(lhs, fsk, stk, padding, bnd)

        def affine(out, scale, shift):
            if out is None:
                return out
            out = out * scale
            if shift is not None:
                out = out + shift
            return out

        b_sq = None if b_std is None else b_std ** 2

        def conv(lhs, bnd):
            return affine(conv_unscaled(lhs, bnd), W_std ** 2, b_sq)

        cov1 = conv(cov1, 1)
        cov2 = conv(cov2, 1)
        if parameterization == 'ntk':
            nngp = conv(nngp, 2)
            if ntk is not None:
                ntk = W_std ** 2 * conv_unscaled(ntk, 2) + nngp
        elif parameterization == 'standard':
            fan_in = k.shape1[-1] * int(np.prod(filter_shape))
            nngp_u = conv_unscaled(nngp, 2)
            if ntk is not None:
                ntk = fan_in / s[0] * nngp_u + W_std ** 2 * conv_unscaled(ntk, 2)
                if b_std is not None:
                    ntk = ntk + 1.
            nngp = affine(nngp_u, W_std ** 2, b_sq)
        else:
            raise ValueError(parameterization)
        return k.replace(cov1=cov1, nngp=nngp, cov2=cov2, ntk=ntk,
                         is_gaussian=True, is_reversed=is_reversed, is_input=False)

    def shape_fn(sh):
        sp = sh[1:-1]
        out = []
        for n, f, st in zip(sp, filter_shape, strides):
            if padding == 'VALID':
                out.append((n - f) // st + 1)
            else:
                out.append(-(-n // st))
        width = out_chan if parameterization == 'ntk' else out_chan * s[1]
        return (sh[0],) + tuple(out) + (width,)

    return Layer('Conv', kernel_fn, Diagonal(output=Bool.NO), shape_fn)


def _get_diagonal(cov, diagonal_spatial):
    """requirements.py:1057-1074 (diagonal batch)."""
    if cov is None:
        return None
    if diagonal_spatial:
        return cov
    return diagonal_between(cov, 1)


def _outer_prods(cov1, cov2, diagonal_spatial, op=np.multiply):
    """requirements.py:1077-1117 (op = mul or add), diagonal batch."""
    d1 = _get_diagonal(cov1, diagonal_spatial)
    d2 = _get_diagonal(cov2, diagonal_spatial)
    if diagonal_spatial:
        # requirements.py:1108: the outer product runs over the batch axis only.
        prod12 = op(d1[:, None], (d1 if d2 is None else d2)[None, :])
    else:
        prod12 = outer_prod(d1, d1 if d2 is None else d2, 0, op)
    if diagonal_spatial:
        prod11 = op(d1, d1)
        prod22 = None if d2 is None else op(d2, d2)
    else:
        prod11 = outer_prod(d1, d1, 1, op)
        prod22 = None if d2 is None else outer_prod(d2, d2, 1, op)
    return prod11, prod12, (prod11 if prod22 is None else prod22)


def _sqrt(x, tol=0.):
    """elementwise.py:1278-1282."""
    return np.sqrt(np.maximum(x, tol))


def _arctan2(x, y, fill_zero=None):
    """elementwise.py:1293-1301."""
    r = np.arctan2(x, y)
    if fill_zero is not None:
        r = np.where((x == 0.) & (y == 0.), fill_zero, r)
    return r


def _elementwise(name, rule):
    """elementwise.py:1250-1275: requires a Gaussian input."""
    def kernel_fn(k: Kernel) -> Kernel:
        if not k.is_gaussian:
            raise ValueError('The input to the activation function must be Gaussian, '
                             'i.e. a random affine transform is required before the '
                             'activation function.')
        k = rule(k)
        return k.replace(is_gaussian=False)
    return Layer(name, kernel_fn, Diagonal(), lambda sh: sh)


def ABRelu(a, b, do_stabilize=False):
    """elementwise.py:403-477."""
    def rule(k: Kernel) -> Kernel:
        cov1, nngp, cov2, ntk = k.cov1, k.nngp, k.cov2, k.ntk
        if do_stabilize:
            factor = max(float(np.max(np.abs(nngp))), 1e-12)
            nngp = nngp / factor
            cov1 = cov1 / factor
            cov2 = None if cov2 is None else cov2 / factor
        prod11, prod12, prod22 = _outer_prods(cov1, cov2, k.diagonal_spatial)

        def nngp_ntk_fn(q, prod, t=None):
            sq = _sqrt(prod - q ** 2)
            ang = _arctan2(sq, q, fill_zero=np.pi / 2)
            factor_ = (a - b) ** 2 / (2 * np.pi)
            dot_sigma = (a ** 2 + b ** 2) / 2 - factor_ * ang
            q = factor_ * sq + dot_sigma * q
            if t is not None:
                t = t * dot_sigma
            return q, t

        nngp, ntk = nngp_ntk_fn(nngp, prod12, ntk)
        if k.diagonal_spatial:
            cov1 = (a ** 2 + b ** 2) / 2 * cov1
            cov2 = None if cov2 is None else (a ** 2 + b ** 2) / 2 * cov2
        else:
            cov1, _ = nngp_ntk_fn(cov1, prod11)
            if cov2 is not None:
                cov2, _ = nngp_ntk_fn(cov2, prod22)
        if do_stabilize:
            nngp = nngp * factor
            cov1 = cov1 * factor
            cov2 = None if cov2 is None else cov2 * factor
        return k.replace(cov1=cov1, nngp=nngp, cov2=cov2, ntk=ntk)
    return _elementwise(f'ABRelu({a},{b})', rule)


def Relu(do_stabilize=False):
    return ABRelu(0, 1, do_stabilize)


def LeakyRelu(alpha, do_stabilize=False):
    return ABRelu(alpha, 1, do_stabilize)


def Abs(do_stabilize=False):
    return ABRelu(-1, 1, do_stabilize)


def Erf(a=1., b=1., c=0.):
    """elementwise.py:47-114."""
    def rule(k: Kernel) -> Kernel:
        k = k.mul(b)
        cov1, nngp, cov2, ntk = k.cov1, k.nngp, k.cov2, k.ntk
        d1 = 1 + 2 * cov1
        d2 = None if cov2 is None else 1 + 2 * cov2
        prod11, prod12, prod22 = _outer_prods(d1, d2, k.diagonal_spatial)
        factor = 2 / np.pi

        def nngp_ntk_fn(q, prod, t=None):
            sq = _sqrt(prod - 4 * q ** 2)
            q = factor * np.arctan2(2 * q, sq)
            if t is not None:
                t = t * (2 * factor / sq)
            return q, t

        def nngp_fn_diag(q):
            return factor * np.arctan2(q, np.sqrt(q + 1. / 4))

        nngp, ntk = nngp_ntk_fn(nngp, prod12, ntk)
        if k.diagonal_spatial:
            cov1 = nngp_fn_diag(cov1)
            cov2 = None if cov2 is None else nngp_fn_diag(cov2)
        else:
            cov1, _ = nngp_ntk_fn(cov1, prod11)
            if cov2 is not None:
                cov2, _ = nngp_ntk_fn(cov2, prod22)
        k = k.replace(cov1=cov1, nngp=nngp, cov2=cov2, ntk=ntk)
        return k.mul(a).add(c)
    return _elementwise(f'Erf({a},{b},{c})', rule)


def Sin(a=1., b=1., c=0.):
    """elementwise.py:275-328: a sin(b x + c)."""
    def rule(k: Kernel) -> Kernel:
        cov1, nngp, cov2, ntk = k.cov1, k.nngp, k.cov2, k.ntk
        sum11, sum12, sum22 = _outer_prods(cov1, cov2, k.diagonal_spatial, np.add)
        half_a_square = a ** 2 / 2.

        def nngp_ntk_fn(q, sum_, t=None):
            s1 = np.exp(b ** 2 * (-0.5 * sum_ + q))
            s2 = np.exp(b ** 2 * (-0.5 * sum_ - q)) * np.cos(2 * c)
            q_out = half_a_square * (s1 - s2)
            if t is not None:
                t = t * (half_a_square * b ** 2 * (s1 + s2))
            return q_out, t

        def nngp_fn_diag(q):
            return half_a_square * (1. - np.exp(-2 * b ** 2 * q) * np.cos(2 * c))

        nngp, ntk = nngp_ntk_fn(nngp, sum12, ntk)
        if k.diagonal_spatial:
            cov1 = nngp_fn_diag(cov1)
            cov2 = None if cov2 is None else nngp_fn_diag(cov2)
        else:
            cov1, _ = nngp_ntk_fn(cov1, sum11)
            if cov2 is not None:
                cov2, _ = nngp_ntk_fn(cov2, sum22)
        return k.replace(cov1=cov1, nngp=nngp, cov2=cov2, ntk=ntk)
    return _elementwise(f'Sin({a},{b},{c})', rule)


def Cos(a=1., b=1., c=0.):
    """elementwise.py:331-345: Sin with the phase shifted by pi / 2."""
    return Sin(a=a, b=b, c=c + np.pi / 2)


def Rbf(gamma=1.0):
    """elementwise.py:348-400: dual activation of the normalised RBF kernel."""
    def rule(k: Kernel) -> Kernel:
        cov1, nngp, cov2, ntk = k.cov1, k.nngp, k.cov2, k.ntk
        sum11, sum12, sum22 = _outer_prods(cov1, cov2, k.diagonal_spatial, np.add)

        def nngp_ntk_fn(q, sum_, t=None):
            q_out = np.exp(gamma * (-sum_ + 2 * q))
            if t is not None:
                t = t * (2 * gamma * q_out)
            return q_out, t

        nngp, ntk = nngp_ntk_fn(nngp, sum12, ntk)
        if k.diagonal_spatial:
            cov1 = np.ones_like(cov1)
            cov2 = None if cov2 is None else np.ones_like(cov2)
        else:
            cov1, _ = nngp_ntk_fn(cov1, sum11)
            if cov2 is not None:
                cov2, _ = nngp_ntk_fn(cov2, sum22)
        return k.replace(cov1=cov1, nngp=nngp, cov2=cov2, ntk=ntk)
    return _elementwise(f'Rbf({gamma})', rule)


def Gelu(approximate=False):
    """elementwise.py:195-272 (the kernel does not depend on `approximate`)."""
    def rule(k: Kernel) -> Kernel:
        cov1, nngp, cov2, ntk = k.cov1, k.nngp, k.cov2, k.ntk
        p1_11, p1_12, p1_22 = _outer_prods(cov1 + 1, None if cov2 is None else cov2 + 1,
                                           k.diagonal_spatial)
        p11, p12, p22 = _outer_prods(cov1, cov2, k.diagonal_spatial)

        def nngp_ntk_fn(q, prod, prod_plus_1, t=None):
            delta_squared = prod_plus_1 - q ** 2
            delta = _sqrt(delta_squared)
            angles = np.arctan2(q, delta)
            q_out = (q ** 2 + prod * delta_squared) / (prod_plus_1 * delta)
            q_out = q_out + q * angles
            q_out = q_out / (2 * np.pi)
            q_out = q_out + 0.25 * q
            if t is not None:
                second = 0.25 + angles / (2 * np.pi)
                first = 1 / delta_squared + (1 - prod) / prod_plus_1 + 1
                first = first * (q / delta / (2. * np.pi))
                t = t * (first + second)
            return q_out, t

        def nngp_fn_diag(q):
            root = np.sqrt(1. + 2. * q)
            out = q / ((q + 1.) * root)
            out = out + np.arctan2(q, root) / 2
            return (out / np.pi + 0.25) * q

        nngp, ntk = nngp_ntk_fn(nngp, p12, p1_12, ntk)
        if k.diagonal_spatial:
            cov1 = nngp_fn_diag(cov1)
            cov2 = None if cov2 is None else nngp_fn_diag(cov2)
        else:
            cov1, _ = nngp_ntk_fn(cov1, p11, p1_11)
            if cov2 is not None:
                cov2, _ = nngp_ntk_fn(cov2, p22, p1_22)
        return k.replace(cov1=cov1, nngp=nngp, cov2=cov2, ntk=ntk)
    return _elementwise('Gelu', rule)


def Identity():
    return Layer('Identity', lambda k: k, Diagonal(), lambda sh: sh)


def _pool_layer(kind, window_shape, strides=None, padding='VALID', normalize_edges=False):
    """linear.py:1457-1671 (kernel_fn :1631-1664, _pool_kernel :3499-3572)."""
    window_shape = tuple(window_shape)
    strides = tuple(strides) if strides else (1,) * len(window_shape)

    def pool_kernel(mat, bnd, wk, sk, diag):
        if mat is None or mat.ndim == 0:
            return mat
        pad = padding
        if pad == 'CIRCULAR':
            axes = list(range(bnd, mat.ndim))
            mat = _pad_axes(mat, axes, wk, sk, 'CIRCULAR')
            pad = 'VALID'
        out = _reduce_window_sum(mat, wk, sk, pad)
        if kind == 'avg':
            if pad == 'SAME' and normalize_edges:
                ones = np.ones_like(mat)
                out = out / _reduce_window_sum(ones, wk, sk, pad)
            else:
                out = out / float(np.prod(wk))
        if diag and kind == 'avg':
            # linear.py:1653-1657: the diagonal-spatial kernel is normalised a
            # second time (the off-diagonal entries it omits are zero).
            if pad == 'SAME' and normalize_edges:
                out = out / _reduce_window_sum(np.ones_like(mat), wk, sk, pad)
            else:
                out = out / float(np.prod(wk))
        return out

    def kernel_fn(k: Kernel) -> Kernel:
        if k.diagonal_spatial:
            wk, sk = window_shape, strides
        else:
            w = window_shape[::-1] if k.is_reversed else window_shape
            st = strides[::-1] if k.is_reversed else strides
            wk = tuple(x for x in w for _ in (0, 1))
            sk = tuple(x for x in st for _ in (0, 1))
        f = lambda m, bnd: pool_kernel(m, bnd, wk, sk, k.diagonal_spatial)
        return k.replace(nngp=f(k.nngp, 2), ntk=f(k.ntk, 2), cov1=f(k.cov1, 1),
                         cov2=f(k.cov2, 1))

    def shape_fn(sh):
        sp = sh[1:-1]
        out = []
        for n, w, st in zip(sp, window_shape, strides):
            if padding == 'VALID':
                out.append((n - w) // st + 1)
            else:
                out.append(-(-n // st))
        return (sh[0],) + tuple(out) + (sh[-1],)

    return Layer('AvgPool' if kind == 'avg' else 'SumPool', kernel_fn,
                 Diagonal(input=Bool.MAYBE), shape_fn)


def AvgPool(window_shape, strides=None, padding='VALID', normalize_edges=False):
    return _pool_layer('avg', window_shape, strides, padding, normalize_edges)


def SumPool(window_shape, strides=None, padding='VALID'):
    return _pool_layer('sum', window_shape, strides, padding, False)


def _global_pool(kind):
    """linear.py:1699-1810 (kernel_fn :1771-1801)."""
    def kernel_fn(k: Kernel) -> Kernel:
        def pool(mat, bnd):
            if mat is None or mat.ndim == 0:
                return mat
            axes = tuple(range(bnd, mat.ndim))
            out = np.mean(mat, axis=axes) if kind == 'avg' else np.sum(mat, axis=axes)
            if k.diagonal_spatial and kind == 'avg':
                out = out / float(np.prod([mat.shape[a] for a in axes]))
            return out
        return k.replace(nngp=pool(k.nngp, 2), ntk=pool(k.ntk, 2), cov1=pool(k.cov1, 1),
                         cov2=pool(k.cov2, 1), is_reversed=False)
    return Layer('GlobalAvgPool' if kind == 'avg' else 'GlobalSumPool', kernel_fn,
                 Diagonal(input=Bool.MAYBE, output=Bool.YES),
                 lambda sh: (sh[0], sh[-1]))


def GlobalAvgPool():
    return _global_pool('avg')


def GlobalSumPool():
    return _global_pool('sum')


def Flatten():
    """linear.py:1813-1906 (kernel_fn :1865-1899)."""
    def kernel_fn(k: Kernel) -> Kernel:
        def trace(x, bnd):
            if x is None or x.ndim == 0:
                return x
            if k.diagonal_spatial:
                return np.mean(x, axis=tuple(range(bnd, x.ndim)))
            while x.ndim > bnd:
                x = np.trace(x, axis1=-2, axis2=-1) / x.shape[-1]
            return x
        return k.replace(nngp=trace(k.nngp, 2), ntk=trace(k.ntk, 2), cov1=trace(k.cov1, 1),
                         cov2=trace(k.cov2, 1), is_gaussian=False, is_reversed=False,
                         diagonal_spatial=False)
    return Layer('Flatten', kernel_fn, Diagonal(output=Bool.YES),
                 lambda sh: (sh[0], int(np.prod(sh[1:]))))


# ---------------------------------------------------------------------------
# serial + kernel_fn entry (combinators.py:40-68, requirements.py:912-1054)
# ---------------------------------------------------------------------------


def fold_diagonal(layers: Sequence[Layer]) -> Diagonal:
    req = None
    for l in layers:
        req = l.diag if req is None else (req >> l.diag)
    return Diagonal() if req is None else req


def serial(*layers: Layer):
    diag = fold_diagonal(layers)

    def kernel_fn(x1, x2=None, get=None, *, diagonal_spatial=None, dtype=np.float64):
        # requirements.py:884-900: a diagonal-spatial output can only be asked of a network
        # that does not need the full spatial covariance.
        if diagonal_spatial is True and diag.input == Bool.NO:
            raise ValueError('Asked to compute `kernel_fn` output with `diagonal_spatial == '
                             f'True`, while `kernel_fn` requires `diagonal_spatial == {diag}`.')
        ds = bool(diag) if diagonal_spatial is None else diagonal_spatial
        compute_ntk = get is None or 'ntk' in (get if isinstance(get, tuple) else (get,))
        k = inputs_to_kernel(x1, x2, diagonal_spatial=ds, compute_ntk=compute_ntk, dtype=dtype)
        shape1, shape2 = k.shape1, k.shape2
        for l in layers:
            k = l.kernel_fn(k)
            shape1, shape2 = l.shape_fn(shape1), l.shape_fn(shape2)
            k = k.replace(shape1=shape1, shape2=shape2)
        if get is None:
            return k
        if isinstance(get, str):
            return getattr(k, get)
        return tuple(getattr(k, g) for g in get)

    def apply_to_kernel(k: Kernel) -> Kernel:
        # requirements.py:100-112: an input kernel that holds only the spatial diagonal lacks
        # what a network needing the full spatial covariance reads.
        if k.diagonal_spatial and diag.input == Bool.NO:
            raise ValueError(f'the network requires `diagonal_spatial == {diag}`, but the input '
                             'kernel has `diagonal_spatial == True`.')
        for l in layers:
            k = l.kernel_fn(k)
        return k

    kernel_fn.layers = layers
    kernel_fn.diagonal = diag
    kernel_fn.apply_to_kernel = apply_to_kernel
    return kernel_fn


def myrtle(depth: int, W_std=math.sqrt(2.), b_std=0., readout='flatten'):
    """The Myrtle conv kernel network (notebooks/myrtle_kernel_with_neural_tangents.ipynb:114-131)."""
    factor = {5: [2, 1, 1], 7: [2, 2, 2], 10: [3, 3, 3]}[depth]
    conv = lambda: Conv(1, (3, 3), padding='SAME', W_std=W_std, b_std=b_std)
    layers = []
    layers += [conv(), Relu()] * 0
    for _ in range(factor[0]):
        layers += [conv(), Relu()]
    layers += [AvgPool((2, 2), (2, 2))]
    for _ in range(factor[1]):
        layers += [conv(), Relu()]
    layers += [AvgPool((2, 2), (2, 2))]
    for _ in range(factor[2]):
        layers += [conv(), Relu()]
    if readout == 'flatten':
        layers += [AvgPool((2, 2), (2, 2))] * 3
        layers += [Flatten(), Dense(10, W_std, b_std)]
    else:
        layers += [GlobalAvgPool(), Dense(10, W_std, b_std)]
    return serial(*layers)


# ---------------------------------------------------------------------------
# predict.gradient_descent_mse (predict.py:71-278, 1180-1258)
# ---------------------------------------------------------------------------


def _add_diagonal_regularizer(A, diag_reg, absolute):
    n = A.shape[0]
    if not absolute:
        diag_reg = diag_reg * np.trace(A) / n
    return A + diag_reg * np.eye(n)


def gradient_descent_mse(k_train_train, y_train, learning_rate=1., diag_reg=0.,
                         diag_reg_absolute_scale=False):
    """predict.py:71-278: infinite (t=None, Cholesky) and finite/infinite (eigh) time
    predictions of gradient flow on the MSE loss.

    Restricted to a 2-D ``k_train_train`` and ``trace_axes=(-1,)``.
    """
    import scipy.linalg as sla
    A = _add_diagonal_regularizer(np.asarray(k_train_train, np.float64), diag_reg,
                                  diag_reg_absolute_scale)
    y = np.asarray(y_train, np.float64)

    def predict_fn(t=None, fx_train_0=0., fx_test_0=None, k_test_train=None):
        if t is None:
            fx_train_t = y
            if fx_test_0 is None:
                return fx_train_t
            rhs = y if fx_train_0 is None else y - fx_train_0
            cf = sla.cho_factor(A, lower=False)
            sol = sla.cho_solve(cf, rhs)
            fx_test_t = fx_test_0 + np.asarray(k_test_train, np.float64) @ sol
            if fx_train_0 is None:
                return fx_test_t
            return fx_train_t, fx_test_t
        evals, evecs = np.linalg.eigh(A)
        # predict.py:197-229: t of any shape; the outputs are t.shape + the fx shape
        t = np.asarray(t, np.float64) * learning_rate
        t_shape = t.shape
        ts = t.reshape(-1, 1)
        rhs = -y if fx_train_0 is None else fx_train_0 - y
        # predict.py:1277-1294: expm1 / inv-expm1 spectral functions with
        # normalisation y_train.size and negative eigenvalues clipped to 0.
        expm1 = np.expm1(-np.maximum(evals, 0.)[None, :] * ts / y.size)  # [T, n]
        inv = expm1 / np.abs(evals)[None, :]
        proj = evecs.T @ rhs
        out_train = out_test = None
        if fx_train_0 is not None:
            d = np.einsum('ji,ti,ik->tjk', evecs, expm1, proj)
            out_train = fx_train_0 + d.reshape(t_shape + d.shape[1:])
        if fx_test_0 is not None:
            d = np.einsum('ji,ti,ik->tjk', evecs, inv, proj)
            d = np.einsum('mj,tjk->tmk', np.asarray(k_test_train, np.float64), d)
            out_test = fx_test_0 + d.reshape(t_shape + d.shape[1:])
        if out_train is not None and out_test is not None:
            return out_train, out_test
        return out_test if out_train is None else out_train

    return predict_fn


# ---------------------------------------------------------------------------
# Gaussian-process inference and the infinite ensemble (predict.py:566-1005)
# ---------------------------------------------------------------------------
Gaussian = collections.namedtuple('Gaussian', 'mean covariance')


def _kattr(k, g):
    """predict.py _get_attr: a field of a kernel container, or the array itself."""
    if isinstance(k, dict):
        return k[g]
    if hasattr(k, g):
        return getattr(k, g)
    return k


def _has(k, g) -> bool:
    return (g in k) if isinstance(k, dict) else hasattr(k, g)


def _canonical_get(get):
    if get is None:
        return None, ('nngp', 'ntk')
    if isinstance(get, str):
        return get, (get,)
    return None, tuple(get)


def _as_gaussians(get, names, out):
    """utils.get_namedtuple('Gaussians'): one value for a string `get`, else a
    namedtuple of the requested fields in order."""
    if isinstance(get, str):
        return out[get]
    return collections.namedtuple('Gaussians', names)(*[out[g] for g in names])


def gp_inference(k_train_train, y_train, diag_reg=0., diag_reg_absolute_scale=False):
    """predict.py:566-745 with trace_axes=(-1,) and 2-D kernels: the NNGP / NTK /
    NTKGP posterior mean and, given k_test_test, covariance."""
    import scipy.linalg as sla
    y = np.asarray(y_train, np.float64)
    factors = {}

    def solve(g):
        if g not in factors:
            a = _add_diagonal_regularizer(np.asarray(_kattr(k_train_train, g), np.float64),
                                          diag_reg, diag_reg_absolute_scale)
            factors[g] = sla.cho_factor(a, lower=False)
        return lambda b: sla.cho_solve(factors[g], b)

    def predict_fn(get=None, k_test_train=None, k_test_test=None):
        _, names = _canonical_get(get)
        out = {}
        for g in names:
            k = 'ntk' if g == 'ntkgp' else g
            k_dd = np.asarray(_kattr(k_train_train, k), np.float64)
            k_td = None if k_test_train is None else np.asarray(_kattr(k_test_train, k),
                                                                  np.float64)
            mean = y if k_td is None else k_td @ solve(k)(y)
            if k_test_test is None:
                out[g] = mean
                continue
            if k_td is None:
                out[g] = Gaussian(mean, np.zeros_like(k_dd))
                continue
            if g == 'ntk' and (not _has(k_train_train, 'nngp') or
                               not _has(k_test_train, 'nngp')):
                raise ValueError('the NTK posterior covariance needs the NNGP kernels too')
            g_init = 'nngp' if g != 'ntkgp' else 'ntk'
            k_td_g_inv_y = solve(k)(np.asarray(_kattr(k_test_train, g_init), np.float64).T)
            k_tt = np.asarray(_kattr(k_test_test, g_init), np.float64)
            if g in ('nngp', 'ntkgp'):
                cov = k_tt - k_td @ k_td_g_inv_y
            else:
                term_1 = solve(g)(k_td.T)
                nngp_dd = np.asarray(_kattr(k_train_train, 'nngp'), np.float64)
                cov = term_1.T @ (nngp_dd @ term_1)
                term_2 = k_td @ k_td_g_inv_y
                cov = cov - (term_2 + term_2.T) + k_tt
            out[g] = Gaussian(mean, cov)
        return _as_gaussians(get, names, out)

    return predict_fn


def _dependency(names, compute_cov):
    """predict.py _get_dependency."""
    dep = ()
    if 'nngp' in names or ('ntk' in names and compute_cov):
        dep += ('nngp',)
    if 'ntk' in names:
        dep += ('ntk',)
    return dep


def gradient_descent_mse_ensemble(kernel_fn, x_train, y_train, learning_rate=1., diag_reg=0.,
                                  diag_reg_absolute_scale=False):
    """predict.py:753-1005 with trace_axes=(-1,): mean (and covariance) of the
    infinite ensemble trained by gradient flow on the MSE loss, at times t
    (eigendecomposition, expm1 spectral functions of predict.py:1277-1294) or at
    t=None (gp_inference, Cholesky)."""
    y = np.asarray(y_train, np.float64)
    k_dd = {}
    eig = {}

    def k_train(g):
        if g not in k_dd:
            k_dd[g] = np.asarray(kernel_fn(x_train, None, g), np.float64)
        return k_dd[g]

    def eigenspace(g):
        if g not in eig:
            a = _add_diagonal_regularizer(k_train(g), diag_reg, diag_reg_absolute_scale)
            eig[g] = np.linalg.eigh(a)
        return eig[g]

    def predict_fn(t=None, x_test=None, get=None, compute_cov=False):
        _, names = _canonical_get(get)
        dep = _dependency(names, compute_cov)
        kd = {g: k_train(g) for g in dep}
        if x_test is None:
            k_td = None
            nngp_tt = True if compute_cov else None
        else:
            k_td = {g: np.asarray(kernel_fn(x_test, x_train, g), np.float64) for g in dep}
            nngp_tt = (np.asarray(kernel_fn(x_test, None, 'nngp'), np.float64)
                       if compute_cov else None)
        if t is None:
            return gp_inference(kd, y, diag_reg, diag_reg_absolute_scale)(
                get=get, k_test_train=k_td, k_test_test=nngp_tt)
        t = np.asarray(t, np.float64) * learning_rate
        t_shape = t.shape
        tf = t.reshape(-1, 1)
        norm = y.size
        out = {}
        for g in names:
            evals, evecs = eigenspace(g)
            ev = evals[None, :]
            pos = np.maximum(ev, 0.)
            neg_expm1 = -np.expm1(-pos * tf / norm)
            neg_inv = neg_expm1 / np.abs(ev)
            if k_td is None:
                mean = np.einsum('ji,ti,ki,kl->tjl', evecs, neg_expm1, evecs, y)
            else:
                ktd = k_td[g]
                mean = np.einsum('lj,ji,ti,ki,km->tlm', ktd, evecs, neg_inv, evecs, y)
            mean = mean.reshape(t_shape + mean.shape[1:])
            if nngp_tt is None:
                out[g] = mean
                continue
            nngp_dd = kd['nngp']
            if k_td is None:
                if g == 'nngp':
                    cov = np.einsum('ji,ti,ki->tjk', evecs, pos * np.exp(-2 * pos * tf / norm),
                                    evecs)
                else:
                    ex = np.einsum('mi,ti,ki->tmk', evecs, np.exp(-pos * tf / norm), evecs)
                    cov = np.einsum('tmk,kl,tnl->tmn', ex, nngp_dd, ex)
            else:
                tt = nngp_tt[None]
                if g == 'nngp':
                    neg_inv2 = -np.expm1(-pos * 2 * tf / norm) / np.abs(ev)
                    cov = tt - np.einsum('mj,ji,ti,ki,lk->tml', ktd, evecs, neg_inv2, evecs, ktd)
                else:
                    term_1 = np.einsum('mi,ti,ki,lk->tml', evecs, neg_inv, evecs, ktd)
                    term_2 = np.einsum('mj,ji,ti,ki,lk->tml', ktd, evecs, neg_inv, evecs,
                                       k_td['nngp'])
                    term_2 = term_2 + np.swapaxes(term_2, 1, 2)
                    cov = np.einsum('tji,jk,tkl->til', term_1, nngp_dd, term_1) - term_2 + tt
            cov = cov.reshape(t_shape + cov.shape[1:])
            out[g] = Gaussian(mean, cov)
        return _as_gaussians(get, names, out)

    return predict_fn
