"""The lax operations the analytic kernel path calls, on numpy (float64 when given float64)."""
import builtins
import itertools
import math

import numpy as np

from ._missing import missing_attr


class Precision:
    DEFAULT = 'DEFAULT'
    HIGH = 'HIGH'
    HIGHEST = 'HIGHEST'


def DotDimensionNumbers(*a):  # noqa: N802
    return tuple(a)


def add(x, y):
    return np.add(x, y)


def mul(x, y):
    return np.multiply(x, y)


def max(x, y):  # noqa: A001
    return np.maximum(x, y)


def padtype_to_pads(in_shape, window_shape, window_strides, padding):
    """'VALID' -> no padding; 'SAME' -> out = ceil(in / stride) with the smaller half first."""
    if not isinstance(padding, str):
        return [tuple(p) for p in padding]
    p = padding.upper()
    if p == 'VALID':
        return [(0, 0)] * len(in_shape)
    if p in ('SAME', 'SAME_LOWER'):
        pads = []
        for n, w, s in zip(in_shape, window_shape, window_strides):
            out = -(-n // s)
            total = builtins.max(0, (out - 1) * s + w - n)
            lo = total // 2 if p == 'SAME' else total - total // 2
            pads.append((lo, total - lo))
        return pads
    raise ValueError(padding)


def _perm(spec, first, second, order):
    """Axis permutation bringing `spec` to (first, second, spatial in `order`)."""
    sp = [i for i, c in enumerate(spec) if c not in (first, second)]
    sp.sort(key=lambda i: order.index(spec[i]))
    return [spec.index(first), spec.index(second)] + sp


def conv_general_dilated(lhs, rhs, window_strides, padding, lhs_dilation=None,
                         rhs_dilation=None, dimension_numbers=None, feature_group_count=1,
                         batch_group_count=1, precision=None, preferred_element_type=None):
    """Grouped cross-correlation (no kernel flip), string dimension numbers."""
    lhs, rhs = np.asarray(lhs), np.asarray(rhs)
    nd = lhs.ndim - 2
    for d in (lhs_dilation, rhs_dilation):
        if d is not None and any(v != 1 for v in d):
            raise missing_attr('conv_general_dilated with dilation')
    if batch_group_count != 1:
        raise missing_attr('conv_general_dilated with batch groups')
    if dimension_numbers is None:
        sp = 'HWDXYZ'[:nd]
        dimension_numbers = ('NC' + sp, 'OI' + sp, 'NC' + sp)
    lhs_spec, rhs_spec, out_spec = dimension_numbers
    if not all(isinstance(s, str) for s in (lhs_spec, rhs_spec, out_spec)):
        raise missing_attr('conv_general_dilated with non-string dimension numbers')
    order = [c for c in rhs_spec if c not in ('O', 'I')]
    x = np.transpose(lhs, _perm(lhs_spec, 'N', 'C', order))
    w = np.transpose(rhs, _perm(rhs_spec, 'O', 'I', order))
    N, C = x.shape[:2]
    O, I = w.shape[:2]
    G = feature_group_count
    assert C == G * I and O % G == 0, (C, G, I, O)
    ksz = w.shape[2:]
    strides = tuple(window_strides)
    pads = padtype_to_pads(x.shape[2:], ksz, strides, padding)
    if any(lo < 0 or hi < 0 for lo, hi in pads):
        raise missing_attr('conv_general_dilated with negative padding')
    x = np.pad(x, [(0, 0), (0, 0)] + [tuple(p) for p in pads])
    outsz = [(x.shape[2 + i] - ksz[i]) // strides[i] + 1 for i in range(nd)]
    dt = np.result_type(lhs, rhs)
    out = np.zeros((N, G, O // G) + tuple(outsz), dt)
    xg = x.reshape((N, G, I) + x.shape[2:])
    wg = w.reshape((G, O // G, I) + ksz)
    letters = 'pqrstuvw'[:nd]
    for off in itertools.product(*[range(k) for k in ksz]):
        sl = tuple(slice(off[i], off[i] + strides[i] * (outsz[i] - 1) + 1, strides[i])
                   for i in range(nd))
        xs = xg[(slice(None),) * 3 + sl]
        ws = wg[(slice(None),) * 3 + tuple(off)]
        out += np.einsum(f'ngi{letters},goi->ngo{letters}', xs, ws)
    out = out.reshape((N, O) + tuple(outsz))
    inv = _perm(out_spec, 'N', 'C', order)
    return np.transpose(out, np.argsort(inv))


def conv_general_shape_tuple(lhs_shape, rhs_shape, window_strides, padding, dimension_numbers):
    z = conv_general_dilated(np.zeros(lhs_shape), np.zeros(rhs_shape), window_strides, padding,
                             dimension_numbers=dimension_numbers)
    return z.shape


def reduce_window(operand, init_value, computation, window_dimensions, window_strides,
                  padding, base_dilation=None, window_dilation=None):
    x = np.asarray(operand)
    for d in (base_dilation, window_dilation):
        if d is not None and any(v != 1 for v in d):
            raise missing_attr('reduce_window with dilation')
    op = {add: np.add, np.add: np.add, max: np.maximum, np.maximum: np.maximum}.get(computation)
    if op is None:
        raise missing_attr(f'reduce_window with {computation}')
    pads = padtype_to_pads(x.shape, window_dimensions, window_strides, padding)
    x = np.pad(x, [tuple(p) for p in pads], constant_values=init_value)
    nd = x.ndim
    outsz = [(x.shape[i] - window_dimensions[i]) // window_strides[i] + 1 for i in range(nd)]
    out = np.full(outsz, init_value, np.result_type(x, np.asarray(init_value)))
    for off in itertools.product(*[range(k) for k in window_dimensions]):
        sl = tuple(slice(off[i], off[i] + window_strides[i] * (outsz[i] - 1) + 1,
                         window_strides[i]) for i in range(nd))
        out = op(out, x[sl])
    return out


def reduce_window_shape_tuple(operand_shape, window_dimensions, window_strides, padding,
                              base_dilation=None, window_dilation=None):
    pads = padtype_to_pads(operand_shape, window_dimensions, window_strides, padding)
    return tuple((n + lo + hi - w) // s + 1 for n, w, s, (lo, hi) in
                 zip(operand_shape, window_dimensions, window_strides, pads))


def dot_general(lhs, rhs, dimension_numbers, precision=None, preferred_element_type=None):
    (lc, rc), (lb, rb) = dimension_numbers
    lhs, rhs = np.asarray(lhs), np.asarray(rhs)
    letters = iter('abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ')
    ls = [None] * lhs.ndim
    rs = [None] * rhs.ndim
    batch = []
    for a, b in zip(lb, rb):
        c = next(letters)
        ls[a] = rs[b] = c
        batch.append(c)
    for a, b in zip(lc, rc):
        c = next(letters)
        ls[a] = rs[b] = c
    lfree = []
    for i in range(lhs.ndim):
        if ls[i] is None:
            ls[i] = next(letters)
            lfree.append(ls[i])
    rfree = []
    for i in range(rhs.ndim):
        if rs[i] is None:
            rs[i] = next(letters)
            rfree.append(rs[i])
    return np.einsum(f"{''.join(ls)},{''.join(rs)}->{''.join(batch + lfree + rfree)}", lhs, rhs)


def pad(operand, padding_value, padding_config):
    x = np.asarray(operand)
    if any(interior for _, _, interior in padding_config):
        raise missing_attr('pad with interior padding')
    out = x
    for ax, (lo, hi, _) in enumerate(padding_config):
        if lo < 0:
            out = np.take(out, range(-lo, out.shape[ax]), axis=ax)
            lo = 0
        if hi < 0:
            out = np.take(out, range(0, out.shape[ax] + hi), axis=ax)
            hi = 0
        widths = [(0, 0)] * out.ndim
        widths[ax] = (lo, hi)
        out = np.pad(out, widths, constant_values=padding_value)
    return out


def rev(operand, dimensions):
    return np.flip(operand, axis=tuple(dimensions))


def concatenate(operands, dimension):
    return np.concatenate(operands, axis=dimension)


def transpose(operand, permutation):
    return np.transpose(operand, permutation)


def broadcast_in_dim(operand, shape, broadcast_dimensions):
    x = np.asarray(operand)
    src = [1] * len(shape)
    for i, d in enumerate(broadcast_dimensions):
        src[d] = x.shape[i]
    return np.broadcast_to(x.reshape(src), shape)


def stop_gradient(x):
    return x


def cond(pred, true_fun, false_fun, *operands):
    return true_fun(*operands) if pred else false_fun(*operands)


def scan(f, init, xs, length=None, reverse=False):
    from .tree_util import tree_leaves, tree_map
    n = length if xs is None else len(tree_leaves(xs)[0])
    carry, ys = init, []
    idx = range(n - 1, -1, -1) if reverse else range(n)
    for i in idx:
        x = None if xs is None else tree_map(lambda a: a[i], xs)
        carry, y = f(carry, x)
        ys.append(y)
    if reverse:
        ys = ys[::-1]
    if not ys or ys[0] is None:
        return carry, None
    return carry, tree_map(lambda *a: np.stack(a), *ys)


def __getattr__(name):
    return missing_attr('lax.' + name, placeholder=True)


_ = math
