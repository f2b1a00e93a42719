"""nt_gb300.batch -- tiled evaluation of kernel functions (neural_tangents/_src/batching.py:76-132).

``batch(kernel_fn, batch_size)`` returns a function with ``kernel_fn``'s
signature that evaluates the N1 x N2 kernel in tiles of at most
``batch_size`` rows and columns. Unlike the reference (batching.py:647-679),
N1 and N2 need not be multiples of ``batch_size``: the edge tiles are ragged.
For networks the fused chain kernel covers, the whole grid is one launch of
that kernel (the per-sample chains run once per sample, in ``batch_size``
chunks) and ``batch_size`` only bounds the per-sample working set.
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from . import _chain
from . import _lib as L
from .kernel import Kernel, analytic_kernel
from .stax import KernelFn, _Ctx, _as_input, _normalize_get


def _tiles(n: int, b: int):
    return [(s, min(b, n - s)) for s in range(0, n, b)]


def tile_grid(n1: int, n2: int, b: int):
    """Row-major (r0, rn, c0, cn) tiles of an n1 x n2 kernel, ragged at the edges."""
    return [(r0, rn, c0, cn) for r0, rn in _tiles(n1, b) for c0, cn in _tiles(n2, b)]


def rank_rows(n: int, b: int, world_size: int, rank: int):
    """The contiguous rows [start, stop) of an n-row kernel that one rank computes when whole
    tile rows (b rows each, the last one ragged) are split evenly across ranks."""
    t = (n + b - 1) // b
    lo, hi = rank * t // world_size, (rank + 1) * t // world_size
    return min(lo * b, n), min(hi * b, n)


def rank_tiles(tiles, world_size: int, rank: int, steps=None):
    """Tiles of one rank when the grid is sharded across ranks (tile k -> rank k % world_size,
    batching.py:505-644 shards x1 rows the same way). Every tile of the grid is independent, so
    the ranks exchange no data; with `steps`, the list wraps to that length."""
    mine = [t for k, t in enumerate(tiles) if k % world_size == rank]
    if steps is None:
        return mine
    return [tiles[(rank + world_size * s) % len(tiles)] for s in range(steps)]


class _CheckpointedKernel(torch.autograd.Function):
    """nngp/ntk over the whole grid with a recompute-per-tile backward.

    The forward keeps nothing but the inputs; the backward re-evaluates each
    tile through the differentiable layer rules and back-propagates that
    tile's cotangents, so at most one tile's layer tensors are alive at once.
    """

    @staticmethod
    def forward(ctx, x1, x2, kfn, bs, precision):
        x2o = None if x2.numel() == 0 else x2
        with torch.no_grad():
            res = _forward_grid(kfn, x1, x2o, bs, precision)
        ctx.save_for_backward(x1, x2)
        ctx.kfn, ctx.bs, ctx.precision = kfn, bs, precision
        return res.nngp, res.ntk

    @staticmethod
    def backward(ctx, gq, gt):
        with L.boundary('nt.batch backward'):
            return _CheckpointedKernel._backward(ctx, gq, gt)

    @staticmethod
    def _backward(ctx, gq, gt):
        from . import _autograd
        x1, x2 = ctx.saved_tensors
        x2o = None if x2.numel() == 0 else x2
        xb = x1 if x2o is None else x2o
        gx1 = torch.zeros_like(x1)
        gxb = gx1 if x2o is None else torch.zeros_like(x2o)
        bs = ctx.bs
        symmetric = x2o is None
        for r0, rn in _tiles(x1.shape[0], bs):
            for c0, cn in _tiles(xb.shape[0], bs):
                # K(x, x) is symmetric: the tile (c, r) is the transpose of the tile (r, c),
                # so each off-diagonal pair of tiles is recomputed once, with both cotangents
                if symmetric and c0 < r0:
                    continue
                with torch.enable_grad():
                    a = x1[r0:r0 + rn].detach().requires_grad_(True)
                    b = xb[c0:c0 + cn].detach().requires_grad_(True)
                    k = _autograd.run_ad(ctx.kfn.specs, a, b, True, ctx.precision,
                                         bool(ctx.kfn.diagonal))
                    outs, grads = [], []
                    for o, g in ((k.nngp, gq), (k.ntk, gt)):
                        if g is not None:
                            gg = g[r0:r0 + rn, c0:c0 + cn]
                            if symmetric and c0 > r0:
                                gg = gg + g[c0:c0 + cn, r0:r0 + rn].transpose(0, 1)
                            outs.append(o)
                            grads.append(gg)
                    torch.autograd.backward(outs, grads)
                gx1[r0:r0 + rn] += a.grad
                gxb[c0:c0 + cn] += b.grad
        return gx1, (None if x2o is None else gxb), None, None, None


def _forward_grid(kernel_fn, x1t, x2t, bs, precision):
    ctx = _Ctx(precision)
    plan = _chain.plan_chain(kernel_fn.specs, tuple(x1t.shape), bool(kernel_fn.diagonal))
    if plan is not None and (x2t is None or x2t.shape[1:] == x1t.shape[1:]):
        old = _chain.SELF_CHUNK
        _chain.SELF_CHUNK = max(1, min(old, bs))
        try:
            k = _chain.run_fused(plan, x1t, x2t, ctx)
        finally:
            _chain.SELF_CHUNK = old
        return kernel_fn.apply_kernel(k, ctx, specs=plan.post)
    xb = x1t if x2t is None else x2t
    rows = []
    for r0, rn in _tiles(x1t.shape[0], bs):
        cols = []
        for c0, cn in _tiles(xb.shape[0], bs):
            cols.append(kernel_fn(x1t[r0:r0 + rn], xb[c0:c0 + cn], ('nngp', 'ntk'),
                                  precision=precision))
        rows.append(cols)
    return _assemble(rows, ('nngp', 'ntk'), None)


def batch(kernel_fn, batch_size: int = 0, device_count: int = -1, store_on_device: bool = True,
          recompute_tile: Optional[int] = None):
    """batching.py:76-132 (one device: serial tiling).

    With inputs that require grad, the returned nngp/ntk carry a checkpointed
    backward (one tile of layer tensors recomputed at a time). Its tile is
    ``recompute_tile`` rows/columns when given, else the autotuned one
    (``tune.recompute_tile``: the fastest probe within the memory budget), never
    more than ``batch_size`` (not in the reference, whose backward is XLA's)."""
    if device_count not in (-1, 0, 1):
        raise NotImplementedError('nt_gb300 runs on one GPU; device_count must be -1, 0 or 1')

    def batched(x1, x2=None, get=None, *, precision='fp32', **kwargs):
        with L.boundary('nt.batch'):
            return _batched(x1, x2, get, precision=precision, **kwargs)

    def _batched(x1, x2=None, get=None, *, precision='fp32', **kwargs):
        if isinstance(x1, Kernel):
            return kernel_fn(x1, x2, get, **kwargs)
        x1t = _as_input(x1)
        x2t = None if x2 is None else _as_input(x2)
        names, single = _normalize_get(get)
        ctx = _Ctx(precision)
        bs = batch_size or max(x1t.shape[0], (x2t if x2t is not None else x1t).shape[0])
        if isinstance(kernel_fn, KernelFn) and torch.is_grad_enabled() and (
                x1t.requires_grad or (x2t is not None and x2t.requires_grad)):
            if names is None or not set(names) <= {'nngp', 'ntk'}:
                raise NotImplementedError('differentiable batch() returns nngp and ntk')
            tile = recompute_tile
            if tile is None:
                from . import tune
                tile = tune.recompute_tile(kernel_fn, tuple(x1t.shape), precision)
            q, t = _CheckpointedKernel.apply(
                x1t, x2t if x2t is not None else torch.empty(0, device=x1t.device), kernel_fn,
                max(1, min(bs, int(tile))), precision)
            vals = tuple(q if n == 'nngp' else t for n in names)
            return vals[0] if single is not None else analytic_kernel(names, vals)
        ds = kwargs.get('diagonal_spatial')
        if isinstance(kernel_fn, KernelFn):
            ds = bool(kernel_fn.diagonal) if ds is None else bool(ds)
        if isinstance(kernel_fn, KernelFn) and not ds:
            plan = _chain.plan_chain(kernel_fn.specs, tuple(x1t.shape), False)
            if plan is not None and (x2t is None or x2t.shape[1:] == x1t.shape[1:]):
                old = _chain.SELF_CHUNK
                _chain.SELF_CHUNK = max(1, min(old, bs))
                try:
                    k = _chain.run_fused(plan, x1t, x2t, ctx)
                finally:
                    _chain.SELF_CHUNK = old
                k = kernel_fn.apply_kernel(k, ctx, specs=plan.post)
                if names is not None and 'ntk' not in names:
                    k = k.replace(ntk=None)
                return _select(k, names, single)
        xb = x1t if x2t is None else x2t
        n1, n2 = x1t.shape[0], xb.shape[0]
        rows = []
        for r0, rn in _tiles(n1, bs):
            cols = []
            for c0, cn in _tiles(n2, bs):
                out = kernel_fn(x1t[r0:r0 + rn], xb[c0:c0 + cn], get, precision=precision,
                                **kwargs)
                if not store_on_device:
                    out = _to_cpu(out)
                cols.append(out)
            rows.append(cols)
        return _assemble(rows, names, single)

    batched.__name__ = getattr(kernel_fn, '__name__', 'kernel_fn')
    return batched


def _to_cpu(out):
    if isinstance(out, torch.Tensor):
        return out.cpu()
    if isinstance(out, tuple):
        return type(out)(*[None if v is None else v.cpu() for v in out])
    return out


def _select(k: Kernel, names, single):
    if names is None:
        return k
    vals = tuple(getattr(k, n) for n in names)
    return vals[0] if single is not None else analytic_kernel(names, vals)


def _cat_grid(grid):
    return torch.cat([torch.cat(row, dim=1) for row in grid], dim=0)


def _assemble(rows, names, single):
    if names is None:
        raise NotImplementedError('batch(get=None) is not supported; pass get=("nngp", "ntk")')
    if single is not None:
        return _cat_grid(rows)
    vals = []
    for idx, n in enumerate(names):
        grid = [[c[idx] for c in row] for row in rows]
        if n in ('nngp', 'ntk'):
            vals.append(_cat_grid(grid))
        elif n == 'cov1':
            vals.append(torch.cat([row[0] for row in grid], dim=0))
        elif n == 'cov2':
            vals.append(torch.cat(grid[0], dim=0))
        else:
            vals.append(grid[0][0])
    return analytic_kernel(names, tuple(vals))


class CapturedBatch:
    """``batch(kernel_fn, batch_size)(x1, x2, get)`` for fixed input shapes, captured
    once as a CUDA graph and replayed: for serving, where the same shapes come back
    and the host-side work of a call (per-sample chains, launches, allocations)
    would otherwise be repeated. Only networks on the fused chain path (whose
    forward has no host synchronisation) can be captured. A call copies the inputs
    into the graph's static buffers, replays, and returns the graph's static
    output tensors, which the next call overwrites (clone them to keep them).
    Not in the reference (XLA compiles, it does not capture)."""

    def __init__(self, kernel_fn, x1_shape, x2_shape=None, get=('nngp', 'ntk'),
                 batch_size: int = 0, precision: str = 'fp32'):
        dev = L.require_cuda()
        if not isinstance(kernel_fn, KernelFn):
            raise TypeError('CapturedBatch needs a kernel_fn from nt_gb300.stax.serial')
        self.names, self.single = _normalize_get(get)
        if self.names is None or not set(self.names) <= {'nngp', 'ntk'}:
            raise NotImplementedError('CapturedBatch returns nngp and/or ntk')
        self.plan = _chain.plan_chain(kernel_fn.specs, tuple(x1_shape), False)
        if self.plan is None or bool(kernel_fn.diagonal) or (
                x2_shape is not None and tuple(x2_shape[1:]) != tuple(x1_shape[1:])):
            raise NotImplementedError('CapturedBatch needs a network on the fused chain path')
        self.kernel_fn, self.precision = kernel_fn, precision
        self.bs = batch_size or max(x1_shape[0], (x2_shape or x1_shape)[0])
        self.x1 = torch.zeros(tuple(x1_shape), device=dev)
        self.x2 = None if x2_shape is None else torch.zeros(tuple(x2_shape), device=dev)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(2):  # warm-up: library load, kernel attributes, allocator pools
                self._run()
        torch.cuda.current_stream().wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode='thread_local'):
            self.out = self._run()

    def _run(self):
        ctx = _Ctx(self.precision)
        old = _chain.SELF_CHUNK
        _chain.SELF_CHUNK = max(1, min(old, self.bs))
        try:
            k = _chain.run_fused(self.plan, self.x1, self.x2, ctx, x1_is_x2=self.x2 is None)
        finally:
            _chain.SELF_CHUNK = old
        k = self.kernel_fn.apply_kernel(k, ctx, specs=self.plan.post)
        return _select(k, self.names, self.single)

    def __call__(self, x1, x2=None):
        self.x1.copy_(_as_input(x1), non_blocking=True)
        if self.x2 is not None:
            if x2 is None:
                raise ValueError('this capture was made with x2')
            self.x2.copy_(_as_input(x2), non_blocking=True)
        elif x2 is not None:
            raise ValueError('this capture was made with x2=None')
        with L.boundary('CapturedBatch'):
            self.graph.replay()
        return self.out
