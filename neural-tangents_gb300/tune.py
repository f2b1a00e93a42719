"""Autotuning of launch shapes that do not change results.

The reference leaves tile shapes to XLA; here they are measured. Two knobs:

* the recompute tile of the checkpointed backward of ``nt.batch`` (how many
  rows / columns of the kernel grid are re-evaluated together through the
  differentiable layer rules). Larger tiles amortise the per-sample chains and
  the launches, but the layer tensors of a tile grow with its pair count
  (16 MiB per pair and 32x32 layer); ``recompute_tile`` times one probe
  forward+backward per candidate, records its peak device memory, and keeps
  the fastest candidate (time per pair) whose memory stays inside a budget;
* the ring depth of the 32x32 stencil (``NTG_TUNE_STENCIL_RING``), timed on a
  materialised conv + ReLU launch by ``stencil_ring``.

Results are cached per (device, network, input shape, precision) in memory
and, when ``NT_GB300_TUNE_CACHE`` names a file, in that JSON file. The cache
is guarded by a lock; tuning runs on the current stream and device.
"""
from __future__ import annotations

import json
import os
import statistics
import threading
from typing import Optional

import torch

from . import _lib as L

TILE_CANDIDATES = (4, 8, 12, 16, 24, 32, 48, 64)
MEMORY_FRACTION = 0.6

_lock = threading.Lock()
_cache: dict = {}
_loaded = False


def _cache_path() -> Optional[str]:
    return os.environ.get('NT_GB300_TUNE_CACHE') or None


def _load() -> None:
    global _loaded
    if _loaded:
        return
    _loaded = True
    path = _cache_path()
    if path and os.path.exists(path):
        try:
            with open(path) as f:
                _cache.update(json.load(f))
        except (OSError, ValueError):
            pass


def _store(key: str, value) -> None:
    _cache[key] = value
    path = _cache_path()
    if path:
        tmp = path + '.tmp'
        with open(tmp, 'w') as f:
            json.dump(_cache, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def _device_name() -> str:
    return torch.cuda.get_device_name(torch.cuda.current_device())


def network_key(kernel_fn) -> str:
    """A stable description of a serial network's layers and parameters."""
    parts = []
    for sp in getattr(kernel_fn, 'specs', ()):
        items = []
        for k, v in sorted(sp.params.items()):
            if isinstance(v, torch.Tensor):
                v = round(float(v.detach().float().reshape(-1)[0]), 6)
            items.append(f'{k}={v}')
        parts.append(sp.kind + '(' + ','.join(items) + ')')
    return '|'.join(parts)


def _probe(kernel_fn, sample: torch.Tensor, t: int, precision: str):
    """Time (ms) and peak memory (bytes) of one t x t tile forward + backward."""
    from . import _autograd
    a = sample[:t].detach().clone().requires_grad_(True)
    b = sample[t:2 * t].detach().clone().requires_grad_(True)
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    ts = []
    for i in range(2):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        k = _autograd.run_ad(kernel_fn.specs, a, b, True, precision,
                             bool(getattr(kernel_fn, 'diagonal', False)))
        torch.autograd.backward([k.nngp, k.ntk], [torch.ones_like(k.nngp), torch.ones_like(k.ntk)])
        e1.record()
        torch.cuda.synchronize()
        a.grad = b.grad = None
        del k
        if i:
            ts.append(e0.elapsed_time(e1))
    peak = torch.cuda.max_memory_allocated() - base
    return statistics.mean(ts), peak


def recompute_tile(kernel_fn, x_shape, precision: str = 'fp32',
                   candidates=TILE_CANDIDATES, memory_fraction: float = MEMORY_FRACTION) -> int:
    """The recompute tile for the checkpointed backward of ``kernel_fn`` on inputs
    of shape ``x_shape`` (batch axis first), chosen by timing probes."""
    dev = L.require_cuda()
    key = json.dumps(['recompute_tile', _device_name(), network_key(kernel_fn),
                      list(x_shape[1:]), precision])
    with _lock:
        _load()
        if key in _cache:
            return int(_cache[key]['tile'])
        free, _ = torch.cuda.mem_get_info()
        budget = memory_fraction * free
        gen = torch.Generator(device='cpu').manual_seed(0)
        tmax = max(candidates)
        sample = torch.randn((2 * tmax,) + tuple(x_shape[1:]), generator=gen).to(dev)
        trials = {}
        prev = None
        for t in sorted(candidates):
            if prev is not None:
                # peak memory grows with the pairs of a tile: skip what cannot fit
                tp, mp = prev
                if mp * (t * t) / (tp * tp) > budget:
                    break
            try:
                ms, peak = _probe(kernel_fn, sample, t, precision)
            except torch.cuda.OutOfMemoryError:
                torch.cuda.empty_cache()
                break
            if peak > budget:
                break
            trials[t] = {'ms': ms, 'peak': int(peak), 'ms_per_pair': ms / (t * t)}
            prev = (t, peak)
        torch.cuda.empty_cache()
        if not trials:
            best = min(candidates)
        else:
            best = min(trials, key=lambda t: trials[t]['ms_per_pair'])
        _store(key, {'tile': int(best), 'trials': {str(k): v for k, v in trials.items()}})
        return int(best)


def stencil_ring(pairs: int = 64, candidates=(2, 3, 4, 6)) -> int:
    """Times the 32x32 conv + ReLU stencil at each ring depth and sets the fastest."""
    from . import _ops as O
    lib = L.load()
    dev = L.require_cuda()
    key = json.dumps(['stencil_ring', _device_name()])
    with _lock:
        _load()
        if key in _cache:
            best = int(_cache[key]['ring'])
        else:
            q = torch.rand((pairs, 32, 32, 32, 32), device=dev) + 1.
            t = torch.rand_like(q)
            var = torch.rand((pairs, 32, 32), device=dev) + 2.
            v = L.Var(var.data_ptr(), 32 * 32, 32, 1)
            act = L.Act(L.NTG_ACT_ABRELU, 0., 1., 0., 0, 0.)
            trials = {}
            for ring in candidates:
                if lib.ntg_tune_set(L.NTG_TUNE_STENCIL_RING, ring) != 0:
                    continue
                ts = []
                for i in range(4):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    O.conv_fs(q, t, pairs, 1, 32, 32, 3, 3, 1, 1, 1, 1, 32, 32, False,
                              O.affine(2., 0., 2.), act, v, v, True, (pairs,))
                    e1.record()
                    torch.cuda.synchronize()
                    if i:
                        ts.append(e0.elapsed_time(e1))
                trials[ring] = statistics.median(ts)
            best = min(trials, key=trials.get)
            _store(key, {'ring': int(best), 'trials': {str(k): v for k, v in trials.items()}})
        if lib.ntg_tune_set(L.NTG_TUNE_STENCIL_RING, best) != 0:
            raise L.NtgError('ntg_tune_set rejected the tuned stencil ring')
        return best


def clear() -> None:
    """Forgets the in-memory cache (the JSON file, if any, is left alone)."""
    global _loaded
    with _lock:
        _cache.clear()
        _loaded = True
