"""Myrtle-5 NNGP+NTK throughput on GB300 (entries/s).

Workload: the full-spatial Myrtle-5 kernel (notebook definition: Conv3x3+Relu
x2, AvgPool, Conv+Relu, AvgPool, Conv+Relu, AvgPool x3, Flatten, Dense;
W_std = sqrt(2), b_std = 0) over 2000 synthetic CIFAR-shaped inputs
[2000, 32, 32, 3] (iid N(0, 1), standardised per channel, seed 0), computed as
the 2000 x 2000 nngp+ntk kernel K(x, x) through nt.batch(batch_size=100).
Because K(x, x) is symmetric, the job is the per-sample chains of the 2000
inputs plus the upper triangle of the 20 x 20 tile grid: 20 diagonal tiles
(pairs i <= j) and 190 off-diagonal tiles whose results are also written at
the mirrored position, 210 tiles in all. Step k is tile k of the triangle plus
1/210 of the per-sample chains, credited with the output entries its tile
produces (2 x 100^2 for an off-diagonal tile, 100^2 for a diagonal one; the 210
credits add up to 2000^2), so `value` estimates the throughput of the whole job
from any sample of steps. Steps are spread evenly over the
triangle; under torchrun rank r takes tiles r, r+N, ... (weak scaling).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line. `value` is device-timed throughput (inputs resident);
`e2e` is the same metric through the public API from pinned host buffers
with host<->device copies inside the timed region; `--impl reference` times
the CPU restatement of the reference's kernel rules (oracle/nt_oracle.py,
float32, one process per host core) on the same workload. Beside them:
`mixed` (the same job in the mixed form), `fwd_bwd` (a bounded sample of the
kernel-ridge forward + backward, fp32 and mixed), `clocks` (SM clock and
throttle reasons sampled during the timed steps), `gpu_launches` (this
library's kernels launched in the timed steps),
`parity` (sampled entries of the timed job against the float64 oracle),
`configs` (configurations 1, 3 and 5 at their stated sizes with their errors
against float64; `--no-full-configs` skips them), `roofline` / `compute` of
the fused kernel, the rooflines of the materialised stencil, the fused
backward (`vjp_roofline`) and the tensor-core Gram (`gram_tc`), and `side`
figures (Myrtle-10 block, Cholesky solve, NLL with its finite-difference
check). The `--profile-*` modes run one small case of a kernel for ncu and
exit.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ORACLE_LABEL = ('float64 oracle (CPU restatement of the reference\'s rules; it reproduces '
                'outputs of the reference\'s own code to 1e-12: tests/golden)')

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SAMPLES, TILE, IMG = 2000, 100, (32, 32, 3)
# Algorithmic HBM bytes per kernel entry of the layer-by-layer Myrtle-5 schedule
# (f32 nngp+ntk, every layer tensor written once and read once):
# (10 * 32^4 + 8 * 16^4 + 8 * 8^4) floats.
BYTES_PER_ENTRY = (10 * 32 ** 4 + 8 * 16 ** 4 + 8 * 8 ** 4) * 4
# FP32 operations per entry of the fused kernel, counted from its source per
# full-spatial element: Gram 4 FMA + 1 MUL; per conv+act layer 4 adds (A
# direction) + 4 adds (C direction) x 2 tensors, affine 4, ABRelu rule ~40.
FLOPS_PER_ELEM_LAYER = 4 * 2 + 4 * 2 + 4 + 40
# Warp instructions one pair costs in the Myrtle-5 fused kernel: smsp__inst_executed.sum of
# chain_fwd_kernel<2, 3, 1, 1, 1, 0, 3> over a 32 x 32 tile (ncu), divided by its 1024 pairs.
WARP_INSTR_PER_PAIR = 4.87e6
# Instruction issue peak: 152 SMs x 4 warp schedulers, one instruction per cycle each.
ISSUE_SLOTS_PER_CYCLE = 152 * 4


def tile_entries(tile) -> int:
    """Output entries of tile (r, c) of the upper triangle of the TILE x TILE grid: an
    off-diagonal tile is written at (r, c) and mirrored at (c, r)."""
    r, c = tile
    return TILE * TILE * (1 if r == c else 2)


def myrtle5(m):
    conv = lambda: m.Conv(1, (3, 3), padding='SAME', W_std=math.sqrt(2.), b_std=0.)
    layers = [conv(), m.Relu(), conv(), m.Relu(), m.AvgPool((2, 2), (2, 2)), conv(), m.Relu(),
              m.AvgPool((2, 2), (2, 2)), conv(), m.Relu()]
    layers += [m.AvgPool((2, 2), (2, 2))] * 3 + [m.Flatten(), m.Dense(10, math.sqrt(2.), 0.)]
    return layers


def make_inputs(n=N_SAMPLES, seed=0):
    x = np.random.default_rng(seed).standard_normal((n,) + IMG).astype(np.float32)
    x = (x - x.mean(axis=(0, 1, 2))) / x.std(axis=(0, 1, 2))
    return x.astype(np.float32)




def dist_env():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return ws, rank, local


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.gpu), f'--query-gpu={self.QUERY}',
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ''
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = [r.split(',') for r in (self.out or '').strip().splitlines() if r.strip()]
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for name, v in zip(names, r[5:9]):
                    if v.strip().lower() == 'active':
                        reasons.add(name)
            except (ValueError, IndexError):
                continue
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': mx,
                'reasons': sorted(reasons), 'samples': len(sm)}


def flush_l2(buf):
    buf.add_(1.0)  # 256 MiB write: larger than the 126 MB L2


def run_gpu(args):
    import torch
    import torch.distributed as dist

    import nt_gb300 as nt
    from nt_gb300 import _chain, _lib, stax
    from nt_gb300.stax import _Ctx

    ws, rank, local = dist_env()
    if ws > 1:
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    dev = torch.device('cuda', torch.cuda.current_device())
    x = make_inputs()
    xd = torch.from_numpy(x).to(dev)
    _, _, kf = stax.serial(*myrtle5(stax))
    plan = _chain.plan_chain(kf.specs, tuple(xd.shape), False)
    assert plan is not None, 'Myrtle-5 must take the fused chain path'
    from nt_gb300 import _ops as O
    from nt_gb300.kernel import Kernel
    # The job is K(x, x) over the 2000 inputs, as nt.batch(kf, 100)(x, None) computes it: the
    # per-sample chains of the 2000 inputs and the upper triangle of the 20 x 20 tile grid
    # (20 diagonal tiles with only i <= j evaluated, 190 off-diagonal tiles written at (i, j)
    # and (j, i)). Step k is tile k of the triangle plus the per-sample chains of samples
    # [k N / 210, (k + 1) N / 210): the 210 steps are the whole job, each credited with its
    # tile's output entries (tile_entries; N^2 over the 210 steps). Steps are spread evenly
    # over a rank's share of the tiles (tile k -> rank k % N).
    nt_ = N_SAMPLES // TILE
    tiles = [(r, c) for r in range(nt_) for c in range(r, nt_)]
    njob = len(tiles)
    slices = [(k * N_SAMPLES // njob, (k + 1) * N_SAMPLES // njob) for k in range(njob)]
    mine_all = list(range(rank, njob, ws))
    total_steps = args.warmup + args.steps
    mine = [mine_all[(s * len(mine_all)) // total_steps % len(mine_all)] for s in range(total_steps)]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    ctx32 = _Ctx('fp32')
    var_all, cov_all = _chain.self_chain(xd, plan, ctx32)
    out_q = torch.empty((N_SAMPLES, N_SAMPLES), device=dev)
    out_t = torch.empty((N_SAMPLES, N_SAMPLES), device=dev)
    shape_out = tuple(xd.shape)
    for sp in plan.spatial:
        shape_out = sp.shape_fn(shape_out)

    progs = {p: _chain._program(plan, 3, _Ctx(p)) for p in ('fp32', 'mixed')}

    def step(k, precision='fp32'):
        ctx = _Ctx(precision)
        r, c = tiles[k]
        # the tile's fused launch is enqueued first, so that the host-side work of the
        # per-sample slice below overlaps it (the variance maps it reads were computed in
        # the set-up; the slice recomputes 1/210 of them, as the job does once)
        O.chain_fwd_sym(progs[precision], xd, r * TILE, TILE, c * TILE, TILE, var_all, out_q,
                        out_t, N_SAMPLES)
        a, b = slices[k]
        v, cr = _chain.self_chain(xd[a:b], plan, ctx)
        var_all[a:b].copy_(v)
        cov_all[a:b].copy_(cr)
        # the layers after the readout (Dense) on the tile
        rs, cs = slice(r * TILE, (r + 1) * TILE), slice(c * TILE, (c + 1) * TILE)
        kt = Kernel(nngp=out_q[rs, cs].contiguous(), ntk=out_t[rs, cs].contiguous(),
                    cov1=cov_all[rs], cov2=cov_all[cs], x1_is_x2=False,
                    is_gaussian=plan.is_gaussian, is_reversed=False, is_input=False,
                    diagonal_batch=True, diagonal_spatial=False, shape1=shape_out,
                    shape2=shape_out)
        kf.apply_kernel(kt, ctx, specs=plan.post)

    stream = torch.cuda.current_stream()
    for s in range(args.warmup):
        step(mine[s])
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    launches0 = _lib.launch_count()
    # the NVTX range lets a profiler's launch list select exactly the timed steps
    torch.cuda.nvtx.range_push('timed_steps')
    with Clocks(local) as clk:
        for s in range(args.steps):
            flush_l2(flush)
            ev[s][0].record(stream)
            step(mine[args.warmup + s])
            ev[s][1].record(stream)
        torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    launches = _lib.launch_count() - launches0
    if ws > 1:
        dist.barrier()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    t = torch.tensor([ms], device=dev)
    if ws > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    e = torch.tensor([float(sum(tile_entries(tiles[mine[args.warmup + s]])
                                for s in range(args.steps)))], device=dev)
    if ws > 1:
        dist.all_reduce(e)
    value = float(e.item()) / (ms_max / 1e3)

    # Dominant kernel alone: the fused chain launch of one off-diagonal tile (10 000 pairs
    # evaluated), CUDA events on the launching stream, L2 flushed before each launch.
    pg = _chain._program(plan, 3, _Ctx('fp32'))
    kt = []
    for i in range(4):
        flush_l2(flush)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        O.chain_fwd_sym(pg, xd, 0, TILE, TILE, TILE, var_all, out_q, out_t, N_SAMPLES)
        b.record(stream)
        torch.cuda.synchronize()
        if i:
            kt.append(a.elapsed_time(b))
    chain_ms = statistics.median(kt)
    achieved_gbs = BYTES_PER_ENTRY * TILE * TILE / (chain_ms / 1e3) / 1e9
    flops_entry = (5 * 32 ** 4 + FLOPS_PER_ELEM_LAYER * (2 * 32 ** 4 + 16 ** 4 + 8 ** 4))
    achieved_tflops = flops_entry * TILE * TILE / (chain_ms / 1e3) / 1e12

    # Materialised per-layer stencil (conv + Relu epilogue) on a 16 x 16 tile at S = 32.
    st_gbs = stencil_roofline(torch, O, dev)
    # the fused backward of conv + ReLU (+ AvgPool) layers: VJP + transposed stencil
    vjp = [vjp_roofline(torch, dev, pooled) for pooled in (True, False)]
    gram_tc = gram_roofline(torch, O, dev)
    fb32, g32 = fwd_bwd_timing(torch, nt, kf, xd, precision='fp32')
    fbmx, gmx = fwd_bwd_timing(torch, nt, kf, xd, precision='mixed')
    fbmx['grad_rel_diff_vs_fp32'] = float((gmx - g32).abs().max() / g32.abs().max())
    fwd_bwd = {'ms': fbmx['ms'], 'fp32': fb32, 'mixed': fbmx}
    side = {'symmetric_grid': symmetric_grid_timing(torch, nt, kf, xd),
            'myrtle10': myrtle10_timing(torch, nt, xd), 'cholesky': cholesky_timing(torch, O, dev),
            'nll': nll_timing(torch, nt, dev)}

    # Mixed precision (compensated) variant of the same step and its error vs plain.
    torch.cuda.synchronize()
    em = []
    for s in range(min(args.steps, 5)):
        flush_l2(flush)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step(mine[args.warmup + s], 'mixed')
        b.record(stream)
        torch.cuda.synchronize()
        em.append(a.elapsed_time(b))
    mixed_value = (sum(tile_entries(tiles[mine[args.warmup + s]]) for s in range(len(em))) /
                   (sum(em) / 1e3))

    # End to end through the public API: the whole job nt.batch(kf, 100)(x, None) from pinned
    # host inputs, nngp and ntk read back to the host.
    # Under torchrun each rank takes a contiguous block of tile rows, K(x[rows], x), and the job
    # time is the slowest rank's.
    xh = torch.from_numpy(x).pin_memory()
    batched = nt.batch(kf, batch_size=TILE)
    if ws > 1:
        from nt_gb300.batching import rank_rows
        r0, r1 = rank_rows(N_SAMPLES, TILE, ws, rank)
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if ws > 1:
        res = batched(xh[r0:r1], xh, ('nngp', 'ntk'))
    else:
        res = batched(xh, None, ('nngp', 'ntk'))
    q, tt = res.nngp.cpu(), res.ntk.cpu()
    e2e_s = time.perf_counter() - t0
    if ws > 1:
        te = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
        e2e_s = float(te.item())
    e2e_value = N_SAMPLES * N_SAMPLES / e2e_s
    h2d = ws * N_SAMPLES * int(np.prod(IMG)) * 4
    d2h = 2 * N_SAMPLES * N_SAMPLES * 4

    # Parity sample of the benchmarked job: PARITY_PAIRS seeded entries of the 2000 x 2000
    # result (some on the diagonal, where the correlation is 1), fp32 as the e2e call returned
    # them, mixed from the same entries evaluated with precision='mixed'; the float64 oracle
    # values are computed in the CPU leg below.
    checks = []
    if ws == 1:
        pairs = parity_pairs(N_SAMPLES, PARITY_PAIRS, seed=7)
        ii = [i for i, _ in pairs]
        jj = [j for _, j in pairs]
        km = kf(xd[ii], xd[jj], ('nngp', 'ntk'), precision='mixed')
        k = torch.arange(len(pairs))
        checks.append({
            'name': 'myrtle5_2000', 'net': 'myrtle5', 'x': x, 'pairs': pairs,
            'got': {'fp32': (q[ii, jj].numpy(), tt[ii, jj].numpy()),
                    'mixed': (km.nngp[k, k].cpu().numpy(), km.ntk[k, k].cpu().numpy())}})
    full = {}
    if ws == 1 and args.full_configs:
        full['config1_fcn'], chk = config1_timing(torch, nt, dev)
        checks.append(chk)
        full['config5_krr'] = config5_timing(torch, nt, kf)
        full['config3_myrtle10'], chk = config3_timing(torch, nt, dev)
        checks.append(chk)

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json')))
    except OSError:
        pass
    hbm_peak = peaks.get('hbm_gbs', 6800.0)
    peak_note = 'of measured' if 'hbm_gbs' in peaks else 'of fallback'
    clocks = clk.summary()
    # The fused kernel's own bound: warp-instruction issue on the CUDA cores, at the SM clock
    # sampled during the timed steps.
    sm_mhz = clocks.get('sm_mhz') or 2070.0
    issue_peak = ISSUE_SLOTS_PER_CYCLE * sm_mhz * 1e6 / 1e9
    issue_achieved = WARP_INSTR_PER_PAIR * TILE * TILE / (chain_ms / 1e3) / 1e9
    issue = {'bound': 'issue', 'achieved': round(issue_achieved, 1), 'peak': round(issue_peak, 1),
             'unit': 'G warp instructions/s', 'frac': round(issue_achieved / issue_peak, 3),
             'warp_instructions_per_pair': WARP_INSTR_PER_PAIR,
             'note': 'instructions per pair from an ncu capture; peak = 152 SMs x 4 schedulers '
                     'x the sampled SM clock'}
    line = {
        'metric': 'Myrtle-5 NTK entries/s mixed vs plain FP32 (<=1e-4 vs FP64); fwd+bwd ms',
        'value': round(value, 1), 'unit': 'entries/s', 'n_gpus': ws, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': round(ms_max / args.steps, 3),
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': 'synthetic: iid N(0,1) [2000,32,32,3], standardised per channel, seed 0',
        'config': {'workload': 'Myrtle-5 full-spatial nngp+ntk K(x, x), x [2000, 32, 32, 3], '
                               'nt.batch(batch_size=100); the job is the per-sample chains and '
                               'the upper triangle of the 20x20 tile grid (210 tiles, '
                               'off-diagonal tiles mirrored); step = one tile of the triangle '
                               'plus 1/210 of the per-sample chains, credited with the output '
                               'entries of its tile (2x100^2 off the diagonal, 100^2 on it)',
                   'n_samples': N_SAMPLES, 'batch_size': TILE, 'input': list(IMG),
                   'precision': 'fp32 (plain)', 'l2': 'flushed before every step (256 MiB write)',
                   'path': 'fused chain kernel (ntg_chain_fwd_sym) + per-sample chains'},
        'mixed': {'value': round(mixed_value, 1), 'unit': 'entries/s',
                  'precision': 'compensated var1*var2 - q^2'},
        'e2e': {'value': round(e2e_value, 1), 'unit': 'entries/s', 'h2d_bytes_per_step': h2d,
                'd2h_bytes_per_step': d2h,
                'api': ('nt.batch(kernel_fn, 100)(x, None, get)' if ws == 1 else
                        'nt.batch(kernel_fn, 100)(x[rows of the rank], x, get) per rank'),
                'note': 'one call of the whole 2000x2000 job from pinned host memory, '
                        f'{e2e_s:.2f} s; bytes are per job'},
        'roofline': {'bound': 'hbm', 'achieved': round(achieved_gbs, 1), 'peak': hbm_peak,
                     'unit': 'GB/s', 'frac': round(achieved_gbs / hbm_peak, 3), 'traffic': None,
                     'kernel': 'chain_fwd_kernel', 'kernel_ms': round(chain_ms, 3),
                     'bytes_per_entry': BYTES_PER_ENTRY,
                     'note': f'{peak_note}; algorithmic bytes of the layer-by-layer schedule; '
                             'the fused kernel keeps them on chip',
                     'issue': issue},
        'compute': {'bound': 'fp32', 'achieved_tflops': round(achieved_tflops, 2),
                    'flops_per_entry': flops_entry},
        'stencil_roofline': st_gbs,
        'vjp_roofline': vjp,
        'gram_tc': gram_tc,
        'fwd_bwd': fwd_bwd,
        'side': side,
        'gpu_launches': int(launches),
        'clocks': clocks,
    }
    if full:
        line['configs'] = full
    if args.cpu_baseline and rank == 0 and ws == 1:
        line['cpu_baseline'] = cpu_baseline(x, args.cpu_seconds)
        parity = cpu_checks(checks)
        line['parity'] = parity.pop('myrtle5_2000')
        for name, res in parity.items():
            key = {'config1_fcn': 'config1_fcn', 'myrtle10_5000': 'config3_myrtle10'}[name]
            full[key]['parity'] = res
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        dist.destroy_process_group()


def stencil_roofline(torch, O, dev, pairs=256, reps=4):
    """Materialised 3x3 conv + Relu rule on [B, 32, 32, 32, 32] pairs (HBM-bound)."""
    from nt_gb300 import _lib as L
    B = pairs
    q = torch.rand((B, 32, 32, 32, 32), device=dev) + 1.
    t = torch.rand_like(q)
    var = torch.rand((B, 32, 32), device=dev) + 2.
    v = L.Var(var.data_ptr(), 32 * 32, 32, 1)
    aff = O.affine(2., 0., 2.)
    act = L.Act(L.NTG_ACT_ABRELU, 0., 1., 0., 0, 0.)
    outs = None
    ts = []
    for i in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        outs = O.conv_fs(q, t, B, 1, 32, 32, 3, 3, 1, 1, 1, 1, 32, 32, False, aff, act, v, v,
                         True, (B,))
        b.record()
        torch.cuda.synchronize()
        if i:
            ts.append(a.elapsed_time(b))
    del outs
    ms = statistics.median(ts) if ts else float('nan')
    nbytes = 4 * q.numel() * 4  # read nngp, ntk; write nngp, ntk
    gbs = nbytes / (ms / 1e3) / 1e9
    return {'kernel': 'conv3_skew_kernel', 'pairs': B, 'bytes': nbytes, 'ms': round(ms, 3),
            'achieved': round(gbs, 1), 'unit': 'GB/s'}


def vjp_roofline(torch, dev, pooled, n1=16, n2=32, reps=4):
    """Fused ReLU VJP + transposed 3x3 stencil (ntg_conv_act_bwd) on [B, 32, 32, 32, 32]
    pair kernels, B = n1 n2 = 512 pairs, both input cotangents written. Algorithmic bytes per
    entry: pre-activations 8, output cotangents 8 (0.5 after the 2x2 AvgPool, which pools
    both (h, h') and (w, w'): one cotangent entry per 16), input cotangents 8."""
    from nt_gb300 import _lib as L
    A = 32
    B = n1 * n2
    shp = (B, A, A, A, A)
    pre_q = torch.rand(shp, device=dev) * 2 - 1
    pre_t = torch.rand(shp, device=dev)
    gshape = (B, 16, 16, 16, 16) if pooled else shp
    gq = torch.rand(gshape, device=dev) - 0.5
    gt = torch.rand(gshape, device=dev) - 0.5
    var = torch.rand((n1 + n2, A, A), device=dev) + 2.
    v1 = L.Var(var[:n1].data_ptr(), A * A, A, 1)
    v2 = L.Var(var[n1:].data_ptr(), A * A, A, 1)
    act = L.Act(L.NTG_ACT_ABRELU, 0., 1., 0., 0, 0.)
    gin_q, gin_t = torch.empty(shp, device=dev), torch.empty(shp, device=dev)
    gd1, gd2 = torch.zeros((n1, A, A), device=dev), torch.zeros((n2, A, A), device=dev)
    ts = []
    for i in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        L.call('ntg_conv_act_bwd', L.stream(), L.ptr(pre_q), L.ptr(pre_t), L.ptr(gq), L.ptr(gt),
               int(pooled), L.ptr(gin_q), L.ptr(gin_t), B, n2, A, 2.0, act, v1, v2,
               gd1.data_ptr(), gd2.data_ptr())
        b.record()
        torch.cuda.synchronize()
        if i:
            ts.append(a.elapsed_time(b))
    L.check_device('ntg_conv_act_bwd')  # a timed call whose ring wait ran out would raise here
    ms = statistics.median(ts)
    entries = B * A ** 4
    per_entry = 8 + (0.5 if pooled else 8) + 8
    nbytes = int(entries * per_entry)
    return {'kernel': f'conv3_skew_vjp_kernel<{int(pooled)}>', 'pairs': B, 'bytes': nbytes,
            'bytes_per_entry': per_entry, 'ms': round(ms, 3),
            'achieved': round(nbytes / (ms / 1e3) / 1e9, 1), 'unit': 'GB/s'}


def fwd_bwd_timing(torch, nt, kf, xd, n_t=128, n_s=64, bs=64, precision='fp32', reps=2,
                   tile=None, xs_in=None, xt_in=None, diag_reg=1e-6):
    """Kernel-ridge loss of the Myrtle-5 NTK, ||y_t - K_ts (K_ss + 1e-6 tr(K_ss)/n I)^-1 y_s||^2,
    and its gradient with respect to the support set x_s (forward through nt.batch's fused
    grid, backward through its checkpointed tiles and the hand-written adjoints; the
    prediction K_ts A^-1 y_s and its adjoint on the library's Cholesky kernels and the
    double-float product, predict.kernel_ridge_predict). A bounded sample of the
    [200]-support / [2000]-target configuration: x_s [n_s], x_t [n_t] from the synthetic
    inputs, one-hot labels over 10 classes (seed 2)."""
    from nt_gb300 import predict
    g = torch.Generator(device='cpu').manual_seed(2)
    ys = torch.nn.functional.one_hot(torch.randint(0, 10, (n_s,), generator=g), 10).float().cuda()
    yt = torch.nn.functional.one_hot(torch.randint(0, 10, (n_t,), generator=g), 10).float().cuda()
    xt = xd[:n_t].contiguous() if xt_in is None else xt_in
    batched = nt.batch(kf, batch_size=bs, recompute_tile=tile)
    ts, grad = [], None
    for i in range(reps + 1):
        src = xd[1000:1000 + n_s] if xs_in is None else xs_in
        xs = src.clone().requires_grad_(True)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        kss = batched(xs, None, 'ntk', precision=precision)
        kts = batched(xt, xs, 'ntk', precision=precision)
        pred = predict.kernel_ridge_predict(kts, kss, ys, diag_reg=diag_reg)
        loss = ((yt - pred) ** 2).sum()
        loss.backward()
        b.record()
        torch.cuda.synchronize()
        if i:
            ts.append(a.elapsed_time(b))
        grad = xs.grad
    ms = statistics.mean(ts) if ts else float('nan')
    entries = n_s * n_s + n_t * n_s
    if tile is None:
        tile = nt.tune.recompute_tile(kf, tuple(xs.shape), precision)
    return {'ms': round(ms, 2), 'entries': entries, 'loss': float(loss.detach()),
            'entries_per_s': round(entries / (ms / 1e3), 1), 'precision': precision,
            'recompute_tile': min(tile, bs),
            'config': f'Myrtle-5 NTK kernel-ridge loss, d/dx_s; x_s [{n_s}], x_t [{n_t}], '
                      f'nt.batch(batch_size={bs}), autotuned recompute tile'}, grad


def myrtle10(m):
    """Myrtle-10: Conv3x3+Relu blocks [3, 3, 3] separated by AvgPool(2, 2), GlobalAvgPool, Dense."""
    conv = lambda: m.Conv(1, (3, 3), padding='SAME', W_std=2 ** .5, b_std=0.)
    layers = []
    for i, n in enumerate((3, 3, 3)):
        for _ in range(n):
            layers += [conv(), m.Relu()]
        if i < 2:
            layers += [m.AvgPool((2, 2), (2, 2))]
    return layers + [m.GlobalAvgPool(), m.Dense(10, 2 ** .5, 0.)]


def _timed(torch, fn, reps=3):
    ts = []
    for i in range(reps + 1):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        torch.cuda.synchronize()
        if i:
            ts.append(a.elapsed_time(b))
    return statistics.median(ts)


def myrtle10_timing(torch, nt, xd, n1=128, n2=200):
    """Myrtle-10 nngp+ntk on a ragged 128 x 200 block of the synthetic inputs (one fused
    launch over the block plus the per-sample chains of its 328 inputs), plain and mixed."""
    from nt_gb300 import stax
    _, _, kf = stax.serial(*myrtle10(stax))
    x1, x2 = xd[:n1].contiguous(), xd[n1:n1 + n2].contiguous()
    out = {'config': f'Myrtle-10 [3,3,3] + GlobalAvgPool, block {n1} x {n2}'}
    for prec in ('fp32', 'mixed'):
        ms = _timed(torch, lambda: kf(x1, x2, ('nngp', 'ntk'), precision=prec))
        out[prec] = {'ms': round(ms, 2), 'entries_per_s': round(n1 * n2 / (ms / 1e3), 1)}
    return out


def symmetric_grid_timing(torch, nt, kf, xd, n=1000):
    """K(x, x) over n inputs through nt.batch(kernel_fn, 100)(x, None): the fused kernel
    evaluates the pairs i <= j once (one persistent launch over the triangle) and mirrors
    them; entries/s counts all n^2 entries of the result."""
    x = xd[:n].contiguous()
    batched = nt.batch(kf, batch_size=100)
    ms = _timed(torch, lambda: batched(x, None, ('nngp', 'ntk')), reps=2)
    return {'n': n, 'ms': round(ms, 2), 'entries_per_s': round(n * n / (ms / 1e3), 1),
            'config': f'Myrtle-5 K(x, x), x [{n}], nt.batch(batch_size=100), symmetric grid'}


def cholesky_timing(torch, O, dev, n=5000, m=10):
    """predict.gradient_descent_mse at t = None for n = 5000 training points and 10 one-hot
    targets: FP32 Cholesky of K + 1e-4 tr(K)/n I on the tensor cores, the solve by the explicit
    inverse factors refined by conjugate gradients with double-float products, and the test
    prediction for 100 points (double-float product with the FP64 solution). K is a synthetic SPD kernel (the Gram of
    iid N(0,1) features of width 6144)."""
    from nt_gb300 import predict
    g = torch.Generator(device='cpu').manual_seed(2)
    x = torch.randn((n, 6144), device=dev)
    k = O.gram(x, x, 0)
    y = torch.nn.functional.one_hot(torch.randint(0, 10, (n,), generator=g), m).float().to(dev)
    kts = k[:100].contiguous()
    res = {}

    def run():
        pred = predict.gradient_descent_mse(k, y, diag_reg=1e-4)
        res['out'] = pred(None, 0., 0., kts)

    ms = _timed(torch, run)
    return {'n': n, 'targets': m, 'ms': round(ms, 2),
            'flops': round(n ** 3 / 3 / 1e9, 1), 'unit_flops': 'GFLOP (factorisation)'}


def nll_timing(torch, nt, dev):
    """NNGP negative log marginal likelihood of a depth-3 FCN (Dense+Relu x 3, Dense) on
    X [4096, 3072], Y [4096, 10] (iid N(0,1)) and its gradient with respect to the shared
    (W_std, b_std): input Gram, layer rules and their adjoints, Cholesky and its adjoint."""
    from nt_gb300 import predict, stax
    gen = torch.Generator(device='cpu').manual_seed(3)
    x = torch.randn((4096, 3072), generator=gen).to(dev)
    y = torch.randn((4096, 10), generator=gen).to(dev)
    out = {'config': 'depth-3 FCN NNGP NLL, X [4096, 3072] and Y [4096, 10] iid N(0, 1) '
                     '(seed 3), d/d(W_std, b_std)'}
    for prec in ('fp32', 'mixed'):
        w = torch.tensor(1.5, device=dev, requires_grad=True)
        b = torch.tensor(0.1, device=dev, requires_grad=True)
        kf = stax.serial(stax.Dense(512, w, b), stax.Relu(), stax.Dense(512, w, b), stax.Relu(),
                         stax.Dense(512, w, b), stax.Relu(), stax.Dense(1, w, b))[2]

        def run():
            w.grad = b.grad = None
            k = kf(x, None, 'nngp', precision=prec)
            predict.negative_log_likelihood(k, y, diag_reg=1e-4).backward()

        ms = _timed(torch, run)
        out[prec] = {'ms': round(ms, 2), 'grad': [float(w.grad), float(b.grad)]}
        if prec == 'fp32':
            # central differences in W_std and b_std, steps h and 2h, Richardson-extrapolated,
            # of the NLL evaluated in FP64 from the same kernel, factorisation and refined
            # solve (the forward returns it rounded to float32); h = 1e-2: the float32 kernel's
            # rounding moves this NLL by about n cond(A) u, which a 1e-3 step would resolve
            # only to ~1e-3 of b_std's gradient
            def nll_at(wv, bv):
                with torch.no_grad():
                    kf2 = stax.serial(stax.Dense(512, wv, bv), stax.Relu(), stax.Dense(512, wv, bv),
                                      stax.Relu(), stax.Dense(512, wv, bv), stax.Relu(),
                                      stax.Dense(1, wv, bv))[2]
                    solver = predict.CholeskySolver(kf2(x, None, 'nngp'), 1e-4, False)
                    _, a64 = solver.solve(y, want_x64=True, residual=False)
                    n, m = y.shape
                    return (0.5 * float((y.double() * a64).sum()) +
                            0.5 * m * float(solver.logdet()[0]) +
                            0.5 * n * m * math.log(2 * math.pi))
            fd = []
            for which in (0, 1):
                base = [1.5, 0.1]

                def central(h):
                    hi, lo = list(base), list(base)
                    hi[which] += h
                    lo[which] -= h
                    return (nll_at(*hi) - nll_at(*lo)) / (2 * h)
                fd.append((4 * central(1e-2) - central(2e-2)) / 3)
            out[prec]['fd_grad'] = fd
            out[prec]['grad_rel_diff_vs_fd'] = max(
                abs(g - f) / abs(f) for g, f in zip(out[prec]['grad'], fd))
    return out


def gram_roofline(torch, O, dev):
    """tcgen05 split-BF16 Gram of the NLL configuration, X [4096, 3072]: X X^T / D, as the
    kernel computes it for x1 is x2 (the 272 tiles of 128 x 256 that reach the diagonal or lie
    below it, mirrored) and for two distinct operands (all 512 tiles). FP32-equivalent rate:
    2 n^2 d over the call; tensor rate: the three BF16 products of the tiles computed."""
    x = torch.randn((4096, 3072), device=dev)
    y = x.clone()
    n, d, nb = 4096, 3072, 4096 // 128
    out = {'kernel': 'gram_tc_kernel (+ bf16 split)', 'shape': [n, n, d], 'unit': 'TFLOP/s'}
    sym_tiles = (nb // 2) * (nb // 2 + 1) if nb % 2 == 0 else (nb // 2 + 1) ** 2
    for name, other, tiles in (('symmetric', x, sym_tiles), ('general', y, nb * (n // 256))):
        ts = []
        for i in range(4):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            O.gram(x, other, 1)
            b.record()
            torch.cuda.synchronize()
            if i:
                ts.append(a.elapsed_time(b))
        ms = statistics.median(ts)
        issued = 3 * 2 * tiles * 128 * 256 * d
        out[name] = {'ms': round(ms, 3),
                     'tflops_fp32_equivalent': round(2 * n * n * d / (ms / 1e3) / 1e12, 1),
                     'tensor_tflops_issued': round(issued / (ms / 1e3) / 1e12, 1)}
    out['ms'] = out['symmetric']['ms']
    return out


PARITY_PAIRS = 48


def parity_pairs(n, count, seed):
    """`count` seeded (i, j) entries of an n x n kernel, one in six on the diagonal."""
    rng = np.random.default_rng(seed)
    pairs = [(int(i), int(i)) for i in rng.choice(n, count // 6, replace=False)]
    while len(pairs) < count:
        i, j = (int(v) for v in rng.integers(0, n, 2))
        if i != j:
            pairs.append((i, j))
    return pairs


def fcn_layers(m):
    return [m.Dense(512, W_std=1.5, b_std=0.05), m.Relu(), m.Dense(512, W_std=1.5, b_std=0.05),
            m.Relu(), m.Dense(1, W_std=1.5, b_std=0.05)]


def fcn_inputs():
    """Configuration 1: x1, x2 [256, 784] iid N(0, 1) (seeds 0 and 1), rows rescaled to norm
    sqrt(784); y [256, 10] one-hot labels drawn uniformly (seed 2)."""
    xs = []
    for seed in (0, 1):
        v = np.random.default_rng(seed).standard_normal((256, 784))
        xs.append((v / np.linalg.norm(v, axis=1, keepdims=True) * math.sqrt(784)).astype(np.float32))
    y = np.eye(10, dtype=np.float32)[np.random.default_rng(2).integers(0, 10, 256)]
    return xs[0], xs[1], y


def config1_timing(torch, nt, dev, reps=5):
    """Configuration 1 end to end on the device: kernel_fn(x1, x2, ('nngp', 'ntk')) of the
    three-layer ReLU FCN, then gradient_descent_mse(k_train_train, y, diag_reg=1e-4) at
    t = None and t = inf (test predictions on x2 with fx_train_0 = fx_test_0 = 0); the
    train-train and test-train NTKs come from the same kernel_fn. Times are medians of
    `reps` calls (CUDA events, inputs resident)."""
    from nt_gb300 import stax
    x1h, x2h, yh = fcn_inputs()
    x1, x2, y = (torch.from_numpy(v).to(dev) for v in (x1h, x2h, yh))
    kf = stax.serial(*fcn_layers(stax))[2]
    out = {'config': 'FCN Dense(512,1.5,0.05)-Relu x2-Dense(1); x1, x2 [256, 784] on the sphere '
                     'of radius sqrt(784) (seeds 0, 1); y one-hot [256, 10] (seed 2); '
                     'gradient_descent_mse diag_reg=1e-4'}
    res = {}

    def kernels():
        res['k12'] = kf(x1, x2, ('nngp', 'ntk'))
    out['kernel_fn_us'] = round(_timed(torch, kernels, reps) * 1e3, 1)
    ktt = kf(x1, None, 'ntk')
    kts = kf(x2, x1, 'ntk')
    for t, name in ((None, 't_none'), (float('inf'), 't_inf')):
        def solve():
            res[name] = nt.predict.gradient_descent_mse(ktt, y, diag_reg=1e-4)(t, 0., 0., kts)
        out[f'gradient_descent_mse_{name}_us'] = round(_timed(torch, solve, reps) * 1e3, 1)

    def whole():
        k = kf(x1, None, 'ntk')
        nt.predict.gradient_descent_mse(k, y, diag_reg=1e-4)(float('inf'), 0., 0.,
                                                              kf(x2, x1, 'ntk'))
    out['end_to_end_us'] = round(_timed(torch, whole, reps) * 1e3, 1)
    check = {'name': 'config1_fcn', 'kind': 'fcn', 'x1': x1h, 'x2': x2h, 'y': yh,
             'got': {'nngp': res['k12'].nngp.cpu().numpy(), 'ntk': res['k12'].ntk.cpu().numpy(),
                     'fx_test_t_none': res['t_none'][1].cpu().numpy(),
                     'fx_test_t_inf': res['t_inf'][1].cpu().numpy()}}
    return out, check


def config5_timing(torch, nt, kf):
    """Configuration 5 at its stated size: the Myrtle-5 NTK kernel-ridge loss
    ||y_t - K_ts (K_ss + 1e-6 tr(K_ss)/n I)^-1 y_s||^2 and d loss / d x_s for x_s [200]
    (iid N(0, 1), seed 5) and x_t [2000] (seed 6), one-hot y_s, y_t over 10 classes
    (seed 2), in the plain FP32 and the mixed forms (one warm-up evaluation, one timed).
    Parity of these gradients against float64 finite differences of the oracle is checked
    at reduced sizes in the test suite (the oracle would need days at this size); here the
    gradient is checked against central differences of the loss along its own direction
    through the same forward path, Richardson-extrapolated from steps h and 2h that move the
    loss by about 1 % and 2 % (the float32 kernels fix the loss to about cond(A) u, which
    bounds any such check at diag_reg = 1e-6)."""
    dev = torch.device('cuda', torch.cuda.current_device())
    xs = torch.from_numpy(np.random.default_rng(5).standard_normal((200,) + IMG).astype(
        np.float32)).to(dev)
    xt = torch.from_numpy(np.random.default_rng(6).standard_normal((2000,) + IMG).astype(
        np.float32)).to(dev)
    out = {}
    grads = {}
    for prec in ('fp32', 'mixed'):
        r, g = fwd_bwd_timing(torch, nt, kf, None, n_t=2000, n_s=200, bs=200, precision=prec,
                              reps=1, xs_in=xs, xt_in=xt)
        out[prec] = r
        grads[prec] = g
    out['mixed']['grad_rel_diff_vs_fp32'] = float(
        (grads['mixed'] - grads['fp32']).abs().max() / grads['fp32'].abs().max())
    # Conditioning of K_ss + 1e-6 tr(K_ss)/n I: its float32 rounding bounds how well any
    # float32 evaluation (the reference's included) determines this loss and its gradient.
    with torch.no_grad():
        kss = nt.batch(kf, batch_size=200)(xs, None, 'ntk').double().cpu().numpy()
    ev = np.linalg.eigvalsh(kss + 1e-6 * np.trace(kss) / 200 * np.eye(200))
    out['cond_kss_reg'] = float(ev[-1] / ev[0])
    # Directional derivative checks of the fp32 gradient along g / |g|: the stated
    # diag_reg = 1e-6, and a better-conditioned diag_reg = 1e-2 that exercises the same
    # kernels with float32 rounding far below the difference quotient.
    for reg, g in ((1e-6, grads['fp32']), (1e-2, None)):
        if g is None:
            _, g = fwd_bwd_timing(torch, nt, kf, None, n_t=2000, n_s=200, bs=200, reps=0,
                                  xs_in=xs, xt_in=xt, diag_reg=reg)
        v = (g / g.norm()).to(dev)
        with torch.no_grad():
            l0 = krr_loss(torch, nt, kf, xs, xt, 'fp32', diag_reg=reg)
            h = 1e-2 * abs(l0) / float(g.norm())

            def central(step):
                lp = krr_loss(torch, nt, kf, xs + step * v, xt, 'fp32', diag_reg=reg)
                lm = krr_loss(torch, nt, kf, xs - step * v, xt, 'fp32', diag_reg=reg)
                return (lp - lm) / (2 * step)
            d1, d2 = central(h), central(2 * h)
        fd_dir = (4 * d1 - d2) / 3
        an = float(g.norm())
        out['fp32'][f'directional_fd_rel_diff_diag_reg_{reg:g}'] = abs(an - fd_dir) / abs(fd_dir)
    out['config'] = ('Myrtle-5 NTK kernel-ridge loss, d/dx_s; x_s [200] (seed 5), x_t [2000] '
                     '(seed 6) iid N(0,1); y one-hot over 10 classes (seed 2); '
                     'nt.batch(batch_size=200) with the autotuned recompute tile')
    return out


def krr_loss(torch, nt, kf, xs, xt, precision, bs=200, diag_reg=1e-6):
    """The configuration-5 loss value (float64 on the host) without gradients."""
    from nt_gb300 import predict
    n_s, n_t = xs.shape[0], xt.shape[0]
    g = torch.Generator(device='cpu').manual_seed(2)
    ys = torch.nn.functional.one_hot(torch.randint(0, 10, (n_s,), generator=g), 10).float().cuda()
    yt = torch.nn.functional.one_hot(torch.randint(0, 10, (n_t,), generator=g), 10).float().cuda()
    batched = nt.batch(kf, batch_size=bs)
    kss = batched(xs, None, 'ntk', precision=precision)
    kts = batched(xt, xs, 'ntk', precision=precision)
    pred = predict.kernel_ridge_predict(kts, kss, ys, diag_reg=diag_reg)
    return float(((yt - pred).double() ** 2).sum())


def config3_timing(torch, nt, dev, n=5000, bs=128):
    """Configuration 3 at its stated size: the Myrtle-10 NTK and NNGP K(x, x) of x
    [5000, 32, 32, 3] iid N(0, 1) (seed 0) in the mixed form (split-precision first layer,
    compensated arccos) through nt.batch(batch_size=128) (ragged: 5000 = 39 x 128 + 8, one
    fused launch over the symmetric grid), then gradient_descent_mse(ntk, y, diag_reg=1e-4)
    at t = None (FP32 Cholesky of the 5000 x 5000 kernel on the tensor cores, refinement by
    conjugate gradients) with y one-hot over 10 classes (seed 2), predicting 100 held-out
    inputs (iid N(0, 1), seed 1). Wall-clock seconds, the job once; the kernel entries, the
    solve A^-1 y and the predictions are checked in the CPU leg against float64."""
    from nt_gb300 import stax
    xh = np.random.default_rng(0).standard_normal((n,) + IMG).astype(np.float32)
    xth = np.random.default_rng(1).standard_normal((100,) + IMG).astype(np.float32)
    yh = np.eye(10, dtype=np.float32)[np.random.default_rng(2).integers(0, 10, n)]
    x, y = torch.from_numpy(xh).to(dev), torch.from_numpy(yh).to(dev)
    xt = torch.from_numpy(xth).to(dev)
    kf = stax.serial(*myrtle10(stax))[2]
    batched = nt.batch(kf, batch_size=bs)
    batched(x[:256], None, ('nngp', 'ntk'), precision='mixed')  # warm-up (library, planner)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    k = batched(x, None, ('nngp', 'ntk'), precision='mixed')
    torch.cuda.synchronize()
    kernel_s = time.perf_counter() - t0
    kts = batched(xt, x, 'ntk', precision='mixed')
    t0 = time.perf_counter()
    pred = nt.predict.gradient_descent_mse(k.ntk, y, diag_reg=1e-4)
    fx = pred(None, 0., 0., kts)[1]
    torch.cuda.synchronize()
    solve_s = time.perf_counter() - t0
    alpha = nt.predict.CholeskySolver(k.ntk, 1e-4, False).solve(y)
    pairs = parity_pairs(n, 24, seed=9)
    ii = [i for i, _ in pairs]
    jj = [j for _, j in pairs]
    out = {'config': f'Myrtle-10 [3,3,3] + GlobalAvgPool + Dense, K(x, x), x [{n}, 32, 32, 3] '
                     f'iid N(0,1) (seed 0), mixed form, nt.batch(batch_size={bs}) ragged; then '
                     'gradient_descent_mse(ntk, one-hot y (seed 2), diag_reg=1e-4) at t=None, '
                     'predictions for 100 held-out inputs (seed 1)',
           'kernel_s': round(kernel_s, 2), 'entries_per_s': round(n * n / kernel_s, 1),
           'solve_ms': round(solve_s * 1e3, 2)}
    check = {'name': 'myrtle10_5000', 'net': 'myrtle10', 'x': xh, 'pairs': pairs,
             'got': {'mixed': (k.nngp[ii, jj].cpu().numpy(), k.ntk[ii, jj].cpu().numpy())},
             'solve': {'k': k.ntk.cpu().numpy(), 'y': yh, 'kts': kts.cpu().numpy(),
                       'fx_test': fx.cpu().numpy(), 'alpha': alpha.cpu().numpy()}}
    return out, check


def _oracle_pair(args):
    """float64 oracle (nngp, ntk) of one pair of images through a Myrtle network."""
    net, a, b = args
    sys.path.insert(0, ROOT)
    from oracle import nt_oracle as o
    layers = myrtle5(o) if net == 'myrtle5' else myrtle10(o)
    q, t = o.serial(*layers)(a[None], b[None], ('nngp', 'ntk'))
    return float(q.reshape(())), float(t.reshape(()))


def _rel(got, want):
    return float(np.max(np.abs(np.asarray(got, np.float64) - want) / np.abs(want)))


def cpu_checks(checks, procs=None):
    """The checker half of the CPU leg: the float64 oracle on the sampled entries (and the
    FCN and solve configurations) of what the GPU computed; max relative errors per form."""
    import multiprocessing as mp
    sys.path.insert(0, ROOT)
    from oracle import nt_oracle as o
    procs = procs or os.cpu_count() or 1
    out = {}
    tasks, owners = [], []
    for c in checks:
        if 'pairs' in c:
            for (i, j) in c['pairs']:
                tasks.append((c['net'], c['x'][i], c['x'][j]))
                owners.append(c['name'])
    t0 = time.perf_counter()
    with mp.get_context('spawn').Pool(procs) as pool:
        vals = pool.map(_oracle_pair, tasks, chunksize=1)
    pair_s = time.perf_counter() - t0
    for c in checks:
        if 'pairs' in c:
            want = np.array([v for v, name in zip(vals, owners) if name == c['name']])
            res = {'entries': len(c['pairs']), 'reference': ORACLE_LABEL,
                   'oracle_s': round(pair_s, 1)}
            for form, (gq, gt) in c['got'].items():
                res[f'max_rel_err_{form}'] = max(_rel(gq, want[:, 0]), _rel(gt, want[:, 1]))
            if 'solve' in c:
                # the solve and the predictions against float64 on the same GPU kernel matrix
                import scipy.linalg as sla
                sv = c['solve']
                k64 = np.asarray(sv['k'], np.float64)
                a = k64 + 1e-4 * np.trace(k64) / k64.shape[0] * np.eye(k64.shape[0])
                alpha = sla.cho_solve(sla.cho_factor(a), np.asarray(sv['y'], np.float64))
                res['solve_max_rel_err_vs_float64'] = float(
                    np.max(np.abs(sv['alpha'] - alpha)) / np.max(np.abs(alpha)))
                ref = np.asarray(sv['kts'], np.float64) @ alpha
                res['predictions_max_rel_err_vs_float64'] = float(
                    np.max(np.abs(sv['fx_test'] - ref)) / np.max(np.abs(ref)))
            out[c['name']] = res
        elif c.get('kind') == 'fcn':
            kf = o.serial(*fcn_layers(o))
            q, t = kf(c['x1'], c['x2'], ('nngp', 'ntk'))
            ktt = kf(c['x1'], None, 'ntk')
            kts = kf(c['x2'], c['x1'], 'ntk')
            pred = o.gradient_descent_mse(ktt, c['y'], diag_reg=1e-4)
            g = c['got']
            res = {'reference': ORACLE_LABEL,
                   'max_rel_err_nngp': _rel(g['nngp'], q), 'max_rel_err_ntk': _rel(g['ntk'], t)}
            for name, t_ in (('t_none', None), ('t_inf', np.inf)):
                want = pred(t_, 0., 0., kts)[1]
                res[f'fx_test_{name}_max_err_rel_to_max'] = float(
                    np.max(np.abs(g[f'fx_test_{name}'] - want)) / np.max(np.abs(want)))
            out[c['name']] = res
    return out


REF_TILE = 4


def _ref_tile(args):
    """A REF_TILE x REF_TILE block of kernel entries (nngp, ntk) from the float32 oracle."""
    x1, x2 = args
    sys.path.insert(0, ROOT)
    from oracle import nt_oracle as o
    kf = o.serial(*myrtle5(o))
    nngp, ntk = kf(x1, x2, ('nngp', 'ntk'), dtype=np.float32)
    return nngp.size


def cpu_baseline(x, seconds=15.0, procs=None):
    """Times the oracle (float32) on tiles of the same workload, one process per core."""
    import multiprocessing as mp
    procs = procs or os.cpu_count() or 1
    ctx = mp.get_context('spawn')
    done = 0
    b = REF_TILE
    with ctx.Pool(procs) as pool:
        pool.map(_ref_tile, [(x[:b], x[b:2 * b])] * procs)  # warm the workers
        t0 = time.perf_counter()
        i = 0
        while time.perf_counter() - t0 < seconds:
            batch = [(x[(i + k) * b % 2000:][:b], x[(1000 + (i + 2 * k) * b) % 2000:][:b])
                     for k in range(procs)]
            done += sum(pool.map(_ref_tile, batch))
            i += procs
        el = time.perf_counter() - t0
    return {'value': round(done / el, 3), 'unit': 'entries/s', 'cores': procs, 'kind': 'port',
            'sample': f'{done} Myrtle-5 entries of the 2000x2000 grid as {b}x{b} tiles (nngp+ntk '
                      f'and the tiles\' per-sample chains), float32 oracle, {procs} processes, '
                      f'{el:.1f} s'}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    x = make_inputs()
    procs = os.cpu_count() or 1
    per_step = []
    for s in range(args.warmup + args.steps):
        r = cpu_baseline(x, seconds=args.ref_step_seconds, procs=procs)
        if s >= args.warmup:
            per_step.append(r['value'])
    value = statistics.mean(per_step)
    line = {
        'impl': 'reference', 'metric': 'Myrtle-5 NTK entries/s mixed vs plain FP32 (<=1e-4 vs '
                                       'FP64); fwd+bwd ms',
        'value': round(value, 3), 'unit': 'entries/s', 'n_gpus': ws, 'steps': args.steps,
        'warmup': args.warmup, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32', 'data': 'synthetic: iid N(0,1) [2000,32,32,3], standardised, seed 0',
        'config': {'workload': 'Myrtle-5 full-spatial nngp+ntk, 2000x2000 via '
                               'nt.batch(batch_size=100); step = a bounded sample of pairs',
                   'n_samples': N_SAMPLES, 'batch_size': TILE},
        'cpu_baseline': {'value': round(value, 3), 'unit': 'entries/s', 'cores': procs,
                         'kind': 'port',
                         'sample': f'{args.ref_step_seconds:.0f} s of {REF_TILE}x{REF_TILE} tiles per step, float32 '
                                   'restatement of the reference rules (oracle/nt_oracle.py); '
                                   'the JAX reference is not installable here'},
        'e2e': {'value': round(value, 3), 'unit': 'entries/s', 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line))


def profile_tile(p: int):
    """One fused-chain launch on a p x p tile (a small case for ncu captures)."""
    import torch
    from nt_gb300 import _chain, _ops as O, stax
    from nt_gb300.stax import _Ctx
    x = torch.from_numpy(make_inputs(2 * p)).cuda()
    _, _, kf = stax.serial(*myrtle5(stax))
    plan = _chain.plan_chain(kf.specs, tuple(x.shape), False)
    ctx = _Ctx('fp32')
    var, _ = _chain.self_chain(x, plan, ctx)
    pg = _chain._program(plan, 3, ctx)
    oq = torch.empty((p, p), device='cuda')
    ot = torch.empty((p, p), device='cuda')
    O.chain_fwd(pg, x[:p], x[p:], 0, p, 0, p, var[:p].contiguous(), var[p:].contiguous(), oq, ot, p)
    torch.cuda.synchronize()
    print(json.dumps({'profile_tile': p, 'nngp_mean': float(oq.mean()), 'ntk_mean': float(ot.mean())}))


def profile_stencil(pairs: int):
    """One materialised conv+ReLU stencil launch on `pairs` 32^4 pairs (ncu small case)."""
    import torch
    from nt_gb300 import _ops as O
    st = stencil_roofline(torch, O, torch.device('cuda'), pairs=pairs, reps=1)
    print(json.dumps({'profile_stencil': pairs, **st}))


def profile_fwd_bwd(n_s: int):
    """The fwd+bwd measurement alone: x_s [n_s], x_t [2 n_s], batch_size and recompute tile n_s
    (no autotuning probes in the launch list)."""
    import torch
    import nt_gb300 as nt
    from nt_gb300 import stax
    _, _, kf = stax.serial(*myrtle5(stax))
    x = torch.from_numpy(make_inputs(2000)).cuda()
    r, _ = fwd_bwd_timing(torch, nt, kf, x, n_t=2 * n_s, n_s=n_s, bs=n_s, reps=1, tile=n_s)
    print(json.dumps({'profile_fwd_bwd': n_s, **r}))


def profile_gram(n: int):
    """One split-BF16 tcgen05 Gram X X^T / D of X [n, 3072] (ncu small case)."""
    import torch
    from nt_gb300 import _ops as O
    x = torch.randn((n, 3072), device='cuda')
    g = O.gram(x, x, 1)
    torch.cuda.synchronize()
    print(json.dumps({'profile_gram': n, 'mean': float(g.mean())}))


def profile_chol(n: int):
    """Factor + solve of gradient_descent_mse's Cholesky path on an SPD kernel of order n (the
    Gram of iid N(0, 1) features [n, 6144] / 6144, diag_reg 1e-4, 10 one-hot targets), after
    a warm-up factorisation; NVTX ranges 'factor' and 'solve' select the launches."""
    import torch
    from nt_gb300 import _ops as O, predict
    dev = torch.device('cuda')
    g = torch.Generator(device='cpu').manual_seed(2)
    x = torch.randn((n, 6144), device=dev)
    k = O.gram(x, x, 0)
    y = torch.nn.functional.one_hot(torch.randint(0, 10, (n,), generator=g), 10).float().to(dev)
    predict.CholeskySolver(k, 1e-4, False)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push('factor')
    s = predict.CholeskySolver(k, 1e-4, False)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    torch.cuda.nvtx.range_push('solve')
    s.solve(y)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print(json.dumps({'profile_chol': n, 'residual': float(s.residual.item()), 'info': s.info}))


def profile_nll():
    """The NLL forward + backward of the bench's depth-3 FCN (X [4096, 3072]), twice (the
    first a warm-up; autograd runs the backward on its own thread, so select by launch
    count rather than NVTX)."""
    import torch
    from nt_gb300 import predict, stax
    dev = torch.device('cuda')
    gen = torch.Generator(device='cpu').manual_seed(3)
    x = torch.randn((4096, 3072), generator=gen).to(dev)
    y = torch.randn((4096, 10), generator=gen).to(dev)
    w = torch.tensor(1.5, device=dev, requires_grad=True)
    b = torch.tensor(0.1, device=dev, requires_grad=True)
    kf = stax.serial(stax.Dense(512, w, b), stax.Relu(), stax.Dense(512, w, b), stax.Relu(),
                     stax.Dense(512, w, b), stax.Relu(), stax.Dense(1, w, b))[2]
    for _ in range(2):
        w.grad = b.grad = None
        predict.negative_log_likelihood(kf(x, None, 'nngp'), y, diag_reg=1e-4).backward()
    torch.cuda.synchronize()
    print(json.dumps({'profile_nll': 4096, 'grad': [float(w.grad), float(b.grad)]}))


def profile_predict(n: int):
    """Finite-time predictions (the eigenbasis paths of predict.py:185-229 and 860-1005) of
    the FCN configuration on n training inputs [n, 784] (seed 0) and 64 test inputs (seed 1):
    gradient_descent_mse at t = [1, 10, 100] with the test predictions, then the infinite
    ensemble's NNGP/NTK means and covariances at t = 10; an NVTX range 'predict' selects the
    launches after a warm-up of the same calls."""
    import torch
    import nt_gb300 as nt
    from nt_gb300 import stax
    dev = torch.device('cuda')
    rows = []
    for seed, count in ((0, n), (1, 64)):
        v = np.random.default_rng(seed).standard_normal((count, 784))
        rows.append(torch.from_numpy((v / np.linalg.norm(v, axis=1, keepdims=True) *
                                      math.sqrt(784)).astype(np.float32)).to(dev))
    x, xt = rows
    y = torch.nn.functional.one_hot(torch.arange(n) % 10, 10).float().to(dev)
    kf = stax.serial(*fcn_layers(stax))[2]
    ktt = kf(x, None, 'ntk')
    kts = kf(xt, x, 'ntk')

    def run():
        pred = nt.predict.gradient_descent_mse(ktt, y, diag_reg=1e-4)
        out = pred([1., 10., 100.], 0., 0., kts)
        ens = nt.predict.gradient_descent_mse_ensemble(kf, x, y, diag_reg=1e-4)
        mean_cov = ens(10., xt, ('nngp', 'ntk'), compute_cov=True)
        return out, mean_cov
    run()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push('predict')
    out, mean_cov = run()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print(json.dumps({'profile_predict': n, 'fx_test_sum': float(out[1].sum())}))


def profile_gemm(n: int):
    """Two n x n x n calls of the 3xTF32 tensor-core GEMM (ntg_gemm_tc), C = A B^T."""
    import torch
    from nt_gb300 import _lib as L
    a = torch.randn((n, n), device='cuda')
    b = torch.randn((n, n), device='cuda')
    c = torch.empty((n, n), device='cuda')
    for _ in range(2):
        L.call('ntg_gemm_tc', L.stream(), a.data_ptr(), n, b.data_ptr(), n, c.data_ptr(), n, n,
               n, n, 1., 0., 0)
    torch.cuda.synchronize()
    print(json.dumps({'profile_gemm': n, 'c00': float(c[0, 0])}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--profile-tile', type=int, default=0)
    ap.add_argument('--profile-stencil', type=int, default=0)
    ap.add_argument('--profile-fwd-bwd', type=int, default=0)
    ap.add_argument('--profile-gram', type=int, default=0)
    ap.add_argument('--profile-chol', type=int, default=0)
    ap.add_argument('--profile-nll', action='store_true')
    ap.add_argument('--profile-gemm', type=int, default=0)
    ap.add_argument('--profile-predict', type=int, default=0)
    ap.add_argument('--profile-gram-timing', action='store_true',
                    help='time the tensor-core Gram (symmetric and general) and exit')
    ap.add_argument('--profile-vjp', action='store_true',
                    help='time the fused backward (pooled and plain) and exit')
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--no-cpu-baseline', dest='cpu_baseline', action='store_false')
    ap.add_argument('--cpu-seconds', type=float, default=15.0)
    ap.add_argument('--ref-step-seconds', type=float, default=5.0)
    ap.add_argument('--no-full-configs', dest='full_configs', action='store_false',
                    help='skip configurations 1, 3 and 5 at their stated sizes')
    args = ap.parse_args()
    if args.profile_tile:
        profile_tile(args.profile_tile)
    elif args.profile_stencil:
        profile_stencil(args.profile_stencil)
    elif args.profile_fwd_bwd:
        profile_fwd_bwd(args.profile_fwd_bwd)
    elif args.profile_gram:
        profile_gram(args.profile_gram)
    elif args.profile_chol:
        profile_chol(args.profile_chol)
    elif args.profile_nll:
        profile_nll()
    elif args.profile_gemm:
        profile_gemm(args.profile_gemm)
    elif args.profile_predict:
        profile_predict(args.profile_predict)
    elif args.profile_gram_timing:
        import torch
        from nt_gb300 import _ops as O
        print(json.dumps({'gram_tc': gram_roofline(torch, O, torch.device('cuda'))}))
    elif args.profile_vjp:
        import torch
        print(json.dumps({'vjp_roofline': [vjp_roofline(torch, torch.device('cuda'), p)
                                           for p in (True, False)]}))
    elif args.impl == 'reference':
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == '__main__':
    main()
