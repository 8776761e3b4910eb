#!/usr/bin/env python
"""Benchmark: agent-steps/s of the plain FP64 per-step update.

Workload (default): 300 m x 300 m field, 600 random wall segments, 100,000
ThreeCircle agents at ~1.1 agents/m^2, cell 3.6 m; one step = the standard
node tree (orientation, adjusting, agent-agent, agent-wall, adaptive
velocity Verlet, reset) -- one MultiAgentSimulation.update().  Synthetic,
seeded inputs (no dataset exists for this path).

Arms:
  ours       device path through the C ABI.  `value`: state resident in HBM,
             each timed step one CUDA-graph launch bracketed by CUDA events on
             the library stream, L2 flushed (256 MiB write) between steps.
             `e2e`: same steps through the C ABI with pinned host records
             copied in and out every step, wall clock.
  reference  the reference algorithm's CPU implementation on the host cores:
             the C restatement of the reference's numba path (the reference
             itself is Python + numba, with nothing compiled to run here),
             agent-parallel over all host threads.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank advances its own replica of the workload (no data
exchange between ranks); rank 0 prints one JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'agent-steps/s at 100k agents on 1 GB300: plain vs batched; adjoint/forward cost'
UNIT = 'agent-steps/s'

# Algorithmic float64 operations per unit of work (add, sub, mul, div, sqrt,
# compare = 1; an elementary function counts the float64 operations of its
# cd_math.h implementation: hypot 4, exp 31).  Units: unordered candidate
# pair (bound check), near pair (distance), interacting pair (h < 3: social
# force, both sides), contact pair (h < 0: contact, both sides), near wall
# (distance), wall contact, agent (adjusting, timestep, Verlet, shoulders).
# Float64 operations of the reference's step per unit of work, on the
# branches it takes (add, sub, mul, div, sqrt, compare = 1; exp = 31, hypot
# = 4, the operation counts of the shared elementary functions): `inter` the
# interacting-pair gate, accumulation, torques and relative speed; `soc` the
# nine sub-pair discriminants of the ThreeCircle social force (Circular: in
# `inter`); `soc_def` per defined time-to-collision root; `soc_valid` the
# gradient, two magnitudes, two forces and truncations of a pair with a valid
# time-to-collision.  A candidate rejected by the distance bound is charged
# the bound check only.
WEIGHTS = {
    'three_circle': dict(cand=6, near=104, inter=19, soc=155, soc_def=3, soc_valid=120,
                         contact=48, wall_near=81, wall_contact=30, agent=64),
    'circular': dict(cand=6, near=11, inter=28, soc=0, soc_def=4, soc_valid=112, contact=48,
                     wall_near=27, wall_contact=24, agent=30),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', default='ours', choices=('ours', 'reference'))
    ap.add_argument('--agents', type=int, default=100_000)
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-batched', action='store_true')
    ap.add_argument('--no-adjoint', action='store_true')
    ap.add_argument('--no-navigation', action='store_true')
    ap.add_argument('--no-noise', action='store_true')
    ap.add_argument('--no-save', action='store_true')
    ap.add_argument('--no-states', action='store_true')
    ap.add_argument('--detail', default=os.path.join('gpurun_out', 'bench_detail.json'),
                    help='file for the per-leg detail the JSON line leaves out')
    ap.add_argument('--profile-range', default=None,
                    choices=('step', 'records', 'adjoint', 'states'),
                    help='bracket one instance of that work with cudaProfilerStart/Stop '
                         '(for ncu --profile-from-start off); no work is skipped')
    return ap.parse_args()


class ProfileRange:
    """cudaProfilerStart/Stop around a block when `on` (one capture range
    for ncu --profile-from-start off), synchronised on both sides."""

    def __init__(self, on):
        self.on = bool(on)

    def __enter__(self):
        if self.on:
            import torch
            torch.cuda.synchronize()
            torch.cuda.profiler.start()
        return self

    def __exit__(self, *exc):
        if self.on:
            import torch
            torch.cuda.synchronize()
            torch.cuda.profiler.stop()


def dist_env():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return ws, rank, local


def max_over_ranks(x, dist=None, device='cuda'):
    """The largest `x` over all ranks (the slowest replica's time); `x` itself
    without a process group."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world_size, agents, steps, seconds):
    """agent-steps/s of all replicas together, timed by the slowest."""
    return world_size * agents * steps / seconds


def workload(n_agents):
    from crowddynamics_gb300 import scenarios as S
    if n_agents == 100_000:
        return S.large_field()
    size = 300.0 * (n_agents / 100_000) ** 0.5
    return S.large_field(n=n_agents, size=size, n_walls=max(1, int(600 * n_agents / 100_000)))


def config_of(scen, nodes_desc):
    return {'workload': 'large_field_threecircle_100k' if len(scen.agents) == 100_000 else scen.name,
            'agents': len(scen.agents), 'walls': len(scen.walls), 'body': scen.body,
            'domain_m': [scen.bounds[2] - scen.bounds[0], scen.bounds[3] - scen.bounds[1]],
            'cell_size_m': scen.cell_size, 'grid': list(scen.grid[3:]),
            'nodes': nodes_desc, 'dt_min': scen.dt_min, 'dt_max': scen.dt_max,
            'l2': 'flushed (256 MiB write) between timed steps',
            'parallelism': 'replicas (one independent workload per GPU)'}


class Clocks:
    """nvidia-smi sampler running during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.Q,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        out = {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': [], 'samples': 0}
        if not self.path or not os.path.exists(self.path):
            return out
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(',')]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return out
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[k] for _, _, r in rows for k in range(4)
                          if r[k].lower() in ('active', '1', 'yes')})
        return {'sm_mhz': statistics.median(r[0] for r in rows), 'sm_max_mhz': max(r[1] for r in rows),
                'reasons': reasons, 'samples': len(rows)}


def algorithmic_flops(scen, counts):
    """Algorithmic float64 operations of one step of the reference algorithm
    on this state (pair columns count each unordered pair twice)."""
    w = WEIGHTS[scen.body]
    tot = counts.sum(axis=0)
    return (w['cand'] * tot[0] / 2 + pair_flops(scen, counts) + w['wall_near'] * tot[4] +
            w['wall_contact'] * tot[5] + w['agent'] * len(scen.agents))


# The float64 results the state depends on, per unit: the distance of the
# minimum sub-pair only (`near`), each defined time-to-collision root
# (`soc_def`: its b, c, discriminant, root and tau), and for a pair with a
# valid time to collision also its normal, moment arms and torques; the other
# sub-pairs' distances and discriminants only select or rule out branches.
WEIGHTS_REQUIRED = {
    'three_circle': dict(near=9, inter=19, soc=0, soc_def=20, soc_valid=140, contact=48),
    'circular': dict(near=11, inter=28, soc=0, soc_def=4, soc_valid=112, contact=48),
}


def pair_flops_required(scen, counts):
    w = WEIGHTS_REQUIRED[scen.body]
    tot = counts.sum(axis=0)
    return (w['near'] * tot[1] / 2 + w['inter'] * tot[2] / 2 + w['contact'] * tot[3] / 2 +
            w['soc'] * tot[6] + w['soc_def'] * tot[7] + w['soc_valid'] * tot[8])


def algorithmic_flops_required(scen, counts):
    """The float64 work of one step the state depends on: the pair kernel's
    required work, walls and the per-agent terms (candidates rejected by the
    distance bound cost float32 only)."""
    w = WEIGHTS[scen.body]
    tot = counts.sum(axis=0)
    return (pair_flops_required(scen, counts) + w['wall_near'] * tot[4] +
            w['wall_contact'] * tot[5] + w['agent'] * len(scen.agents))


def pair_flops(scen, counts):
    """The part of algorithmic_flops done by the pair kernel: every unordered
    pair that passes the bound check, once (distance, social force, contact).
    Columns 1-3 count each pair twice, the social-branch columns 6-8 once."""
    w = WEIGHTS[scen.body]
    tot = counts.sum(axis=0)
    return (w['near'] * tot[1] / 2 + w['inter'] * tot[2] / 2 + w['contact'] * tot[3] / 2 +
            w['soc'] * tot[6] + w['soc_def'] * tot[7] + w['soc_valid'] * tot[8])


def cpu_sample(scen, nodes_orc, steps, nthreads):
    """Time `steps` oracle steps of the workload with `nthreads` threads."""
    from oracle import oracle as O
    a = scen.agents.copy()
    grid = O.make_grid(*scen.grid)
    O.step(a, grid, scen.walls, flags=nodes_orc, dt_min=scen.dt_min, dt_max=scen.dt_max,
           nthreads=nthreads)                      # warm-up
    t0 = time.perf_counter()
    for _ in range(steps):
        O.step(a, grid, scen.walls, flags=nodes_orc, dt_min=scen.dt_min, dt_max=scen.dt_max,
               nthreads=nthreads)
    return time.perf_counter() - t0


ORC_NODES = 2 | 4 | 8 | 16 | 32 | 64    # orientation .. reset, no fluctuation


def run_reference(args, ws, rank):
    if rank != 0:
        return
    from oracle import build as ob
    ob.build()
    scen = workload(args.agents)
    nthreads = os.cpu_count() or 1
    from oracle import oracle as O
    a = scen.agents.copy()
    grid = O.make_grid(*scen.grid)
    for _ in range(args.warmup):
        O.step(a, grid, scen.walls, flags=ORC_NODES, dt_min=scen.dt_min, dt_max=scen.dt_max,
               nthreads=nthreads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.step(a, grid, scen.walls, flags=ORC_NODES, dt_min=scen.dt_min, dt_max=scen.dt_max,
               nthreads=nthreads)
    el = time.perf_counter() - t0
    value = len(scen.agents) * args.steps / el
    sample = ('%d full steps of the %d-agent workload, C restatement of the reference '
              'algorithm, agent-parallel OpenMP' % (args.steps, len(scen.agents)))
    line = {'metric': METRIC, 'value': value, 'unit': UNIT, 'impl': 'reference',
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': el / args.steps * 1e3, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic (seeded)',
            'config': config_of(scen, 'orientation+adjusting+agent_agent+agent_obstacle+integrate+reset'),
            'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': nthreads, 'kind': 'port',
                             'sample': sample, 'numba': numba_probe()},
            'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import numpy as np
    import torch
    dist = None
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    torch.cuda.set_device(local)
    from crowddynamics_gb300 import build as B
    B.build()
    from crowddynamics_gb300 import _native as N
    from crowddynamics_gb300.engine import batch_from_scenarios

    scen = workload(args.agents)
    n = len(scen.agents)
    nodes = N.NODE_ALL & ~N.NODE_FLUCTUATION
    b, agents, _ = batch_from_scenarios([scen])
    counts0 = b.pair_counts()
    peak_gflops = N.measure_fp64_peak()

    flush = torch.empty(256 << 20, dtype=torch.uint8, device='cuda')

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    # `value`: events around each step's graph launch only (no event node
    # inside the step graph, whose kernels then stay chained to each other)
    b.set_timing(True, kernels=False)
    b.run(max(args.warmup, 3), nodes)          # warm-up (graph capture happens here)
    b.synchronize()
    barrier()
    b.set_timing(True, kernels=False)
    with Clocks(local) as clk:
        for k in range(args.steps):
            flush.fill_(k & 0xff)
            torch.cuda.synchronize()
            with ProfileRange(args.profile_range == 'step' and k == args.steps - 1):
                b.run(1, nodes)
    barrier()
    run_ms = max_over_ranks(b.kernel_time()['run_ms'], dist)
    value = whole_job_rate(ws, n, args.steps, run_ms / 1e3)
    # the kernels' own times: the same steps again with CUDA events inside the
    # step graph around the force stage, the float32 pair pass and k_pairs
    b.set_timing(True, kernels=True)
    b.run(2, nodes)
    b.synchronize()
    b.set_timing(True, kernels=True)
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        torch.cuda.synchronize()
        b.run(1, nodes)
    kt = b.kernel_time()
    b.set_timing(False)
    force_ms = kt['force_ms'] / max(kt['force_launches'], 1)
    pair_ms = kt['pair_ms'] / max(kt['pair_launches'], 1) if kt['pair_launches'] else None
    light_ms = kt['light_ms'] / max(kt['pair_launches'], 1) if kt['pair_launches'] else None
    pairs_ms = kt['pairs_ms'] / max(kt['pair_launches'], 1) if kt['pair_launches'] else None
    stepk_ms = kt['run_ms'] / max(kt['run_steps'], 1)
    split = b.pair_split() if pair_ms else None     # the last timed step's flat list
    counts1 = b.pair_counts()
    flops = 0.5 * (algorithmic_flops(scen, counts0) + algorithmic_flops(scen, counts1))
    flops_req = 0.5 * (algorithmic_flops_required(scen, counts0) +
                       algorithmic_flops_required(scen, counts1))
    pflops = 0.5 * (pair_flops(scen, counts0) + pair_flops(scen, counts1))
    rflops = 0.5 * (pair_flops_required(scen, counts0) + pair_flops_required(scen, counts1))
    stage_achieved = flops_req / (force_ms / 1e3) / 1e12
    stage_effective = flops / (force_ms / 1e3) / 1e12
    peak = peak_gflops / 1e3
    # the pair pipeline: its pair stage (the float32 pass k_pairs_light, then
    # k_pairs) dominates the step, and k_pairs the stage
    if pair_ms:
        kernel, kernel_ms, kflops, kreq = 'k_pairs', pair_ms, pflops, rflops
        label = 'k_pairs'
    else:
        kernel, kernel_ms, kflops, kreq = 'k_forces', force_ms, flops, flops_req
        label = kernel
    effective = kflops / (kernel_ms / 1e3) / 1e12

    # end to end through the C ABI with pinned host records
    host = torch.empty(n * agents.dtype.itemsize, dtype=torch.uint8, pin_memory=True)
    rec = host.numpy().view(agents.dtype)
    b.download(rec)
    # host wall clock: three timed passes of `steps` steps, the median kept
    # (a single pass can catch an unrelated host stall)
    trials = []
    for trial in range(3):
        barrier()
        t0 = time.perf_counter()
        for k in range(args.steps):
            with ProfileRange(args.profile_range == 'records' and trial == 2 and
                              k == args.steps - 1):
                # upload, one graph step and download in one call (the host
                # waits once, for the download, which checks the step status)
                b.step_records(rec, 1, nodes)
        e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
        trials.append(whole_job_rate(ws, n, args.steps, e2e_s))
    e2e = sorted(trials)[1]

    # DRAM bytes, executed float64 flops (DADD + DMUL + 2 DFMA thread
    # instructions) and FP64 pipe activity of the dominant kernels per step,
    # from the committed summary of one ncu capture of this workload
    traffic = pipe = executed = None
    stage = None
    tpath = os.path.join(ROOT, 'profiles', 'pair_stage_field100k_threecircle.json')
    if n == 100_000 and scen.body == 'three_circle' and kernel == 'k_pairs' and \
            os.path.exists(tpath):
        prof = json.load(open(tpath))
        traffic = prof['dram_bytes_by_kernel']['k_pairs']
        pipe = prof['fp64_pipe_active_by_kernel']['k_pairs']
        executed = prof['fp64_flops_by_kernel']['k_pairs']
        stage = {'kernels': 'k_pairs_light + k_pairs', 'ms': pair_ms, 'light_ms': light_ms,
                 'flops': prof['fp64_flops_per_step'], 'traffic': prof['dram_bytes_per_step'],
                 'fp64_pipe_active_ncu': prof['fp64_pipe_active'],
                 'frac': prof['fp64_flops_per_step'] / (pair_ms / 1e3) / 1e12 / (peak_gflops / 1e3)}
        kernel_ms = pairs_ms
    # achieved: the float64 work the kernel executes (the float32 certificates
    # decide the rest exactly); without a capture of this workload, the model
    # count of the float64 results the state depends on over the whole stage
    work = executed if executed else kreq
    achieved = work / (kernel_ms / 1e3) / 1e12

    # the HBM side of the roofline: the state read and written once per step
    # and the cell list (ThreeCircle: 29 float64 read, 13 written with the
    # shoulders; Circular: 19 and 6; cell list 24 B), against the measured copy
    # bandwidth
    hbm_peak = None
    ppath = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(ppath):
        hbm_peak = json.load(open(ppath)).get('hbm_gbs')
    bytes_agent = (29 + 13) * 8 + 24 if scen.body == 'three_circle' else (19 + 6) * 8 + 24
    hbm_gbs = value * bytes_agent / 1e9

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    # The JSON line stays short (the driver keeps its tail): headline, roofline,
    # baselines, then the batched and adjoint parts of the metric last; the
    # per-leg detail goes to args.detail.
    detail = {'e2e_trials': trials,
              'e2e_timing': 'host wall clock around cd_step_records per step: upload of the '
                            'pinned records, one graph step and download, enqueued together '
                            '(the call waits for the download and checks the step status); '
                            'median of 3 passes',
              'roofline_work': 'achieved counts the float64 operations whose results the state '
                               'depends on (branch-exact for the state); reference_algorithm '
                               'counts every float64 operation the reference executes on it '
                               '(an effective rate: float32 decides most of them exactly)',
              'force_stage_kernels': 'k_nl_count, near scans (one launch), k_nl_fill, '
                                     'k_pairs_light, k_pairs, k_forces_gather, k_forces_fallback '
                                     '(exits at once unless the near lists overflowed)'}
    line = {'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': ws, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': run_ms / args.steps, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic (seeded)',
            'config': config_of(scen, 'orientation+adjusting+agent_agent+agent_obstacle+integrate+reset'),
            'e2e': {'value': e2e, 'unit': UNIT,
                    'h2d_bytes_per_step': n * agents.dtype.itemsize,
                    'd2h_bytes_per_step': n * agents.dtype.itemsize},
            'gpu_launches': b.kernels_per_step(nodes) * args.steps,
            'roofline': {'bound': 'fp64', 'achieved': achieved, 'peak': peak, 'unit': 'TFLOP/s',
                         'frac': achieved / peak, 'traffic': traffic,
                         'kernel': label, 'kernel_ms': kernel_ms, 'flops_per_launch': work,
                         'work': 'float64 flops executed per step (ncu DADD+DMUL+2*DFMA)'
                                 if executed else 'model count of float64 results',
                         'peak_source': 'measured live (FP64 FMA chain, 2 flops per FMA)',
                         'fp64_pipe_active_ncu': pipe, 'pair_stage': stage,
                         'model_flops_per_stage': kreq,
                         'reference_algorithm_frac': effective / peak,
                         'hbm_frac': hbm_gbs / hbm_peak if hbm_peak else None,
                         'force_stage_ms': force_ms, 'force_stage_frac': stage_achieved / peak,
                         'step_ms_with_kernel_events': stepk_ms},
            'clocks': clk.summary()}
    detail['roofline'] = {'pair_split': split,
                          'hbm': {'bytes_per_agent_step': bytes_agent, 'achieved_gbs': hbm_gbs,
                                  'peak_gbs': hbm_peak,
                                  'peak_source': 'MEASURED_PEAKS.json hbm_gbs (copy)'},
                          'reference_algorithm': {'flops_per_launch': kflops,
                                                  'achieved': effective},
                          'force_stage': {'ms': force_ms, 'flops_per_step': flops_req,
                                          'achieved': stage_achieved,
                                          'reference_algorithm_flops_per_step': flops,
                                          'reference_algorithm_achieved': stage_effective}}
    if ws == 1 and not args.no_cpu_baseline:
        line['cpu_baseline'], detail['cpu_baseline'] = cpu_baseline(scen, n)
    legs = {}
    if not args.no_navigation:
        d = run_navigation(args.steps)
        detail['navigation'] = d
        legs['navigation_device_over_host'] = d['device_navigation'] / d['host_navigation']
    if not args.no_noise:
        d = run_noise(b, agents, scen, args.steps)
        detail['fluctuation'] = d
        legs['device_noise'] = d['device_noise']
    if not args.no_save:
        d = run_save(max(args.steps, 20))
        detail['save'] = d
        legs['async_save_over_host_save'] = d['async_save'] / d['host_save']
    if not args.no_states:
        detail['states'] = run_states(max(args.steps, 10), profile=args.profile_range == 'states')
    if legs:
        line['legs'] = legs
    if not args.no_batched:
        line['batched'], detail['batched'] = run_batched(args.steps, args.warmup, flush)
    if not args.no_adjoint:
        line['adjoint'], detail['adjoint'] = run_adjoint(profile=args.profile_range == 'adjoint')
    if args.detail:
        try:
            os.makedirs(os.path.dirname(os.path.abspath(args.detail)), exist_ok=True)
            with open(args.detail, 'w') as f:
                json.dump(detail, f, indent=1)
        except OSError:
            pass
    print(json.dumps(line, separators=(',', ':')), flush=True)
    b.close()
    if dist is not None:
        dist.destroy_process_group()


def numba_probe():
    """Whether the reference's own numba path could be timed here.  It needs
    numba and the reference's source files, which are not shipped with this
    repository; the C port (bit-identical to the device in exact-math mode)
    is timed instead."""
    try:
        import numba  # noqa: F401
        return 'numba imports, but the reference source is not on this box'
    except Exception as e:                        # noqa: BLE001
        return 'unavailable on this box (import numba: %s)' % type(e).__name__


def cpu_baseline(scen, n):
    """The oracle's agent-parallel C port on all host cores (20 steps after
    one warm-up step) and on one core (3 steps): the reference's algorithm
    on the host, a baseline reported beside the device number."""
    nthreads = os.cpu_count() or 1
    steps, steps1 = 20, 3
    el = cpu_sample(scen, ORC_NODES, steps, nthreads)
    el1 = cpu_sample(scen, ORC_NODES, steps1, 1)
    probe = numba_probe()
    line = {'value': n * steps / el, 'unit': UNIT, 'cores': nthreads, 'kind': 'port',
            'sample': '%d steps of the %d-agent workload, OpenMP x %d' % (steps, n, nthreads),
            'single_thread': n * steps1 / el1, 'numba': probe}
    detail = dict(line, sample_single_thread='%d steps on one thread' % steps1,
                  what='C restatement of the reference algorithm (oracle/cd_oracle.c), '
                       'bit-identical to the device in exact-math mode')
    return line, detail


def run_save(steps, n=2000, size=30.0):
    """SaveSimulationData every update on the ThreeCircle room (2000 agents,
    632 kB of records per frame), dumping every 10 frames: the standard tree
    with device noise and no saving, with the node (asynchronous snapshots
    and a writer thread), and with the reference's way (the host array
    downloaded after every update, then its save_npy / save_csv protocol)."""
    import shutil
    import tempfile
    import numpy as np
    from crowddynamics_gb300 import io as IO
    from crowddynamics_gb300 import scenarios as S
    from crowddynamics_gb300.simulation import logic as L
    from crowddynamics_gb300.simulation.agents import Agents
    from crowddynamics_gb300.simulation.field import Field
    from crowddynamics_gb300.simulation.multiagent import MultiAgentSimulation
    scen = S.room(n=n, size=size, seed=1)
    base = tempfile.mkdtemp(prefix='cdsave')

    def make():
        sim = MultiAgentSimulation(agents=Agents(array=scen.agents.copy()),
                                   field=Field(domain=scen.bounds, obstacles=scen.walls),
                                   device_noise_seed=7, name='room')
        sim.logic = L.Reset(sim) << (L.Integrator(sim, dt_min=0.001, dt_max=0.01) << (
            L.Fluctuation(sim), L.Adjusting(sim) << L.Orientation(sim),
            L.AgentAgentInteractions(sim, max_agent_radius=0.35), L.AgentObstacleInteractions(sim)))
        return sim

    def timed(sim, each=None):
        for _ in range(3):
            sim.update()
            if each:
                each(sim)
        sim.finish_writers()
        sim._batch.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            sim.update()
            if each:
                each(sim)
        sim.finish_writers()
        sim._batch.synchronize()
        return n * steps / (time.perf_counter() - t0)

    out = {'workload': 'room_30x30_threecircle_2000, save every update, dump every 10',
           'unit': UNIT, 'bytes_per_frame': n * scen.agents.dtype.itemsize}
    sim = make()
    out['no_save'] = timed(sim)
    sim.close()
    sim = make()
    node = L.SaveSimulationData(sim, base_directory=base, save_directory='async',
                                save_condition=lambda s: (s.data['iterations'] + 1) % 10 == 0)
    node.add_to_simulation_logic()
    out['async_save'] = timed(sim)
    sim.close()
    sim = make()
    d = os.path.join(base, 'sync')
    os.makedirs(d)
    npy, rows = IO.save_npy(d, 'agents'), IO.save_csv(d, 'data')
    npy.send(None)
    rows.send(None)

    def host_save(s):
        save = s.data['iterations'] % 10 == 0
        npy.send(s.agents.array)
        npy.send(save)
        rows.send(dict(s.data))
        rows.send(save)
    out['host_save'] = timed(sim, host_save)
    sim.close()
    shutil.rmtree(base, ignore_errors=True)
    out['timing'] = 'wall clock around `steps` updates, writers drained before and after'
    return out


def run_states(steps, n=2000, size=30.0, profile=False):
    """The state nodes between steps on the ThreeCircle room (2000 agents,
    5 walls plus 3 interior walls): LeaderFollowerWithHerding (10% leaders,
    70% followers, 5 nearest within 10 m), InsideDomain and TargetReached;
    agent-updates/s of each call (CUDA-synchronised wall clock)."""
    import numpy as np
    from crowddynamics_gb300 import scenarios as S
    from crowddynamics_gb300.engine import DeviceBatch, walls_as_rows
    rng = np.random.default_rng(3)
    scen = S.room(n=n, size=size, seed=1)
    walls = np.concatenate([scen.walls, S.walls_array([((8.0, 5.0), (8.0, 20.0)),
                                                       ((15.0, 25.0), (25.0, 15.0)),
                                                       ((2.0, 12.0), (12.0, 12.5))])])
    a = scen.agents
    a['velocity'] = rng.normal(0, 1, (n, 2))
    a['is_leader'] = rng.uniform(size=n) < 0.1
    a['is_follower'] = ~a['is_leader'] & (rng.uniform(size=n) < 0.7)
    a['target'] = np.where(a['is_leader'], 0, -1)
    b = DeviceBatch('three_circle', [dict(n_agents=n, n_walls=len(walls), grid=scen.grid)])
    b.upload(a)
    b.set_walls(walls)
    domain = np.array([[0, 0], [size, 0], [size, size], [0, size], [0, 0]], float)
    exit_ = [np.array([[size - 1, size / 2 - 1], [size, size / 2 - 1], [size, size / 2 + 1],
                       [size - 1, size / 2 + 1]], float)]
    out = {'workload': 'room_30x30_threecircle_2000, 8 walls', 'unit': 'agent-updates/s'}
    for name, fn in (('leader_follower_with_herding', lambda: b.herding(True)),
                     ('leader_follower', lambda: b.herding(False, sight_follower=1.0)),
                     ('inside_domain', lambda: b.inside_domain(0, domain)),
                     ('target_reached', lambda: b.target_reached(0, exit_))):
        with ProfileRange(profile):
            fn()
        b.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        b.synchronize()
        out[name] = n * steps / (time.perf_counter() - t0)
    b.close()
    out['timing'] = 'wall clock around `steps` calls, each synchronised (they return host values)'
    return out


def run_noise(b, agents, scen, steps):
    """The full step including Fluctuation on the 100k field: noise drawn on
    the device inside the step graph, against noise drawn on the host with
    numpy/scipy (as the reference does) and copied in before each step."""
    from crowddynamics_gb300 import _native as N
    from crowddynamics_gb300 import scenarios as S
    import numpy as np
    n = len(agents)
    b.upload(agents)
    b.set_noise_mode(True, 2024, 0)
    b.run(3, N.NODE_ALL)
    b.synchronize()
    b.set_timing(True)
    b.run(steps, N.NODE_ALL)
    dev = n * steps / (b.kernel_time()['run_ms'] / 1e3)
    b.set_timing(False)
    b.set_noise_mode(False)
    rng = np.random.default_rng(5)
    host_steps = max(3, steps // 4)
    t0 = time.perf_counter()
    for _ in range(host_steps):
        b.set_noise(*S.draw_noise(scen.agents, rng))
        b.step(N.NODE_ALL)
    b.synchronize()
    host = n * host_steps / (time.perf_counter() - t0)
    return {'device_noise': dev, 'host_noise': host, 'unit': UNIT,
            'workload': 'large_field_threecircle_100k, standard tree with Fluctuation',
            'timing': 'device: CUDA events around graph launches; host: wall clock around '
                      'numpy/scipy draw, cd_set_noise and cd_step'}


def run_batched(steps, warmup, flush=None):
    """Batched form: the 512-scenario mix held in two contexts (one per body
    type, each with its autotuned force-stage variant) and advanced by one
    graph launch per step for both (cd_group_*), then one device
    synchronisation; against the same scenarios as 512 single-scenario
    contexts (the plain step run scenario by scenario): every scenario's step
    graph launched back to back with one device synchronisation per step (the
    fair baseline), and each scenario's step awaited before the next
    (cd_synchronize per scenario, as a caller stepping one simulation after
    another does).  The detail adds the two contexts launched separately and
    the group with 10 steps per launch.  The same number of steps in every
    leg, L2 flushed before each step (per launch for the 10-step group).
    Returns (the line's part, the detail)."""
    import torch
    from crowddynamics_gb300 import _native as N
    from crowddynamics_gb300 import autotune
    from crowddynamics_gb300 import scenarios as S
    from crowddynamics_gb300.engine import DeviceGroup, batch_from_scenarios
    nodes = N.NODE_ALL & ~N.NODE_FLUCTUATION
    mix = S.batch_mix()
    groups = [[s for s in mix if s.body == b] for b in ('circular', 'three_circle')]

    def timed(ctxs, per_scenario_sync=False):
        for c in ctxs:
            c.run(max(warmup, 3), nodes)
        torch.cuda.synchronize()
        el = 0.0
        for k in range(steps):
            if flush is not None:
                flush.fill_(k & 0xff)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for c in ctxs:
                c.launch(1, nodes)
                if per_scenario_sync:
                    c.synchronize()
            torch.cuda.synchronize()
            el += time.perf_counter() - t0
        for c in ctxs:
            c.synchronize()                      # status of every context checked
        return el

    batches, tuned = [], {}
    for g in groups:
        b, agents, _ = batch_from_scenarios(g)
        v, times = autotune.tune(b, agents)
        tuned[b.body] = {'variant': v, 'shape': N.variants()[v],
                         'ms_per_variant': None if times is None else
                         {str(k): round(t, 4) for k, t in times.items()}}
        batches.append(b)
    n_total = sum(b.n_agents for b in batches)

    def timed_group(per_launch):
        grp = DeviceGroup(batches, nodes, steps_per_launch=per_launch)
        grp.launch(max(1, warmup // per_launch))
        grp.synchronize()
        el = 0.0
        for k in range(steps // per_launch):
            if flush is not None:
                flush.fill_(k & 0xff)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            grp.launch(1)
            torch.cuda.synchronize()
            el += time.perf_counter() - t0
        grp.synchronize()
        grp.close()
        return n_total * (steps // per_launch) * per_launch / el

    batched = timed_group(1)
    group10 = timed_group(10) if steps >= 10 else None
    two_launches = n_total * steps / timed(batches)
    for b in batches:
        b.close()
    singles = [batch_from_scenarios([s])[0] for s in mix]
    back_to_back = n_total * steps / timed(singles)
    synchronised = n_total * steps / timed(singles, per_scenario_sync=True)
    for b in singles:
        b.close()
    line = {'value': batched, 'scenario_by_scenario': back_to_back,
            'speedup': batched / back_to_back, 'speedup_vs_synchronised': batched / synchronised,
            'steps': steps, 'scenarios': len(mix), 'agents': n_total}
    detail = dict(line, unit=UNIT, scenario_by_scenario_synchronised=synchronised,
                  two_contexts_launched_separately=two_launches, group_10_steps_per_launch=group10,
                  walls=sum(len(s.walls) for s in mix), autotune=tuned,
                  timing='host wall clock per step from the first launch to the device '
                         'synchronisation, L2 flushed (256 MiB write) before each step')
    return line, detail


def run_adjoint(n=5000, width=80.0, height=20.0, steps=400, ckpt=20, seed=4, fd_steps=10,
                profile=False):
    """Differentiable form: Circular hallway 80 m x 20 m, 5000 agents,
    400-step rollout, loss = mean squared position error against a rollout
    with hidden tau_adj ~ U(0.3, 0.7) and target speed ~ N(1.2, 0.2); the
    gradient of the loss with respect to per-agent tau_adj, target speed,
    tau_0 and k_soc through the hand-written adjoint, checkpoint every 20
    steps.  Times (CUDA events inside the call) the forward rollout alone and
    the forward + adjoint.  Central differences (h = 1e-6 relative to each
    parameter, 1e-7 where the first straddles a force cut-off) are taken on
    the same 5000 agents over the first ``fd_steps`` steps: over 400 steps the
    dynamics' sensitivity grows by many orders of magnitude (reported as the
    gradient's largest entry against the horizon) and no difference quotient
    resolves the derivative."""
    import numpy as np
    from crowddynamics_gb300 import scenarios as S
    from crowddynamics_gb300.adjoint import PARAMS, make_target
    from crowddynamics_gb300.engine import batch_from_scenarios
    scen = S.hallway(n=n, width=width, height=height, seed=seed)
    rng = np.random.default_rng(seed)
    hidden = {'tau_adj': rng.uniform(0.3, 0.7, n), 'target_velocity': rng.normal(1.2, 0.2, n)}
    target = make_target(scen, hidden, steps)
    a = scen.agents.copy()
    b, _, _ = batch_from_scenarios([scen])

    def rollout(agents, grads, t=steps):
        b.upload(agents)
        return b.rollout_loss(t, target[:t], ckpt, grads=grads)

    rollout(a, True)                                    # warm-up (graph capture, allocation)
    if profile:
        with ProfileRange(True):
            rollout(a, True, ckpt)                      # one checkpoint segment
    fwd_only = []
    full = []
    for _ in range(3):
        fwd_only.append(rollout(a, False)[2])
        loss, g, fms, ams = rollout(a, True)
        full.append((fms, ams))
    f_only = float(np.median(fwd_only))
    f_ms = float(np.median([x[0] for x in full]))
    a_ms = float(np.median([x[1] for x in full]))

    # central differences over the first fd_steps steps
    _, g_s, _, _ = rollout(a, True, fd_steps)
    base = np.stack([np.ascontiguousarray(a[k]) for k in PARAMS], 1)

    def check(direction):
        ad = float((g_s * direction).sum())
        out = {'adjoint': ad}
        for h in (1e-6, 1e-7):
            lo, hi = a.copy(), a.copy()
            for col, name in enumerate(PARAMS):
                hi[name] = a[name] + h * direction[:, col]
                lo[name] = a[name] - h * direction[:, col]
            fd = (rollout(hi, False, fd_steps)[0] - rollout(lo, False, fd_steps)[0]) / (2 * h)
            out[str(h)] = {'central_difference': fd, 'rel_diff': abs(ad - fd) / abs(fd)}
            if out[str(h)]['rel_diff'] <= 1e-5:
                break
        return out

    checks = {'random_direction': check(rng.normal(size=base.shape) * np.abs(base))}
    for col, name in enumerate(PARAMS):
        i = int(np.argmax(np.abs(g_s[:, col])))
        e = np.zeros_like(base)
        e[i, col] = abs(base[i, col])
        checks['%s[%d]' % (name, i)] = check(e)
    worst = max(min(v['rel_diff'] for k, v in c.items() if k != 'adjoint')
                for c in checks.values())
    growth = {}
    for t in (10, 50, 100, 200):
        growth[str(t)] = float(np.abs(rollout(a, True, t)[1]).max())
    growth[str(steps)] = float(np.abs(g).max())
    b.close()
    line = {'adjoint_over_forward': a_ms / f_only, 'gradient_over_forward': (f_ms + a_ms) / f_only,
            'forward_ms': f_only, 'adjoint_ms': a_ms, 'worst_rel_diff': worst,
            'fd_steps': fd_steps, 'steps': steps, 'checkpoint_every': ckpt}
    return line, {'workload': 'hallway_80x20_circular_5000_rollout400_ckpt20', 'loss': loss,
            'forward_only_ms': f_only, 'forward_ms': f_ms, 'adjoint_ms': a_ms,
            'adjoint_over_forward': a_ms / f_only,
            'gradient_over_forward': (f_ms + a_ms) / f_only,
            'agent_steps_per_s_forward': n * steps / (f_only / 1e3),
            'central_differences': {'steps': fd_steps, 'agents': n, 'checks': checks,
                                    'worst_rel_diff': worst},
            'max_abs_gradient_by_horizon': growth,
            'timing': 'CUDA events around the rollout and the adjoint inside cd_rollout_loss, '
                      'median of 3 calls after one warm-up call; adjoint_ms includes the '
                      'recomputation of each 20-step segment'}


def run_navigation(steps, n=2000, size=30.0):
    """Navigation on the device: the ThreeCircle room (30 m x 30 m, one 1.2 m
    exit, 2000 agents) steering by the exit direction map on a 0.05 m grid,
    every agent with target 0.  Agent-steps/s of the standard step without
    navigation, with CD_NODE_NAVIGATION in the same graph, and with the lookup
    done on the host between device steps (download, lookup, upload: the round
    trip the device node removes)."""
    import numpy as np
    import torch
    from crowddynamics_gb300 import _native as N
    from crowddynamics_gb300 import scenarios as S
    from crowddynamics_gb300.engine import batch_from_scenarios
    scen = S.room(n=n, size=size, seed=1)
    scen.agents['target'] = 0
    e0, e1 = size / 2 - 0.6, size / 2 + 0.6
    mx, my, step = S.room_exit_direction_map(size, size, e0, e1, step=0.05)
    b, agents, _ = batch_from_scenarios([scen])
    b.set_direction_maps(0, mx, my, 0.0, 0.0, step)
    base = N.NODE_ALL & ~N.NODE_FLUCTUATION
    out = {'workload': 'room_30x30_threecircle_2000_exit_map_0.05m', 'map_cells': int(mx.size)}

    def timed(nodes):
        b.upload(agents)
        b.run(3, nodes)
        b.synchronize()
        b.set_timing(True)
        b.run(steps, nodes)
        kt = b.kernel_time()
        b.set_timing(False)
        return n * steps / (kt['run_ms'] / 1e3)

    out['without_navigation'] = timed(base)
    out['device_navigation'] = timed(base | N.NODE_NAVIGATION)
    # host lookup between steps: pinned records down, lookup, up, step
    host = torch.empty(n * agents.dtype.itemsize, dtype=torch.uint8, pin_memory=True)
    rec = host.numpy().view(agents.dtype)
    rec[:] = agents
    b.upload(rec)
    b.run(3, base)
    b.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        b.download(rec)
        rec['target_direction'] = S.lookup_direction(rec['position'], (mx, my), step,
                                                     defaults=rec['target_direction'])
        b.upload(rec)
        b.run(1, base)
    out['host_navigation'] = n * steps / (time.perf_counter() - t0)
    out['unit'] = UNIT
    out['timing'] = ('device: CUDA events around `steps` graph launches; host: wall clock '
                     'around download, numpy lookup, upload and one graph launch per step')
    b.close()
    return out


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == 'reference':
        run_reference(args, ws, rank)
    else:
        run_ours(args, ws, rank, local)


if __name__ == '__main__':
    main()
