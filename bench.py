#!/usr/bin/env python3
"""Benchmark: particle-substeps/s of the deterministic Q16.16 PBF substep on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Headline workload (one GPU): the 2D large scene — 1,048,576 fluid particles in
a 1024 x 1024 lattice at 1 wu with seeded +/-0.25 wu jitter, WATER/OIL in
alternating 64-column bands, per-particle temperatures uniform in
[10, 90] degrees, 4 density iterations, chain (H_set || H_slot every substep)
on. One step = one substep of that scene. The working set (~0.5 GB) is far
larger than the 129 MB L2, so no L2 flush is needed between substeps.

Printed: one JSON line with the device-timed value over substeps
[warmup, warmup + steps) (`config.timed_substeps`), the chain at the window's
end against the oracle's record (`parity_ok`), the whole stated run of 1000
substeps (`full_config`, with its own parity), the end-to-end value through
the public API (scene upload from host memory, a digest read back after every
substep, final state read back), the per-phase roofline of the dominant
kernel, the CPU baseline, the batched workload (256 scenes of 1k-64k
particles with stir impulses, also over its full 1000 substeps) against the
same scenes stepped one at a time on the plain path, the 3D dam break (with
its 4096 bonds; also over its full 500 substeps), the serving stream, the
construction site (rigid bodies and containment at scale, with and without
its bodies) and GPU clock samples.

--impl reference times the reference's algorithm on the host cores: the
reference itself is JavaScript + WGSL for WebGPU and cannot run here (no JS
runtime, no WebGPU), so its CPU restatement (oracle/, pinned bit-exact to the
reference's golden chain) is timed instead, with all host threads, on the
same scene and the same substep window as the GPU arm (a 256 x 256 slice when
the window is longer than 60 substeps). The CPU baseline in the GPU arm's
line is the same measurement.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = 'particle-substeps/s'
FULL_SUBSTEPS = 1000    # the stated length of the 2D workloads
FULL_SUBSTEPS_3D = 500  # and of the 3D dam break
UNIT = 'particle-substeps/s'
WORKLOAD = ('2D large scene: 1,048,576 fluid particles (1024x1024 lattice, 1 wu, +/-0.25 wu seeded jitter), '
            'WATER/OIL 64-column bands, temps U[10,90] deg, ITERS 4, H_slot every substep')


def _peaks():
    p = ROOT / 'MEASURED_PEAKS.json'
    if p.exists():
        d = json.loads(p.read_text())
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.device), f'--query-gpu={self.FIELDS}',
                                          '--format=csv,noheader,nounits', '-lms', '100'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ('active', '1', 'yes'):
                    reasons.add(nm)
        if not sm:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unavailable'], 'samples': 0}
        return {'sm_mhz': float(np.median(sm)), 'sm_max_mhz': float(max(smax)), 'reasons': sorted(reasons),
                'samples': len(sm)}


def _dist():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = 'nccl' if torch.cuda.is_available() else 'gloo'
        if backend == 'nccl':
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        return ws, rank, local, dist
    return 1, 0, 0, None


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(dist, x: float, local: int) -> float:
    if dist is None:
        return x
    import torch
    dev = f'cuda:{local}' if dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --- algorithmic bytes per unit (phase-minimal convention) -------------------------
# Per fluid particle, per launch of the phase. Each dependent phase reads the
# fields it needs once and writes its outputs once; neighbour data is served
# on chip and the neighbour list is not counted.
PHASE_NAMES_HEAD = ['predict', 'grid sort', 'cell ranges + gather', 'neighbour lists']
BYTES = {
    'predict': 48,               # R state 32 + stAcc 8; W pred 8
    'grid sort': 20,             # R pred 8; W key 4 + sorted id 4; R key 4
    'cell ranges + gather': 0,
    'neighbour lists': 16,       # R pred 8 + flags 4; W count 4
    'solveA': 20,                # R pred 8 + mat 4; W rho 4 + lam 4
    'colour x4': 88,             # 4 colours: R pred + lam, W dp (56) + apply R dp/pred W pred (32)
    'friction': 8,
    'finalize+xsph+normals+conduct': 140,  # finalize 88 + xsph 32 + normals 20
    'surfaceTension+thermal+digest': 104,  # surfaceTension 32 + conduct/thermal 40 + hash 32
    'fold': 0,
}


# The oracle's recorded chains of the workloads at their full lengths
# (tests/golden/make_config_vectors.py): a run's chain after substep k equals
# the recorded one only if every digest up to k matched.
VECTORS = ROOT / 'tests' / 'golden' / 'config_vectors'


def recorded_chain(workload: str, k: int):
    """The oracle's chain of `workload` after substep k, or None when k is not recorded."""
    p = VECTORS / f'{workload}.json'
    if not p.exists() or k <= 0:
        return None
    d = json.loads(p.read_text())
    chain = d.get('chain')
    if isinstance(chain, list):
        return chain[k - 1] if k <= len(chain) else None
    return None


def parity_against(workload: str, k: int, got: str):
    want = recorded_chain(workload, k)
    return {'checked_at_substep': k, 'ok': (got == want) if want is not None else None,
            'against': f'tests/golden/config_vectors/{workload}.json' if want is not None else 'not recorded'}


# ncu summaries under profiles/ that carry the DRAM traffic of a dominant kernel
PROFILE_OF = {'colour x4': 'k_colour_2d_large.md', 'solve+apply': 'k3_solve_3d_dam.md', 'density': 'kernels_3d_dam.md'}


def profiled_traffic(phase: str):
    """DRAM bytes (read + write) per launch from the committed ncu summary of
    this phase's kernel, or None when there is none."""
    f = PROFILE_OF.get(phase)
    if not f or not (ROOT / 'profiles' / f).exists():
        return None
    for line in (ROOT / 'profiles' / f).read_text().splitlines():
        if line.startswith('traffic_bytes_per_launch:'):
            return int(line.split(':', 1)[1].strip())
    return None


def phase_names(iters: int):
    names = list(PHASE_NAMES_HEAD)
    for _ in range(iters):
        names += ['solveA', 'colour x4', 'friction']
    names += ['finalize+xsph+normals+conduct', 'surfaceTension+thermal+digest', 'fold']
    return names


def run_cpu_baseline(warmup: int, steps: int, threads: int = 0, side: int = 1024):
    """The oracle (CPU restatement of the reference substep) on the same scene
    and the same substep window as the GPU's timed region: `warmup` untimed
    substeps from the load, then `steps` timed ones, all host threads. The
    1 M-particle scene takes about a second per substep on 16 cores, so the
    default window (5 + 20 substeps) is about half a minute of CPU work; past
    60 substeps the window runs on a side x side slice of the scene instead."""
    import oracle
    from sunaengine_gb300 import scenes
    threads = threads or os.cpu_count() or 1
    if warmup + steps > 60:
        side = 256
    sc = scenes.large_two_fluid(side=side)
    e = oracle.OracleEngine(sc.n + 64, threads=threads).load_scene(sc)
    e.step(warmup)
    t0 = time.perf_counter()
    e.step(steps)
    dt = time.perf_counter() - t0
    out = {'value': sc.nFluid * steps / dt, 'unit': UNIT, 'cores': threads, 'kind': 'port',
           'sample': f'{sc.nFluid} fluid particles ({side}x{side} lattice of the same workload), substeps '
                     f'[{warmup}, {warmup + steps}) timed, {dt:.1f} s'}
    # one thread, on a 256 x 256 slice of the scene, the same window
    small = scenes.large_two_fluid(side=256)
    e1 = oracle.OracleEngine(small.n + 64, threads=1).load_scene(small)
    e1.step(warmup)
    t0 = time.perf_counter()
    e1.step(min(steps, 10))
    dt1 = time.perf_counter() - t0
    out['single_thread'] = {'value': small.nFluid * min(steps, 10) / dt1, 'unit': UNIT, 'cores': 1,
                            'sample': f'{small.nFluid} fluid particles (256x256 slice), substeps '
                                      f'[{warmup}, {warmup + min(steps, 10)}), {dt1:.1f} s'}
    return out


def reference_arm(args):
    ws, rank, local, dist = _dist()
    if rank != 0:
        return 0
    cb = run_cpu_baseline(args.warmup, args.steps)
    v = cb['value']
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': UNIT, 'n_gpus': args.gpus,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': None,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'int32', 'data': 'synthetic',
        'config': {'workload': WORKLOAD, 'sample': cb['sample'], 'parallelism': 'cpu',
                   'timed_substeps': [args.warmup, args.warmup + args.steps]},
        'cpu_baseline': cb,
        'e2e': {'value': v, 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
        'note': 'the reference is JS+WGSL for WebGPU (no JS runtime or WebGPU here); its CPU restatement, '
                'pinned bit-exact to the reference golden chain, is timed on the same window of the same scene',
    }
    n = int(cb['sample'].split()[0])
    line['ms_per_step'] = 1e3 * n / v
    print(json.dumps(line), flush=True)
    return 0


# 3D phase bytes per particle (phase-minimal): predict 52, sort 24, neighbour set 16,
# per iteration density 24 + solveDp/applyDp 64, integrate 48 + hash 28.
BYTES_3D = {'predict': 52, 'grid sort': 24, 'cell ranges + gather': 0, 'neighbour lists': 16,
            'density': 24, 'solve+apply': 64, 'integrate+hash': 76, 'fold': 0}
WORKLOAD_3D = ('3D dam break: 262,144 water particles (64^3 lattice at 1 wu, smix jitter) in the corner of a '
               '48x40x48-cell (96x80x96 wu) walled box, 4096 seeded bonds between lattice neighbours, ITERS 4, '
               'H_set||H_slot every substep')


def workload_3d(steps: int, warmup: int, device: int, cpu_seconds: float = 6.0, with_cpu: bool = True):
    """The 3D dam break (262,144 particles, 4 iterations): device-timed
    particle-substeps/s, end to end through the public API, the per-phase
    roofline of its dominant kernel, and the oracle on a sample."""
    from sunaengine_gb300 import tables3d
    from sunaengine_gb300.engine3d import Engine3D
    sc = tables3d.dam3d_large()
    rows = tables3d.bond_rows(sc, tables3d.dam3d_bonds(sc))
    e = Engine3D(max_particles=sc.n, iters=4, device=device).load_scene(sc)
    e.write_bonds(rows, tables3d.DAM3D_BOND_K, tables3d.DAM3D_BOND_BRK)
    e.step(warmup)
    e.sync()
    e.step(steps)
    e.sync()
    ms, launches = e.last_timing()
    value = sc.n * steps / (ms / 1e3)
    parity = parity_against('dam3d_64cubed', warmup + steps, e.chain_hex())
    names = ['predict', 'grid sort', 'cell ranges + gather', 'neighbour lists']
    names += ['density', 'solve+apply'] * e.iters + ['integrate+hash', 'fold']
    ph = e.profile_substep(max(3, min(steps, 10)))
    agg = {}
    for nm, t in zip(names, ph):
        agg.setdefault(nm, [0.0, 0])
        agg[nm][0] += float(t)
        agg[nm][1] += 1
    dom = max((k for k in agg if k != 'fold'), key=lambda k: agg[k][0])
    per_launch = agg[dom][0] / agg[dom][1]
    bpl = BYTES_3D[dom] * sc.n
    peak, kind = _peaks()
    achieved = bpl / (per_launch / 1e3) / 1e9
    roof = {'kernel': dom, 'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s', 'frac': achieved / peak,
            'peak_source': kind, 'traffic': profiled_traffic(dom),
            'traffic_source': f'profiles/{PROFILE_OF[dom]}' if dom in PROFILE_OF else None,
            'algorithmic_bytes_per_launch': bpl, 'launch_ms': per_launch,
            'phases_ms_per_substep': {k: v[0] for k, v in agg.items()}}
    e.close()
    # the whole stated run (500 substeps), device-timed, chain against the oracle's at the end
    ef = Engine3D(max_particles=sc.n, iters=4, device=device).load_scene(sc)
    ef.write_bonds(rows, tables3d.DAM3D_BOND_K, tables3d.DAM3D_BOND_BRK)
    ef.sync()
    ef.step(FULL_SUBSTEPS_3D)
    ef.sync()
    fms, _ = ef.last_timing()
    full = {'substeps': FULL_SUBSTEPS_3D, 'value': sc.n * FULL_SUBSTEPS_3D / (fms / 1e3), 'unit': UNIT,
            'ms_per_step': fms / FULL_SUBSTEPS_3D,
            'parity': parity_against('dam3d_64cubed', FULL_SUBSTEPS_3D, ef.chain_hex())}
    ef.close()
    # end to end: upload the scene, step(1) + digest() per substep, read the state back
    e2 = Engine3D(max_particles=sc.n, iters=4, device=device).load_scene(sc)
    e2.step(1)
    outbuf = e2.read_state()  # the caller's state buffer, allocated (and its pages touched) once
    e2.sync()
    t0 = time.perf_counter()
    e2.load_scene(sc)
    e2.write_bonds(rows, tables3d.DAM3D_BOND_K, tables3d.DAM3D_BOND_BRK)
    t1 = time.perf_counter()
    for _ in range(steps):
        e2.step(1)
        e2.digest()
    t2 = time.perf_counter()
    final = e2.read_state(out=outbuf)
    wall = time.perf_counter() - t0
    parts3 = {'load_ms': 1e3 * (t1 - t0), 'steps_ms': 1e3 * (t2 - t1), 'read_state_ms': 1e3 * (t0 + wall - t2)}
    e2.close()
    out = {'workload': WORKLOAD_3D, 'particles': sc.n, 'steps': steps, 'value': value, 'unit': UNIT,
           'ms_per_step': ms / steps, 'gpu_launches': int(launches), 'roofline': roof, 'parity': parity,
           'full_config': full,
           'e2e': {'value': sc.n * steps / wall, 'unit': UNIT, 'h2d_bytes_per_step': (sc.n * 28 + rows.nbytes) / steps,
                   'd2h_bytes_per_step': 32 + final.nbytes / steps, 'parts': parts3}}
    if with_cpu:
        import oracle
        threads = os.cpu_count() or 1
        small = tables3d.column_fast(32, 32, 32, 48, 40, 48)
        o = oracle.Oracle3D(small.n, iters=4, threads=threads).load_scene(small)
        # the same bond density: 512 seeded lattice bonds in the 32^3 block
        o.write_bonds(tables3d.bond_rows(small, tables3d.lattice_bonds(32, 32, 32, 512, tables3d.DAM3D_BOND_SEED)),
                      tables3d.DAM3D_BOND_K, tables3d.DAM3D_BOND_BRK)
        o.step(1)
        t0 = time.perf_counter()
        k = 0
        while time.perf_counter() - t0 < cpu_seconds:
            o.step(1)
            k += 1
        dt = time.perf_counter() - t0
        out['cpu_baseline'] = {'value': small.n * k / dt, 'unit': UNIT, 'cores': threads, 'kind': 'port',
                               'sample': f'{small.n}-particle 32^3 block of the same box with 512 lattice bonds, '
                                         f'{k} substeps, {dt:.1f} s'}
    return out


def serving_workload(device: int, count: int = 40, rate_hz: float = 4.0, budget_gb: float = 24.0,
                     seed: int = 0x5e7e):
    """A seeded Poisson stream of replay and rewind-scrub jobs (2D and 3D, 4k-256k
    particles, N in [100, 2000]) served with continuous batching in real time."""
    from sunaengine_gb300 import serving
    jobs = serving.poisson_jobs(count, rate_hz, seed=seed)
    s = serving.Server(int(budget_gb * (1 << 30)), device=device)
    stats = s.run(jobs, realtime=True)
    s.close()
    stats.update({'rate_hz': rate_hz, 'hbm_budget_gb': budget_gb, 'quantum_substeps': s.quantum,
                  'checkpoint_every': s.ckpt_every})
    return stats


def batched_workload(steps: int, warmup: int, device: int, plain_sample: int = 24, seed: int = 0xba7c4,
                     full_run: bool = True):
    """256 scenes (1k-64k particles, log-uniform) with stir schedules: batched
    vs the same scenes stepped one at a time on the plain path."""
    from sunaengine_gb300 import scenes
    from sunaengine_gb300.engine import Batch, Engine
    scs, sched = scenes.batch_scenes(count=256, seed=seed, substeps=warmup + steps)
    total = sum(s.n for s in scs)
    nf = sum(s.nFluid for s in scs)
    def make():
        bb = Batch(max_particles=total + 16, max_scenes=len(scs), max_cells=1 << 22, device=device)
        for sid, (s, ev) in enumerate(zip(scs, sched)):
            assert bb.add_scene(s) == sid
            for (at, cx, cy, r, ix, iy) in ev:
                bb.schedule_impulse(sid, at, cx, cy, r, ix, iy)
        return bb
    # layout, then lanes, tuned on a separate run advanced to the middle of the
    # timed window
    t = make()
    t.step(warmup + steps // 2)
    layout = t.autotune_layout(1)
    t.autotune(2)
    pick = t.lanes()
    t.destroy()

    def with_layout(x):
        if layout['layout']:
            x.set_staged(True).set_tile_shape(layout['layout'])
        return x

    b = with_layout(make())
    b.set_lanes(pick)
    b.step(warmup)
    b.sync()
    b.step(steps)
    ms, launches = b.last_timing()
    b.check_errors()
    batched = nf * steps / (ms / 1e3)
    lanes_b = b.lanes()
    # the same window with the solver iterations as one persistent kernel per
    # substep (sn_batch_set_persistent), for comparison with the graph of
    # per-phase launches
    bp = with_layout(make())
    bp.set_lanes(lanes_b)
    bp.set_persistent(True)
    bp.step(warmup)
    bp.sync()
    bp.step(steps)
    pms, plaunch = bp.last_timing()
    bp.check_errors()
    same = all(bp.chain_hex(i) == b.chain_hex(i) for i in range(len(scs)))
    bp.destroy()
    persistent = {'value': nf * steps / (pms / 1e3), 'ms_per_step': pms / steps,
                  'gpu_launches_per_step': plaunch // max(1, steps), 'vs_graph': (nf * steps / (pms / 1e3)) / batched,
                  'chains_equal_to_graph': same}
    # parity: advance (untimed) to the next substep the oracle's sample recorded
    # and compare those scenes' chains
    parity = {'ok': None, 'against': 'not recorded'}
    vp = VECTORS / 'batch_256.json'
    if vp.exists() and seed == 0xba7c4:
        vec = json.loads(vp.read_text())
        every = vec['every']
        at = -(-(warmup + steps) // every) * every
        if at <= vec['substeps']:
            scs_full, sched_full = scenes.batch_scenes(count=256, seed=seed, substeps=at)
            # the schedules drawn for `at` substeps extend the ones loaded (a prefix)
            for sid, ev in enumerate(sched_full):
                for (t_at, cx, cy, r, ix, iy) in ev:
                    if t_at >= warmup + steps:
                        b.schedule_impulse(sid, t_at, cx, cy, r, ix, iy)
            b.step(at - (warmup + steps))
            bad = [sid for sid, rec in vec['scenes'].items()
                   if str(at) in rec['chain'] and b.chain_hex(int(sid)) != rec['chain'][str(at)]]
            parity = {'checked_at_substep': at, 'ok': not bad, 'scenes_checked': len(vec['scenes']),
                      'mismatched': bad, 'against': 'tests/golden/config_vectors/batch_256.json'}
    # where a batched substep's time goes: CUDA events between the phases over
    # three substeps after the parity check (the stir impulses run before the
    # first phase and are not in it)
    phases = {}
    for nm, t_ in zip(phase_names(4), b.profile_substep(3)):
        phases[nm] = phases.get(nm, 0.0) + float(t_)
    b.destroy()
    # the whole stated run: FULL_SUBSTEPS substeps of every scene with its
    # full stir schedule, device-timed in chunks of 100 substeps, the sampled
    # scenes' chains checked against the oracle's record after every chunk
    full = None
    if full_run:
        scs_f, sched_f = scenes.batch_scenes(count=256, seed=seed, substeps=FULL_SUBSTEPS)
        bf = Batch(max_particles=total + 16, max_scenes=len(scs_f), max_cells=1 << 22, device=device)
        for sid, (s_, ev) in enumerate(zip(scs_f, sched_f)):
            assert bf.add_scene(s_) == sid
            for (at, cx, cy, r, ix, iy) in ev:
                bf.schedule_impulse(sid, at, cx, cy, r, ix, iy)
        with_layout(bf).set_lanes(lanes_b)
        vec = json.loads(vp.read_text()) if vp.exists() and seed == 0xba7c4 else None
        fms, bad, checked = 0.0, [], 0
        for k in range(100, FULL_SUBSTEPS + 1, 100):
            bf.step(100)
            bf.sync()
            fms += bf.last_timing()[0]
            if vec is not None:
                for sid, rec in vec['scenes'].items():
                    want = rec['chain'].get(str(k))
                    if want is not None:
                        checked += 1
                        if bf.chain_hex(int(sid)) != want:
                            bad.append((int(sid), k))
        bf.check_errors()
        bf.destroy()
        full = {'substeps': FULL_SUBSTEPS, 'value': nf * FULL_SUBSTEPS / (fms / 1e3), 'unit': UNIT,
                'ms_per_step': fms / FULL_SUBSTEPS,
                'parity': {'ok': (not bad) if vec is not None else None, 'chains_checked': checked,
                           'mismatched': bad[:8],
                           'against': 'tests/golden/config_vectors/batch_256.json' if vec is not None
                           else 'not recorded'}}
    # plain path on a sample of the same scenes, one engine per scene, sequentially
    rng = np.random.Generator(np.random.PCG64(seed ^ 0x5a5a))
    pick = rng.choice(len(scs), size=min(plain_sample, len(scs)), replace=False)
    pn, pms = 0, 0.0
    for k in pick:
        s = scs[int(k)]
        e = Engine(max_particles=s.n + 16, max_cells=1 << 20, device=device).load_scene(s)
        e.step(warmup)
        e.autotune(1)
        e.sync()
        e.step(steps)
        t, _ = e.last_timing()
        pn += s.nFluid * steps
        pms += t
        e.destroy()
    plain = pn / (pms / 1e3)
    return {'scenes': len(scs), 'particles': int(nf), 'value': batched, 'unit': UNIT,
            'ms_per_step': ms / steps, 'gpu_launches_per_step': launches // max(1, steps),
            'plain_same_scenes': plain, 'plain_sample_scenes': int(len(pick)), 'lanes': lanes_b,
            'batched_vs_plain': batched / plain, 'parity': parity, 'full_config': full,
            'persistent_loop': persistent, 'phases_ms_per_substep': phases, 'layout_tuning': layout}


def construction_workload(steps: int, warmup: int, device: int, with_cpu: bool = True, cpu_seconds: float = 4.0):
    """The widened rows at scale: 24 bays of a METAL plank (free rigid body), a
    WOOD disc (axis body) and a held STONE rail (containment) over one WATER
    pool, 74,384 particles, 48 bodies, ITERS 4, chain on. The same scene
    without bodies (the planks and discs loose) shows what the three rigid
    passes cost."""
    from sunaengine_gb300 import scenes
    from sunaengine_gb300.engine import Engine
    sc = scenes.construction_site()
    out = {'workload': 'construction site: 24 bays of a METAL plank (free body, 63 members), a WOOD disc '
                       '(axis body, 81 members) and a held STONE rail over a 44-row WATER pool; '
                       f'{sc.n} particles, 48 bodies, ITERS 4, H_set||H_slot every substep',
           'particles': sc.n, 'steps': steps, 'unit': UNIT}
    for label, bodies in (('with_bodies', True), ('without_bodies', False)):
        e = Engine(max_particles=sc.n, device=device).load_scene(sc)
        if bodies:
            for pl, wh, pv in zip(sc.meta['planks'], sc.meta['wheels'], sc.meta['wheel_pivots']):
                e.make_rigid_body(pl)
                e.make_axis_body(wh, *pv)
        e.step(warmup)
        e.sync()
        e.step(steps)
        e.sync()
        ms, launches = e.last_timing()
        e.check_errors()
        out[label] = {'value': sc.n * steps / (ms / 1e3), 'ms_per_step': ms / steps,
                      'gpu_launches_per_step': launches / steps}
        if bodies:
            out['bodies_live'] = int((e.read_bodies()[:, 0] == 1).sum())
            out['chain'] = e.chain_hex()
            out['parity'] = parity_against('construction_site', warmup + steps, e.chain_hex())
        e.destroy()
    out['rigid_share'] = 1.0 - out['without_bodies']['ms_per_step'] / out['with_bodies']['ms_per_step']
    if with_cpu:
        import oracle
        small = scenes.construction_site(tiles=2)
        o = oracle.OracleEngine(small.n, threads=os.cpu_count() or 1).load_scene(small)
        for pl, wh, pv in zip(small.meta['planks'], small.meta['wheels'], small.meta['wheel_pivots']):
            o.make_rigid_body(pl)
            o.make_axis_body(wh, *pv)
        o.step(2)
        k, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < cpu_seconds:
            o.step(5)
            k += 5
        dt = time.perf_counter() - t0
        out['cpu_baseline'] = {'value': small.n * k / dt, 'unit': UNIT, 'cores': os.cpu_count() or 1, 'kind': 'port',
                               'sample': f'the same bays, 2 of 24 ({small.n} particles, 4 bodies), {k} substeps, '
                                         f'{dt:.1f} s'}
    return out


def sections_only(args):
    """--no-2d: the 3D / batched / serving sections alone (a profiling aid; the
    line carries no headline value)."""
    ws, rank, local, dist = _dist()
    line = {'metric': METRIC, 'value': None, 'unit': UNIT, 'n_gpus': ws, 'steps': args.steps,
            'warmup': args.warmup, 'note': 'headline section skipped (--no-2d)'}
    if rank == 0 and not args.no_batched:
        line['batched'] = batched_workload(args.steps, args.warmup, local, full_run=not args.no_full)
    if rank == 0 and not args.no_3d:
        line['cfg3_3d'] = workload_3d(args.steps, args.warmup, local, with_cpu=not args.no_cpu)
    if rank == 0 and not args.no_serving:
        line['serving'] = serving_workload(local)
    if rank == 0 and not args.no_construction:
        line['construction'] = construction_workload(args.steps, args.warmup, local, with_cpu=not args.no_cpu)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def ours(args):
    if args.no_2d:
        return sections_only(args)
    ws, rank, local, dist = _dist()
    from sunaengine_gb300 import scenes
    from sunaengine_gb300.engine import Engine
    sc = scenes.large_two_fluid(side=1024)
    tuned_at = None
    lanes_pick = None
    layout = {'layout': 2 if args.staged else 0, 'tuned': False}
    if not args.no_autotune:
        # The layout (list gathers, or staged gathers and their tile shape)
        # and then the lane split per gather class are tuned on a separate run
        # of the same scene, advanced to the middle of the timed window: the
        # lattice the scene starts from settles within a few hundred substeps
        # and the best choice changes with it (untimed; the measured engines
        # only receive the result). --staged pins the staged layout.
        tuned_at = args.warmup + args.steps // 2
        t = Engine(max_particles=sc.n, max_cells=1 << 20, device=local).set_staged(args.staged).load_scene(sc)
        t.step(tuned_at)
        if not args.staged:
            layout = dict(t.autotune_layout(2), tuned=True)
        t.autotune(3)
        lanes_pick = t.lanes()
        t.destroy()

    def with_layout(x):
        if layout['layout']:
            x.set_staged(True).set_tile_shape(layout['layout'])
        return x

    e = with_layout(Engine(max_particles=sc.n, max_cells=1 << 20, device=local))
    e.load_scene(sc)
    if lanes_pick is not None:
        e.set_lanes(lanes_pick)
    e.step(args.warmup)
    e.sync()
    _barrier(dist)
    with ClockSampler(local) as clk:
        e.sync()
        _barrier(dist)
        t0 = time.perf_counter()
        e.step(args.steps)
        e.sync()
        wall = time.perf_counter() - t0
        _barrier(dist)
    dev_ms, launches = e.last_timing()
    lanes_used = e.lanes()
    e.check_errors()
    parity = parity_against('two_fluid_1024', args.warmup + args.steps, e.chain_hex())
    dev_ms = _max_over_ranks(dist, dev_ms, local)
    ms_step = dev_ms / args.steps
    value = ws * sc.nFluid * args.steps / (dev_ms / 1e3)

    # per-phase device times (CUDA events on the engine's stream) over real substeps
    names = phase_names(e.iters)
    reps = max(3, min(args.steps, 10))
    ph = e.profile_substep(reps)
    agg = {}
    for nm, t in zip(names, ph):
        agg.setdefault(nm, [0.0, 0])
        agg[nm][0] += float(t)
        agg[nm][1] += 1
    dom = max((k for k in agg if k != 'fold'), key=lambda k: agg[k][0])
    launches_of = {'colour x4': 4}
    nl = launches_of.get(dom, 1)
    per_launch_ms = agg[dom][0] / (agg[dom][1] * nl)
    units = sc.nFluid // nl
    bytes_per_launch = BYTES[dom] * sc.nFluid / nl
    achieved = bytes_per_launch / (per_launch_ms / 1e3) / 1e9
    peak, peak_kind = _peaks()
    roof = {'kernel': dom, 'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
            'frac': achieved / peak, 'peak_source': peak_kind, 'traffic': profiled_traffic(dom),
            'traffic_source': f'profiles/{PROFILE_OF[dom]}' if dom in PROFILE_OF else None,
            'algorithmic_bytes_per_launch': bytes_per_launch, 'units_per_launch': units,
            'launch_ms': per_launch_ms,
            'phases_ms_per_substep': {k: v[0] for k, v in agg.items()}}

    # end to end through the public API: upload from host, H_slot read back every
    # substep, final state read back
    e2 = with_layout(Engine(max_particles=sc.n, max_cells=1 << 20, device=local))
    if lanes_pick is not None:
        e2.set_lanes(lanes_pick)
    e2.load_scene(sc)
    e2.step(1)
    outbuf = e2.read_state()  # the caller's state buffer, allocated (and its pages touched) once
    e2.sync()
    _barrier(dist)
    t0 = time.perf_counter()
    e2.load_scene(sc)
    t1 = time.perf_counter()
    for _ in range(args.steps):
        e2.step(1)
        e2.digest()
    t2 = time.perf_counter()
    final = e2.read_state(out=outbuf)
    e2wall = time.perf_counter() - t0
    e2parts = {'load_ms': 1e3 * (t1 - t0), 'steps_ms': 1e3 * (t2 - t1), 'read_state_ms': 1e3 * (t0 + e2wall - t2)}
    e2wall = _max_over_ranks(dist, e2wall, local)
    scene_bytes = sc.n * (8 + 8 + 4 + 4)
    e2e = {'value': ws * sc.nFluid * args.steps / e2wall, 'unit': UNIT,
           'h2d_bytes_per_step': scene_bytes / args.steps,
           'd2h_bytes_per_step': 32 + final.nbytes / args.steps,
           'how': 'loadScene from host arrays, then per substep step(1) + digest() readback, then readState into '
                  'the caller\'s state buffer',
           'parts': e2parts}
    e2.destroy()
    e.destroy()

    # The whole stated run: all FULL_SUBSTEPS substeps of the workload from its
    # load, device-timed, and its chain against the oracle's at the last one.
    full = None
    if not args.no_full:
        e3 = with_layout(Engine(max_particles=sc.n, max_cells=1 << 20, device=local))
        if lanes_pick is not None:
            e3.set_lanes(lanes_pick)
        e3.load_scene(sc)
        e3.sync()
        e3.step(FULL_SUBSTEPS)
        e3.sync()
        fms, _ = e3.last_timing()
        e3.check_errors()
        full = {'substeps': FULL_SUBSTEPS, 'value': sc.nFluid * FULL_SUBSTEPS / (fms / 1e3), 'unit': UNIT,
                'ms_per_step': fms / FULL_SUBSTEPS,
                'parity': parity_against('two_fluid_1024', FULL_SUBSTEPS, e3.chain_hex())}
        # where the settled substep's time goes: the per-phase profile of the
        # three substeps after the run (the compressed column, crowded edge cell)
        late = {}
        for nm, t in zip(phase_names(e3.iters), e3.profile_substep(3)):
            late[nm] = late.get(nm, 0.0) + float(t)
        full['phases_ms_per_substep_after'] = late
        e3.destroy()

    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': ws, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': ms_step, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'int32', 'data': 'synthetic',
        'config': {'workload': WORKLOAD, 'particles': sc.n, 'fluid_particles': sc.nFluid,
                   'parallelism': 'replicas' if ws > 1 else 'single', 'l2': 'working set > L2, no flush',
                   'lanes': lanes_used, 'lanes_tuned_at_substep': tuned_at,
                   'timed_substeps': [args.warmup, args.warmup + args.steps],
                   'gathers': (f"tile-staged (shared memory, bulk copies), tiles of {1 << layout['layout']} cells"
                               if layout['layout'] else 'neighbour-list (global)'),
                   'layout_tuning': layout},
        'parity_ok': parity['ok'],
        'parity': parity,
        'full_config': full,
        'wall_ms_per_step': 1e3 * wall / args.steps,
        'gpu_launches': int(launches),
        'roofline': roof,
        'e2e': e2e,
        'clocks': clk.summary(),
    }
    if rank == 0 and not args.no_batched:
        line['batched'] = batched_workload(args.steps, args.warmup, local, full_run=not args.no_full)
    if rank == 0 and not args.no_3d:
        line['cfg3_3d'] = workload_3d(args.steps, args.warmup, local, with_cpu=not args.no_cpu)
    if rank == 0 and not args.no_serving:
        line['serving'] = serving_workload(local)
    if rank == 0 and not args.no_construction:
        line['construction'] = construction_workload(args.steps, args.warmup, local, with_cpu=not args.no_cpu)
    if rank == 0 and not args.no_cpu:
        line['cpu_baseline'] = run_cpu_baseline(args.warmup, args.steps)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=300)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--no-batched', action='store_true')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-3d', action='store_true')
    ap.add_argument('--no-2d', action='store_true', help='skip the headline 2D section (profiling runs)')
    ap.add_argument('--no-autotune', action='store_true',
                    help='keep the rule-based lanes (profiling runs: a tuner under ncu sees serialised timings)')
    ap.add_argument('--no-serving', action='store_true')
    ap.add_argument('--no-construction', action='store_true')
    ap.add_argument('--no-full', action='store_true', help='skip the full 1000-substep run of the headline workload')
    ap.add_argument('--staged', action='store_true',
                    help='headline engines use the tile-staged gathers (sn_set_staged) instead of the list gathers')
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == 'reference':
        return reference_arm(args)
    return ours(args)


if __name__ == '__main__':
    sys.exit(main())
