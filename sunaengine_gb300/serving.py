"""Serving loop: replay and rewind-scrub jobs with continuous batching.

No counterpart in the reference (its pages run one scene at a time). A job is
a seeded initial scene plus its input schedule (2D: stir impulses at substep
indices; 3D: a stir amplitude with the page's per-frame phase), asking either
to advance N substeps ("advance") or to play to N and then rewind to substep
k < N ("scrub"). Jobs arrive over time; the server

  * admits a job when its slots fit the 2D or 3D engine's free slot ranges and
    its checkpoints fit the remaining checkpoint-pool budget (the HBM budget is
    split between the two engines' slot arrays and the pool at start);
  * runs every admitted job of a dimension in ONE engine: all of its scenes
    advance together, one launch sequence per substep, and jobs join and leave
    between quanta (continuous batching); the 2D and 3D engines run on their
    own CUDA streams, so their work overlaps on the device;
  * keeps on-device checkpoints every `ckpt_every` substeps of each job (and
    at substep 0) and serves a scrub by loading the checkpoint at or below k
    and advancing the remainder;
  * reports per-job latency (arrival to result) and aggregate throughput.

Every job's result (its H_set || H_slot digest and chain at the end) is the
same whether it runs alone or in any mix: scenes share no state, impulses are
keyed to each scene's own substep clock, 3D stir phases are per frame, and a
checkpoint load restores a scene exactly.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import scenes, tables3d
from .checkpoints import CheckpointPool
from .engine import Batch, EngineError
from .engine3d import Engine3D

# Device bytes per slot, from the engines' allocations (the arrays sized by
# max_particles): 2D state 32, stAcc 8, predSlot 8, sceneOf/keys/inv 12, bond
# and bond candidates 384, sorted keys/ids 8, PL/PL2/RX/NQ 64, POS 8, SCN 4,
# DP 8, HEAT/CORR 8, neighbour lists 196, sort scratch 8 + histogram;
# 3D state 32, sceneOf 4, PRS 16, keys 12, PW/PW2/PL 48, neighbour lists 196,
# sort scratch 8.
BYTES_PER_SLOT_2D = 768
BYTES_PER_SLOT_3D = 320


@dataclass
class Job:
    jid: int
    dim: int               # 2 or 3
    op: str                # 'advance' or 'scrub'
    n: int                 # requested particle count
    target: int            # N: substeps to advance
    scrub_to: int          # k: where a scrub ends (op == 'scrub')
    seed: int
    arrival: float = 0.0   # seconds after the stream starts
    # filled by the server
    digest: Optional[str] = None
    chain: Optional[str] = None
    t_admit: Optional[float] = None
    t_done: Optional[float] = None
    substeps_run: int = 0
    particles: int = 0

    @property
    def latency_ms(self) -> float:
        return 1e3 * (self.t_done - self.arrival)


def job_scene_2d(job: Job):
    """The job's seeded 2D scene and its stir schedule over `target` substeps."""
    rng = np.random.Generator(np.random.PCG64(job.seed))
    aspect = float(rng.uniform(0.5, 2.0))
    sc = scenes.jittered_block(job.n, aspect, rng)
    return sc, scenes.stir_schedule(sc, job.target, rng)


def job_scene_3d(job: Job):
    """The job's seeded 3D scene (a jittered column, the page's smix jitter) and
    its stir amplitude."""
    rng = np.random.Generator(np.random.PCG64(job.seed))
    side = max(4, round(job.n ** (1.0 / 3.0)))
    by = max(4, int(round(job.n / (side * side))))
    gx = min(52, max(8, math.ceil((side + 3) * 1.6 / 2)))
    gz = gx
    gy = min(52, max(8, math.ceil((by + 3) / 2) + 4))
    sc = tables3d.column_fast(side, min(by, 2 * gy - 4), side, gx, gy, gz)
    return sc, int(rng.integers(0, 1500))


def scenes_cells_2d(sc) -> int:
    """Grid cells a 2D scene takes (4 wu cells over its domain)."""
    cs = 1 << int(sc.cellShift)
    return (-(-int(sc.domW) // cs)) * (-(-int(sc.domH) // cs))


def poisson_jobs(count: int, rate_hz: float, seed: int = 0x5e7e, n_lo: int = 4096, n_hi: int = 262144,
                 t_lo: int = 100, t_hi: int = 2000, p_scrub: float = 0.4, p3d: float = 0.3) -> List[Job]:
    """A seeded request stream: Poisson arrivals at `rate_hz`, particle counts
    log-uniform in [n_lo, n_hi], N uniform in [t_lo, t_hi], scrubs to a uniform
    k below N."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    jobs = []
    for j in range(count):
        t += float(rng.exponential(1.0 / rate_hz)) if rate_hz > 0 else 0.0
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        target = int(rng.integers(t_lo, t_hi + 1))
        op = 'scrub' if rng.random() < p_scrub else 'advance'
        k = int(rng.integers(0, target)) if op == 'scrub' else target
        dim = 3 if rng.random() < p3d else 2
        jobs.append(Job(jid=j, dim=dim, op=op, n=n, target=target, scrub_to=k,
                        seed=int(rng.integers(1, 2 ** 31)), arrival=t))
    return jobs


@dataclass
class _Run:
    job: Job
    scene: int
    substep: int = 0
    phase: str = 'play'                  # 'play' to target, then 'rewind' to scrub_to
    ckpts: Dict[int, int] = field(default_factory=dict)
    ckpt_bytes: int = 0
    reserved: int = 0
    cells: int = 0


class Server:
    """`engines` = (batch2d, engine3d, pool) replaces the device objects (the
    CPU tests drive the scheduling with stand-ins that keep the same calls)."""

    MAX_CELLS_2D = 1 << 22
    MAX_CELLS_3D = 1 << 23

    def __init__(self, hbm_budget_bytes: int, device: int = 0, quantum: int = 25, ckpt_every: int = 100,
                 max_scenes: int = 64, iters: int = 4, iters3: int = 4, split=(0.45, 0.25, 0.30), engines=None):
        self.quantum = int(quantum)
        self.ckpt_every = int(ckpt_every)
        b2, b3, bp = (int(hbm_budget_bytes * f) for f in split)
        self.slots2 = max(8192, b2 // BYTES_PER_SLOT_2D)
        self.slots3 = max(8192, b3 // BYTES_PER_SLOT_3D)
        self.pool_bytes = max(1 << 20, bp)
        if engines is None:
            self.b2 = Batch(max_particles=self.slots2, max_scenes=max_scenes, max_cells=self.MAX_CELLS_2D,
                            iters=iters, device=device)
            self.e3 = Engine3D(max_particles=self.slots3, max_scenes=max_scenes, max_cells=self.MAX_CELLS_3D,
                               iters=iters3, device=device)
            self.pool = CheckpointPool(self.pool_bytes, device)
        else:
            self.b2, self.e3, self.pool = engines
        self.reserved = 0
        self.cells = {2: 0, 3: 0}
        self.active: Dict[int, _Run] = {}
        self._scene_cache: Dict[int, tuple] = {}

    def close(self):
        for r in list(self.active.values()):
            self._release(r)
        self.pool.close()
        self.b2.destroy()
        self.e3.close()

    # ---- admission -------------------------------------------------------
    def _engine(self, dim):
        return self.b2 if dim == 2 else self.e3

    def _scene_of(self, job: Job):
        if job.jid not in self._scene_cache:
            self._scene_cache[job.jid] = job_scene_2d(job) if job.dim == 2 else job_scene_3d(job)
        return self._scene_cache[job.jid]

    def try_admit(self, job: Job, now: float) -> bool:
        """Admit `job` if its slots, grid cells and checkpoints fit the budget."""
        sc, inputs = self._scene_of(job)
        if job.dim == 2:
            cells = scenes_cells_2d(sc)
            if self.cells[2] + cells > self.MAX_CELLS_2D:
                return False
            try:
                sid = self.b2.add_scene(sc, capacity=sc.n)
            except EngineError:
                return False
            for (at, cx, cy, r, ix, iy) in inputs:
                self.b2.schedule_impulse(sid, at, cx, cy, r, ix, iy)
            job.particles = int(sc.nFluid)
        else:
            cells = sc.gx * sc.gy * sc.gz
            if self.cells[3] + cells > self.MAX_CELLS_3D:
                return False
            try:
                sid = self.e3.add_scene(sc, cap=sc.n, stir_amp=inputs, frame=2)
            except EngineError:
                return False
            job.particles = int(sc.n)
        eng = self._engine(job.dim)
        per_r = (eng.ckpt_bytes(sid) + 255) // 256 * 256
        need = per_r * (job.target // self.ckpt_every + 1)
        if self.reserved + need > self.pool_bytes:
            eng.remove_scene(sid)
            return False
        run = _Run(job=job, scene=sid, ckpt_bytes=per_r, reserved=need)
        run.cells = cells
        self.reserved += need
        self.cells[job.dim] += cells
        run.ckpts[0] = eng.ckpt_save(sid, self.pool)
        job.t_admit = now
        self.active[job.jid] = run
        self._scene_cache.pop(job.jid, None)
        return True

    def _release(self, r: _Run):
        for h in r.ckpts.values():
            self.pool.free(h)
        r.ckpts.clear()
        self.reserved -= r.reserved
        self.cells[r.job.dim] -= r.cells
        self._engine(r.job.dim).remove_scene(r.scene)
        self.active.pop(r.job.jid, None)

    # ---- stepping --------------------------------------------------------
    def _next_stop(self, r: _Run) -> int:
        j = r.job
        if r.phase == 'play':
            nxt = (r.substep // self.ckpt_every + 1) * self.ckpt_every
            return min(nxt, j.target)
        return j.scrub_to

    def _finish(self, r: _Run, now: float):
        eng = self._engine(r.job.dim)
        r.job.digest = eng.digest(r.scene).hex
        r.job.chain = eng.chain_hex(r.scene)
        r.job.t_done = now
        self._release(r)

    def _after_quantum(self, r: _Run, now_fn):
        j = r.job
        eng = self._engine(j.dim)
        if r.phase == 'play':
            if r.substep % self.ckpt_every == 0 and r.substep not in r.ckpts and r.substep < j.target:
                r.ckpts[r.substep] = eng.ckpt_save(r.scene, self.pool)
            if r.substep == j.target:
                if j.op == 'advance' or j.scrub_to == j.target:
                    self._finish(r, now_fn())
                    return
                base = (j.scrub_to // self.ckpt_every) * self.ckpt_every
                eng.ckpt_load(r.scene, self.pool, r.ckpts[base])
                r.substep = base
                r.phase = 'rewind'
                if base == j.scrub_to:
                    self._finish(r, now_fn())
        elif r.substep == j.scrub_to:
            self._finish(r, now_fn())

    def step_quantum(self, now_fn) -> int:
        """Advance every active scene by one quantum (bounded by each job's next
        stop); returns the substeps stepped (0 when idle)."""
        qs = {2: None, 3: None}
        for r in self.active.values():
            q = min(self.quantum, self._next_stop(r) - r.substep)
            d = r.job.dim
            qs[d] = q if qs[d] is None else min(qs[d], q)
        if qs[2] is None and qs[3] is None:
            return 0
        # both engines are queued before either is waited on: their streams overlap
        if qs[2]:
            self.b2.step(qs[2])
        if qs[3]:
            self.e3.step(qs[3])
        if qs[2]:
            self.b2.sync()
        if qs[3]:
            self.e3.sync()
        for r in list(self.active.values()):
            q = qs[r.job.dim]
            r.substep += q
            r.job.substeps_run += q
        for r in list(self.active.values()):
            self._after_quantum(r, now_fn)
        return max(q for q in qs.values() if q)

    def run(self, jobs: List[Job], realtime: bool = True) -> dict:
        """Serve `jobs` (sorted by arrival). With realtime=False every job counts
        as arrived at once, so only the budget limits the mix."""
        pending = deque(sorted(jobs, key=lambda j: (j.arrival, j.jid)))
        waiting: deque = deque()
        t0 = time.perf_counter()
        now_fn = (lambda: time.perf_counter() - t0)
        while pending or waiting or self.active:
            now = now_fn()
            while pending and (not realtime or pending[0].arrival <= now):
                waiting.append(pending.popleft())
            while waiting and self.try_admit(waiting[0], now_fn()):
                waiting.popleft()
            if not self.active:
                if waiting:
                    raise EngineError(f'job {waiting[0].jid} does not fit an empty server (budget too small)')
                if pending and realtime:
                    time.sleep(max(0.0, pending[0].arrival - now_fn()))
                continue
            self.step_quantum(now_fn)
        wall = now_fn()
        return summarize(jobs, wall)


def summarize(jobs: List[Job], wall_s: float) -> dict:
    lat = np.array([j.latency_ms for j in jobs if j.t_done is not None])
    ps = sum(j.particles * j.substeps_run for j in jobs)
    return {
        'jobs': len(jobs), 'done': int(lat.size),
        'p50_ms': float(np.percentile(lat, 50)) if lat.size else None,
        'p99_ms': float(np.percentile(lat, 99)) if lat.size else None,
        'particle_substeps': int(ps),
        'value': ps / wall_s if wall_s > 0 else None, 'unit': 'particle-substeps/s',
        'wall_s': wall_s,
        'jobs_2d': sum(1 for j in jobs if j.dim == 2), 'jobs_3d': sum(1 for j in jobs if j.dim == 3),
        'scrubs': sum(1 for j in jobs if j.op == 'scrub'),
    }


def run_alone(job: Job, hbm_budget_bytes: int, device: int = 0, **kw) -> Job:
    """The same job on an otherwise empty server."""
    j = Job(jid=job.jid, dim=job.dim, op=job.op, n=job.n, target=job.target, scrub_to=job.scrub_to,
            seed=job.seed, arrival=0.0)
    s = Server(hbm_budget_bytes, device=device, **kw)
    try:
        s.run([j], realtime=False)
    finally:
        s.close()
    return j
