"""Scene construction: the reference's canonical scenes and the benchmark workloads.

Integer-only, seeded construction as in the reference's ``makeScene``
(``src/engine.js:2469-2648``): positions are Q16.16 ticks, the only entropy is
``xorshift32`` (``src/engine.js:2153-2161``), and every boundary container is
``boundaryRing`` (``src/engine.js:2416-2432``).

``dambreak_v1`` is the reference's frozen determinism-gate scene; it must stay
byte-identical to the reference's or the golden chain cannot match.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace
from typing import Optional

import numpy as np

from .data import mat_id

ONE = 65536
H = 163840
CELL_SHIFT = 18
AMBIENT = 20 * ONE
MAX_POS = 1 << 27
DOM_W, DOM_H = 128, 72
MAT_WATER = 0
MAT_GEL = 1
MAT_OIL = 4


def deg(d: int) -> int:
    return d * ONE


def wu(x: float) -> int:
    """World units to ticks, rounded like the reference's ``wu()`` helper."""
    return int(round(x * ONE))


@dataclass
class Scene:
    """A loadable scene: the argument of ``Engine.loadScene``.

    ``pos`` and ``vel`` are int32 arrays of shape (n, 2); ``matId`` is uint32
    (n,); ``flags``/``temp``/``fuel`` are optional per-particle arrays (absent
    means the loader's defaults: 0, AMBIENT and the material's ``fuel0``).
    """
    n: int
    nFluid: int
    pos: np.ndarray
    vel: np.ndarray
    matId: np.ndarray
    domW: int
    domH: int
    cellShift: int = CELL_SHIFT
    flags: Optional[np.ndarray] = None
    temp: Optional[np.ndarray] = None
    fuel: Optional[np.ndarray] = None
    name: str = ''
    meta: dict = field(default_factory=dict)

    def copy(self) -> 'Scene':
        cp = lambda a: None if a is None else a.copy()
        return replace(self, pos=self.pos.copy(), vel=self.vel.copy(), matId=self.matId.copy(),
                       flags=cp(self.flags), temp=cp(self.temp), fuel=cp(self.fuel), meta=dict(self.meta))


class Xorshift32:
    """``xorshift32`` (``src/engine.js:2153-2161``); seed 0 maps to 0x2545f491."""

    def __init__(self, seed: int):
        self.s = (seed & 0xffffffff) or 0x2545f491

    def __call__(self) -> int:
        s = self.s
        s ^= (s << 13) & 0xffffffff
        s ^= s >> 17
        s ^= (s << 5) & 0xffffffff
        self.s = s & 0xffffffff
        return self.s


def boundary_ring(dom_w_wu: int, dom_h_wu: int, wall_rows: int) -> np.ndarray:
    """Static container: 2 floor rows plus 2 columns up each side.

    Same particle order as ``boundaryRing`` (``src/engine.js:2416-2432``).
    """
    half = ONE >> 1
    out = []
    for row in range(2):
        y = dom_h_wu * ONE - half - row * ONE
        for c in range(dom_w_wu):
            out.append((half + c * ONE, y))
    for x_base in (half, dom_w_wu * ONE - half):
        for col in range(2):
            x = half + col * ONE if x_base == half else x_base - col * ONE
            for r in range(wall_rows):
                out.append((x, dom_h_wu * ONE - half - (2 + r) * ONE))
    return np.array(out, dtype=np.int64).reshape(-1, 2).astype(np.int32)


def _assemble(fluid_pos, fluid_mat, bnd, dom_w_wu, dom_h_wu, name, vel=None, temp=None):
    nf = len(fluid_pos)
    n = nf + len(bnd)
    pos = np.zeros((n, 2), np.int32)
    if nf:
        pos[:nf] = np.asarray(fluid_pos, dtype=np.int64).reshape(nf, 2)
    pos[nf:] = bnd
    matId = np.zeros(n, np.uint32)
    matId[:nf] = fluid_mat
    v = np.zeros((n, 2), np.int32)
    if vel is not None:
        v[:nf] = vel
    sc = Scene(n=n, nFluid=nf, pos=pos, vel=v, matId=matId,
               domW=dom_w_wu * ONE, domH=dom_h_wu * ONE, name=name)
    if temp is not None:
        t = np.full(n, AMBIENT, np.int32)
        t[:nf] = temp
        sc.temp = t
    return sc


FLAG_ANCHOR = 4


def sealed_box(spacing: float = 0.6, held: bool = True, seal: str = 'RUBBER', seed: int = 0x5ea1,
               membrane: bool = False, closed: bool = True) -> Scene:
    """Containment scenes (build-defined; the reference ships no frozen one).

    ``membrane=False``: a box of seal-class particles (1 wu apart, held with
    FLAG_ANCHOR when ``held``; without its lid when ``closed`` is False) in a
    48 x 40 wu walled box, filled with a jittered WATER block at ``spacing``
    wu. Below rest spacing (1 wu) the block starts compressed: pressure drives
    it into the seal and crowded rows fill their 48-entry neighbour lists
    (containOverflow's path).
    ``membrane=True``: a free horizontal strip of seal particles (welded at
    load) carrying a WATER block over empty space.
    """
    rng = Xorshift32(seed)
    dom_w, dom_h = 48, 40
    half = ONE >> 1
    sm = mat_id(seal)
    seal_pts = []
    if membrane:
        for c in range(10, 39):
            seal_pts.append((c * ONE + half, 22 * ONE + half))
        x0, x1, y0, y1 = 11.0, 37.0, 12.0, 21.5
    else:
        for c in range(8, 41):
            seal_pts.append((c * ONE + half, 34 * ONE + half))
        for r in range(12, 34):
            seal_pts.append((8 * ONE + half, r * ONE + half))
            seal_pts.append((40 * ONE + half, r * ONE + half))
        if closed:
            for c in range(9, 40):
                seal_pts.append((c * ONE + half, 11 * ONE + half))
        x0, x1, y0, y1 = 9.6, 39.4, 14.0, 33.6
    water = []
    sp = int(round(spacing * ONE))
    jit = max(1, sp // 8)
    y = int(y1 * ONE)
    while y >= int(y0 * ONE):
        x = int(x0 * ONE)
        while x <= int(x1 * ONE):
            jx = (rng() % (2 * jit + 1)) - jit
            jy = (rng() % (2 * jit + 1)) - jit
            water.append((x + jx, y + jy))
            x += sp
        y -= sp
    fl_pos = seal_pts + water
    fl_mat = np.array([sm] * len(seal_pts) + [MAT_WATER] * len(water), np.uint32)
    sc = _assemble(fl_pos, fl_mat, boundary_ring(dom_w, dom_h, dom_h - 4), dom_w, dom_h,
                   f"{'membrane' if membrane else 'sealed_box'}_{seal.lower()}")
    if held and not membrane:
        fl = np.zeros(sc.n, np.uint32)
        fl[:len(seal_pts)] = FLAG_ANCHOR
        sc.flags = fl
    sc.meta = {'seal': len(seal_pts), 'water': len(water), 'box': (8, 40, 12, 35) if not membrane else None}
    return sc


def rigid_tank(plank: str = 'METAL', wheel: str = 'WOOD', rail: bool = True, seed: int = 0x71a9,
               plank_temp: Optional[int] = None, water: bool = True) -> Scene:
    """Rigid-body scenes (build-defined; the reference ships no frozen one).

    A 64 x 44 wu walled tank with a jittered WATER pool (y 30.5..41.5 wu), an
    L-shaped plank of ``plank`` (a 16 x 3 bar with a 3 x 5 leg, 1 wu lattice)
    above it, a disc of radius 5 wu of ``wheel`` at (46, 20) and, with
    ``rail``, a held STONE rail (FLAG_ANCHOR; STONE is seal class, so it also
    wears FLAG_SEAL) under the plank. ``meta`` names the slot lists; a body is
    made from them with ``makeRigidBody`` / ``makeAxisBody`` after the load.
    """
    rng = Xorshift32(seed)
    dom_w, dom_h = 64, 44
    half = ONE >> 1
    pos, mat, temp = [], [], []
    meta = {}
    if plank:
        pm = mat_id(plank)
        sl = []
        for r in range(3):
            for c in range(16):
                sl.append(len(pos))
                pos.append((8 * ONE + half + c * ONE, 14 * ONE + half + r * ONE))
                mat.append(pm)
        for r in range(3, 8):
            for c in range(3):
                sl.append(len(pos))
                pos.append((21 * ONE + half + c * ONE, 14 * ONE + half + r * ONE))
                mat.append(pm)
        meta['plank'] = sl
    if wheel:
        wm = mat_id(wheel)
        sl = []
        for r in range(-5, 6):
            for c in range(-5, 6):
                if r * r + c * c <= 25:
                    sl.append(len(pos))
                    pos.append((46 * ONE + c * ONE, 20 * ONE + r * ONE))
                    mat.append(wm)
        meta['wheel'] = sl
        meta['wheel_centre'] = (46 * ONE, 20 * ONE)
    if rail:
        sl = []
        for c in range(7):
            sl.append(len(pos))
            pos.append((9 * ONE + half + c * ONE, 24 * ONE + half))
            mat.append(mat_id('STONE'))
        meta['rail'] = sl
    if water:
        jit = ONE // 8
        y = 30 * ONE + half
        w = []
        while y <= 41 * ONE + half:
            x = 3 * ONE + half
            while x <= 60 * ONE + half:
                jx = (rng() % (2 * jit + 1)) - jit
                jy = (rng() % (2 * jit + 1)) - jit
                w.append(len(pos))
                pos.append((x + jx, y + jy))
                mat.append(MAT_WATER)
                x += ONE
            y += ONE
        meta['water'] = w
    sc = _assemble(pos, np.array(mat, np.uint32), boundary_ring(dom_w, dom_h, dom_h - 4), dom_w, dom_h,
                   f'rigid_tank_{plank.lower() if plank else "none"}')
    fl = np.zeros(sc.n, np.uint32)
    for i in meta.get('rail', []):
        fl[i] = FLAG_ANCHOR
    sc.flags = fl
    if plank_temp is not None and plank:
        t = np.full(sc.n, AMBIENT, np.int32)
        t[meta['plank']] = plank_temp
        sc.temp = t
    sc.meta = meta
    return sc


def construction_site(tiles: int = 24, depth: int = 44, seed: int = 0xc0457) -> Scene:
    """The widened rows at scale (build-defined): ``tiles`` 64-wu bays side by
    side, each with an L-shaped METAL plank (63 members), a WOOD disc of
    radius 5 wu (81 members) and a held STONE rail (seal class: containment
    runs) above one WATER pool ``depth`` rows deep spanning the whole width.
    ``meta`` lists each bay's plank and wheel slots and the wheel centres, so
    a caller makes one free body per plank and one axis body per wheel."""
    rng = Xorshift32(seed)
    dom_w, dom_h = 64 * tiles, depth + 52
    half = ONE >> 1
    pos, mat = [], []
    planks, wheels, centres, rails = [], [], [], []
    metal, wood, stone = mat_id('METAL'), mat_id('WOOD'), mat_id('STONE')
    for t in range(tiles):
        ox = t * 64 * ONE
        sl = []
        for r in range(3):
            for c in range(16):
                sl.append(len(pos))
                pos.append((ox + 8 * ONE + half + c * ONE, 14 * ONE + half + r * ONE))
                mat.append(metal)
        for r in range(3, 8):
            for c in range(3):
                sl.append(len(pos))
                pos.append((ox + 21 * ONE + half + c * ONE, 14 * ONE + half + r * ONE))
                mat.append(metal)
        planks.append(sl)
        sl = []
        cx, cy = ox + 46 * ONE, 20 * ONE
        for r in range(-5, 6):
            for c in range(-5, 6):
                if r * r + c * c <= 25:
                    sl.append(len(pos))
                    pos.append((cx + c * ONE, cy + r * ONE))
                    mat.append(wood)
        wheels.append(sl)
        centres.append((cx + ONE, cy))
        for c in range(7):
            rails.append(len(pos))
            pos.append((ox + 9 * ONE + half + c * ONE, 28 * ONE + half))
            mat.append(stone)
    jit = ONE // 8
    y = (dom_h - 2 - depth) * ONE + half
    while y <= (dom_h - 3) * ONE + half:
        x = 3 * ONE + half
        while x <= (dom_w - 4) * ONE + half:
            jx = (rng() % (2 * jit + 1)) - jit
            jy = (rng() % (2 * jit + 1)) - jit
            pos.append((x + jx, y + jy))
            mat.append(MAT_WATER)
            x += ONE
        y += ONE
    sc = _assemble(pos, np.array(mat, np.uint32), boundary_ring(dom_w, dom_h, dom_h - 4), dom_w, dom_h,
                   f'construction_site_{tiles}')
    fl = np.zeros(sc.n, np.uint32)
    fl[rails] = FLAG_ANCHOR
    sc.flags = fl
    sc.meta = {'planks': planks, 'wheels': wheels, 'wheel_pivots': centres, 'rails': rails}
    return sc


def make_scene(name: str, **opts) -> Scene:
    """The reference's canonical scenes (``makeScene``, ``src/engine.js:2469-2648``)."""
    if name == 'dambreak_v1':
        rnd = Xorshift32(0x1234567)
        fl = []
        for gy in range(60):
            for gx in range(60):
                jx = (rnd() % 4097) - 2048
                jy = (rnd() % 4097) - 2048
                fl.append((3 * ONE + gx * ONE + jx, (DOM_H - 3) * ONE - gy * ONE + jy))
        return _assemble(fl, MAT_WATER, boundary_ring(DOM_W, DOM_H, 60), DOM_W, DOM_H, name)
    if name == 'overdense_v1':
        side, sp = 32, ONE >> 1
        cx, cy = 64 * ONE, 40 * ONE
        fl = [(cx + (gx - side // 2) * sp, cy + (gy - side // 2) * sp)
              for gy in range(side) for gx in range(side)]
        return _assemble(fl, MAT_WATER, boundary_ring(DOM_W, DOM_H, 60), DOM_W, DOM_H, name)
    if name == 'pool_v1':
        cw, ch = opts.get('w', 100), opts.get('h', 24)
        mat = opts.get('mat', MAT_WATER)
        if not (13 + cw <= DOM_W - 2 and ch <= DOM_H - 5):
            raise ValueError(f'pool_v1 w={cw} h={ch} does not fit the {DOM_W}x{DOM_H} wu domain')
        rnd = Xorshift32(0x0be7a1)
        fl = []
        for gy in range(ch):
            for gx in range(cw):
                jx = (rnd() % 4097) - 2048
                jy = (rnd() % 4097) - 2048
                fl.append((13 * ONE + gx * ONE + jx, (DOM_H - 3) * ONE - gy * ONE + jy))
        return _assemble(fl, mat, boundary_ring(DOM_W, DOM_H, 60), DOM_W, DOM_H, name)
    if name == 'droplet_v1':
        mat = opts.get('mat', MAT_WATER)
        rx, ry = opts.get('rx', 13), opts.get('ry', 2)
        cx, cy = 64 * ONE, 22 * ONE
        fl = []
        for gy in range(-ry, ry + 1):
            for gx in range(-rx, rx + 1):
                nx, ny = gx / rx, gy / ry
                if nx * nx + ny * ny > 1.0:
                    continue
                fl.append((cx + gx * ONE, cy + gy * ONE))
        return _assemble(fl, mat, boundary_ring(DOM_W, DOM_H, 60), DOM_W, DOM_H, name)
    if name == 'stretch_v1':
        mat = opts.get('mat', MAT_GEL)
        pull = opts.get('pull', 8000)
        fl, vel = [], []
        r = 6
        for side in (-1, 1):
            cx, cy = 64 * ONE + side * 8 * ONE, 36 * ONE
            for gy in range(-r, r + 1):
                for gx in range(-r, r + 1):
                    if gx * gx + gy * gy > r * r:
                        continue
                    fl.append((cx + gx * ONE, cy + gy * ONE))
                    vel.append((side * pull, 0))
        return _assemble(fl, mat, boundary_ring(DOM_W, DOM_H, 60), DOM_W, DOM_H, name,
                         vel=np.array(vel, np.int32))
    if name == 'empty_v1':
        w = max(8, int(opts.get('domWwu', DOM_W)))
        h = max(16, int(opts.get('domHwu', DOM_H)))
        return _assemble([], MAT_WATER, boundary_ring(w, h, h - 12), w, h, name)
    raise ValueError(f'unknown scene "{name}"')


def permute_scene(scene: Scene, seed: int) -> Scene:
    """Deterministic permutation of the fluid block (``permuteScene``, ``src/engine.js:2651-2679``)."""
    out = scene.copy()
    rnd = Xorshift32(seed)
    nf = scene.nFluid
    perm = list(range(nf))
    for i in range(nf - 1, 0, -1):
        j = rnd() % (i + 1)
        perm[i], perm[j] = perm[j], perm[i]
    perm = np.array(perm, dtype=np.int64)
    out.pos[:nf] = scene.pos[perm]
    out.vel[:nf] = scene.vel[perm]
    out.matId[:nf] = scene.matId[perm]
    for k in ('temp', 'fuel', 'flags'):
        a = getattr(scene, k)
        if a is not None:
            getattr(out, k)[:nf] = a[perm]
    return out


def make_droplet(cx: int, cy: int, rx: int, ry: int, vx: int = 0, vy: int = 0, spacing: int = ONE):
    """A small elliptical blob of particles, as a list of dicts for ``inject``."""
    out = []
    for gy in range(-ry, ry + 1):
        for gx in range(-rx, rx + 1):
            if rx and ry and (gx / rx) ** 2 + (gy / ry) ** 2 > 1.0:
                continue
            out.append({'x': cx + gx * spacing, 'y': cy + gy * spacing, 'vx': vx, 'vy': vy})
    return out


# ---------------------------------------------------------------------------
# Benchmark workloads. Synthetic, seeded; shapes follow the workload table.
# ---------------------------------------------------------------------------

def lattice_dambreak(nx: int = 64, ny: int = 64, spacing: int = ONE * 5 // 4,
                     mat: int = MAT_WATER) -> Scene:
    """Dam break: an nx x ny lattice at ``spacing`` in the left quarter of a walled box.

    Default: 64 x 64 WATER particles at 1.25 wu (half the 2.5 wu smoothing
    length), zero velocity, AMBIENT temperature, standing on the floor against
    the left wall of a box four block-widths wide. The container is
    ``boundary_ring`` with side walls stopping 12 wu short of the top, like
    the reference's ``empty_v1``.
    """
    bw = -(-(nx * spacing) // ONE)          # block width, wu (ceil)
    bh = -(-(ny * spacing) // ONE)
    dom_w = 4 * (bw + 4)
    dom_h = bh + 16
    fl = []
    for gy in range(ny):
        for gx in range(nx):
            fl.append((3 * ONE + gx * spacing, (dom_h - 3) * ONE - gy * spacing))
    return _assemble(fl, mat, boundary_ring(dom_w, dom_h, dom_h - 12), dom_w, dom_h,
                     f'dambreak_{nx}x{ny}')


def large_two_fluid(side: int = 1024, seed: int = 0x5eed2, band: int = 64,
                    t_lo: int = deg(10), t_hi: int = deg(90)) -> Scene:
    """Large 2D scene: a side x side lattice at 1 wu with seeded +/-0.25 wu jitter.

    Materials alternate WATER / OIL in ``band``-column bands; every particle's
    temperature is drawn uniformly from [t_lo, t_hi] (inside both rows'
    transition thresholds). Default 1024 x 1024 = 1,048,576 fluid particles.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    gx, gy = np.meshgrid(np.arange(side, dtype=np.int64), np.arange(side, dtype=np.int64))
    gx = gx.ravel()
    gy = gy.ravel()
    jit = rng.integers(-(ONE // 4), ONE // 4 + 1, size=(side * side, 2), dtype=np.int64)
    dom_w = side + 16
    dom_h = side + 36
    x = 8 * ONE + gx * ONE + jit[:, 0]
    y = (dom_h - 4) * ONE - gy * ONE + jit[:, 1]
    mats = np.where((gx // band) % 2 == 0, MAT_WATER, MAT_OIL).astype(np.uint32)
    temp = rng.integers(t_lo, t_hi + 1, size=side * side, dtype=np.int64).astype(np.int32)
    fl = np.stack([x, y], axis=1)
    sc = _assemble(fl, mats, boundary_ring(dom_w, dom_h, dom_h - 12), dom_w, dom_h,
                   f'two_fluid_{side}x{side}', temp=temp)
    return sc


def jittered_block(n_target: int, aspect: float, rng: np.random.Generator,
                   mat: int = MAT_WATER) -> Scene:
    """One scene of a batch: a jittered 1 wu lattice block of about ``n_target``
    particles with width/height ``aspect``, in a walled box twice its width."""
    h = max(2, int(round(math.sqrt(n_target / aspect))))
    w = max(2, int(round(n_target / h)))
    dom_w = 2 * w + 8
    dom_h = h + 20
    gx, gy = np.meshgrid(np.arange(w, dtype=np.int64), np.arange(h, dtype=np.int64))
    gx = gx.ravel()
    gy = gy.ravel()
    jit = rng.integers(-(ONE // 4), ONE // 4 + 1, size=(w * h, 2), dtype=np.int64)
    x = 4 * ONE + gx * ONE + jit[:, 0]
    y = (dom_h - 4) * ONE - gy * ONE + jit[:, 1]
    fl = np.stack([x, y], axis=1)
    return _assemble(fl, mat, boundary_ring(dom_w, dom_h, dom_h - 12), dom_w, dom_h,
                     f'block_{w}x{h}')


def stir_schedule(scene: Scene, substeps: int, rng: np.random.Generator, mean_gap: int = 50):
    """Seeded stir events for a scene: disc impulses at seeded substep indices.

    About one event per ``mean_gap`` substeps; radius 2..8 wu; impulse up to
    0.45 wu/substep per axis. Each event is (substep, cx, cy, r, ix, iy) in ticks.
    """
    ev = []
    s = int(rng.integers(0, mean_gap))
    stir_max = wu(0.45)
    while s < substeps:
        fl = scene.pos[:scene.nFluid]
        k = int(rng.integers(0, max(1, scene.nFluid)))
        cx, cy = int(fl[k, 0]), int(fl[k, 1])
        r = int(rng.integers(2 * ONE, 8 * ONE))
        ix = int(rng.integers(-stir_max, stir_max + 1))
        iy = int(rng.integers(-stir_max, stir_max + 1))
        ev.append((s, cx, cy, r, ix, iy))
        s += 1 + int(rng.integers(mean_gap // 2, 3 * mean_gap // 2))
    return ev


def batch_scenes(count: int = 256, seed: int = 0xba7c4, n_lo: int = 1024, n_hi: int = 65536,
                 substeps: int = 1000):
    """Batched workload: ``count`` independent scenes, particle counts log-uniform
    in [n_lo, n_hi], aspect ratios uniform in [0.5, 2], each with its own stir
    schedule. Returns (scenes, schedules).

    The scenes come from one seeded stream and each schedule from a stream of
    its own (seeded by the workload seed and the scene index), so the scenes do
    not depend on ``substeps`` and a shorter schedule is a prefix of a longer
    one: scene ``i`` is the same scene in a 60-substep test and a 1000-substep
    run.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    scenes, sched = [], []
    for sid in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        aspect = float(rng.uniform(0.5, 2.0))
        sc = jittered_block(n, aspect, rng)
        scenes.append(sc)
        sched.append(stir_schedule(sc, substeps, np.random.Generator(np.random.PCG64([seed, sid]))))
    return scenes, sched
