"""Kernel tables, materials and scenes of the 3D solver.

The reference builds its 3D tables on the host in double precision
(``buildLUTs``, ``3d/app.js:85-160``) with only +, -, *, / and sqrt, all
correctly rounded in IEEE-754, so any IEEE double host reproduces them bit for
bit; this module restates that construction (JavaScript's ``Math.round`` is
round-half-up, i.e. ``floor(x + 0.5)``). Table image layout:
``W[2049] | G[2049] | planeW[513] | planeG[513]``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from functools import lru_cache

import numpy as np

ONE = 65536
LUT_N = 2049
PLANE_N = 513
RHO0 = 1048576
H_WU = 2.0
SPACING = 1.0
H = 131072           # smoothing radius, ticks
MAT_WORDS = 4        # grav, rhoW, damp, f0

# 3d/app.js:180-187 (grav: per-substep velocity step; rhoW: volume claim; damp: Q16 multiplier)
MATERIALS = [
    ('water', 180, 0, 65340, 20),
    ('oil', 110, 30, 65180, 35),
    ('mercury', 440, 0, 65420, 700),
    ('gas', -46, 120, 64700, 10),
    ('orbies', 88, 210, 65330, 60),
    ('goo', 92, 50, 62900, 45),
]


def js_round(x: float) -> int:
    """JavaScript's Math.round: the nearest integer, ties toward +infinity."""
    f = math.floor(x)
    return int(f + 1) if x - f >= 0.5 else int(f)


@lru_cache(maxsize=1)
def luts3d() -> np.ndarray:
    """The 3D kernel + wall tables as int32[2*2049 + 2*513]."""
    N, h = LUT_N, H_WU
    h2 = h * h
    rawW = [0.0] * N
    rawG = [0.0] * N
    for ui in range(N):
        r2 = ui / 512
        if r2 >= h2:
            continue
        t = h2 - r2
        rawW[ui] = t * t * t
        r = math.sqrt(r2)
        hr = h - r
        rawG[ui] = (hr * hr) / r if r > 1e-6 else 0.0
    for ui in range(N):
        if rawG[ui] > 0:
            rawG[0] = rawG[ui]
            break
    sum_raw = 0.0
    rad = math.ceil(h / SPACING)
    for i in range(-rad, rad + 1):
        for j in range(-rad, rad + 1):
            for k in range(-rad, rad + 1):
                r2 = (i * i + j * j + k * k) * SPACING * SPACING
                if r2 >= h2:
                    continue
                t = h2 - r2
                sum_raw += t * t * t
    SW = RHO0 / sum_raw
    SG = SW * 6 * (h2 - 1) * (h2 - 1)
    sp = SPACING
    lat = math.ceil(h / sp)
    planeW = [0] * PLANE_N
    planeG = [0] * PLANE_N
    for b in range(PLANE_N):
        dist = b / 256
        sw = 0.0
        sg = 0.0
        k = 0
        while True:
            pd = dist + k * sp
            if pd >= h:
                break
            for i in range(-lat, lat + 1):
                for j in range(-lat, lat + 1):
                    r2 = pd * pd + (i * sp) * (i * sp) + (j * sp) * (j * sp)
                    if r2 >= h2:
                        continue
                    t = h2 - r2
                    sw += t * t * t
                    sg += pd * t * t
            k += 1
        planeW[b] = js_round(sw * SW)
        planeG[b] = js_round(6 * sg * SW)
    out = np.zeros(2 * N + 2 * PLANE_N, np.int64)
    for ui in range(N):
        out[ui] = js_round(rawW[ui] * SW)
        out[N + ui] = js_round(rawG[ui] * SG)
    out[2 * N:2 * N + PLANE_N] = planeW
    out[2 * N + PLANE_N:] = planeG
    assert np.abs(out).max() < 2 ** 31
    return out.astype(np.int32)


BALL_N = 1024


@lru_cache(maxsize=16)
def _ball_tables(radius_wu: float):
    lut = luts3d()
    pw = lut[2 * LUT_N:2 * LUT_N + PLANE_N]
    pg = lut[2 * LUT_N + PLANE_N:]
    w = np.zeros(BALL_N, np.int32)
    g = np.zeros(BALL_N, np.int32)
    for b in range(BALL_N):
        r = math.sqrt(b * 4096) / 256
        depth = r - radius_wu
        if depth >= H_WU:
            continue
        d = max(depth, 0.0)
        at = max(0, min(512, js_round(d * 256)))
        w[b] = pw[at]
        g[b] = min(js_round(int(pg[at]) / r), 1 << 24) if r > 1e-6 else 0
    return w, g


def ball_tables(radius_wu: float):
    """The cursor-ball density and gradient tables (``buildBallLUT``,
    ``3d/app.js:212-230``), int32[1024] each, indexed by ``r2q >> 12``."""
    w, g = _ball_tables(float(radius_wu))
    return w.copy(), g.copy()


def mats3d() -> np.ndarray:
    return np.array([[g, r, d, f] for (_, g, r, d, f) in MATERIALS], np.int32)


def smix(x: int) -> int:
    """splitmix32 finaliser (``smix``, ``3d/app.js:232-239``)."""
    x = (x + 0x9e3779b9) & 0xffffffff
    z = x
    z = ((z ^ (z >> 16)) * 0x21f0aaad) & 0xffffffff
    z = ((z ^ (z >> 15)) * 0x735a2d97) & 0xffffffff
    return (z ^ (z >> 15)) & 0xffffffff


@dataclass
class Scene3D:
    n: int
    pos: np.ndarray   # int32 (n, 3)
    vel: np.ndarray   # int32 (n, 3)
    mat: np.ndarray   # uint32 (n,)
    gx: int
    gy: int
    gz: int
    name: str = ''


def column(bx: int, by: int, bz: int, gx: int, gy: int, gz: int, spacing: float = SPACING,
           mat: int = 0, name: str = '') -> Scene3D:
    """A jittered lattice block of bx*by*bz particles in the low corner of a
    gx*gy*gz-cell box (cells are 2 wu), x fastest, then z, then y, with the
    reference's splitmix jitter of +-1/16 wu per axis (``3d/app.js:321-361``)."""
    n = bx * by * bz
    pos = np.zeros((n, 3), np.int64)
    c = 0
    for j in range(by):
        for k in range(bz):
            for i in range(bx):
                jx = (smix(c * 3 + 0) % 8192) - 4096
                jy = (smix(c * 3 + 1) % 8192) - 4096
                jz = (smix(c * 3 + 2) % 8192) - 4096
                pos[c, 0] = js_round((1.5 + i * spacing) * ONE) + jx
                pos[c, 1] = js_round((1.5 + j * spacing) * ONE) + jy
                pos[c, 2] = js_round((1.5 + k * spacing) * ONE) + jz
                c += 1
    return Scene3D(n=n, pos=pos.astype(np.int32), vel=np.zeros((n, 3), np.int32),
                   mat=np.full(n, mat, np.uint32), gx=gx, gy=gy, gz=gz, name=name or f'column_{bx}x{by}x{bz}')


def column_fast(bx: int, by: int, bz: int, gx: int, gy: int, gz: int, mat: int = 0) -> Scene3D:
    """``column`` vectorised (same particles, same order) for large blocks."""
    n = bx * by * bz
    c = np.arange(n, dtype=np.uint64)

    def smix_v(x):
        x = (x + np.uint64(0x9e3779b9)) & np.uint64(0xffffffff)
        z = ((x ^ (x >> np.uint64(16))) * np.uint64(0x21f0aaad)) & np.uint64(0xffffffff)
        z = ((z ^ (z >> np.uint64(15))) * np.uint64(0x735a2d97)) & np.uint64(0xffffffff)
        return (z ^ (z >> np.uint64(15))) & np.uint64(0xffffffff)
    jx = (smix_v(c * np.uint64(3)) % np.uint64(8192)).astype(np.int64) - 4096
    jy = (smix_v(c * np.uint64(3) + np.uint64(1)) % np.uint64(8192)).astype(np.int64) - 4096
    jz = (smix_v(c * np.uint64(3) + np.uint64(2)) % np.uint64(8192)).astype(np.int64) - 4096
    ci = c.astype(np.int64)
    i = ci % bx
    k = (ci // bx) % bz
    j = ci // (bx * bz)
    base = lambda t: np.floor((1.5 + t * SPACING) * ONE + 0.5).astype(np.int64)
    pos = np.stack([base(i) + jx, base(j) + jy, base(k) + jz], axis=1)
    return Scene3D(n=n, pos=pos.astype(np.int32), vel=np.zeros((n, 3), np.int32),
                   mat=np.full(n, mat, np.uint32), gx=gx, gy=gy, gz=gz, name=f'column_{bx}x{by}x{bz}')


def dam3d_large() -> Scene3D:
    """3D dam break: a 64x64x64 water block (262,144 particles) in the corner of
    a 48 x 40 x 48-cell box (96 x 80 x 96 wu)."""
    return column_fast(64, 64, 64, 48, 40, 48)


def initial_state(n: int, scene: str = 'pool', gx: int = 28, gy: int = 30, gz: int = 28) -> Scene3D:
    """The reference's starting column (``initialState``, ``3d/app.js:321-361``):
    'pool' at 1 wu spacing over 55% of the floor, 'overdense' at 0.4 wu over 28%
    (the neighbour-truncation stress case), 'layers' with oil / water / mercury
    stacked out of density order."""
    dense = scene == 'overdense'
    sp = 0.4 if dense else SPACING
    world = (gx * H_WU, gy * H_WU, gz * H_WU)
    frac = 0.28 if dense else 0.55
    bx = math.floor((world[0] * frac) / sp)
    bz = math.floor((world[2] * frac) / sp)
    by_max = math.floor((world[1] * 0.92) / sp)
    by = min(by_max, math.ceil(n / (bx * bz)))
    pos, mat = [], []
    c = 0
    for j in range(by):
        for k in range(bz):
            for i in range(bx):
                if c >= n:
                    break
                jx = (smix(c * 3 + 0) % 8192) - 4096
                jy = (smix(c * 3 + 1) % 8192) - 4096
                jz = (smix(c * 3 + 2) % 8192) - 4096
                pos.append((js_round((1.5 + i * sp) * ONE) + jx, js_round((1.5 + j * sp) * ONE) + jy,
                            js_round((1.5 + k * sp) * ONE) + jz))
                if scene == 'layers':
                    f = j / by
                    mat.append(1 if f < 0.34 else (0 if f < 0.67 else 2))
                else:
                    mat.append(0)
                c += 1
    m = len(pos)
    return Scene3D(n=m, pos=np.array(pos, np.int32).reshape(m, 3), vel=np.zeros((m, 3), np.int32),
                   mat=np.array(mat, np.uint32), gx=gx, gy=gy, gz=gz, name=f'{scene}_{m}')


class SpawnSeed:
    """The pour's running splitmix seed and rejection-sampled disc (``spawn``,
    ``3d/app.js:575-597``): positions inside 0.8 x the ball radius."""

    def __init__(self, seed: int = 0x9e37):
        self.seed = seed

    def positions(self, cx: float, cy: float, cz: float, k: int, ball_r: float) -> np.ndarray:
        rad = ball_r * 0.8
        out = np.zeros((k, 3), np.int32)
        for i in range(k):
            while True:
                dx = ((smix(self.seed) % 2001) - 1000) / 1000
                dy = ((smix(self.seed + 1) % 2001) - 1000) / 1000
                dz = ((smix(self.seed + 2) % 2001) - 1000) / 1000
                self.seed += 3
                if dx * dx + dy * dy + dz * dz <= 1:
                    break
            out[i] = (js_round((cx + dx * rad) * ONE), js_round((cy + dy * rad) * ONE),
                      js_round((cz + dz * rad) * ONE))
        return out


# ---- build-defined 3D bonds -------------------------------------------------------
# The reference's 3D page has no bonds; the 3D dam-break workload asks for
# 4096 seeded bonds between lattice neighbours. They use the 2D engine's bond
# distance constraint restated over three axes (the engine's sn3_write_bonds):
# a row of BOND3_CAP entries {partner + 1, L0} per particle, L0 the rest
# length in ticks >> 5.
BOND3_CAP = 6
BOND3_WORDS = 2 * BOND3_CAP
BOND3_L0_MIN, BOND3_L0_MAX = 512, 5120
DAM3D_BONDS = 4096
DAM3D_BOND_SEED = 0xb0d3
DAM3D_BOND_K = 32768          # stiffness 0.5 (Q16)
DAM3D_BOND_BRK = 4 * 65536    # breaks past twice its rest length


def lattice_index(bx: int, by: int, bz: int, i: int, j: int, k: int) -> int:
    """Particle index of lattice site (i, j, k) in a ``column_fast`` block:
    x fastest, then z, then y."""
    return (j * bz + k) * bx + i


def lattice_bonds(bx: int, by: int, bz: int, count: int, seed: int) -> np.ndarray:
    """``count`` distinct bonds between face-adjacent lattice sites of a
    bx x by x bz block, drawn from a seeded stream: a site and an axis (+x,
    +y, +z), redrawn when the neighbour is outside the block or the pair is
    already bonded. Returns (count, 2) particle indices, first < second, in
    draw order."""
    rng = np.random.Generator(np.random.PCG64(seed))
    seen, out = set(), []
    while len(out) < count:
        i, j, k = (int(v) for v in rng.integers(0, (bx, by, bz)))
        axis = int(rng.integers(0, 3))
        i2, j2, k2 = i + (axis == 0), j + (axis == 1), k + (axis == 2)
        if i2 >= bx or j2 >= by or k2 >= bz:
            continue
        a, b = lattice_index(bx, by, bz, i, j, k), lattice_index(bx, by, bz, i2, j2, k2)
        if (a, b) in seen:
            continue
        seen.add((a, b))
        out.append((a, b))
    return np.array(out, np.int64)


def dam3d_bonds(sc: 'Scene3D') -> np.ndarray:
    """The 3D dam break's 4096 seeded lattice-neighbour bonds."""
    assert sc.n == 64 * 64 * 64
    return lattice_bonds(64, 64, 64, DAM3D_BONDS, DAM3D_BOND_SEED)


def _shr_rne(x: np.ndarray, s: int) -> np.ndarray:
    """Arithmetic shift right by s, rounding half to even (the engine's shr_rne)."""
    x = np.asarray(x, np.int64)
    q = x >> s
    r = x - (q << s)
    half = 1 << (s - 1)
    return q + ((r > half) | ((r == half) & (q & 1 == 1))).astype(np.int64)


def bond_rows(sc: 'Scene3D', bonds: np.ndarray) -> np.ndarray:
    """Rows for sn3_write_bonds: each bond (a, b) appended to both ends' rows
    in bond order, with rest length L0 = floor(sqrt(|d4|^2)) of the scene's
    starting positions (d4 = (p_a - p_b) >> 5, rounded half to even), clamped
    to [512, 5120]."""
    rows = np.zeros((sc.n, BOND3_CAP, 2), np.uint32)
    fill = np.zeros(sc.n, np.int64)
    pos = np.asarray(sc.pos, np.int64)
    for a, b in np.asarray(bonds, np.int64):
        d4 = _shr_rne(pos[a] - pos[b], 5)
        L0 = min(max(math.isqrt(int((d4 * d4).sum())), BOND3_L0_MIN), BOND3_L0_MAX)
        for u, v in ((a, b), (b, a)):
            if fill[u] >= BOND3_CAP:
                raise ValueError(f'particle {u} has more than {BOND3_CAP} bonds')
            rows[u, fill[u]] = (v + 1, L0)
            fill[u] += 1
    return rows.reshape(-1)
