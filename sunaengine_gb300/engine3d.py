"""The reference's 3D solver surface (class App in ``3d/app.js``) on the GB300 C ABI.

``Engine3D`` holds one or more independent 3D scenes on the device and steps
them together. The single-scene calls mirror the page: ``reset(n, scene)``
(``3d/app.js:561-568``), ``run_substeps(k)`` (``:709-714``), ``spawn(mat, cx,
cy, cz, k)`` (``:575-597``), ``set_ball_radius(R)`` / ``set_ball(...)`` (the
cursor ball, ``:599-629``) and ``chain()`` (the striped FNV digest,
``:717-744``). ``digest()`` / ``chain_hex()`` are the build-defined
H_set || H_slot hash of the 8 state words, folded every substep. Every call
goes through ``include/suna.h``; there is no CPU path.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _native, tables3d
from .engine import Digest, EngineError, _out_words

SUBSTEPS_PER_FRAME = 2   # CFG.substeps (3d/app.js:20)
ITERS = 3                # CFG.iters (3d/app.js:21)
GRID = (28, 30, 28)      # CFG.GX, GY, GZ (3d/app.js:12)
NMAX = 60000             # CFG.NMAX (3d/app.js:14)


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class _Scene3Args:
    def __init__(self, sc: tables3d.Scene3D, stir_amp: int = 0, frame: int = 0):
        n = int(sc.n)
        self.pos = np.ascontiguousarray(np.asarray(sc.pos).reshape(-1), dtype=np.int32)
        self.vel = np.ascontiguousarray(np.asarray(sc.vel).reshape(-1), dtype=np.int32)
        self.mat = np.ascontiguousarray(np.asarray(sc.mat).reshape(-1), dtype=np.uint32)
        if self.pos.size != 3 * n or self.vel.size != 3 * n or self.mat.size != n:
            raise EngineError('3D scene array lengths must be n*3 / n*3 / n')
        self.c = _native.Sn3Scene(n=n, pos=self.pos.ctypes.data, vel=self.vel.ctypes.data,
                                  mat=self.mat.ctypes.data, gx=int(sc.gx), gy=int(sc.gy), gz=int(sc.gz),
                                  stir_amp=int(stir_amp), frame=int(frame))


class Engine3D:
    """Device-resident 3D scenes advanced by one launch sequence per substep."""

    def __init__(self, max_particles: int = NMAX, max_cells: int = 0, max_scenes: int = 1,
                 iters: int = ITERS, debug: bool = False, chain: bool = True, device: int = 0, lanes: int = 0):
        self._lib = _native.load()
        self._luts = np.ascontiguousarray(tables3d.luts3d(), dtype=np.int32)
        self._mats = np.ascontiguousarray(tables3d.mats3d().reshape(-1), dtype=np.int32)
        o = _native.Sn3Opts(max_particles=int(max_particles), max_cells=int(max_cells),
                            max_scenes=int(max_scenes), iters=int(iters), debug=1 if debug else 0,
                            chain=1 if chain else 0, device=int(device), luts=self._luts.ctypes.data,
                            mats=self._mats.ctypes.data, mat_count=self._mats.size // 4, lanes=int(lanes))
        h = ctypes.c_void_p()
        rc = self._lib.sn3_create(ctypes.byref(o), ctypes.byref(h))
        if rc != 0 or not h.value:
            raise EngineError(f'sn3_create failed ({rc})')
        self.h = h
        self.max_particles = int(max_particles)
        self.iters = int(iters)
        self._seed = tables3d.SpawnSeed()
        self._ball = {'x': 0.0, 'y': 0.0, 'z': 0.0, 'on': False, 'r': 3.0}

    def close(self):
        if getattr(self, 'h', None):
            self._lib.sn3_destroy(self.h)
            self.h = None

    __del__ = close

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self._lib.sn3_last_error(self.h)
            raise EngineError(f'[aether-3d] {what}: {msg.decode() if msg else rc}')

    # ---- scenes -------------------------------------------------------------
    def load_scene(self, sc: tables3d.Scene3D, stir_amp: int = 0, frame: int = 0) -> 'Engine3D':
        a = _Scene3Args(sc, stir_amp, frame)
        self._check(self._lib.sn3_load_scene(self.h, ctypes.byref(a.c)), 'load_scene')
        self._seed = tables3d.SpawnSeed()
        return self

    def reset(self, n: int = 16000, scene: str = 'pool', grid=GRID, stir_amp: int = 0) -> 'Engine3D':
        """reset(n, scene) (3d/app.js:561-568): the page's starting column."""
        return self.load_scene(tables3d.initial_state(min(n, self.max_particles), scene, *grid), stir_amp)

    def add_scene(self, sc: tables3d.Scene3D, cap: int = 0, stir_amp: int = 0, frame: int = 0) -> int:
        a = _Scene3Args(sc, stir_amp, frame)
        out = ctypes.c_uint32()
        self._check(self._lib.sn3_add_scene(self.h, ctypes.byref(a.c), int(cap), ctypes.byref(out)), 'add_scene')
        return int(out.value)

    def remove_scene(self, scene: int):
        self._check(self._lib.sn3_remove_scene(self.h, int(scene)), 'remove_scene')

    # ---- stepping -----------------------------------------------------------
    def step(self, count: int = 1) -> int:
        if int(count) < 0:
            raise EngineError('[aether-3d] step(count) needs a non-negative integer')
        self._check(self._lib.sn3_step(self.h, int(count)), 'step')
        return self.info(0)['substep_count'] if self._has(0) else 0

    def run_substeps(self, k: int = SUBSTEPS_PER_FRAME) -> int:
        return self.step(k)

    def _has(self, scene: int) -> bool:
        out = _native.Sn3Info()
        return self._lib.sn3_get_info(self.h, int(scene), ctypes.byref(out)) == 0

    # ---- inputs -------------------------------------------------------------
    def spawn_positions(self, pos, mat, scene: int = 0) -> int:
        pos = np.ascontiguousarray(np.asarray(pos).reshape(-1), dtype=np.int32)
        mat = np.ascontiguousarray(np.asarray(mat).reshape(-1), dtype=np.uint32)
        if pos.size != 3 * mat.size:
            raise EngineError('spawn: pos must hold 3 words per particle')
        added = ctypes.c_uint32()
        self._check(self._lib.sn3_spawn(self.h, int(scene), _ptr(pos), _ptr(mat), mat.size, ctypes.byref(added)),
                    'spawn')
        return int(added.value)

    def spawn(self, mat: int, cx: float, cy: float, cz: float, k: int, scene: int = 0) -> int:
        """spawn(mat, cx, cy, cz, k) (3d/app.js:575-597): k particles inside
        0.8 x the ball radius around (cx, cy, cz) world units, from the page's
        running splitmix seed; returns how many fit."""
        room = self.max_particles - self.info(scene)['n']
        k = min(int(k), room)
        if k <= 0:
            return 0
        pos = self._seed.positions(cx, cy, cz, k, self._ball['r'])
        return self.spawn_positions(pos, np.full(k, int(mat), np.uint32), scene)

    def set_ball(self, on: bool, x: float, y: float, z: float, radius: Optional[float] = None, scene: int = 0):
        """The cursor ball at (x, y, z) world units (quantised with Math.round,
        3d/app.js:620-624)."""
        if radius is not None:
            self._ball['r'] = float(radius)
        self._ball.update(x=float(x), y=float(y), z=float(z), on=bool(on))
        q = lambda v: tables3d.js_round(v * tables3d.ONE)
        self._check(self._lib.sn3_set_ball(self.h, int(scene), 1 if on else 0, q(x), q(y), q(z),
                                           ctypes.c_double(self._ball['r'])), 'set_ball')

    def set_ball_radius(self, R: float, scene: int = 0):
        b = self._ball
        self.set_ball(b['on'], b['x'], b['y'], b['z'], R, scene)

    # ---- readback -----------------------------------------------------------
    def _words(self, fn, scene, k=8):
        a = np.zeros(k, np.uint32)
        self._check(fn(self.h, int(scene), _ptr(a)), fn.__name__)
        return a

    def chain(self, scene: int = 0) -> str:
        """The page's digest (3d/app.js:717-744): 64 hex characters."""
        return ''.join(f'{int(w):08x}' for w in self._words(self._lib.sn3_fnv, scene))

    fnv_hex = chain

    def digest(self, scene: int = 0) -> Digest:
        return Digest(self._words(self._lib.sn3_digest, scene))

    def chain_hex(self, scene: int = 0) -> str:
        return ''.join(f'{int(w):08x}' for w in self._words(self._lib.sn3_chain, scene))

    def read_state(self, scene: int = 0, out: Optional[np.ndarray] = None) -> np.ndarray:
        a = _out_words(out, self.info(scene)['n'] * 8)
        self._check(self._lib.sn3_read_state(self.h, int(scene), _ptr(a), a.size), 'read_state')
        return a

    def write_bonds(self, rows, stiffness: int, break_ratio: int, scene: int = 0):
        """Build-defined bonds of a scene (sn3_write_bonds): rows of
        tables3d.BOND3_WORDS words per particle (tables3d.bond_rows)."""
        a = np.ascontiguousarray(np.asarray(rows, np.uint32).reshape(-1))
        self._check(self._lib.sn3_write_bonds(self.h, int(scene), _ptr(a), a.size, int(stiffness), int(break_ratio)),
                    'write_bonds')

    def read_bonds(self, scene: int = 0) -> np.ndarray:
        n = self.info(scene)['n']
        a = np.zeros(max(1, n * tables3d.BOND3_WORDS), np.uint32)
        self._check(self._lib.sn3_read_bonds(self.h, int(scene), _ptr(a), a.size), 'read_bonds')
        return a[:n * tables3d.BOND3_WORDS]

    def write_state(self, state, substeps: int, chain_words=None, scene: int = 0):
        st = np.ascontiguousarray(np.asarray(state).reshape(-1), dtype=np.int32)
        if st.size % 8:
            raise EngineError('[aether-3d] write_state: 8 words per particle')
        ch = None if chain_words is None else np.ascontiguousarray(chain_words, dtype=np.uint32)
        self._check(self._lib.sn3_write_state(self.h, int(scene), _ptr(st), st.size // 8, int(substeps), _ptr(ch)),
                    'write_state')

    def chain_words(self, scene: int = 0) -> np.ndarray:
        return self._words(self._lib.sn3_chain, scene)

    # device keyframes (sn3_ckpt_*): see checkpoints.CheckpointPool
    def ckpt_bytes(self, scene: int = 0) -> int:
        out = ctypes.c_size_t()
        self._check(self._lib.sn3_ckpt_bytes(self.h, int(scene), ctypes.byref(out)), 'ckpt_bytes')
        return int(out.value)

    def ckpt_save(self, scene: int, pool) -> int:
        out = ctypes.c_uint64()
        self._check(self._lib.sn3_ckpt_save(self.h, int(scene), pool.h, ctypes.byref(out)), 'ckpt_save')
        return int(out.value)

    def ckpt_load(self, scene: int, pool, handle: int):
        self._check(self._lib.sn3_ckpt_load(self.h, int(scene), pool.h, int(handle)), 'ckpt_load')

    def debug_counters(self) -> np.ndarray:
        a = np.zeros(16, np.uint32)
        self._check(self._lib.sn3_debug_counters(self.h, _ptr(a)), 'debug_counters')
        return a

    def sync(self):
        self._check(self._lib.sn3_sync(self.h), 'sync')

    def info(self, scene: int = 0) -> dict:
        out = _native.Sn3Info()
        self._check(self._lib.sn3_get_info(self.h, int(scene), ctypes.byref(out)), 'info')
        return {f: getattr(out, f) for f, _ in _native.Sn3Info._fields_}

    @property
    def n(self) -> int:
        return self.info(0)['n']

    @property
    def substep_count(self) -> int:
        return self.info(0)['substep_count']

    def last_timing(self):
        ms = ctypes.c_float()
        launches = ctypes.c_uint64()
        self._check(self._lib.sn3_last_timing(self.h, ctypes.byref(ms), ctypes.byref(launches)), 'last_timing')
        return float(ms.value), int(launches.value)

    def profile_substep(self, reps: int = 10):
        ms = np.zeros(64, np.float32)
        n = ctypes.c_uint32()
        self._check(self._lib.sn3_profile_substep(self.h, int(reps), _ptr(ms), 64, ctypes.byref(n)), 'profile')
        return ms[:n.value].copy()

    # camelCase aliases of the page's method names
    runSubsteps = run_substeps
    setBallRadius = set_ball_radius
