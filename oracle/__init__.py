"""ORACLE — test infrastructure only.

A CPU restatement of the reference substep (``suna_oracle.cpp``) behind a small
ctypes wrapper. The test suite, ``__graft_entry__.smoke()`` and the benchmark's
CPU-baseline leg use it as the checker; the product package never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / '_build'
LIB = BUILD / 'libsuna_oracle.so'


def build(force: bool = False) -> Path:
    """Compile the oracle with g++ (OpenMP) into oracle/_build."""
    src = [HERE / 'suna_oracle.cpp', HERE / 'suna3d_oracle.cpp', HERE / 'fixed_ref.h']
    if LIB.exists() and not force and all(LIB.stat().st_mtime >= s.stat().st_mtime for s in src):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = BUILD / f'libsuna_oracle.{os.getpid()}.so'
    cmd = ['g++', '-O2', '-std=c++17', '-fopenmp', '-ffp-contract=off', '-shared', '-fPIC',
           str(HERE / 'suna_oracle.cpp'), str(HERE / 'suna3d_oracle.cpp'), '-o', str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        l = ctypes.CDLL(str(build()))
        P = ctypes.c_void_p
        i32p = np.ctypeslib.ndpointer(np.int32, flags='C')
        u32p = np.ctypeslib.ndpointer(np.uint32, flags='C')
        l.sno_create.restype = P
        l.sno_create.argtypes = [ctypes.c_uint32, i32p, i32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]
        l.sno_destroy.argtypes = [P]
        l.sno_set_nbr_cut.argtypes = [P, ctypes.c_int]
        l.sno_load_scene.restype = ctypes.c_int
        l.sno_load_scene.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32, i32p, i32p, u32p,
                                     P, P, P, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint32]
        l.sno_step.restype = ctypes.c_int
        l.sno_step.argtypes = [P, ctypes.c_uint32]
        for f in ('sno_digest', 'sno_chain', 'sno_dbg'):
            getattr(l, f).argtypes = [P, u32p]
        l.sno_reset_chain.argtypes = [P]
        for f in ('sno_n', 'sno_nfluid'):
            getattr(l, f).restype = ctypes.c_uint32
            getattr(l, f).argtypes = [P]
        for f in ('sno_substeps', 'sno_formation_clock'):
            getattr(l, f).restype = ctypes.c_uint64
            getattr(l, f).argtypes = [P]
        l.sno_read_state.restype = ctypes.c_int
        l.sno_read_state.argtypes = [P, i32p, ctypes.c_size_t]
        l.sno_read_derived.restype = ctypes.c_int
        l.sno_read_derived.argtypes = [P, i32p, ctypes.c_size_t]
        l.sno_read_bonds.restype = ctypes.c_int
        l.sno_read_bonds.argtypes = [P, u32p, ctypes.c_size_t]
        l.sno_write_state.restype = ctypes.c_int
        l.sno_write_state.argtypes = [P, i32p, P]
        l.sno_set_formation_clock.argtypes = [P, ctypes.c_uint64, ctypes.c_int]
        l.sno_spawn.restype = ctypes.c_int64
        l.sno_spawn.argtypes = [P, i32p, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        l.sno_set_walls.restype = ctypes.c_int
        l.sno_set_walls.argtypes = [P, ctypes.c_int]
        l.sno_hold_weld_group.restype = ctypes.c_int
        l.sno_hold_weld_group.argtypes = [P, ctypes.c_uint32]
        l.sno_end_weld_group.restype = ctypes.c_uint32
        l.sno_end_weld_group.argtypes = [P]
        l.sno_begin_weld_group.restype = ctypes.c_uint32
        l.sno_begin_weld_group.argtypes = [P]
        l.sno_arm_fuse.restype = ctypes.c_int
        l.sno_arm_fuse.argtypes = [P]
        l.sno_weld_state.argtypes = [P, u32p]
        for f in ('sno_read_nbr_counts', 'sno_read_cell_start'):
            getattr(l, f).restype = ctypes.c_int
            getattr(l, f).argtypes = [P, u32p, ctypes.c_size_t]
        l.sno_write_bonds.restype = ctypes.c_int
        l.sno_write_bonds.argtypes = [P, u32p, ctypes.c_size_t]
        l.sno_erase.restype = ctypes.c_int64
        l.sno_erase.argtypes = [P, np.ctypeslib.ndpointer(np.uint8, flags='C')]
        l.sno_set_jets.restype = ctypes.c_uint32
        l.sno_set_jets.argtypes = [P, i32p, ctypes.c_uint32]
        for f in ('sno_make_rigid_body',):
            getattr(l, f).restype = ctypes.c_int32
            getattr(l, f).argtypes = [P, u32p, ctypes.c_uint32, P, ctypes.c_int]
        l.sno_promote_weld_group.restype = ctypes.c_int32
        l.sno_promote_weld_group.argtypes = [P, ctypes.c_uint32, P, ctypes.c_int]
        l.sno_end_weld_group_and_promote.restype = ctypes.c_int32
        l.sno_end_weld_group_and_promote.argtypes = [P, P, ctypes.c_int]
        for f in ('sno_dissolve_all_bodies', 'sno_body_count'):
            getattr(l, f).restype = ctypes.c_uint32
            getattr(l, f).argtypes = [P]
        for f in ('sno_read_bodies', 'sno_read_rest'):
            getattr(l, f).restype = ctypes.c_int
            getattr(l, f).argtypes = [P, i32p, ctypes.c_size_t]
        l.sno_set_body_user.restype = ctypes.c_int
        l.sno_set_body_user.argtypes = [P, ctypes.c_uint32, ctypes.c_int]
        l.sno_set_body_driver.restype = ctypes.c_int
        l.sno_set_body_driver.argtypes = [P, ctypes.c_uint32, ctypes.c_int32, i32p]
        l.sno_clear_body_drivers.restype = ctypes.c_int
        l.sno_clear_body_drivers.argtypes = [P]
        l.sno_set_user_drive.restype = ctypes.c_int32
        l.sno_set_user_drive.argtypes = [P, ctypes.c_int32, ctypes.c_int32]
        l.sno_drag_body.restype = ctypes.c_int
        l.sno_drag_body.argtypes = [P, ctypes.c_uint32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.c_int32]
        l.sno_write_body.restype = ctypes.c_int32
        l.sno_write_body.argtypes = [P, u32p, ctypes.c_uint32, ctypes.c_uint32, P, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_uint32)]
        l.sno_set_material.restype = ctypes.c_int
        l.sno_set_material.argtypes = [P, ctypes.c_uint32, i32p]
        l.sno_clear_materials.argtypes = [P]
        l.sno_set_gravity_scale.restype = ctypes.c_int32
        l.sno_set_gravity_scale.argtypes = [P, ctypes.c_int32]
        l.sno_mat_count.restype = ctypes.c_uint32
        l.sno_mat_count.argtypes = [P]
        l.sno_restore_bodies.restype = ctypes.c_int
        l.sno_restore_bodies.argtypes = [P, i32p, ctypes.c_uint32, P, ctypes.c_size_t]
        l.sno_impulse.restype = ctypes.c_int64
        l.sno_impulse.argtypes = [P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_int32, ctypes.c_uint32]
        l.sno3_create.restype = P
        l.sno3_create.argtypes = [ctypes.c_uint32, i32p, ctypes.c_uint32, i32p, ctypes.c_uint32, ctypes.c_uint32,
                                  ctypes.c_int]
        l.sno3_destroy.argtypes = [P]
        l.sno3_load.restype = ctypes.c_int
        l.sno3_load.argtypes = [P, ctypes.c_uint32, i32p, i32p, u32p, ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint32]
        l.sno3_write_state.restype = ctypes.c_int
        l.sno3_write_state.argtypes = [P, i32p, ctypes.c_uint32, ctypes.c_uint64, P]
        l.sno3_step.restype = ctypes.c_int
        l.sno3_step.argtypes = [P, ctypes.c_uint32]
        l.sno3_write_bonds.restype = ctypes.c_int
        l.sno3_write_bonds.argtypes = [P, u32p, ctypes.c_size_t, ctypes.c_int32, ctypes.c_int32]
        l.sno3_read_bonds.restype = ctypes.c_int
        l.sno3_read_bonds.argtypes = [P, u32p, ctypes.c_size_t]
        for f in ('sno3_fnv', 'sno3_digest', 'sno3_chain', 'sno3_dbg'):
            getattr(l, f).argtypes = [P, u32p]
        l.sno3_read_state.restype = ctypes.c_int
        l.sno3_read_state.argtypes = [P, i32p, ctypes.c_size_t]
        l.sno3_spawn.restype = ctypes.c_uint32
        l.sno3_spawn.argtypes = [P, i32p, u32p, ctypes.c_uint32]
        l.sno3_set_ball.argtypes = [P, ctypes.c_int, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    i32p, i32p]
        l.sno3_n.restype = ctypes.c_uint32
        l.sno3_n.argtypes = [P]
        l.sno3_substeps.restype = ctypes.c_uint64
        l.sno3_substeps.argtypes = [P]
        _lib = l
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def hex8(words) -> str:
    return ''.join(f'{int(w) & 0xffffffff:08x}' for w in words)


class OracleEngine:
    """CPU reference engine: ``createEngine`` + ``Engine`` semantics on the host."""

    def __init__(self, max_particles: int = 8192, iters: int = 4, threads: int = 1,
                 luts=None, mats=None):
        from sunaengine_gb300 import data
        l = lib()
        self._luts = np.ascontiguousarray(data.luts() if luts is None else luts, dtype=np.int32)
        m = data.mats() if mats is None else mats
        self._mats = np.ascontiguousarray(m, dtype=np.int32).reshape(-1)
        self.mat_count = self._mats.size // 48
        self.h = l.sno_create(max_particles, self._luts, self._mats, self.mat_count, iters, threads)
        self._mats_rows = self._mats.reshape(-1, 48)
        if not self.h:
            raise ValueError('oracle create failed')
        self.max_particles = max_particles

    def close(self):
        if self.h:
            lib().sno_destroy(self.h)
            self.h = None

    __del__ = close

    def load_scene(self, sc):
        self._keep = []

        def arr(a, dt):
            if a is None:
                return None
            b = np.ascontiguousarray(a, dtype=dt)
            self._keep.append(b)
            return b
        pos = arr(sc.pos.reshape(-1), np.int32)
        vel = arr(sc.vel.reshape(-1), np.int32)
        mat = arr(sc.matId, np.uint32)
        rc = lib().sno_load_scene(self.h, sc.n, sc.nFluid, pos, vel, mat,
                                  _ptr(arr(sc.flags, np.uint32)), _ptr(arr(sc.temp, np.int32)),
                                  _ptr(arr(sc.fuel, np.int32)), int(sc.domW), int(sc.domH), int(sc.cellShift))
        if rc != 0:
            raise ValueError(f'oracle loadScene refused the scene (code {rc})')
        return self

    def step(self, count: int = 1):
        rc = lib().sno_step(self.h, count)
        if rc != 0:
            raise RuntimeError(f'oracle step failed (code {rc})')
        return self.substep_count

    @property
    def n(self):
        return lib().sno_n(self.h)

    @property
    def n_fluid(self):
        return lib().sno_nfluid(self.h)

    @property
    def substep_count(self):
        return lib().sno_substeps(self.h)

    @property
    def formation_clock(self):
        return lib().sno_formation_clock(self.h)

    def digest_words(self):
        a = np.zeros(8, np.uint32)
        lib().sno_digest(self.h, a)
        return a

    def digest(self) -> str:
        return hex8(self.digest_words())

    def chain_words(self):
        a = np.zeros(8, np.uint32)
        lib().sno_chain(self.h, a)
        return a

    def chain_hex(self) -> str:
        return hex8(self.chain_words())

    def reset_chain(self):
        lib().sno_reset_chain(self.h)

    def debug_counters(self):
        a = np.zeros(16, np.uint32)
        lib().sno_dbg(self.h, a)
        return a

    def read_state(self):
        a = np.zeros(self.n * 8, np.int32)
        lib().sno_read_state(self.h, a, a.size)
        return a

    def read_derived(self):
        a = np.zeros(self.n * 16, np.int32)
        lib().sno_read_derived(self.h, a, a.size)
        return a

    def set_nbr_cut(self, on: bool = True):
        """Stop a full neighbour list's scan when no flag bit can change (only
        the overflow debug counter then differs from the full scan)."""
        lib().sno_set_nbr_cut(self.h, 1 if on else 0)
        return self

    def read_nbr_counts(self):
        a = np.zeros(max(1, self.n), np.uint32)
        lib().sno_read_nbr_counts(self.h, a, a.size)
        return a[:self.n]

    def read_cell_start(self, cell_total: int):
        a = np.zeros(cell_total + 1, np.uint32)
        if lib().sno_read_cell_start(self.h, a, a.size) != 0:
            raise ValueError('oracle read_cell_start: wrong size')
        return a

    def read_bonds(self):
        a = np.zeros(self.n_fluid * 48, np.uint32)
        lib().sno_read_bonds(self.h, a, a.size)
        return a

    def write_state(self, state, derived=None):
        st = np.ascontiguousarray(state, dtype=np.int32)
        dv = None if derived is None else np.ascontiguousarray(derived, dtype=np.int32)
        lib().sno_write_state(self.h, st, _ptr(dv))
        self._keep2 = dv

    def set_formation_clock(self, clk: int, dirty: bool):
        lib().sno_set_formation_clock(self.h, clk, 1 if dirty else 0)

    def begin_weld_group(self) -> int:
        return int(lib().sno_begin_weld_group(self.h))

    def hold_weld_group(self, tag: int) -> int:
        r = lib().sno_hold_weld_group(self.h, int(tag))
        if r < 0:
            raise ValueError('holdWeldGroup(0): use endWeldGroup() to release')
        return r

    def end_weld_group(self) -> int:
        return int(lib().sno_end_weld_group(self.h))

    def arm_fuse(self) -> int:
        r = lib().sno_arm_fuse(self.h)
        if r < 0:
            raise ValueError('armFuse(): no weld group is open')
        return r

    def weld_state(self):
        a = np.zeros(4, np.uint32)
        lib().sno_weld_state(self.h, a)
        return dict(zip(('weld_hold', 'fuse_tag', 'last_weld_tag', 'weld_seq'), (int(x) for x in a)))

    def spawn(self, particles, no_weld: bool = True, own_group: bool = False) -> int:
        rows = np.zeros((len(particles), 8), np.int32)
        has_t = any('temp' in p for p in particles)
        has_f = any('fuel' in p for p in particles)
        for k, p in enumerate(particles):
            rows[k] = (p['x'], p['y'], p.get('vx', 0), p.get('vy', 0), p.get('mat', 0),
                       p.get('flags', 0), p.get('temp', 0), p.get('fuel', 0))
        r = lib().sno_spawn(self.h, rows.reshape(-1), len(particles), int(has_t), int(has_f),
                            (1 if no_weld else 0) | (2 if own_group else 0))
        if r < 0:
            raise ValueError(f'oracle spawn refused (code {r})')
        return int(r)

    def impulse(self, cx, cy, r, ix, iy, limit=3000) -> int:
        return int(lib().sno_impulse(self.h, cx, cy, r, ix, iy, limit))

    def write_state_keep_scratch(self, state):
        self.write_state(state)  # derived rows (stAcc included) untouched

    def write_bonds(self, bonds):
        b = np.ascontiguousarray(bonds, dtype=np.uint32).reshape(-1)
        if lib().sno_write_bonds(self.h, b, b.size) != 0:
            raise ValueError('oracle write_bonds: wrong size')

    def erase(self, keep) -> int:
        k = np.ascontiguousarray(np.asarray(keep, dtype=bool).astype(np.uint8))
        if k.size != self.n_fluid:
            raise ValueError('erase: one keep flag per fluid slot')
        return int(lib().sno_erase(self.h, k))

    def set_jets(self, jets) -> int:
        q = np.array([[j['x'], j['y'], j['r'], j.get('fx', 0), j.get('fy', 0)] for j in jets] or np.zeros((0, 5)),
                     dtype=np.int32).reshape(-1)
        q = np.ascontiguousarray(q if q.size else np.zeros(5, np.int32))
        return int(lib().sno_set_jets(self.h, q, len(jets)))

    def set_walls(self, on: bool) -> bool:
        return bool(lib().sno_set_walls(self.h, 1 if on else 0))

    # §20 rigid bodies (src/engine.js:5452-5811)
    @staticmethod
    def _pivot(pivot):
        if pivot is None:
            return None, None
        a = np.ascontiguousarray([int(pivot[0]), int(pivot[1])], dtype=np.int32)
        return a, a.ctypes.data_as(ctypes.c_void_p)

    def make_rigid_body(self, slots, pivot=None, user: bool = False):
        s = np.ascontiguousarray(np.asarray(slots, dtype=np.int64).clip(0, 2**32 - 1).astype(np.uint32))
        keep, pp = self._pivot(pivot)
        r = lib().sno_make_rigid_body(self.h, s if s.size else np.zeros(1, np.uint32), s.size, pp, int(bool(user)))
        if r == -2:
            raise ValueError('[aether] §20: no free weld tag for a new body')
        return None if r < 0 else int(r)

    # runtime material rows (src/engine.js:4843-4855, 5115-5245)
    def set_material(self, row: int, words) -> int:
        w = np.ascontiguousarray(np.asarray(words, dtype=np.int64).reshape(48).astype(np.int32))
        r = lib().sno_set_material(self.h, int(row), w)
        if r < 0:
            raise ValueError(f'set_material refused (code {r})')
        return int(r)

    def clear_materials(self):
        lib().sno_clear_materials(self.h)

    def set_gravity_scale(self, q: int) -> int:
        return int(lib().sno_set_gravity_scale(self.h, int(q)))

    def write_body(self, members, tag: int = 0, pivot=None, user: bool = False):
        s = np.ascontiguousarray(np.asarray(members, dtype=np.int64).reshape(-1).astype(np.uint32))
        keep, pp = self._pivot(pivot)
        t = ctypes.c_uint32()
        r = lib().sno_write_body(self.h, s if s.size else np.zeros(1, np.uint32), s.size, int(tag), pp,
                                 int(bool(user)), ctypes.byref(t))
        if r == -3:
            raise ValueError('body member outside the fluid slots')
        return (None if r < 0 else int(r)), int(t.value)

    def make_axis_body(self, slots, px: int, py: int, user: bool = False):
        return self.make_rigid_body(slots, (px, py), user)

    def promote_weld_group(self, tag: int = 0, pivot=None, user: bool = False):
        keep, pp = self._pivot(pivot)
        r = lib().sno_promote_weld_group(self.h, int(tag), pp, int(bool(user)))
        return None if r < 0 else int(r)

    def end_weld_group_and_promote(self, pivot=None, user: bool = False):
        keep, pp = self._pivot(pivot)
        r = lib().sno_end_weld_group_and_promote(self.h, pp, int(bool(user)))
        return None if r < 0 else int(r)

    def dissolve_all_bodies(self) -> int:
        return int(lib().sno_dissolve_all_bodies(self.h))

    @property
    def body_count(self) -> int:
        return int(lib().sno_body_count(self.h))

    def read_bodies(self) -> np.ndarray:
        a = np.zeros(max(1, self.body_count) * 32, np.int32)
        lib().sno_read_bodies(self.h, a, a.size)
        return a[:self.body_count * 32].reshape(-1, 32)

    def read_rest_offsets(self) -> np.ndarray:
        a = np.zeros(max(1, self.n) * 2, np.int32)
        lib().sno_read_rest(self.h, a, a.size)
        return a[:self.n * 2]

    def set_body_user(self, index: int, on: bool) -> bool:
        return bool(lib().sno_set_body_user(self.h, int(index), int(bool(on))))

    def set_body_driver(self, index: int, mask: int, values):
        v = np.zeros(9, np.int32)
        v[:len(values)] = np.asarray(values, dtype=np.int64).clip(-2**31, 2**31 - 1)
        if lib().sno_set_body_driver(self.h, int(index), int(mask), v) != 0:
            raise ValueError('body driver: no such body or bad mask')

    def clear_body_drivers(self):
        lib().sno_clear_body_drivers(self.h)

    def set_user_drive(self, ax: int, ay: int):
        lib().sno_set_user_drive(self.h, int(ax), int(ay))

    def drag_body(self, tag: int, tx: int, ty: int, vx: int = 0, vy: int = 0) -> int:
        return int(lib().sno_drag_body(self.h, int(tag), int(tx), int(ty), int(vx), int(vy)))

    def restore_bodies(self, records, rest=None):
        r = np.ascontiguousarray(np.asarray(records, dtype=np.int32).reshape(-1))
        nb = r.size // 32
        rr = None if rest is None else np.ascontiguousarray(np.asarray(rest, dtype=np.int32).reshape(-1))
        if lib().sno_restore_bodies(self.h, r if r.size else np.zeros(32, np.int32), nb,
                                    None if rr is None else rr.ctypes.data_as(ctypes.c_void_p),
                                    0 if rr is None else rr.size) != 0:
            raise ValueError('restore_bodies: bad sizes')

    # the Engine method names, so the demo layer can drive either engine
    def spawn_fluid(self, particles, no_weld: bool = True, own_group: bool = False) -> int:
        return self.spawn(particles, no_weld, own_group)

    def apply_impulse(self, cx, cy, r, ix, iy, limit=3000) -> int:
        return self.impulse(cx, cy, r, ix, iy, limit)

    def read_scratch(self):
        d = self.read_derived().reshape(-1, 16)
        return np.ascontiguousarray(d[:, 8:10]).reshape(-1)

    def write_scratch_state(self, state, scratch):
        der = np.zeros((self.n, 16), np.int32)
        st = np.asarray(state, dtype=np.int32).reshape(-1, 8)
        der[:, 0:2] = st[:, 0:2]
        if scratch is not None:
            der[:, 8:10] = np.asarray(scratch, dtype=np.int32).reshape(-1, 2)
        self.write_state(st.reshape(-1), der.reshape(-1))

    def digest_hex(self) -> str:
        return self.digest()


class Oracle3D:
    """CPU reference of the 3D solver (3d/sim3d.wgsl driven as 3d/app.js drives it)."""

    def __init__(self, max_particles: int = 65536, iters: int = 3, threads: int = 1):
        from sunaengine_gb300 import tables3d
        l = lib()
        self._luts = np.ascontiguousarray(tables3d.luts3d(), dtype=np.int32)
        self._mats = np.ascontiguousarray(tables3d.mats3d().reshape(-1), dtype=np.int32)
        self.h = l.sno3_create(max_particles, self._luts, self._luts.size, self._mats, self._mats.size // 4,
                               iters, threads)
        self.max_particles = max_particles

    def close(self):
        if self.h:
            lib().sno3_destroy(self.h)
            self.h = None

    __del__ = close

    def load_scene(self, sc, stir_amp: int = 0, frame: int = 0):
        pos = np.ascontiguousarray(sc.pos.reshape(-1), dtype=np.int32)
        vel = np.ascontiguousarray(sc.vel.reshape(-1), dtype=np.int32)
        mat = np.ascontiguousarray(sc.mat, dtype=np.uint32)
        rc = lib().sno3_load(self.h, sc.n, pos, vel, mat, sc.gx, sc.gy, sc.gz, stir_amp, frame)
        if rc != 0:
            raise ValueError(f'oracle 3D load refused the scene (code {rc})')
        return self

    def step(self, count: int = 1):
        lib().sno3_step(self.h, count)
        return self.substep_count

    @property
    def n(self):
        return lib().sno3_n(self.h)

    @property
    def substep_count(self):
        return lib().sno3_substeps(self.h)

    def _words(self, f):
        a = np.zeros(8 if f != 'sno3_dbg' else 16, np.uint32)
        getattr(lib(), f)(self.h, a)
        return a

    def write_bonds(self, rows, stiffness: int, break_ratio: int):
        """Build-defined 3D bonds (sno3_write_bonds): n * 12 words of rows."""
        a = np.ascontiguousarray(np.asarray(rows, np.uint32).reshape(-1))
        if lib().sno3_write_bonds(self.h, a, a.size, int(stiffness), int(break_ratio)) != 0:
            raise ValueError('oracle 3D write_bonds: malformed rows')
        return self

    def read_bonds(self):
        a = np.zeros(max(1, self.n * 12), np.uint32)
        lib().sno3_read_bonds(self.h, a, a.size)
        return a[:self.n * 12]

    def fnv_hex(self) -> str:
        return hex8(self._words('sno3_fnv'))

    def digest(self) -> str:
        return hex8(self._words('sno3_digest'))

    def chain_hex(self) -> str:
        return hex8(self._words('sno3_chain'))

    def debug_counters(self):
        return self._words('sno3_dbg')

    def read_state(self):
        a = np.zeros(self.n * 8, np.int32)
        lib().sno3_read_state(self.h, a, a.size)
        return a

    def write_state(self, state, substeps: int, chain_words=None):
        st = np.ascontiguousarray(np.asarray(state).reshape(-1), dtype=np.int32)
        ch = None if chain_words is None else np.ascontiguousarray(chain_words, dtype=np.uint32)
        self._ch = ch
        if lib().sno3_write_state(self.h, st, st.size // 8, int(substeps), _ptr(ch)) != 0:
            raise ValueError('oracle 3D write_state refused')

    def chain_words(self):
        return self._words('sno3_chain')

    def spawn(self, pos, mat) -> int:
        pos = np.ascontiguousarray(np.asarray(pos).reshape(-1), dtype=np.int32)
        mat = np.ascontiguousarray(mat, dtype=np.uint32)
        return int(lib().sno3_spawn(self.h, pos, mat, mat.size))

    def set_ball(self, on: bool, x: int = 0, y: int = 0, z: int = 0, radius_wu: float = 3.0):
        from sunaengine_gb300 import tables3d
        w, g = tables3d.ball_tables(radius_wu)
        reach = tables3d.js_round((radius_wu + tables3d.H_WU) * tables3d.ONE)
        self._ball = (w, g)
        lib().sno3_set_ball(self.h, int(on), x, y, z, reach, w, g)
