"""The engine surface of the reference's ``src/engine.js``, on the GB300 C ABI.

``create_engine`` / ``Engine`` mirror ``createEngine`` (``src/engine.js:2786``)
and ``class Engine`` (``src/engine.js:3523``): same method names (camelCase
aliases included), same argument meaning, same error behaviour (bad input
raises ``EngineError`` synchronously, the reference's ``assert``; device-side
problems surface from ``check_errors()``). Every call goes through
``include/suna.h``; there is no CPU path.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Iterable, Optional

import numpy as np

from . import _native, data
from .scenes import Scene

SUBSTEPS_PER_FRAME = 2
ITERS = 4
MAXNBR = 48
BOND_CAP = 48
VMAX = 65536


def authoring_kerf() -> int:
    """sliceBondsMany's default kerf, Math.round(ONE * 0.52) (src/engine.js:6240)."""
    return 34079


class EngineError(RuntimeError):
    """Raised for refused input and for errors the device reported."""


@dataclass
class Digest:
    acc: np.ndarray

    @property
    def hex(self) -> str:
        return ''.join(f'{int(a):08x}' for a in self.acc)

    @property
    def set_hex(self) -> str:
        return self.hex[:32]

    @property
    def slot_hex(self) -> str:
        return self.hex[32:]

    setHex = set_hex
    slotHex = slot_hex


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _out_words(out: Optional[np.ndarray], words: int) -> np.ndarray:
    """A fresh int32 array of `words`, or the first `words` of a caller's buffer."""
    if out is None:
        return np.empty(words, np.int32)
    if not isinstance(out, np.ndarray) or out.dtype != np.int32 or out.ndim != 1 or \
            not out.flags.c_contiguous or not out.flags.writeable or out.size < words:
        raise EngineError(f'[aether] read_state: out must be a writeable contiguous 1-D int32 array of at least '
                          f'{words} words')
    return out[:words]


def _opts(max_particles, max_cells, iters, debug, chain, device, luts, mats, lanes=0):
    luts = np.ascontiguousarray(data.luts() if luts is None else luts, dtype=np.int32)
    if luts.size != data.LUT_WORDS or data.table_hash(luts) != data.TABLE_HASH:
        raise EngineError('kernel tables do not match the frozen TABLE_HASH')
    mats = np.ascontiguousarray(data.mats() if mats is None else mats, dtype=np.int32).reshape(-1, 48)
    o = _native.SnOpts(max_particles=int(max_particles), max_cells=int(max_cells), iters=int(iters),
                       debug=1 if debug else 0, chain=1 if chain else 0, device=int(device),
                       luts=luts.ctypes.data, mats=mats.ctypes.data, mat_count=mats.shape[0],
                       lanes=int(lanes))
    return o, (luts, mats)


class _SceneArgs:
    """Keeps the numpy arrays alive for the duration of a C call."""

    def __init__(self, sc: Scene):
        n = int(sc.n)
        self.pos = np.ascontiguousarray(np.asarray(sc.pos).reshape(-1), dtype=np.int32)
        self.vel = np.ascontiguousarray(np.asarray(sc.vel).reshape(-1), dtype=np.int32)
        self.mat = np.ascontiguousarray(np.asarray(sc.matId).reshape(-1), dtype=np.uint32)
        if self.pos.size != 2 * n or self.vel.size != 2 * n or self.mat.size != n:
            raise EngineError('scene array lengths must be n*2 / n*2 / n')
        conv = lambda a, dt: None if a is None else np.ascontiguousarray(np.asarray(a).reshape(-1), dtype=dt)
        self.flags = conv(sc.flags, np.uint32)
        self.temp = conv(sc.temp, np.int32)
        self.fuel = conv(sc.fuel, np.int32)
        self.c = _native.SnScene(n=n, n_fluid=int(sc.nFluid), pos=_ptr(self.pos), vel=_ptr(self.vel),
                                 mat_id=_ptr(self.mat), flags=_ptr(self.flags), temp=_ptr(self.temp),
                                 fuel=_ptr(self.fuel), dom_w=int(sc.domW), dom_h=int(sc.domH),
                                 cell_shift=int(sc.cellShift))


def _particles(lst: Iterable[dict]):
    lst = list(lst)
    arr = (_native.SnParticle * max(1, len(lst)))()
    for k, p in enumerate(lst):
        arr[k].x = int(p['x'])
        arr[k].y = int(p['y'])
        arr[k].vx = int(p.get('vx', 0))
        arr[k].vy = int(p.get('vy', 0))
        arr[k].mat = int(p.get('mat', 0))
        arr[k].flags = int(p.get('flags', 0))
        arr[k].has_temp = 1 if p.get('temp') is not None else 0
        arr[k].temp = int(p.get('temp') or 0)
        arr[k].has_fuel = 1 if p.get('fuel') is not None else 0
        arr[k].fuel = int(p.get('fuel') or 0)
    return arr, len(lst)


class Engine:
    """One scene on one GB300 (``class Engine``, ``src/engine.js:3523``)."""

    def __init__(self, max_particles: int = 8192, max_cells: int = 0, iters: int = ITERS, debug: bool = False,
                 chain: bool = True, device: int = 0, tables=None, mats=None, lanes: int = 0):
        self._lib = _native.load()
        o, self._keep = _opts(max_particles, max_cells, iters, debug, chain, device, tables, mats, lanes)
        self._mats_rows = self._keep[1]
        h = ctypes.c_void_p()
        rc = self._lib.sn_create(ctypes.byref(o), ctypes.byref(h))
        if rc != 0:
            raise EngineError(f'sn_create failed ({rc})')
        self._h = h
        self.max_particles = int(max_particles)
        self.iters = int(iters)
        self.debug = bool(debug)
        self.chain_enabled = bool(chain)
        self.mat_count = self._keep[1].shape[0]
        self._n = 0
        self._n_fluid = 0
        self._substeps = 0
        self._scene: Optional[Scene] = None
        self._loaded_n = 0

    # -- plumbing ------------------------------------------------------------------
    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self._lib.sn_last_error(self._h)
            raise EngineError(f'[aether] {what}: {msg.decode() if msg else rc}')

    def destroy(self):
        if getattr(self, '_h', None):
            self._lib.sn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    # -- engine.js surface -----------------------------------------------------------
    def load_scene(self, scene: Scene) -> 'Engine':
        args = _SceneArgs(scene)
        self._check(self._lib.sn_load_scene(self._h, ctypes.byref(args.c)), 'loadScene')
        self._n, self._n_fluid = int(scene.n), int(scene.nFluid)
        self._substeps = 0
        self._scene = scene
        self._loaded_n = int(scene.n)
        return self

    def step(self, count: int = 1) -> int:
        if not isinstance(count, (int, np.integer)) or count < 0:
            raise EngineError('[aether] step(count) needs a non-negative integer')
        out = ctypes.c_uint64()
        self._check(self._lib.sn_step(self._h, int(count), ctypes.byref(out)), 'step')
        self._substeps = int(out.value)
        return self._substeps

    def frame(self) -> int:
        return self.step(SUBSTEPS_PER_FRAME)

    def digest(self) -> Digest:
        a = np.zeros(8, np.uint32)
        self._check(self._lib.sn_digest(self._h, _ptr(a)), 'digest')
        return Digest(a)

    def chain_words(self) -> np.ndarray:
        a = np.zeros(8, np.uint32)
        self._check(self._lib.sn_chain(self._h, _ptr(a)), 'chain')
        return a

    def chain_hex(self) -> str:
        return ''.join(f'{int(x):08x}' for x in self.chain_words())

    def reset_chain(self):
        self._check(self._lib.sn_reset_chain(self._h), 'resetChain')

    def read_state(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """readState: the scene's state words (8 per slot). `out`, when given, is
        a caller-owned contiguous int32 array of at least n * 8 words that
        receives them (and is returned), so repeated reads reuse one buffer."""
        a = _out_words(out, self.n * 8)
        self._check(self._lib.sn_read_state(self._h, _ptr(a), a.size), 'readState')
        return a

    def read_scratch(self) -> np.ndarray:
        a = np.zeros(self.n * 2, np.int32)
        self._check(self._lib.sn_read_scratch(self._h, _ptr(a), a.size), 'readScratch')
        return a

    def write_state(self, state: np.ndarray, scratch: Optional[np.ndarray] = None):
        st = np.ascontiguousarray(state, dtype=np.int32).reshape(-1)
        sc = None if scratch is None else np.ascontiguousarray(scratch, dtype=np.int32).reshape(-1)
        if st.size != self.n * 8 or (sc is not None and sc.size != self.n * 2):
            raise EngineError('[aether] write_state: wrong buffer size')
        self._check(self._lib.sn_write_state(self._h, _ptr(st), _ptr(sc), self.n), 'writeState')

    def read_fields(self):
        """(rho, nbr_count) of the last substep per slot: readDerived's rho
        column and readNbrN's counts (src/engine.js:4290-4291)."""
        rho = np.zeros(max(1, self.n), np.int32)
        nbr = np.zeros(max(1, self.n), np.uint32)
        self._check(self._lib.sn_read_fields(self._h, _ptr(rho), _ptr(nbr), rho.size), 'readDerived')
        return rho[:self.n], nbr[:self.n]

    def read_cell_start(self) -> np.ndarray:
        """readCellStart (src/engine.js:4292): cell_total + 1 words (colour-major keys)."""
        a = np.zeros(self.info()['cell_total'] + 1, np.uint32)
        self._check(self._lib.sn_read_cell_start(self._h, _ptr(a), a.size), 'readCellStart')
        return a

    def liveness(self, window: int = 0) -> dict:
        """Engine.liveness (src/engine.js:4490-4511). With window > 0 the
        positions are snapshotted and the simulation ADVANCES `window`
        substeps, so movement over that recent interval is measured too."""
        from .liveness import compute_liveness
        recent = None
        if window > 0:
            before = self.read_state().reshape(-1, 8)
            recent = np.ascontiguousarray(before[:self.n_fluid, :2]).reshape(-1)
            self.step(window)
        st = self.read_state()
        rho, nbr = self.read_fields()
        cs = self.read_cell_start()
        sc = self._scene
        return compute_liveness(st, self.n, self.n_fluid, int(sc.domW), int(sc.domH), rho=rho, nbr_count=nbr,
                                cell_start=cs, initial_pos=self.read_initial_positions(), recent_pos=recent)

    def read_initial_positions(self) -> np.ndarray:
        """The positions the last load_scene loaded (the reference engine's
        _initialPos, src/engine.js:3947), 2 words per particle of that load."""
        a = np.empty(max(1, self._loaded_n) * 2, np.int32)
        got = ctypes.c_size_t()
        self._check(self._lib.sn_read_initial_positions(self._h, _ptr(a), a.size, ctypes.byref(got)),
                    'readInitialPositions')
        return a[:int(got.value)]

    def read_bonds(self) -> np.ndarray:
        a = np.zeros(max(1, self.n_fluid * BOND_CAP), np.uint32)
        self._check(self._lib.sn_read_bonds(self._h, _ptr(a), a.size), 'readBond')
        return a[:self.n_fluid * BOND_CAP]

    # weld groups (src/engine.js:4570-4680)
    def begin_weld_group(self) -> int:
        t = ctypes.c_uint32()
        self._check(self._lib.sn_begin_weld_group(self._h, ctypes.byref(t)), 'beginWeldGroup')
        return int(t.value)

    def hold_weld_group(self, tag: int) -> int:
        self._check(self._lib.sn_hold_weld_group(self._h, int(tag)), 'holdWeldGroup')
        return int(tag) & 0x000fff00

    def end_weld_group(self) -> int:
        t = ctypes.c_uint32()
        self._check(self._lib.sn_end_weld_group(self._h, ctypes.byref(t)), 'endWeldGroup')
        return int(t.value)

    def arm_fuse(self) -> int:
        t = ctypes.c_uint32()
        self._check(self._lib.sn_arm_fuse(self._h, ctypes.byref(t)), 'armFuse')
        return int(t.value)

    def weld_state(self):
        a = np.zeros(4, np.uint32)
        self._check(self._lib.sn_weld_state(self._h, _ptr(a)), 'weldState')
        return dict(zip(('weld_hold', 'fuse_tag', 'last_weld_tag', 'weld_seq'), (int(x) for x in a)))

    beginWeldGroup = begin_weld_group
    holdWeldGroup = hold_weld_group
    endWeldGroup = end_weld_group
    armFuse = arm_fuse

    def write_bonds(self, bonds: np.ndarray):
        b = np.ascontiguousarray(bonds, dtype=np.uint32).reshape(-1)
        self._check(self._lib.sn_write_bonds(self._h, _ptr(b), b.size), 'writeBonds')

    def write_state_keep_scratch(self, state: np.ndarray):
        self.write_state(state, self.read_scratch())

    def erase(self, keep) -> int:
        """The device compaction of eraseWhere: keep one flag per fluid slot."""
        k = np.ascontiguousarray(np.asarray(keep, dtype=bool).astype(np.uint8))
        out = ctypes.c_uint32()
        self._check(self._lib.sn_erase(self._h, _ptr(k), k.size, ctypes.byref(out)), 'eraseWhere')
        i = self.info()
        self._n, self._n_fluid = int(i['n']), int(i['n_fluid'])
        return int(out.value)

    # authoring edits, same host logic as the reference (see authoring.py)
    def erase_where(self, keep) -> int:
        from . import authoring
        return authoring.erase_where(self, keep)

    def replace_where(self, test, new_mat: int) -> int:
        from . import authoring
        return authoring.replace_where(self, test, new_mat)

    def slice_bonds_many(self, segments, kerf: int = authoring_kerf()) -> int:
        from . import authoring
        return authoring.slice_bonds_many(self, segments, kerf)

    def slice_bonds(self, x0: int, y0: int, x1: int, y1: int) -> int:
        return self.slice_bonds_many([{'x0': x0, 'y0': y0, 'x1': x1, 'y1': y1}])

    eraseWhere = erase_where
    replaceWhere = replace_where
    sliceBondsMany = slice_bonds_many
    sliceBonds = slice_bonds

    def spawn_fluid(self, particles, no_weld: bool = True, own_group: bool = False) -> int:
        arr, k = _particles(particles)
        out = ctypes.c_uint32()
        opts = (1 if no_weld else 0) | (2 if own_group else 0)
        self._check(self._lib.sn_spawn(self._h, arr, k, opts, ctypes.byref(out)), 'spawnFluid')
        n = int(out.value)
        if n != self._n:
            self._n_fluid += n - self._n
            self._n = n
        return n

    def apply_impulse(self, cx: int, cy: int, radius: int, ix: int, iy: int, limit: int = 3000) -> int:
        out = ctypes.c_uint32()
        self._check(self._lib.sn_impulse(self._h, int(cx), int(cy), int(radius), int(ix), int(iy), int(limit),
                                         ctypes.byref(out)), 'applyImpulse')
        return int(out.value)

    def debug_counters(self) -> np.ndarray:
        a = np.zeros(16, np.uint32)
        self._check(self._lib.sn_debug_counters(self._h, _ptr(a)), 'debugCounters')
        return a

    def check_errors(self):
        rc = self._lib.sn_check_errors(self._h)
        if rc != 0:
            self._check(rc, 'checkErrors')

    def sync(self):
        self._check(self._lib.sn_sync(self._h), 'sync')

    def info(self) -> dict:
        i = _native.SnInfo()
        self._check(self._lib.sn_get_info(self._h, ctypes.byref(i)), 'info')
        return {k: getattr(i, k) for k, _ in i._fields_}

    def set_walls(self, on: bool) -> bool:
        """setWalls (src/engine.js:5262): remove or restore the boundary container."""
        out = ctypes.c_uint32()
        self._check(self._lib.sn_set_walls(self._h, 1 if on else 0, ctypes.byref(out)), 'setWalls')
        self._n = self.info()['n']
        return bool(out.value)

    def set_formation_clock(self, clock: int, dirty: bool):
        self._check(self._lib.sn_set_formation_clock(self._h, int(clock), 1 if dirty else 0), 'formationClock')

    def last_timing(self):
        ms = ctypes.c_float()
        l = ctypes.c_uint64()
        self._check(self._lib.sn_last_timing(self._h, ctypes.byref(ms), ctypes.byref(l)), 'timing')
        return float(ms.value), int(l.value)

    @staticmethod
    def _jet_words(jets):
        q = np.zeros(max(1, len(jets)) * 5, np.int32)
        for k, j in enumerate(jets):
            q[k * 5:k * 5 + 5] = (int(j['x']), int(j['y']), int(j['r']), int(j.get('fx', 0)), int(j.get('fy', 0)))
        return q

    def set_jets(self, jets) -> int:
        """setJets (src/engine.js:4740): list of {x, y, r, fx, fy} in ticks; the
        first 8 are kept. Returns how many the engine holds."""
        jets = list(jets or [])
        q = self._jet_words(jets)
        n = ctypes.c_uint32()
        self._check(self._lib.sn_set_jets(self._h, _ptr(q), len(jets), ctypes.byref(n)), 'setJets')
        return int(n.value)

    def set_user_drive(self, ax: int, ay: int):
        """setUserDrive (src/engine.js:4797): stored clamped to +-32768; added
        to the velocity of free bodies flagged as the user's."""
        out = np.zeros(2, np.int32)
        self._check(self._lib.sn_set_user_drive(self._h, int(ax), int(ay), _ptr(out)), 'setUserDrive')
        return [int(out[0]), int(out[1])]

    setJets = set_jets
    setUserDrive = set_user_drive

    # ---- §20 rigid bodies (src/engine.js:5452-5811) ------------------------------
    @staticmethod
    def _pivot(pivot):
        if pivot is None:
            return None
        return np.ascontiguousarray([int(pivot[0]), int(pivot[1])], dtype=np.int32)

    def make_rigid_body(self, slots, pivot=None, user: bool = False) -> Optional[int]:
        """makeRigidBody(slots, pivot, user) (src/engine.js:5722): one body of
        the listed fluid slots whose row is solidMode rigid (not anchored, not
        already in a body) under a fresh tag; ``pivot`` = (x, y) ticks makes
        an axis body. Returns the body index, or None below 4 members."""
        s = np.ascontiguousarray(np.asarray(slots, dtype=np.int64).reshape(-1).clip(0, 2**32 - 1).astype(np.uint32))
        pv = self._pivot(pivot)
        out = ctypes.c_int32()
        self._check(self._lib.sn_make_rigid_body(self._h, _ptr(s), s.size, _ptr(pv), int(bool(user)),
                                                 ctypes.byref(out)), 'makeRigidBody')
        return None if out.value < 0 else int(out.value)

    # ---- runtime material rows (src/engine.js:4843-4855, 5115-5245) -------------
    def set_material(self, row: int, words) -> int:
        """_internUpload: write one row past the authored ones (rampInv baked,
        grav scaled by the gravity scale); returns the table size."""
        w = np.ascontiguousarray(np.asarray(words, dtype=np.int64).reshape(48).astype(np.int32))
        out = ctypes.c_uint32()
        self._check(self._lib.sn_set_material(self._h, int(row), _ptr(w), ctypes.byref(out)), 'internUpload')
        return int(out.value)

    def clear_materials(self):
        self._check(self._lib.sn_clear_materials(self._h), 'clearInterned')

    def set_gravity_scale(self, q: int) -> int:
        out = ctypes.c_int32()
        self._check(self._lib.sn_set_gravity_scale(self._h, int(q), ctypes.byref(out)), 'setGravityScale')
        return int(out.value)

    setGravityScale = set_gravity_scale

    def write_body(self, members, tag: int = 0, pivot=None, user: bool = False):
        """_writeBodyRecord for host-side rebuilds (members as given, tag 0 =
        a fresh tag); returns (index or None, tag)."""
        s = np.ascontiguousarray(np.asarray(members, dtype=np.int64).reshape(-1).astype(np.uint32))
        pv = self._pivot(pivot)
        out, t = ctypes.c_int32(), ctypes.c_uint32()
        self._check(self._lib.sn_write_body(self._h, _ptr(s) if s.size else None, s.size, int(tag), _ptr(pv),
                                            int(bool(user)), ctypes.byref(out), ctypes.byref(t)), 'writeBodyRecord')
        return (None if out.value < 0 else int(out.value)), int(t.value)

    def make_axis_body(self, slots, px: int, py: int, user: bool = False) -> Optional[int]:
        return self.make_rigid_body(slots, (px, py), user)

    def promote_weld_group(self, tag: int = 0, pivot=None, user: bool = False) -> Optional[int]:
        """promoteWeldGroup(tag = held, pivot, user) (src/engine.js:5584)."""
        pv = self._pivot(pivot)
        out = ctypes.c_int32()
        self._check(self._lib.sn_promote_weld_group(self._h, int(tag), _ptr(pv), int(bool(user)),
                                                    ctypes.byref(out)), 'promoteWeldGroup')
        return None if out.value < 0 else int(out.value)

    def end_weld_group_and_promote(self, pivot=None, user: bool = False) -> Optional[int]:
        pv = self._pivot(pivot)
        out = ctypes.c_int32()
        self._check(self._lib.sn_end_weld_group_and_promote(self._h, _ptr(pv), int(bool(user)), ctypes.byref(out)),
                    'endWeldGroupAndPromote')
        return None if out.value < 0 else int(out.value)

    def dissolve_all_bodies(self) -> int:
        out = ctypes.c_uint32()
        self._check(self._lib.sn_dissolve_all_bodies(self._h, ctypes.byref(out)), 'dissolveAllBodies')
        return int(out.value)

    @property
    def body_count(self) -> int:
        out = ctypes.c_uint32()
        self._check(self._lib.sn_read_bodies(self._h, None, 0, ctypes.byref(out)), 'readBodies')
        return int(out.value)

    def read_bodies(self) -> np.ndarray:
        """readBodies(): one row of 32 record words per body."""
        nb = self.body_count
        a = np.zeros(max(1, nb) * 32, np.int32)
        out = ctypes.c_uint32()
        self._check(self._lib.sn_read_bodies(self._h, _ptr(a), a.size, ctypes.byref(out)), 'readBodies')
        return a[:int(out.value) * 32].reshape(-1, 32)

    def read_rest_offsets(self) -> np.ndarray:
        a = np.zeros(max(1, self.n) * 2, np.int32)
        self._check(self._lib.sn_read_rest_offsets(self._h, _ptr(a), a.size), 'readRestOffsets')
        return a[:self.n * 2]

    def set_body_user(self, index: int, on: bool) -> bool:
        out = ctypes.c_uint32()
        self._check(self._lib.sn_set_body_user(self._h, int(index), int(bool(on)), ctypes.byref(out)), 'setBodyUser')
        return bool(out.value)

    def set_body_driver(self, index: int, mask: int, values):
        """The driver sidecar of one body: RD_HAS_* mask and the nine values
        {px, py, angle, vx, vy, omega, fx, fy, torque}, held until changed."""
        v = np.zeros(9, np.int32)
        v[:len(values)] = np.asarray(values, dtype=np.int64).clip(-2**31, 2**31 - 1)
        self._check(self._lib.sn_set_body_driver(self._h, int(index), int(mask), _ptr(v)), 'setBodyConstraint')

    def clear_body_drivers(self):
        self._check(self._lib.sn_clear_body_drivers(self._h), 'clearBodyConstraints')

    def drag_body(self, tag: int, x: int, y: int, vx: int = 0, vy: int = 0) -> bool:
        """dragGrab's rigid branch (src/engine.js:6111): the free body wearing
        ``tag`` is put one velocity behind (x, y)."""
        out = ctypes.c_uint32()
        self._check(self._lib.sn_drag_body(self._h, int(tag), int(x), int(y), int(vx), int(vy), ctypes.byref(out)),
                    'dragGrab')
        return bool(out.value)

    def restore_bodies(self, records, rest=None):
        r = np.ascontiguousarray(np.asarray(records, dtype=np.int32).reshape(-1))
        rr = None if rest is None else np.ascontiguousarray(np.asarray(rest, dtype=np.int32).reshape(-1))
        self._check(self._lib.sn_restore_bodies(self._h, _ptr(r) if r.size else None, r.size // 32, _ptr(rr),
                                                0 if rr is None else rr.size), 'restoreAuthoringSnapshot')

    makeRigidBody = make_rigid_body
    makeAxisBody = make_axis_body
    promoteWeldGroup = promote_weld_group
    endWeldGroupAndPromote = end_weld_group_and_promote
    dissolveAllBodies = dissolve_all_bodies
    readBodies = read_bodies
    readRestOffsets = read_rest_offsets
    setBodyUser = set_body_user

    def autotune(self, reps: int = 1) -> int:
        """Pick the gather lanes per kernel class on real substeps (the scene
        advances by the returned count, exactly as step() would)."""
        n = ctypes.c_uint32()
        self._check(self._lib.sn_autotune(self._h, int(reps), ctypes.byref(n)), 'autotune')
        return int(n.value)

    def lanes(self):
        a = np.zeros(5, np.uint32)
        self._check(self._lib.sn_lanes(self._h, _ptr(a)), 'lanes')
        return dict(zip(('solveA', 'colours', 'post1', 'post2', 'nbr'), (int(x) for x in a)))

    def set_lanes(self, lanes: dict):
        """Pin the per-class lane split (the dict `lanes()` returns)."""
        a = np.array([lanes[k] for k in ('solveA', 'colours', 'post1', 'post2', 'nbr')], np.uint32)
        self._check(self._lib.sn_set_lanes(self._h, _ptr(a)), 'setLanes')

    # device keyframes (sn_ckpt_*): see checkpoints.CheckpointPool
    def ckpt_bytes(self) -> int:
        out = ctypes.c_size_t()
        self._check(self._lib.sn_ckpt_bytes(self._h, ctypes.byref(out)), 'ckpt_bytes')
        return int(out.value)

    def ckpt_save(self, pool) -> int:
        """Save the scene (state, stAcc, chain, bond rows, bodies, clocks) into
        `pool` on the device; returns the checkpoint's handle."""
        out = ctypes.c_uint64()
        self._check(self._lib.sn_ckpt_save(self._h, pool.h, ctypes.byref(out)), 'ckpt_save')
        return int(out.value)

    def ckpt_load(self, pool, handle: int):
        """Restore the scene to the checkpoint exactly (same n and n_fluid)."""
        self._check(self._lib.sn_ckpt_load(self._h, pool.h, int(handle)), 'ckpt_load')
        self._substeps = int(self.info()['substep_count'])
        return self

    def set_tile_shape(self, shift: int):
        """The staged layout's tiles: 2**shift cells a side (2, 3 or 4)."""
        self._check(self._lib.sn_set_tile_shape(self._h, int(shift)), 'setTileShape')
        return self

    def autotune_layout(self, reps: int = 2) -> dict:
        """Time real substeps under the list gathers and the staged gathers at
        each tile shape (sn_autotune_layout) and keep the fastest. Returns the
        pick (0 = list gathers, else the tile side's log2) and the measured
        ms per substep of each candidate."""
        used, pick = ctypes.c_uint32(), ctypes.c_uint32()
        ms = (ctypes.c_float * 4)()
        self._check(self._lib.sn_autotune_layout(self._h, int(reps), ctypes.byref(used), ctypes.byref(pick), ms),
                    'autotuneLayout')
        self._substeps += int(used.value)
        return {'layout': int(pick.value), 'substeps': int(used.value),
                'ms_per_substep': dict(zip(('list', 'tiles4', 'tiles8', 'tiles16'), (float(x) for x in ms)))}

    def set_staged(self, on: bool = True):
        """Tile-major sorted space with shared-memory staged gathers for solveA
        and the colour passes (same results; see sn_set_staged)."""
        self._check(self._lib.sn_set_staged(self._h, 1 if on else 0), 'setStaged')
        return self

    def set_persistent(self, on: bool = True):
        """The solver iterations as one persistent cooperative kernel (same
        results; see sn_set_persistent)."""
        self._check(self._lib.sn_set_persistent(self._h, 1 if on else 0), 'setPersistent')
        return self

    def profile_substep(self, reps: int = 3) -> np.ndarray:
        """Mean device ms per kernel phase over `reps` real substeps (profileSubstep)."""
        out = np.zeros(64, np.float32)
        n = ctypes.c_uint32()
        self._check(self._lib.sn_profile_substep(self._h, int(reps), _ptr(out), 64, ctypes.byref(n)), 'profile')
        self._substeps += int(reps)
        return out[:n.value].copy()

    @property
    def n(self) -> int:
        return self._n

    @property
    def n_fluid(self) -> int:
        return self._n_fluid

    @property
    def substep_count(self) -> int:
        return self._substeps

    @property
    def formation_clock(self) -> int:
        return int(self.info()['formation_clock'])

    def frame(self) -> int:
        """frame() (src/engine.js:4001): SUBSTEPS_PER_FRAME = 2 substeps."""
        return self.step(2)

    def sync_mirror(self):
        """syncMirror(): the reference copies the state to a host mirror before
        applyImpulse reads it; here impulses are applied on the device at the
        substep boundary and readState is always current, so there is nothing
        to wait for beyond the queued work."""
        self.sync()

    # camelCase aliases: the reference's method names
    syncMirror = sync_mirror
    readDerived = read_scratch   # the derived words that cross substeps (stAcc), n x 2
    readBond = read_bonds
    setWalls = set_walls
    loadScene = load_scene
    chainHex = chain_hex
    resetChain = reset_chain
    readState = read_state
    spawnFluid = spawn_fluid
    applyImpulse = apply_impulse
    debugCounters = debug_counters
    checkErrors = check_errors
    nFluid = n_fluid
    substepCount = substep_count


def create_engine(max_particles: int = 8192, **kw) -> Engine:
    """``createEngine`` (``src/engine.js:2786``): ``maxParticles``, ``maxCells``,
    ``debug``, ``chain``, ``iters``, ``mats``, ``tables``."""
    alias = {'maxParticles': 'max_particles', 'maxCells': 'max_cells'}
    kw = {alias.get(k, k): v for k, v in kw.items()}
    kw.pop('submitBatch', None)
    if 'max_particles' in kw:
        max_particles = kw.pop('max_particles')
    return Engine(max_particles=max_particles, **kw)


createEngine = create_engine


class Batch:
    """Many independent scenes stepped together (``sn_batch_*``).

    Every scene behaves exactly as it would alone in an ``Engine``: same digests,
    same chain. Scenes can be added and removed between steps; impulses are
    queued per scene against its own substep clock.
    """

    def __init__(self, max_particles: int, max_scenes: int, max_cells: int = 0, iters: int = ITERS,
                 debug: bool = False, chain: bool = True, device: int = 0, tables=None, mats=None, lanes: int = 0):
        self._lib = _native.load()
        o, self._keep = _opts(max_particles, max_cells, iters, debug, chain, device, tables, mats, lanes)
        h = ctypes.c_void_p()
        rc = self._lib.sn_batch_create(ctypes.byref(o), int(max_scenes), ctypes.byref(h))
        if rc != 0:
            raise EngineError(f'sn_batch_create failed ({rc})')
        self._h = h
        self.scenes = {}

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self._lib.sn_batch_last_error(self._h)
            raise EngineError(f'[batch] {what}: {msg.decode() if msg else rc}')

    def destroy(self):
        if getattr(self, '_h', None):
            self._lib.sn_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def add_scene(self, scene: Scene, capacity: int = 0) -> int:
        args = _SceneArgs(scene)
        sid = ctypes.c_uint32()
        self._check(self._lib.sn_batch_add_scene(self._h, ctypes.byref(args.c), int(capacity), ctypes.byref(sid)),
                    'add_scene')
        self.scenes[int(sid.value)] = scene
        return int(sid.value)

    def remove_scene(self, sid: int):
        self._check(self._lib.sn_batch_remove_scene(self._h, int(sid)), 'remove_scene')
        self.scenes.pop(int(sid), None)

    def step(self, count: int = 1):
        self._check(self._lib.sn_batch_step(self._h, int(count)), 'step')

    def schedule_impulse(self, sid: int, at_substep: int, cx: int, cy: int, r: int, ix: int, iy: int,
                         limit: int = 3000):
        self._check(self._lib.sn_batch_schedule_impulse(self._h, int(sid), int(at_substep), int(cx), int(cy), int(r),
                                                          int(ix), int(iy), int(limit)), 'schedule_impulse')

    def digest(self, sid: int) -> Digest:
        a = np.zeros(8, np.uint32)
        self._check(self._lib.sn_batch_digest(self._h, int(sid), _ptr(a)), 'digest')
        return Digest(a)

    def chain_hex(self, sid: int) -> str:
        a = np.zeros(8, np.uint32)
        self._check(self._lib.sn_batch_chain(self._h, int(sid), _ptr(a)), 'chain')
        return ''.join(f'{int(x):08x}' for x in a)

    def info(self, sid: int) -> dict:
        i = _native.SnInfo()
        self._check(self._lib.sn_batch_get_info(self._h, int(sid), ctypes.byref(i)), 'info')
        return {k: getattr(i, k) for k, _ in i._fields_}

    def erase(self, sid: int, keep) -> int:
        """eraseWhere's compaction on scene ``sid``: one keep flag per fluid slot;
        returns the number erased. The other scenes are untouched."""
        k = np.ascontiguousarray(np.asarray(keep, dtype=bool).astype(np.uint8))
        out = ctypes.c_uint32()
        self._check(self._lib.sn_batch_erase(self._h, int(sid), _ptr(k), k.size, ctypes.byref(out)), 'eraseWhere')
        return int(out.value)

    def write_bonds(self, sid: int, bonds: np.ndarray):
        b = np.ascontiguousarray(bonds, dtype=np.uint32).reshape(-1)
        self._check(self._lib.sn_batch_write_bonds(self._h, int(sid), _ptr(b), b.size), 'writeBonds')

    def read_state(self, sid: int, out: Optional[np.ndarray] = None) -> np.ndarray:
        a = _out_words(out, self.info(sid)['n'] * 8)
        self._check(self._lib.sn_batch_read_state(self._h, int(sid), _ptr(a), a.size), 'read_state')
        return a

    # ---- rigid bodies of one scene (the Engine calls, src/engine.js:5319-6111) ----
    def make_rigid_body(self, sid: int, slots, pivot=None, user: bool = False) -> Optional[int]:
        """makeRigidBody on scene ``sid``; the index counts that scene's bodies."""
        s = np.ascontiguousarray(np.asarray(slots, dtype=np.int64).reshape(-1).clip(0, 2**32 - 1).astype(np.uint32))
        pv = Engine._pivot(pivot)
        out = ctypes.c_int32()
        self._check(self._lib.sn_batch_make_rigid_body(self._h, int(sid), _ptr(s), s.size, _ptr(pv),
                                                       int(bool(user)), ctypes.byref(out)), 'makeRigidBody')
        return None if out.value < 0 else int(out.value)

    def make_axis_body(self, sid: int, slots, px: int, py: int, user: bool = False) -> Optional[int]:
        return self.make_rigid_body(sid, slots, (px, py), user)

    def promote_weld_group(self, sid: int, tag: int = 0, pivot=None, user: bool = False) -> Optional[int]:
        pv = Engine._pivot(pivot)
        out = ctypes.c_int32()
        self._check(self._lib.sn_batch_promote_weld_group(self._h, int(sid), int(tag), _ptr(pv), int(bool(user)),
                                                          ctypes.byref(out)), 'promoteWeldGroup')
        return None if out.value < 0 else int(out.value)

    def dissolve_all_bodies(self, sid: int) -> int:
        out = ctypes.c_uint32()
        self._check(self._lib.sn_batch_dissolve_all_bodies(self._h, int(sid), ctypes.byref(out)), 'dissolveAllBodies')
        return int(out.value)

    def body_count(self, sid: int) -> int:
        out = ctypes.c_uint32()
        self._check(self._lib.sn_batch_read_bodies(self._h, int(sid), None, 0, ctypes.byref(out)), 'readBodies')
        return int(out.value)

    def read_bodies(self, sid: int) -> np.ndarray:
        nb = self.body_count(sid)
        a = np.zeros(max(1, nb) * 32, np.int32)
        out = ctypes.c_uint32()
        self._check(self._lib.sn_batch_read_bodies(self._h, int(sid), _ptr(a), a.size, ctypes.byref(out)),
                    'readBodies')
        return a[:int(out.value) * 32].reshape(-1, 32)

    def read_rest_offsets(self, sid: int) -> np.ndarray:
        n = self.info(sid)['n']
        a = np.zeros(max(1, n) * 2, np.int32)
        self._check(self._lib.sn_batch_read_rest_offsets(self._h, int(sid), _ptr(a), a.size), 'readRestOffsets')
        return a[:n * 2]

    def set_body_user(self, sid: int, index: int, on: bool) -> bool:
        out = ctypes.c_uint32()
        self._check(self._lib.sn_batch_set_body_user(self._h, int(sid), int(index), int(bool(on)), ctypes.byref(out)),
                    'setBodyUser')
        return bool(out.value)

    def set_body_driver(self, sid: int, index: int, mask: int, values):
        v = np.zeros(9, np.int32)
        v[:len(values)] = np.asarray(values, dtype=np.int64).clip(-2**31, 2**31 - 1)
        self._check(self._lib.sn_batch_set_body_driver(self._h, int(sid), int(index), int(mask), _ptr(v)),
                    'setBodyConstraint')

    def clear_body_drivers(self, sid: int):
        self._check(self._lib.sn_batch_clear_body_drivers(self._h, int(sid)), 'clearBodyConstraints')

    def drag_body(self, sid: int, tag: int, x: int, y: int, vx: int = 0, vy: int = 0) -> bool:
        out = ctypes.c_uint32()
        self._check(self._lib.sn_batch_drag_body(self._h, int(sid), int(tag), int(x), int(y), int(vx), int(vy),
                                                 ctypes.byref(out)), 'dragGrab')
        return bool(out.value)

    def read_scratch(self, sid: int) -> np.ndarray:
        n = self.info(sid)['n']
        a = np.zeros(n * 2, np.int32)
        self._check(self._lib.sn_batch_read_scratch(self._h, int(sid), _ptr(a), a.size), 'read_scratch')
        return a

    def write_state(self, sid: int, state, scratch, substep_count: int, formation_clock: int, dirty: bool):
        st = np.ascontiguousarray(state, dtype=np.int32).reshape(-1)
        sc = None if scratch is None else np.ascontiguousarray(scratch, dtype=np.int32).reshape(-1)
        self._check(self._lib.sn_batch_write_state(self._h, int(sid), _ptr(st), _ptr(sc), st.size // 8,
                                                    int(substep_count), int(formation_clock), 1 if dirty else 0),
                    'write_state')

    def check_errors(self):
        self._check(self._lib.sn_batch_check_errors(self._h), 'check_errors')

    def sync(self):
        self._check(self._lib.sn_batch_sync(self._h), 'sync')

    def autotune(self, reps: int = 1) -> int:
        n = ctypes.c_uint32()
        self._check(self._lib.sn_batch_autotune(self._h, int(reps), ctypes.byref(n)), 'autotune')
        return int(n.value)

    def set_jets(self, sid: int, jets) -> int:
        jets = list(jets or [])
        q = Engine._jet_words(jets)
        n = ctypes.c_uint32()
        self._check(self._lib.sn_batch_set_jets(self._h, int(sid), _ptr(q), len(jets), ctypes.byref(n)), 'set_jets')
        return int(n.value)

    def lanes(self):
        a = np.zeros(5, np.uint32)
        self._check(self._lib.sn_batch_lanes(self._h, _ptr(a)), 'lanes')
        return dict(zip(('solveA', 'colours', 'post1', 'post2', 'nbr'), (int(x) for x in a)))

    def set_lanes(self, lanes: dict):
        a = np.array([lanes[k] for k in ('solveA', 'colours', 'post1', 'post2', 'nbr')], np.uint32)
        self._check(self._lib.sn_batch_set_lanes(self._h, _ptr(a)), 'setLanes')

    def set_tile_shape(self, shift: int):
        """The staged layout's tiles: 2**shift cells a side (2, 3 or 4)."""
        self._check(self._lib.sn_batch_set_tile_shape(self._h, int(shift)), 'setTileShape')
        return self

    def autotune_layout(self, reps: int = 2) -> dict:
        """sn_batch_autotune_layout: the fastest of the list and staged layouts
        on real substeps of every scene (see Engine.autotune_layout)."""
        used, pick = ctypes.c_uint32(), ctypes.c_uint32()
        ms = (ctypes.c_float * 4)()
        self._check(self._lib.sn_batch_autotune_layout(self._h, int(reps), ctypes.byref(used), ctypes.byref(pick),
                                                       ms), 'autotuneLayout')
        return {'layout': int(pick.value), 'substeps': int(used.value),
                'ms_per_substep': dict(zip(('list', 'tiles4', 'tiles8', 'tiles16'), (float(x) for x in ms)))}

    def set_staged(self, on: bool = True):
        """Tile-major sorted space with shared-memory staged gathers (sn_batch_set_staged)."""
        self._check(self._lib.sn_batch_set_staged(self._h, 1 if on else 0), 'setStaged')
        return self

    def set_persistent(self, on: bool = True):
        """The solver iterations as one persistent cooperative kernel (sn_batch_set_persistent)."""
        self._check(self._lib.sn_batch_set_persistent(self._h, 1 if on else 0), 'setPersistent')
        return self

    # device keyframes (sn_batch_ckpt_*): see checkpoints.CheckpointPool
    def ckpt_bytes(self, sid: int) -> int:
        out = ctypes.c_size_t()
        self._check(self._lib.sn_batch_ckpt_bytes(self._h, int(sid), ctypes.byref(out)), 'ckpt_bytes')
        return int(out.value)

    def ckpt_save(self, sid: int, pool) -> int:
        out = ctypes.c_uint64()
        self._check(self._lib.sn_batch_ckpt_save(self._h, int(sid), pool.h, ctypes.byref(out)), 'ckpt_save')
        return int(out.value)

    def ckpt_load(self, sid: int, pool, handle: int):
        self._check(self._lib.sn_batch_ckpt_load(self._h, int(sid), pool.h, int(handle)), 'ckpt_load')

    def profile_substep(self, reps: int = 3) -> np.ndarray:
        out = np.zeros(64, np.float32)
        n = ctypes.c_uint32()
        self._check(self._lib.sn_batch_profile_substep(self._h, int(reps), _ptr(out), 64, ctypes.byref(n)),
                    'profile')
        return out[:n.value].copy()

    def last_timing(self):
        ms = ctypes.c_float()
        l = ctypes.c_uint64()
        self._check(self._lib.sn_batch_last_timing(self._h, ctypes.byref(ms), ctypes.byref(l)), 'timing')
        return float(ms.value), int(l.value)
