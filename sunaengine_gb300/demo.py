"""The demo layer: deterministic input schedules, keyframes, record and replay.

Mirrors ``WaterDemo`` (``src/demo_boot.js:71-420``): water injections and
cursor pushes quantised to substep indices, exact keyframes (state words plus
the cross-substep scratch), `.sunar` recording that normalises the live run
onto the load boundary its replay will reconstruct, and replay from a
`.sunar` file. It drives any engine with the ``Engine`` method names, so the
same schedule can run on the GPU engine and on the CPU checker.
"""
from __future__ import annotations

from typing import Optional

import numpy as np

from . import formats, scenes

DEMO_PARTICLE_CAP = 6000
DEMO_SUBMIT_BATCH = 25
SPEC_VERSION = 24
FLAG_MASK = 7
MAT_WATER = 0
ONE = scenes.ONE


def wu(x: float) -> int:
    """World units to ticks, rounding half up like JavaScript's Math.round."""
    import math
    return int(math.floor(x * ONE + 0.5))


def make_droplet(cx: int, cy: int, w: int = 3, h: int = 3, vx: int = 0, vy: int = 0):
    """A w x h square of water particles at 1 wu pitch centred on (cx, cy)
    (``makeDroplet``, ``src/demo_boot.js:33-44``)."""
    _int(cx, 'cx')
    _int(cy, 'cy')
    x0 = cx - (((w - 1) * ONE) >> 1)
    y0 = cy - (((h - 1) * ONE) >> 1)
    return [{'x': x0 + gx * ONE, 'y': y0 + gy * ONE, 'vx': int(vx), 'vy': int(vy)}
            for gy in range(h) for gx in range(w)]


def _int(x, label):
    if isinstance(x, bool) or not isinstance(x, (int, np.integer)):
        raise ValueError(f'[demo_boot] {label} must be an integer, got {x}')
    return int(x)


def _i32(x) -> int:
    """JavaScript `x | 0` for the integer inputs the demo accepts."""
    v = int(x) & 0xffffffff
    return v - (1 << 32) if v >= 1 << 31 else v


def _hex(d) -> str:
    return d if isinstance(d, str) else d.hex


class WaterDemo:
    """``WaterDemo`` over an engine (``src/demo_boot.js:127-420``)."""

    def __init__(self, engine, cap: int = DEMO_PARTICLE_CAP, engine_factory=None):
        self.engine = engine
        self.cap = cap
        self.substep = 0
        self._schedule: dict = {}
        self._pushes: dict = {}
        self.push_hits = 0
        self._rec: Optional[dict] = None
        self.replay_doc = None
        self._factory = engine_factory

    # -- passthroughs --------------------------------------------------------------------
    @property
    def n(self):
        return self.engine.n

    @property
    def n_fluid(self):
        return self.engine.n_fluid

    def digest(self) -> str:
        return _hex(self.engine.digest())

    def chain_hex(self) -> str:
        return self.engine.chain_hex()

    def debug_counters(self):
        return list(self.engine.debug_counters())

    def check_errors(self):
        if hasattr(self.engine, 'check_errors'):
            self.engine.check_errors()

    def destroy(self):
        if hasattr(self.engine, 'destroy'):
            self.engine.destroy()

    # -- input schedules -------------------------------------------------------------------
    def inject_water(self, schedule_or_event):
        lst = schedule_or_event if isinstance(schedule_or_event, list) else [schedule_or_event]
        for ev in lst:
            s = _int(ev['substep'], 'event.substep')
            if s < self.substep:
                raise ValueError(f'[demo_boot] injection at substep {s} is in the past (now {self.substep})')
            ps = [{'x': _int(p['x'], 'particle.x'), 'y': _int(p['y'], 'particle.y'),
                   'vx': _i32(p.get('vx', 0) or 0), 'vy': _i32(p.get('vy', 0) or 0)}
                  for p in ev.get('particles') or []]
            if not ps:
                continue
            self._schedule.setdefault(s, []).extend(ps)
            if self._rec is not None:
                self._rec['events'].append({'frame': s - self._rec['startSubstep'], 'order': self._rec['order'],
                                            'type': 'inject', 'particles': ps})
                self._rec['order'] += 1

    def push_at(self, ev):
        s = _int(ev['substep'], 'push.substep')
        if s < self.substep:
            raise ValueError(f'[demo_boot] push at substep {s} is in the past (now {self.substep})')
        p = {'x': _int(ev['x'], 'push.x'), 'y': _int(ev['y'], 'push.y'), 'r': _int(ev['r'], 'push.r'),
             'ix': _i32(ev.get('ix', 0) or 0), 'iy': _i32(ev.get('iy', 0) or 0)}
        if not p['ix'] and not p['iy']:
            return
        self._pushes.setdefault(s, []).append(p)
        if self._rec is not None:
            self._rec['events'].append(dict({'frame': s - self._rec['startSubstep'], 'order': self._rec['order'],
                                             'type': 'push'}, **p))
            self._rec['order'] += 1

    def step(self, count: int = 1) -> int:
        end = self.substep + _int(count, 'count')
        for s in self._pushes:
            if self.substep <= s < end:
                raise ValueError(f'[demo_boot] push armed at substep {s}: use step_through()')
        return self._step_inject_only(count)

    def _step_inject_only(self, count: int) -> int:
        remaining = _int(count, 'count')
        while remaining > 0:
            due = self._schedule.pop(self.substep, None)
            if due:
                self.engine.spawn_fluid([dict(p, mat=MAT_WATER) for p in due], no_weld=True)
            chunk = remaining
            for s in self._schedule:
                if s > self.substep and s - self.substep < chunk:
                    chunk = s - self.substep
            self.engine.step(chunk)
            self.substep += chunk
            remaining -= chunk
        return self.substep

    def step_through(self, count: int = 1) -> int:
        remaining = _int(count, 'count')
        while remaining > 0:
            due = self._pushes.pop(self.substep, None)
            if due:
                for p in due:
                    self.push_hits += self.engine.apply_impulse(p['x'], p['y'], p['r'], p['ix'], p['iy'])
            chunk = remaining
            for s in self._pushes:
                if s > self.substep and s - self.substep < chunk:
                    chunk = s - self.substep
            target = self.substep + chunk
            while self.substep < target:
                inj = target - self.substep
                for s in self._schedule:
                    if s > self.substep and s - self.substep < inj:
                        inj = s - self.substep
                self._step_inject_only(inj)
            remaining -= chunk
        return self.substep

    # -- keyframes ---------------------------------------------------------------------------
    def snapshot(self, exact: bool = True) -> dict:
        e = self.engine
        state = np.asarray(e.read_state(), dtype=np.int32).copy()
        sc = getattr(e, '_scene', None)
        dom = (sc.domW, sc.domH, sc.cellShift) if sc is not None else self._dom
        info = {
            'n': int(e.n), 'nFluid': int(e.n_fluid), 'domW': int(dom[0]), 'domH': int(dom[1]),
            'cellShift': int(dom[2]), 'wallsOn': bool(getattr(self, '_walls_on', True)),
            'substepCount': int(e.substep_count), 'formationClock': int(e.formation_clock),
        }
        return {
            'app': {'name': 'SunaEngine demo', 'specVersion': SPEC_VERSION, 'demoParticleCap': self.cap},
            'scene': info,
            'state': state,
            'tints': np.zeros(int(e.n), np.uint32),
            'derived': np.asarray(e.read_scratch(), dtype=np.int32).copy() if exact else None,
            'substep': self.substep,
        }

    def restore(self, snap: dict):
        self._load_payload(snap)
        if snap.get('derived') is not None:
            _write_state(self.engine, snap['state'], snap['derived'])
        self.substep = int(snap.get('substep') or 0)

    def _load_payload(self, p: dict):
        s = p.get('scene') or (p.get('initial') or {}).get('scene')
        state = p.get('state') if p.get('state') is not None else (p.get('initial') or {}).get('state')
        if not s or state is None:
            raise ValueError('[demo_boot] payload has no scene/state')
        n = int(s['n'])
        w = np.asarray(state, dtype=np.int32).reshape(-1)[:n * 8].reshape(n, 8)
        sc = scenes.Scene(n=n, nFluid=int(s['nFluid']), pos=w[:, 0:2].copy(), vel=w[:, 2:4].copy(),
                          matId=w[:, 4].astype(np.uint32), domW=int(s['domW']), domH=int(s['domH']),
                          cellShift=int(s['cellShift']), flags=(w[:, 5].astype(np.uint32) & FLAG_MASK),
                          temp=w[:, 6].copy(), fuel=w[:, 7].copy())
        self._dom = (sc.domW, sc.domH, sc.cellShift)
        self.engine.load_scene(sc)
        self._walls_on = True
        if s.get('wallsOn') is False:
            self.engine.set_walls(False)
            self._walls_on = False
        self._schedule.clear()
        self._pushes.clear()
        self._rec = None
        self.substep = 0

    # -- record / replay --------------------------------------------------------------------
    def start_recording(self):
        start = self.substep
        initial = self.snapshot(exact=False)
        pend_s = {k: list(v) for k, v in self._schedule.items()}
        pend_p = {k: [dict(x) for x in v] for k, v in self._pushes.items()}
        self._load_payload(initial)
        self._schedule = pend_s
        self._pushes = pend_p
        self.substep = start
        self._rec = {'startSubstep': start, 'initial': initial, 'events': [], 'order': 0}
        for s in sorted(self._schedule):
            self._rec['events'].append({'frame': s - start, 'order': self._rec['order'], 'type': 'inject',
                                        'particles': [dict(p) for p in self._schedule[s]]})
            self._rec['order'] += 1
        for s in sorted(self._pushes):
            for p in self._pushes[s]:
                self._rec['events'].append(dict({'frame': s - start, 'order': self._rec['order'],
                                                 'type': 'push'}, **p))
                self._rec['order'] += 1

    def stop_recording(self):
        if self._rec is None:
            raise ValueError('[demo_boot] stop_recording without start_recording')
        rec = self._rec
        self._rec = None
        rec['events'].sort(key=lambda e: (e['frame'], e['order']))
        for i, e in enumerate(rec['events']):
            e['order'] = i
        dur = self.substep - rec['startSubstep']
        doc = {
            'app': rec['initial']['app'],
            'initial': rec['initial'],
            'events': rec['events'],
            'substepsPerFrame': 1,
            'durationFrames': dur,
            'durationSubsteps': dur,
            'final': {'digest': self.digest(), 'n': int(self.n), 'nFluid': int(self.n_fluid)},
        }
        return formats.encode_sunar(doc), doc


def _write_state(engine, state, scratch):
    if hasattr(engine, 'write_scratch_state'):
        engine.write_scratch_state(state, scratch)
    else:
        engine.write_state(state, scratch)


def _default_engine(cap: int, chain: bool = True):
    from .engine import Engine
    return Engine(max_particles=cap, chain=chain)


def boot_water_demo(scene='pool', pool_w: int = 60, pool_h: int = 20, max_particles: int = DEMO_PARTICLE_CAP,
                    engine_factory=None) -> WaterDemo:
    """``bootWaterDemo`` (``src/demo_boot.js:80-101``)."""
    if max_particles > DEMO_PARTICLE_CAP:
        raise ValueError(f'[demo_boot] maxParticles {max_particles} exceeds the demo cap {DEMO_PARTICLE_CAP}')
    if isinstance(scene, scenes.Scene):
        sc = scene
    elif scene == 'empty':
        sc = scenes.make_scene('empty_v1')
    elif scene == 'pool':
        sc = scenes.make_scene('pool_v1', w=pool_w, h=pool_h, mat=MAT_WATER)
    else:
        sc = scenes.make_scene(scene)
    if sc.n > max_particles:
        raise ValueError(f'[demo_boot] scene has {sc.n} particles; the demo cap is {max_particles}')
    if np.any(np.asarray(sc.matId) != MAT_WATER):
        raise ValueError('[demo_boot] water-only harness: scene contains a non-WATER particle')
    factory = engine_factory or _default_engine
    eng = factory(max_particles)
    eng.load_scene(sc)
    d = WaterDemo(eng, max_particles, factory)
    d._dom = (sc.domW, sc.domH, sc.cellShift)
    d._walls_on = True
    return d


def replay_from_sunar(source, engine_factory=None) -> WaterDemo:
    """``replayFromSunar`` (``src/demo_boot.js:104-125``)."""
    doc = formats.decode_sunar(source)
    cap = int(((doc.get('app') or {}).get('demoParticleCap')) or DEMO_PARTICLE_CAP)
    factory = engine_factory or _default_engine
    demo = WaterDemo(factory(cap), cap, factory)
    demo._load_payload(doc)
    for e in doc['events']:
        if e['type'] == 'inject':
            demo.inject_water({'substep': e['frame'], 'particles': e['particles']})
        elif e['type'] == 'push':
            demo.push_at({'substep': e['frame'], 'x': e['x'], 'y': e['y'], 'r': e['r'],
                          'ix': e.get('ix', 0), 'iy': e.get('iy', 0)})
    demo.replay_doc = doc
    return demo
