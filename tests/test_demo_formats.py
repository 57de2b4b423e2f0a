"""`.suna`/`.sunar` codecs and the demo layer's determinism checks, on the CPU checker.

The checks are the reference's own in-page gates (test/extraction_gate.html:63-132):
twins under one injection schedule, record -> replay byte identity with a
one-tick negative control, and keyframe rejoin (and that a state-only restore
does not rejoin).
"""
import json

import numpy as np
import pytest

from sunaengine_gb300 import demo, formats, scenes
from sunaengine_gb300.demo import make_droplet, wu


def oracle_factory(cap):
    import oracle
    return oracle.OracleEngine(cap, threads=8)


def test_suna_round_trip_and_validation():
    st = np.arange(16, dtype=np.int32) - 5
    payload = {'app': {'name': 'x'}, 'scene': {'n': 2, 'nFluid': 1, 'domW': 65536 * 8, 'domH': 65536 * 8,
                                               'cellShift': 18}, 'state': st, 'tints': np.zeros(2, np.uint32)}
    text = formats.encode_suna(payload)
    doc = formats.decode_suna(text)
    assert np.array_equal(doc['state'], st) and doc['scene']['nFluid'] == 1
    bad = json.loads(text)
    bad['magic'] = 'nope'
    with pytest.raises(formats.FormatError):
        formats.decode_suna(json.dumps(bad))
    bad = json.loads(text)
    bad['formatVersion'] = 2
    with pytest.raises(formats.FormatError):
        formats.decode_suna(json.dumps(bad))
    bad = json.loads(text)
    bad['scene']['n'] = 3
    with pytest.raises(formats.FormatError):
        formats.decode_suna(json.dumps(bad))
    with pytest.raises(formats.FormatError):
        formats.decode_suna('{not json')
    with pytest.raises(formats.FormatError):
        formats.encode_suna(dict(payload, state=st.astype(np.int64)))


def test_sunar_event_order_is_enforced():
    st = np.zeros(8, np.int32)
    init = {'app': {}, 'scene': {'n': 1, 'nFluid': 1, 'domW': 1 << 20, 'domH': 1 << 20, 'cellShift': 18},
            'state': st, 'tints': np.zeros(1, np.uint32)}
    ok = formats.encode_sunar({'initial': init, 'events': [{'frame': 1, 'order': 0, 'type': 'inject'},
                                                           {'frame': 1, 'order': 1, 'type': 'push'}],
                               'durationSubsteps': 5, 'durationFrames': 5, 'substepsPerFrame': 1})
    d = formats.decode_sunar(ok)
    assert d['durationSubsteps'] == 5 and len(d['events']) == 2
    with pytest.raises(formats.FormatError):
        formats.encode_sunar({'initial': init, 'events': [{'frame': 2, 'order': 0, 'type': 'a'},
                                                          {'frame': 1, 'order': 1, 'type': 'b'}]})
    with pytest.raises(formats.FormatError):
        formats.encode_sunar({'initial': init, 'events': [{'frame': 1, 'order': 0, 'type': ''}]})


def test_droplet_and_wu_follow_the_reference_helpers():
    assert wu(0.2) == 13107 and wu(64) == 64 * 65536 and wu(-0.5) == -32768
    d = make_droplet(wu(40), wu(12), 2, 2)
    assert [(p['x'], p['y']) for p in d] == [(wu(40) - 32768, wu(12) - 32768), (wu(40) + 32768, wu(12) - 32768),
                                             (wu(40) - 32768, wu(12) + 32768), (wu(40) + 32768, wu(12) + 32768)]


def _twins(factory, steps=120):
    schedule = [{'substep': s, 'particles': make_droplet(wu(64), wu(10), 3, 3, 0, wu(0.2))} for s in range(0, 60, 8)]
    out = []
    for _ in range(2):
        d = demo.boot_water_demo('pool', engine_factory=factory)
        d.inject_water(schedule)
        d.step(steps)
        out.append((d.chain_hex(), d.digest(), d.n, d.n_fluid))
    return out


def _record_replay(factory):
    d = demo.boot_water_demo('pool', engine_factory=factory)
    d.step(30)
    d.start_recording()
    for s in range(d.substep, d.substep + 50, 10):
        d.inject_water({'substep': s, 'particles': make_droplet(wu(40), wu(12), 2, 2)})
    d.push_at({'substep': d.substep + 7, 'x': wu(30), 'y': wu(62), 'r': wu(5), 'ix': 9000, 'iy': -7000})
    d.step_through(80)
    text, doc = d.stop_recording()
    live = doc['final']['digest']
    r = demo.replay_from_sunar(text, engine_factory=factory)
    r.step_through(r.replay_doc['durationSubsteps'])
    replay = r.digest()
    mut = json.loads(text)
    first_inject = next(e for e in mut['events'] if e['type'] == 'inject')
    first_inject['particles'][0]['x'] += 1
    m = demo.replay_from_sunar(json.dumps(mut), engine_factory=factory)
    m.step_through(m.replay_doc['durationSubsteps'])
    return live, replay, m.digest()


def _keyframe(factory):
    d = demo.boot_water_demo('pool', engine_factory=factory)
    d.step(30)
    key = d.snapshot()
    d.step(20)
    ahead = d.digest()
    d.restore(key)
    d.step(20)
    rejoined = d.digest()
    state_only = dict(key, derived=None)
    d.restore(state_only)
    d.step(20)
    return ahead, rejoined, d.digest()


def test_twins_on_the_checker():
    a, b = _twins(oracle_factory)
    assert a == b


def test_record_replay_identity_and_negative_control_on_the_checker():
    live, replay, mutated = _record_replay(oracle_factory)
    assert replay == live
    assert mutated != live


def test_keyframe_rejoin_on_the_checker():
    ahead, rejoined, state_only = _keyframe(oracle_factory)
    assert rejoined == ahead
    assert state_only != ahead


def test_demo_refuses_past_events_and_unsynced_pushes():
    d = demo.boot_water_demo('pool', engine_factory=oracle_factory)
    d.step(3)
    with pytest.raises(ValueError):
        d.inject_water({'substep': 1, 'particles': make_droplet(wu(40), wu(12))})
    d.push_at({'substep': 5, 'x': wu(30), 'y': wu(60), 'r': wu(4), 'ix': 100, 'iy': 0})
    with pytest.raises(ValueError):
        d.step(5)  # a push is armed inside the span: step_through() is required
    with pytest.raises(ValueError):
        demo.boot_water_demo(scenes.make_scene('pool_v1', mat=4), engine_factory=oracle_factory)
