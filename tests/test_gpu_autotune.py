"""The lane autotuner runs real substeps and never changes results."""
import pytest

from sunaengine_gb300 import scenes
from sunaengine_gb300.engine import Batch, Engine

pytestmark = pytest.mark.gpu


def test_autotune_keeps_the_chain():
    sc = scenes.large_two_fluid(side=192)
    a = Engine(max_particles=sc.n).load_scene(sc)
    ran = a.autotune(1)
    assert ran == 8          # 4 lane counts x (1 untimed + 1 timed)
    lanes = a.lanes()
    assert set(lanes) == {'solveA', 'colours', 'post1', 'post2', 'nbr'}
    assert all(v in (1, 2, 4, 8) for v in lanes.values())
    a.step(6)
    b = Engine(max_particles=sc.n, lanes=1).load_scene(sc)
    b.step(ran + 6)
    assert a.chain_hex() == b.chain_hex() and a.digest().hex == b.digest().hex


def test_batch_autotune_keeps_every_scene():
    scs, sched = scenes.batch_scenes(count=12, seed=5, n_lo=1024, n_hi=16384, substeps=60)
    bt = Batch(max_particles=sum(s.n for s in scs), max_scenes=12)
    ids = [bt.add_scene(s) for s in scs]
    for sid, ev in zip(ids, sched):
        for e in ev:
            bt.schedule_impulse(sid, *e)
    ran = bt.autotune(2)
    bt.step(30 - ran)
    ref = Batch(max_particles=sum(s.n for s in scs), max_scenes=12, lanes=2)
    rid = [ref.add_scene(s) for s in scs]
    for sid, ev in zip(rid, sched):
        for e in ev:
            ref.schedule_impulse(sid, *e)
    ref.step(30)
    for i, j in zip(ids, rid):
        assert bt.chain_hex(i) == ref.chain_hex(j)


def test_pinned_lanes_survive_a_load():
    sc = scenes.make_scene('dambreak_v1')
    e = Engine(max_particles=sc.n + 64)
    want = {'solveA': 2, 'colours': 4, 'post1': 1, 'post2': 8, 'nbr': 2}
    e.set_lanes(want)
    e.load_scene(sc)
    assert e.lanes() == want
    e.step(3)
    e.autotune(1)
    assert e.lanes() == want
