"""Jets on the GPU against the oracle, single engine and per scene in a batch."""
import pytest

from sunaengine_gb300 import scenes
from sunaengine_gb300.engine import Batch, Engine

import test_oracle_jets as t

pytestmark = pytest.mark.gpu


def test_jets_match_oracle_every_substep():
    sc = scenes.make_scene('pool_v1', w=40, h=14)
    g = Engine(max_particles=sc.n + 64, debug=True).load_scene(sc)
    r = t.oracle(sc)
    assert g.set_jets(t.JETS) == r.set_jets(t.JETS) == 3
    for k in range(12):
        g.step(2)
        r.step(2)
        assert g.chain_hex() == r.chain_hex()
        if k == 6:
            assert g.set_jets(t.JETS[:1]) == r.set_jets(t.JETS[:1]) == 1
    assert list(g.debug_counters()) == list(r.debug_counters())
    assert g.set_user_drive(99999, -5) == [32768, -5]


def test_jets_per_scene_in_a_batch():
    a = scenes.make_scene('pool_v1', w=40, h=14)
    b = scenes.make_scene('pool_v1', w=30, h=12)
    bt = Batch(max_particles=a.n + b.n, max_scenes=2)
    ia, ib = bt.add_scene(a), bt.add_scene(b)
    bt.set_jets(ia, t.JETS)
    bt.step(20)
    ra, rb = t.oracle(a), t.oracle(b)
    ra.set_jets(t.JETS)
    ra.step(20)
    rb.step(20)
    assert bt.chain_hex(ia) == ra.chain_hex() and bt.chain_hex(ib) == rb.chain_hex()
