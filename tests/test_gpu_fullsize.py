"""The headline workload at full size (1,048,576 fluid particles, WATER/OIL
bands, seeded temperatures): six substeps bit-exact against the oracle, then
size-independent properties over more substeps — H_set is invariant under a
permutation of the particles while H_slot sees it, and the result does not
depend on the lane split or the build (debug counters on or off)."""
import os

import numpy as np
import pytest

from sunaengine_gb300 import scenes
from sunaengine_gb300.engine import Engine

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def big():
    return scenes.large_two_fluid(side=1024)


def _engine(sc, **kw):
    return Engine(max_particles=sc.n, max_cells=1 << 20, **kw).load_scene(sc)


def test_full_size_matches_oracle(big):
    import oracle
    g = _engine(big, debug=True)
    r = oracle.OracleEngine(big.n, threads=os.cpu_count() or 1).load_scene(big)
    assert g.digest().hex == r.digest()
    for _ in range(2):
        g.step(1)
        r.step(1)
        assert g.digest().hex == r.digest()
    assert g.chain_hex() == r.chain_hex()
    g.step(4)   # through a bond-formation substep (every 4th) of the closure's passes
    r.step(4)
    assert g.chain_hex() == r.chain_hex()
    assert np.array_equal(g.read_state(), r.read_state())
    assert np.array_equal(g.debug_counters(), r.debug_counters())


def test_full_size_permutation_moves_only_the_slot_hash(big):
    a = _engine(big)
    b = _engine(scenes.permute_scene(big, 0x5151))
    for k in (0, 3, 5):
        a.step(k)
        b.step(k)
        da, db = a.digest(), b.digest()
        assert da.set_hex == db.set_hex
        assert da.slot_hex != db.slot_hex
    assert a.chain_hex() != b.chain_hex()


def test_full_size_lanes_and_builds_agree(big):
    a = _engine(big, lanes=1, debug=True)
    b = _engine(big, lanes=4)
    a.step(6)
    b.step(6)
    assert a.chain_hex() == b.chain_hex()
    assert np.array_equal(a.read_state(), b.read_state())
    assert not a.debug_counters()[[0, 1, 2, 5]].any()


def test_batched_workload_matches_oracle_on_a_sample():
    """The batched workload at full size (256 seeded scenes of 1 k-64 k
    particles, 3.86 M in all, each with its own stir schedule) in one batch;
    twelve of its scenes, the largest and smallest among them, stepped on the
    oracle with the same impulses: chains equal after 60 substeps."""
    import oracle
    from sunaengine_gb300.engine import Batch
    scs, sched = scenes.batch_scenes(count=256, seed=0xba7c4, substeps=60)
    b = Batch(max_particles=sum(s.n for s in scs) + 16, max_scenes=len(scs), max_cells=1 << 22)
    for sid, (s, ev) in enumerate(zip(scs, sched)):
        assert b.add_scene(s) == sid
        for (at, cx, cy, r, ix, iy) in ev:
            b.schedule_impulse(sid, at, cx, cy, r, ix, iy)
    by_size = sorted(range(len(scs)), key=lambda i: scs[i].n)
    pick = sorted({by_size[0], by_size[-1]} | set(by_size[::len(scs) // 10]))[:12]
    refs = {i: oracle.OracleEngine(scs[i].n + 8, threads=os.cpu_count() or 1).load_scene(scs[i]) for i in pick}
    events = 0
    for s in range(60):
        for i, r in refs.items():
            for (at, cx, cy, rad, ix, iy) in sched[i]:
                if at == s:
                    r.impulse(cx, cy, rad, ix, iy)
                    events += 1
        for r in refs.values():
            r.step(1)
    b.step(60)
    assert events > 0
    for i, r in refs.items():
        assert b.chain_hex(i) == r.chain_hex(), f'scene {i} (n={scs[i].n})'
    b.check_errors()
