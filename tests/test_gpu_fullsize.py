"""The headline workload at full size (1,048,576 fluid particles, WATER/OIL
bands, seeded temperatures): two substeps bit-exact against the oracle, then
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
