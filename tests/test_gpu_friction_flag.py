"""The friction and applyFric kernels return at once while the world has no
friction or bond row (a device flag k_gather raises each substep). A pool
whose water is driven below freezing turns into ICE (a friction and bond
row) partway through the run, so the flag flips from 0 to 1 between two
launches of the captured substep; the chain must follow the oracle on both
sides."""
import numpy as np
import pytest

from sunaengine_gb300 import data, scenes
from sunaengine_gb300.engine import Engine

pytestmark = pytest.mark.gpu
ONE = 65536


def _cold_drive():
    m = data.mats().copy()
    F = data.MAT_FIELDS
    w = data.mat_id('WATER')
    m[w, F.index('tempTarget')] = -20 * ONE   # driven toward -20 deg ...
    m[w, F.index('tempDrive')] = 655          # ... at 1% a substep: freezes near substep 71
    return m


@pytest.mark.parametrize('debug', [False, True])
def test_friction_pass_opens_when_the_pool_freezes(debug):
    import oracle as o
    m = _cold_drive()
    sc = scenes.make_scene('dambreak_v1')
    g = Engine(max_particles=sc.n + 256, mats=m, debug=debug).load_scene(sc)
    r = o.OracleEngine(sc.n + 256, threads=16, mats=m).load_scene(sc)
    ice = data.mat_id('ICE')
    seen = []
    for k in (40, 25, 5, 3, 3, 4, 20):
        g.step(k)
        r.step(k)
        assert g.chain_hex() == r.chain_hex(), f'diverged by substep {r.substep_count}'
        seen.append(int((g.read_state().reshape(-1, 8)[:, 4] == ice).sum()))
    assert seen[0] == 0 and seen[-1] > 0          # the flag flipped during the run
    assert np.array_equal(g.read_state(), r.read_state())
    if debug:
        assert np.array_equal(g.debug_counters(), r.debug_counters())
    g.check_errors()
