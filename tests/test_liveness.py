"""Liveness metrics (src/engine.js:6878-7143) on the CPU.

checkLiveness must not be vacuous: the all-zero state and each of the four
degenerate states the reference lists must be rejected, while a real dam
break (run on the oracle) passes with DAMBREAK_EXPECT and a frozen copy of it
does not.
"""
import numpy as np

import oracle
from sunaengine_gb300 import liveness, scenes


def test_zero_state_is_rejected():
    L, v = liveness.zero_state_liveness()
    assert len(v) >= 3, v


def test_every_degenerate_control_is_rejected():
    out = liveness.degenerate_state_controls()
    assert set(out) == {'rigid block drifting uniformly', 'frozen crystal, 1-tick jitter',
                        'frozen solid (no motion at all)', 'all stacked at one point'}
    for name, (L, v) in out.items():
        assert v, f'{name} accepted as live'
    # the reasons the reference gives for each
    drift = out['rigid block drifting uniformly'][1]
    assert any('internalKePerParticle' in s for s in drift)
    frozen = out['frozen solid (no motion at all)'][1]
    assert any('recentMovedFraction' in s for s in frozen)
    stacked = out['all stacked at one point'][1]
    assert any('bbox span' in s for s in stacked)


def _oracle_liveness(e, sc, recent):
    rho = e.read_derived().reshape(-1, 16)[:, 10]
    ct = ((sc.domW + (1 << sc.cellShift) - 1) >> sc.cellShift) * ((sc.domH + (1 << sc.cellShift) - 1) >> sc.cellShift)
    return liveness.compute_liveness(e.read_state(), e.n, e.n_fluid, sc.domW, sc.domH, rho=rho,
                                     nbr_count=e.read_nbr_counts(), cell_start=e.read_cell_start(ct),
                                     initial_pos=np.asarray(sc.pos, np.int32).reshape(-1), recent_pos=recent)


def test_dambreak_is_alive_and_a_frozen_copy_is_not():
    sc = scenes.make_scene('dambreak_v1')
    e = oracle.OracleEngine(sc.n + 64, threads=4).load_scene(sc)
    e.step(150)
    before = e.read_state().reshape(-1, 8)[:sc.nFluid, :2].reshape(-1).copy()
    e.step(20)
    L = _oracle_liveness(e, sc, before)
    assert liveness.check_liveness(L, liveness.DAMBREAK_EXPECT) == []
    assert 4 <= L['maxNbr'] <= 48 and L['maxCellOccupancy'] > 0
    assert 0.98 <= L['meanDensity'] <= 1.04
    # the same state measured against itself as the recent snapshot: frozen
    now = e.read_state().reshape(-1, 8)[:sc.nFluid, :2].reshape(-1).copy()
    F = _oracle_liveness(e, sc, now)
    assert any('FROZEN' in s for s in liveness.check_liveness(F, liveness.DAMBREAK_EXPECT))


def test_slots_past_the_loaded_positions_count_as_moved():
    """A spawn that outgrows the load leaves fluid slots with no initial
    position; computeLiveness reads undefined there, which compares unequal,
    so they count as moved."""
    from sunaengine_gb300.liveness import compute_liveness
    n = 6
    st = np.zeros((n, 8), np.int32)
    st[:, 0] = np.arange(n) * 65536
    st[:, 1] = 65536
    init = st[:4, :2].reshape(-1).copy()  # four loaded, six fluid now
    init[2] += 1                          # the second loaded particle moved
    m = compute_liveness(st.reshape(-1), n, n, 10 * 65536, 10 * 65536, initial_pos=init)
    assert m['movedFraction'] * n == 1 + 2
