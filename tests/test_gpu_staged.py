"""The tile-staged gathers (sn_set_staged: tile-major sorted space, each tile's
neighbourhood bulk-copied into shared memory, tile-local neighbour lists) give
the same results as the default colour-major list gathers, which the other
GPU tests hold to the oracle: chains after every substep, the final state and
the debug counters of the debug build. The overdense scene has tiles whose
neighbourhood exceeds the staging capacity, so the global fallback runs too.
"""
import numpy as np
import pytest

from sunaengine_gb300 import scenes
from sunaengine_gb300.engine import Batch, Engine

from test_gpu_parity import SCENES

pytestmark = pytest.mark.gpu

CASES = ['dambreak_v1', 'overdense_v1', 'stretch_gel', 'thermal_mix', 'rice_pool', 'two_fluid_48',
         'lattice_dambreak_64', 'one_drop']


@pytest.mark.parametrize('name', CASES)
@pytest.mark.parametrize('debug', [False, True])
def test_staged_equals_list_gathers(name, debug):
    make, steps = SCENES[name]
    sc = make()
    cap = max(8192, sc.n + 64)
    a = Engine(max_particles=cap, debug=debug).load_scene(sc)
    b = Engine(max_particles=cap, debug=debug).set_staged(True).load_scene(sc)
    for k in range(steps):
        a.step(1)
        b.step(1)
        assert a.chain_hex() == b.chain_hex(), f'{name}: substep {k + 1}'
    assert np.array_equal(a.read_state(), b.read_state())
    assert np.array_equal(a.debug_counters(), b.debug_counters())
    b.check_errors()


@pytest.mark.parametrize('lanes', [1, 2, 4, 8])
def test_staged_lane_splits(lanes):
    sc = scenes.large_two_fluid(side=96, band=16)
    a = Engine(max_particles=sc.n + 64).load_scene(sc)
    b = Engine(max_particles=sc.n + 64, lanes=lanes).set_staged(True).load_scene(sc)
    a.step(12)
    b.step(12)
    assert a.chain_hex() == b.chain_hex()


def test_staged_batch_with_impulses():
    scs, sched = scenes.batch_scenes(count=12, seed=0x51a9, n_lo=1024, n_hi=8192, substeps=40)
    out = []
    for staged in (False, True):
        bt = Batch(max_particles=sum(s.n for s in scs) + 16, max_scenes=len(scs), max_cells=1 << 20)
        if staged:
            bt.set_staged(True)
        for sid, (s, ev) in enumerate(zip(scs, sched)):
            assert bt.add_scene(s) == sid
            for (at, cx, cy, r, ix, iy) in ev:
                bt.schedule_impulse(sid, at, cx, cy, r, ix, iy)
        bt.step(40)
        bt.check_errors()
        out.append([bt.chain_hex(i) for i in range(len(scs))])
        bt.destroy()
    assert out[0] == out[1]


@pytest.mark.parametrize('shift', [3, 4])
@pytest.mark.parametrize('name', ['dambreak_v1', 'overdense_v1', 'stretch_gel', 'two_fluid_48'])
def test_larger_tiles_equal_list_gathers(name, shift):
    """Tiles of 8 and 16 cells a side (sn_set_tile_shape): the run table's
    longer halo columns, and more tiles past the staging capacity."""
    make, steps = SCENES[name]
    sc = make()
    cap = max(8192, sc.n + 64)
    a = Engine(max_particles=cap, debug=True).load_scene(sc)
    b = Engine(max_particles=cap, debug=True).set_staged(True).set_tile_shape(shift).load_scene(sc)
    for k in range(steps):
        a.step(1)
        b.step(1)
        assert a.chain_hex() == b.chain_hex(), f'{name}, tiles of {1 << shift}: substep {k + 1}'
    assert np.array_equal(a.read_state(), b.read_state())
    assert np.array_equal(a.debug_counters(), b.debug_counters())
    b.check_errors()


def test_layout_autotune_runs_real_substeps():
    """sn_autotune_layout times every layout on the scene's own substeps: the
    chain after it equals a plain engine's after as many substeps, and the
    picked layout keeps stepping identically."""
    from sunaengine_gb300.engine import EngineError
    sc = scenes.large_two_fluid(side=96, band=16)
    a = Engine(max_particles=sc.n + 64).load_scene(sc)
    b = Engine(max_particles=sc.n + 64).load_scene(sc)
    res = b.autotune_layout(2)
    assert res['layout'] in (0, 2, 3, 4) and res['substeps'] == 12
    assert all(v > 0 for v in res['ms_per_substep'].values())
    assert b.substep_count == 12
    a.step(12)
    assert a.chain_hex() == b.chain_hex()
    a.step(6)
    b.step(6)
    assert a.chain_hex() == b.chain_hex()
    for bad in (1, 5):
        with pytest.raises(EngineError):
            b.set_tile_shape(bad)
    b.check_errors()


def test_batch_layout_autotune_runs_real_substeps():
    scs, sched = scenes.batch_scenes(count=10, seed=0x7a11, n_lo=1024, n_hi=8192, substeps=30)
    out = []
    for tune in (False, True):
        bt = Batch(max_particles=sum(s.n for s in scs) + 16, max_scenes=len(scs), max_cells=1 << 20)
        for sid, (s, ev) in enumerate(zip(scs, sched)):
            assert bt.add_scene(s) == sid
            for (at, cx, cy, r, ix, iy) in ev:
                bt.schedule_impulse(sid, at, cx, cy, r, ix, iy)
        if tune:
            res = bt.autotune_layout(1)
            assert res['substeps'] == 8 and res['layout'] in (0, 2, 3, 4)
            bt.step(30 - 8)
        else:
            bt.step(30)
        bt.check_errors()
        out.append([bt.chain_hex(i) for i in range(len(scs))])
        bt.destroy()
    assert out[0] == out[1]
