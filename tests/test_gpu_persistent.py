"""The persistent form of the solver loop (sn_set_persistent: solveA, the four
colour passes and friction/applyFric of every iteration in one cooperative
launch with grid barriers) gives the same results as the per-phase launches,
which the other GPU tests hold to the oracle: chains after every substep,
final state, debug counters. Scenes with friction and bond rows (sand, the
stretched gel) take its friction phases; a world with rigid bodies keeps the
per-phase launches."""
import numpy as np
import pytest

from sunaengine_gb300 import scenes
from sunaengine_gb300.engine import Batch, Engine

from test_gpu_parity import SCENES

pytestmark = pytest.mark.gpu

CASES = ['dambreak_v1', 'overdense_v1', 'pool_water', 'droplet_oil', 'two_fluid_48', 'lattice_dambreak_64',
         'thermal_mix', 'stretch_gel', 'sand_pool', 'anchored_sand', 'rice_pool']


@pytest.mark.parametrize('name', CASES)
@pytest.mark.parametrize('debug', [False, True])
def test_persistent_equals_per_phase(name, debug):
    make, steps = SCENES[name]
    sc = make()
    cap = max(8192, sc.n + 64)
    a = Engine(max_particles=cap, debug=debug).load_scene(sc)
    b = Engine(max_particles=cap, debug=debug).set_persistent(True).load_scene(sc)
    for k in range(steps):
        a.step(1)
        b.step(1)
        assert a.chain_hex() == b.chain_hex(), f'{name}: substep {k + 1}'
    assert np.array_equal(a.read_state(), b.read_state())
    assert np.array_equal(a.debug_counters(), b.debug_counters())
    b.check_errors()


@pytest.mark.parametrize('lanes', [1, 2, 4, 8])
def test_persistent_lane_splits(lanes):
    sc = scenes.large_two_fluid(side=96, band=16)
    a = Engine(max_particles=sc.n + 64).load_scene(sc)
    b = Engine(max_particles=sc.n + 64, lanes=lanes).set_persistent(True).load_scene(sc)
    a.step(12)
    b.step(12)
    assert a.chain_hex() == b.chain_hex()
    b.check_errors()


def test_persistent_batch_with_impulses():
    scs, sched = scenes.batch_scenes(count=12, seed=0x51a9, n_lo=1024, n_hi=8192, substeps=40)
    out = []
    for persistent in (False, True):
        bt = Batch(max_particles=sum(s.n for s in scs) + 16, max_scenes=len(scs), max_cells=1 << 20)
        bt.set_persistent(persistent)
        for sid, (s, ev) in enumerate(zip(scs, sched)):
            assert bt.add_scene(s) == sid
            for (at, cx, cy, r, ix, iy) in ev:
                bt.schedule_impulse(sid, at, cx, cy, r, ix, iy)
        bt.step(40)
        bt.check_errors()
        out.append([bt.chain_hex(i) for i in range(len(scs))])
        bt.destroy()
    assert out[0] == out[1]


def test_persistent_world_with_bodies_keeps_per_phase_launches():
    sc = scenes.rigid_tank()
    runs = []
    for persistent in (False, True):
        e = Engine(max_particles=sc.n + 64).set_persistent(persistent).load_scene(sc)
        e.make_rigid_body(sc.meta['plank'])
        e.make_rigid_body(sc.meta['wheel'])
        e.step(20)
        e.check_errors()
        runs.append(e.chain_hex())
    assert runs[0] == runs[1]
