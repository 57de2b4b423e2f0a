"""Engine.liveness on the GPU (src/engine.js:4490-4511, 6881-7096).

The per-slot fields it reads (the last substep's rho, neighbour counts and
cell starts) equal the oracle's after the same substeps, and the dam break
stays alive (DAMBREAK_EXPECT) through 1000 substeps plus a 20-substep window.
"""
import numpy as np
import pytest

import oracle
from sunaengine_gb300 import liveness, scenes
from sunaengine_gb300.engine import Engine, EngineError

pytestmark = pytest.mark.gpu


def test_fields_match_the_oracle():
    sc = scenes.make_scene('dambreak_v1')
    g = Engine(max_particles=8192).load_scene(sc)
    with pytest.raises(EngineError):
        g.read_fields()  # nothing has been sorted since the load
    r = oracle.OracleEngine(8192, threads=8).load_scene(sc)
    g.step(37)
    r.step(37)
    rho, nbr = g.read_fields()
    assert np.array_equal(rho[:sc.nFluid], r.read_derived().reshape(-1, 16)[:sc.nFluid, 10])
    assert np.array_equal(nbr[:sc.nFluid], r.read_nbr_counts()[:sc.nFluid])
    assert not rho[sc.nFluid:].any() and not nbr[sc.nFluid:].any()
    ct = g.info()['cell_total']
    assert np.array_equal(g.read_cell_start(), r.read_cell_start(ct))  # the reference's row-major layout
    # an edit that changes slots invalidates them until the next substep
    g.spawn_fluid([{'x': 40 * 65536, 'y': 40 * 65536, 'mat': 0}])
    with pytest.raises(EngineError):
        g.read_fields()
    g.step(1)
    assert g.read_fields()[0].size == g.n


def test_dambreak_alive_after_1000_substeps():
    sc = scenes.make_scene('dambreak_v1')
    g = Engine(max_particles=8192).load_scene(sc)
    g.step(1000)
    L = g.liveness(window=20)
    assert g.substep_count == 1020
    assert liveness.check_liveness(L, liveness.DAMBREAK_EXPECT) == [], L
    # and the reference's non-vacuity controls still fail
    assert len(liveness.zero_state_liveness()[1]) >= 3
    assert all(v for _, v in liveness.degenerate_state_controls().values())


def test_initial_positions_are_the_loaded_ones_and_spawns_outgrow_them():
    """The engine keeps loadScene's positions on the device (_initialPos):
    they equal the scene's, steps and spawns leave them alone, and liveness
    after a spawn of more particles than the load held counts the slots past
    them as moved (the reference reads undefined there)."""
    sc = scenes.make_scene('droplet_v1')
    e = Engine(max_particles=sc.n + 4096).load_scene(sc)
    assert np.array_equal(e.read_initial_positions(), np.asarray(sc.pos, np.int32).reshape(-1))
    e.step(3)
    drop = scenes.make_droplet(64 * scenes.ONE, 36 * scenes.ONE, 14, 14)  # 615 particles: more than the load held
    assert e.spawn_fluid([dict(p, mat=0) for p in drop]) == sc.n + len(drop)
    assert e.n_fluid > sc.n
    assert np.array_equal(e.read_initial_positions(), np.asarray(sc.pos, np.int32).reshape(-1))
    e.step(2)
    m = e.liveness()
    assert m['movedFraction'] * e.n_fluid >= e.n_fluid - sc.n
    e.load_scene(sc)
    assert np.array_equal(e.read_initial_positions(), np.asarray(sc.pos, np.int32).reshape(-1))
    e.check_errors()
