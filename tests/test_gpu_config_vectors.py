"""The benchmark workloads replayed at their full lengths against the oracle's
recorded chains (tests/golden/config_vectors/, written by
make_config_vectors.py), through the C ABI, with no oracle in the loop.

The chain after substep k folds H_set || H_slot of every substep up to k, so
equal chains at every recorded substep mean every digest matched:

* the 64 x 64 dam break: every substep of 1000;
* the 1,048,576-particle WATER/OIL scene: every substep of 1000;
* the 262,144-particle 3D dam break with its 4096 lattice bonds: every substep
  of 500;
* the 256-scene batch (stir impulses on each scene's own clock): the sampled
  scenes' chains every 100 substeps of 1000, all 256 scenes stepped together;
* the 74,384-particle construction site with its 48 rigid bodies and held
  seal rail: every substep of 500.

The 2D workloads replay in each mode of the substep: the default per-phase
graph, the tile-staged shared-memory gathers (sn_set_staged) and the
persistent solver loop (sn_set_persistent).
"""
import json
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

VEC = Path(__file__).resolve().parent / 'golden' / 'config_vectors'


def _vector(name):
    p = VEC / f'{name}.json'
    if not p.exists():
        pytest.skip(f'{p.name} not recorded')
    return json.loads(p.read_text())


MODES = ['graph', 'staged', 'persistent']


def _mode(x, mode):
    if mode == 'staged':
        x.set_staged(True)
    elif mode == 'persistent':
        x.set_persistent(True)
    return x


def _replay_2d(sc, vec, mode, max_cells=0):
    from sunaengine_gb300.engine import Engine
    assert sc.n == vec['particles'] and sc.nFluid == vec['fluid_particles']
    e = _mode(Engine(max_particles=sc.n, max_cells=max_cells, iters=vec['iters']), mode).load_scene(sc)
    for k, want in enumerate(vec['chain'], start=1):
        e.step(1)
        got = e.chain_hex()
        assert got == want, f'chain differs at substep {k}'
        d = vec['digest'].get(str(k))
        if d is not None:
            assert e.digest().hex == d, f'digest differs at substep {k}'
    assert e.substep_count == vec['substeps']
    e.check_errors()
    e.destroy()


@pytest.mark.parametrize('mode', MODES)
def test_dambreak_64x64_full_length(mode):
    from sunaengine_gb300 import scenes
    vec = _vector('dambreak_64x64')
    _replay_2d(scenes.lattice_dambreak(), vec, mode)


@pytest.mark.parametrize('mode', MODES)
def test_two_fluid_1024_full_length(mode):
    from sunaengine_gb300 import scenes
    vec = _vector('two_fluid_1024')
    _replay_2d(scenes.large_two_fluid(side=1024), vec, mode, max_cells=1 << 20)


def test_dam3d_64cubed_full_length():
    from sunaengine_gb300 import tables3d
    from sunaengine_gb300.engine3d import Engine3D
    vec = _vector('dam3d_64cubed')
    sc = tables3d.dam3d_large()
    e = Engine3D(max_particles=sc.n, iters=vec['iters']).load_scene(sc)
    bonds = tables3d.dam3d_bonds(sc)
    assert len(bonds) == vec['bonds']
    e.write_bonds(tables3d.bond_rows(sc, bonds), tables3d.DAM3D_BOND_K, tables3d.DAM3D_BOND_BRK)
    for k, want in enumerate(vec['chain'], start=1):
        e.step(1)
        assert e.chain_hex() == want, f'chain differs at substep {k}'
    assert e.fnv_hex() == vec["fnv"]
    e.close()


@pytest.mark.parametrize('mode', MODES)
def test_construction_site_full_length(mode):
    from sunaengine_gb300 import scenes
    from sunaengine_gb300.engine import Engine
    vec = _vector('construction_site')
    sc = scenes.construction_site()
    assert sc.n == vec['particles'] and sc.nFluid == vec['fluid_particles']
    # (the persistent loop serves worlds without bodies; this one steps the graph)
    e = _mode(Engine(max_particles=sc.n, iters=vec['iters']), mode).load_scene(sc)
    for pl, wh, pv in zip(sc.meta['planks'], sc.meta['wheels'], sc.meta['wheel_pivots']):
        e.make_rigid_body(pl)
        e.make_axis_body(wh, *pv)
    assert int(e.read_bodies().shape[0]) == vec['bodies']
    for k, want in enumerate(vec['chain'], start=1):
        e.step(1)
        assert e.chain_hex() == want, f'chain differs at substep {k}'
        d = vec['digest'].get(str(k))
        if d is not None:
            assert e.digest().hex == d, f'digest differs at substep {k}'
    e.check_errors()
    e.destroy()


@pytest.mark.parametrize('mode', MODES)
def test_batch_256_full_length(mode):
    from sunaengine_gb300 import scenes
    from sunaengine_gb300.engine import Batch
    vec = _vector('batch_256')
    total = vec['substeps']
    scs, sched = scenes.batch_scenes(count=vec['scenes_total'], seed=vec['seed'], substeps=total)
    b = _mode(Batch(max_particles=sum(s.n for s in scs) + 16, max_scenes=len(scs), max_cells=1 << 22), mode)
    for sid, (s, ev) in enumerate(zip(scs, sched)):
        assert b.add_scene(s) == sid
        for (at, cx, cy, r, ix, iy) in ev:
            b.schedule_impulse(sid, at, cx, cy, r, ix, iy)
    recorded = {int(k): v for k, v in vec['scenes'].items()}
    assert len(recorded) >= 64
    for k in range(vec['every'], total + 1, vec['every']):
        b.step(vec['every'])
        for sid, rec in recorded.items():
            assert scs[sid].n == rec['particles']
            want = rec['chain'].get(str(k))
            if want is not None:
                assert b.chain_hex(sid) == want, f'scene {sid} (n={scs[sid].n}) differs at substep {k}'
    b.check_errors()
    b.destroy()
