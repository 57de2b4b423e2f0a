"""3D solver on the GPU against the oracle, through the C ABI.

Every comparison is bit-exact: state words, the per-substep H_set || H_slot
chain, and the page's own FNV stripe digest.
"""
import numpy as np
import pytest

from sunaengine_gb300 import tables3d
from sunaengine_gb300.engine3d import Engine3D

pytestmark = pytest.mark.gpu


def oracle3(n, iters=3):
    import oracle
    return oracle.Oracle3D(n, iters=iters, threads=16)


def both(sc, cap=None, iters=3, debug=False, stir_amp=0):
    cap = cap or sc.n
    g = Engine3D(max_particles=cap, iters=iters, debug=debug).load_scene(sc, stir_amp)
    r = oracle3(cap, iters).load_scene(sc, stir_amp)
    return g, r


def same(g, r, scene=0):
    assert g.chain_hex(scene) == r.chain_hex()
    assert g.digest(scene).hex == r.digest()
    assert g.chain(scene) == r.fnv_hex()
    assert np.array_equal(g.read_state(scene), r.read_state())


@pytest.mark.parametrize('name,n,grid', [('pool', 16000, (28, 30, 28)), ('layers', 12000, (24, 30, 24)),
                                         ('overdense', 24000, (28, 30, 28))])
def test_page_scenes_every_substep(name, n, grid):
    sc = tables3d.initial_state(n, name, *grid)
    g, r = both(sc, debug=True)
    for k in (1, 1, 3, 10, 25):
        g.step(k)
        r.step(k)
        assert g.chain_hex() == r.chain_hex(), f'{name} diverged by substep {r.substep_count}'
    same(g, r)
    assert np.array_equal(g.debug_counters(), r.debug_counters())
    if name == 'overdense':
        assert g.debug_counters()[6] > 0


@pytest.mark.parametrize('iters', [1, 4])
def test_iteration_counts(iters):
    sc = tables3d.initial_state(9000, 'pool', 20, 26, 20)
    g, r = both(sc, iters=iters)
    g.step(20)
    r.step(20)
    same(g, r)


def test_release_equals_debug_build():
    sc = tables3d.initial_state(20000, 'overdense')
    a = Engine3D(max_particles=sc.n, debug=False).load_scene(sc)
    b = Engine3D(max_particles=sc.n, debug=True).load_scene(sc)
    a.step(15)
    b.step(15)
    assert a.chain_hex() == b.chain_hex() and np.array_equal(a.read_state(), b.read_state())


def test_stir_ball_and_spawn_inputs():
    sc = tables3d.initial_state(6000, 'pool', 20, 24, 20)
    cap = 6600
    g = Engine3D(max_particles=cap).load_scene(sc, stir_amp=1200)
    r = oracle3(cap).load_scene(sc, stir_amp=1200)
    for x in (g, r):
        x.step(2)
        x.step(2)
    seed = tables3d.SpawnSeed()
    pos = seed.positions(20.0, 34.0, 20.0, 400, 3.0)
    mat = np.full(400, 4, np.uint32)
    assert g.spawn_positions(pos, mat) == 400
    assert r.spawn(pos, mat) == 400
    g.set_ball(True, 14.0, 6.0, 14.0, 3.0)
    r.set_ball(True, tables3d.js_round(14.0 * 65536), tables3d.js_round(6.0 * 65536),
               tables3d.js_round(14.0 * 65536), 3.0)
    for k in (2, 2, 1, 5):
        g.step(k)
        r.step(k)
    same(g, r)
    # the page's spawn helper: what does not fit is dropped
    assert g.spawn(2, 10.0, 30.0, 10.0, 500) == cap - 6400


def test_keyframe_rejoins():
    sc = tables3d.initial_state(8000, 'pool', 20, 24, 20)
    g = Engine3D(max_particles=sc.n).load_scene(sc, stir_amp=700)
    g.step(12)
    key = (g.read_state(), g.substep_count, g.chain_words())
    g.step(9)
    ahead = (g.chain_hex(), g.chain())
    g.write_state(key[0], key[1], key[2])
    g.step(9)
    assert (g.chain_hex(), g.chain()) == ahead


def test_many_scenes_in_one_launch_equal_each_alone():
    scs = [tables3d.initial_state(5000, 'pool', 16, 20, 16), tables3d.initial_state(9000, 'layers', 20, 26, 20),
           tables3d.initial_state(7000, 'overdense', 12, 20, 12), tables3d.initial_state(3000, 'pool', 10, 22, 14)]
    e = Engine3D(max_particles=sum(s.n for s in scs) + 1000, max_scenes=8)
    ids = [e.add_scene(s, cap=s.n + 200, stir_amp=(300 if i == 1 else 0)) for i, s in enumerate(scs)]
    refs = [oracle3(s.n + 200).load_scene(s, 300 if i == 1 else 0) for i, s in enumerate(scs)]
    e.step(6)
    for r in refs:
        r.step(6)
    for i, r in zip(ids, refs):
        same(e, r, i)
    # remove one, add another mid-run; the others carry on unchanged
    e.remove_scene(ids[2])
    extra = tables3d.initial_state(4000, 'pool', 14, 18, 14)
    j = e.add_scene(extra)
    rj = oracle3(extra.n).load_scene(extra)
    e.step(5)
    for i, r in zip(ids, refs):
        if i != ids[2]:
            r.step(5)
            same(e, r, i)
    rj.step(5)
    same(e, rj, j)


def test_large_dam_break_block():
    # the 262,144-particle block of the bench, ten substeps bit-exact
    sc = tables3d.dam3d_large()
    g, r = both(sc, iters=4)
    for k in (3, 7):
        g.step(k)
        r.step(k)
        same(g, r)


def test_bad_input_is_refused():
    from sunaengine_gb300.engine import EngineError
    e = Engine3D(max_particles=100)
    with pytest.raises(EngineError):
        e.step(1)
    sc = tables3d.initial_state(50, 'pool', 60, 20, 20)
    with pytest.raises(EngineError):
        e.load_scene(sc)
    sc = tables3d.initial_state(200, 'pool', 20, 20, 20)
    with pytest.raises(EngineError):
        e.load_scene(sc)
    sc = tables3d.initial_state(50, 'pool', 20, 20, 20)
    sc.mat[3] = 99
    with pytest.raises(EngineError):
        e.load_scene(sc)


@pytest.mark.parametrize('lanes', [1, 2, 4])
@pytest.mark.parametrize('name,n', [('pool', 16000), ('overdense', 24000)])
def test_lane_split_gathers_are_exact(lanes, name, n):
    sc = tables3d.initial_state(n, name)
    g = Engine3D(max_particles=sc.n, iters=4, lanes=lanes, debug=(lanes == 2)).load_scene(sc, stir_amp=500)
    r = oracle3(sc.n, 4).load_scene(sc, stir_amp=500)
    for k in (1, 4, 10):
        g.step(k)
        r.step(k)
    same(g, r)
    if lanes == 2:
        assert np.array_equal(g.debug_counters(), r.debug_counters())


@pytest.mark.parametrize('debug,brk', [(False, 4 * 65536), (True, 4 * 65536), (False, 70000)])
def test_bonds_match_oracle(debug, brk):
    """Build-defined 3D bonds on the GPU against the oracle: chain, state,
    bond rows (tombstones included: brk 70000 breaks some) and, in the debug
    build, the fixed-point event counters."""
    sc = tables3d.column_fast(16, 16, 16, 20, 20, 20)
    rows = tables3d.bond_rows(sc, tables3d.lattice_bonds(16, 16, 16, 600, 7))
    g, r = both(sc, iters=4, debug=debug)
    g.write_bonds(rows, 32768, brk)
    r.write_bonds(rows, 32768, brk)
    for k in (1, 5, 20, 14):
        g.step(k)
        r.step(k)
        same(g, r)
    assert np.array_equal(g.read_bonds(), r.read_bonds())
    if debug:
        assert np.array_equal(g.debug_counters(), r.debug_counters())


def test_bonds_refused_and_cleared():
    from sunaengine_gb300.engine import EngineError
    sc = tables3d.column_fast(8, 8, 8, 12, 12, 12)
    rows = tables3d.bond_rows(sc, tables3d.lattice_bonds(8, 8, 8, 40, 3)).reshape(-1, 6, 2)
    g = Engine3D(max_particles=sc.n).load_scene(sc)
    bad = rows.copy()
    bad[0, 0, 1] = 100  # rest length below the minimum
    with pytest.raises(EngineError):
        g.write_bonds(bad, 32768, 0)
    with pytest.raises(EngineError):
        g.write_bonds(rows, 70000, 0)  # stiffness above 1.0
    g.write_bonds(rows, 32768, 0)
    assert (g.read_bonds().reshape(-1, 6, 2)[:, :, 0] != 0).sum() == 80
    g.load_scene(sc)  # a load clears the scene's bonds
    assert not g.read_bonds().any()
