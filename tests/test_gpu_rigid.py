"""§20 rigid bodies on the GPU against the oracle, through the C ABI.

Every comparison is bit-exact: the chain after each batch of substeps, the
state words, the body records, the rest offsets and (debug builds) the
debug counters."""
import numpy as np
import pytest

from sunaengine_gb300 import data, scenes
from sunaengine_gb300.engine import Engine

import test_oracle_rigid as t

pytestmark = pytest.mark.gpu
ONE = 65536


def both(sc, mats=None, debug=True, lanes=0, extra=256):
    g = Engine(max_particles=sc.n + extra, debug=debug, mats=mats, lanes=lanes).load_scene(sc)
    r = t.oracle(sc, mats=mats, threads=16)
    return g, r


def same(g, r, debug=True):
    assert g.chain_hex() == r.chain_hex()
    assert np.array_equal(g.read_state(), r.read_state())
    assert np.array_equal(g.read_bodies(), r.read_bodies())
    assert np.array_equal(g.read_rest_offsets(), r.read_rest_offsets())
    if debug:
        assert np.array_equal(g.debug_counters(), r.debug_counters())
    g.check_errors()


def run(g, r, ks=(1, 2, 5, 12, 30)):
    for k in ks:
        g.step(k)
        r.step(k)
        assert g.chain_hex() == r.chain_hex(), f'diverged by substep {r.substep_count}'


def test_free_and_axis_bodies_in_water():
    sc = scenes.rigid_tank()
    g, r = both(sc)
    cx, cy = sc.meta['wheel_centre']
    for x in (g, r):
        assert x.make_rigid_body(sc.meta['plank']) == 0
        assert x.make_axis_body(sc.meta['wheel'], cx + 2 * ONE, cy) == 1
    same(g, r)
    run(g, r, (1, 2, 5, 12, 30, 60, 90))
    same(g, r)
    assert g.read_bodies()[0][5] > 20 * ONE


@pytest.mark.parametrize('lanes', [1, 2, 4, 8])
def test_release_build_and_lane_splits(lanes):
    # release builds split the friction lists over `lanes` and give each
    # member a lane group for the seal-contact search; the plank meets the
    # held rail between substeps 20 and 60 (26 contacts on the oracle)
    sc = scenes.rigid_tank(seed=0x5151)
    g, r = both(sc, debug=False, lanes=lanes)
    for x in (g, r):
        x.make_rigid_body(sc.meta['plank'])
        x.make_rigid_body(sc.meta['wheel'])
    run(g, r, (3, 17, 40))
    same(g, r, debug=False)


def test_dry_symmetric_body_and_centroid_axle():
    sc = scenes.rigid_tank(plank='', rail=False, water=False)
    g, r = both(sc)
    for x in (g, r):
        x.make_rigid_body(sc.meta['wheel'])
    run(g, r, (10, 50, 100))
    same(g, r)
    assert g.read_bodies()[0][8] == 0
    g2, r2 = both(sc)
    for x in (g2, r2):
        x.make_axis_body(sc.meta['wheel'], *sc.meta['wheel_centre'])
    run(g2, r2, (100, 100))
    same(g2, r2)
    assert g2.read_bodies()[0][8] == 0


def test_user_drive_and_drivers():
    sc = scenes.rigid_tank(rail=False)
    g, r = both(sc)
    cx, cy = sc.meta['wheel_centre']
    for x in (g, r):
        x.make_rigid_body(sc.meta['plank'], user=True)
        x.make_axis_body(sc.meta['wheel'], cx, cy - ONE, user=True)
        x.set_user_drive(700, -300)
    run(g, r, (4, 8))
    same(g, r)
    R0 = g.read_bodies()[0]
    for x in (g, r):
        x.set_body_driver(0, 1 | 4 | 256, [R0[4] + ONE, 0, 5000000, 0, 0, 0, 0, 0, 40000])
        x.set_body_driver(1, 32 | 64, [0, 0, 0, 0, 0, 3000000, 900, 0, 0])
    run(g, r, (3, 9))
    same(g, r)
    for x in (g, r):
        x.set_body_user(0, False)
        x.clear_body_drivers()
        x.set_user_drive(0, 0)
    run(g, r, (10,))
    same(g, r)


def _ice_mats():
    m = data.mats().copy()
    m[data.mat_id('ICE'), data.MAT_FIELDS.index('meltPt')] = 10 * ONE
    return m


@pytest.mark.parametrize('cold', [32, 3])
def test_members_leave_and_bodies_dissolve(cold):
    m = _ice_mats()
    sc = scenes.rigid_tank(plank='ICE')
    pl = sc.meta['plank']
    tt = np.full(sc.n, scenes.AMBIENT, np.int32)
    tt[pl[:cold]] = -10 * ONE
    sc.temp = tt
    g, r = both(sc, mats=m)
    for x in (g, r):
        x.make_rigid_body(pl)
        x.make_rigid_body(sc.meta['wheel'])
    run(g, r, (1, 1, 8, 30))
    same(g, r)
    assert g.read_bodies()[0][0] == (1 if cold >= 4 else 0)


def test_erase_repair_and_gesture_promotion():
    sc = scenes.rigid_tank(rail=False)
    g, r = both(sc)
    for x in (g, r):
        x.make_rigid_body(sc.meta['plank'])
        x.make_rigid_body(sc.meta['wheel'])
    run(g, r, (6,))
    keep = np.ones(sc.nFluid, bool)
    keep[sc.meta['plank'][5:15]] = False
    keep[sc.meta['wheel'][:-2]] = False
    keep[sc.meta['water'][::7]] = False
    assert g.erase(keep) == r.erase(keep)
    same(g, r)
    run(g, r, (1, 9))
    metal = data.mat_id('WOOD')
    pts = [{'x': (30 + c) * ONE + ONE // 2, 'y': (8 + rr) * ONE + ONE // 2, 'mat': metal}
           for rr in range(4) for c in range(6)]
    for x in (g, r):
        x.begin_weld_group()
        x.spawn_fluid(pts, no_weld=False)
        assert x.end_weld_group_and_promote() == 1
    same(g, r)
    run(g, r, (1, 4, 20))
    same(g, r)


def test_restore_and_drag():
    sc = scenes.rigid_tank()
    g, r = both(sc)
    for x in (g, r):
        x.make_rigid_body(sc.meta['plank'])
        x.make_axis_body(sc.meta['wheel'], *sc.meta['wheel_centre'])
    run(g, r, (20,))
    tag = int(g.read_bodies()[0][1])
    for x in (g, r):
        assert x.drag_body(tag, 40 * ONE, 10 * ONE, -2000, 500)
    run(g, r, (1, 10))
    same(g, r)
    # keyframe: state, stAcc, bonds, bodies, rest offsets, formation clock
    key = (g.read_state(), g.read_scratch(), g.read_bonds(), g.read_bodies(), g.read_rest_offsets())
    clk = g.info()['formation_clock']
    g.step(15)
    r.step(15)
    ahead = g.read_state().copy(), g.read_bodies().copy()
    h = Engine(max_particles=sc.n + 256, debug=True).load_scene(sc)
    h.write_state(key[0], key[1])
    h.write_bonds(key[2])
    h.restore_bodies(key[3], key[4])
    h.set_formation_clock(clk, False)
    h.step(15)
    assert np.array_equal(h.read_state(), ahead[0])
    assert np.array_equal(h.read_bodies(), ahead[1])
    assert g.dissolve_all_bodies() == r.dissolve_all_bodies()
    run(g, r, (5,))
    assert g.body_count == 0 == r.body_count
    assert np.array_equal(g.read_state(), r.read_state())


def test_split_and_loose_promotion_match():
    from sunaengine_gb300 import authoring
    sc = scenes.rigid_tank()
    g, r = both(sc)
    cx, cy = sc.meta['wheel_centre']
    for x in (g, r):
        x.make_rigid_body(sc.meta['plank'], user=True)
        x.make_axis_body(sc.meta['wheel'], cx + ONE, cy)
    run(g, r, (2, 7))
    cut = [{'x0': 16 * ONE, 'y0': 5 * ONE, 'x1': 17 * ONE, 'y1': 40 * ONE},
           {'x0': 40 * ONE, 'y0': 20 * ONE, 'x1': 52 * ONE, 'y1': 21 * ONE}]
    assert authoring.split_disconnected_bodies(g, cuts=cut) == authoring.split_disconnected_bodies(r, cuts=cut)
    same(g, r)
    run(g, r, (1, 10))
    same(g, r)
    s2 = scenes.rigid_tank(wheel='', rail=False, plank='STONE', seed=0x3131)
    g2, r2 = both(s2)
    run(g2, r2, (1,))
    w = [{'slot': s2.meta['plank'][7], 'mat': data.mat_id('STONE')}]
    assert authoring.promote_loose_rigid_components(g2, eligible=w) == \
        authoring.promote_loose_rigid_components(r2, eligible=w) == 1
    same(g2, r2)
    run(g2, r2, (1, 12))
    same(g2, r2)


def test_exact_suna_save_loads_on_both_engines():
    import oracle as o
    from sunaengine_gb300 import authoring, materials
    sc = scenes.rigid_tank()
    e = Engine(max_particles=sc.n + 256, debug=True).load_scene(sc)
    it = materials.Interner(e)
    row = it.intern(data.mat_id('SAND'), materials.MOD['E'])['rowId']
    e.spawn_fluid([{'x': (50 + c) * ONE, 'y': 6 * ONE, 'mat': row} for c in range(8)], no_weld=False)
    e.make_rigid_body(sc.meta['plank'])
    e.make_axis_body(sc.meta['wheel'], *sc.meta['wheel_centre'])
    e.step(25)
    text = authoring.save_suna(e, sc, it)
    g, _ = authoring.load_suna(text, lambda: Engine(max_particles=sc.n + 256, debug=True))
    r, _ = authoring.load_suna(text, lambda: o.OracleEngine(sc.n + 256, threads=16))
    e.write_state(e.read_state(), np.zeros(e.n * 2, np.int32))   # a save carries no scratch
    for x in (e, g, r):
        x.step(20)
    assert np.array_equal(g.read_state(), r.read_state()) and np.array_equal(g.read_state(), e.read_state())
    assert np.array_equal(g.read_bodies(), r.read_bodies())
    assert np.array_equal(g.debug_counters(), r.debug_counters())


def test_bodies_in_a_batch_match_each_scene_alone():
    """Rigid bodies in a batched world: two rigid tanks (different seeds, one
    with a held rail, one with a driven wheel) in one batch, each against its
    own oracle; removing the first keeps the second exact."""
    from sunaengine_gb300.engine import Batch
    a = scenes.rigid_tank(seed=0x1111)
    c = scenes.rigid_tank(seed=0x2222, rail=False)
    bt = Batch(max_particles=a.n + c.n + 512, max_scenes=3)
    ia, ic = bt.add_scene(a), bt.add_scene(c)
    ra, rc = t.oracle(a, threads=16), t.oracle(c, threads=16)
    assert bt.make_rigid_body(ia, a.meta['plank']) == 0 and ra.make_rigid_body(a.meta['plank']) == 0
    assert bt.make_rigid_body(ia, a.meta['wheel']) == 1 and ra.make_rigid_body(a.meta['wheel']) == 1
    cx, cy = c.meta['wheel_centre']
    assert bt.make_axis_body(ic, c.meta['wheel'], cx, cy) == 0 and rc.make_axis_body(c.meta['wheel'], cx, cy) == 0
    spin = [0, 0, 0, 0, 0, 40000, 0, 0, 0]                # RD_HAS_W (32): drive the wheel's spin
    bt.set_body_driver(ic, 0, 32, spin)
    rc.set_body_driver(0, 32, spin)
    assert bt.body_count(ia) == 2 and bt.body_count(ic) == 1
    for k in (5, 20, 35):
        bt.step(k)
        ra.step(k)
        rc.step(k)
        assert bt.chain_hex(ia) == ra.chain_hex() and bt.chain_hex(ic) == rc.chain_hex()
    assert np.array_equal(bt.read_bodies(ia), ra.read_bodies())
    assert np.array_equal(bt.read_bodies(ic), rc.read_bodies())
    assert np.array_equal(bt.read_rest_offsets(ic), rc.read_rest_offsets())
    bt.remove_scene(ia)
    bt.step(20)
    rc.step(20)
    assert bt.chain_hex(ic) == rc.chain_hex()
    assert np.array_equal(bt.read_bodies(ic), rc.read_bodies())
    bt.check_errors()


def test_device_checkpoint_carries_bodies():
    """A checkpoint of a scene with bodies (records, drivers, rest offsets)
    rewinds it exactly: replaying from it repeats the chain and the body
    records, also after the bodies were dissolved in between; a checkpoint
    taken before the bodies existed removes them again."""
    from sunaengine_gb300.checkpoints import CheckpointPool
    from sunaengine_gb300.engine import Batch
    a = scenes.rigid_tank(seed=0x3333)
    bt = Batch(max_particles=a.n + 256, max_scenes=2)
    ia = bt.add_scene(a)
    pool = CheckpointPool(64 << 20)
    h0 = bt.ckpt_save(ia, pool)                   # no bodies yet
    bt.make_rigid_body(ia, a.meta['plank'])
    cx, cy = a.meta['wheel_centre']
    bt.make_axis_body(ia, a.meta['wheel'], cx, cy)
    bt.set_body_driver(ia, 1, 32, [0, 0, 0, 0, 0, 30000, 0, 0, 0])
    bt.step(15)
    h1 = bt.ckpt_save(ia, pool)
    bt.step(40)
    want = (bt.chain_hex(ia), bt.read_bodies(ia).copy(), bt.read_rest_offsets(ia).copy())
    bt.dissolve_all_bodies(ia)
    bt.step(5)
    bt.ckpt_load(ia, pool, h1)
    assert bt.body_count(ia) == 2
    bt.step(40)
    assert bt.chain_hex(ia) == want[0]
    assert np.array_equal(bt.read_bodies(ia), want[1])
    assert np.array_equal(bt.read_rest_offsets(ia), want[2])
    bt.ckpt_load(ia, pool, h0)
    assert bt.body_count(ia) == 0
    r = t.oracle(a, threads=16)
    bt.step(10)
    r.step(10)
    assert bt.chain_hex(ia) == r.chain_hex()
    bt.check_errors()
    pool.close()
