"""GPU parity: the CUDA engine, called through the C ABI, against the oracle.

Bar: bit-exact. Every comparison is of the reference's own state digest
(H_set || H_slot, src/hash/statehash.js:80-159) and of the per-substep chain,
so one differing bit in any particle word on any substep fails the test.
"""
import numpy as np
import pytest

from sunaengine_gb300 import data, scenes
from sunaengine_gb300.engine import Batch, Engine, EngineError

from test_oracle import GOLDEN_CHAIN, GOLDEN_CHECKPOINTS

pytestmark = pytest.mark.gpu

M = data.mat_id
ONE = scenes.ONE


def _pool(mat, w=30, h=10):
    return scenes.make_scene('pool_v1', w=w, h=h, mat=M(mat))


def _mixed_thermal():
    """OIL pool with a hot FIRE blob and a WATER strip: ignition, burning,
    boiling to STEAM, smoke venting (split to ASH), all through `thermal`."""
    sc = scenes.make_scene('pool_v1', w=40, h=12, mat=M('OIL'))
    nf = sc.nFluid
    mat = sc.matId.copy()
    temp = np.full(sc.n, scenes.AMBIENT, np.int32)
    fuel = np.zeros(sc.n, np.int32)
    fuel[:nf] = scenes.deg(100)
    for i in range(nf):
        x, y = sc.pos[i]
        if x < 18 * ONE:
            mat[i] = M('WATER')
            temp[i] = scenes.deg(130 if i % 3 == 0 else 97)
            fuel[i] = 0
        elif x < 22 * ONE:
            mat[i] = M('STEAM')
            temp[i] = scenes.deg(50)
            fuel[i] = 0
        elif 30 * ONE <= x < 36 * ONE and y < 64 * ONE:
            mat[i] = M('FIRE')
            temp[i] = scenes.deg(900)
            fuel[i] = 100000 * (1 + i % 4)
    sc.matId = mat.astype(np.uint32)
    sc.temp = temp
    sc.fuel = fuel
    return sc


def _hot_rice():
    sc = _pool('RICE', 30, 12)
    sc.temp = np.full(sc.n, scenes.deg(90), np.int32)
    return sc


def _walls_only():
    """No fluid at all: the boundary block alone (nFluid = 0)."""
    return scenes._assemble([], np.zeros(0, np.uint32), scenes.boundary_ring(40, 24, 20), 40, 24, 'walls_only')


def _one_drop():
    """A single WATER particle falling onto the floor of an empty box."""
    return scenes._assemble([(20 * ONE + 777, 5 * ONE)], np.zeros(1, np.uint32), scenes.boundary_ring(40, 24, 20),
                            40, 24, 'one_drop')


def _anchored():
    sc = _pool('SAND', 30, 10)
    fl = np.zeros(sc.n, np.uint32)
    fl[: sc.nFluid: 7] = 4  # FLAG_ANCHOR on every 7th particle
    sc.flags = fl
    return sc


SCENES = {
    'dambreak_v1': (lambda: scenes.make_scene('dambreak_v1'), 40),
    'overdense_v1': (lambda: scenes.make_scene('overdense_v1'), 25),
    'pool_water': (lambda: _pool('WATER', 40, 12), 40),
    'droplet_oil': (lambda: scenes.make_scene('droplet_v1', mat=M('OIL')), 40),
    'stretch_gel': (lambda: scenes.make_scene('stretch_v1'), 60),
    'sand_pool': (lambda: _pool('SAND', 30, 12), 40),
    'rice_pool': (_hot_rice, 40),
    'tar_pool': (lambda: _pool('TAR', 30, 10), 30),
    'thermal_mix': (_mixed_thermal, 60),
    'anchored_sand': (_anchored, 30),
    'two_fluid_48': (lambda: scenes.large_two_fluid(side=48, band=8), 30),
    'lattice_dambreak_64': (lambda: scenes.lattice_dambreak(), 30),
    'walls_only': (_walls_only, 10),
    'one_drop': (_one_drop, 60),
}


def _pair(sc, debug=True, iters=4):
    cap = max(8192, sc.n + 64)
    gpu = Engine(max_particles=cap, debug=debug, iters=iters).load_scene(sc)
    import oracle
    ref = oracle.OracleEngine(cap, iters=iters, threads=8).load_scene(sc)
    return gpu, ref


def test_golden_dambreak_chain():
    e = Engine(max_particles=8192, debug=True).load_scene(scenes.make_scene('dambreak_v1'))
    done = 0
    for c, want in GOLDEN_CHECKPOINTS.items():
        e.step(c - done)
        done = c
        assert e.digest().hex == want, f'checkpoint {c}'
    assert e.chain_hex() == GOLDEN_CHAIN
    assert not e.debug_counters().any()
    e.check_errors()


@pytest.mark.parametrize('name', sorted(SCENES))
def test_every_substep_matches_oracle(name, oracle_mod):
    make, steps = SCENES[name]
    sc = make()
    gpu, ref = _pair(sc)
    assert gpu.digest().hex == ref.digest()
    for s in range(1, steps + 1):
        gpu.step(1)
        ref.step(1)
        g, r = gpu.digest().hex, ref.digest()
        assert g == r, f'{name}: substep {s}'
    assert gpu.chain_hex() == ref.chain_hex()
    assert np.array_equal(gpu.debug_counters(), ref.debug_counters())
    assert np.array_equal(gpu.read_state(), ref.read_state())
    if sc.n:
        assert np.array_equal(gpu.read_bonds(), ref.read_bonds())
    gpu.check_errors()


@pytest.mark.parametrize('lanes', [1, 2, 4, 8])
def test_lane_split_is_exact(lanes, oracle_mod):
    import oracle
    sc = scenes.make_scene('stretch_v1')
    e = Engine(max_particles=sc.n + 64, lanes=lanes).load_scene(sc)
    r = oracle.OracleEngine(sc.n + 64, threads=8).load_scene(sc)
    sc2 = scenes.large_two_fluid(side=40, band=8)
    e2 = Engine(max_particles=sc2.n + 64, lanes=lanes).load_scene(sc2)
    r2 = oracle.OracleEngine(sc2.n + 64, threads=8).load_scene(sc2)
    for x in (e, r, e2, r2):
        x.step(24)
    assert e.chain_hex() == r.chain_hex()
    assert e2.chain_hex() == r2.chain_hex()


def test_release_build_matches_debug_build(oracle_mod):
    sc = scenes.make_scene('overdense_v1')
    a = Engine(max_particles=8192, debug=True).load_scene(sc)
    b = Engine(max_particles=8192, debug=False).load_scene(sc)
    a.step(30)
    b.step(30)
    assert a.chain_hex() == b.chain_hex()
    assert not b.debug_counters().any()


@pytest.mark.parametrize('iters', [1, 3, 7])
def test_iteration_count_option(iters, oracle_mod):
    sc = _pool('WATER', 25, 10)
    gpu, ref = _pair(sc, iters=iters)
    gpu.step(25)
    ref.step(25)
    assert gpu.chain_hex() == ref.chain_hex()


def test_spawn_and_impulse_match_oracle(oracle_mod):
    sc = _pool('WATER', 40, 12)
    gpu, ref = _pair(sc)
    drop = scenes.make_droplet(64 * ONE, 10 * ONE, 3, 3, vy=ONE // 5)
    for s in range(60):
        if s % 8 == 0:
            assert gpu.spawn_fluid([dict(p, mat=0) for p in drop]) == ref.spawn([dict(p, mat=0) for p in drop])
        if s % 10 == 5:
            args = (50 * ONE, 60 * ONE, 6 * ONE, 9000, -12000)
            assert gpu.apply_impulse(*args) == ref.impulse(*args)
        if s == 33:
            # limit binds: only the first 7 hits in slot order are pushed
            assert gpu.apply_impulse(40 * ONE, 62 * ONE, 20 * ONE, -5000, 3000, 7) == \
                ref.impulse(40 * ONE, 62 * ONE, 20 * ONE, -5000, 3000, 7)
        gpu.step(1)
        ref.step(1)
        assert gpu.digest().hex == ref.digest(), f'substep {s}'
    assert gpu.n == ref.n and gpu.n_fluid == ref.n_fluid
    assert gpu.chain_hex() == ref.chain_hex()


def test_impulse_disc_near_ties_match_oracle(oracle_mod):
    """applyImpulse's disc test (src/engine.js:6077-6098) where the reference's
    double rounding decides: particles at |dx| = r ~ 2^27 with dy = 0..11, so
    dx^2 + dy^2 - r^2 = dy^2 (at dy = 1 the exact sum is outside the disc and
    the doubles put it inside), beside particles far inside and far outside."""
    sc = _pool('WATER', 30, 10)
    gpu, ref = _pair(sc)
    st = gpu.read_state().reshape(-1, 8).copy()
    nf = sc.nFluid
    half = nf // 2
    cy = 1000
    for k, r in enumerate([(1 << 27) - 1, (1 << 27) - 37, 3 * (1 << 25) + 5]):
        s = st.copy()
        for i in range(half):
            # two in three on the rim (dx = r, dy = 0..11); the rest at dx = 0,
            # dy ~ 2^27 - 1000 (well inside or well outside, by r)
            rim = (i + k) % 3 != 0
            s[i, 0] = r if rim else 0
            s[i, 1] = cy + (i % 12) if rim else (1 << 27) - (i % 5)
        gpu.write_state_keep_scratch(s.reshape(-1))
        ref.write_state(s.reshape(-1))
        for cx, lim in [(0, 3000), (0, 5), (2 * r, 3000)]:  # cx = 2r: the rim at dx = -r
            assert gpu.apply_impulse(cx, cy, r, 777, -555, lim) == ref.impulse(cx, cy, r, 777, -555, lim)
            assert np.array_equal(gpu.read_state(), ref.read_state()), (r, cx, lim)
        # a disc around the untouched pool: the exact integer decision alone
        args = (20 * ONE, 5 * ONE, 8 * ONE, -300, 900)
        assert gpu.apply_impulse(*args) == ref.impulse(*args)
        assert np.array_equal(gpu.read_state(), ref.read_state())


def test_read_state_into_caller_buffer():
    sc = _pool('WATER', 20, 8)
    e = Engine(max_particles=sc.n + 64).load_scene(sc)
    e.step(3)
    buf = np.full(sc.n * 8 + 5, -1, np.int32)
    got = e.read_state(out=buf)
    assert got.base is buf and np.array_equal(got, e.read_state())
    assert (buf[sc.n * 8:] == -1).all()


def test_spawn_refused_at_capacity():
    sc = _pool('WATER', 10, 5)
    e = Engine(max_particles=sc.n + 2).load_scene(sc)
    n0 = e.n
    assert e.spawn_fluid([{'x': 60 * ONE, 'y': 20 * ONE}] * 3) == n0  # silently unchanged, like the reference
    assert e.spawn_fluid([{'x': 60 * ONE, 'y': 20 * ONE}] * 2) == n0 + 2


def test_keyframe_rejoins_timeline():
    sc = _pool('WATER', 40, 12)
    e = Engine(max_particles=8192).load_scene(sc)
    e.step(60)
    st, scr, clk = e.read_state(), e.read_scratch(), e.formation_clock
    e.step(40)
    ahead = e.digest().hex
    e.load_scene(sc)
    e.write_state(st, scr)
    e.set_formation_clock(clk, False)
    e.step(40)
    assert e.digest().hex == ahead
    # state-only restore (no scratch) is a load boundary: it diverges
    e.load_scene(sc)
    e.write_state(st, None)
    e.set_formation_clock(clk, False)
    e.step(40)
    assert e.digest().hex != ahead


def test_batch_scenes_match_oracle(oracle_mod):
    import oracle
    mk = [lambda: scenes.make_scene('dambreak_v1'), lambda: _pool('SAND', 25, 10),
          lambda: scenes.make_scene('stretch_v1'), lambda: scenes.large_two_fluid(side=40, band=8),
          lambda: scenes.make_scene('droplet_v1', mat=M('OIL'))]
    scs = [f() for f in mk]
    b = Batch(max_particles=sum(s.n for s in scs) + 1024, max_scenes=8, debug=True)
    ids = [b.add_scene(s) for s in scs]
    refs = [oracle.OracleEngine(s.n + 64, threads=8).load_scene(s) for s in scs]
    # impulses at scene-specific substeps
    ev = {ids[0]: [(5, 20 * ONE, 60 * ONE, 5 * ONE, 8000, -9000)], ids[3]: [(7, 20 * ONE, 30 * ONE, 6 * ONE, -7000, 0),
                                                                          (7, 25 * ONE, 30 * ONE, 4 * ONE, 3000, 3000)]}
    for sid, lst in ev.items():
        for (at, cx, cy, r, ix, iy) in lst:
            b.schedule_impulse(sid, at, cx, cy, r, ix, iy)
    for s in range(20):
        for k, sid in enumerate(ids):
            for (at, cx, cy, r, ix, iy) in ev.get(sid, []):
                if at == s:
                    refs[k].impulse(cx, cy, r, ix, iy)
        b.step(1)
        for r in refs:
            r.step(1)
    for k, sid in enumerate(ids):
        assert b.chain_hex(sid) == refs[k].chain_hex(), f'scene {k}'
        assert b.digest(sid).hex == refs[k].digest()
    b.check_errors()


def test_batch_remove_and_add_keeps_others_exact(oracle_mod):
    import oracle
    a, c = _pool('WATER', 30, 10), scenes.make_scene('droplet_v1')
    b = Batch(max_particles=20000, max_scenes=4)
    ia = b.add_scene(a)
    ib = b.add_scene(scenes.make_scene('dambreak_v1'))
    ra = oracle.OracleEngine(a.n + 8, threads=8).load_scene(a)
    b.step(10)
    ra.step(10)
    b.remove_scene(ib)
    ic = b.add_scene(c)
    rc = oracle.OracleEngine(c.n + 8, threads=8).load_scene(c)
    b.step(15)
    ra.step(15)
    rc.step(15)
    assert b.chain_hex(ia) == ra.chain_hex()
    assert b.chain_hex(ic) == rc.chain_hex()


def test_empty_scene_steps_and_hashes():
    sc = scenes._assemble([], np.zeros(0, np.uint32), np.zeros((0, 2), np.int32), 40, 24, 'empty')
    e = Engine(max_particles=1024).load_scene(sc)
    d0 = e.digest().hex
    e.step(5)
    assert e.digest().hex == d0 and e.info()['substep_count'] == 5
    assert e.read_state().size == 0
    e.check_errors()


def test_refuses_bad_input():
    e = Engine(max_particles=1024)
    with pytest.raises(EngineError):
        e.step(1)  # before loadScene
    sc = _pool('WATER', 10, 5)
    bad = sc.copy()
    bad.matId[0] = 99
    with pytest.raises(EngineError):
        e.load_scene(bad)
    flags = sc.copy()
    flags.flags = np.zeros(sc.n, np.uint32)
    flags.flags[0] = 16  # FLAG_RIGID is the engine's to set, never the scene's
    with pytest.raises(EngineError):
        e.load_scene(flags)
    big = scenes.make_scene('dambreak_v1')
    with pytest.raises(EngineError):
        e.load_scene(big)  # n > maxParticles


def test_load_checks_report_the_first_bad_particle():
    """loadScene's per-particle checks run on the device; the refusal names the
    first failing particle and its first failing rule, as the host rules read,
    and a refused load leaves the loaded scene as it was."""
    sc = _pool('WATER', 20, 8)
    e = Engine(max_particles=sc.n + 64).load_scene(sc)
    e.step(3)
    before = e.read_state().copy()
    cases = []
    b1 = sc.copy(); b1.pos = b1.pos.copy(); b1.pos[7, 0] = -5; b1.matId = b1.matId.copy(); b1.matId[40] = 99
    cases.append((b1, 'pos[7]'))
    b2 = sc.copy(); b2.temp = np.full(sc.n, 65536 * 20, np.int32); b2.temp[30] = 1 << 30; b2.fuel = np.zeros(sc.n, np.int32)
    b2.fuel[12] = -1
    cases.append((b2, 'fuel[12]'))
    b3 = sc.copy(); b3.flags = np.zeros(sc.n, np.uint32); b3.flags[5] = 2  # FLAG_DEAD on a WATER (live) row
    cases.append((b3, 'flags[5] sets FLAG_DEAD'))
    for bad, want in cases:
        with pytest.raises(EngineError) as ex:
            e.load_scene(bad)
        assert want in str(ex.value), str(ex.value)
        assert np.array_equal(e.read_state(), before)
    e.load_scene(sc)  # a good load after refused ones
    e.step(3)
    assert np.array_equal(e.read_state(), before)
