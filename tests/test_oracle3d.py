"""The 3D oracle and tables on the CPU.

The reference's 3D page ships no golden digests, so these pin the restatement
by construction checks: the host tables against the values their build implies,
invariances the solver guarantees (thread count, particle-order permutation of
H_set when nothing saturates or truncates), and the reference's own controls
(the overdense scene must truncate; the stir phase is fixed per runSubsteps
call, 3d/app.js:700-714).
"""
import numpy as np
import pytest

from sunaengine_gb300 import tables3d


def oracle3(n=70000, iters=3, threads=8):
    import oracle
    return oracle.Oracle3D(n, iters=iters, threads=threads)


def test_kernel_and_wall_tables():
    l = tables3d.luts3d()
    N, PN = tables3d.LUT_N, tables3d.PLANE_N
    W, G, PW, PG = l[:N], l[N:2 * N], l[2 * N:2 * N + PN], l[2 * N + PN:]
    assert l.size == 2 * N + 2 * PN
    # the density kernel is poly6-shaped: positive, non-increasing, zero at r^2 >= h^2 (ui = 2048)
    assert W[0] == 203360 and np.all(np.diff(W) <= 0) and W[-1] == 0 and W[1500] > 0
    # the gradient table's r = 0 entry is copied from the first non-zero one (3d/app.js:107-110)
    assert G[0] == G[1] > 0 and G[-1] == 0
    # the wall half-space: density and push fall to zero at one smoothing length
    assert np.all(np.diff(PW) <= 0) and PW[-1] == 0 and PW[0] > 0
    assert PG[0] > 0 and PG[-1] == 0
    # lattice sum at rest spacing reproduces RHO0 to rounding (SW normalisation)
    sp = 1.0
    tot = 0
    for i in range(-2, 3):
        for j in range(-2, 3):
            for k in range(-2, 3):
                r2 = (i * i + j * j + k * k) * sp * sp
                if r2 < 4.0:
                    tot += int(W[int(r2 * 512)])
    assert abs(tot - tables3d.RHO0) < 64


def test_ball_tables():
    w, g = tables3d.ball_tables(3.0)
    # inside the sphere the wall table's contact value; beyond R + h nothing
    assert w[0] == tables3d.luts3d()[2 * tables3d.LUT_N]
    r = np.sqrt(np.arange(1024) * 4096) / 256
    assert np.all(w[r - 3.0 >= 2.0] == 0) and np.all(g[r - 3.0 >= 2.0] == 0)
    assert g[0] == 0 and g.max() <= 1 << 24


def test_js_round_is_math_round():
    assert [tables3d.js_round(x) for x in (0.5, 1.5, -0.5, -1.5, 2.4999, -2.5000001)] == [1, 2, 0, -1, 2, -3]


def test_initial_state_matches_the_page_layout():
    sc = tables3d.initial_state(16000, 'pool')
    assert sc.n == 16000 and sc.pos.shape == (16000, 3)
    # bx = floor(56 * 0.55) = 30 columns in x, first particle at 1.5 wu plus jitter
    assert abs(int(sc.pos[0, 0]) - 98304) <= 4096 and abs(int(sc.pos[29, 0]) - (98304 + 29 * 65536)) <= 4096
    lay = tables3d.initial_state(12000, 'layers')
    assert set(np.unique(lay.mat)) == {0, 1, 2}
    big = tables3d.dam3d_large()
    col = tables3d.column(64, 64, 64, 48, 40, 48)
    assert big.n == 262144 and np.array_equal(big.pos, col.pos)


def test_thread_count_invariance_and_clean_counters():
    sc = tables3d.initial_state(8000, 'pool', 20, 24, 20)
    a = oracle3(threads=1).load_scene(sc)
    b = oracle3(threads=8).load_scene(sc)
    a.step(25)
    b.step(25)
    assert a.chain_hex() == b.chain_hex() and a.fnv_hex() == b.fnv_hex()
    assert not a.debug_counters().any()


def test_overdense_scene_truncates_neighbour_lists():
    o = oracle3().load_scene(tables3d.initial_state(20000, 'overdense'))
    o.step(1)
    assert o.debug_counters()[6] > 0


def test_permutation_keeps_h_set():
    sc = tables3d.initial_state(6000, 'pool', 20, 24, 20)
    rng = np.random.default_rng(7)
    perm = rng.permutation(sc.n)
    ps = tables3d.Scene3D(n=sc.n, pos=sc.pos[perm].copy(), vel=sc.vel[perm].copy(), mat=sc.mat[perm].copy(),
                          gx=sc.gx, gy=sc.gy, gz=sc.gz)
    a = oracle3().load_scene(sc)
    b = oracle3().load_scene(ps)
    a.step(30)
    b.step(30)
    assert not a.debug_counters().any() and not b.debug_counters().any()
    assert a.digest()[:32] == b.digest()[:32]
    assert a.digest()[32:] != b.digest()[32:]
    sa = a.read_state().reshape(-1, 8)
    sb = b.read_state().reshape(-1, 8)
    assert np.array_equal(sa[perm], sb)


def test_stir_phase_is_fixed_per_call():
    sc = tables3d.initial_state(4000, 'pool', 16, 20, 16)
    runs = []
    for amp, calls in ((0, (2, 2)), (0, (1, 1, 1, 1)), (900, (2, 2)), (900, (1, 1, 1, 1))):
        o = oracle3().load_scene(sc, stir_amp=amp)
        for c in calls:
            o.step(c)
        runs.append(o.chain_hex())
    assert runs[0] == runs[1]
    assert runs[2] != runs[3] and runs[2] != runs[0]


def test_spawn_and_ball_inputs():
    sc = tables3d.initial_state(3000, 'pool', 16, 20, 16)
    o = oracle3(n=3100).load_scene(sc)
    o.step(4)
    seed = tables3d.SpawnSeed()
    pos = seed.positions(16.0, 30.0, 16.0, 150, 3.0)
    assert np.all(np.linalg.norm(pos / 65536.0 - [16.0, 30.0, 16.0], axis=1) <= 2.4 + 1e-6)
    assert o.spawn(pos, np.full(150, 3, np.uint32)) == 100  # capacity 3100
    o.set_ball(True, 8 * 65536, 6 * 65536, 8 * 65536, 3.0)
    before = o.read_state().reshape(-1, 8)
    o.step(6)
    after = o.read_state().reshape(-1, 8)
    assert o.n == 3100 and not np.array_equal(before, after[:3100])
    # the spawned particles start at rest where they were put, then move
    assert not np.array_equal(after[3000:, :3], pos) and np.all(after[3000:, 3] == 3)
