"""The serving loop on the GPU: every job's result is the same alone and in
the mix (bit-exact digest and chain), served jobs equal the oracle's straight
runs, a scrub equals advancing straight to the scrub point, and device
checkpoints restore scenes exactly."""
import numpy as np
import pytest

from sunaengine_gb300 import serving, tables3d
from sunaengine_gb300.checkpoints import CheckpointPool
from sunaengine_gb300.engine import Batch
from sunaengine_gb300.engine3d import Engine3D

pytestmark = pytest.mark.gpu

BUDGET = 600 << 20


def test_each_job_is_the_same_alone_and_in_the_mix():
    jobs = serving.poisson_jobs(10, rate_hz=0, seed=21, n_lo=4096, n_hi=40000, t_lo=100, t_hi=320)
    s = serving.Server(BUDGET, quantum=25)
    stats = s.run(jobs, realtime=False)
    s.close()
    assert stats['done'] == len(jobs) and stats['jobs_3d'] > 0 and stats['scrubs'] > 0
    for j in jobs:
        k = serving.run_alone(j, BUDGET)
        assert (k.digest, k.chain) == (j.digest, j.chain), f'job {j.jid} ({j.dim}D {j.op}) differs in the mix'


def test_scrub_equals_advancing_straight_to_the_scrub_point():
    for dim in (2, 3):
        j = serving.Job(jid=1, dim=dim, op='scrub', n=9000, target=260, scrub_to=137, seed=77 + dim)
        got = serving.run_alone(j, BUDGET)
        if dim == 2:
            sc, sched = serving.job_scene_2d(j)
            b = Batch(max_particles=sc.n, max_scenes=1)
            sid = b.add_scene(sc, capacity=sc.n)
            for ev in sched:
                b.schedule_impulse(sid, *ev)
            b.step(137)
            want = (b.digest(sid).hex, b.chain_hex(sid))
            b.destroy()
        else:
            sc, amp = serving.job_scene_3d(j)
            e = Engine3D(max_particles=sc.n, iters=4).load_scene(sc, stir_amp=amp, frame=2)
            for q in (1, 36, 100):
                e.step(q)
            want = (e.digest().hex, e.chain_hex())
            e.close()
        assert (got.digest, got.chain) == want


def test_device_checkpoints_restore_exactly():
    pool = CheckpointPool(64 << 20)
    from sunaengine_gb300 import scenes
    sc = scenes.make_scene('pool_v1', w=40, h=14)
    b = Batch(max_particles=sc.n + 64, max_scenes=2)
    sid = b.add_scene(sc)
    b.schedule_impulse(sid, 12, sc.pos[5, 0], sc.pos[5, 1], 5 * 65536, 9000, -4000)
    b.step(8)
    h = b.ckpt_save(sid, pool)
    b.step(20)
    ahead = (b.digest(sid).hex, b.chain_hex(sid), b.read_state(sid).tobytes())
    b.ckpt_load(sid, pool, h)
    assert b.info(sid)['substep_count'] == 8
    b.step(20)
    assert (b.digest(sid).hex, b.chain_hex(sid), b.read_state(sid).tobytes()) == ahead
    sc3 = tables3d.initial_state(6000, 'pool', 16, 22, 16)
    e = Engine3D(max_particles=6000, max_scenes=2).load_scene(sc3, stir_amp=800, frame=2)
    e.step(5)
    h3 = e.ckpt_save(0, pool)
    e.step(11)
    ahead3 = (e.chain_hex(), e.chain())
    e.ckpt_load(0, pool, h3)
    e.step(11)
    assert (e.chain_hex(), e.chain()) == ahead3
    used, cap = pool.usage()
    assert 0 < used <= cap
    pool.free(h)
    pool.free(h3)
    assert pool.usage()[0] == 0


def test_adding_a_scene_keeps_the_others_clocks():
    """A scene's impulse clock lives on the device; adding or removing another
    scene mid-run must not move it."""
    from sunaengine_gb300 import scenes
    a = scenes.make_scene('pool_v1', w=36, h=12)
    other = scenes.make_scene('dambreak_v1')
    ev = [(14, a.pos[3, 0], a.pos[3, 1], 6 * 65536, 12000, 3000), (27, a.pos[40, 0], a.pos[40, 1], 4 * 65536, -9000, 0)]
    solo = Batch(max_particles=a.n, max_scenes=1)
    s0 = solo.add_scene(a)
    for e in ev:
        solo.schedule_impulse(s0, *e)
    solo.step(40)
    want = (solo.digest(s0).hex, solo.chain_hex(s0))
    mix = Batch(max_particles=a.n + other.n, max_scenes=3)
    sa = mix.add_scene(a)
    for e in ev:
        mix.schedule_impulse(sa, *e)
    mix.step(10)
    sb = mix.add_scene(other)
    mix.step(12)
    mix.remove_scene(sb)
    mix.step(18)
    assert (mix.digest(sa).hex, mix.chain_hex(sa)) == want


@pytest.mark.parametrize('kind', ['bonds', 'bodies'])
def test_engine_device_checkpoints_restore_exactly(kind):
    """sn_ckpt_save / sn_ckpt_load on the single-scene engine: after a load,
    the next substeps repeat the ones that followed the save bit for bit
    (state, chain, bond rows, body records, rest offsets, clocks)."""
    from sunaengine_gb300 import scenes
    from sunaengine_gb300.engine import Engine
    pool = CheckpointPool(64 << 20)
    if kind == 'bonds':
        sc = scenes.make_scene('stretch_v1')
        e = Engine(max_particles=sc.n + 64).load_scene(sc)
    else:
        sc = scenes.rigid_tank()
        e = Engine(max_particles=sc.n + 256).load_scene(sc)
        cx, cy = sc.meta['wheel_centre']
        assert e.make_rigid_body(sc.meta['plank']) == 0
        assert e.make_axis_body(sc.meta['wheel'], cx + 2 * 65536, cy) == 1
    e.step(9)
    assert e.ckpt_bytes() > sc.n * 40
    h = e.ckpt_save(pool)

    def now():
        out = [e.digest().hex, e.chain_hex(), e.read_state().tobytes(), e.read_bonds().tobytes()]
        if kind == 'bodies':
            out += [e.read_bodies().tobytes(), e.read_rest_offsets().tobytes()]
        return out

    e.step(23)
    ahead = now()
    e.ckpt_load(pool, h)
    assert e.substep_count == 9 and e.info()['substep_count'] == 9
    e.step(23)
    assert now() == ahead
    e.check_errors()
    pool.free(h)
    e.destroy()


def test_served_jobs_match_the_oracle(oracle_mod):
    """Jobs served in a mixed stream against the oracle run straight to each
    job's final substep (target, or the scrub point): the three smallest 2D
    jobs (stir impulses at their substep indices) and the two smallest 3D
    jobs (stir phase per frame of 2 substeps)."""
    import oracle
    jobs = serving.poisson_jobs(10, rate_hz=0, seed=21, n_lo=4096, n_hi=40000, t_lo=100, t_hi=320)
    s = serving.Server(BUDGET, quantum=25)
    s.run(jobs, realtime=False)
    s.close()
    two = sorted((j for j in jobs if j.dim == 2), key=lambda j: j.n)[:3]
    three = sorted((j for j in jobs if j.dim == 3), key=lambda j: j.n)[:2]
    assert two and three
    for j in two:
        end = j.scrub_to if j.op == 'scrub' else j.target
        sc, sched = serving.job_scene_2d(j)
        o = oracle.OracleEngine(sc.n + 8, iters=4, threads=16).load_scene(sc)
        at = {}
        for (t, cx, cy, r, ix, iy) in sched:
            at.setdefault(t, []).append((cx, cy, r, ix, iy))
        for k in range(end):
            for ev in at.get(k, ()):
                o.impulse(*ev)
            o.step(1)
        assert (o.digest(), o.chain_hex()) == (j.digest, j.chain), f'2D job {j.jid} ({j.op}, n={sc.n})'
    for j in three:
        end = j.scrub_to if j.op == 'scrub' else j.target
        sc, amp = serving.job_scene_3d(j)
        o = oracle.Oracle3D(sc.n, iters=4, threads=16).load_scene(sc, stir_amp=amp, frame=2)
        o.step(end)
        assert (o.digest(), o.chain_hex()) == (j.digest, j.chain), f'3D job {j.jid} ({j.op}, n={sc.n})'
