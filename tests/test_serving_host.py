"""Host logic of the serving loop on the CPU, with stand-in engines.

The stand-ins keep the engines' calls (add/remove scene, step, checkpoint
save/load, digest) and a toy deterministic state per scene (its own substep
clock folded into a hash), so the tests check what the server itself decides:
admission against slot and pool budgets, quanta that stop exactly on
checkpoint boundaries and targets, scrubs served from checkpoints, and results
independent of the mix.
"""
import hashlib

import pytest

from sunaengine_gb300 import serving
from sunaengine_gb300.engine import EngineError


class FakePool:
    def __init__(self, nbytes):
        self.cap = nbytes
        self.used = 0
        self.recs = {}
        self.next = 1
        self.peak = 0

    def put(self, nbytes, rec):
        r = (nbytes + 255) // 256 * 256
        if self.used + r > self.cap:
            raise EngineError('pool full')
        self.used += r
        self.peak = max(self.peak, self.used)
        h = self.next
        self.next += 1
        self.recs[h] = (r, rec)
        return h

    def free(self, h):
        r, _ = self.recs.pop(h)
        self.used -= r

    def close(self):
        pass


class FakeEngine:
    """Scenes whose state is (seed, substep, chain); step advances every scene."""

    def __init__(self, slots, dim, log):
        self.slots = slots
        self.dim = dim
        self.scenes = {}
        self.log = log
        self.next = 0

    def _used(self):
        return sum(s['cap'] for s in self.scenes.values())

    def _add(self, sc, cap):
        if self._used() + cap > self.slots:
            raise EngineError('no room')
        sid = self.next
        self.next += 1
        seed = int(abs(hash(bytes(sc.pos.tobytes()[:64]))) % (1 << 31))
        self.scenes[sid] = {'cap': cap, 'seed': seed, 'sub': 0, 'chain': '0'}
        return sid

    def add_scene(self, sc, capacity=0, cap=0, stir_amp=0, frame=0):
        return self._add(sc, capacity or cap or sc.n)

    def schedule_impulse(self, sid, *a):
        pass

    def remove_scene(self, sid):
        del self.scenes[sid]

    def step(self, q):
        self.log.append((self.dim, q, len(self.scenes), self._used()))
        assert self._used() <= self.slots
        for s in self.scenes.values():
            for _ in range(q):
                s['sub'] += 1
                s['chain'] = hashlib.sha256(f"{s['chain']}{s['seed']}{s['sub']}".encode()).hexdigest()[:16]

    def sync(self):
        pass

    def ckpt_bytes(self, sid):
        return self.scenes[sid]['cap'] * 40

    def ckpt_save(self, sid, pool):
        s = self.scenes[sid]
        self.log.append(('save', self.dim, s['sub']))
        return pool.put(self.ckpt_bytes(sid), (s['sub'], s['chain']))

    def ckpt_load(self, sid, pool, h):
        s = self.scenes[sid]
        s['sub'], s['chain'] = pool.recs[h][1]

    def digest(self, sid):
        s = self.scenes[sid]

        class D:
            hex = f"{s['seed']:08x}{s['sub']:08x}"
        return D()

    def chain_hex(self, sid):
        return self.scenes[sid]['chain']

    def destroy(self):
        pass

    close = destroy


def make_server(slots2=60000, slots3=60000, pool=1 << 26, log=None):
    log = [] if log is None else log
    eng = (FakeEngine(slots2, 2, log), FakeEngine(slots3, 3, log), FakePool(pool))
    return serving.Server(1 << 30, engines=eng), log


def small_jobs(count=12, seed=3):
    return serving.poisson_jobs(count, rate_hz=0, seed=seed, n_lo=1000, n_hi=12000, t_lo=100, t_hi=450)


def test_request_stream_is_seeded_and_in_range():
    a = serving.poisson_jobs(50, 4.0, seed=9)
    b = serving.poisson_jobs(50, 4.0, seed=9)
    assert [(j.n, j.target, j.op, j.scrub_to, j.dim, j.arrival) for j in a] == \
           [(j.n, j.target, j.op, j.scrub_to, j.dim, j.arrival) for j in b]
    assert all(4096 <= j.n <= 262144 and 100 <= j.target <= 2000 for j in a)
    assert all(0 <= j.scrub_to < j.target for j in a if j.op == 'scrub')
    assert all(x.arrival <= y.arrival for x, y in zip(a, a[1:]))
    assert {j.dim for j in a} == {2, 3} and {j.op for j in a} == {'advance', 'scrub'}


def test_all_jobs_finish_and_match_their_solo_runs():
    jobs = small_jobs()
    s, log = make_server(slots2=30000, slots3=30000)
    stats = s.run(jobs, realtime=False)
    assert stats['done'] == len(jobs) and not s.active and s.reserved == 0
    assert s.pool.used == 0
    # more than one job ran at once (continuous batching), and the budget held
    assert max(e[2] for e in log if e[0] in (2, 3)) > 1
    for j in jobs:
        solo, _ = make_server()
        k = serving.Job(jid=j.jid, dim=j.dim, op=j.op, n=j.n, target=j.target, scrub_to=j.scrub_to, seed=j.seed)
        solo.run([k], realtime=False)
        assert (k.digest, k.chain) == (j.digest, j.chain)


def test_scrub_equals_advancing_to_the_scrub_point():
    jobs = [j for j in small_jobs(30, seed=11) if j.op == 'scrub'][:4]
    assert jobs
    for j in jobs:
        s, _ = make_server()
        s.run([j], realtime=False)
        a = serving.Job(jid=j.jid, dim=j.dim, op='advance', n=j.n, target=j.scrub_to, scrub_to=j.scrub_to,
                        seed=j.seed)
        if a.target == 0:
            continue
        s2, _ = make_server()
        s2.run([a], realtime=False)
        assert (a.digest, a.chain) == (j.digest, j.chain)


def test_checkpoints_land_on_boundaries_and_quanta_never_overshoot():
    jobs = small_jobs(8, seed=5)
    s, log = make_server()
    s.run(jobs, realtime=False)
    saves = [e for e in log if e[0] == 'save']
    assert saves and all(e[2] % s.ckpt_every == 0 for e in saves)
    assert all(e[1] <= s.quantum for e in log if e[0] in (2, 3))


def test_admission_waits_for_room():
    jobs = small_jobs(10, seed=7)
    s, log = make_server(slots2=14000, slots3=14000, pool=1 << 30)
    s.run(jobs, realtime=False)
    assert all(e[3] <= 14000 for e in log if e[0] in (2, 3))
    assert all(j.digest for j in jobs)


def test_a_job_that_can_never_fit_is_reported():
    s, _ = make_server(slots2=500, slots3=500)
    with pytest.raises(EngineError):
        s.run(small_jobs(2), realtime=False)
