"""Authoring edits on the GPU engine against the oracle, op by op."""
import numpy as np
import pytest

from sunaengine_gb300 import authoring, data
from sunaengine_gb300.engine import Engine

import test_authoring as t

pytestmark = pytest.mark.gpu


def test_edit_sequence_matches_oracle():
    sc = t.gel()
    g = Engine(max_particles=sc.n + 64, debug=True).load_scene(sc)
    r = t.oracle(sc)

    def both(fn):
        a, b = fn(g), fn(r)
        assert a == b
        assert g.n == r.n and g.n_fluid == r.n_fluid
        assert np.array_equal(g.read_state(), r.read_state())
        assert np.array_equal(g.read_bonds(), r.read_bonds())

    def steps(k):
        g.step(k)
        r.step(k)
        assert g.chain_hex() == r.chain_hex()

    steps(3)
    st = r.read_state().reshape(-1, 8)
    rubber = data.mat_id('RUBBER')
    cx = int(np.median(st[:sc.nFluid, 0]))
    both(lambda e: authoring.replace_where(e, lambda p: p['mat'] == rubber and p['x'] < cx, 0))
    steps(4)
    st = r.read_state().reshape(-1, 8)
    y0, y1 = int(st[:r.n_fluid, 1].min()) - 4 * t.ONE, int(st[:r.n_fluid, 1].max()) + 4 * t.ONE
    x = int(np.percentile(st[:r.n_fluid, 0], 75))
    both(lambda e: authoring.slice_bonds_many(e, [{'x0': x, 'y0': y0, 'x1': x, 'y1': y1}]))
    steps(4)
    cy = int(np.median(st[:r.n_fluid, 1]))
    both(lambda e: authoring.erase_where(e, lambda p: p['y'] < cy))
    steps(6)
    assert g.digest().hex == r.digest()
    assert list(g.debug_counters()) == list(r.debug_counters())


def test_weld_gestures_and_fusion_match_oracle():
    import test_weld as w
    sc = w.pole_scene()
    g = Engine(max_particles=6000, debug=True).load_scene(sc)
    r = w.oracle(sc)

    def steps(k):
        g.step(k)
        r.step(k)
        assert g.chain_hex() == r.chain_hex()
        assert g.weld_state() == r.weld_state()

    steps(2)
    assert g.begin_weld_group() == r.begin_weld_group()
    for k in range(3):
        assert g.spawn_fluid(w.stroke(30 * w.ONE + k * 3 * w.ONE, 10 * w.ONE, 3), no_weld=False) == \
            r.spawn_fluid(w.stroke(30 * w.ONE + k * 3 * w.ONE, 10 * w.ONE, 3), no_weld=False)
        steps(1)
    assert g.end_weld_group() == r.end_weld_group()
    steps(3)
    g.spawn_fluid(w.stroke(8 * w.ONE, 8 * w.ONE, 4), no_weld=False, own_group=True)
    r.spawn_fluid(w.stroke(8 * w.ONE, 8 * w.ONE, 4), no_weld=False, own_group=True)
    steps(2)
    g.begin_weld_group(), r.begin_weld_group()
    assert g.arm_fuse() == r.arm_fuse()
    band = w.stroke(21 * w.ONE, 25 * w.ONE + w.ONE // 2, 6)
    g.spawn_fluid(band, no_weld=False)
    r.spawn_fluid(band, no_weld=False)
    steps(1)
    g.end_weld_group(), r.end_weld_group()
    steps(5)
    assert np.array_equal(g.read_bonds(), r.read_bonds())
    assert list(g.debug_counters()) == list(r.debug_counters())


def test_device_erase_at_size_matches_oracle():
    """eraseWhere's device compaction on a 65,536-particle two-fluid scene
    (two in three particles of a horizontal band erased): state and counts
    equal to the oracle's right after, chains equal after more substeps."""
    from sunaengine_gb300 import scenes
    sc = scenes.large_two_fluid(side=256)
    g = Engine(max_particles=sc.n + 64).load_scene(sc)
    r = t.oracle(sc)
    for x in (g, r):
        x.step(3)
    st = r.read_state().reshape(-1, 8)
    nf = r.n_fluid
    ys = st[:nf, 1]
    lo, hi = np.percentile(ys, 40), np.percentile(ys, 60)
    keep = ~((ys > lo) & (ys < hi) & (np.arange(nf) % 3 != 0))
    assert g.erase(keep) == r.erase(keep) == int((~keep).sum())
    assert g.n == r.n and g.n_fluid == r.n_fluid
    assert np.array_equal(g.read_state(), r.read_state())
    for x in (g, r):
        x.step(5)
    assert g.chain_hex() == r.chain_hex()
    g.check_errors()


def test_batch_erase_leaves_the_other_scenes_alone():
    """sn_batch_erase on the middle scene of three: the erased scene equals the
    oracle's, the others equal a twin batch that erased nothing."""
    from sunaengine_gb300 import scenes
    from sunaengine_gb300.engine import Batch
    scs = [t.gel(), scenes.make_scene('pool_v1', w=40, h=12), scenes.make_scene('stretch_v1')]
    twins = []
    for _ in range(2):
        b = Batch(max_particles=sum(s.n for s in scs) + 256, max_scenes=3)
        for s in scs:
            b.add_scene(s)
        b.step(4)
        twins.append(b)
    a, b = twins
    r = t.oracle(scs[1])
    r.step(4)
    st = r.read_state().reshape(-1, 8)
    keep = st[:r.n_fluid, 0] < np.median(st[:r.n_fluid, 0])
    assert b.erase(1, keep) == r.erase(keep)
    assert np.array_equal(b.read_state(1), r.read_state())
    for x in (a, b, r):
        x.step(6)
    assert b.chain_hex(1) == r.chain_hex()
    for sid in (0, 2):
        assert b.chain_hex(sid) == a.chain_hex(sid)
        assert np.array_equal(b.read_state(sid), a.read_state(sid))
    for x in (a, b):
        x.check_errors()
        x.destroy()
