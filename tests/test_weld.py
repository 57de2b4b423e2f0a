"""Weld groups and draw-time fusion (src/engine.js:4570-4680, §18.24) on the
CPU oracle: one gesture is one bonding group, a spawn outside a gesture is its
own group, and an armed gesture fuses to existing bonded-family matter."""
import numpy as np

from sunaengine_gb300 import data, scenes

ONE = 65536
RUBBER = data.mat_id('RUBBER')


def oracle(sc, cap=6000):
    import oracle as o
    return o.OracleEngine(cap, threads=8).load_scene(sc)


def stroke(x0, y, n, dx=ONE):
    return [{'x': x0 + i * dx, 'y': y, 'mat': RUBBER} for i in range(n)]


def bond_pairs(e):
    b = e.read_bonds().reshape(e.n_fluid, 48)
    out = set()
    for i in range(b.shape[0]):
        for w in b[i]:
            w = int(w)
            if not w:
                break
            if not (w & 0x40000000):
                out.add((i, w & 0x1ffff))
    return out


def pole_scene():
    """A held RUBBER pole (welded at load) standing in an empty walled box."""
    half = ONE >> 1
    pole = [(20 * ONE + half, (20 + r) * ONE + half) for r in range(12)]
    sc = scenes._assemble(pole, RUBBER, scenes.boundary_ring(48, 40, 36), 48, 40, 'pole')
    sc.flags = np.zeros(sc.n, np.uint32)
    sc.flags[:len(pole)] = 4   # FLAG_ANCHOR
    return sc


def test_one_gesture_is_one_group():
    e = oracle(pole_scene())
    e.step(2)
    tag = e.begin_weld_group()
    assert tag == (2 << 8) and e.weld_state()['weld_hold'] == tag
    first = e.n_fluid
    for k in range(3):
        e.spawn_fluid(stroke(30 * ONE + k * 3 * ONE, 10 * ONE, 3), no_weld=False)
        e.step(1)
    st = e.read_state().reshape(-1, 8)
    assert ((st[first:e.n_fluid, 5].astype(np.uint32) & 0xfff00) == tag).all()
    assert e.end_weld_group() == tag
    e.step(4)
    st = e.read_state().reshape(-1, 8)
    assert ((st[first:e.n_fluid, 5].astype(np.uint32) & 0xfff00) == 0).all()
    pairs = bond_pairs(e)
    # bonds link the three spawn batches into one body
    assert any(first <= i < first + 3 and first + 3 <= j < first + 9 for i, j in pairs)


def test_spawns_outside_a_gesture_are_separate_groups():
    e = oracle(pole_scene())
    e.step(2)
    a = e.n_fluid
    e.spawn_fluid(stroke(30 * ONE, 10 * ONE, 3), no_weld=False)
    b = e.n_fluid
    e.spawn_fluid(stroke(33 * ONE, 10 * ONE, 3), no_weld=False)
    assert e.weld_state()['weld_seq'] == 3
    e.step(3)
    pairs = bond_pairs(e)
    assert not any(a <= i < b <= j for i, j in pairs)


def test_armed_fuse_bonds_to_the_pole():
    e = oracle(pole_scene())
    e.step(2)
    pole = set(range(12))
    e.begin_weld_group()
    e.arm_fuse()
    first = e.n_fluid
    e.spawn_fluid(stroke(21 * ONE, 25 * ONE + ONE // 2, 6), no_weld=False)
    e.step(1)
    pairs = bond_pairs(e)
    assert any(i in pole and j >= first for i, j in pairs)
    e.end_weld_group()
    e.step(1)
    assert e.weld_state()['fuse_tag'] == 0
