"""Authoring edits (replaceWhere, sliceBonds, eraseWhere) on the CPU oracle:
the host logic of src/engine.js:6191-6650 over the engine surface."""
import numpy as np

from sunaengine_gb300 import authoring, data, scenes

ONE = 65536


def oracle(sc, cap_extra=64):
    import oracle as o
    return o.OracleEngine(sc.n + cap_extra, threads=8).load_scene(sc)


def gel():
    """A free (unheld) RUBBER box welded at load, holding WATER: a bonded frame."""
    return scenes.sealed_box(held=False, spacing=0.8)


def bonds_of(e):
    return e.read_bonds().reshape(e.n_fluid, 48)


def live_pairs(b):
    out = set()
    for i in range(b.shape[0]):
        for w in b[i]:
            w = int(w)
            if not w:
                break
            if w & authoring.BOND_TOMB:
                continue
            out.add((i, w & authoring.BOND_J_MASK))
    return out


def test_replace_where_tombstones_touching_bonds():
    sc = gel()
    e = oracle(sc)
    e.step(2)
    st = e.read_state().reshape(-1, 8)
    rubber = data.mat_id('RUBBER')
    cx = int(np.median(st[:sc.nFluid, 0]))
    was = st[:sc.nFluid, 4] == rubber
    n = authoring.replace_where(e, lambda p: p['mat'] == rubber and p['x'] < cx, 0)
    assert 0 < n < int(was.sum())
    st2 = e.read_state().reshape(-1, 8)
    changed = was & (st2[:sc.nFluid, 4] == 0)
    assert changed.sum() == n
    assert (st2[:sc.nFluid, 5][changed] & authoring.WELD_TAG_MASK == 0).all()
    b = bonds_of(e)
    pairs = live_pairs(b)
    assert pairs
    for i, j in pairs:
        assert not changed[i] and not changed[j]
    e.step(5)


def test_slice_bonds_cuts_both_ends():
    sc = gel()
    e = oracle(sc)
    e.step(2)
    before = live_pairs(bonds_of(e))
    st = e.read_state().reshape(-1, 8)
    cx = int(np.median(st[:sc.nFluid, 0]))
    y0, y1 = int(st[:sc.nFluid, 1].min()) - 4 * ONE, int(st[:sc.nFluid, 1].max()) + 4 * ONE
    cut = authoring.slice_bonds_many(e, [{'x0': cx, 'y0': y0, 'x1': cx, 'y1': y1}])
    after = live_pairs(bonds_of(e))
    assert cut > 0 and len(before) - len(after) == 2 * cut
    assert all((j, i) in after for i, j in after)
    e.step(5)


def test_erase_where_renumbers_bond_partners():
    sc = gel()
    e = oracle(sc)
    e.step(2)
    nf0 = e.n_fluid
    st = e.read_state().reshape(-1, 8)
    cy = int(np.median(st[:nf0, 1]))
    removed = authoring.erase_where(e, lambda p: p['y'] < cy)
    assert removed > 0 and e.n_fluid == nf0 - removed and e.n == sc.n - removed
    b = bonds_of(e)
    pairs = live_pairs(b)
    assert pairs and all(j < e.n_fluid for _, j in pairs)
    assert all((j, i) in pairs for i, j in pairs)
    st2 = e.read_state().reshape(-1, 8)
    assert (st2[:e.n_fluid, 1] < cy).all()
    e.step(5)
