"""§25 composed materials (synth + the intern cache) and §26.C gravity scale,
on the CPU oracle. synth() is a pure function of the authored table, checked
here against the algebra's stated laws; the intern cache against its policy
(hit, mint, products closure, recycle, project, replay)."""
import numpy as np
import pytest

from sunaengine_gb300 import data, materials, scenes
from sunaengine_gb300.materials import MOD, F, synth

ONE = 65536
M = data.mats()


def test_synth_laws():
    water, sand, oil = 0, data.mat_id('SAND'), data.mat_id('OIL')
    # D+L cancels exactly: the base row itself, nothing minted
    w, needs, dropped, ident = synth(water, MOD['D'] | MOD['L'], M)
    assert ident and w == [int(x) for x in M[water]]
    w, *_ = synth(water, MOD['V'], M)
    assert w[F('xsph')] == min(int(M[water][F('xsph')]) * 4, 45000)
    w, *_ = synth(water, MOD['D'], M)
    assert w[F('grav')] == int(M[water][F('grav')]) + 600
    w, *_ = synth(sand, MOD['E'], M)
    assert (w[F('bondK')], w[F('solidMode')], w[F('bondGroup')]) == (24576, 1, -2)
    w, _, dropped, _ = synth(sand, MOD['E'] | MOD['K'], M)
    assert w[F('rampSign')] == 0 and any('K wins' in d for d in dropped)
    w, *_ = synth(sand, MOD['E'] | MOD['B'], M)
    assert w[F('bondBreak')] == 79299
    _, _, dropped, _ = synth(water, MOD['B'], M)
    assert any('B inert' in d for d in dropped)
    w, needs, _, _ = synth(water, MOD['Y'], M)
    assert needs == [{'field': 'meltTo', 'base': 0, 'bits': MOD['YPROD']}] and w[F('bondK')] == int(M[2][F('bondK')])
    w, *_ = synth(water, MOD['YPROD'], M)
    assert w[F('freezePt')] == -2147483648
    w, _, dropped, _ = synth(oil, MOD['H'] | MOD['C'], M)
    assert w[F('tempDrive')] == 0 and dropped
    with pytest.raises(materials.SynthError):
        synth(water, MOD['H'], M)                    # a heater above water's own boiling point
    w, *_ = synth(data.mat_id('STONE'), MOD['H'], M)
    assert w[F('tempTarget')] == 900 * ONE and w[F('spawnTemp')] == 900 * ONE
    w, *_ = synth(water, MOD['T'], M)
    assert w[F('gammaCoh')] == 4 * int(M[water][F('gammaCoh')]) and w[F('adhesion')] == 0


def _oracle(n=8192):
    import oracle as o
    return o.OracleEngine(n)


def test_intern_cache_policy_and_replay():
    e = _oracle()
    sc = scenes.make_scene('dambreak_v1')
    e.load_scene(sc)
    it = materials.Interner(e)
    r = it.intern(0, MOD['V'])
    assert r['kind'] == 'mint' and r['rowId'] == 28
    assert it.intern(0, MOD['V'])['kind'] == 'hit'
    assert it.intern(0, MOD['D'] | MOD['L'])['rowId'] == 0            # identity: no row
    snow = it.intern(0, MOD['Y'])
    assert [x['type'] for x in snow['events']] == ['MINT', 'MINT']
    sw = snow['events'][0]['rowId']
    assert snow['rowId'] == sw + 1 and it.by_row[snow['rowId']]['words'][F('meltTo')] == sw
    sand = data.mat_id('SAND')
    bonded = it.intern(sand, MOD['E'])
    assert it.by_row[bonded['rowId']]['words'][F('bondGroup')] == 64 + bonded['rowId']
    # fill the table, then the least recently used bare row is recycled
    letters = ['V', 'T', 'D', 'E', 'S', 'FLOAT']
    combos = [sum(MOD[c] for i, c in enumerate(letters) if k >> i & 1) for k in range(1, 64)]
    for bits in combos:
        if it.mat_count >= 64:
            break
        it.intern(sand, bits)
    assert it.mat_count == 64
    r = it.intern(data.mat_id('OIL'), MOD['V'])
    assert r['kind'] == 'recycle' and r['rowId'] == 28                # the oldest untouched row
    # every live row pinned: project onto the nearest one
    r = it.intern(data.mat_id('OIL'), MOD['T'], pinned=set(range(64)))
    assert r['kind'] == 'project' and 28 <= r['rowId'] < 64
    # a replay re-derives every mint; a tampered record is refused
    f = _oracle()
    f.load_scene(sc)
    j = materials.Interner(f)
    j.apply_events(it.events)
    assert {k: v['words'] for k, v in j.by_row.items()} == {k: v['words'] for k, v in it.by_row.items()}
    bad = [dict(ev) for ev in it.events]
    mint = next(ev for ev in bad if ev['type'] == 'MINT')
    mint['words'] = list(mint['words'])
    mint['words'][F('xsph')] += 1
    g = _oracle()
    g.load_scene(sc)
    with pytest.raises(materials.SynthError):
        materials.Interner(g).apply_events(bad)


def test_worn_rows_are_not_recycled():
    e = _oracle()
    e.load_scene(scenes.make_scene('dambreak_v1'))
    it = materials.Interner(e)
    row = it.intern(0, MOD['V'])['rowId']
    pts = [{'x': (40 + c) * ONE, 'y': 20 * ONE, 'mat': row} for c in range(4)]
    e.spawn(pts)
    it.note_spawn([row] * 4)
    assert not it._recyclable(row, set())
    keep = np.ones(e.n_fluid, bool)
    keep[-4:] = False
    e.erase(keep)
    assert it._recyclable(row, set())


def test_composed_rows_and_gravity_change_the_physics():
    sc = scenes.make_scene('dambreak_v1')
    a, b = _oracle(), _oracle()
    for x in (a, b):
        x.load_scene(sc)
    it = materials.Interner(b)
    row = it.intern(0, MOD['V'])['rowId']
    pts = [{'x': (70 + c) * ONE, 'y': (10 + r) * ONE, 'mat': 0} for r in range(4) for c in range(6)]
    a.spawn(pts)
    b.spawn([dict(p, mat=row) for p in pts])
    a.step(20)
    b.step(20)
    assert a.chain_hex() != b.chain_hex()
    c = _oracle()
    c.load_scene(sc)
    assert c.set_gravity_scale(ONE) == ONE
    c.step(5)
    d = _oracle()
    d.load_scene(sc)
    d.step(5)
    assert c.chain_hex() == d.chain_hex()            # the default multiplier is bit-inert
    assert c.set_gravity_scale(ONE // 2) == ONE // 2
    c.step(5)
    d.step(5)
    assert c.chain_hex() != d.chain_hex()
