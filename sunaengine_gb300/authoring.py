"""Host-side authoring edits, as the reference performs them in JavaScript.

``replace_where`` (``src/engine.js:6191-6238``), ``slice_bonds_many``
(``:6240-6300``) and ``erase_where`` (``:6460-6650``) evaluate the caller's
predicate on a ``readState`` copy and write the result back. They work on any
engine with the ``Engine`` surface (the GPU engine, or the oracle in tests):
``read_state``, ``write_state_keep_scratch``, ``read_bonds``/``write_bonds``,
``erase``, ``formation_clock`` and ``set_formation_clock``. Segment geometry is evaluated in IEEE
doubles in the same operation order as the reference's JavaScript numbers.
"""
from __future__ import annotations

import numpy as np

from . import data

FLAG_DEAD, FLAG_SEAL, FLAG_CONGEAL, FLAG_BURST, FLAG_RIGID = 2, 128, 32, 64, 16
WELD_TAG_MASK = 0x000fff00
BOND_CAP = 48
BOND_J_MASK = 0x0001ffff
BOND_TOMB = 0x40000000


def _row(eng, m):
    mats = getattr(eng, '_mats_rows', None)
    if mats is None:
        mats = data.mats()
    return np.asarray(mats).reshape(-1, 48)[m]


def _seal_row(r):
    f = data.MAT_FIELDS.index
    return r[f('bondK')] != 0 and r[f('bondReform')] == 0 and r[f('solidMode')] != 0 and r[f('phantom')] == 0


def _fields(st, i):
    o = st[i]
    return {'i': i, 'x': int(o[0]), 'y': int(o[1]), 'vx': int(o[2]), 'vy': int(o[3]), 'mat': int(o[4]) & 0xffffffff,
            'flags': int(o[5]) & 0xffffffff, 'temp': int(o[6]), 'fuel': int(o[7])}


def _mark_dirty(eng):
    eng.set_formation_clock(eng.formation_clock, True)


def replace_where(eng, test, new_mat: int) -> int:
    """replaceWhere (src/engine.js:6191-6238): rows passing `test` become `new_mat`
    (new matter at an old position: authored BURNING/ANCHOR kept, weld group and
    body membership severed, spawnTemp and fuel0 of the new row); every bond
    touching a changed particle is tombstoned. Returns how many changed."""
    m = int(new_mat)
    r = _row(eng, m)
    f = data.MAT_FIELDS.index
    if r[f('phantom')] != 0:
        raise ValueError(f'replaceWhere material {m} is not live')
    nf = eng.n_fluid
    if nf == 0:
        return 0
    st = eng.read_state().reshape(-1, 8).copy()
    changed = np.zeros(nf, bool)
    for i in range(nf):
        if not test(_fields(st, i)) or (int(st[i, 4]) & 0xffffffff) == m:
            continue
        changed[i] = True
        st[i, 4] = m
        fl = int(st[i, 5]) & 0xffffffff
        fl &= ~(FLAG_DEAD | FLAG_SEAL | FLAG_CONGEAL | FLAG_BURST | FLAG_RIGID | WELD_TAG_MASK) & 0xffffffff
        fl |= (FLAG_DEAD if r[f('phantom')] != 0 else 0) | (FLAG_SEAL if _seal_row(r) else 0)
        st[i, 5] = np.int32(np.uint32(fl).view(np.int32))
        st[i, 6] = r[f('spawnTemp')]
        st[i, 7] = r[f('fuel0')]
    n = int(changed.sum())
    if not n:
        return 0
    bonds = eng.read_bonds().reshape(nf, BOND_CAP).copy()
    for i in range(nf):
        for k in range(BOND_CAP):
            w = int(bonds[i, k])
            if not w:
                break
            j = w & BOND_J_MASK
            if changed[i] or (j < nf and changed[j]):
                bonds[i, k] = w | BOND_TOMB
    eng.write_state_keep_scratch(st.reshape(-1))
    eng.write_bonds(bonds.reshape(-1))
    _mark_dirty(eng)
    return n


def _orient(ax, ay, bx, by, cx, cy):
    return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax)


def _crosses(ax, ay, bx, by, cx, cy, dx, dy):
    if (max(ax, bx) < min(cx, dx) or max(cx, dx) < min(ax, bx) or
            max(ay, by) < min(cy, dy) or max(cy, dy) < min(ay, by)):
        return False
    a, b = _orient(ax, ay, bx, by, cx, cy), _orient(ax, ay, bx, by, dx, dy)
    c, d = _orient(cx, cy, dx, dy, ax, ay), _orient(cx, cy, dx, dy, bx, by)
    return ((a == 0 or b == 0 or (a < 0) != (b < 0)) and (c == 0 or d == 0 or (c < 0) != (d < 0)))


def _point_seg_d2(px, py, ax, ay, bx, by):
    ex, ey = bx - ax, by - ay
    den = ex * ex + ey * ey
    t = max(0.0, min(1.0, ((px - ax) * ex + (py - ay) * ey) / den)) if den > 0 else 0.0
    dx, dy = px - (ax + ex * t), py - (ay + ey * t)
    return dx * dx + dy * dy


def slice_bonds_many(eng, segments, kerf: int = 34079) -> int:
    """sliceBondsMany (src/engine.js:6240-6300): tombstone every live bond whose
    particle-to-particle segment crosses (or comes within `kerf` of) a cut, on
    both ends. Positions are JavaScript numbers there, so the geometry runs in
    doubles here. Returns the number of bonds cut."""
    nf = eng.n_fluid
    if nf == 0 or not segments:
        return 0
    st = eng.read_state().reshape(-1, 8)
    bond = eng.read_bonds().reshape(nf, BOND_CAP).copy()
    kerf2 = float(max(0, int(kerf)) ** 2)
    segs = [(float(int(s['x0'])), float(int(s['y0'])), float(int(s['x1'])), float(int(s['y1']))) for s in segments]

    def in_kerf(ax, ay, bx, by, s):
        x0, y0, x1, y1 = s
        return (_crosses(ax, ay, bx, by, x0, y0, x1, y1) or _point_seg_d2(ax, ay, x0, y0, x1, y1) <= kerf2 or
                _point_seg_d2(bx, by, x0, y0, x1, y1) <= kerf2 or _point_seg_d2(x0, y0, ax, ay, bx, by) <= kerf2 or
                _point_seg_d2(x1, y1, ax, ay, bx, by) <= kerf2)

    cut = 0
    for i in range(nf):
        for k in range(BOND_CAP):
            w = int(bond[i, k])
            if not w:
                break
            if w & BOND_TOMB:
                continue
            j = w & BOND_J_MASK
            if j <= i or j >= nf:
                continue
            a = (float(st[i, 0]), float(st[i, 1]), float(st[j, 0]), float(st[j, 1]))
            if not any(in_kerf(*a, s) for s in segs):
                continue
            cut += 1
            bond[i, k] = w | BOND_TOMB
            for z in range(BOND_CAP):
                w2 = int(bond[j, z])
                if not w2:
                    break
                if (w2 & BOND_J_MASK) == i:
                    bond[j, z] = w2 | BOND_TOMB
                    break
    if cut:
        eng.write_bonds(bond.reshape(-1))
        _mark_dirty(eng)
    return cut


def erase_where(eng, keep) -> int:
    """eraseWhere (src/engine.js:6460-6650): keep the fluid particles `keep`
    accepts, compacting slots on the device (state, stAcc and bond partners
    move with their particle). Returns how many were removed."""
    nf = eng.n_fluid
    if nf == 0:
        return 0
    st = eng.read_state().reshape(-1, 8)
    mask = np.array([bool(keep(_fields(st, i))) for i in range(nf)], bool)
    return eng.erase(mask)
