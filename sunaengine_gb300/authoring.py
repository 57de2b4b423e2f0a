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

import math

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


# ---- §20 host-side body rebuilds ---------------------------------------------------
ONE = 65536
FLAG_ANCHOR = 4
RIGID_MIN_MEMBERS = 4
RG_MAX_BODIES = 1024
RB_TAG, RB_FIRST, RB_LAST, RB_CX, RB_CY, RB_AXIS, RB_USER = 1, 2, 3, 4, 5, 27, 28


def _js_round(x: float) -> int:
    """Math.round: ties towards +infinity."""
    r = math.floor(x)
    return int(r + 1 if x - r >= 0.5 else r)


def _i32(v) -> int:
    """JS `x | 0` on an integral number."""
    v = int(v) & 0xffffffff
    return v - (1 << 32) if v & 0x80000000 else v


def _components(st, members, link_ticks, severed):
    """The connected pieces of `members` (src/engine.js:6353-6383): a 3x3 scan
    of link-sized cells, pairs within the link radius and not severed."""
    if len(members) < 2:
        return [list(members)]
    cell = max(1, link_ticks)
    lim2 = float(link_ticks) * float(link_ticks)
    grid = {}
    for i in members:
        k = (math.floor(float(st[i, 0]) / cell), math.floor(float(st[i, 1]) / cell))
        grid.setdefault(k, []).append(i)
    seen, out = set(), []
    for seed in members:
        if seed in seen:
            continue
        comp, q = [], [seed]
        seen.add(seed)
        while q:
            i = q.pop()
            comp.append(i)
            xi, yi = float(st[i, 0]), float(st[i, 1])
            cx, cy = math.floor(xi / cell), math.floor(yi / cell)
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    for j in grid.get((cx + dx, cy + dy), ()):
                        if j in seen:
                            continue
                        ex, ey = float(st[j, 0]) - xi, float(st[j, 1]) - yi
                        if ex * ex + ey * ey > lim2 or severed(xi, yi, float(st[j, 0]), float(st[j, 1])):
                            continue
                        seen.add(j)
                        q.append(j)
        comp.sort()
        out.append(comp)
    out.sort(key=lambda c: (-len(c), c[0]))
    return out


def split_disconnected_bodies(eng, link_ticks: int = None, cuts=(), kerf: int = None) -> dict:
    """splitDisconnectedBodies (src/engine.js:6312-6440): after a cut, every
    body whose members fall into several connected pieces (1.65 wu links, no
    link across a cut line or within the kerf of one) is rebuilt as one body
    per piece of at least 4 members; only the largest piece keeps the axle
    and the user flag. Returns {'split': pieces added, 'bodies': bodies now}."""
    link_ticks = _js_round(1.65 * ONE) if link_ticks is None else int(link_ticks)
    kerf = _js_round(ONE * 0.52) if kerf is None else int(kerf)
    nb = eng.body_count
    nf = eng.n_fluid
    if nb == 0 or nf == 0:
        return {'split': 0, 'bodies': nb}
    st = eng.read_state().reshape(-1, 8).copy()
    recs = eng.read_bodies()
    segs = [(float(_i32(s['x0'])), float(_i32(s['y0'])), float(_i32(s['x1'])), float(_i32(s['y1']))) for s in cuts]
    kerf2 = float(max(0, _i32(kerf))) ** 2

    def point_seg_d2(px, py, ax, ay, bx, by):
        ex, ey = bx - ax, by - ay
        den = ex * ex + ey * ey
        t = max(0.0, min(1.0, ((px - ax) * ex + (py - ay) * ey) / den)) if den > 0 else 0.0
        dx, dy = px - (ax + ex * t), py - (ay + ey * t)
        return dx * dx + dy * dy

    def orient(ax, ay, bx, by, cx, cy):
        return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax)

    def crosses(ax, ay, bx, by, cx, cy, dx, dy):
        if (max(ax, bx) < min(cx, dx) or max(cx, dx) < min(ax, bx) or
                max(ay, by) < min(cy, dy) or max(cy, dy) < min(ay, by)):
            return False
        a, b = orient(ax, ay, bx, by, cx, cy), orient(ax, ay, bx, by, dx, dy)
        c, d = orient(cx, cy, dx, dy, ax, ay), orient(cx, cy, dx, dy, bx, by)
        return ((a == 0 or b == 0 or (a < 0) != (b < 0)) and (c == 0 or d == 0 or (c < 0) != (d < 0)))

    def severed(ax, ay, bx, by):
        for x0, y0, x1, y1 in segs:
            if (crosses(ax, ay, bx, by, x0, y0, x1, y1) or point_seg_d2(ax, ay, x0, y0, x1, y1) <= kerf2 or
                    point_seg_d2(bx, by, x0, y0, x1, y1) <= kerf2 or point_seg_d2(x0, y0, ax, ay, bx, by) <= kerf2 or
                    point_seg_d2(x1, y1, ax, ay, bx, by) <= kerf2):
                return True
        return False

    fl = st[:, 5].astype(np.int64) & 0xffffffff
    specs, split = [], 0
    for R in recs:
        tag = int(R[RB_TAG]) & 0xffffffff
        members = [i for i in range(int(R[RB_FIRST]), min(int(R[RB_LAST]) + 1, nf))
                   if (fl[i] & FLAG_RIGID) and (fl[i] & WELD_TAG_MASK) == tag]
        if not members:
            continue
        parts = _components(st, members, link_ticks, severed)
        split += len(parts) - 1
        axis = bool(R[RB_AXIS])
        specs.append((parts, axis, bool(R[RB_USER]), (int(R[RB_CX]), int(R[RB_CY])) if axis else None))
    if not split:
        return {'split': 0, 'bodies': nb}
    rigid = (fl[:nf] & FLAG_RIGID) != 0
    st[:nf, 5] = np.where(rigid, (fl[:nf] & ~(FLAG_RIGID | WELD_TAG_MASK)), fl[:nf]).astype(np.uint32).view(np.int32)
    eng.write_state_keep_scratch(st.reshape(-1))
    eng.restore_bodies(np.zeros((0, 32), np.int32))
    made = 0
    for parts, axis, user, pivot in specs:
        for p, members in enumerate(parts):
            if len(members) < RIGID_MIN_MEMBERS or made >= RG_MAX_BODIES:
                continue
            idx, _ = eng.write_body(members, 0, pivot if (p == 0 and axis) else None, p == 0 and user)
            made += idx is not None
    _mark_dirty(eng)
    return {'split': split, 'bodies': eng.body_count}


def promote_loose_rigid_components(eng, link_ticks: int = None, eligible=()) -> int:
    """promoteLooseRigidComponents (src/engine.js:5636-5710): clusters of loose
    rigid-row matter (not anchored, not in a body) of one material, linked
    within 1.65 wu, that hold a live bond and one of the caller's freshly
    congealed witnesses ({'slot', 'mat'}) become bodies. Returns how many."""
    link_ticks = _js_round(1.65 * ONE) if link_ticks is None else int(link_ticks)
    nf = eng.n_fluid
    if nf == 0 or eng.body_count >= RG_MAX_BODIES:
        return 0
    wit = {int(w['slot']): int(w['mat']) & 0xffffffff for w in eligible
           if isinstance(w.get('slot'), int) and isinstance(w.get('mat'), int)}
    if not wit:
        return 0
    st = eng.read_state().reshape(-1, 8)
    bonds = eng.read_bonds().reshape(-1, BOND_CAP)
    solid = data.MAT_FIELDS.index('solidMode')
    cell = max(1, _i32(link_ticks))
    live = np.zeros(nf, bool)
    for i in range(nf):
        for w in bonds[i]:
            w = int(w) & 0xffffffff
            if not w:
                break
            if not (w & BOND_TOMB):
                live[i] = True
                break
    grid, cand = {}, []
    fl = st[:, 5].astype(np.int64) & 0xffffffff
    for i in range(nf):
        m = int(st[i, 4]) & 0xffffffff
        if (fl[i] & (FLAG_ANCHOR | FLAG_RIGID)) or _row(eng, m)[solid] != 2:
            continue
        k = (math.floor(float(st[i, 0]) / cell), math.floor(float(st[i, 1]) / cell), m)
        grid.setdefault(k, []).append(i)
        cand.append(i)
    if not cand:
        return 0
    lim2 = float(cell) * float(cell)
    seen, groups = set(), []
    for seed in cand:
        if seed in seen:
            continue
        mat = int(st[seed, 4]) & 0xffffffff
        part, todo = [], [seed]
        bonded = congealed = False
        seen.add(seed)
        while todo:
            i = todo.pop()
            part.append(i)
            bonded = bonded or bool(live[i])
            congealed = congealed or wit.get(i) == (int(st[i, 4]) & 0xffffffff)
            xi, yi = float(st[i, 0]), float(st[i, 1])
            cx, cy = math.floor(xi / cell), math.floor(yi / cell)
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    for j in grid.get((cx + dx, cy + dy, mat), ()):
                        if j in seen:
                            continue
                        ex, ey = float(st[j, 0]) - xi, float(st[j, 1]) - yi
                        if ex * ex + ey * ey > lim2:
                            continue
                        seen.add(j)
                        todo.append(j)
        part.sort()
        if bonded and congealed and len(part) >= RIGID_MIN_MEMBERS:
            groups.append(part)
    made = 0
    for members in groups:
        if eng.body_count >= RG_MAX_BODIES:
            break
        idx, _ = eng.write_body(members, 0)
        made += idx is not None
    if made:
        _mark_dirty(eng)
    return made


# ---- exact authoring saves (.suna with bonds, bodies and composed rows) -------------
RG_BODY_WORDS = 32


def authoring_snapshot(eng) -> dict:
    """The engine-owned parts of an exact save (the payload of encodeSuna,
    src/suna.js:46-84, and the input of restoreAuthoringSnapshot,
    src/engine.js:5838): state, bond rows (also as the candidate table),
    the body-record image (RG_MAX_BODIES x 32 words), rest offsets, the body
    descriptors and the formation clock."""
    n, nf = eng.n, eng.n_fluid
    recs = eng.read_bodies()
    image = np.zeros(RG_MAX_BODIES * RG_BODY_WORDS, np.int32)
    image[:recs.size] = recs.reshape(-1)
    bonds = np.zeros(n * BOND_CAP, np.uint32)
    if nf:
        bonds[:nf * BOND_CAP] = np.asarray(eng.read_bonds(), dtype=np.uint32).reshape(-1)[:nf * BOND_CAP]
    bodies = [{'tag': int(R[RB_TAG]) & 0xffffffff, 'first': int(R[RB_FIRST]), 'last': int(R[RB_LAST]),
               'n': int(R[14]), 'index': k, 'axis': bool(R[RB_AXIS]), 'user': bool(R[RB_USER])}
              for k, R in enumerate(recs)]
    return {'state': np.ascontiguousarray(eng.read_state(), dtype=np.int32), 'bonds': bonds, 'bondCand': bonds.copy(),
            'bodyRecords': image, 'restOffsets': np.ascontiguousarray(eng.read_rest_offsets(), dtype=np.int32),
            'bodies': bodies, 'formationClock': int(eng.formation_clock)}


def restore_authoring_snapshot(eng, snap: dict):
    """restoreAuthoringSnapshot (src/engine.js:5838-5888) after load_scene:
    state, bond rows, body records and rest offsets, formation clock (no
    pending formation)."""
    n, nf = eng.n, eng.n_fluid
    state = np.ascontiguousarray(snap['state'], dtype=np.int32).reshape(-1)
    if state.size != n * 8:
        raise ValueError(f'snapshot state has {state.size} words; expected {n * 8}')
    eng.write_state_keep_scratch(state)
    bonds = np.ascontiguousarray(snap['bonds'], dtype=np.uint32).reshape(-1)
    if nf:
        eng.write_bonds(bonds[:nf * BOND_CAP])
    k = len(snap.get('bodies') or [])
    recs = np.ascontiguousarray(snap['bodyRecords'], dtype=np.int32).reshape(-1)[:k * RG_BODY_WORDS]
    eng.restore_bodies(recs.reshape(-1, RG_BODY_WORDS), snap.get('restOffsets'))
    eng.set_formation_clock(int(snap.get('formationClock', 0)), False)


def save_suna(eng, scene, interner=None, app=None) -> str:
    """An exact `.suna` save of the engine's scene (`scene` gives the domain:
    domW, domH, cellShift) with its composed-material record."""
    from . import formats
    snap = authoring_snapshot(eng)
    header = {'n': int(eng.n), 'nFluid': int(eng.n_fluid), 'domW': int(scene.domW), 'domH': int(scene.domH),
              'cellShift': int(scene.cellShift), 'formationClock': snap['formationClock']}
    payload = dict(snap, scene=header, tints=np.zeros(int(eng.n), np.uint32), app=app,
                   materials={'events': list(interner.events) if interner is not None else []})
    return formats.encode_suna(payload)


def load_suna(text, new_engine):
    """Load an exact `.suna`: a fresh engine from `new_engine()`, the composed
    rows re-derived from the record (applyMintEvents refuses any mismatch),
    the scene loaded from the saved words, then restoreAuthoringSnapshot.
    Returns (engine, interner)."""
    from . import formats, materials, scenes as sc_mod
    doc = formats.decode_suna(text)
    s = doc['scene']
    n, nf = int(s['n']), int(s['nFluid'])
    st = np.asarray(doc['state'], dtype=np.int32).reshape(n, 8)
    sc = sc_mod.Scene(n=n, nFluid=nf, pos=st[:, 0:2].copy(), vel=st[:, 2:4].copy(),
                      matId=st[:, 4].astype(np.uint32), domW=int(s['domW']), domH=int(s['domH']),
                      cellShift=int(s['cellShift']), flags=(st[:, 5].astype(np.uint32) & 5),
                      temp=st[:, 6].copy(), fuel=st[:, 7].copy(), name='suna')
    eng = new_engine()
    it = materials.Interner(eng)
    it.apply_events((doc.get('materials') or {}).get('events') or [])
    eng.load_scene(sc)
    if doc.get('bonds') is not None:
        restore_authoring_snapshot(eng, {'state': doc['state'], 'bonds': doc['bonds'],
                                         'bodyRecords': doc['bodyRecords'], 'restOffsets': doc['restOffsets'],
                                         'bodies': doc.get('bodies') or [],
                                         'formationClock': int(s.get('formationClock', 0))})
    else:
        eng.write_state_keep_scratch(np.asarray(doc['state'], dtype=np.int32))
    return eng, it
