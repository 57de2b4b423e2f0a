"""Runtime material rows: §25 composed ("interned") materials and §26.C gravity.

The reference composes materials on the host (``src/engine.js:828-1170``):
``synth(base, bits)`` is a pure function from an authored row and a set of
modifier bits (viscous, tensile, dense, light, elastic, brittle, ...) to a
48-word row; ``Engine.internMaterial`` (``:4981-5245``) caches composed rows
in the table's tail [authored rows, 64), keyed by (base, bits), minting,
recycling the least recently used row nothing wears any more, or projecting
onto the nearest live row when the table is full, and records every outcome
as an event a replay re-applies. The engine itself only holds the table, so
this module is host logic over one call, ``set_material(row, words)``, on any
engine with that surface (the GPU engine, or the oracle in tests).

Words are integers throughout; the only JS arithmetic with fractions is
``(gammaCoh / 4) | 0`` (truncation) and the tint channel clamp.
"""
from __future__ import annotations

from typing import Dict, List, Optional

import numpy as np

from . import data

ONE = 65536
MAT_MAX = 64
NEVER_COLD = -2147483648
SYNTH_VERSION = 4
XSPH_MAX, COND_MAX, BOND_K_MAX = 45000, 32768, 32768
SOLID_BOND = 1


def DEG(d: int) -> int:
    return d * ONE


# Modifier bits (src/engine.js:853-874)
MOD = dict(V=1 << 0, T=1 << 1, D=1 << 2, L=1 << 3, E=1 << 4, B=1 << 5, M=1 << 6, K=1 << 7, S=1 << 8, H=1 << 9,
           C=1 << 10, Y=1 << 11, YPROD=1 << 12, I=1 << 13, O=1 << 14, IO_NULL=1 << 15, FLOAT=1 << 16)
MOD_LETTERS = 'VTDLEBMKSHCYIO'

# The algebra's constants per SYNTH_VERSION (src/engine.js:908-950)
_V1 = dict(V_XSPH_MUL=4, V_XSPH_CLAMP=45000, T_COH_MUL=4, DL_GRAV=600, E_BONDK=16384, E_BONDBREAK=409600,
           B_BONDBREAK=79299, M_BONDK=8192, M_ADHESION_MIN=260, S_BONDK=8192, S_BONDBREAK=165000,
           H_TARGET=DEG(900), C_TARGET=DEG(-150), HC_DRIVE=300)
SYNTH_CONSTS = {1: _V1, 2: dict(_V1, E_BONDK=24576)}
SYNTH_CONSTS[3] = dict(SYNTH_CONSTS[2])
SYNTH_CONSTS[4] = dict(SYNTH_CONSTS[3], FLOAT_GRAV=1050)
BOND_PRECEDENCE = 'KMES'          # the first present bond template wins
BOND_BLOCK = ('bondK', 'bondBreak', 'bondReform', 'bondFormV', 'bondFormP', 'bondMu', 'rampLo', 'rampHi', 'rampSign')
PRODUCTS = ('meltTo', 'freezeTo', 'boilTo', 'condTo', 'burnTo', 'splitTo', 'corrTo')
PROJECT_AXES = ('xsph', 'gammaCoh', 'gammaCur', 'adhesion', 'grav', 'fric', 'bondK', 'bondBreak', 'bondReform',
                'solidMode', 'tempTarget', 'tempDrive', 'burstP', 'sealMode')

F = data.MAT_FIELDS.index
MAT_WATER, MAT_ICE, MAT_RUBBER, MAT_RICE = 0, 2, 17, 25


class SynthError(ValueError):
    pass


def mod_letters(bits: int) -> str:
    s = ''.join(c for c in MOD_LETTERS if bits & MOD[c])
    if bits & MOD['YPROD']:
        s += 'y'
    if bits & MOD['IO_NULL']:
        s += '0'
    if bits & MOD['FLOAT']:
        s += 'f'
    return s


def _clamp8(x: int) -> int:
    return max(0, min(255, int(x)))


def compose_tint(tint: int, bits: int) -> int:
    """The composed swatch colour (host-only word 27; no pass reads it)."""
    if bits == MOD['C']:
        return 0x0000ff
    r, g, b = (tint >> 16) & 255, (tint >> 8) & 255, tint & 255
    shifts = (('V', 0, 24, 0), ('T', 16, 16, 16), ('D', -24, -24, -24), ('L', 24, 24, 24), ('E', 20, 0, 20),
              ('B', 20, 10, 0), ('M', 24, 12, -12), ('K', 12, 12, 0), ('S', 0, 0, 28), ('H', 48, 0, -24),
              ('C', -24, 0, 48))
    for c, dr, dg, db in shifts:
        if bits & MOD[c]:
            r, g, b = r + dr, g + dg, b + db
    if bits & (MOD['Y'] | MOD['YPROD']):
        r, g, b = r + 16, g + 24, b + 24
    if bits & MOD['I']:
        g, b = g + 42, b + 18
    if bits & MOD['O']:
        r, b = r + 42, b + 18
    return (_clamp8(r) << 16) | (_clamp8(g) << 8) | _clamp8(b)


def synth(base: int, bits: int, mats, version: int = SYNTH_VERSION):
    """synth (src/engine.js:991-1170): (words, needs, dropped, identity).

    Order of application: bond template, Brittle, scalars (V, T, D, L, FLOAT),
    thermal (H, C), products closure. A composed row that bonds gets the
    group sentinel -2 (the interner assigns 64 + rowId); D+L and the other
    exact cancellations return the base row itself (identity)."""
    if version not in SYNTH_CONSTS:
        raise SynthError(f'synth: unknown SYNTH_VERSION {version}')
    C = SYNTH_CONSTS[version]
    mats = np.asarray(mats).reshape(-1, 48)
    if not (0 <= base < len(mats)):
        raise SynthError(f'synth: baseId {base} is not an authored material')
    if mats[base][F('phantom')] != 0:
        raise SynthError(f'synth: base {base} is phantom')
    if not (0 < bits < (1 << 17)):
        raise SynthError(f'synth: bits {bits} outside the modifier bitset')
    has = lambda c: bool(bits & MOD[c])
    mech = MAT_ICE if has('Y') else base
    row = [int(x) for x in mats[mech]]
    dropped, needs = [], []
    templates = [c for c in BOND_PRECEDENCE if has(c)]
    if templates:
        t = templates[0]
        rice, rubber = mats[MAT_RICE], mats[MAT_RUBBER]
        src = rice if t in 'KM' else rubber
        for f in BOND_BLOCK:
            row[F(f)] = int(src[F(f)])
        if t == 'K':
            row[F('rampSign')] = 0
        elif t == 'M':
            row[F('rampSign')] = 0
            row[F('bondK')] = C['M_BONDK']
            row[F('bondReform')] = 1
            row[F('adhesion')] = max(row[F('adhesion')], C['M_ADHESION_MIN'])
        elif t == 'E':
            row[F('bondK')] = C['E_BONDK']
        else:
            row[F('bondK')] = C['S_BONDK']
            row[F('bondBreak')] = C['S_BONDBREAK']
            row[F('bondReform')] = 0
        row[F('solidMode')] = SOLID_BOND
        row[F('bondGroup')] = -2
        if len(templates) > 1:
            dropped.append(f"bond template {t} wins over {','.join(templates[1:])} (K>M>E>S)")
    elif has('B') and row[F('bondK')] == 0:
        dropped.append('B inert without a bond template')
    if has('B') and templates:
        row[F('bondBreak')] = C['B_BONDBREAK']
    if has('V'):
        row[F('xsph')] = min(row[F('xsph')] * C['V_XSPH_MUL'], C['V_XSPH_CLAMP'])
    if has('T'):
        row[F('gammaCoh')] = row[F('gammaCoh')] * C['T_COH_MUL']
        row[F('gammaCur')] = int(row[F('gammaCoh')] / 4)        # JS (x / 4) | 0 truncates
        row[F('adhesion')] = 0
    if has('D'):
        row[F('grav')] += C['DL_GRAV']
    if has('L'):
        row[F('grav')] -= C['DL_GRAV']
    if bits & MOD['FLOAT']:
        row[F('grav')] = C['FLOAT_GRAV'] if version >= 4 else 0
    if has('H') and has('C'):
        row[F('tempTarget')] = 0
        row[F('tempDrive')] = 0
        dropped.append('H+C annul')
    elif has('H'):
        row[F('tempTarget')] = C['H_TARGET']
        row[F('tempDrive')] = C['HC_DRIVE']
        row[F('spawnTemp')] = C['H_TARGET']
    elif has('C'):
        row[F('tempTarget')] = C['C_TARGET']
        row[F('tempDrive')] = C['HC_DRIVE']
        row[F('spawnTemp')] = C['C_TARGET']
    if has('Y'):
        needs.append({'field': 'meltTo', 'base': MAT_WATER, 'bits': MOD['YPROD']})
    if bits & MOD['YPROD']:
        row[F('freezePt')] = NEVER_COLD
        row[F('freezeTo')] = 0
    io = bits & (MOD['I'] | MOD['O'] | MOD['IO_NULL'])
    if io == 0 and mech == base and not needs and all(
            i == F('tint') or w == int(mats[base][i]) for i, w in enumerate(row)):
        return [int(x) for x in mats[base]], [], dropped, True
    if row[F('bondK')] != 0:
        row[F('bondGroup')] = -2
    row[F('tint')] = compose_tint(int(mats[mech][F('tint')]), bits)
    if row[F('tempDrive')] != 0:
        tt = row[F('tempTarget')]
        if not (tt < row[F('meltPt')] and tt < row[F('boilPt')]):
            raise SynthError(f'synth: {mod_letters(bits)} on {base} refused: tempTarget at or above its own meltPt/boilPt')
        if not (tt > row[F('freezePt')] and tt > row[F('condPt')]):
            raise SynthError(f'synth: {mod_letters(bits)} on {base} refused: tempTarget at or below its own freezePt/condPt')
    return row, needs, dropped, False


class Interner:
    """The intern cache (src/engine.js:4981-5245) over one engine.

    ``intern(base, bits)`` answers a row id: a cache hit, a new row minted in
    the table's free tail, a recycled row (the least recently used one that
    no live particle and no other row's products can still reach), or a
    projection onto the nearest live interned row when nothing is free.
    ``events`` is the ordered record (MINT / RECYCLE / PROJECT) a replay
    re-applies with ``apply_events``. ``note_spawn(mats)`` is the spawn
    accounting the reference's ``spawnFluid`` does for interned rows.
    """

    def __init__(self, eng, authored=None, mat_count: Optional[int] = None):
        self.eng = eng
        self.authored = np.asarray(data.mats() if authored is None else authored).reshape(-1, 48).copy()
        self.authored_count = len(self.authored)
        self.mat_count = self.authored_count if mat_count is None else int(mat_count)
        self.by_row: Dict[int, dict] = {}
        self.by_key: Dict[tuple, int] = {}
        self.spawned: Dict[int, int] = {}
        self.events: List[dict] = []
        self.tick = 0
        self.substep = self._clock

    def _clock(self) -> int:
        try:
            return int(self.eng.formation_clock)
        except Exception:  # no scene loaded yet (a replay applies its record first)
            return 0

    @staticmethod
    def _key(base, bits, mask):
        return (int(base), int(bits), None if mask is None else int(mask) & 0xffffffff)

    def _row_words(self, m: int):
        if m < self.authored_count:
            return [int(x) for x in self.authored[m]]
        return self.by_row[m]['words']

    # -- the policy ----------------------------------------------------------------------
    def intern(self, base: int, bits: int, pinned=(), recipe_mask: Optional[int] = None) -> dict:
        before = len(self.events)
        row = self._resolve(int(base), int(bits), 1, set(pinned), recipe_mask)
        ev = self.events[before:]
        kind = ('hit' if not ev else 'project' if any(e['type'] == 'PROJECT' for e in ev)
                else 'recycle' if any(e['type'] == 'RECYCLE' for e in ev) else 'mint')
        return {'rowId': row, 'kind': kind, 'events': ev}

    def _resolve(self, base, bits, depth, pinned, mask=None) -> int:
        key = self._key(base, bits, mask)
        hit = self.by_key.get(key)
        if hit is not None:
            self.tick += 1
            self.by_row[hit]['tick'] = self.tick
            return hit
        words, needs, dropped, identity = synth(base, bits, self.authored)
        if identity:
            return base
        for need in needs:
            f = F(need['field'])
            if depth + 1 > 2:
                self.events.append({'type': 'PROJECT', 'substep': self.substep(), 'base': need['base'],
                                    'bits': need['bits'], 'rowId': words[f],
                                    'reason': 'products-closure depth > 2'})
                continue
            words[f] = self._resolve(need['base'], need['bits'], depth + 1, pinned)
        if self.mat_count < MAT_MAX:
            return self._mint(self.mat_count, base, bits, words, dropped, mask)
        victim = None
        for e in self.by_row.values():
            if not self._recyclable(e['rowId'], pinned):
                continue
            if victim is None or e['tick'] < victim['tick'] or (e['tick'] == victim['tick'] and e['rowId'] < victim['rowId']):
                victim = e
        if victim is not None:
            ev = {'type': 'RECYCLE', 'substep': self.substep(), 'rowId': victim['rowId'], 'base': victim['base'],
                  'bits': victim['bits']}
            if victim.get('recipeMask') is not None:
                ev['recipeMask'] = victim['recipeMask']
            self.events.append(ev)
            self._forget(victim['rowId'])
            return self._mint(victim['rowId'], base, bits, words, dropped, mask)
        target = self._project(words, bits, mask)
        if target < 0 and bits & (MOD['I'] | MOD['O']):
            raise SynthError('internMaterial: the cache is full and no row with the same Inflow/Outflow recipe exists')
        ev = {'type': 'PROJECT', 'substep': self.substep(), 'base': base, 'bits': bits, 'rowId': target,
              'reason': 'intern cache full and nothing recyclable'}
        if mask is not None:
            ev['recipeMask'] = int(mask) & 0xffffffff
        self.events.append(ev)
        return target

    def _forget(self, row):
        e = self.by_row.pop(row)
        self.by_key.pop(self._key(e['base'], e['bits'], e.get('recipeMask')), None)
        self.spawned.pop(row, None)

    def _recyclable(self, row: int, pinned) -> bool:
        if row in pinned:
            return False
        for e in self.by_row.values():
            if e['rowId'] != row and any(e['words'][F(p)] == row for p in PRODUCTS):
                return False
        if self.spawned.get(row, 0) <= 0:
            return True
        # a row ever worn is free only when no particle wears it now (the
        # reference reads its position mirror; this reads the state)
        st = self.eng.read_state().reshape(-1, 8)
        if ((st[:, 4].astype(np.int64) & 0xffffffff) == row).any():
            return False
        self.spawned[row] = 0
        return True

    def _project(self, words, bits, mask) -> int:
        best, best_d = -1, None
        io = bits & (MOD['I'] | MOD['O'])
        for e in self.by_row.values():
            if io:
                if (e['bits'] & (MOD['I'] | MOD['O'])) != io or e.get('recipeMask') != mask:
                    continue
            d = sum(abs(words[F(a)] - e['words'][F(a)]) for a in PROJECT_AXES)
            if best_d is None or d < best_d or (d == best_d and e['rowId'] < best):
                best, best_d = e['rowId'], d
        if best < 0 and io:
            return -1
        if best < 0:
            for m in range(self.authored_count):
                if self.authored[m][F('phantom')] != 0:
                    continue
                d = sum(abs(words[F(a)] - int(self.authored[m][F(a)])) for a in PROJECT_AXES)
                if best_d is None or d < best_d:
                    best, best_d = m, d
        return best

    def _validate(self, words, row):
        def bad(msg):
            raise SynthError(f'intern row {row}: {msg}')
        for w in words:
            if not (-2147483648 <= int(w) <= 2147483647):
                bad('a word is not an i32')
        if words[F('eps')] < 32768:
            bad('eps < 32768')
        if words[F('dpMax')] <= 0:
            bad('dpMax <= 0')
        if not (0 <= words[F('xsph')] <= XSPH_MAX):
            bad('xsph range')
        if not (0 <= words[F('cond')] <= COND_MAX):
            bad('cond range')
        if not (0 <= words[F('coolRate')] <= 65536) or not (0 <= words[F('tempDrive')] <= 65536):
            bad('coolRate/tempDrive range')
        if words[F('burstP')] < 0 or words[F('sealMode')] not in (0, 1):
            bad('burstP/sealMode')
        if words[F('bondK')] != 0 and words[F('bondGroup')] != 64 + row:
            bad('bondGroup is not 64 + rowId')
        if not (0 <= words[F('bondK')] <= BOND_K_MAX):
            bad('bondK range')
        if words[F('rampHi')] - words[F('rampLo')] < 65536:
            bad('ramp narrower than 1 degree')
        for p in PRODUCTS:
            t = words[F(p)]
            if not (0 <= t and (t < self.mat_count or t == row)):
                bad(f'{p} = {t} is not a live material id')

    def _mint(self, row, base, bits, words, dropped, mask=None) -> int:
        words = list(words)
        if words[F('bondGroup')] == -2:
            words[F('bondGroup')] = 64 + row
        self._validate(words, row)
        self.mat_count = self.eng.set_material(row, words)
        self.tick += 1
        entry = {'rowId': row, 'base': base, 'bits': bits, 'synthVersion': SYNTH_VERSION, 'words': words,
                 'tick': self.tick, 'dropped': list(dropped)}
        if mask is not None:
            entry['recipeMask'] = int(mask) & 0xffffffff
        self.by_key[self._key(base, bits, mask)] = row
        self.by_row[row] = entry
        ev = {'type': 'MINT', 'substep': self.substep(), 'rowId': row, 'base': base, 'bits': bits,
              'synthVersion': SYNTH_VERSION, 'words': list(words), 'dropped': list(dropped)}
        if mask is not None:
            ev['recipeMask'] = int(mask) & 0xffffffff
        self.events.append(ev)
        return row

    def note_spawn(self, mats):
        """spawnFluid's accounting (src/engine.js:5944-5952): an interned row
        being painted is in use (its wearer count and LRU clock move)."""
        for m in mats:
            m = int(m)
            if m >= self.authored_count:
                self.spawned[m] = self.spawned.get(m, 0) + 1
                if m in self.by_row:
                    self.tick += 1
                    self.by_row[m]['tick'] = self.tick

    # -- replay ------------------------------------------------------------------------
    def apply_events(self, events):
        """applyMintEvents (src/engine.js:5211-5233): re-derive every MINT at its
        recorded version and refuse the list on any disagreeing word."""
        for ev in events or ():
            t = ev.get('type')
            if t == 'RECYCLE':
                e = self.by_row.get(ev['rowId'])
                if (e is None or e['base'] != ev['base'] or e['bits'] != ev['bits'] or
                        e.get('recipeMask') != ev.get('recipeMask')):
                    raise SynthError(f"applyMintEvents: RECYCLE of row {ev['rowId']} does not match the live entry")
                self.events.append(dict(ev))
                self._forget(ev['rowId'])
                continue
            if t == 'PROJECT':
                self.events.append(dict(ev))
                continue
            if t != 'MINT':
                raise SynthError(f'applyMintEvents: unknown event {t}')
            words, needs, _, _ = synth(ev['base'], ev['bits'], self.authored, ev['synthVersion'])
            for need in needs:
                child = self.by_key.get(self._key(need['base'], need['bits'], None))
                words[F(need['field'])] = child if child is not None else ev['words'][F(need['field'])]
            if words[F('bondGroup')] == -2:
                words[F('bondGroup')] = 64 + ev['rowId']
            for w in range(48):
                if int(words[w]) != int(ev['words'][w]):
                    raise SynthError(f"applyMintEvents refused: row {ev['rowId']} re-derives "
                                     f"{data.MAT_FIELDS[w]} = {words[w]}, the record holds {ev['words'][w]}")
            if ev['rowId'] in self.by_row:
                raise SynthError(f"applyMintEvents: row {ev['rowId']} minted twice without a RECYCLE")
            self._mint(ev['rowId'], ev['base'], ev['bits'], words, ev.get('dropped', []), ev.get('recipeMask'))
            self.events[-1]['substep'] = ev.get('substep', 0)

    def clear(self):
        """clearInterned (src/engine.js:5235-5245)."""
        self.eng.clear_materials()
        self.mat_count = self.authored_count
        self.by_row.clear()
        self.by_key.clear()
        self.spawned.clear()
        self.events.clear()
