"""Generate the frozen data files the engine ships with.

Run once, in a checkout that has the SunaEngine reference tree available::

    python sunaengine_gb300/data/gen_data.py /path/to/sunaengine

It writes two files next to itself and nothing else:

``luts.bin``
    The five frozen kernel tables (W, G, C, A, S; 3202 little-endian int32
    words each, 16010 words in all), decoded from the reference's
    ``src/tables.json`` (``b64`` field) and checked against the table hash the
    reference verifies at every load (``src/tables.js:158-178``,
    ``src/engine.js:501``). The tables are never regenerated from the f64
    generator: that generator uses ``pow`` and is deliberately offline-only
    (``src/tables.js:9-18``).

``mats.json``
    The 28 authored material rows as 48-word integer arrays in the reference's
    field order (``MAT_FIELDS``, ``src/engine.js:678-705``), obtained by
    evaluating every ``mat({...})`` call of ``MATS`` (``src/engine.js:1192``)
    with the reference's defaults (``MAT_DEFAULTS``, ``src/engine.js:713-731``),
    its ``gammaCur = gammaCoh / 4`` default rule and its ``rampInv`` bake
    (``mat()``, ``src/engine.js:733-756``).

Both are data the solver's results depend on bit for bit, so they are carried
verbatim; the table hash is re-checked by the engine at load time.
"""
from __future__ import annotations

import base64
import json
import re
import struct
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent

ONE = 65536
TEMP_ONE = 65536
NEVER_HOT = 2147483647
NEVER_COLD = -2147483648
TEMP_MIN = -33554432
AMBIENT = 20 * TEMP_ONE

MAT_FIELDS = [
    'eps', 'dpMax', 'xsph', 'phantom', 'gammaCoh', 'gammaCur', 'adhesion', 'grav',
    'cond', 'coolRate', 'heatCap',
    'meltPt', 'meltTo', 'freezePt', 'freezeTo', 'boilPt', 'boilTo', 'condPt', 'condTo',
    'ignitePt', 'fuel0', 'burnRate', 'burnHeat', 'burnTo',
    'splitTo', 'splitPct', 'spawnTemp', 'tint',
    'corrode', 'corrPt', 'corrTo', 'fric',
    'bondK', 'bondBreak', 'bondReform', 'bondFormV', 'bondFormP', 'bondMu',
    'bondGroup', 'rampLo', 'rampHi', 'rampInv', 'rampSign',
    'solidMode', 'tempTarget', 'tempDrive', 'burstP', 'sealMode',
]
assert len(MAT_FIELDS) == 48

MAT_DEFAULTS = dict(
    eps=40000, dpMax=16384, xsph=6000, phantom=0,
    gammaCoh=240, gammaCur=60, adhesion=0, grav=1200,
    cond=0, coolRate=0, heatCap=0,
    meltPt=NEVER_HOT, meltTo=0, freezePt=NEVER_COLD, freezeTo=0,
    boilPt=NEVER_HOT, boilTo=0, condPt=NEVER_COLD, condTo=0,
    ignitePt=NEVER_HOT, fuel0=0, burnRate=0, burnHeat=0, burnTo=0,
    splitTo=0, splitPct=0, spawnTemp=AMBIENT, tint=0x8090a0,
    corrode=0, corrPt=NEVER_HOT, corrTo=0, fric=0,
    bondK=0, bondBreak=0, bondReform=0, bondFormV=0, bondFormP=0, bondMu=0,
    bondGroup=-1, rampLo=0, rampHi=65536, rampInv=0, rampSign=0,
    solidMode=0, tempTarget=0, tempDrive=0, burstP=0, sealMode=0,
)

MAT_NAMES = [
    'WATER', 'GEL', 'ICE', 'STEAM', 'OIL', 'FIRE', 'SMOKE', 'WOOD',
    'ASH', 'LAVA', 'STONE', 'SAND', 'METAL', 'MOLTEN', 'GAS', 'PHOTO',
    'CRYO', 'RUBBER', 'TAR', 'MERCURY', 'DUST', 'ACID', 'NITRO', 'BLAST',
    'VOID', 'RICE', 'BEDROCK', 'ORBIES',
]

TABLE_HASH = '31ebf1f3e1b168a800f0f180007dd390d0dc182fd06e398adfeec08e8a62908b'


def _mm_step(h: int, k: int) -> int:
    k = (k * 0xcc9e2d51) & 0xffffffff
    k = ((k << 15) | (k >> 17)) & 0xffffffff
    k = (k * 0x1b873593) & 0xffffffff
    h ^= k
    h = ((h << 13) | (h >> 19)) & 0xffffffff
    return (h * 5 + 0xe6546b64) & 0xffffffff


def _fmix(h: int) -> int:
    h ^= h >> 16
    h = (h * 0x85ebca6b) & 0xffffffff
    h ^= h >> 13
    h = (h * 0xc2b2ae35) & 0xffffffff
    return h ^ (h >> 16)


def table_hash(words) -> str:
    """Hash of a table image: 4 salted Murmur lanes, set + slot accumulators.

    Follows ``tableHash`` (``src/tables.js:158-178``).
    """
    seeds = (0x9e3779b1, 0x85ebca77, 0xc2b2ae3d, 0x27d4eb2f)
    salts = (0x00000000, 0x51633e2d, 0x9c8f2a17, 0xd0e5b943)
    acc = [0] * 8
    for i, w in enumerate(words):
        k = w & 0xffffffff
        h = [_mm_step(seeds[l], k ^ salts[l]) for l in range(4)]
        for l in range(4):
            acc[l] = (acc[l] + _fmix(h[l] ^ 1)) & 0xffffffff
            acc[4 + l] = (acc[4 + l] + _fmix(_mm_step(h[l], i) ^ 2)) & 0xffffffff
    return ''.join(f'{a:08x}' for a in acc)


def _eval_mats(engine_js: str):
    start = engine_js.index('export const MATS = [')
    end = engine_js.index('\n];', start)
    body = engine_js[start:end]
    body = re.sub(r'//[^\n]*', '', body)
    ids = {f'MAT_{n}': i for i, n in enumerate(MAT_NAMES)}
    ids['MAT_GOO'] = 1
    env = dict(ids, DEG=lambda d: d * TEMP_ONE, NEVER_HOT=NEVER_HOT, NEVER_COLD=NEVER_COLD,
               TEMP_MIN=TEMP_MIN, AMBIENT=AMBIENT, SOLID_NONE=0, SOLID_BOND=1, SOLID_RIGID=2)
    rows = []
    for m in re.finditer(r'mat\(\{(.*?)\}\)', body, re.S):
        fields = {}
        for part in m.group(1).split(','):
            part = part.strip()
            if not part:
                continue
            key, expr = part.split(':', 1)
            key = key.strip()
            if key not in MAT_DEFAULTS:
                raise ValueError(f'unknown material field {key}')
            fields[key] = int(eval(expr.strip(), {'__builtins__': {}}, env))
        row = [fields.get(f, MAT_DEFAULTS[f]) for f in MAT_FIELDS]
        if 'gammaCoh' in fields and 'gammaCur' not in fields:
            # JS `(x / 4) | 0` truncates toward zero.
            g = fields['gammaCoh']
            row[MAT_FIELDS.index('gammaCur')] = int(g / 4)
        span = row[MAT_FIELDS.index('rampHi')] - row[MAT_FIELDS.index('rampLo')]
        row[MAT_FIELDS.index('rampInv')] = (2 ** 32) // span if span > 0 else 0
        rows.append(row)
    if len(rows) != len(MAT_NAMES):
        raise ValueError(f'parsed {len(rows)} material rows, expected {len(MAT_NAMES)}')
    return rows


def main(ref_root: str) -> None:
    ref = Path(ref_root)
    tables = json.loads((ref / 'src' / 'tables.json').read_text())
    raw = base64.b64decode(tables['b64'])
    words = list(struct.unpack(f'<{len(raw) // 4}i', raw))
    if len(words) != 5 * 3202:
        raise ValueError('unexpected table length')
    h = table_hash(words)
    if h != TABLE_HASH or h != tables['tableHash']:
        raise ValueError(f'table hash mismatch {h}')
    (HERE / 'luts.bin').write_bytes(raw)

    rows = _eval_mats((ref / 'src' / 'engine.js').read_text())
    doc = {'fields': MAT_FIELDS, 'names': MAT_NAMES, 'rows': rows}
    (HERE / 'mats.json').write_text(json.dumps(doc, indent=1) + '\n')
    print('wrote luts.bin', h, 'and', len(rows), 'material rows')


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: python gen_data.py <path of a SunaEngine checkout>')
    main(sys.argv[1])
