"""The `.suna` scene container and `.sunar` replay formats.

`.suna` (``src/suna.js:46-124``) is JSON: header, scene scalars, and exact
integer buffers as base64 little-endian words (``state``: n x 8 int32,
``tints``: n uint32, optional exact sidecars). `.sunar`
(``src/sunar.js:27-92``) is one initial `.suna` plus a journal of inputs
sorted by (frame, order), the timing block and the final digest.

Field names, magic strings and validation rules follow the reference so
files are interchangeable; the codec here is this package's own.
"""
from __future__ import annotations

import base64
import json
from typing import Any, Optional

import numpy as np

SUNA_MAGIC = 'SunaBox Scene'
SUNA_FORMAT_VERSION = 1
SUNA_EXTENSION = '.suna'
SUNAR_MAGIC = 'SunaBox Replay'
SUNAR_FORMAT_VERSION = 1
SUNAR_EXTENSION = '.sunar'
MAX_SUNA_PARTICLES = 131072


class FormatError(ValueError):
    pass


def _integer(x, label, lo=-2147483648, hi=2147483647):
    if isinstance(x, bool) or not isinstance(x, (int, np.integer)) or x < lo or x > hi:
        raise FormatError(f'{label} is outside {lo}..{hi}')
    return int(x)


def _pack(a: np.ndarray, dtype) -> str:
    return base64.b64encode(np.ascontiguousarray(a, dtype=dtype).astype(dtype).tobytes()).decode('ascii')


def _unpack(s: str, dtype, words: int, label: str) -> np.ndarray:
    raw = base64.b64decode(s or '')
    if len(raw) != words * 4:
        raise FormatError(f'{label} has {len(raw)} bytes; expected {words * 4}')
    return np.frombuffer(raw, dtype=dtype).copy()


def encode_suna(payload: dict) -> str:
    """encodeSuna (src/suna.js:46-84). payload: {app, scene:{n, nFluid, ...},
    state: int32[n*8], tints: uint32[n], optional bonds/bondCand/bodyRecords/restOffsets}."""
    state = payload.get('state')
    tints = payload.get('tints')
    if not isinstance(state, np.ndarray) or state.dtype != np.int32:
        raise FormatError('Suna save needs an Int32Array state')
    if not isinstance(tints, np.ndarray) or tints.dtype != np.uint32:
        raise FormatError('Suna save needs a Uint32Array tint buffer')
    scene = dict(payload.get('scene') or {})
    n = _integer(scene.get('n'), 'scene.n', 0, MAX_SUNA_PARTICLES)
    _integer(scene.get('nFluid'), 'scene.nFluid', 0, n)
    if state.size != n * 8:
        raise FormatError(f'state has {state.size} words; expected {n * 8}')
    if tints.size != n:
        raise FormatError(f'tints has {tints.size} words; expected {n}')
    ex = [payload.get(k) for k in ('bonds', 'bondCand', 'bodyRecords', 'restOffsets')]
    exact = all(isinstance(a, np.ndarray) for a in ex)
    if exact:
        bonds, cand, bodies, rest = ex
        if bonds.size != cand.size:
            raise FormatError('bond and candidate tables differ in size')
        if rest.size != n * 2:
            raise FormatError(f'rest offsets have {rest.size} words; expected {n * 2}')
    sc = dict(scene)
    sc['state'] = {'encoding': 'i32le/base64', 'words': int(state.size), 'data': _pack(state, '<i4')}
    sc['tints'] = {'encoding': 'u32le/base64', 'words': int(tints.size), 'data': _pack(tints, '<u4')}
    if exact:
        sc['bonds'] = {'encoding': 'u32le/base64', 'words': int(bonds.size), 'data': _pack(bonds, '<u4')}
        sc['bondCandidates'] = {'encoding': 'u32le/base64', 'words': int(cand.size), 'data': _pack(cand, '<u4')}
        sc['bodyRecords'] = {'encoding': 'i32le/base64', 'words': int(bodies.size), 'data': _pack(bodies, '<i4')}
        sc['restOffsets'] = {'encoding': 'i32le/base64', 'words': int(rest.size), 'data': _pack(rest, '<i4')}
    doc = {
        'magic': SUNA_MAGIC,
        'formatVersion': SUNA_FORMAT_VERSION,
        'app': payload.get('app'),
        'scene': sc,
        'materials': payload.get('materials') or {'events': []},
        'bodies': payload.get('bodies') or [],
        'drivers': payload.get('drivers') or [],
        'devices': payload.get('devices') or [],
        'settings': payload.get('settings') or {},
    }
    return json.dumps(doc, indent=2) + '\n'


def decode_suna(source) -> dict:
    """decodeSuna (src/suna.js:86-124)."""
    text = source.decode() if isinstance(source, (bytes, bytearray)) else source
    try:
        doc = json.loads(text)
    except json.JSONDecodeError as e:
        raise FormatError(f'not valid JSON: {e}') from None
    if not isinstance(doc, dict) or doc.get('magic') != SUNA_MAGIC:
        raise FormatError(f'not a {SUNA_MAGIC} file')
    if doc.get('formatVersion') != 1:
        raise FormatError(f'unsupported .suna formatVersion {doc.get("formatVersion")}; this build reads 1')
    s = doc.get('scene') or {}
    n = _integer(s.get('n'), 'scene.n', 0, MAX_SUNA_PARTICLES)
    _integer(s.get('nFluid'), 'scene.nFluid', 0, n)
    _integer(s.get('domW'), 'scene.domW', 1)
    _integer(s.get('domH'), 'scene.domH', 1)
    _integer(s.get('cellShift'), 'scene.cellShift', 1, 27)
    state = _unpack((s.get('state') or {}).get('data', ''), '<i4', n * 8, 'scene.state').astype(np.int32)
    tints = _unpack((s.get('tints') or {}).get('data', ''), '<u4', n, 'scene.tints').astype(np.uint32)
    has_exact = all(s.get(k) for k in ('bonds', 'bondCandidates', 'bodyRecords', 'restOffsets'))
    ex = {}
    if has_exact:
        for key, name, dt in (('bonds', 'bonds', '<u4'), ('bondCandidates', 'bondCand', '<u4'),
                              ('bodyRecords', 'bodyRecords', '<i4'), ('restOffsets', 'restOffsets', '<i4')):
            words = _integer(s[key].get('words'), f'scene.{key}.words', 0)
            ex[name] = _unpack(s[key].get('data', ''), dt, words, f'scene.{key}')
    scene = {k: v for k, v in s.items()
             if k not in ('state', 'tints', 'bonds', 'bondCandidates', 'bodyRecords', 'restOffsets')}
    out = dict(doc)
    out.update({'scene': scene, 'state': state, 'tints': tints,
                'bonds': ex.get('bonds'), 'bondCand': ex.get('bondCand'),
                'bodyRecords': ex.get('bodyRecords'), 'restOffsets': ex.get('restOffsets')})
    return out


def _check_events(events):
    prev_f, prev_o = -1, -1
    for i, e in enumerate(events):
        e = e or {}
        f = _integer(e.get('frame'), f'events[{i}].frame', 0, 0x7fffffff)
        o = _integer(e.get('order'), f'events[{i}].order', 0, 0x7fffffff)
        if f < prev_f or (f == prev_f and o <= prev_o):
            raise FormatError(f'events[{i}] is not in stable frame/order sequence')
        if not isinstance(e.get('type'), str) or not e.get('type'):
            raise FormatError(f'events[{i}].type is empty')
        prev_f, prev_o = f, o


def encode_sunar(replay: dict) -> str:
    """encodeSunar (src/sunar.js:27-56)."""
    if not replay or not replay.get('initial'):
        raise FormatError('Suna replay needs an initial scene')
    events = list(replay.get('events') or [])
    _check_events(events)
    initial = json.loads(encode_suna(replay['initial']))
    doc = {
        'magic': SUNAR_MAGIC,
        'formatVersion': SUNAR_FORMAT_VERSION,
        'app': replay.get('app', initial.get('app')),
        'timing': {
            'substepsPerFrame': _integer(replay.get('substepsPerFrame', 2), 'substepsPerFrame', 1, 32),
            'durationFrames': _integer(replay.get('durationFrames', 0), 'durationFrames', 0, 0x7fffffff),
            'durationSubsteps': _integer(replay.get('durationSubsteps', 0), 'durationSubsteps', 0, 0x7fffffff),
        },
        'initial': initial,
        'events': events,
        'final': replay.get('final'),
    }
    return json.dumps(doc, indent=2) + '\n'


def decode_sunar(source) -> dict:
    """decodeSunar (src/sunar.js:58-92)."""
    text = source.decode() if isinstance(source, (bytes, bytearray)) else source
    try:
        doc = json.loads(text)
    except json.JSONDecodeError as e:
        raise FormatError(f'not valid JSON: {e}') from None
    if not isinstance(doc, dict) or doc.get('magic') != SUNAR_MAGIC:
        raise FormatError(f'not a {SUNAR_MAGIC} file')
    if doc.get('formatVersion') != SUNAR_FORMAT_VERSION:
        raise FormatError(f'unsupported .sunar formatVersion {doc.get("formatVersion")}; this build reads 1')
    timing = doc.get('timing') or {}
    _integer(timing.get('substepsPerFrame'), 'timing.substepsPerFrame', 1, 32)
    _integer(timing.get('durationFrames'), 'timing.durationFrames', 0, 0x7fffffff)
    _integer(timing.get('durationSubsteps'), 'timing.durationSubsteps', 0, 0x7fffffff)
    events = doc.get('events') if isinstance(doc.get('events'), list) else []
    _check_events(events)
    return {
        'app': doc.get('app'),
        'substepsPerFrame': timing['substepsPerFrame'],
        'durationFrames': timing['durationFrames'],
        'durationSubsteps': timing['durationSubsteps'],
        'initial': decode_suna(json.dumps(doc.get('initial'))),
        'events': events,
        'final': doc.get('final'),
    }
