"""Frozen data the engine depends on bit for bit: kernel LUTs and material rows.

``luts.bin`` is the reference's frozen kernel table image (5 x 3202 int32,
``src/tables.json``); ``mats.json`` holds the 28 authored material rows of
``MATS`` (``src/engine.js:1192``) in ``MAT_FIELDS`` order. Both are produced by
``gen_data.py`` in this folder. The table hash is re-verified on every load,
as the reference does (``src/engine.js:2945-2989``).
"""
from __future__ import annotations

import json
from functools import lru_cache
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

TABLE_HASH = '31ebf1f3e1b168a800f0f180007dd390d0dc182fd06e398adfeec08e8a62908b'
TN = 3202
LUT_WORDS = 5 * TN
MAT_WORDS = 48
MAT_MAX = 64


def _mm_step(h, k):
    k = (k * np.uint32(0xcc9e2d51)).astype(np.uint32)
    k = ((k << np.uint32(15)) | (k >> np.uint32(17))).astype(np.uint32)
    k = (k * np.uint32(0x1b873593)).astype(np.uint32)
    h = h ^ k
    h = ((h << np.uint32(13)) | (h >> np.uint32(19))).astype(np.uint32)
    return (h * np.uint32(5) + np.uint32(0xe6546b64)).astype(np.uint32)


def _fmix(h):
    h = h ^ (h >> np.uint32(16))
    h = (h * np.uint32(0x85ebca6b)).astype(np.uint32)
    h = h ^ (h >> np.uint32(13))
    h = (h * np.uint32(0xc2b2ae35)).astype(np.uint32)
    return h ^ (h >> np.uint32(16))


def table_hash(words: np.ndarray) -> str:
    """4-lane salted Murmur hash of a table image (``src/tables.js:158-178``)."""
    k = words.astype(np.int64).astype(np.uint32)
    idx = np.arange(k.size, dtype=np.uint32)
    seeds = (0x9e3779b1, 0x85ebca77, 0xc2b2ae3d, 0x27d4eb2f)
    salts = (0x00000000, 0x51633e2d, 0x9c8f2a17, 0xd0e5b943)
    acc = []
    hs = []
    with np.errstate(over='ignore'):
        for lane in range(4):
            h = _mm_step(np.full(k.size, seeds[lane], np.uint32), k ^ np.uint32(salts[lane]))
            hs.append(h)
            acc.append(int(_fmix(h ^ np.uint32(1)).astype(np.uint64).sum()) & 0xffffffff)
        for lane in range(4):
            acc.append(int(_fmix(_mm_step(hs[lane], idx) ^ np.uint32(2)).astype(np.uint64).sum()) & 0xffffffff)
    return ''.join(f'{a:08x}' for a in acc)


@lru_cache(maxsize=1)
def luts() -> np.ndarray:
    """The frozen LUT image as int32[16010]; raises if its hash is wrong."""
    w = np.frombuffer((HERE / 'luts.bin').read_bytes(), dtype='<i4').astype(np.int32)
    if w.size != LUT_WORDS:
        raise RuntimeError(f'luts.bin has {w.size} words, expected {LUT_WORDS}')
    h = table_hash(w)
    if h != TABLE_HASH:
        raise RuntimeError(f'TABLE_HASH mismatch: {h} != {TABLE_HASH}')
    return w


@lru_cache(maxsize=1)
def _mats_doc():
    return json.loads((HERE / 'mats.json').read_text())


MAT_FIELDS = tuple(_mats_doc()['fields'])
MAT_NAMES = tuple(_mats_doc()['names'])


def mats() -> np.ndarray:
    """The authored material table as int32[rows, 48]."""
    rows = np.array(_mats_doc()['rows'], dtype=np.int64)
    return rows.astype(np.int32)


def mat_field(name: str) -> int:
    return MAT_FIELDS.index(name)


def mat_id(name: str) -> int:
    return MAT_NAMES.index(name)
