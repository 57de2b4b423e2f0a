"""The C-ABI library builds for sm_103a and exports every symbol include/suna.h declares.

No compute calls are made here, so this runs without a GPU.
"""
import ctypes
import re
from pathlib import Path

from sunaengine_gb300 import _native

HEADER = Path(__file__).resolve().parent.parent / 'include' / 'suna.h'


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(sn3?_[a-z0-9_]+)\s*\(', text)))


def test_header_declares_the_engine_surface():
    names = declared_symbols()
    for n in ('sn_create', 'sn_load_scene', 'sn_step', 'sn_digest', 'sn_chain', 'sn_spawn', 'sn_impulse',
              'sn_batch_create', 'sn_batch_step', 'sn3_create', 'sn3_load_scene', 'sn3_step', 'sn3_fnv',
              'sn3_chain', 'sn3_spawn', 'sn3_set_ball', 'sn3_add_scene'):
        assert n in names


def test_library_exports_every_declared_symbol():
    path = _native.build()
    lib = ctypes.CDLL(str(path))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, f'not exported: {missing}'
    # and the python binding covers the same set
    assert set(_native.SIGNATURES) == set(declared_symbols())
