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


def test_noalloc_digest_refuses_oversize_without_a_launch():
    """sn_digest_device_noalloc refuses a size past its fixed scratch on the
    host, before any CUDA call, so host pointers are never dereferenced."""
    import numpy as np
    lib = _native.load()
    one = np.zeros(8, np.int32)
    out = np.zeros(8, np.uint32)
    rc = lib.sn_digest_device_noalloc(one.ctypes.data_as(ctypes.c_void_p), (1 << 24) + 1, 0, None,
                                      out.ctypes.data_as(ctypes.c_void_p), None)
    assert rc == -2  # SN_E_CAPACITY


def test_read_state_out_buffer_rules():
    """read_state(out=...) takes a caller's writeable contiguous 1-D int32
    array of at least the needed words and returns its leading view."""
    import numpy as np
    import pytest as _pt
    from sunaengine_gb300.engine import EngineError, _out_words
    buf = np.zeros(100, np.int32)
    v = _out_words(buf, 64)
    assert v.size == 64 and v.base is buf
    assert _out_words(None, 8).size == 8
    for bad in (np.zeros(63, np.int32), np.zeros(64, np.int64), np.zeros((8, 8), np.int32),
                np.zeros(128, np.int32)[::2]):
        with _pt.raises(EngineError):
            _out_words(bad, 64)
    ro = np.zeros(64, np.int32)
    ro.flags.writeable = False
    with _pt.raises(EngineError):
        _out_words(ro, 64)
