"""Device checkpoint pool (``sn_ckpt_pool`` in include/suna.h).

A pool is one device allocation. ``Engine.ckpt_save`` / ``Batch.ckpt_save`` /
``Engine3D.ckpt_save`` copy a scene's keyframe into it on the engine's stream
(no host round trip)
and return a handle; ``ckpt_load`` restores the scene to exactly that point.
"""
from __future__ import annotations

import ctypes

from . import _native
from .engine import EngineError


class CheckpointPool:
    def __init__(self, nbytes: int, device: int = 0):
        self._lib = _native.load()
        h = ctypes.c_void_p()
        rc = self._lib.sn_ckpt_pool_create(int(nbytes), int(device), ctypes.byref(h))
        if rc != 0 or not h.value:
            raise EngineError(f'sn_ckpt_pool_create({nbytes}) failed ({rc})')
        self.h = h

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self._lib.sn_ckpt_pool_last_error(self.h)
            raise EngineError(f'[ckpt] {what}: {msg.decode() if msg else rc}')

    def usage(self):
        used = ctypes.c_size_t()
        cap = ctypes.c_size_t()
        self._check(self._lib.sn_ckpt_pool_usage(self.h, ctypes.byref(used), ctypes.byref(cap)), 'usage')
        return int(used.value), int(cap.value)

    def free(self, handle: int):
        self._check(self._lib.sn_ckpt_free(self.h, int(handle)), 'free')

    def close(self):
        if getattr(self, 'h', None):
            self._lib.sn_ckpt_pool_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
