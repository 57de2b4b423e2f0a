"""The no-allocation digest entry point against the engine's own digest.

sn_digest_device_noalloc serves callers that cannot allocate device memory
when they need a digest (latency-bound loops that cannot take cudaMalloc's
device synchronisation, hosts that own all device memory). Its scratch is a
fixed array in the library's device image. These tests call it through the C
ABI on buffers the test owns and require the 8 digest words to equal
sn_digest's bit for bit: on two calls in a row over two different states, and
under a second CUDA context created on the same device, where the scratch
array has a different device address than under the primary context. (The
over-limit refusal is a host check; tests/test_native_abi.py covers it
without a GPU.) They are kept in a file of their own so that they run last and
run the same alone or after the other tests.
"""
import ctypes

import numpy as np
import pytest

from sunaengine_gb300 import _native, scenes
from sunaengine_gb300.engine import Engine

pytestmark = pytest.mark.gpu


def _noalloc_digest(lib, torch, state: np.ndarray, n: int, n_fluid: int, bonds: np.ndarray):
    d_state = torch.from_numpy(state.astype(np.int32)).cuda()
    d_bond = torch.from_numpy(bonds.view(np.int32)).cuda() if bonds is not None else None
    d_out = torch.full((8,), -1, dtype=torch.int32, device='cuda')
    stream = torch.cuda.current_stream()
    rc = lib.sn_digest_device_noalloc(ctypes.c_void_p(d_state.data_ptr()), n, n_fluid,
                                      ctypes.c_void_p(d_bond.data_ptr()) if d_bond is not None else None,
                                      ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(np.uint32)


def test_noalloc_digest_matches_engine_digest_twice():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    lib = _native.load()
    sc = scenes.make_scene('stretch_v1')  # GEL: bonds form, so the bond fold is exercised
    e = Engine(max_particles=sc.n + 64).load_scene(sc)
    seen = []
    for steps in (9, 21):
        e.step(steps)
        want = e.digest().acc
        got = _noalloc_digest(lib, torch, e.read_state(), e.n, e.n_fluid, e.read_bonds())
        assert np.array_equal(got, want), f'after {e.substep_count} substeps'
        seen.append(got.tobytes())
    assert seen[0] != seen[1]
    # a state with no bond rows at all
    e2 = Engine(max_particles=8192).load_scene(scenes.make_scene('dambreak_v1'))
    e2.step(5)
    got = _noalloc_digest(lib, torch, e2.read_state(), e2.n, e2.n_fluid, None)
    assert np.array_equal(got, e2.digest().acc)


class _DriverContext:
    """A context created with the driver API on device 0, made current on this
    thread while the `with` block runs, with buffers allocated in it."""

    def __init__(self):
        self.cu = ctypes.CDLL('libcuda.so.1')
        self.ctx = ctypes.c_void_p()
        self.bufs = []

    def _ok(self, rc, what):
        assert rc == 0, f'{what} returned CUresult {rc}'

    def __enter__(self):
        dev = ctypes.c_int()
        self._ok(self.cu.cuDeviceGet(ctypes.byref(dev), 0), 'cuDeviceGet')
        # the new context is pushed current on this thread
        if hasattr(self.cu, 'cuCtxCreate_v2'):
            rc = self.cu.cuCtxCreate_v2(ctypes.byref(self.ctx), 0, dev)
        else:
            rc = self.cu.cuCtxCreate_v4(ctypes.byref(self.ctx), None, 0, dev)
        self._ok(rc, 'cuCtxCreate')
        return self

    def to_device(self, arr: np.ndarray) -> int:
        ptr = ctypes.c_uint64()
        self._ok(self.cu.cuMemAlloc_v2(ctypes.byref(ptr), ctypes.c_size_t(max(arr.nbytes, 4))), 'cuMemAlloc')
        self.bufs.append(ptr.value)
        if arr.nbytes:
            self._ok(self.cu.cuMemcpyHtoD_v2(ctypes.c_uint64(ptr.value), arr.ctypes.data_as(ctypes.c_void_p),
                                             ctypes.c_size_t(arr.nbytes)), 'cuMemcpyHtoD')
        return ptr.value

    def to_host(self, ptr: int, arr: np.ndarray) -> np.ndarray:
        self._ok(self.cu.cuCtxSynchronize(), 'cuCtxSynchronize')
        self._ok(self.cu.cuMemcpyDtoH_v2(arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint64(ptr),
                                         ctypes.c_size_t(arr.nbytes)), 'cuMemcpyDtoH')
        return arr

    def __exit__(self, *exc):
        for ptr in self.bufs:
            self.cu.cuMemFree_v2(ctypes.c_uint64(ptr))
        popped = ctypes.c_void_p()
        self.cu.cuCtxPopCurrent_v2(ctypes.byref(popped))
        self.cu.cuCtxDestroy_v2(self.ctx)
        return False


def test_noalloc_digest_under_a_second_context():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('needs a GPU')
    lib = _native.load()
    sc = scenes.make_scene('stretch_v1')
    e = Engine(max_particles=sc.n + 64).load_scene(sc)
    e.step(13)
    want = e.digest().acc
    state = np.ascontiguousarray(e.read_state().astype(np.int32))
    bonds = np.ascontiguousarray(e.read_bonds().view(np.uint32))
    # under the primary context first, so its address is cached before the new context exists
    assert np.array_equal(_noalloc_digest(lib, torch, state, e.n, e.n_fluid, bonds), want)
    for _ in range(2):  # two contexts in a row, each created, used and destroyed
        with _DriverContext() as ctx:
            d_state = ctx.to_device(state)
            d_bond = ctx.to_device(bonds)
            out = np.full(8, 0xffffffff, np.uint32)
            d_out = ctx.to_device(out)
            rc = lib.sn_digest_device_noalloc(ctypes.c_void_p(d_state), e.n, e.n_fluid, ctypes.c_void_p(d_bond),
                                              ctypes.c_void_p(d_out), None)
            assert rc == 0
            got = ctx.to_host(d_out, out)
            assert np.array_equal(got, want)
    # and back under the primary context, where the cached address still holds
    assert np.array_equal(_noalloc_digest(lib, torch, state, e.n, e.n_fluid, bonds), want)
