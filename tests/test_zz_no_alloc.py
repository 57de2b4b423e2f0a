"""The no-allocation digest entry point against the engine's own digest.

sn_digest_device_noalloc serves callers that cannot allocate device memory
when they need a digest (inside a stream capture, in latency-bound loops, or
under a host that owns all device memory). Its scratch is a fixed array in the
library's device image. This test calls it through the C ABI on buffers the
test owns and requires the 8 digest words to equal sn_digest's bit for bit,
on two calls in a row over two different states, and checks that an
over-limit size is refused. It is kept in its own file so that it runs last
and runs the same alone or after the other tests.
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


def test_noalloc_digest_refuses_oversize():
    lib = _native.load()
    one = np.zeros(8, np.int32)
    out = np.zeros(8, np.uint32)
    # refused on the host before any launch, so host pointers are never dereferenced
    rc = lib.sn_digest_device_noalloc(one.ctypes.data_as(ctypes.c_void_p), (1 << 24) + 1, 0, None,
                                      out.ctypes.data_as(ctypes.c_void_p), None)
    assert rc == -2  # SN_E_CAPACITY
