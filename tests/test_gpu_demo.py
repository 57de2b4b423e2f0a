"""The demo layer's gates on the GPU engine, and GPU == CPU checker on each flow."""
import pytest

from sunaengine_gb300.engine import Engine

import test_demo_formats as t

pytestmark = pytest.mark.gpu


def gpu_factory(cap):
    return Engine(max_particles=cap)


def test_twins_gpu_and_match_checker():
    g = t._twins(gpu_factory)
    assert g[0] == g[1]
    assert g[0] == t._twins(t.oracle_factory)[0]


def test_record_replay_gpu_and_match_checker():
    live, replay, mutated = t._record_replay(gpu_factory)
    assert replay == live and mutated != live
    assert (live, replay, mutated) == t._record_replay(t.oracle_factory)


def test_keyframe_gpu_and_match_checker():
    ahead, rejoined, state_only = t._keyframe(gpu_factory)
    assert rejoined == ahead and state_only != ahead
    assert (ahead, rejoined, state_only) == t._keyframe(t.oracle_factory)


def test_walls_off_and_on_match_checker():
    import oracle
    from sunaengine_gb300 import scenes
    sc = scenes.make_scene('pool_v1', w=30, h=10)
    g = Engine(max_particles=4096).load_scene(sc)
    r = oracle.OracleEngine(4096, threads=8).load_scene(sc)
    for x in (g, r):
        x.step(5)
        x.set_walls(False)
        x.step(5)
        x.spawn_fluid([{'x': 40 * 65536, 'y': 30 * 65536, 'mat': 0}])
        x.set_walls(True)
        x.step(5)
    assert g.n == r.n and g.chain_hex() == r.chain_hex()
