"""§29 containment on the GPU against the oracle, substep by substep."""
import numpy as np
import pytest

from sunaengine_gb300 import scenes
from sunaengine_gb300.engine import Engine

import test_oracle_containment as t

pytestmark = pytest.mark.gpu

CASES = {
    'closed_held': dict(sc=dict(spacing=0.6)),
    'open_held': dict(sc=dict(spacing=0.6, closed=False)),
    'membrane_welded': dict(sc=dict(spacing=0.8, membrane=True)),
    'burst': dict(sc=dict(spacing=0.5), mats=dict(burstP=30000)),
    'permeable': dict(sc=dict(spacing=0.6), mats=dict(sealMode=1)),
    'photo_seal': dict(sc=dict(spacing=0.6, seal='PHOTO')),
    'stone_seal': dict(sc=dict(spacing=0.6, seal='STONE')),
    'bedrock_seal': dict(sc=dict(spacing=0.6, seal='BEDROCK')),
}


@pytest.mark.parametrize('case', sorted(CASES))
def test_containment_matches_oracle(case):
    spec = CASES[case]
    sc = scenes.sealed_box(**spec['sc'])
    mats = t.custom_rubber(**spec['mats']) if 'mats' in spec else None
    g = Engine(max_particles=sc.n + 64, debug=True, mats=mats).load_scene(sc)
    r = t.oracle(sc, mats=mats, threads=16)
    for k in (1, 3, 6, 10, 20):
        g.step(k)
        r.step(k)
        assert g.chain_hex() == r.chain_hex(), f'{case}: diverged by substep {r.substep_count}'
    assert np.array_equal(g.read_state(), r.read_state())
    assert np.array_equal(g.debug_counters(), r.debug_counters())
    g.check_errors()


@pytest.mark.parametrize('lanes', [1, 4])
def test_containment_lanes_and_release_build(lanes):
    sc = scenes.sealed_box(spacing=0.55)
    g = Engine(max_particles=sc.n + 64, lanes=lanes).load_scene(sc)
    r = t.oracle(sc, threads=16)
    g.step(30)
    r.step(30)
    assert g.chain_hex() == r.chain_hex()
