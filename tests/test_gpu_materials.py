"""Composed (interned) material rows and the gravity scale on the GPU against
the oracle: the same host cache drives both engines; every result bit-exact."""
import numpy as np
import pytest

from sunaengine_gb300 import data, materials, scenes
from sunaengine_gb300.engine import Engine
from sunaengine_gb300.materials import MOD

import test_oracle_rigid as tr

pytestmark = pytest.mark.gpu
ONE = 65536


def test_interned_rows_and_gravity_match_the_oracle():
    import oracle as o
    sc = scenes.make_scene('dambreak_v1')
    g = Engine(max_particles=8192, debug=True).load_scene(sc)
    r = o.OracleEngine(8192, threads=16).load_scene(sc)
    ig, ir = materials.Interner(g), materials.Interner(r)
    sand = data.mat_id('SAND')
    recipes = [(0, MOD['V']), (sand, MOD['E']), (0, MOD['Y']), (data.mat_id('OIL'), MOD['T'] | MOD['D']),
               (sand, MOD['M'] | MOD['B']), (data.mat_id('STONE'), MOD['H'])]
    rows = []
    for base, bits in recipes:
        a, b = ig.intern(base, bits), ir.intern(base, bits)
        assert a['rowId'] == b['rowId'] and a['events'] == b['events']
        rows.append(a['rowId'])
    for k, row in enumerate(rows):
        pts = [{'x': (8 + 14 * k + c) * ONE + ONE // 2, 'y': (8 + q) * ONE, 'mat': row, 'temp': 20 * ONE}
               for q in range(4) for c in range(5)]
        for x, it in ((g, ig), (r, ir)):
            x.spawn_fluid(pts, no_weld=False)
            it.note_spawn([row] * len(pts))
    for k in (1, 3, 10):
        g.step(k)
        r.step(k)
        assert g.chain_hex() == r.chain_hex()
    for x in (g, r):
        x.set_gravity_scale(ONE // 3)
    for k in (2, 12):
        g.step(k)
        r.step(k)
        assert g.chain_hex() == r.chain_hex()
    assert np.array_equal(g.read_state(), r.read_state())
    assert np.array_equal(g.debug_counters(), r.debug_counters())


def test_bodies_under_a_scaled_world():
    sc = scenes.rigid_tank()
    import oracle as o
    g = Engine(max_particles=sc.n + 64, debug=True).load_scene(sc)
    r = tr.oracle(sc, threads=16)
    for x in (g, r):
        x.set_gravity_scale(2 * ONE)
        x.make_rigid_body(sc.meta['plank'])
    assert g.read_bodies()[0][16] == r.read_bodies()[0][16] == 2 * 2000 * len(sc.meta['plank'])
    for k in (1, 5, 20):
        g.step(k)
        r.step(k)
        assert g.chain_hex() == r.chain_hex()
    assert np.array_equal(g.read_bodies(), r.read_bodies())
