"""Build-defined regression cases for the paths the reference ships no frozen
values for (OIL, thermal transitions, containment, rigid bodies, jets,
composed materials, the 3D solver). Each case runs on any engine with the
Engine surface (the GPU engine or the oracle) and returns the hex chain (2D:
H_set || H_slot folded every substep; 3D: the same chain plus the page's FNV
digest). make_oracle_vectors.py records the oracle's answers in
oracle_vectors.json; the tests replay them on the oracle (CPU) and on the GPU.
"""
import numpy as np

from sunaengine_gb300 import data, materials, scenes, tables3d

ONE = 65536


def _mat(name):
    return data.mat_id(name)


def _thermal_mix():
    sc = scenes.make_scene('pool_v1', w=40, h=12, mat=_mat('OIL'))
    nf = sc.nFluid
    mat = sc.matId.copy()
    temp = np.full(sc.n, scenes.AMBIENT, np.int32)
    fuel = np.zeros(sc.n, np.int32)
    fuel[:nf] = scenes.deg(100)
    for i in range(nf):
        x, y = sc.pos[i]
        if x < 18 * ONE:
            mat[i], temp[i], fuel[i] = _mat('WATER'), scenes.deg(130 if i % 3 == 0 else 97), 0
        elif x < 22 * ONE:
            mat[i], temp[i], fuel[i] = _mat('STEAM'), scenes.deg(50), 0
        elif 30 * ONE <= x < 36 * ONE and y < 64 * ONE:
            mat[i], temp[i], fuel[i] = _mat('FIRE'), scenes.deg(900), 100000 * (1 + i % 4)
    sc.matId, sc.temp, sc.fuel = mat.astype(np.uint32), temp, fuel
    return sc


def oil_pool(new2d, new3d):
    e = new2d(scenes.make_scene('pool_v1', w=30, h=10, mat=_mat('OIL')))
    e.step(50)
    return e.chain_hex()


def thermal_mix(new2d, new3d):
    e = new2d(_thermal_mix())
    e.step(60)
    return e.chain_hex()


def sealed_box(new2d, new3d):
    e = new2d(scenes.sealed_box(spacing=0.6))
    e.step(40)
    return e.chain_hex()


def rigid_tank(new2d, new3d):
    sc = scenes.rigid_tank()
    e = new2d(sc)
    e.make_rigid_body(sc.meta['plank'])
    cx, cy = sc.meta['wheel_centre']
    e.make_axis_body(sc.meta['wheel'], cx + 2 * ONE, cy)
    e.step(60)
    return e.chain_hex()


def jets(new2d, new3d):
    e = new2d(scenes.make_scene('dambreak_v1'))
    e.set_jets([{'x': 30 * ONE, 'y': 60 * ONE, 'r': 6 * ONE, 'fx': 900, 'fy': -2600},
                {'x': 90 * ONE, 'y': 50 * ONE, 'r': 4 * ONE, 'fx': -700, 'fy': 0}])
    e.step(40)
    return e.chain_hex()


def composed(new2d, new3d):
    e = new2d(scenes.make_scene('dambreak_v1'))
    it = materials.Interner(e)
    rows = [it.intern(0, materials.MOD['V'])['rowId'], it.intern(_mat('SAND'), materials.MOD['E'])['rowId']]
    for k, row in enumerate(rows):
        pts = [{'x': (70 + 10 * k + c) * ONE, 'y': (8 + r) * ONE, 'mat': row} for r in range(4) for c in range(6)]
        e.spawn_fluid(pts, no_weld=False)
    e.step(30)
    return e.chain_hex()


def pool_3d(new2d, new3d):
    e = new3d(tables3d.initial_state(16000, 'pool'), 300)
    e.step(20)
    return e.chain_hex() + ':' + e.fnv_hex()


CASES = {f.__name__: f for f in (oil_pool, thermal_mix, sealed_box, rigid_tank, jets, composed, pool_3d)}
