"""§23.B jets on the CPU oracle: inert without jets, an acceleration inside
their discs, the first JET_MAX = 8 kept (src/engine.js:4740-4770)."""
from sunaengine_gb300 import scenes

ONE = 65536
JETS = [{'x': 40 * ONE, 'y': 60 * ONE, 'r': 6 * ONE, 'fx': 900, 'fy': -2400},
        {'x': 44 * ONE, 'y': 58 * ONE, 'r': 5 * ONE, 'fx': -300, 'fy': -1800},
        {'x': 20 * ONE, 'y': 64 * ONE, 'r': 3 * ONE, 'fx': 2147483000, 'fy': 0}]


def oracle(sc):
    import oracle as o
    return o.OracleEngine(sc.n + 64, threads=8).load_scene(sc)


def test_jets_push_and_removal_is_inert():
    sc = scenes.make_scene('pool_v1', w=40, h=14)
    plain, jet, off = oracle(sc), oracle(sc), oracle(sc)
    assert jet.set_jets(JETS) == 3
    assert off.set_jets(JETS) == 3 and off.set_jets([]) == 0
    for e in (plain, jet, off):
        e.step(30)
    assert jet.chain_hex() != plain.chain_hex()
    assert off.chain_hex() == plain.chain_hex()


def test_only_eight_jets_are_kept():
    sc = scenes.make_scene('pool_v1', w=20, h=10)
    e = oracle(sc)
    assert e.set_jets(JETS * 4) == 8
