"""The CPU oracle against the reference's own golden vectors (no GPU needed).

Golden values: the frozen dambreak_v1 chain and checkpoint digests recorded in
the reference's test/extraction_gate.md:62-68 (also test/site_gates.mjs:53-61),
and the frozen LUT hash (src/engine.js:501), carried in
tests/golden/reference_dambreak_v1.json (written from those files by
tests/golden/extract_reference_golden.py).
"""
import json
from pathlib import Path

import numpy as np
import pytest

from sunaengine_gb300 import data, scenes

GOLDEN = json.loads((Path(__file__).parent / 'golden' / 'reference_dambreak_v1.json').read_text())
GOLDEN_CHAIN = GOLDEN['chain']
GOLDEN_CHECKPOINTS = {int(k): v for k, v in GOLDEN['checkpoints'].items()}


def test_table_hash_and_layout():
    w = data.luts()
    assert w.size == 5 * 3202
    assert data.table_hash(w) == data.TABLE_HASH == GOLDEN['table_hash']
    # the s_corr table is all zeros (scorrK = 0, src/tables.js:41)
    assert not w[4 * 3202:].any()


def test_material_rows():
    m = data.mats()
    assert m.shape == (28, 48)
    F = data.mat_field
    water = m[data.mat_id('WATER')]
    assert water[F('grav')] == 1200 and water[F('xsph')] == 6000 and water[F('cond')] == 9000
    assert water[F('freezePt')] == 0 and water[F('boilPt')] == 100 * 65536
    oil = m[data.mat_id('OIL')]
    assert oil[F('grav')] == 900 and oil[F('ignitePt')] == 180 * 65536 and oil[F('fuel0')] == 100 * 65536
    # gammaCur defaults to gammaCoh / 4 (src/engine.js:740-744)
    assert m[data.mat_id('TAR')][F('gammaCur')] == 650 // 4
    # rampInv is baked floor(2^32 / (hi - lo))
    ice = m[data.mat_id('ICE')]
    assert int(ice[F('rampInv')]) == (2 ** 32) // (int(ice[F('rampHi')]) - int(ice[F('rampLo')]))


def test_xorshift_and_dambreak_layout():
    r = scenes.Xorshift32(0)
    assert r.s == 0x2545f491
    sc = scenes.make_scene('dambreak_v1')
    assert (sc.n, sc.nFluid) == (4096, 3600)
    assert (sc.domW, sc.domH) == (128 * 65536, 72 * 65536)
    # boundaryRing(128, 72, 60): 2*128 + 4*60 walls
    assert sc.n - sc.nFluid == 496
    assert tuple(sc.pos[sc.nFluid]) == (32768, 72 * 65536 - 32768)


def test_oracle_golden_chain(oracle_mod):
    e = oracle_mod.OracleEngine(8192, threads=8).load_scene(scenes.make_scene('dambreak_v1'))
    done = 0
    for c, want in GOLDEN_CHECKPOINTS.items():
        e.step(c - done)
        done = c
        assert e.digest() == want, f'checkpoint {c}'
    assert e.chain_hex() == GOLDEN_CHAIN
    assert not e.debug_counters().any()


def test_oracle_overdense_truncates(oracle_mod):
    # overdense_v1 exists to exercise the MAXNBR truncation path (src/engine.js:2503-2523)
    e = oracle_mod.OracleEngine(8192, threads=4).load_scene(scenes.make_scene('overdense_v1'))
    e.step(1)
    assert e.debug_counters()[6] > 0


def test_oracle_permutation_moves_slot_digest_only(oracle_mod):
    sc = scenes.make_scene('pool_v1', w=30, h=10)
    a = oracle_mod.OracleEngine(4096, threads=4).load_scene(sc)
    b = oracle_mod.OracleEngine(4096, threads=4).load_scene(scenes.permute_scene(sc, 0x5151))
    for _ in range(2):
        da, db = a.digest(), b.digest()
        assert da[:32] == db[:32], 'H_set must be permutation invariant'
        assert da[32:] != db[32:], 'H_slot must see the reordering'
        a.step(10)
        b.step(10)


def test_oracle_is_deterministic_across_thread_counts(oracle_mod):
    sc = scenes.make_scene('droplet_v1', mat=scenes.MAT_OIL)
    a = oracle_mod.OracleEngine(4096, threads=1).load_scene(sc)
    b = oracle_mod.OracleEngine(4096, threads=8).load_scene(sc)
    a.step(30)
    b.step(30)
    assert a.chain_hex() == b.chain_hex()


def test_oracle_one_tick_control(oracle_mod):
    sc = scenes.make_scene('pool_v1', w=30, h=10)
    sc2 = sc.copy()
    sc2.pos[0, 0] += 1
    a = oracle_mod.OracleEngine(4096, threads=4).load_scene(sc)
    b = oracle_mod.OracleEngine(4096, threads=4).load_scene(sc2)
    a.step(20)
    b.step(20)
    assert a.digest() != b.digest()


def test_neighbour_cut_changes_no_state(oracle_mod):
    """The oracle's neighbour-list cut (stop a full list's scan when no fluid
    particle carries a seal or congeal flag) leaves every state word, chain
    and neighbour count as the full scan gives them; only the overflow debug
    counter stops counting. The overdense scene overflows its lists."""
    import numpy as np
    sc = scenes.make_scene('overdense_v1')
    a = oracle_mod.OracleEngine(sc.n + 64, threads=4).load_scene(sc)
    b = oracle_mod.OracleEngine(sc.n + 64, threads=4).load_scene(sc).set_nbr_cut(True)
    for _ in range(4):
        a.step(5)
        b.step(5)
        assert a.chain_hex() == b.chain_hex()
        assert np.array_equal(a.read_state(), b.read_state())
        assert np.array_equal(a.read_nbr_counts(), b.read_nbr_counts())
    assert a.debug_counters()[6] > 0 and b.debug_counters()[6] < a.debug_counters()[6]
