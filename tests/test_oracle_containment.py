"""§29 containment on the CPU oracle (build-defined scenes; the reference
ships no frozen containment vectors, so these are behaviour checks of the
restatement plus the invariances it must keep)."""
import numpy as np
import pytest

from sunaengine_gb300 import data, scenes

ONE = 65536


def oracle(sc, mats=None, threads=8):
    import oracle as o
    return o.OracleEngine(sc.n + 64, threads=threads, mats=mats).load_scene(sc)


def inside_box(st, sc):
    w = st[sc.meta['seal']:sc.nFluid]
    return int(((w[:, 0] > 8.5 * ONE) & (w[:, 0] < 40.5 * ONE) & (w[:, 1] > 11.5 * ONE) &
                (w[:, 1] < 34.5 * ONE)).sum()), len(w)


def custom_rubber(**fields):
    m = data.mats().copy()
    r = data.mat_id('RUBBER')
    for k, v in fields.items():
        m[r, data.MAT_FIELDS.index(k)] = v
    return m


def test_closed_box_holds_compressed_water():
    sc = scenes.sealed_box(spacing=0.6)
    o = oracle(sc)
    for _ in range(3):
        o.step(40)
        got, total = inside_box(o.read_state().reshape(-1, 8), sc)
        assert got == total
    d = o.debug_counters()
    assert d[6] > 0                       # crowded rows: the overflow path ran
    assert (d[[0, 1, 2, 5]] == 0).all()


def test_thread_count_invariance_with_containment():
    sc = scenes.sealed_box(spacing=0.55)
    a, b = oracle(sc, threads=1), oracle(sc, threads=8)
    a.step(25)
    b.step(25)
    assert a.chain_hex() == b.chain_hex()


def test_permeable_seal_lets_liquid_through():
    sc = scenes.sealed_box(spacing=0.6)
    o = oracle(sc, mats=custom_rubber(sealMode=1))
    o.step(160)
    got, total = inside_box(o.read_state().reshape(-1, 8), sc)
    assert got < total


def test_finite_burst_pressure_releases_held_particles():
    sc = scenes.sealed_box(spacing=0.5)
    o = oracle(sc, mats=custom_rubber(burstP=30000))
    o.step(40)
    st = o.read_state().reshape(-1, 8)
    fl = st[:sc.meta['seal'], 5].astype(np.uint32)
    burst = (fl & 64) != 0
    assert burst.any() and not (fl[burst] & 4).any()
    held = oracle(sc)
    held.step(40)
    assert not (held.read_state().reshape(-1, 8)[:sc.meta['seal'], 5].astype(np.uint32) & 64).any()


def test_loose_rigid_rows_seal_like_any_seal_row():
    # BEDROCK and STONE are rigid-body rows; outside a body they are ordinary
    # seal matter: BEDROCK (burstP 0) holds the compressed water, STONE
    # (burstP 2.5) bursts under it
    sc = scenes.sealed_box(seal='BEDROCK', spacing=0.6)
    o = oracle(sc)
    o.step(60)
    got, total = inside_box(o.read_state().reshape(-1, 8), sc)
    assert got == total
    sc = scenes.sealed_box(seal='STONE', spacing=0.6)
    o = oracle(sc)
    o.step(60)
    fl = o.read_state().reshape(-1, 8)[:sc.meta['seal'], 5].astype(np.uint32)
    assert (fl & 64).any()
