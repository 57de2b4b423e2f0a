"""Record the oracle's chain for the benchmark workloads at their full lengths.

The workloads (sizes and inputs as the benchmark builds them):

* ``dambreak_64x64``: 64 x 64 WATER lattice at 1.25 wu in a walled box, no
  input, 1000 substeps;
* ``two_fluid_1024``: the 1,048,576-particle WATER/OIL scene with seeded
  jitter and temperatures, 1000 substeps;
* ``dam3d_64cubed``: the 262,144-particle 3D dam break with its 4096 seeded
  lattice-neighbour bonds, 4 iterations, 500 substeps;
* ``construction_site``: the 74,384-particle construction site (24 bays of a
  METAL plank made a free rigid body, a WOOD disc made an axis body and a
  held STONE rail, over a WATER pool), its 48 bodies made in the order the
  benchmark makes them, 500 substeps;
* ``batch_256``: the 256 seeded scenes of 1 k-64 k particles with their stir
  schedules, 1000 substeps; a sample of scenes spanning the size range (every
  ``--stride``-th scene by size, plus the smallest and largest), each stepped
  on its own oracle engine with the same impulses.

For each 2D/3D scene the file holds the chain (H_set || H_slot of every
substep folded in order) after EVERY substep, so a run of any length up to
the stated one can be checked at its last substep, and the digest every 50
substeps. For the batch, each sampled scene's chain every 100 substeps.

The chain after substep k pins every digest up to k: a GPU run whose chain
equals the recorded one at its last substep matched the oracle on every
substep before it.

    python tests/golden/make_config_vectors.py dambreak_64x64 two_fluid_1024 construction_site
    python tests/golden/make_config_vectors.py batch_256 --stride 4 --procs 8

Outputs go to tests/golden/config_vectors/<workload>.json. Each run takes
the oracle's time at full size: seconds (dam break), about an hour on 8 host
cores (the 1 M scene and the batch sample), minutes (3D).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

OUT = HERE / 'config_vectors'
DIGEST_EVERY = 50
BATCH_EVERY = 100


def _scene2d(name):
    from sunaengine_gb300 import scenes
    if name == 'dambreak_64x64':
        return scenes.lattice_dambreak(), 1000
    if name == 'two_fluid_1024':
        return scenes.large_two_fluid(side=1024), 1000
    raise KeyError(name)


def record_2d(name: str, threads: int):
    import oracle
    sc, total = _scene2d(name)
    # the neighbour-list cut changes no state word, list or flag (only the
    # overflow debug counter); without it the crowded corner cell these scenes
    # build (up to 10^5 particles) makes each substep O(occupancy^2)
    e = oracle.OracleEngine(sc.n + 64, threads=threads).load_scene(sc).set_nbr_cut(True)
    chain, digest = [], {}
    t0 = time.time()
    for k in range(1, total + 1):
        e.step(1)
        chain.append(e.chain_hex())
        if k % DIGEST_EVERY == 0:
            digest[str(k)] = e.digest()
        if k % 50 == 0:
            print(f'{name}: {k}/{total} substeps, {time.time() - t0:.0f} s', flush=True)
    return {'workload': name, 'particles': int(sc.n), 'fluid_particles': int(sc.nFluid), 'iters': 4,
            'substeps': total, 'chain': chain, 'digest': digest}


def record_construction(threads: int, total: int = 500):
    import oracle
    from sunaengine_gb300 import scenes
    sc = scenes.construction_site()
    # no neighbour-list cut: the held rail is seal-class, so flags can still change
    e = oracle.OracleEngine(sc.n, threads=threads).load_scene(sc)
    for pl, wh, pv in zip(sc.meta['planks'], sc.meta['wheels'], sc.meta['wheel_pivots']):
        e.make_rigid_body(pl)
        e.make_axis_body(wh, *pv)
    chain, digest = [], {}
    t0 = time.time()
    for k in range(1, total + 1):
        e.step(1)
        chain.append(e.chain_hex())
        if k % DIGEST_EVERY == 0:
            digest[str(k)] = e.digest()
        if k % 50 == 0:
            print(f'construction_site: {k}/{total} substeps, {time.time() - t0:.0f} s', flush=True)
    return {'workload': 'construction_site', 'particles': int(sc.n), 'fluid_particles': int(sc.nFluid),
            'bodies': int(e.body_count), 'iters': 4, 'substeps': total, 'chain': chain, 'digest': digest}


def record_3d(name: str, threads: int):
    import oracle
    from sunaengine_gb300 import tables3d
    if name != 'dam3d_64cubed':
        raise KeyError(name)
    sc = tables3d.dam3d_large()
    total = 500
    o = oracle.Oracle3D(sc.n, iters=4, threads=threads).load_scene(sc)
    bonds = tables3d.dam3d_bonds(sc)
    o.write_bonds(tables3d.bond_rows(sc, bonds), tables3d.DAM3D_BOND_K, tables3d.DAM3D_BOND_BRK)
    chain, digest = [], {}
    t0 = time.time()
    for k in range(1, total + 1):
        o.step(1)
        chain.append(o.chain_hex())
        if k % DIGEST_EVERY == 0:
            digest[str(k)] = o.digest()
        if k % 50 == 0:
            print(f'{name}: {k}/{total} substeps, {time.time() - t0:.0f} s', flush=True)
    return {'workload': name, 'particles': int(sc.n), 'bonds': int(len(bonds)), 'iters': 4, 'substeps': total,
            'chain': chain, 'digest': digest, 'fnv': o.fnv_hex()}


def _batch_one(args):
    sid, total = args
    import oracle
    from sunaengine_gb300 import scenes
    scs, sched = scenes.batch_scenes(count=256, seed=0xba7c4, substeps=total)
    sc, ev = scs[sid], sched[sid]
    e = oracle.OracleEngine(sc.n + 8, threads=1).load_scene(sc).set_nbr_cut(True)
    at = {}
    for (s, cx, cy, r, ix, iy) in ev:
        at.setdefault(s, []).append((cx, cy, r, ix, iy))
    chain = {}
    for s in range(total):
        for (cx, cy, r, ix, iy) in at.get(s, ()):
            e.impulse(cx, cy, r, ix, iy)
        e.step(1)
        if (s + 1) % BATCH_EVERY == 0:
            chain[str(s + 1)] = e.chain_hex()
    return sid, {'particles': int(sc.n), 'fluid_particles': int(sc.nFluid), 'events': len(ev), 'chain': chain}


def record_batch(stride: int, procs: int, total: int = 1000):
    from sunaengine_gb300 import scenes
    scs, _ = scenes.batch_scenes(count=256, seed=0xba7c4, substeps=total)
    by_size = sorted(range(len(scs)), key=lambda i: scs[i].n)
    pick = sorted({by_size[0], by_size[-1]} | set(by_size[::stride]))
    path = OUT / 'batch_256.json'
    done = json.loads(path.read_text())['scenes'] if path.exists() else {}
    todo = [i for i in pick if str(i) not in done]
    # biggest first, so the pool's tail is short
    todo.sort(key=lambda i: -scs[i].n)
    ctx = mp.get_context('spawn')
    t0 = time.time()
    with ctx.Pool(procs) as pool:
        for sid, rec in pool.imap_unordered(_batch_one, [(i, total) for i in todo]):
            done[str(sid)] = rec
            _write('batch_256', {'workload': 'batch_256', 'seed': 0xba7c4, 'scenes_total': len(scs),
                                 'iters': 4, 'substeps': total, 'every': BATCH_EVERY,
                                 'scenes': dict(sorted(done.items(), key=lambda kv: int(kv[0])))})
            print(f'batch: scene {sid} (n={rec["particles"]}) done, {len(done)}/{len(pick)} '
                  f'recorded, {time.time() - t0:.0f} s', flush=True)


def _write(name, obj):
    OUT.mkdir(exist_ok=True)
    tmp = OUT / f'.{name}.json.tmp'
    tmp.write_text(json.dumps(obj, separators=(',', ':')) + '\n')
    os.replace(tmp, OUT / f'{name}.json')


if __name__ == '__main__':
    ap = argparse.ArgumentParser()
    ap.add_argument('workloads', nargs='+')
    ap.add_argument('--threads', type=int, default=os.cpu_count() or 1)
    ap.add_argument('--stride', type=int, default=4)
    ap.add_argument('--procs', type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()
    for w in a.workloads:
        if w == 'batch_256':
            record_batch(a.stride, a.procs)
        elif w == 'dam3d_64cubed':
            _write(w, record_3d(w, a.threads))
        elif w == 'construction_site':
            _write(w, record_construction(a.threads))
        else:
            _write(w, record_2d(w, a.threads))
