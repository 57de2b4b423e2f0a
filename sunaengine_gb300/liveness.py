"""Liveness metrics: is a run physically alive, not just reproducible?

A digest only says two engines agree. A frozen lattice, a block drifting at
uniform velocity or a state blown up to saturated words hashes just as
consistently, so the reference pairs its determinism gate with these checks
(src/engine.js:6878-7143, "Liveness (§7.7)"):

* ``compute_liveness`` — ``computeLiveness`` (:6881-7009): kinetic energy
  (total, and about the mean velocity), moved fractions against the initial
  and a recent snapshot, density statistics from the last substep's rho,
  neighbour counts, cell occupancy, bounding box, saturated words, thermal
  totals and a material histogram.
* ``check_liveness`` — ``checkLiveness`` (:7036-7081): the list of violated
  bounds (empty = alive).
* ``DAMBREAK_EXPECT`` (:7093-7096): the relaxed density band a transient dam
  break needs.
* ``zero_state_liveness`` / ``degenerate_state_controls`` (:7099-7143): the
  controls that prove the check is not vacuous; every one must be rejected.

Arithmetic follows the reference: BigInt sums are Python ints, JS number sums
are IEEE doubles accumulated in index order (``np.cumsum`` is sequential, so
its last element is the reference's running sum).
"""
from __future__ import annotations

import math

import numpy as np

ONE = 65536
RHO0 = 1048576
MAXNBR = 48
PARTICLE_WORDS = 8
I32_MAX, I32_MIN = 2147483647, -2147483648


def _seq_sum(a: np.ndarray) -> float:
    """A JS running sum of doubles in index order."""
    return float(np.cumsum(np.asarray(a, np.float64))[-1]) if len(a) else 0.0


def compute_liveness(state, n: int, n_fluid: int, dom_w: int, dom_h: int, rho=None, nbr_count=None,
                     cell_start=None, initial_pos=None, recent_pos=None) -> dict:
    """computeLiveness (src/engine.js:6881-7009).

    ``state``: n*8 words (slot order). ``rho``: the last substep's rho per slot
    (the reference reads Derived word 10); ``nbr_count``: neighbour counts per
    slot; ``cell_start``: cell-start words (occupancy = consecutive
    differences); ``initial_pos`` / ``recent_pos``: 2 words per slot.
    """
    st = np.asarray(state, np.int64).reshape(-1, PARTICLE_WORDS)[:n]
    x, y, vx, vy = st[:, 0], st[:, 1], st[:, 2], st[:, 3]
    f = slice(0, n_fluid)
    fx, fy, fvx, fvy = x[f], y[f], vx[f], vy[f]
    ke = int(np.sum(fvx * fvx + fvy * fvy, dtype=object)) if n_fluid else 0
    vx_sum, vy_sum = int(fvx.sum()), int(fvy.sum())
    moved = 0
    if initial_pos is not None:
        # a fluid slot past the loaded positions (a spawn that outgrew the
        # load) has no initial position and counts as moved, as the
        # reference's typed-array read of undefined compares unequal
        ip = np.asarray(initial_pos, np.int64).reshape(-1, 2)[:n_fluid]
        k = ip.shape[0]
        moved = int(np.count_nonzero((fx[:k] != ip[:, 0]) | (fy[:k] != ip[:, 1]))) + (n_fluid - k)
    recent_moved = 0
    if recent_pos is not None:
        rp = np.asarray(recent_pos, np.int64).reshape(-1, 2)[:n_fluid]
        recent_moved = int(np.count_nonzero((fx != rp[:, 0]) | (fy != rp[:, 1])))
    outside = int(np.count_nonzero((fx < 0) | (fy < 0) | (fx > dom_w) | (fy > dom_h)))
    first4 = st[:, :4]
    saturated = int(np.count_nonzero((first4 == I32_MAX) | (first4 == I32_MIN)))
    if n:
        bbox = [int(x.min()), int(y.min()), int(x.max()), int(y.max())]
    else:
        bbox = [math.inf, math.inf, -math.inf, -math.inf]

    vx_bar = vx_sum / n_fluid if n_fluid else 0.0
    vy_bar = vy_sum / n_fluid if n_fluid else 0.0
    dx = fvx.astype(np.float64) - vx_bar
    dy = fvy.astype(np.float64) - vy_bar
    ke_about_mean = _seq_sum(dx * dx + dy * dy)
    internal_ke = ke_about_mean / n_fluid if n_fluid else 0.0
    internal_vrms = math.sqrt(internal_ke) / ONE

    mean_density = rho_max = density_std = 0.0
    if rho is not None and len(rho) >= n_fluid and n_fluid:
        r = np.asarray(rho, np.int64)[:n_fluid].astype(np.float64) / RHO0
        mean_density = _seq_sum(r) / n_fluid
        rho_max = max(0.0, float(r.max()))
        density_std = math.sqrt(_seq_sum((r - mean_density) * (r - mean_density)) / n_fluid)

    max_nbr, nbr_sum = 0, 0
    if nbr_count is not None and n_fluid:
        c = np.asarray(nbr_count, np.int64)[:n_fluid]
        max_nbr, nbr_sum = int(c.max()), int(c.sum())

    max_cell = 0
    if cell_start is not None and len(cell_start) > 1:
        cs = np.asarray(cell_start, np.int64)
        occ = cs[1:] - cs[:-1]
        occ = occ[occ < 0x7fffffff]
        max_cell = int(max(0, occ.max())) if len(occ) else 0

    temp = st[f, 6]
    temp_sum = int(temp.sum())
    mats, counts = np.unique(st[f, 4] & 0xffffffff, return_counts=True)
    burning = int(np.count_nonzero(st[f, 5] & 1))
    return {
        'particleCount': n,
        'fluidCount': n_fluid,
        'tempSum': str(temp_sum),
        'tempMean': temp_sum / n_fluid if n_fluid else 0,
        'tempMin': int(temp.min()) if n_fluid else 0,
        'tempMax': int(temp.max()) if n_fluid else 0,
        'burningCount': burning,
        'matHistogram': {int(m): int(k) for m, k in zip(mats, counts)},
        'kineticEnergy': str(ke),
        'kineticEnergyPerParticle': ke / n_fluid if n_fluid else 0,
        'internalKePerParticle': internal_ke,
        'internalVrms': internal_vrms,
        'meanVelocity': [vx_bar, vy_bar],
        'meanDensity': mean_density,
        'maxDensity': rho_max,
        'densityStd': density_std,
        'movedFraction': moved / n_fluid if n_fluid else 0,
        'recentMovedFraction': (recent_moved / n_fluid if n_fluid else 0) if recent_pos is not None else None,
        'outsideDomain': outside,
        'maxNbr': max_nbr,
        'meanNbr': nbr_sum / n_fluid if n_fluid else 0,
        'bbox': bbox,
        'nonFinite': saturated,
        'maxCellOccupancy': max_cell,
        'restDensity': 1.0,
    }


def check_liveness(L: dict, expect: dict | None = None) -> list[str]:
    """checkLiveness (src/engine.js:7036-7081): the violated bounds; empty = alive."""
    e = expect or {}
    min_moved = e.get('minMovedFraction', 0.5)
    min_recent = e.get('minRecentMovedFraction', 0.5)
    dens_lo, dens_hi = e.get('densityRange', (0.98, 1.03))
    max_std = e.get('maxDensityStd', 0.035)
    min_ke = e.get('minKePerParticle', 1)
    min_internal = e.get('minInternalKePerParticle', 1000)
    vrms_lo, vrms_hi = e.get('internalVrmsRange', (1e-4, 0.5))
    max_outside = e.get('maxOutside', 0)
    nbr_lo, nbr_hi = e.get('nbrRange', (4, MAXNBR))
    min_span = e.get('minBboxSpan', ONE)
    v = []
    if L['particleCount'] <= 0:
        v.append(f"particleCount {L['particleCount']} <= 0")
    if L['movedFraction'] < min_moved:
        v.append(f"movedFraction {L['movedFraction']:.4f} < {min_moved} (particles are not moving)")
    if L['recentMovedFraction'] is not None and L['recentMovedFraction'] < min_recent:
        v.append(f"recentMovedFraction {L['recentMovedFraction']:.4f} < {min_recent} "
                 f"(state is FROZEN: it moved once and then stopped)")
    if not (dens_lo <= L['meanDensity'] <= dens_hi):
        v.append(f"meanDensity {L['meanDensity']:.4f} outside [{dens_lo}, {dens_hi}]")
    if L['densityStd'] > max_std:
        v.append(f"densityStd {L['densityStd']:.4f} > {max_std}")
    if L['kineticEnergyPerParticle'] < min_ke:
        v.append(f"kineticEnergyPerParticle {L['kineticEnergyPerParticle']} < {min_ke} (state is frozen)")
    if L['internalKePerParticle'] < min_internal:
        v.append(f"internalKePerParticle {L['internalKePerParticle']:.1f} < {min_internal} (no internal "
                 f"dynamics: a rigid body drifting, or a frozen lattice)")
    if not (vrms_lo <= L['internalVrms'] <= vrms_hi):
        v.append(f"internalVrms {L['internalVrms']:.3e} wu/substep outside [{vrms_lo}, {vrms_hi}]")
    if L['outsideDomain'] > max_outside:
        v.append(f"outsideDomain {L['outsideDomain']} > {max_outside}")
    if L['maxNbr'] < nbr_lo:
        v.append(f"maxNbr {L['maxNbr']} < {nbr_lo} (no neighbours found: grid is dead)")
    if L['maxNbr'] > nbr_hi:
        v.append(f"maxNbr {L['maxNbr']} > {nbr_hi} (neighbour list overflowed)")
    if L['nonFinite'] > 0:
        v.append(f"{L['nonFinite']} saturated i32 words in state (I32_MAX/I32_MIN)")
    span_x, span_y = L['bbox'][2] - L['bbox'][0], L['bbox'][3] - L['bbox'][1]
    if not (span_x >= min_span and span_y >= min_span):
        v.append(f"bbox span ({span_x}, {span_y}) collapsed below {min_span} ticks")
    return v


# The relaxation a transient, flowing scene needs against the settled-pool
# defaults (src/engine.js:7093-7096).
DAMBREAK_EXPECT = {'densityRange': (0.98, 1.04), 'maxDensityStd': 0.055}


def zero_state_liveness(n: int = 4096, n_fluid: int = 3600):
    """zeroStateLiveness (src/engine.js:7099-7111): an all-zero state must fail."""
    L = compute_liveness(np.zeros(n * PARTICLE_WORDS, np.int32), n, n_fluid, 128 * ONE, 72 * ONE,
                         rho=np.zeros(n, np.int32), nbr_count=np.zeros(n, np.uint32),
                         initial_pos=np.zeros(n * 2, np.int32), recent_pos=np.zeros(n * 2, np.int32))
    return L, check_liveness(L)


def degenerate_state_controls(n: int = 1024) -> dict:
    """degenerateStateControls (src/engine.js:7113-7143): four states that must
    all be rejected — a block drifting uniformly, a frozen crystal with a
    one-tick jitter, a frozen solid, and every particle stacked at one point."""

    def mk(fill):
        o = {'state': np.zeros(n * PARTICLE_WORDS, np.int64), 'rho': np.zeros(n, np.int64),
             'nbr': np.zeros(n, np.int64), 'initial': np.zeros(n * 2, np.int64), 'recent': np.zeros(n * 2, np.int64)}
        fill(o)
        return compute_liveness(o['state'], n, n, 128 * ONE, 128 * ONE, rho=o['rho'], nbr_count=o['nbr'],
                                initial_pos=o['initial'], recent_pos=o['recent'])

    def lattice(jitter, vx, vy):
        def fill(o):
            i = np.arange(n)
            gx, gy = i % 32, i // 32
            st = o['state'].reshape(-1, PARTICLE_WORDS)
            o['initial'][0::2], o['initial'][1::2] = gx * ONE, gy * ONE
            st[:, 0] = (gx + 30) * ONE + jitter
            st[:, 1] = (gy + 30) * ONE + jitter
            o['recent'][0::2], o['recent'][1::2] = st[:, 0] - jitter, st[:, 1] - jitter
            st[:, 2], st[:, 3] = vx, vy
            o['rho'][:] = RHO0
            o['nbr'][:] = 20
        return fill

    def stacked(o):
        st = o['state'].reshape(-1, PARTICLE_WORDS)
        st[:, 0] = st[:, 1] = 64 * ONE
        st[:, 2] = 8
        o['rho'][:] = RHO0
        o['nbr'][:] = 20

    cases = {
        'rigid block drifting uniformly': mk(lattice(1, 1000, 0)),
        'frozen crystal, 1-tick jitter': mk(lattice(1, 1, 0)),
        'frozen solid (no motion at all)': mk(lattice(0, 0, 0)),
        'all stacked at one point': mk(stacked),
    }
    return {k: (L, check_liveness(L)) for k, L in cases.items()}
