"""Seeded synthetic systems with the shapes of the named benchmark workloads.

All inputs are synthetic (no dataset exists for this path). Starting
configurations are random sequential addition (RSA) without overlap at the
contact distance sigma, because the reference's RandomInserter checks only
container overlap (molecule.h:100-107).
"""
import math

import numpy as np

from .params import FG_MODEL_DH_LJ, FG_MODEL_EWALD_WCA, make_params


def rsa_positions(n, box, min_dist, seed):
    """n points uniform in the periodic box [-L/2, L/2)^3, no two closer
    than ``min_dist`` (minimum image). Cell grid keeps it O(n)."""
    rng = np.random.default_rng(seed)
    L = np.asarray(box if hasattr(box, "__len__") else (box, box, box), dtype=np.float64)
    ncell = np.maximum((L // min_dist).astype(int), 1)
    csize = L / ncell
    grid = {}
    out = np.empty((n, 3), dtype=np.float64)
    md2 = min_dist * min_dist
    placed = 0
    tries = 0
    while placed < n:
        tries += 1
        if tries > 200 * n + 10000:
            raise RuntimeError("RSA failed: density too high")
        r = (rng.random(3) - 0.5) * L
        c = tuple(((r + 0.5 * L) // csize).astype(int) % ncell)
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    cc = ((c[0] + dx) % ncell[0], (c[1] + dy) % ncell[1], (c[2] + dz) % ncell[2])
                    for j in grid.get(cc, ()):
                        d = r - out[j]
                        d -= L * np.round(d / L)
                        if d @ d < md2:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            out[placed] = r
            grid.setdefault(c, []).append(placed)
            placed += 1
    return out


def scatter_positions(n, box, min_dist, seed, max_rounds=1000):
    """n points uniform in [-L/2, L/2)^3 with no two closer than ``min_dist``
    (minimum image): draw all points at once, then redraw one point of every
    overlapping pair until none is left. Vectorised, so large systems start in
    well under a second; at the low packing fractions used here it converges
    in a handful of rounds. Unlike rsa_positions this is not sequential
    addition, but the result has the same property the workloads need: a
    seeded, uniform, overlap-free start."""
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(seed)
    L = np.asarray(box if hasattr(box, "__len__") else (box, box, box), dtype=np.float64)
    pts = rng.random((n, 3)) * L
    pairs = cKDTree(pts, boxsize=L).query_pairs(min_dist, output_type="ndarray")
    redo = np.unique(pairs.max(axis=1)) if len(pairs) else np.empty(0, dtype=np.int64)
    for _ in range(max_rounds):
        if len(redo) == 0:
            return pts - 0.5 * L
        pts[redo] = rng.random((len(redo), 3)) * L
        # only redrawn points can overlap now; each one counts itself once
        cnt = cKDTree(pts, boxsize=L).query_ball_point(pts[redo], min_dist, return_length=True)
        redo = redo[cnt > 1]
    raise RuntimeError("scatter_positions did not converge: density too high")


def start_positions(n, box, min_dist, seed, start):
    """Start configuration: 'rsa', 'scatter', or given positions (n, 3)."""
    if isinstance(start, np.ndarray):
        if start.shape != (n, 3):
            raise ValueError("given start positions must have shape (n, 3)")
        return np.array(start, dtype=np.float64)
    if start == "rsa":
        return rsa_positions(n, box, min_dist, seed)
    if start == "scatter":
        return scatter_positions(n, box, min_dist, seed)
    raise ValueError("start must be 'rsa' or 'scatter'")


def salt_types(sigma, eps, dp):
    """A 1:1 salt: type 0 has q=+1, type 1 has q=-1."""
    return [dict(q=1.0, sigma=sigma, eps=eps, dp=dp), dict(q=-1.0, sigma=sigma, eps=eps, dp=dp)]


def salt_ids(n):
    """Cations first, then anions (n even)."""
    ids = np.zeros(n, dtype=np.int32)
    ids[n // 2:] = 1
    return ids


def rpm_ewald(n, box, kc, seed, update_frequency=1000, bjerrum=7.1, alpha=0.2, cutoff=20.0,
              wca_eps=0.1, sigma=4.0, dp=2.0, eps_surf=1e11, use_cell_list=0, start="rsa"):
    """Restricted primitive model with Ewald (alpha, real cutoff, |n|<=kc)
    plus WCA repulsion. Returns (params, xyz[n,3], charges[n], type_ids[n])."""
    types = salt_types(sigma, wca_eps, dp)
    p = make_params(FG_MODEL_EWALD_WCA, box, bjerrum, types, ewald_alpha=alpha, ewald_cutoff=cutoff,
                    ewald_cutoff_k=float(kc), ewald_debye_length=1e30, ewald_eps_surf=eps_surf,
                    ewald_spherical_sum=1, ewald_update_frequency=update_frequency,
                    use_cell_list=use_cell_list)
    xyz = start_positions(n, box, sigma, seed, start)
    ids = salt_ids(n)
    q = np.where(ids == 0, 1.0, -1.0)
    return p, xyz, q, ids


def rpm800(seed=1, **kw):
    """800 ions, L=60, |n|^2<=49: the plain CPU-runnable Ewald workload."""
    return rpm_ewald(800, 60.0, 7, seed, **kw)


def rpm16k(seed=1, **kw):
    """16384 ions, L=163 (same density), |n|^2<=100, cell list for rc=20."""
    kw.setdefault("use_cell_list", 1)
    return rpm_ewald(16384, 163.0, 10, seed, **kw)


def dh_lj_salt(n, seed, density=0.002, debye_length=10.0, bjerrum=7.1, sigma=4.0, lj_eps=0.2,
               dp=2.0, kT_scale=1.0, start="rsa"):
    """Debye-Hueckel + Lennard-Jones salt at number density ``density``."""
    box = (n / density) ** (1.0 / 3.0)
    types = salt_types(sigma, lj_eps, dp)
    p = make_params(FG_MODEL_DH_LJ, box, bjerrum, types, dh_debye_length=debye_length,
                    kT_scale=kT_scale)
    xyz = start_positions(n, box, sigma, seed, start)
    ids = salt_ids(n)
    q = np.where(ids == 0, 1.0, -1.0)
    return p, xyz, q, ids


def pt_ladder_sizes(n_replicas=64, n_min=500, n_max=4000, seed=7):
    """Per-replica particle counts, log-uniform in [n_min, n_max], even."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_replicas))
    return (2 * np.round(n / 2)).astype(int)


def pt_temperatures(n_replicas=64, t_min=0.8, t_max=2.0):
    """Geometric temperature ladder (reduced units)."""
    return t_min * (t_max / t_min) ** (np.arange(n_replicas) / max(n_replicas - 1, 1))
