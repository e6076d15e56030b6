"""Seeded synthetic systems with the shapes of the named benchmark workloads.

All inputs are synthetic (no dataset exists for this path). Starting
configurations are random sequential addition (RSA) without overlap at the
contact distance sigma, because the reference's RandomInserter checks only
container overlap (molecule.h:100-107).
"""
import math

import numpy as np

from .params import (FG_EWALD_DIPOLE_DIPOLE, FG_EWALD_ION_ION, FG_MODEL_DH_LJ, FG_MODEL_EWALD_DIPOLE,
                     FG_MODEL_EWALD_WCA, FG_MODEL_MULTIPOLE_RF, make_params)


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


# ---------------------------------------------------------------- rigid dipolar molecules
def bjerrum_unit(temperature=298.0):
    """pc::lB(1.0): the Bjerrum length at eps_r = 1 with the reference's
    constants (physconst.h:52-64, 91-94), in Angstrom."""
    e, e0, kB = 1.602177e-19, 8.85419e-12, 1.380658e-23
    return e * e / (4 * math.pi * e0 * 1.0 * 1e-10 * kB * temperature)


def molecule_conformation(rng, molsize, radius, min_dist):
    """One rigid molecule: ``molsize`` sites uniform in a ball of ``radius``,
    no two closer than ``min_dist``, centred on their geometric centre."""
    pts = []
    while len(pts) < molsize:
        v = rng.uniform(-radius, radius, 3)
        if v @ v > radius * radius:
            continue
        if all(np.sum((v - q) ** 2) >= min_dist * min_dist for q in pts):
            pts.append(v)
    pts = np.array(pts)
    return pts - pts.mean(axis=0)


def dipolar_molecules(n_mol=1000, seed=1, molsize=20, box=None, sigma=3.5, lj_eps=0.2, mu=1.5, bjerrum=7.1,
                      cutoff=15.0, eps_rf=1e11, mol_radius=4.0, temperature=298.0):
    """Rigid ``molsize``-site molecules: site charges from {-1, 0, +1} with net
    zero per molecule (half the sites drawn, the other half their negatives),
    site LJ sigma, one point dipole |mu| (e*Angstrom) in random orientation on
    site 0. Default box keeps 1000 molecules in a 150 Angstrom cube.

    Returns (params, xyz[N,3], mu_unit[N,3], mu_scalar[N], type_ids[N]);
    types 0, 1, 2 carry q = -1, 0, +1."""
    rng = np.random.default_rng(seed)
    if box is None:
        box = 150.0 * (n_mol / 1000.0) ** (1.0 / 3.0)
    L = float(box)
    types = [dict(q=-1.0, sigma=sigma, eps=lj_eps), dict(q=0.0, sigma=sigma, eps=lj_eps),
             dict(q=1.0, sigma=sigma, eps=lj_eps)]
    eps_r = bjerrum_unit(temperature) / bjerrum
    p = make_params(FG_MODEL_MULTIPOLE_RF, L, bjerrum, types, rf_cutoff=cutoff, rf_eps_rf=eps_rf,
                    rf_eps_r=eps_r)
    # molecule centres at least 2 R + sigma apart: no two sites of different
    # molecules overlap at the start
    centres = scatter_positions(n_mol, L, 2 * mol_radius + sigma, int(rng.integers(1 << 31)))
    n = n_mol * molsize
    xyz = np.empty((n, 3))
    mu_u = np.zeros((n, 3))
    mu_s = np.zeros(n)
    ids = np.empty(n, dtype=np.int32)
    half = molsize // 2
    for m in range(n_mol):
        conf = molecule_conformation(rng, molsize, mol_radius, 2.0)
        r = centres[m] + conf
        r -= L * np.round(r / L)
        xyz[m * molsize:(m + 1) * molsize] = r
        q = rng.integers(-1, 2, half)
        qs = np.concatenate([q, -q, np.zeros(molsize - 2 * half, dtype=q.dtype)])
        rng.shuffle(qs)
        ids[m * molsize:(m + 1) * molsize] = qs + 1
        v = rng.normal(size=3)
        mu_u[m * molsize] = v / np.linalg.norm(v)
        mu_s[m * molsize] = mu
    return p, xyz, mu_u, mu_s, ids


# ---------------------------------------------------------------- point dipoles under Ewald
def dipolar_fluid(n=100, seed=1, box=None, sigma=2.8863, eps_kjmol=1.97, mu=1.652, temperature=315.8,
                  alpha=0.25, cutoff=None, kc=7.0, dp=0.7, n_ions=0, terms=FG_EWALD_ION_ION | FG_EWALD_DIPOLE_DIPOLE,
                  quirk=0, eps_surf=1e11, update_frequency=1000):
    """Lennard-Jones point dipoles with the shape of the reference's Stockmayer
    example (stockmayer.json: 100 dipoles, |mu| 1.652 e A, sigma 2.8863 A,
    eps 1.97 kJ/mol, L 29.6336 A at 100 particles, T 315.8 K, dp 0.7 A,
    tin-foil surroundings), at that density for any n. The Ewald sum is
    alpha 0.25 / A, real-space cutoff L/2 - 0.4 A and a spherical k-space
    cutoff kc (the example's own cutoffK 0 leaves no reciprocal sum).

    With n_ions > 0 the first n_ions particles are ions (charge +1 and -1 in
    turn, no dipole) and the rest neutral dipoles. Type 0 carries +1 and type 1
    -1: every type is charged, so the effective-charge ratio of ewald.h:539
    is 1 (a neutral type makes it 0/0 in the reference); the per-particle
    charges say which particles are ions.

    Returns (params, xyz[n,3], mu_unit[n,3], mu_scalar[n], type_ids[n], charges[n])."""
    rng = np.random.default_rng(seed)
    if box is None:
        box = 29.6336 * (n / 100.0) ** (1.0 / 3.0)
    L = float(box)
    if cutoff is None:
        cutoff = 0.5 * L - 0.4
    bjerrum = bjerrum_unit(temperature)
    eps = eps_kjmol / (8.314462618e-3 * temperature)
    types = [dict(q=1.0, sigma=sigma, eps=eps, dp=dp), dict(q=-1.0, sigma=sigma, eps=eps, dp=dp)]
    p = make_params(FG_MODEL_EWALD_DIPOLE, L, bjerrum, types, ewald_alpha=alpha, ewald_cutoff=cutoff,
                    ewald_cutoff_k=kc, ewald_eps_surf=eps_surf, ewald_update_frequency=update_frequency,
                    ewald_terms=terms, ewald_dipole_quirk=quirk, kT_scale=1.0)
    xyz = scatter_positions(n, L, 0.9 * sigma, int(rng.integers(1 << 31)))
    v = rng.normal(size=(n, 3))
    mu_u = v / np.linalg.norm(v, axis=1, keepdims=True)
    mu_s = np.full(n, float(mu))
    q = np.zeros(n)
    ids = np.zeros(n, dtype=np.int32)
    for i in range(n_ions):
        q[i] = 1.0 if i % 2 == 0 else -1.0
        ids[i] = 0 if i % 2 == 0 else 1
        mu_s[i] = 0.0
    return p, xyz, mu_u, mu_s, ids, q
