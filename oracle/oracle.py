"""ctypes front end of the FP64 oracle (oracle/fg_oracle.cpp) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker or the timed CPU baseline. The product library never
imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libfg_oracle.so")
SRCS = [os.path.join(HERE, f) for f in ("fg_oracle.cpp", "fg_oracle_mol.cpp", "fg_oracle_dip.cpp", "or_common.h")]


def build(force=False):
    """Compile the oracle with the host g++ (plain C++17, no GPU)."""
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(f) for f in SRCS):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-o", LIB] +
                          [f for f in SRCS if f.endswith(".cpp")])
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, i32, i64, dp, u32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_uint32
        L.or_create.restype = vp
        L.or_create.argtypes = [vp]
        L.or_destroy.argtypes = [vp]
        L.or_num_kvectors.argtypes = [vp]
        L.or_set_state.argtypes = [vp, i32, dp, dp, dp]
        L.or_get_positions.argtypes = [vp, dp]
        L.or_get_qk.argtypes = [vp, dp, dp, dp]
        L.or_pair_energy.restype = ctypes.c_double
        L.or_pair_energy.argtypes = [vp, i32, i32]
        L.or_trial_du.restype = ctypes.c_double
        L.or_trial_du.argtypes = [vp, i32, dp, dp]
        L.or_commit.restype = ctypes.c_double
        L.or_commit.argtypes = [vp, i32]
        L.or_total_energy.argtypes = [vp, dp]
        L.or_boundary.argtypes = [vp, dp]
        L.or_draw_translation_stream.argtypes = [u32, i32, dp, i64, dp, dp, dp]
        L.or_uniforms.argtypes = [u32, i64, dp]
        L.or_pt_streams.argtypes = [u32, i32, dp, i64, i32, dp, dp, dp, dp, dp]
        L.or_mc_run.restype = ctypes.c_double
        L.or_mc_run.argtypes = [vp, u32, i64, dp, dp, dp, dp]
        L.or_philox.argtypes = [dp, dp, dp]
        L.or_philox_stream.argtypes = [u32, u32, i64, i64, ctypes.c_int32, dp, dp, dp, dp, dp, dp]
        L.or_set_kT.argtypes = [vp, ctypes.c_double]
        L.or_mc_run_stream.restype = ctypes.c_double
        L.or_mc_run_stream.argtypes = [vp, i64, dp, dp, dp, dp, dp]
        L.or_mol_create.restype = vp
        L.or_mol_create.argtypes = [vp, i32, i32]
        L.or_mol_destroy.argtypes = [vp]
        L.or_mol_set_state.argtypes = [vp, dp, dp, dp, dp, dp]
        L.or_mol_get_state.argtypes = [vp, dp, dp, dp]
        L.or_mol_pair.restype = ctypes.c_double
        L.or_mol_pair.argtypes = [vp, i32, i32]
        L.or_mol_trial_du_explicit.restype = ctypes.c_double
        L.or_mol_trial_du_explicit.argtypes = [vp, i32, dp, dp]
        L.or_mol_commit.argtypes = [vp, i32]
        L.or_mol_total_energy.argtypes = [vp, dp]
        L.or_mol_draw_stream.argtypes = [u32, i32, ctypes.c_double, ctypes.c_double, i32, i64, dp, dp, dp, dp, dp, dp]
        L.or_mol_run_stream.restype = ctypes.c_double
        L.or_mol_run_stream.argtypes = [vp, i64, dp, dp, dp, dp, dp, dp, i32, i32, dp, dp]
        L.or_dip_create.restype = vp
        L.or_dip_create.argtypes = [vp]
        L.or_dip_destroy.argtypes = [vp]
        L.or_dip_num_kvectors.argtypes = [vp]
        L.or_dip_set_state.argtypes = [vp, i32, dp, dp, dp, dp, dp]
        L.or_dip_get_state.argtypes = [vp, dp, dp]
        L.or_dip_pair.restype = ctypes.c_double
        L.or_dip_pair.argtypes = [vp, i32, i32, i32]
        L.or_dip_trial_du.restype = ctypes.c_double
        L.or_dip_trial_du.argtypes = [vp, i32, dp, dp]
        L.or_dip_commit.restype = ctypes.c_double
        L.or_dip_commit.argtypes = [vp, i32]
        L.or_dip_total_energy.argtypes = [vp, dp]
        L.or_dip_run_stream.restype = ctypes.c_double
        L.or_dip_run_stream.argtypes = [vp, i64, dp, dp, dp, dp, dp, dp, dp, dp]
        L.or_dip_draw_stream.argtypes = [u32, i32, i64, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         dp, dp, dp, dp, dp, dp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class OracleSystem:
    """FP64 restatement of one reference system (Space + energy + Ewald state)."""

    def __init__(self, params, xyz, q, ids):
        self._p = params
        self.h = lib().or_create(ctypes.byref(params))
        if not self.h:
            raise RuntimeError("oracle create failed")
        self.n = len(xyz)
        self.set_state(xyz, q, ids)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_destroy(self.h)
            self.h = None

    def set_state(self, xyz, q, ids):
        self._xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self._q = np.ascontiguousarray(q, dtype=np.float64)
        self._ids = np.ascontiguousarray(ids, dtype=np.int32)
        self.n = len(self._xyz)
        lib().or_set_state(self.h, self.n, _ptr(self._xyz), _ptr(self._q), _ptr(self._ids))

    @property
    def num_kvectors(self):
        return lib().or_num_kvectors(self.h)

    def positions(self):
        out = np.empty((self.n, 3), dtype=np.float64)
        lib().or_get_positions(self.h, _ptr(out))
        return out

    def qk(self):
        K = self.num_kvectors
        q = np.empty(2 * K)
        kv = np.empty(3 * K)
        ak = np.empty(K)
        lib().or_get_qk(self.h, _ptr(q), _ptr(kv), _ptr(ak))
        return q[0::2] + 1j * q[1::2], kv.reshape(K, 3), ak

    def pair_energy(self, i, j):
        return lib().or_pair_energy(self.h, i, j)

    def trial_du(self, idx, new_xyz):
        idx = np.ascontiguousarray(np.atleast_1d(idx), dtype=np.int32)
        new_xyz = np.ascontiguousarray(np.reshape(new_xyz, (-1, 3)), dtype=np.float64)
        return lib().or_trial_du(self.h, len(idx), _ptr(idx), _ptr(new_xyz))

    def commit(self, accepted):
        return lib().or_commit(self.h, 1 if accepted else 0)

    def total_energy(self):
        """{pairs, reciprocal, self, surface, total} (kT)."""
        c = np.empty(5)
        lib().or_total_energy(self.h, _ptr(c))
        return dict(pairs=c[0], reciprocal=c[1], self=c[2], surface=c[3], total=c[4])

    def boundary(self, xyz):
        a = np.ascontiguousarray(xyz, dtype=np.float64).copy()
        lib().or_boundary(self.h, _ptr(a))
        return a

    def mc_run(self, seed, n_trials, log=True):
        """Metropolis run with the reference's RNG stream; returns dict."""
        n = int(n_trials)
        idx = np.empty(n, np.int32) if log else None
        txyz = np.empty((n, 3)) if log else None
        du = np.empty(n) if log else None
        acc = np.empty(n, np.uint8) if log else None
        utot = lib().or_mc_run(self.h, seed, n, _ptr(idx), _ptr(txyz), _ptr(du), _ptr(acc))
        return dict(utot=utot, idx=idx, trial_xyz=txyz, du=du, acc=acc)


def _mc_run_stream(self, idx, disp, u):
    """Metropolis run from an explicit stream; returns dict(utot, du, acc)."""
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    disp = np.ascontiguousarray(disp, dtype=np.float64).reshape(-1, 3)
    u = np.ascontiguousarray(u, dtype=np.float64)
    n = len(idx)
    du = np.empty(n)
    acc = np.empty(n, np.uint8)
    utot = lib().or_mc_run_stream(self.h, n, _ptr(idx), _ptr(disp), _ptr(u), _ptr(du), _ptr(acc))
    return dict(utot=utot, du=du, acc=acc)


OracleSystem.mc_run_stream = _mc_run_stream
OracleSystem.set_kT = lambda self, kT: lib().or_set_kT(self.h, float(kT))


def replay_chain(args):
    """FP64 replay of one AtomicTranslation chain (a process-pool worker:
    start the pool with the spawn method). args = (params as bytes, xyz, q,
    ids, idx, disp, u[, kT]); returns (du, acc) per trial."""
    from beofaunus_gb300.params import FgParams
    pb, xyz, q, ids, idx, disp, u = args[:7]
    o = OracleSystem(FgParams.from_buffer_copy(pb), xyz, q, ids)
    if len(args) > 7 and args[7] != 1.0:
        o.set_kT(args[7])
    r = o.mc_run_stream(idx, disp, u)
    return r["du"], r["acc"]


def compare_chain(du_dev, acc_dev, du_ref, acc_ref, u, tol):
    """Trial-by-trial comparison of a device chain with the oracle's on the
    same stream. The chains are compared up to and including the first trial
    whose decision differs; a differing decision is legitimate only if the
    threshold lies within tol of the oracle's dU (then the chains part from
    there on). Returns dict(max_err, rms_err, compared, diverged_at,
    divergence_in_band, decisions_identical)."""
    du_dev = np.asarray(du_dev, dtype=np.float64)
    du_ref = np.asarray(du_ref, dtype=np.float64)
    n = len(du_ref)
    mism = np.nonzero(np.asarray(acc_dev) != np.asarray(acc_ref))[0]
    upto, at, in_band = n, None, True
    if len(mism):
        at = int(mism[0])
        in_band = bool(abs(du_ref[at] + np.log(u[at])) < tol)
        upto = at + 1
    err = np.abs(du_dev[:upto] - du_ref[:upto])
    finite = bool(np.all(np.isfinite(du_dev[:upto])))
    return dict(max_err=float(err.max()) if finite and upto else float("inf"),
                rms_err=float(np.sqrt(np.mean(err ** 2))) if finite and upto else float("inf"),
                compared=int(upto), diverged_at=at, divergence_in_band=in_band,
                decisions_identical=at is None)


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.empty(4, dtype=np.uint32)
    lib().or_philox(_ptr(c), _ptr(k), _ptr(out))
    return out


def philox_stream(seed, stream, first, n, types, type_dp, box):
    """The device trial-stream definition regenerated on the host."""
    types = np.ascontiguousarray(types, dtype=np.int32)
    tdp = np.ascontiguousarray(type_dp, dtype=np.float64)
    b = np.ascontiguousarray(box, dtype=np.float64)
    idx = np.empty(n, np.int32)
    disp = np.empty((n, 3))
    u = np.empty(n)
    lib().or_philox_stream(seed, stream, first, n, len(types), _ptr(types), _ptr(tdp), _ptr(b), _ptr(idx),
                           _ptr(disp), _ptr(u))
    return idx, disp, u


def translation_stream(seed, dp_per_particle, n_trials):
    """The reference's per-trial randoms for AtomicTranslation on one atomic
    group: (index[n], displacement[n,3], u_metropolis[n])."""
    dpp = np.ascontiguousarray(dp_per_particle, dtype=np.float64)
    n = int(n_trials)
    idx = np.empty(n, np.int32)
    disp = np.empty((n, 3))
    u = np.empty(n)
    lib().or_draw_translation_stream(seed, len(dpp), _ptr(dpp), n, _ptr(idx), _ptr(disp), _ptr(u))
    return idx, disp, u


def pt_streams(seed, dp_per_particle, trials_per_round, rounds):
    """The reference's parallel-tempering random streams (the same on every
    rank): per round the AtomicTranslation trials (idx, disp, u), the
    exchange's Metropolis uniform and findPartner's uniform."""
    dpp = np.ascontiguousarray(dp_per_particle, dtype=np.float64)
    n = int(trials_per_round) * int(rounds)
    idx = np.empty(n, np.int32)
    disp = np.empty((n, 3))
    u = np.empty(n)
    ua = np.empty(rounds)
    ud = np.empty(rounds)
    lib().or_pt_streams(seed, len(dpp), _ptr(dpp), int(trials_per_round), int(rounds), _ptr(idx), _ptr(disp),
                        _ptr(u), _ptr(ua), _ptr(ud))
    T = int(trials_per_round)
    return [(idx[r * T:(r + 1) * T], disp[r * T:(r + 1) * T], u[r * T:(r + 1) * T]) for r in range(rounds)], ua, ud


def pt_exchange(energies, temps, perm, u_direction, u_accept):
    """One exchange attempt of Move::ParallelTempering (move.h:6621-6771)
    restated over a ladder held in one process: rung i holds configuration
    perm[i] with energy energies[perm[i]] (kT at unit temperature). findPartner:
    dr = +1 if u_direction > 0.5 else -1; even rungs pair with i + dr, odd ones
    with i - dr. Each pair tests dU = [U_i(x_p) - U_i(x_i)] + [U_p(x_i) - U_p(x_p)],
    U_i = E / T_i, against the shared uniform: exchanged iff not u > exp(-dU).
    Returns the new perm and, per rung, whether it exchanged."""
    n = len(perm)
    perm = list(perm)
    dr = 1 if u_direction > 0.5 else -1
    swapped = [0] * n
    for i in range(n):
        p = i + dr if i % 2 == 0 else i - dr
        if p <= i or p >= n:
            continue
        ea, eb = energies[perm[i]], energies[perm[p]]
        du = (eb - ea) / temps[i] + (ea - eb) / temps[p]
        if not (u_accept > np.exp(-du)):
            perm[i], perm[p] = perm[p], perm[i]
            swapped[i] = swapped[p] = 1
    return perm, swapped


class OracleMol:
    """FP64 restatement of a reference system of rigid dipolar molecules
    (NonbondedVector + CoulombGalore/LJ/IonDipole/DipoleDipoleGalore RF,
    TranslateRotate)."""

    def __init__(self, params, xyz, mu, mus, type_ids, group_size, cms=None):
        n = len(type_ids)
        self.n, self.gs, self.m = n, group_size, n // group_size
        self.h = lib().or_mol_create(ctypes.byref(params), n, group_size)
        if not self.h:
            raise ValueError("bad molecule system")
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        mu = np.ascontiguousarray(mu, dtype=np.float64).reshape(-1, 3)
        mus = np.ascontiguousarray(mus, dtype=np.float64)
        ids = np.ascontiguousarray(type_ids, dtype=np.int32)
        c = None if cms is None else np.ascontiguousarray(cms, dtype=np.float64).reshape(-1, 3)
        lib().or_mol_set_state(self.h, _ptr(xyz), _ptr(mu), _ptr(mus), _ptr(ids), _ptr(c))

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_mol_destroy(self.h)
            self.h = None

    def state(self):
        xyz = np.empty((self.n, 3))
        mu = np.empty((self.n, 3))
        cm = np.empty((self.m, 3))
        lib().or_mol_get_state(self.h, _ptr(xyz), _ptr(mu), _ptr(cm))
        return xyz, mu, cm

    def pair(self, i, j):
        return lib().or_mol_pair(self.h, i, j)

    def trial_du(self, g, xyz, mu=None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        mu = None if mu is None else np.ascontiguousarray(mu, dtype=np.float64).reshape(-1, 3)
        return lib().or_mol_trial_du_explicit(self.h, g, _ptr(xyz), _ptr(mu))

    def commit(self, accepted):
        lib().or_mol_commit(self.h, 1 if accepted else 0)

    def total_energy(self):
        """(intermolecular, intramolecular, total) as systemEnergy sums them."""
        c = np.empty(3)
        lib().or_mol_total_energy(self.h, _ptr(c))
        return c

    def run_stream(self, st, rotate=True, translate=True):
        n = len(st["group"])
        du = np.empty(n)
        acc = np.empty(n, np.uint8)
        g = np.ascontiguousarray(st["group"], dtype=np.int32)
        ax = np.ascontiguousarray(st["axis"], dtype=np.float64)
        ce = np.ascontiguousarray(st["center"], dtype=np.int32)
        an = np.ascontiguousarray(st["angle"], dtype=np.float64)
        tr = np.ascontiguousarray(st["trans"], dtype=np.float64)
        u = np.ascontiguousarray(st["u"], dtype=np.float64)
        usum = lib().or_mol_run_stream(self.h, n, _ptr(g), _ptr(ax), _ptr(ce), _ptr(an), _ptr(tr), _ptr(u),
                                       1 if rotate else 0, 1 if translate else 0, _ptr(du), _ptr(acc))
        return dict(usum=usum, du=du, acc=acc)


def mol_stream(seed, n_groups, dp, dprot, center_rotation, n):
    """The reference's global-slump draws for n TranslateRotate trials."""
    g = np.empty(n, np.int32)
    ax = np.empty((n, 3))
    ce = np.empty(n, np.int32)
    an = np.empty(n)
    tr = np.empty((n, 3))
    u = np.empty(n)
    lib().or_mol_draw_stream(seed, n_groups, dp, dprot, 1 if center_rotation else 0, n, _ptr(g), _ptr(ax),
                             _ptr(ce), _ptr(an), _ptr(tr), _ptr(u))
    return dict(group=g, axis=ax, center=ce, angle=an, trans=tr, u=u)


# ---------------------------------------------------------------- analysis
def atom_rdf_counts(xyz, types, box, t1, t2, dr, n_bins):
    """AtomRDF::update (analysis.h:2116-2134) on one configuration, FP64:
    every pair i < j whose types are {t1, t2} counts once at the
    minimum-image distance (Cuboid::sqdist, geometry.h:507-515: |a - b| per
    axis, minus L where above L/2), in bin int(r / dr + 0.5) (Table2D::round,
    auxiliary.h:831). Returns (counts of bins 0 .. n_bins-1, pairs at any
    distance)."""
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    tp = np.asarray(types)
    L = np.asarray(box, dtype=np.float64)
    n = len(x)
    hist = np.zeros(n_bins, np.int64)
    total = 0
    for i in range(n - 1):
        j = np.arange(i + 1, n)
        sel = ((tp[i] == t1) & (tp[j] == t2)) | ((tp[i] == t2) & (tp[j] == t1))
        j = j[sel]
        if len(j) == 0:
            continue
        d = np.abs(x[i] - x[j])
        d = np.where(d > 0.5 * L, d - L, d)
        r = np.sqrt((d * d).sum(axis=1))
        b = (r / dr + 0.5).astype(np.int64)
        total += len(j)
        np.add.at(hist, b[b < n_bins], 1)
    return hist, total


def rdf_normalize(hist, total, volume, dr):
    """PairFunctionBase::normalize (analysis.cpp:190-205) for dim = 3:
    g(r_b) = N(r_b) / sum N * <V> / (4 pi r_b^2 dr), r_b = b dr (bin 0 has no
    volume element: inf or nan there, as in the reference)."""
    r = np.arange(len(hist)) * dr
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.asarray(hist, dtype=np.float64) / total * volume / (4.0 * np.pi * r * r * dr)


# ---------------------------------------------------------------- volume move
def slump_uniforms(seed, n):
    """The reference's global slump() draws (slump.h:62-95) from seed."""
    u = np.empty(int(n))
    lib().or_uniforms(seed, int(n), _ptr(u))
    return u


# particles per cubic Angstrom in one mM (physconst.h:161-173, Nav = 6.022137e23)
MILLIMOLAR = 1.0e-3 * 6.022137e23 / 1e27


def reciprocal_unscaled(o_new, xyz_old, q, eff):
    """The trial reciprocal energy the reference forms for a volume move:
    the structure factor of the positions before scaling with the new box's
    k-vectors and weights (NonbondedEwald::setGeometry rebuilding Q(k) from
    spc->p, ewald.h:731-756; getReciprocalEnergy, ewald.h:298-311)."""
    K = o_new.num_kvectors
    qk, kv, ak = np.empty(2 * K), np.empty(3 * K), np.empty(K)
    lib().or_get_qk(o_new.h, _ptr(qk), _ptr(kv), _ptr(ak))
    kv = kv.reshape(K, 3)
    qe = np.asarray(q) * np.asarray(eff)
    Q = (qe[None, :] * np.exp(1j * (kv @ np.asarray(xyz_old).T))).sum(axis=1)
    return float(np.sum(ak * np.abs(Q) ** 2))


def volume_move(params, xyz, q, ids, half, dp, pressure, u, kT=1.0, reference_quirk=False):
    """Move::Isobaric (move.h:5529-5624) with ExternalPressure
    (energy.h:1817-1890) on one atomic group, FP64: V' = exp(ln V + half dp),
    positions scaled by (V'/V)^(1/3) about the origin (Cuboid::scale,
    geometry.cpp:325-332), dU = E(V') - E(V) + P (V' - V) - (N + 1) ln(V'/V)
    with E the system energy and P in particles per cubic Angstrom;
    Metropolis as move.h:567-573. Returns (dU, accepted, params, xyz) with
    the new box and positions when accepted."""
    from beofaunus_gb300.params import FgParams
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    L = np.array(params.box[:3], dtype=np.float64)
    V = float(np.prod(L))
    Vn = float(np.exp(np.log(V) + half * dp))
    f = float(np.cbrt(Vn / V))
    e0 = OracleSystem(params, x, q, ids).total_energy()["total"]
    pn = FgParams.from_buffer_copy(bytes(params))
    for a in range(3):
        pn.box[a] = params.box[a] * f
    xn = x * f
    o1 = OracleSystem(pn, xn, q, ids)
    en = o1.total_energy()
    e1 = en["total"]
    n = len(x)
    du = e1 - e0 + pressure * (Vn - V) - (n + 1) * np.log(Vn / V)
    if reference_quirk and params.model == 1:
        # the reciprocal energy as returned carries the prefactor 2 pi lB / V';
        # the raw sum is rescaled by the same factor
        # effective charges (ewald.h:532-549): sinh(kappa R) / (kappa R), R = sigma / 2
        kap = 1.0 / params.ewald_debye_length
        eff = []
        for t in ids:
            kr = kap * 0.5 * params.type_sigma[t]
            eff.append(np.sinh(kr) / kr if abs(kr) > 1e-9 else 1.0)
        raw = reciprocal_unscaled(o1, x, q, eff)
        prefactor = 2.0 * np.pi / Vn * pn.bjerrum
        du += raw * prefactor - en["reciprocal"]
    acc = not (u > np.exp(-du / kT))
    return du, acc, (pn if acc else params), (xn if acc else x)


# ---------------------------------------------------------------- point dipoles
class OracleDip:
    """FP64 restatement of NonbondedEwald<Tspace, LennardJonesLB, ...> on point
    charges and point dipoles with AtomicRotation / AtomicTranslation
    (oracle/fg_oracle_dip.cpp)."""

    def __init__(self, params, xyz, mu, mus, ids, q=None):
        self.h = lib().or_dip_create(ctypes.byref(params))
        if not self.h:
            raise ValueError("bad dipole system")
        self.n = len(ids)
        self.set_state(xyz, mu, mus, ids, q)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_dip_destroy(self.h)
            self.h = None

    def set_state(self, xyz, mu, mus, ids, q=None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        mu = np.ascontiguousarray(mu, dtype=np.float64).reshape(-1, 3)
        mus = np.ascontiguousarray(mus, dtype=np.float64)
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        q = None if q is None else np.ascontiguousarray(q, dtype=np.float64)
        self.n = len(ids)
        lib().or_dip_set_state(self.h, self.n, _ptr(xyz), _ptr(mu), _ptr(mus), _ptr(q), _ptr(ids))

    @property
    def num_kvectors(self):
        return lib().or_dip_num_kvectors(self.h)

    def state(self):
        xyz = np.empty((self.n, 3))
        mu = np.empty((self.n, 3))
        lib().or_dip_get_state(self.h, _ptr(xyz), _ptr(mu))
        return xyz, mu

    def pair(self, i, j, real_only=False):
        return lib().or_dip_pair(self.h, i, j, 1 if real_only else 0)

    def trial_du(self, i, xyz, mu=None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        mu = None if mu is None else np.ascontiguousarray(mu, dtype=np.float64)
        return lib().or_dip_trial_du(self.h, int(i), _ptr(xyz), _ptr(mu))

    def commit(self, accepted):
        return lib().or_dip_commit(self.h, 1 if accepted else 0)

    def total_energy(self):
        """{real-space Ewald pairs, LJ pairs, reciprocal, self, surface, total}"""
        c = np.empty(6)
        lib().or_dip_total_energy(self.h, _ptr(c))
        return c

    def run_stream(self, st):
        n = len(st["idx"])
        du = np.empty(n)
        acc = np.empty(n, np.uint8)
        arr = {k: np.ascontiguousarray(st[k], dtype=np.int32 if k in ("kind", "idx") else np.float64)
               for k in ("kind", "idx", "axis", "angle", "disp", "u")}
        s = lib().or_dip_run_stream(self.h, n, _ptr(arr["kind"]), _ptr(arr["idx"]), _ptr(arr["axis"]),
                                    _ptr(arr["angle"]), _ptr(arr["disp"]), _ptr(arr["u"]), _ptr(du), _ptr(acc))
        return dict(usum=s, du=du, acc=acc)


def dip_stream(seed, n_particles, n, p_rotate, dp, dprot, kinds=None):
    """Draws of n AtomicRotation / AtomicTranslation trials (see
    or_dip_draw_stream): dict(kind, idx, axis, angle, disp, u). With kinds
    given (1 rotation, 2 translation per trial) p_rotate is not used."""
    kind = np.empty(n, np.int32) if kinds is None else np.array(kinds, dtype=np.int32)
    if kinds is not None:
        p_rotate = -1.0
    idx = np.empty(n, np.int32)
    axis = np.empty((n, 3))
    angle = np.empty(n)
    disp = np.empty((n, 3))
    u = np.empty(n)
    lib().or_dip_draw_stream(seed, n_particles, n, p_rotate, dp, dprot, _ptr(kind), _ptr(idx), _ptr(axis),
                             _ptr(angle), _ptr(disp), _ptr(u))
    return dict(kind=kind, idx=idx, axis=axis, angle=angle, disp=disp, u=u)
