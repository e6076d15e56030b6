"""ctypes front end of libfaunus_gb300.so (include/faunus_gb300.h).

Mirrors the reference's energy/move interface for the Metropolis path:
``System.trial_du`` + ``System.commit`` are Energybase::updateChange /
Energy::energyChange / Energybase::update as Movebase::move calls them
(move.h:515-555); ``System.sweep`` runs that whole loop on the device.
Raises if the compiled library is missing: there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

from . import build as _build
from .params import FgParams

_lib = None


class FgError(RuntimeError):
    pass


class SweepStats(ctypes.Structure):
    _fields_ = [("trials", ctypes.c_int64), ("accepted", ctypes.c_int64), ("rebuilds", ctypes.c_int64),
                ("energy_change", ctypes.c_double), ("device_ms", ctypes.c_double),
                ("sweep_kernel_ms", ctypes.c_double), ("sweep_launches", ctypes.c_int32),
                ("error_flags", ctypes.c_int32), ("kernel_launches", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def library_path():
    return _build.LIB


def lib(build_if_missing=True):
    """Load the in-tree library (building it first if allowed)."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise FgError("libfaunus_gb300.so not built: run __graft_entry__.build()")
            _build.build()
        L = ctypes.CDLL(path)
        vp, i32, i64, u32, dp = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32, ctypes.c_void_p
        sig = {
            "fg_version": ([], ctypes.c_int),
            "fg_last_error": ([], ctypes.c_char_p),
            "fg_create": ([vp, i32, ctypes.POINTER(vp)], ctypes.c_int),
            "fg_destroy": ([vp], ctypes.c_int),
            "fg_set_state": ([vp, dp, dp, dp], ctypes.c_int),
            "fg_get_state": ([vp, dp], ctypes.c_int),
            "fg_trial_du": ([vp, i32, dp, dp, dp], ctypes.c_int),
            "fg_commit": ([vp, i32, dp], ctypes.c_int),
            "fg_total_energy": ([vp, dp], ctypes.c_int),
            "fg_num_kvectors": ([vp], ctypes.c_int),
            "fg_get_qk": ([vp, dp], ctypes.c_int),
            "fg_rebuild_qk": ([vp, dp], ctypes.c_int),
            "fg_draw_translation_stream": ([vp, u32, i64, dp, dp, dp], ctypes.c_int),
            "fg_sweep": ([vp, i64, dp, dp, dp, dp, dp, dp], ctypes.c_int),
            "fg_stream_upload": ([vp, i64, dp, dp, dp], ctypes.c_int),
            "fg_stream_philox": ([vp, i64, u32, u32], ctypes.c_int),
            "fg_stream_get": ([vp, i64, i64, dp, dp, dp], ctypes.c_int),
            "fg_stream_run": ([vp, dp], ctypes.c_int),
            "fg_synchronize": ([vp], ctypes.c_int),
            "fg_set_threads": ([vp, i32], ctypes.c_int),
            "fg_get_threads": ([vp], ctypes.c_int),
            "fg_set_cluster": ([vp, i32], ctypes.c_int),
            "fg_get_cluster": ([vp, dp, dp], ctypes.c_int),
            "fg_philox4x32_10": ([dp, dp, dp], None),
            "fg_set_rebuild_policy": ([vp, i32], ctypes.c_int),
            "fg_running_energy": ([vp, dp], ctypes.c_int),
            "fg_device_bytes": ([vp], ctypes.c_int64),
            "fg_batch_create": ([dp, i32, ctypes.POINTER(vp)], ctypes.c_int),
            "fg_batch_destroy": ([vp], ctypes.c_int),
            "fg_batch_set_threads": ([vp, i32], ctypes.c_int),
            "fg_batch_stream_philox": ([vp, dp, u32, dp], ctypes.c_int),
            "fg_batch_run": ([vp, dp, dp], ctypes.c_int),
            "fg_batch_stream_upload": ([vp, i32, i64, dp, dp, dp], ctypes.c_int),
            "fg_batch_set_log": ([vp, i32, i32], ctypes.c_int),
            "fg_batch_set_rebuild_mode": ([vp, i32], ctypes.c_int),
            "fg_log_get": ([vp, i64, i64, dp, dp], ctypes.c_int),
            "fg_pt_setup": ([vp, dp, u32], ctypes.c_int),
            "fg_pt_run": ([vp, i32, i32, dp], ctypes.c_int),
            "fg_pt_get": ([vp, dp, dp, dp, dp], ctypes.c_int),
            "fg_pt_swap": ([vp, ctypes.c_double, ctypes.c_double, dp, dp], ctypes.c_int),
            "fg_server_create": ([i64, i32, i64, ctypes.POINTER(vp)], ctypes.c_int),
            "fg_server_destroy": ([vp], ctypes.c_int),
            "fg_server_submit": ([vp, vp, i32, dp, dp, dp, u32, i64, dp], ctypes.c_int),
            "fg_server_step": ([vp, dp, dp, dp], ctypes.c_int),
            "fg_server_poll": ([vp, i64, dp, dp, dp, dp, dp], ctypes.c_int),
            "fg_server_release": ([vp, i64], ctypes.c_int),
            "fg_server_cancel": ([vp, i64], ctypes.c_int),
            "fg_server_bytes_in_use": ([vp], ctypes.c_int64),
            "fg_snapshot_bytes": ([vp], ctypes.c_int64),
            "fg_snapshot": ([vp, dp, i64], ctypes.c_int),
            "fg_restore": ([vp, dp, i64], ctypes.c_int),
            "fg_snapshot_info": ([dp, i64, dp, dp, dp, dp, dp, dp, dp], ctypes.c_int),
            "fg_server_snapshot_bytes": ([vp, i64], ctypes.c_int64),
            "fg_server_snapshot": ([vp, i64, dp, i64], ctypes.c_int),
            "fg_server_resume": ([vp, dp, i64, dp], ctypes.c_int),
            "fg_mol_create": ([vp, i32, i32, ctypes.POINTER(vp)], ctypes.c_int),
            "fg_mol_destroy": ([vp], ctypes.c_int),
            "fg_mol_set_state": ([vp, dp, dp, dp, dp, dp], ctypes.c_int),
            "fg_mol_get_state": ([vp, dp, dp, dp], ctypes.c_int),
            "fg_mol_set_cluster": ([vp, i32], ctypes.c_int),
            "fg_mol_get_cluster": ([vp, dp, dp], ctypes.c_int),
            "fg_mol_trial_du": ([vp, i32, dp, dp, dp, dp], ctypes.c_int),
            "fg_mol_commit": ([vp, i32], ctypes.c_int),
            "fg_mol_draw_stream": ([u32, i32, i64, ctypes.c_double, ctypes.c_double, i32, dp, dp, dp, dp, dp, dp],
                                   ctypes.c_int),
            "fg_mol_sweep": ([vp, i64, dp, dp, dp, dp, dp, dp, i32, i32, dp, dp, dp], ctypes.c_int),
            "fg_mol_total_energy": ([vp, dp], ctypes.c_int),
            "fg_mol_stream_upload": ([vp, i64, dp, dp, dp, dp, dp, dp, i32, i32], ctypes.c_int),
            "fg_mol_run_many": ([dp, i32, dp, dp], ctypes.c_int),
            "fg_mol_running_energy": ([vp, dp], ctypes.c_int),
            "fg_mol_device_bytes": ([vp], ctypes.c_int64),
            "fg_autotune": ([vp, i64, dp], ctypes.c_int),
            "fg_total_energy_fp64": ([vp, dp], ctypes.c_int),
            "fg_volume_move": ([vp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, i32, dp, dp],
                               ctypes.c_int),
            "fg_get_box": ([vp, dp], ctypes.c_int),
            "fg_slump_uniforms": ([u32, i64, dp], ctypes.c_int),
            "fg_rdf_sample": ([vp, i32, i32, ctypes.c_double, i32, dp, dp], ctypes.c_int),
            "fg_state_read": ([ctypes.c_char_p, i32, i32, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, i32, dp, dp, dp],
                              ctypes.c_int),
            "fg_state_write": ([ctypes.c_char_p, i32, dp, i32, dp, dp, dp, dp, dp, dp, dp, dp, i32, dp, dp, u32],
                               ctypes.c_int),
            "fg_batch_autotune": ([vp, i64, dp], ctypes.c_int),
            "fg_mol_autotune": ([vp, i64, dp], ctypes.c_int),
            "fg_tune_reset": ([], ctypes.c_int),
            "fg_dip_create": ([vp, i32, ctypes.POINTER(vp)], ctypes.c_int),
            "fg_dip_destroy": ([vp], ctypes.c_int),
            "fg_dip_num_kvectors": ([vp], ctypes.c_int),
            "fg_dip_set_state": ([vp, dp, dp, dp, dp, dp], ctypes.c_int),
            "fg_dip_get_state": ([vp, dp, dp], ctypes.c_int),
            "fg_dip_set_threads": ([vp, i32], ctypes.c_int),
            "fg_dip_trial_du": ([vp, i32, dp, dp, dp], ctypes.c_int),
            "fg_dip_commit": ([vp, i32, dp], ctypes.c_int),
            "fg_dip_sweep": ([vp, i64, dp, dp, dp, dp, dp, dp, dp, dp, dp], ctypes.c_int),
            "fg_dip_stream_upload": ([vp, i64, dp, dp, dp, dp, dp, dp], ctypes.c_int),
            "fg_dip_run_many": ([dp, i32, dp, dp], ctypes.c_int),
            "fg_dip_draw_stream": ([u32, i32, i64, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp, dp, dp, dp,
                                    dp, dp], ctypes.c_int),
            "fg_dip_total_energy": ([vp, dp], ctypes.c_int),
            "fg_dip_running_energy": ([vp, dp], ctypes.c_int),
            "fg_dip_device_bytes": ([vp], ctypes.c_int64),
            "fg_dip_autotune": ([dp, i32, i64, dp], ctypes.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class TuneReport(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("chosen", ctypes.c_int32), ("value", ctypes.c_int32 * 8),
                ("us_per_trial", ctypes.c_double * 8)]

    def as_dict(self):
        c = [(int(self.value[i]), float(self.us_per_trial[i])) for i in range(self.n)]
        return {"candidates": c, "chosen": c[self.chosen][0] if self.n else None}


def _tune(fn, h, n_trials):
    r = TuneReport()
    _check(fn(h, int(n_trials), ctypes.byref(r)))
    return r.as_dict()


def read_state(path, kind=0, n_max=1 << 22, g_max=1 << 20):
    """Read a reference state file (fg_state_read): dict of box, xyz, charge,
    radius, mw, ids, hydrophobic (and mu_unit, mu_scalar for kind 1),
    groups [G, 4] and group_cm [G, 3]. ids are the file's atom ids (the
    reference's first atom type is id 1)."""
    n = np.zeros(1, np.int32)
    ng = np.zeros(1, np.int32)
    box = np.zeros(3)
    # first pass: counts only
    _check(lib().fg_state_read(str(path).encode(), kind, n_max, _p(box), _p(n), None, None, None, None, None, None,
                               None, None, 0, _p(ng), None, None))
    N, G = int(n[0]), int(ng[0])
    out = dict(box=box, xyz=np.zeros((N, 3)), charge=np.zeros(N), radius=np.zeros(N), mw=np.zeros(N),
               ids=np.zeros(N, np.int32), hydrophobic=np.zeros(N, np.int32), groups=np.zeros((G, 4), np.int32),
               group_cm=np.zeros((G, 3)))
    mu = np.zeros((N, 3)) if kind == 1 else None
    mus = np.zeros(N) if kind == 1 else None
    _check(lib().fg_state_read(str(path).encode(), kind, N, _p(box), _p(n), _p(out["xyz"]), _p(out["charge"]),
                               _p(out["radius"]), _p(out["mw"]), _p(out["ids"]), _p(out["hydrophobic"]), _p(mu),
                               _p(mus), G, _p(ng), _p(out["groups"]), _p(out["group_cm"])))
    if kind == 1:
        out.update(mu_unit=mu, mu_scalar=mus)
    return out


def write_state(path, box, xyz, charge, radius, mw, ids, hydrophobic=None, mu_unit=None, mu_scalar=None,
                groups=None, group_cm=None, rng_seed=5489, kind=None):
    """Write a reference state file (fg_state_write); kind 1 (dipole
    records) when mu_unit is given."""
    f64 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
    i32 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.int32)
    x = f64(xyz).reshape(-1, 3)
    g = i32(groups) if groups is not None else np.zeros((0, 4), np.int32)
    k = (1 if mu_unit is not None else 0) if kind is None else kind
    _check(lib().fg_state_write(str(path).encode(), k, _p(f64(box)), len(x), _p(x), _p(f64(charge)),
                                _p(f64(radius)), _p(f64(mw)), _p(i32(ids)), _p(i32(hydrophobic)), _p(f64(mu_unit)),
                                _p(f64(mu_scalar)), len(g), _p(g), _p(f64(group_cm)), int(rng_seed)))


def slump_uniforms(seed, n):
    """The reference's global slump() draws from seed (fg_slump_uniforms)."""
    u = np.empty(int(n))
    _check(lib().fg_slump_uniforms(int(seed), int(n), _p(u)))
    return u


def tune_reset():
    """Forget the autotuner's recorded launch shapes (fg_tune_reset)."""
    _check(lib().fg_tune_reset())


def _check(rc):
    if rc != 0:
        raise FgError("%d: %s" % (rc, lib().fg_last_error().decode()))


def philox4x32_10(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.empty(4, dtype=np.uint32)
    lib().fg_philox4x32_10(_p(c), _p(k), _p(out))
    return out


class System:
    """One Monte Carlo system resident on the GPU."""

    def __init__(self, params, xyz, charge=None, type_ids=None, threads=0):
        if not isinstance(params, FgParams):
            raise TypeError("params must be FgParams")
        self.params = FgParams.from_buffer_copy(bytes(params))   # own copy: volume moves change the box
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        self.n = len(xyz)
        h = ctypes.c_void_p()
        _check(lib().fg_create(ctypes.byref(params), self.n, ctypes.byref(h)))
        self.h = h
        if threads:
            _check(lib().fg_set_threads(self.h, threads))
        self.set_state(xyz, charge, type_ids)

    @classmethod
    def from_snapshot(cls, blob, threads=0):
        """A new system holding the state of a snapshot (fg_snapshot_info,
        fg_create, fg_restore)."""
        buf = np.frombuffer(blob, dtype=np.uint8)
        params, n = FgParams(), np.zeros(1, np.int32)
        _check(lib().fg_snapshot_info(_p(buf), len(buf), ctypes.byref(params), _p(n), None, None, None, None, None))
        ids, q = np.zeros(int(n[0]), np.int32), np.zeros(int(n[0]))
        _check(lib().fg_snapshot_info(_p(buf), len(buf), None, None, None, None, None, _p(ids), _p(q)))
        self = cls.__new__(cls)
        self.params = params
        self.n = int(n[0])
        h = ctypes.c_void_p()
        _check(lib().fg_create(ctypes.byref(params), self.n, ctypes.byref(h)))
        self.h = h
        if threads:
            _check(lib().fg_set_threads(self.h, threads))
        self._ids, self._q = ids, q
        self.restore(blob)
        return self

    def snapshot(self):
        """Device -> host snapshot of the whole state (bytes)."""
        buf = np.zeros(int(lib().fg_snapshot_bytes(self.h)), np.uint8)
        _check(lib().fg_snapshot(self.h, _p(buf), len(buf)))
        return buf.tobytes()

    def restore(self, blob):
        buf = np.frombuffer(blob, dtype=np.uint8)
        _check(lib().fg_restore(self.h, _p(buf), len(buf)))

    def close(self):
        if getattr(self, "h", None):
            lib().fg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, xyz, charge=None, type_ids=None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        if type_ids is None:
            type_ids = np.zeros(self.n, dtype=np.int32)
        self._ids = np.ascontiguousarray(type_ids, dtype=np.int32)
        q = None if charge is None else np.ascontiguousarray(charge, dtype=np.float64)
        self._q = q if q is not None else np.array([self.params.type_charge[t] for t in self._ids])
        _check(lib().fg_set_state(self.h, _p(xyz), _p(q), _p(self._ids)))

    @property
    def charges(self):
        """Per-particle charges as uploaded (host copy)."""
        return self._q

    @property
    def type_ids(self):
        return self._ids

    def save_state(self, path, mw=None, rng_seed=5489, id_offset=1):
        """The current configuration as a reference state file (one atomic
        group; radius sigma/2 and mw per type, mw 1 when not given). Atom ids
        are type + id_offset: the reference's atom list keeps a dummy entry at
        id 0 (AtomMap(), species.h:493-503), so its first type is id 1."""
        ids = self._ids
        radius = np.array([0.5 * self.params.type_sigma[t] for t in ids])
        m = None if mw is None else np.asarray([mw[t] for t in ids], dtype=np.float64)
        write_state(path, np.array(self.params.box[:3]), self.positions(), self._q, radius, m, ids + id_offset,
                    groups=np.array([[0, self.n - 1, 0, 1]], np.int32), rng_seed=rng_seed)   # atomic: molsize 1

    @property
    def threads(self):
        return lib().fg_get_threads(self.h)

    @threads.setter
    def threads(self, t):
        _check(lib().fg_set_threads(self.h, int(t)))

    @property
    def cluster(self):
        """CTAs of the thread-block cluster an Ewald system run alone sweeps
        on (fg_set_cluster / fg_get_cluster; 0 sets the built-in choice)."""
        c = np.zeros(2, np.int32)
        _check(lib().fg_get_cluster(self.h, _p(c[:1]), _p(c[1:])))
        return int(c[0])

    @cluster.setter
    def cluster(self, c):
        _check(lib().fg_set_cluster(self.h, int(c)))

    @property
    def max_cluster(self):
        c = np.zeros(2, np.int32)
        _check(lib().fg_get_cluster(self.h, _p(c[:1]), _p(c[1:])))
        return int(c[1])

    def autotune(self, n_trials=2048):
        """Time candidate launch shapes on a clone (fg_autotune) and apply the
        fastest; returns {"candidates": [(value, us/trial)], "chosen": value}."""
        return _tune(lib().fg_autotune, self.h, n_trials)

    def total_energy_fp64(self):
        """systemEnergy with every term in FP64 (fg_total_energy_fp64)."""
        c = np.empty(5)
        _check(lib().fg_total_energy_fp64(self.h, _p(c)))
        return dict(pairs=c[0], reciprocal=c[1], self=c[2], surface=c[3], total=c[4])

    def volume_move(self, half, dp, pressure, u, reference_quirk=False):
        """Isobaric volume move (fg_volume_move): half = slump.half(), dp the
        log-volume step, pressure in particles per cubic Angstrom, u the
        Metropolis uniform. Returns (dU, accepted); the box follows."""
        du = np.zeros(1)
        acc = np.zeros(1, np.int32)
        _check(lib().fg_volume_move(self.h, float(half), float(dp), float(pressure), float(u),
                                    1 if reference_quirk else 0, _p(du), _p(acc)))
        if acc[0]:
            b = np.zeros(3)
            _check(lib().fg_get_box(self.h, _p(b)))
            for a in range(3):
                self.params.box[a] = b[a]
        return float(du[0]), bool(acc[0])

    @property
    def box(self):
        b = np.zeros(3)
        _check(lib().fg_get_box(self.h, _p(b)))
        return b

    def rdf_sample(self, type1, type2, dr, n_bins, hist=None):
        """Add the current configuration's type1-type2 pair counts (AtomRDF
        binning) to hist (int64[n_bins], new if None); returns (hist, pairs
        at any distance counted by this call)."""
        h = np.zeros(n_bins, np.int64) if hist is None else hist
        assert h.dtype == np.int64 and h.flags.c_contiguous and len(h) == n_bins
        tot = np.zeros(1, np.int64)
        _check(lib().fg_rdf_sample(self.h, int(type1), int(type2), float(dr), int(n_bins), _p(h), _p(tot)))
        return h, int(tot[0])

    def positions(self):
        out = np.empty((self.n, 3))
        _check(lib().fg_get_state(self.h, _p(out)))
        return out

    @property
    def num_kvectors(self):
        return lib().fg_num_kvectors(self.h)

    def qk(self):
        K = self.num_kvectors
        q = np.empty(2 * max(K, 1))
        _check(lib().fg_get_qk(self.h, _p(q)))
        return q[0:2 * K:2] + 1j * q[1:2 * K:2]

    def trial_du(self, idx, new_xyz):
        idx = np.ascontiguousarray(np.atleast_1d(idx), dtype=np.int32)
        x = np.ascontiguousarray(new_xyz, dtype=np.float64).reshape(-1, 3)
        du = np.zeros(1)
        _check(lib().fg_trial_du(self.h, len(idx), _p(idx), _p(x), _p(du)))
        return float(du[0])

    def commit(self, accepted):
        c = np.zeros(1)
        _check(lib().fg_commit(self.h, 1 if accepted else 0, _p(c)))
        return float(c[0])

    def rebuild_qk(self):
        c = np.zeros(1)
        _check(lib().fg_rebuild_qk(self.h, _p(c)))
        return float(c[0])

    def total_energy(self):
        c = np.zeros(5)
        _check(lib().fg_total_energy(self.h, _p(c)))
        return dict(pairs=c[0], reciprocal=c[1], self=c[2], surface=c[3], total=c[4])

    def draw_translation_stream(self, seed, n):
        n = int(n)
        idx = np.empty(n, np.int32)
        disp = np.empty((n, 3))
        u = np.empty(n)
        _check(lib().fg_draw_translation_stream(self.h, seed, n, _p(idx), _p(disp), _p(u)))
        return idx, disp, u

    def sweep(self, idx, disp, u, log=True):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        disp = np.ascontiguousarray(disp, dtype=np.float64).reshape(-1, 3)
        u = np.ascontiguousarray(u, dtype=np.float64)
        n = len(idx)
        acc = np.empty(n, np.uint8) if log else None
        du = np.empty(n) if log else None
        st = SweepStats()
        _check(lib().fg_sweep(self.h, n, _p(idx), _p(disp), _p(u), _p(acc), _p(du), ctypes.byref(st)))
        return dict(acc=acc, du=du, stats=st.as_dict())

    def stream_upload(self, idx, disp, u):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        disp = np.ascontiguousarray(disp, dtype=np.float64).reshape(-1, 3)
        u = np.ascontiguousarray(u, dtype=np.float64)
        _check(lib().fg_stream_upload(self.h, len(idx), _p(idx), _p(disp), _p(u)))

    def stream_philox(self, n, seed, stream_id=0):
        _check(lib().fg_stream_philox(self.h, int(n), seed, stream_id))

    def stream_get(self, first, n):
        idx = np.empty(n, np.int32)
        disp = np.empty((n, 3))
        u = np.empty(n)
        _check(lib().fg_stream_get(self.h, first, n, _p(idx), _p(disp), _p(u)))
        return idx, disp, u

    def stream_run(self):
        st = SweepStats()
        _check(lib().fg_stream_run(self.h, ctypes.byref(st)))
        return st.as_dict()

    def log_get(self, first, n):
        """dU and acceptance of trials [first, first + n) of the last logged
        run (a logged sweep, or a batch run with set_log on)."""
        du = np.empty(n)
        acc = np.empty(n, np.uint8)
        _check(lib().fg_log_get(self.h, int(first), int(n), _p(du), _p(acc)))
        return du, acc

    def synchronize(self):
        _check(lib().fg_synchronize(self.h))

    def set_rebuild_policy(self, skip):
        _check(lib().fg_set_rebuild_policy(self.h, 1 if skip else 0))

    def running_energy(self):
        u = np.zeros(1)
        _check(lib().fg_running_energy(self.h, _p(u)))
        return float(u[0])

    @property
    def device_bytes(self):
        return int(lib().fg_device_bytes(self.h))


class Batch:
    """Independent systems advanced together, one CTA per system."""

    def __init__(self, systems, threads=0):
        self.systems = list(systems)
        arr = (ctypes.c_void_p * len(self.systems))(*[s.h.value for s in self.systems])
        h = ctypes.c_void_p()
        _check(lib().fg_batch_create(ctypes.cast(arr, ctypes.c_void_p), len(self.systems), ctypes.byref(h)))
        self.h = h
        if threads:
            _check(lib().fg_batch_set_threads(self.h, threads))

    def close(self):
        if getattr(self, "h", None):
            lib().fg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stream_philox(self, counts, seed, stream_ids=None):
        c = np.ascontiguousarray(counts, dtype=np.int64)
        ids = None if stream_ids is None else np.ascontiguousarray(stream_ids, dtype=np.uint32)
        _check(lib().fg_batch_stream_philox(self.h, _p(c), seed, _p(ids)))

    def autotune(self, n_trials=1024):
        """Time schedules on clones of the members (fg_batch_autotune) and
        apply the fastest; returns {"candidates": [...], "chosen": value}."""
        return _tune(lib().fg_batch_autotune, self.h, n_trials)

    def stream_upload(self, member, idx, disp, u):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        disp = np.ascontiguousarray(disp, dtype=np.float64).reshape(-1, 3)
        u = np.ascontiguousarray(u, dtype=np.float64)
        _check(lib().fg_batch_stream_upload(self.h, member, len(idx), _p(idx), _p(disp), _p(u)))

    def set_rebuild_mode(self, mode):
        """0: Q(k) rebuilds inside the sweep launch when the batch fills the
        GPU, 1: always inside, 2: always in the separate rebuild kernel."""
        _check(lib().fg_batch_set_rebuild_mode(self.h, int(mode)))

    def set_log(self, member, on=True):
        """Log per-trial dU/acceptance of one member in later runs
        (System.log_get reads it)."""
        _check(lib().fg_batch_set_log(self.h, int(member), 1 if on else 0))

    def run(self):
        n = len(self.systems)
        per = (SweepStats * n)()
        tot = SweepStats()
        _check(lib().fg_batch_run(self.h, ctypes.cast(per, ctypes.c_void_p), ctypes.byref(tot)))
        return [p.as_dict() for p in per], tot.as_dict()

    # parallel tempering
    def pt_setup(self, temperatures, seed):
        t = np.ascontiguousarray(temperatures, dtype=np.float64)
        _check(lib().fg_pt_setup(self.h, _p(t), seed))

    def pt_run(self, rounds, sweeps_per_round):
        tot = SweepStats()
        _check(lib().fg_pt_run(self.h, rounds, sweeps_per_round, ctypes.byref(tot)))
        return tot.as_dict()

    def pt_swap(self, u_direction, u_accept, energies=None):
        """One exchange attempt with given uniforms (and per-system
        energies); returns per rung whether its system changed."""
        n = len(self.systems)
        ex = np.zeros(n, np.int32)
        e = None if energies is None else np.ascontiguousarray(energies, dtype=np.float64)
        _check(lib().fg_pt_swap(self.h, float(u_direction), float(u_accept), _p(e), _p(ex)))
        return ex

    def pt_state(self):
        n = len(self.systems)
        perm = np.empty(n, np.int32)
        e = np.empty(n)
        att = np.empty(n, np.int64)
        acc = np.empty(n, np.int64)
        _check(lib().fg_pt_get(self.h, _p(perm), _p(e), _p(att), _p(acc)))
        return dict(perm=perm, energies=e, attempts=att, accepts=acc)


class Server:
    """Continuous-batching job server (admission by device footprint)."""

    def __init__(self, max_bytes, threads=0, round_pairs=0):
        h = ctypes.c_void_p()
        _check(lib().fg_server_create(int(max_bytes), threads, int(round_pairs), ctypes.byref(h)))
        self.h = h
        self._n = {}

    def close(self):
        if getattr(self, "h", None):
            lib().fg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, params, xyz, charge, type_ids, seed, n_trials):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        q = None if charge is None else np.ascontiguousarray(charge, dtype=np.float64)
        ids = np.ascontiguousarray(type_ids, dtype=np.int32)
        jid = np.zeros(1, np.int64)
        _check(lib().fg_server_submit(self.h, ctypes.byref(params), len(xyz), _p(xyz), _p(q), _p(ids), seed,
                                      int(n_trials), _p(jid)))
        self._n[int(jid[0])] = len(xyz)
        return int(jid[0])

    def step(self):
        r = np.zeros(1, np.int32)
        f = np.zeros(1, np.int32)
        ms = np.zeros(1)
        _check(lib().fg_server_step(self.h, _p(r), _p(f), _p(ms)))
        return int(r[0]), int(f[0]), float(ms[0])

    def poll(self, job_id, positions=False):
        st = np.zeros(1, np.int32)
        done = np.zeros(1, np.int64)
        acc = np.zeros(1, np.int64)
        e = np.zeros(1)
        xyz = np.empty((self._n[job_id], 3)) if positions else None
        _check(lib().fg_server_poll(self.h, job_id, _p(st), _p(done), _p(acc), _p(e), _p(xyz)))
        return dict(state=int(st[0]), trials=int(done[0]), accepted=int(acc[0]), energy=float(e[0]), xyz=xyz)

    def release(self, job_id):
        _check(lib().fg_server_release(self.h, job_id))

    def cancel(self, job_id):
        """Drop a job in any state; a running one stops between rounds."""
        _check(lib().fg_server_cancel(self.h, job_id))

    @property
    def bytes_in_use(self):
        return int(lib().fg_server_bytes_in_use(self.h))

    def snapshot(self, job_id):
        """A running job's snapshot (bytes), taken between steps."""
        buf = np.zeros(int(lib().fg_server_snapshot_bytes(self.h, job_id)), np.uint8)
        _check(lib().fg_server_snapshot(self.h, job_id, _p(buf), len(buf)))
        return buf.tobytes()

    def resume(self, blob):
        """Queue a job that continues from a job snapshot; returns its id."""
        buf = np.frombuffer(blob, dtype=np.uint8)
        jid = np.zeros(1, np.int64)
        _check(lib().fg_server_resume(self.h, _p(buf), len(buf), _p(jid)))
        hdr = 48   # the job fields ahead of the system snapshot (JobSnapHeader)
        n = np.zeros(1, np.int32)
        _check(lib().fg_snapshot_info(_p(buf[hdr:]), len(buf) - hdr, None, _p(n), None, None, None, None, None))
        self._n[int(jid[0])] = int(n[0])
        return int(jid[0])


def mol_run_many(systems):
    """Run the staged streams of several MolSystems in one launch."""
    arr = (ctypes.c_void_p * len(systems))(*[s.h.value for s in systems])
    per = (SweepStats * len(systems))()
    tot = SweepStats()
    _check(lib().fg_mol_run_many(ctypes.cast(arr, ctypes.c_void_p), len(systems), ctypes.cast(per, ctypes.c_void_p),
                                 ctypes.byref(tot)))
    return [p.as_dict() for p in per], tot.as_dict()


def mol_draw_stream(seed, n_molecules, n, dp=1.0, dprot=0.3, center_rotation=True):
    """The reference's draws for n TranslateRotate trials (host only)."""
    g = np.empty(n, np.int32)
    ax = np.empty((n, 3))
    ce = np.empty(n, np.int32)
    an = np.empty(n)
    tr = np.empty((n, 3))
    u = np.empty(n)
    _check(lib().fg_mol_draw_stream(seed, n_molecules, n, dp, dprot, 1 if center_rotation else 0, _p(g), _p(ax),
                                    _p(ce), _p(an), _p(tr), _p(u)))
    return dict(group=g, axis=ax, center=ce, angle=an, trans=tr, u=u)


class MolSystem:
    """Rigid dipolar molecules on one GPU (fg_mol_* C-ABI)."""

    def __init__(self, params, xyz, mu_unit, mu_scalar, type_ids, sites_per_molecule, mass_centers=None,
                 cluster=0):
        n = len(type_ids)
        h = ctypes.c_void_p()
        _check(lib().fg_mol_create(ctypes.byref(params), n, sites_per_molecule, ctypes.byref(h)))
        self.h = h
        self.n, self.gs, self.m = n, sites_per_molecule, n // sites_per_molecule
        if cluster:
            self.cluster = cluster
        self.set_state(xyz, mu_unit, mu_scalar, type_ids, mass_centers)

    def close(self):
        if getattr(self, "h", None):
            lib().fg_mol_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, xyz, mu_unit, mu_scalar, type_ids, mass_centers=None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        mu = None if mu_unit is None else np.ascontiguousarray(mu_unit, dtype=np.float64).reshape(-1, 3)
        ms = None if mu_scalar is None else np.ascontiguousarray(mu_scalar, dtype=np.float64)
        ids = np.ascontiguousarray(type_ids, dtype=np.int32)
        cm = None if mass_centers is None else np.ascontiguousarray(mass_centers, dtype=np.float64).reshape(-1, 3)
        _check(lib().fg_mol_set_state(self.h, _p(xyz), _p(mu), _p(ms), _p(ids), _p(cm)))

    def state(self):
        xyz = np.empty((self.n, 3))
        mu = np.empty((self.n, 3))
        cm = np.empty((self.m, 3))
        _check(lib().fg_mol_get_state(self.h, _p(xyz), _p(mu), _p(cm)))
        return xyz, mu, cm

    @property
    def cluster(self):
        c = np.zeros(2, np.int32)
        _check(lib().fg_mol_get_cluster(self.h, _p(c[:1]), _p(c[1:])))
        return int(c[0])

    @cluster.setter
    def cluster(self, c):
        _check(lib().fg_mol_set_cluster(self.h, int(c)))

    @property
    def max_cluster(self):
        c = np.zeros(2, np.int32)
        _check(lib().fg_mol_get_cluster(self.h, _p(c[:1]), _p(c[1:])))
        return int(c[1])

    def autotune(self, n_trials=256):
        """Time cluster sizes on a clone (fg_mol_autotune) and apply the fastest."""
        return _tune(lib().fg_mol_autotune, self.h, n_trials)

    def trial_du(self, molecule, new_xyz, new_mu=None, new_cm=None):
        x = np.ascontiguousarray(new_xyz, dtype=np.float64).reshape(-1, 3)
        m = None if new_mu is None else np.ascontiguousarray(new_mu, dtype=np.float64).reshape(-1, 3)
        c = None if new_cm is None else np.ascontiguousarray(new_cm, dtype=np.float64)
        du = np.zeros(1)
        _check(lib().fg_mol_trial_du(self.h, molecule, _p(x), _p(m), _p(c), _p(du)))
        return float(du[0])

    def commit(self, accepted):
        _check(lib().fg_mol_commit(self.h, 1 if accepted else 0))

    def sweep(self, st, rotate=True, translate=True, log=True):
        n = len(st["group"])
        g = np.ascontiguousarray(st["group"], dtype=np.int32)
        ax = np.ascontiguousarray(st["axis"], dtype=np.float64)
        an = np.ascontiguousarray(st["angle"], dtype=np.float64)
        ce = np.ascontiguousarray(st["center"], dtype=np.int32)
        tr = np.ascontiguousarray(st["trans"], dtype=np.float64)
        u = np.ascontiguousarray(st["u"], dtype=np.float64)
        acc = np.empty(n, np.uint8) if log else None
        du = np.empty(n) if log else None
        stats = SweepStats()
        _check(lib().fg_mol_sweep(self.h, n, _p(g), _p(ax), _p(an), _p(ce), _p(tr), _p(u), 1 if rotate else 0,
                                  1 if translate else 0, _p(acc), _p(du), ctypes.byref(stats)))
        out = stats.as_dict()
        out.update(acc=acc, du=du)
        return out

    def stream_upload(self, st, rotate=True, translate=True):
        g = np.ascontiguousarray(st["group"], dtype=np.int32)
        ax = np.ascontiguousarray(st["axis"], dtype=np.float64)
        an = np.ascontiguousarray(st["angle"], dtype=np.float64)
        ce = np.ascontiguousarray(st["center"], dtype=np.int32)
        tr = np.ascontiguousarray(st["trans"], dtype=np.float64)
        u = np.ascontiguousarray(st["u"], dtype=np.float64)
        _check(lib().fg_mol_stream_upload(self.h, len(g), _p(g), _p(ax), _p(an), _p(ce), _p(tr), _p(u),
                                          1 if rotate else 0, 1 if translate else 0))

    def total_energy(self):
        c = np.empty(3)
        _check(lib().fg_mol_total_energy(self.h, _p(c)))
        return c

    def running_energy(self):
        u = np.zeros(1)
        _check(lib().fg_mol_running_energy(self.h, _p(u)))
        return float(u[0])

    @property
    def device_bytes(self):
        return int(lib().fg_mol_device_bytes(self.h))


# ---------------------------------------------------------------- point dipoles under Ewald
def dip_draw_stream(seed, n_particles, n, p_rotate=0.5, dp=0.7, dprot=1.0, kinds=None):
    """The reference's slump draws for n AtomicRotation / AtomicTranslation
    trials (fg_dip_draw_stream): dict(kind, idx, axis, angle, disp, u). With
    kinds given (1 rotation, 2 translation) p_rotate is not used."""
    kind = np.empty(n, np.int32) if kinds is None else np.array(kinds, dtype=np.int32)
    if kinds is not None:
        p_rotate = -1.0
    idx = np.empty(n, np.int32)
    axis = np.empty((n, 3))
    angle = np.empty(n)
    disp = np.empty((n, 3))
    u = np.empty(n)
    _check(lib().fg_dip_draw_stream(int(seed), int(n_particles), int(n), float(p_rotate), float(dp), float(dprot),
                                    _p(kind), _p(idx), _p(axis), _p(angle), _p(disp), _p(u)))
    return dict(kind=kind, idx=idx, axis=axis, angle=angle, disp=disp, u=u)


def _dip_stream_arrays(st):
    return [np.ascontiguousarray(st[k], dtype=np.int32 if k in ("kind", "idx") else np.float64)
            for k in ("kind", "idx", "axis", "angle", "disp", "u")]


def dip_autotune(systems, n_trials=256):
    """Threads per system timed on clones of these DipoleSystems run together
    (fg_dip_autotune); the fastest is applied to them and remembered."""
    arr = (ctypes.c_void_p * len(systems))(*[s.h.value for s in systems])
    r = TuneReport()
    _check(lib().fg_dip_autotune(ctypes.cast(arr, ctypes.c_void_p), len(systems), int(n_trials), ctypes.byref(r)))
    return r.as_dict()


def dip_run_many(systems):
    """Run the staged streams of several DipoleSystems in one launch sequence
    (one CTA per system)."""
    arr = (ctypes.c_void_p * len(systems))(*[s.h.value for s in systems])
    per = (SweepStats * len(systems))()
    tot = SweepStats()
    _check(lib().fg_dip_run_many(ctypes.cast(arr, ctypes.c_void_p), len(systems), ctypes.cast(per, ctypes.c_void_p),
                                 ctypes.byref(tot)))
    return [p.as_dict() for p in per], tot.as_dict()


class DipoleSystem:
    """Point charges and point dipoles under Ewald summation on one GPU
    (fg_dip_* C-ABI): AtomicRotation / AtomicTranslation with the energy of
    NonbondedEwald<Tspace, LennardJonesLB, ...>."""

    def __init__(self, params, xyz, mu_unit, mu_scalar, type_ids, charges=None, threads=None):
        n = len(type_ids)
        h = ctypes.c_void_p()
        _check(lib().fg_dip_create(ctypes.byref(params), n, ctypes.byref(h)))
        self.h = h
        self.n = n
        if threads:
            _check(lib().fg_dip_set_threads(self.h, int(threads)))
        self.set_state(xyz, mu_unit, mu_scalar, type_ids, charges)

    def close(self):
        if getattr(self, "h", None):
            lib().fg_dip_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_kvectors(self):
        return int(lib().fg_dip_num_kvectors(self.h))

    def set_threads(self, threads):
        """Threads of the system's CTA (multiple of 32, 32..256)."""
        _check(lib().fg_dip_set_threads(self.h, int(threads)))

    def set_state(self, xyz, mu_unit, mu_scalar, type_ids, charges=None):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        mu = np.ascontiguousarray(mu_unit, dtype=np.float64).reshape(-1, 3)
        ms = np.ascontiguousarray(mu_scalar, dtype=np.float64)
        ids = np.ascontiguousarray(type_ids, dtype=np.int32)
        q = None if charges is None else np.ascontiguousarray(charges, dtype=np.float64)
        _check(lib().fg_dip_set_state(self.h, _p(xyz), _p(mu), _p(ms), _p(q), _p(ids)))

    def state(self):
        xyz = np.empty((self.n, 3))
        mu = np.empty((self.n, 3))
        _check(lib().fg_dip_get_state(self.h, _p(xyz), _p(mu)))
        return xyz, mu

    def trial_du(self, i, new_xyz, new_mu=None):
        x = np.ascontiguousarray(new_xyz, dtype=np.float64)
        m = None if new_mu is None else np.ascontiguousarray(new_mu, dtype=np.float64)
        du = np.zeros(1)
        _check(lib().fg_dip_trial_du(self.h, int(i), _p(x), _p(m), _p(du)))
        return float(du[0])

    def commit(self, accepted):
        """Returns the Q(k) rebuild correction (NonbondedEwald::update)."""
        c = np.zeros(1)
        _check(lib().fg_dip_commit(self.h, 1 if accepted else 0, _p(c)))
        return float(c[0])

    def sweep(self, st, log=True):
        kind, idx, axis, angle, disp, u = _dip_stream_arrays(st)
        n = len(idx)
        acc = np.empty(n, np.uint8) if log else None
        du = np.empty(n) if log else None
        stats = SweepStats()
        _check(lib().fg_dip_sweep(self.h, n, _p(kind), _p(idx), _p(axis), _p(angle), _p(disp), _p(u), _p(acc),
                                  _p(du), ctypes.byref(stats)))
        out = stats.as_dict()
        out.update(acc=acc, du=du)
        return out

    def stream_upload(self, st):
        kind, idx, axis, angle, disp, u = _dip_stream_arrays(st)
        _check(lib().fg_dip_stream_upload(self.h, len(idx), _p(kind), _p(idx), _p(axis), _p(angle), _p(disp), _p(u)))

    def total_energy(self):
        """{EwaldReal pairs, LJ pairs, reciprocal, self, surface, total} in FP64."""
        c = np.empty(6)
        _check(lib().fg_dip_total_energy(self.h, _p(c)))
        return c

    def running_energy(self):
        u = np.zeros(1)
        _check(lib().fg_dip_running_energy(self.h, _p(u)))
        return float(u[0])

    @property
    def device_bytes(self):
        return int(lib().fg_dip_device_bytes(self.h))
