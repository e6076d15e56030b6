"""fg_pair_energy_noalloc: the pair energy for callers that cannot call
cudaMalloc (a plugin inside a host application that owns the GPU memory
pool, or a loop that must not call the allocator). The caller passes device
buffers; the library's temporaries live in one fixed __device__ array.

Checked through the C-ABI against the existing entry point (component 0 of
fg_total_energy) on consecutive calls with different systems, within the
1e-6 kT tolerance the parity tests use, and against the FP64 oracle's pair
energy within the tolerance of the total-energy parity test (FP32 pair terms
summed over ~1e5 pairs). This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from beofaunus_gb300 import workloads
from beofaunus_gb300.params import FG_MODEL_DH_LJ, make_params

pytestmark = pytest.mark.gpu

TOL = 1e-6          # against the existing entry point (same pair kernel)
TOL_ORACLE = 2e-4   # against the FP64 oracle, as test_total_energy_matches_oracle


def _fn():
    from beofaunus_gb300.gpu import lib
    f = lib().fg_pair_energy_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _noalloc(params, xyz, charge, types):
    import torch

    from beofaunus_gb300.gpu import FgError, lib
    dev = torch.device("cuda", 0)
    d_xyz = torch.tensor(np.ascontiguousarray(xyz, dtype=np.float64).ravel(), device=dev)
    d_q = None if charge is None else torch.tensor(np.ascontiguousarray(charge, dtype=np.float64), device=dev)
    d_t = torch.tensor(np.ascontiguousarray(types, dtype=np.int32), device=dev)
    d_e = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = _fn()(ctypes.byref(params), len(types), d_xyz.data_ptr(), None if d_q is None else d_q.data_ptr(),
               d_t.data_ptr(), d_e.data_ptr(), stream)
    if rc != 0:
        raise FgError("%d: %s" % (rc, lib().fg_last_error().decode()))
    torch.cuda.synchronize(dev)
    return float(d_e.cpu().numpy()[0])


def _reference(params, xyz, charge, types):
    from beofaunus_gb300.gpu import System
    s = System(params, xyz, charge, types)
    e = s.total_energy()["pairs"]
    s.close()
    return e


def _oracle(params, xyz, charge, types):
    from oracle.oracle import OracleSystem
    return OracleSystem(params, xyz, charge, types).total_energy()["pairs"]


def _mixed_salt(n=500, seed=45):
    """Debye-Hueckel + LJ with three atom types of different sigma and
    charge: the type-pair tables are not uniform and the repulsive-core
    pairs read the Taylor table at several sigma_ij."""
    types = [dict(q=1.0, sigma=3.0, eps=0.2, dp=2.0), dict(q=-1.0, sigma=4.5, eps=0.3, dp=2.0),
             dict(q=-2.0, sigma=6.0, eps=0.1, dp=2.0)]
    box = (n / 0.002) ** (1.0 / 3.0)
    p = make_params(FG_MODEL_DH_LJ, box, 7.1, types, dh_debye_length=10.0)
    xyz = workloads.scatter_positions(n, box, 6.0, seed)
    ids = np.array([0] * (3 * n // 5) + [1] * (n // 5) + [2] * (n // 5), dtype=np.int32)   # neutral
    q = np.array([types[t]["q"] for t in ids])
    return p, xyz, q, ids


def test_no_alloc_pair_energy_matches_existing_entry_point_and_oracle():
    cases = [workloads.rpm800(seed=41), workloads.dh_lj_salt(700, seed=42), workloads.rpm800(seed=43),
             _mixed_salt()]
    for p, x, q, t in cases:
        want = _reference(p, x, q, t)
        got = _noalloc(p, x, q, t)
        ref = _oracle(p, x, q, t)
        print("no-alloc %.12f  fg_total_energy %.12f  oracle %.12f" % (got, want, ref))
        assert got == pytest.approx(want, abs=TOL)
        assert got == pytest.approx(ref, abs=TOL_ORACLE)
    # the same system twice in a row, charges taken from the atom types
    p, x, q, t = cases[0]
    a = _noalloc(p, x, None, t)
    b = _noalloc(p, x, None, t)
    assert a == b
    assert a == pytest.approx(_reference(p, x, q, t), abs=TOL)


def test_no_alloc_bad_type_id_gives_nan_and_the_next_call_recovers():
    p, x, q, t = workloads.rpm800(seed=46)
    bad = t.copy()
    bad[17] = p.n_types          # one past the last type
    assert np.isnan(_noalloc(p, x, q, bad))
    bad[17] = -1
    assert np.isnan(_noalloc(p, x, None, bad))
    # the error word is cleared by every call
    assert _noalloc(p, x, q, t) == pytest.approx(_reference(p, x, q, t), abs=TOL)


def test_no_alloc_rejects_sizes_beyond_its_limit():
    from beofaunus_gb300.gpu import lib
    p, x, q, t = workloads.rpm800(seed=44)
    f = _fn()
    dummy = ctypes.c_void_p(16)
    rc = f(ctypes.byref(p), 65537, dummy, None, dummy, dummy, None)
    assert rc == -5   # FG_ERR_CAPACITY, before any device access
    assert b"limit" in lib().fg_last_error()
    # a core-pair table longer than the array's slot (sigma 200 A at
    # kappa 0.1/A needs ceil(0.1 * 200 * 128) + 4 entries), also refused
    # before any device access
    big = make_params(FG_MODEL_DH_LJ, 500.0, 7.1, [dict(q=1.0, sigma=200.0, eps=0.1)], dh_debye_length=10.0)
    rc = f(ctypes.byref(big), 100, dummy, None, dummy, dummy, None)
    assert rc == -5
    assert b"core table" in lib().fg_last_error()
