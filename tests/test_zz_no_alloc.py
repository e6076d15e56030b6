"""fg_pair_energy_noalloc: the pair energy for callers that cannot call
cudaMalloc (a plugin inside a host application that owns the GPU memory
pool, or a loop that must not call the allocator). The caller passes device
buffers; the library's temporaries live in one fixed __device__ array.

Checked through the C-ABI against the existing entry point (component 0 of
fg_total_energy) on consecutive calls with different systems, within the
1e-6 kT tolerance the parity tests use. This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from beofaunus_gb300 import workloads

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _noalloc(params, xyz, charge, types):
    import torch

    from beofaunus_gb300.gpu import FgError, lib
    L = lib()
    f = L.fg_pair_energy_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    dev = torch.device("cuda", 0)
    d_xyz = torch.tensor(np.ascontiguousarray(xyz, dtype=np.float64).ravel(), device=dev)
    d_q = None if charge is None else torch.tensor(np.ascontiguousarray(charge, dtype=np.float64), device=dev)
    d_t = torch.tensor(np.ascontiguousarray(types, dtype=np.int32), device=dev)
    d_e = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = f(ctypes.byref(params), len(types), d_xyz.data_ptr(), None if d_q is None else d_q.data_ptr(),
           d_t.data_ptr(), d_e.data_ptr(), stream)
    if rc != 0:
        raise FgError("%d: %s" % (rc, L.fg_last_error().decode()))
    torch.cuda.synchronize(dev)
    return float(d_e.cpu().numpy()[0])


def _reference(params, xyz, charge, types):
    from beofaunus_gb300.gpu import System
    s = System(params, xyz, charge, types)
    e = s.total_energy()["pairs"]
    s.close()
    return e


def test_no_alloc_pair_energy_matches_existing_entry_point():
    cases = [workloads.rpm800(seed=41), workloads.dh_lj_salt(700, seed=42), workloads.rpm800(seed=43)]
    for p, x, q, t in cases:
        want = _reference(p, x, q, t)
        got = _noalloc(p, x, q, t)
        assert got == pytest.approx(want, abs=TOL)
    # the same system twice in a row, charges taken from the atom types
    p, x, q, t = cases[0]
    a = _noalloc(p, x, None, t)
    b = _noalloc(p, x, None, t)
    assert a == b
    assert a == pytest.approx(_reference(p, x, q, t), abs=TOL)


def test_no_alloc_rejects_sizes_beyond_its_limit():
    from beofaunus_gb300.gpu import FgError, lib
    p, x, q, t = workloads.rpm800(seed=44)
    f = lib().fg_pair_energy_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    dummy = ctypes.c_void_p(16)
    rc = f(ctypes.byref(p), 65537, dummy, None, dummy, dummy, None)
    assert rc == -5   # FG_ERR_CAPACITY, before any device access
    assert b"limit" in lib().fg_last_error()
