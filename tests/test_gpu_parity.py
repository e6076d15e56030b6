"""GPU parity: the CUDA path against the FP64 oracle (pinned to the reference)
on the same seeded inputs and the same random stream.

Tolerance (written here, used everywhere below): every dU within 1e-6 kT of
the FP64 oracle; acceptance sequences identical except for trials whose
|dU - (-ln u)| is inside that tolerance band.
"""
import os

import numpy as np
import pytest

from beofaunus_gb300 import workloads
from beofaunus_gb300.params import FgParams
from oracle.oracle import OracleSystem, translation_stream

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL_DU = 1e-6


def gpu_system(params, xyz, q, ids, **kw):
    from beofaunus_gb300.gpu import System
    return System(params, xyz, q, ids, **kw)


def assert_same_chain(du_gpu, acc_gpu, du_ref, acc_ref, u):
    """dU within TOL_DU everywhere the chains agree; acceptance identical
    unless the threshold is inside the tolerance band (then stop comparing:
    the chains legitimately diverge from there)."""
    n = len(du_ref)
    err = np.abs(du_gpu - du_ref)
    mism = np.nonzero(acc_gpu != acc_ref)[0]
    upto = n
    if len(mism):
        t = mism[0]
        band = abs(du_ref[t] + np.log(u[t]))
        assert band < TOL_DU, "acceptance differs at trial %d outside the band (%g)" % (t, band)
        upto = t + 1
    assert np.all(np.isfinite(du_gpu[:upto]))
    assert err[:upto].max() <= TOL_DU, "max |dU err| = %g at trial %d" % (err[:upto].max(), err[:upto].argmax())
    return err[:upto]


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def params_of(g):
    p = FgParams.from_buffer_copy(g["params"].tobytes())
    p.bjerrum = float(g["bjerrum"])
    return p


@pytest.mark.parametrize("name", ["ewald_small_uf1", "ewald_surface_uf5", "ewald_rpm800", "ewald_iso", "dhlj_small",
                                  "dhlj_500"])
def test_sweep_reproduces_reference_log(name):
    """Device sweep with the host replay of the reference's RNG reproduces the
    reference's own per-trial log (dU, acceptance) and final positions."""
    g = load(name)
    p = params_of(g)
    s = gpu_system(p, g["xyz"], g["q"], g["ids"])
    n = len(g["idx"])
    idx, disp, u = s.draw_translation_stream(int(g["seed"]), n)
    np.testing.assert_array_equal(idx, g["idx"])
    r = s.sweep(idx, disp, u)
    assert_same_chain(r["du"], r["acc"], g["du"], g["acc"], u)
    np.testing.assert_array_equal(r["acc"], g["acc"])
    np.testing.assert_allclose(s.positions(), g["final_positions"], rtol=0, atol=1e-9)
    assert r["stats"]["energy_change"] == pytest.approx(float(g["u_move_sum"]), abs=1e-5)


def test_plain_trial_commit_matches_oracle_rpm800():
    """The per-trial drop-in (fg_trial_du + fg_commit) on the 800-ion Ewald system."""
    p, xyz, q, ids = workloads.rpm800(seed=3, update_frequency=50)
    s = gpu_system(p, xyz, q, ids)
    o = OracleSystem(p, xyz, q, ids)
    dpp = np.array([p.type_dp[i] for i in ids])
    idx, disp, u = translation_stream(77, dpp, 300)
    errs = []
    for t in range(300):
        i = int(idx[t])
        new = o.boundary(o.positions()[i] + disp[t])
        dg = s.trial_du(i, new)
        do = o.trial_du(i, new)
        errs.append(abs(dg - do))
        acc = not (u[t] > np.exp(-do))
        cg = s.commit(acc)
        co = o.commit(acc)
        assert cg == pytest.approx(co, abs=1e-6)
    assert max(errs) <= TOL_DU, max(errs)
    np.testing.assert_allclose(s.positions(), o.positions(), rtol=0, atol=1e-9)


def test_sweep_rpm16k_cell_list_full_size():
    """16384 ions, L=163, |n|^2<=100 (K=2242), cell list: 2000 trials."""
    p, xyz, q, ids = workloads.rpm16k(seed=5, update_frequency=1000)
    s = gpu_system(p, xyz, q, ids)
    o = OracleSystem(p, xyz, q, ids)
    assert s.num_kvectors == o.num_kvectors == 2242
    idx, disp, u = s.draw_translation_stream(2024, 2000)
    r = s.sweep(idx, disp, u)
    ro = o.mc_run_stream(idx, disp, u)
    err = assert_same_chain(r["du"], r["acc"], ro["du"], ro["acc"], u)
    print("rpm16k: max |dU err| %.3g rms %.3g" % (err.max(), np.sqrt(np.mean(err ** 2))))
    np.testing.assert_allclose(s.positions(), o.positions(), rtol=0, atol=1e-9)
    # Q(k) is the exact sum of per-particle terms on a 2^-22 grid (rounding
    # error <= 1.2e-7 each, rms 6.9e-8) from FP32 products (~1e-7 each): its
    # distance from the FP64 sum has rms ~ sqrt(N) * 1.2e-7 = 1.5e-5 per
    # component here, and stays below 4 sigma = 6e-5 over the 2 x 2242
    # components; the running energy sees it only through the FP32 Q(k)
    qg = s.qk()
    qo = o.qk()[0]
    dq = np.abs(qg - qo)
    print("rpm16k Q(k) vs FP64: max %.3g rms %.3g" % (dq.max(), np.sqrt(np.mean(dq ** 2))))
    assert dq.max() < 6e-5


def test_total_energy_matches_oracle():
    p, xyz, q, ids = workloads.rpm800(seed=8, update_frequency=1000)
    s = gpu_system(p, xyz, q, ids)
    o = OracleSystem(p, xyz, q, ids)
    eg, eo = s.total_energy(), o.total_energy()
    assert eg["pairs"] == pytest.approx(eo["pairs"], abs=2e-4)
    assert eg["reciprocal"] == pytest.approx(eo["reciprocal"], abs=2e-4)
    assert eg["self"] == pytest.approx(eo["self"], rel=1e-12)
    assert eg["surface"] == pytest.approx(eo["surface"], abs=1e-9)
    assert eg["total"] == pytest.approx(eo["total"], abs=2e-4)
    # and after a device sweep the running energy tracks the total
    idx, disp, u = s.draw_translation_stream(99, 1600)
    r = s.sweep(idx, disp, u, log=False)
    ro = o.mc_run_stream(idx, disp, u)
    e1 = s.total_energy()["total"]
    assert e1 == pytest.approx(o.total_energy()["total"], abs=5e-4)
    assert r["stats"]["energy_change"] == pytest.approx(ro["utot"], abs=1e-4)


@pytest.mark.parametrize("n", [500, 4000])
def test_dh_lj_sweep_matches_oracle(n):
    p, xyz, q, ids = workloads.dh_lj_salt(n, seed=n)
    s = gpu_system(p, xyz, q, ids)
    o = OracleSystem(p, xyz, q, ids)
    idx, disp, u = s.draw_translation_stream(n + 1, 3 * n)
    r = s.sweep(idx, disp, u)
    ro = o.mc_run_stream(idx, disp, u)
    assert_same_chain(r["du"], r["acc"], ro["du"], ro["acc"], u)
    np.testing.assert_allclose(s.positions(), o.positions(), rtol=0, atol=1e-9)


def test_philox_stream_run_matches_oracle():
    """Device-generated stream: downloaded and replayed by the oracle."""
    p, xyz, q, ids = workloads.rpm800(seed=21, update_frequency=200)
    s = gpu_system(p, xyz, q, ids)
    o = OracleSystem(p, xyz, q, ids)
    s.stream_philox(1600, seed=1234, stream_id=7)
    idx, disp, u = s.stream_get(0, 1600)
    assert idx.min() >= 0 and idx.max() < 800
    assert np.all(np.abs(disp) <= 1.0 + 1e-12)
    st = s.stream_run()
    assert st["trials"] == 1600
    ro = o.mc_run_stream(idx, disp, u)
    assert st["accepted"] == int(ro["acc"].sum())
    np.testing.assert_allclose(s.positions(), o.positions(), rtol=0, atol=1e-9)


def test_rebuild_reproduces_running_qk_exactly():
    """Q(k) is an exact integer sum of per-particle contributions: after
    thousands of accepted moves a rebuild from scratch gives the same bits
    (correction exactly 0), and Q(k) stays within FP32-term accuracy of the
    oracle's FP64 sum."""
    p, xyz, q, ids = workloads.rpm800(seed=31, update_frequency=100000)
    s = gpu_system(p, xyz, q, ids)
    o = OracleSystem(p, xyz, q, ids)
    idx, disp, u = s.draw_translation_stream(5, 4000)
    r = s.sweep(idx, disp, u, log=False)
    o.mc_run_stream(idx, disp, u)
    q_inc = s.qk()
    assert s.rebuild_qk() == 0.0
    np.testing.assert_array_equal(s.qk(), q_inc)
    assert np.max(np.abs(q_inc - o.qk()[0])) < 2e-5
    assert r["stats"]["rebuilds"] == 0


def test_update_frequency_rebuilds_verify_exactly():
    """update_frequency=5: the sweep stops for a rebuild every 5 accepted
    trials (as NonbondedEwald::update does); each must reproduce Q(k)."""
    p, xyz, q, ids = workloads.rpm800(seed=32, update_frequency=5)
    s = gpu_system(p, xyz, q, ids)
    idx, disp, u = s.draw_translation_stream(6, 400)
    r = s.sweep(idx, disp, u, log=False)
    st = r["stats"]
    assert st["rebuilds"] == st["accepted"] // 5
    assert st["error_flags"] == 0


def test_invalid_arguments_fail_loudly():
    from beofaunus_gb300.gpu import FgError
    p, xyz, q, ids = workloads.rpm800(seed=1)
    s = gpu_system(p, xyz, q, ids)
    with pytest.raises(FgError):
        s.trial_du(800, [0.0, 0.0, 0.0])
    with pytest.raises(FgError):
        s.commit(True)   # no pending trial
    bad = FgParams.from_buffer_copy(bytes(p))
    bad.type_charge[0] = 0.0   # ewald.h:539 would divide by zero
    with pytest.raises(FgError):
        gpu_system(bad, xyz, q, ids)


def test_isotropic_pbc_qk_exact_and_energies():
    """isotropic_pbc (ewald.h:347-360, 394-399, 669-675): the positive-octant
    k-set, a real Q(k) (zero imaginary parts, bit for bit) that a rebuild
    reproduces exactly after a thousand trials, the plain per-trial path and
    the totals against the FP64 oracle."""
    p, xyz, q, ids = workloads.rpm_ewald(150, 26.0, 6, seed=41, update_frequency=50, cutoff=11.0, eps_surf=1.0)
    p.ewald_isotropic_pbc = 1
    s = gpu_system(p, xyz, q, ids)
    o = OracleSystem(p, xyz, q, ids)
    assert s.num_kvectors == o.num_kvectors
    idx, disp, u = s.draw_translation_stream(9, 1200)
    r = s.sweep(idx, disp, u)
    ro = o.mc_run_stream(idx, disp, u)
    assert_same_chain(r["du"], r["acc"], ro["du"], ro["acc"], u)
    assert r["stats"]["rebuilds"] > 0 and r["stats"]["error_flags"] == 0
    qk = s.qk()
    assert np.all(qk.imag == 0.0)
    assert s.rebuild_qk() == 0.0
    np.testing.assert_array_equal(s.qk(), qk)
    e64 = s.total_energy_fp64()
    eo = o.total_energy()
    assert e64["reciprocal"] == pytest.approx(eo["reciprocal"], abs=1e-9)
    assert e64["total"] == pytest.approx(eo["total"], abs=1e-8)
    # the plain drop-in path
    pos = o.positions()
    idx2, disp2, u2 = translation_stream(77, np.array([p.type_dp[i] for i in ids]), 100)
    for t in range(100):
        i = int(idx2[t])
        new = o.boundary(pos[i] + disp2[t])
        dg, do = s.trial_du(i, new), o.trial_du(i, new)
        assert abs(dg - do) <= TOL_DU
        acc = not (u2[t] > np.exp(-do))
        s.commit(acc)
        o.commit(acc)
        if acc:
            pos[i] = new


def test_rebuild_with_few_kvector_runs():
    """A k-set of fewer runs (k-vectors sharing n_x, n_y) than particles per
    rebuild pass: the rebuild's block then has fewer threads than a pass has
    particles, and each pass may hold no more particles than threads. 150
    ions, |n| <= 2: every rebuild (update_frequency 5) reproduces the running
    Q(k) exactly, and the chain is the oracle's."""
    p, xyz, q, ids = workloads.rpm_ewald(150, 32.0, 2, seed=43, update_frequency=5, cutoff=12.0)
    s = gpu_system(p, xyz, q, ids)
    o = OracleSystem(p, xyz, q, ids)
    idx, disp, u = s.draw_translation_stream(8, 600)
    r = s.sweep(idx, disp, u)
    ro = o.mc_run_stream(idx, disp, u)
    assert_same_chain(r["du"], r["acc"], ro["du"], ro["acc"], u)
    assert r["stats"]["rebuilds"] == r["stats"]["accepted"] // 5 and r["stats"]["error_flags"] == 0
    assert s.rebuild_qk() == 0.0
