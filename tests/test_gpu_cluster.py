"""GPU: the Ewald block sweep of a system alone on a thread-block cluster
(fg_set_cluster): the k-vectors split over the CTAs, partial sums meeting in
CTA 0. Parity against the reference's own logs and the FP64 oracle, and
against the same stream on one CTA.

Tolerances: every dU within 1e-6 kT of the FP64 oracle (as in
test_gpu_parity); between the cluster and one CTA the sums run in another
order, so dU agree within 1e-6 kT, while the chain itself (acceptances,
positions, the integer Q(k)) is identical unless a threshold falls inside
that band.
"""
import numpy as np
import pytest

from beofaunus_gb300 import workloads
from oracle.oracle import OracleSystem

from test_gpu_parity import TOL_DU, assert_same_chain, load, params_of

pytestmark = pytest.mark.gpu


def gpu_system(params, xyz, q, ids, cluster):
    from beofaunus_gb300.gpu import System
    s = System(params, xyz, q, ids)
    s.cluster = cluster
    return s


@pytest.mark.parametrize("cluster", [2, 4, 8])
@pytest.mark.parametrize("name", ["ewald_small_uf1", "ewald_surface_uf5", "ewald_rpm800"])
def test_cluster_sweep_reproduces_reference_log(name, cluster):
    """The reference's per-trial log (dU, acceptance) and final positions,
    with rebuilds every update_frequency accepted trials (uf 1 and 5: the
    cluster launch ends at each and the rebuild kernel takes over)."""
    g = load(name)
    p = params_of(g)
    s = gpu_system(p, g["xyz"], g["q"], g["ids"], cluster)
    assert s.cluster == min(cluster, s.max_cluster) and s.cluster > 1
    n = len(g["idx"])
    idx, disp, u = s.draw_translation_stream(int(g["seed"]), n)
    r = s.sweep(idx, disp, u)
    assert_same_chain(r["du"], r["acc"], g["du"], g["acc"], u)
    np.testing.assert_array_equal(r["acc"], g["acc"])
    np.testing.assert_allclose(s.positions(), g["final_positions"], rtol=0, atol=1e-9)
    assert r["stats"]["energy_change"] == pytest.approx(float(g["u_move_sum"]), abs=1e-5)
    assert r["stats"]["error_flags"] == 0


@pytest.mark.parametrize("cluster", [8, 16])
def test_cluster_rpm16k_matches_oracle_and_one_cta(cluster):
    """16384 ions with a cell list (K = 2242): 2000 trials on the cluster
    against the FP64 oracle, and the same stream on one CTA: same chain, same
    integer Q(k), and a rebuild from scratch reproduces the cluster's Q(k)."""
    p, xyz, q, ids = workloads.rpm16k(seed=5, update_frequency=1000)
    s = gpu_system(p, xyz, q, ids, cluster)
    if s.max_cluster < cluster:
        pytest.skip("the device co-schedules at most %d CTAs of this kernel" % s.max_cluster)
    assert s.cluster == cluster
    one = gpu_system(p, xyz, q, ids, 1)
    assert one.cluster == 1
    o = OracleSystem(p, xyz, q, ids)
    idx, disp, u = s.draw_translation_stream(2024, 2000)
    r = s.sweep(idx, disp, u)
    r1 = one.sweep(idx, disp, u)
    ro = o.mc_run_stream(idx, disp, u)
    err = assert_same_chain(r["du"], r["acc"], ro["du"], ro["acc"], u)
    print("rpm16k cluster %d: max |dU err| %.3g" % (cluster, err.max()))
    assert_same_chain(r["du"], r["acc"], r1["du"], r1["acc"], u)
    np.testing.assert_array_equal(s.positions(), one.positions())
    np.testing.assert_allclose(s.positions(), o.positions(), rtol=0, atol=1e-9)
    np.testing.assert_array_equal(s.qk(), one.qk())
    assert s.rebuild_qk() == 0.0
    assert r["stats"]["error_flags"] == 0


@pytest.mark.parametrize("cluster", [2, 8])
def test_cluster_philox_stream_same_chain_as_one_cta(cluster):
    """A device-generated stream on 800 ions (no cell list at this size or
    with one, whichever the library picks), rebuilds every 20 accepted
    trials: the cluster and one CTA run the same chain (accepted count,
    positions and Q(k) bit for bit), which the oracle replays."""
    p, xyz, q, ids = workloads.rpm800(seed=21, update_frequency=20)
    s = gpu_system(p, xyz, q, ids, cluster)
    one = gpu_system(p, xyz, q, ids, 1)
    for sys_ in (s, one):
        sys_.stream_philox(3000, seed=99, stream_id=3)
    st = s.stream_run()
    st1 = one.stream_run()
    assert st["trials"] == st1["trials"] == 3000
    assert st["accepted"] == st1["accepted"]
    assert st["rebuilds"] == st1["rebuilds"] == st["accepted"] // 20
    np.testing.assert_array_equal(s.positions(), one.positions())
    np.testing.assert_array_equal(s.qk(), one.qk())
    # each accepted dU within TOL_DU, their rounding differences add up like
    # a random walk over the accepted trials
    assert st["energy_change"] == pytest.approx(st1["energy_change"], abs=TOL_DU * np.sqrt(st["accepted"]))
    idx, disp, u = s.stream_get(0, 3000)
    o = OracleSystem(p, xyz, q, ids)
    ro = o.mc_run_stream(idx, disp, u)
    assert st["accepted"] == int(ro["acc"].sum())
    np.testing.assert_allclose(s.positions(), o.positions(), rtol=0, atol=1e-9)
    # the running energy (start + accepted dU + rebuild corrections) against
    # a fresh FP64 total, as for a restored system
    assert abs(s.running_energy() - s.total_energy_fp64()["total"]) < 1e-3


def test_cluster_setting_is_validated():
    from beofaunus_gb300.gpu import FgError
    p, xyz, q, ids = workloads.rpm800(seed=1)
    s = gpu_system(p, xyz, q, ids, 0)
    assert s.cluster >= 1 and s.max_cluster >= s.cluster
    for bad in (3, -1, 32):
        with pytest.raises(FgError):
            s.cluster = bad
    s.cluster = 1
    assert s.cluster == 1
