"""Pin the FP64 oracle against the reference: the Ewald known answers of the
reference's unit test (unittests.cpp:131-170, doi:10.1063/1.481216) and the
per-trial logs the reference itself produced (tests/golden/*.npz)."""
import os

import numpy as np
import pytest

from beofaunus_gb300.params import FG_MODEL_EWALD_WCA, FgParams, make_params
from oracle.oracle import OracleSystem, atom_rdf_counts, rdf_normalize, translation_stream

from conftest import GOLDEN

MC_CASES = ["ewald_small_uf1", "ewald_surface_uf5", "ewald_rpm800", "ewald_iso", "dhlj_small", "dhlj_500", "dhlj_rdf"]


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def params_of(g):
    p = FgParams.from_buffer_copy(g["params"].tobytes())
    p.bjerrum = float(g["bjerrum"])  # the exact lB the reference computed from epsr
    return p


def known_system():
    g = load("ewald_known")
    lB = float(g["bjerrum"][0])
    types = [dict(q=1.0, sigma=0.0, eps=0.0), dict(q=-1.0, sigma=0.0, eps=0.0)]
    p = make_params(FG_MODEL_EWALD_WCA, 10.0, lB, types, ewald_alpha=0.894427190999916, ewald_cutoff=5.0,
                    ewald_cutoff_k=11.0, ewald_eps_surf=1.0, ewald_update_frequency=10)
    xyz = np.array([[0.5, 0, 0], [1, 0, 0], [0, 0, 1], [1, 0, 1]], dtype=np.float64)
    ids = np.array([0, 1, 0, 0], dtype=np.int32)
    q = np.array([1.0, -1.0, 0.0, 0.0])
    s = OracleSystem(p, xyz, q, ids)
    # the unit test's incremental round trip: particle 0 back to the origin
    s.trial_du([0], [[0.0, 0.0, 0.0]])
    s.commit(True)
    return s, g, lB


def test_ewald_known_answers_published():
    s, g, lB = known_system()
    e = s.total_energy()
    # published values (units of lB) carried by the reference's unit test;
    # tolerance = Catch's default Approx epsilon used there
    assert e["pairs"] / lB == pytest.approx(-0.205903210732068, rel=1.2e-5)
    assert (e["reciprocal"] + e["surface"]) / lB == pytest.approx(0.215125076289333, rel=1.2e-5)
    assert e["self"] / lB == pytest.approx(-1.009253008808064, rel=1.2e-5)
    assert e["total"] / lB == pytest.approx(-1.0000311, rel=1.2e-5)


def test_ewald_known_answers_match_reference_build():
    s, g, lB = known_system()
    e = s.total_energy()
    assert e["pairs"] == pytest.approx(float(g["real"][0]), rel=1e-13)
    assert e["reciprocal"] + e["surface"] == pytest.approx(float(g["recip_surf"][0]), rel=1e-12)
    assert e["self"] == pytest.approx(float(g["self"][0]), rel=1e-13)
    assert e["total"] == pytest.approx(float(g["total"][0]), rel=1e-12)


@pytest.mark.parametrize("name", MC_CASES)
def test_mc_run_matches_reference_log(name):
    g = load(name)
    p = params_of(g)
    s = OracleSystem(p, g["xyz"], g["q"], g["ids"])
    e0 = s.total_energy()["total"]
    assert e0 == pytest.approx(float(g["u0"]), abs=1e-9)
    n = len(g["idx"])
    r = s.mc_run(int(g["seed"]), n)
    np.testing.assert_array_equal(r["idx"], g["idx"])
    np.testing.assert_allclose(r["trial_xyz"], g["trial_xyz"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(r["du"], g["du"], rtol=0, atol=1e-9)
    np.testing.assert_array_equal(r["acc"], g["acc"])
    assert r["utot"] == pytest.approx(float(g["u_move_sum"]), abs=1e-8)
    np.testing.assert_allclose(s.positions(), g["final_positions"], rtol=0, atol=1e-12)
    assert s.total_energy()["total"] == pytest.approx(float(g["u1"]), abs=1e-8)


@pytest.mark.parametrize("name", ["ewald_small_uf1", "dhlj_small"])
def test_translation_stream_matches_reference_draws(name):
    """The host-side replay of the reference's RNG calls gives the same
    particle indices the reference picked."""
    g = load(name)
    p = params_of(g)
    n = len(g["idx"])
    dpp = np.array([p.type_dp[i] for i in g["ids"]])
    idx, disp, u = translation_stream(int(g["seed"]), dpp, n)
    np.testing.assert_array_equal(idx, g["idx"])


def rdf_bins(g, n_bins):
    """The reference's AtomRDF keys (bin centres b dr) as bin counts."""
    counts = np.zeros(n_bins, np.int64)
    b = np.rint(g["rdf_key"] / float(g["rdf_dr"])).astype(np.int64)
    counts[b] = g["rdf_count"].astype(np.int64)
    return counts


def test_rdf_matches_reference_analysis():
    """AtomRDF (analysis.h:2116-2134) sampled by the reference after each
    sweep of its own run: the oracle's restatement over the same trajectory
    gives the same counts, and the normalised g(r) follows from them."""
    g = load("dhlj_rdf")
    p = params_of(g)
    s = OracleSystem(p, g["xyz"], g["q"], g["ids"])
    n, N = len(g["idx"]), len(g["ids"])
    dpp = np.array([p.type_dp[i] for i in g["ids"]])
    idx, disp, u = translation_stream(int(g["seed"]), dpp, n)
    t1, t2 = (int(x) for x in g["rdf_types"])
    dr = float(g["rdf_dr"])
    n_bins = int(np.rint(g["rdf_key"].max() / dr)) + 1
    hist, total = np.zeros(n_bins, np.int64), 0
    for k in range(0, n, N):
        s.mc_run_stream(idx[k:k + N], disp[k:k + N], u[k:k + N])
        h, t = atom_rdf_counts(s.positions(), g["ids"], list(p.box), t1, t2, dr, n_bins)
        hist += h
        total += t
    np.testing.assert_array_equal(hist, rdf_bins(g, n_bins))
    assert total == int(g["rdf_count"].sum())
    gr = rdf_normalize(hist, total, float(g["rdf_volume"]), dr)
    assert np.all(np.isfinite(gr[1:])) and gr[-1] > 0


@pytest.mark.parametrize("name", ["iso_dhlj", "iso_ewald"])
def test_volume_moves_match_reference_log(name):
    """Move::Isobaric with ExternalPressure run by the reference itself
    (tests/golden/iso_*.npz): the oracle's restatement, fed the same global
    slump() draws (half, then the Metropolis uniform per move), gives the
    same dU, decisions, volumes and final positions. Ewald: with the
    reference's trial reciprocal term (the unscaled positions' structure
    factor in the new box); the physically scaled term differs from it."""
    from oracle.oracle import MILLIMOLAR, slump_uniforms, volume_move
    g = load(name)
    p = params_of(g)
    x, q, ids = g["xyz"], g["q"], g["ids"]
    moves = int(g["moves"])
    u = slump_uniforms(int(g["seed"]), 2 * moves)
    P = float(g["pressure_mM"]) * MILLIMOLAR
    assert np.prod(p.box[:3]) == pytest.approx(float(g["v0"]), rel=1e-14)
    for m in range(moves):
        quirk = p.model == FG_MODEL_EWALD_WCA
        du, acc, p, x = volume_move(p, x, q, ids, u[2 * m] - 0.5, float(g["volume_dp"]), P, u[2 * m + 1],
                                    reference_quirk=quirk)
        assert du == pytest.approx(float(g["du"][m]), abs=1e-9), m
        if quirk and m == 0:
            plain = volume_move(params_of(g), g["xyz"], q, ids, u[0] - 0.5, float(g["volume_dp"]), P, u[1])[0]
            assert abs(plain - du) > 1e-3   # the quirk is not a rounding effect
        assert acc == bool(g["acc"][m]), m
        assert np.prod(p.box[:3]) == pytest.approx(float(g["volume"][m]), rel=1e-13), m
    np.testing.assert_allclose(x, g["final_positions"], rtol=0, atol=1e-10)
