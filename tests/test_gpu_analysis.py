"""Device g(r) sampling (fg_rdf_sample) against the reference's own AtomRDF
histogram of the same trajectory (tests/golden/dhlj_rdf.npz) and against
the FP64 oracle's restatement; the running energy at each sample point
against the oracle's total energy (the ensemble averages <U> and g(r) agree
sample by sample, not only within statistical error)."""
import os

import numpy as np
import pytest

from beofaunus_gb300.params import FgParams
from oracle.oracle import OracleSystem, atom_rdf_counts

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_rdf_and_energy_samples_match_reference_and_oracle():
    from beofaunus_gb300.gpu import System
    g = np.load(os.path.join(GOLDEN, "dhlj_rdf.npz"))
    p = FgParams.from_buffer_copy(g["params"].tobytes())
    p.bjerrum = float(g["bjerrum"])
    s = System(p, g["xyz"], g["q"], g["ids"])
    o = OracleSystem(p, g["xyz"], g["q"], g["ids"])
    n, N = len(g["idx"]), len(g["ids"])
    idx, disp, u = s.draw_translation_stream(int(g["seed"]), n)
    np.testing.assert_array_equal(idx, g["idx"])
    t1, t2 = (int(x) for x in g["rdf_types"])
    dr = float(g["rdf_dr"])
    n_bins = int(np.rint(g["rdf_key"].max() / dr)) + 1
    ref = np.zeros(n_bins, np.int64)
    ref[np.rint(g["rdf_key"] / dr).astype(np.int64)] = g["rdf_count"].astype(np.int64)
    hist, total = np.zeros(n_bins, np.int64), 0
    u_gpu, u_orc = [], []
    for k in range(0, n, N):
        s.sweep(idx[k:k + N], disp[k:k + N], u[k:k + N], log=False)
        o.mc_run_stream(idx[k:k + N], disp[k:k + N], u[k:k + N])
        _, t = s.rdf_sample(t1, t2, dr, n_bins, hist)
        total += t
        ho, to = atom_rdf_counts(o.positions(), g["ids"], list(p.box), t1, t2, dr, n_bins)
        assert t == to
        u_gpu.append(s.running_energy())
        u_orc.append(o.total_energy()["total"])
    np.testing.assert_array_equal(hist, ref)
    assert total == int(g["rdf_count"].sum())
    np.testing.assert_allclose(u_gpu, u_orc, rtol=0, atol=1e-6 * n)
    assert np.mean(u_gpu) == pytest.approx(np.mean(u_orc), abs=1e-6 * n)
    assert s.running_energy() == pytest.approx(float(g["u1"]), abs=1e-6 * n)


def test_rdf_large_system_matches_oracle():
    """3000-ion Ewald configuration: every like and unlike pair binned as
    the FP64 restatement bins it."""
    from beofaunus_gb300 import workloads
    from beofaunus_gb300.gpu import System
    p, xyz, q, ids = workloads.rpm_ewald(3000, 80.0, 6, seed=9, update_frequency=1000, cutoff=20.0)
    s = System(p, xyz, q, ids)
    for t1, t2 in ((0, 1), (0, 0)):
        h, t = s.rdf_sample(t1, t2, 0.25, 300)
        ho, to = atom_rdf_counts(s.positions(), ids, list(p.box), t1, t2, 0.25, 300)
        assert t == to
        np.testing.assert_array_equal(h, ho)


def test_rdf_invalid_arguments():
    from beofaunus_gb300 import workloads
    from beofaunus_gb300.gpu import FgError, System
    p, xyz, q, ids = workloads.dh_lj_salt(100, seed=1)
    s = System(p, xyz, q, ids)
    with pytest.raises(FgError):
        s.rdf_sample(0, 5, 0.1, 10)
    with pytest.raises(FgError):
        s.rdf_sample(0, 1, 0.0, 10)
    with pytest.raises(FgError):
        s.rdf_sample(0, 1, 0.1, 100000)
