"""Rigid dipolar molecules through the C-ABI (fg_mol_*) against the
reference's own runs (tests/golden/mol_*.npz) and the FP64 oracle.

Tolerance: every trial's dU within 1e-6 kT of the FP64 reference/oracle."""
import os

import numpy as np
import pytest

from beofaunus_gb300 import workloads
from beofaunus_gb300.gpu import MolSystem, mol_draw_stream
from beofaunus_gb300.params import FgParams
from oracle.oracle import OracleMol

from conftest import GOLDEN

TOL_DU = 1e-6


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def golden_system(g, cluster=0):
    p = FgParams.from_buffer_copy(g["params"].tobytes())
    return p, MolSystem(p, g["xyz"], g["mu"], g["mus"], g["ids"], 20, mass_centers=g["cm0"], cluster=cluster)


def test_mol_draws_match_reference():
    """Host replay of the reference's RNG calls picks the same molecules."""
    for name in ["mol_small", "mol_endrot", "mol_125"]:
        g = load(name)
        n = len(g["group"])
        st = mol_draw_stream(int(g["seed"]), len(g["ids"]) // 20, n, float(g["dp"]), float(g["dprot"]),
                             bool(g["center_rotation"]))
        np.testing.assert_array_equal(st["group"], g["group"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["mol_small", "mol_endrot", "mol_125"])
def test_mol_sweep_matches_reference_log(name):
    g = load(name)
    p, s = golden_system(g)
    n = len(g["group"])
    st = mol_draw_stream(int(g["seed"]), s.m, n, float(g["dp"]), float(g["dprot"]), bool(g["center_rotation"]))
    e0 = s.total_energy()
    assert e0[2] == pytest.approx(float(g["u0"]), rel=1e-9)
    r = s.sweep(st)
    err = np.abs(r["du"] - g["du"])
    assert err.max() < TOL_DU, (err.max(), int(err.argmax()))
    np.testing.assert_array_equal(r["acc"], g["acc"])
    xyz, mu, cm = s.state()
    L = p.box[0]
    dx = xyz - g["final_positions"]
    dx -= L * np.round(dx / L)
    assert np.abs(dx).max() < 1e-9
    assert np.abs(mu - g["final_mu"]).max() < 1e-12
    dc = cm - g["final_cm"]
    dc -= L * np.round(dc / L)
    assert np.abs(dc).max() < 1e-9
    e1 = s.total_energy()
    assert e1[2] == pytest.approx(float(g["u1"]), rel=1e-9)
    assert s.running_energy() == pytest.approx(float(g["u1"]), rel=1e-9)


@pytest.mark.gpu
def test_mol_cluster_sizes_agree():
    g = load("mol_125")
    n = len(g["group"])
    res = []
    p, s = golden_system(g)
    cmax = s.max_cluster
    s.close()
    for c in [1, 2, 4, 8]:
        if c > cmax:
            continue
        p, s = golden_system(g, cluster=c)
        assert s.cluster == c
        st = mol_draw_stream(int(g["seed"]), s.m, n, 1.0, 0.3, True)
        r = s.sweep(st)
        assert np.abs(r["du"] - g["du"]).max() < TOL_DU
        res.append(r["acc"])
        s.close()
    for a in res[1:]:
        np.testing.assert_array_equal(a, res[0])


@pytest.mark.gpu
def test_mol_explicit_trial_matches_oracle():
    """The plain per-trial path (host-computed trial coordinates)."""
    p, xyz, mu, mus, ids = workloads.dipolar_molecules(60, seed=31)
    s = MolSystem(p, xyz, mu, mus, ids, 20)
    o = OracleMol(p, xyz, mu, mus, ids, 20)
    rng = np.random.default_rng(4)
    L = p.box[0]
    cur, curmu = xyz.copy(), mu.copy()
    for t in range(40):
        g = int(rng.integers(0, 60))
        sl = slice(20 * g, 20 * g + 20)
        ang = rng.normal(size=3) * 0.1
        th = np.linalg.norm(ang)
        k = ang / th
        K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
        R = np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * K @ K
        c = cur[sl][9]
        off = cur[sl] - c
        off -= L * np.round(off / L)
        new = c + off @ R.T + rng.uniform(-0.5, 0.5, 3)
        new -= L * np.round(new / L)
        newmu = curmu[sl] @ R.T
        du = s.trial_du(g, new, newmu)
        du_o = o.trial_du(g, new, newmu)
        assert abs(du - du_o) < TOL_DU, (t, du, du_o)
        acc = bool(rng.random() < 0.6)
        s.commit(acc)
        o.commit(acc)
        if acc:
            cur[sl], curmu[sl] = new, newmu
    x1, m1, _ = s.state()
    d = x1 - cur
    d -= L * np.round(d / L)
    assert np.abs(d).max() < 1e-9
    assert s.total_energy()[2] == pytest.approx(o.total_energy()[2], rel=1e-9)


@pytest.mark.gpu
def test_mol_full_size_against_oracle():
    """1000 rigid 20-site dipolar molecules, L = 150, rc = 15: a stream of
    the reference's draws on the device, checked trial by trial."""
    p, xyz, mu, mus, ids = workloads.dipolar_molecules(1000, seed=41)
    s = MolSystem(p, xyz, mu, mus, ids, 20)
    o = OracleMol(p, xyz, mu, mus, ids, 20)
    st = mol_draw_stream(5489, 1000, 150, 1.0, 0.3, True)
    r = s.sweep(st)
    ro = o.run_stream(st)
    err = np.abs(r["du"] - ro["du"])
    assert err.max() < TOL_DU, (err.max(), int(err.argmax()))
    np.testing.assert_array_equal(r["acc"], ro["acc"])
    assert s.running_energy() - s.total_energy()[2] == pytest.approx(0.0, abs=1e-6 * 150)


@pytest.mark.gpu
def test_mol_invalid_arguments():
    from beofaunus_gb300.gpu import FgError
    p, xyz, mu, mus, ids = workloads.dipolar_molecules(10, seed=3)
    s = MolSystem(p, xyz, mu, mus, ids, 20)
    with pytest.raises(FgError):
        s.trial_du(10, xyz[:20])
    with pytest.raises(FgError):
        s.commit(True)   # nothing pending
    with pytest.raises(FgError):
        s.cluster = 3
    from beofaunus_gb300.gpu import mol_draw_stream, mol_run_many
    s.stream_upload(mol_draw_stream(1, 10, 8, 1.0, 0.3, True))
    with pytest.raises(FgError):
        s.trial_du(0, xyz[:20])   # the staged stream would be overwritten
    mol_run_many([s])
    s.trial_du(0, xyz[:20])         # allowed once the stream has run
    s.commit(False)


@pytest.mark.gpu
def test_mol_run_many_equals_alone():
    """Independent systems in one launch end exactly where each ends alone."""
    from beofaunus_gb300.gpu import mol_run_many
    data = [workloads.dipolar_molecules(50, seed=s) for s in (61, 62, 63)]
    alone = []
    for k, (p, xyz, mu, mus, ids) in enumerate(data):
        s = MolSystem(p, xyz, mu, mus, ids, 20, cluster=2)
        s.sweep(mol_draw_stream(300 + k, 50, 400, 1.0, 0.3, True), log=False)
        alone.append(s.state())
        s.close()
    many = [MolSystem(p, xyz, mu, mus, ids, 20, cluster=2) for (p, xyz, mu, mus, ids) in data]
    for k, s in enumerate(many):
        s.stream_upload(mol_draw_stream(300 + k, 50, 400, 1.0, 0.3, True))
    per, tot = mol_run_many(many)
    assert tot["trials"] == 1200
    for k, s in enumerate(many):
        for a, b in zip(s.state(), alone[k]):
            np.testing.assert_array_equal(a, b)
