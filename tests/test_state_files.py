"""State files in the reference's Space::save/load format (fg_state_read,
fg_state_write; host only): the file the reference itself wrote at the end
of its run (tests/golden/dhlj_rdf.npz, Space::save, space.h:736-764) reads
back as the run's final configuration, and files written here carry the
same records."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


def golden():
    return np.load(os.path.join(GOLDEN, "dhlj_rdf.npz"))


def tokens(text):
    head, _, rng = text.partition("randomstate")
    return [float(t) for t in head.split()], rng.split()


def test_read_reference_state(tmp_path):
    from beofaunus_gb300.gpu import read_state
    g = golden()
    path = tmp_path / "ref.state"
    path.write_bytes(bytes(g["state_text"]))
    st = read_state(path)
    np.testing.assert_allclose(st["xyz"], g["final_positions"], rtol=1e-15, atol=1e-13)
    # the reference's atom list starts with a dummy entry (species.h:493-503):
    # its first type has id 1
    np.testing.assert_array_equal(st["ids"], g["ids"] + 1)
    np.testing.assert_array_equal(st["charge"], g["q"])
    assert np.all(st["radius"] == 2.0) and np.all(st["mw"] == 1.0) and np.all(st["hydrophobic"] == 0)
    n = len(g["ids"])
    np.testing.assert_array_equal(st["groups"], [[0, n - 1, 0, 1]])   # atomic group: molsize 1
    np.testing.assert_allclose(st["box"], [46.41588833612778] * 3, rtol=1e-15)


def test_write_matches_reference_records(tmp_path):
    from beofaunus_gb300.gpu import read_state, write_state
    g = golden()
    ref = bytes(g["state_text"]).decode()
    p_ref = tmp_path / "ref.state"
    p_ref.write_text(ref)
    st = read_state(p_ref)
    p_out = tmp_path / "ours.state"
    write_state(p_out, st["box"], st["xyz"], st["charge"], st["radius"], st["mw"], st["ids"], st["hydrophobic"],
                groups=st["groups"], group_cm=st["group_cm"], rng_seed=1234)
    a, rng_a = tokens(ref)
    b, rng_b = tokens(p_out.read_text())
    assert len(a) == len(b)
    np.testing.assert_allclose(b, a, rtol=1e-15, atol=0)
    # the engine state of std::mt19937(1234), in the reference's own layout
    assert len(rng_b) == len(rng_a) and int(rng_b[0]) == 1234
    back = read_state(p_out)
    for k in ("xyz", "charge", "radius", "mw", "ids", "groups", "group_cm"):
        np.testing.assert_array_equal(back[k], st[k])


def test_dipole_records_round_trip(tmp_path):
    from beofaunus_gb300.gpu import read_state, write_state
    rng = np.random.default_rng(3)
    n = 40
    xyz = rng.uniform(-10, 10, (n, 3))
    mu = rng.normal(size=(n, 3))
    mu /= np.linalg.norm(mu, axis=1)[:, None]
    mus = rng.uniform(0, 2, n)
    ids = rng.integers(0, 3, n).astype(np.int32)
    groups = np.array([[20 * k, 20 * k + 19, 0, 20] for k in range(2)], np.int32)
    cm = rng.uniform(-5, 5, (2, 3))
    p = tmp_path / "mol.state"
    write_state(p, [20.0, 20.0, 20.0], xyz, np.zeros(n), np.full(n, 1.75), None, ids, mu_unit=mu, mu_scalar=mus,
                groups=groups, group_cm=cm)
    st = read_state(p, kind=1)
    np.testing.assert_allclose(st["xyz"], xyz, rtol=1e-15, atol=1e-14)
    np.testing.assert_allclose(st["mu_unit"], mu, rtol=1e-15, atol=1e-15)
    np.testing.assert_allclose(st["mu_scalar"], mus, rtol=1e-15)
    np.testing.assert_array_equal(st["groups"], groups)
    np.testing.assert_allclose(st["group_cm"], cm, rtol=1e-15)
    assert len(p.read_text().partition("randomstate")[0].split()) == 3 + 1 + 27 * n + 1 + 7 * 2


def test_bad_files_fail_loudly(tmp_path):
    from beofaunus_gb300.gpu import FgError, read_state
    p = tmp_path / "short.state"
    p.write_text("10 10 10\n3\n0 0 0 1 2 1 0 0\n")
    with pytest.raises(FgError):
        read_state(p)
    with pytest.raises(FgError):
        read_state(tmp_path / "missing.state")


@pytest.mark.gpu
def test_system_state_round_trip(tmp_path):
    """A device system saved in the reference format and loaded into a new
    system gives the same configuration and total energy."""
    from beofaunus_gb300 import workloads
    from beofaunus_gb300.gpu import System, read_state
    p, xyz, q, ids = workloads.dh_lj_salt(500, seed=8)
    s = System(p, xyz, q, ids)
    idx, disp, u = s.draw_translation_stream(3, 1000)
    s.sweep(idx, disp, u, log=False)
    path = tmp_path / "run.state"
    s.save_state(path)
    st = read_state(path)
    np.testing.assert_allclose(st["xyz"], s.positions(), rtol=1e-15, atol=1e-13)
    np.testing.assert_array_equal(st["ids"], ids + 1)
    t = System(p, st["xyz"], st["charge"], st["ids"] - 1)
    assert t.total_energy()["total"] == pytest.approx(s.total_energy()["total"], abs=1e-9)


def test_read_reference_dipole_state(tmp_path):
    """The DipoleParticle records the reference saved after its AtomicRotation /
    AtomicTranslation run (tests/golden/dip_fluid.npz) read back as that run's
    final positions, dipole unit vectors and scalars."""
    from beofaunus_gb300.gpu import read_state
    g = np.load(os.path.join(GOLDEN, "dip_fluid.npz"))
    path = tmp_path / "dip.state"
    path.write_bytes(bytes(g["state_text"]))
    st = read_state(path, kind=1)
    np.testing.assert_allclose(st["xyz"], g["final_positions"], rtol=1e-15, atol=1e-13)
    np.testing.assert_allclose(st["mu_unit"], g["final_mu"], rtol=1e-15, atol=1e-15)
    np.testing.assert_array_equal(st["mu_scalar"], g["mus"])
    np.testing.assert_array_equal(st["charge"], g["q"])
    np.testing.assert_array_equal(st["ids"], g["ids"] + 1)
    np.testing.assert_allclose(np.linalg.norm(st["mu_unit"], axis=1), 1.0, atol=1e-12)
