"""Pin the point-dipole Ewald oracle: the dipole-dipole and ion-ion known
answers of the reference's unit test (unittests.cpp:131-193, values of
doi:10.1063/1.481216), and its own consistency (trial dU against whole-system
energy differences, both readings of the sum)."""
import numpy as np
import pytest

from beofaunus_gb300.params import (FG_EWALD_DIPOLE_DIPOLE, FG_EWALD_ION_DIPOLE, FG_EWALD_ION_ION,
                                    FG_MODEL_EWALD_DIPOLE, make_params)
from oracle.oracle import OracleDip, dip_stream

# Catch's default Approx epsilon, as the unit test compares
REL = 1.2e-5


def known_params(terms, quirk=0):
    types = [dict(q=1.0, sigma=0.0, eps=0.0)]
    return make_params(FG_MODEL_EWALD_DIPOLE, 10.0, 1.0, types, ewald_alpha=0.894427190999916, ewald_cutoff=5.0,
                       ewald_cutoff_k=11.0, ewald_eps_surf=1.0, ewald_update_frequency=10, ewald_terms=terms,
                       ewald_dipole_quirk=quirk)


XYZ = np.array([[0.0, 0, 0], [1, 0, 0], [0, 0, 1], [1, 0, 1]])
IDS = np.zeros(4, np.int32)


def test_known_answers_ion_ion():
    # unittests.cpp:141-173: +1 and -1 at unit distance, dipoles off
    p = known_params(FG_EWALD_ION_ION | FG_EWALD_DIPOLE_DIPOLE)
    mu = np.tile([1.0, 0, 0], (4, 1))
    s = OracleDip(p, XYZ, mu, np.zeros(4), IDS, q=np.array([1.0, -1.0, 0, 0]))
    e = s.total_energy()
    assert s.pair(0, 1, real_only=True) == pytest.approx(-0.205903210732068, rel=REL)
    assert e[2] + e[4] == pytest.approx(0.215125076289333, rel=REL)
    assert e[3] == pytest.approx(-1.009253008808064, rel=REL)
    assert e[5] == pytest.approx(-1.0000311, rel=REL)


def test_known_answers_dipole_dipole():
    # unittests.cpp:175-192: two unit dipoles along x at unit distance along x
    p = known_params(FG_EWALD_ION_ION | FG_EWALD_DIPOLE_DIPOLE)
    mu = np.tile([1.0, 0, 0], (4, 1))
    s = OracleDip(p, XYZ, mu, np.array([0.0, 0, 1, 1]), IDS, q=np.zeros(4))
    e = s.total_energy()
    assert s.pair(2, 3, real_only=True) == pytest.approx(-2.044358213791836, rel=REL)
    assert e[2] + e[4] == pytest.approx(0.582251578315622, rel=REL)
    assert e[3] == pytest.approx(-0.538268271364301, rel=REL)
    assert e[5] == pytest.approx(-2.0003749, rel=REL)


def test_quirk_drops_real_space_dipole_terms():
    # the live EwaldReal returns after its ion-ion line (ewald.h:109-110)
    p = known_params(FG_EWALD_ION_ION | FG_EWALD_DIPOLE_DIPOLE, quirk=1)
    mu = np.tile([1.0, 0, 0], (4, 1))
    s = OracleDip(p, XYZ, mu, np.array([0.0, 0, 1, 1]), IDS, q=np.zeros(4))
    assert s.pair(2, 3, real_only=True) == 0.0
    e = s.total_energy()
    assert e[2] + e[4] == pytest.approx(0.582251578315622, rel=REL)   # k space and surface as before


def random_system(n=24, box=12.0, terms=7, quirk=0, seed=3, uf=1000):
    rng = np.random.default_rng(seed)
    types = [dict(q=1.0, sigma=2.0, eps=0.3), dict(q=-1.0, sigma=2.4, eps=0.2), dict(q=1.0, sigma=2.2, eps=0.5)]
    p = make_params(FG_MODEL_EWALD_DIPOLE, box, 7.0, types, ewald_alpha=0.35, ewald_cutoff=6.0, ewald_cutoff_k=5.0,
                    ewald_eps_surf=80.0, ewald_update_frequency=uf, ewald_terms=terms, ewald_dipole_quirk=quirk)
    g = np.stack(np.meshgrid(*[np.arange(3)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    xyz = (g + 0.5) * (box / 3) - box / 2 + rng.uniform(-0.4, 0.4, (n, 3))
    mu = rng.normal(size=(n, 3))
    mu /= np.linalg.norm(mu, axis=1, keepdims=True)
    ids = (np.arange(n) % 3).astype(np.int32)
    q = np.where(ids == 1, -1.0, 1.0) * (np.arange(n) % 2)   # half the particles charged
    mus = np.where(ids == 2, 0.0, 1.3)
    return p, xyz, mu, mus, ids, q


@pytest.mark.parametrize("terms,quirk", [(7, 0), (7, 1), (5, 0), (4, 0), (3, 0)])
def test_trial_du_is_energy_difference(terms, quirk):
    p, xyz, mu, mus, ids, q = random_system(terms=terms, quirk=quirk)
    s = OracleDip(p, xyz, mu, mus, ids, q=q)
    e0 = s.total_energy()[5]
    rng = np.random.default_rng(5)
    for t in range(6):
        i = int(rng.integers(len(ids)))
        x, m = s.state()
        nx = x[i] + rng.uniform(-0.5, 0.5, 3) * (t % 2)
        nm = m[i] if t % 2 else rng.normal(size=3)
        nm = nm / np.linalg.norm(nm)
        du = s.trial_du(i, nx, nm)
        s.commit(True)
        e1 = s.total_energy()[5]
        assert du == pytest.approx(e1 - e0, abs=1e-9)
        e0 = e1


def test_stream_sum_matches_energy_change():
    p, xyz, mu, mus, ids, q = random_system(terms=7)
    s = OracleDip(p, xyz, mu, mus, ids, q=q)
    e0 = s.total_energy()[5]
    st = dip_stream(11, len(ids), 400, 0.5, 0.6, 1.5)
    r = s.run_stream(st)
    assert 0.1 < r["acc"].mean() < 0.95
    assert (st["kind"] == 1).sum() > 100 and (st["kind"] == 2).sum() > 100
    assert r["usum"] == pytest.approx(s.total_energy()[5] - e0, abs=1e-8)
    _, m = s.state()
    np.testing.assert_allclose(np.linalg.norm(m, axis=1), 1.0, atol=1e-12)   # rotations keep unit vectors


# ---------------------------------------------------------------- against the reference itself
import os  # noqa: E402

from beofaunus_gb300.params import FgParams  # noqa: E402
from conftest import GOLDEN  # noqa: E402

DIP_CASES = ["dip_fluid", "dip_mixture", "dip_mixture_id"]


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def test_known_answers_live_reference():
    # the reference's live code on the unit test's configurations: ion-ion as
    # published; dipole-dipole without its real-space term (ewald.h:109-110)
    g = load("dip_known")
    for quirk, dd_real in ((1, 0.0), (0, -2.044358213791836)):
        p = known_params(FG_EWALD_ION_ION | FG_EWALD_DIPOLE_DIPOLE, quirk=quirk)
        mu = np.tile([1.0, 0, 0], (4, 1))
        s = OracleDip(p, XYZ, mu, np.zeros(4), IDS, q=np.array([1.0, -1.0, 0, 0]))
        e = s.total_energy()
        assert s.pair(0, 1, real_only=True) == pytest.approx(float(g["ii_real"][0]), rel=1e-13)
        assert e[2] + e[4] == pytest.approx(float(g["ii_recip_surf"][0]), rel=1e-12)
        assert e[3] == pytest.approx(float(g["ii_self"][0]), rel=1e-13)
        assert e[5] == pytest.approx(float(g["ii_total"][0]), rel=1e-12)
        s = OracleDip(p, XYZ, mu, np.array([0.0, 0, 1, 1]), IDS, q=np.zeros(4))
        e = s.total_energy()
        assert s.pair(2, 3, real_only=True) == pytest.approx(dd_real, rel=1e-12)
        assert e[2] + e[4] == pytest.approx(float(g["dd_recip_surf"][0]), rel=1e-12)
        assert e[3] == pytest.approx(float(g["dd_self"][0]), rel=1e-13)
        if quirk:
            assert e[5] == pytest.approx(float(g["dd_total"][0]), rel=1e-11)


def dip_case(name, quirk=1):
    g = load(name)
    p = FgParams.from_buffer_copy(g["params"].tobytes())
    p.bjerrum = float(g["bjerrum"])
    p.ewald_dipole_quirk = quirk
    return g, p


@pytest.mark.parametrize("name", DIP_CASES)
def test_reference_log_replay(name):
    """AtomicRotation / AtomicTranslation trials logged by the reference,
    replayed through the oracle's live-code reading: every dU, the final
    energy and the sum of accepted dU."""
    g, p = dip_case(name)
    s = OracleDip(p, g["xyz"], g["mu"], g["mus"], g["ids"], q=g["q"])
    assert s.total_energy()[5] == pytest.approx(float(g["u0"]), abs=1e-9)
    usum = 0.0
    for t in range(len(g["idx"])):
        du = s.trial_du(int(g["idx"][t]), g["trial_xyz"][t], g["trial_mu"][t])
        assert du == pytest.approx(float(g["du"][t]), abs=1e-9), t
        s.commit(bool(g["acc"][t]))
        if g["acc"][t]:
            usum += du
    assert s.total_energy()[5] == pytest.approx(float(g["u1"]), abs=1e-8)
    assert usum == pytest.approx(float(g["u_move_sum"]), abs=1e-8)
    assert {1, 2} <= set(np.unique(g["kind"]).tolist())


@pytest.mark.parametrize("name", DIP_CASES)
def test_reference_stream_rerun(name):
    """The reference's own draws regenerated (particle, ranunit axis and angle,
    displacement, Metropolis uniform) and run through the oracle: the same
    trials, dU and decisions as the reference's log."""
    g, p = dip_case(name)
    s = OracleDip(p, g["xyz"], g["mu"], g["mus"], g["ids"], q=g["q"])
    n = len(g["idx"])
    st = dip_stream(int(g["seed"]), len(g["ids"]), n, 0.0, float(p.type_dp[0]), float(g["dprot"]), kinds=g["kind"])
    np.testing.assert_array_equal(st["idx"], g["idx"])
    r = s.run_stream(st)
    np.testing.assert_allclose(r["du"], g["du"], rtol=0, atol=1e-9)
    np.testing.assert_array_equal(r["acc"], g["acc"])
    assert r["usum"] == pytest.approx(float(g["u_move_sum"]), abs=1e-8)


def _tinfoil_system(terms, quirk=0, seed=8):
    p, xyz, mu, mus, ids, q = random_system(terms=terms, quirk=quirk, seed=seed)
    p.ewald_eps_surf = 0.5   # < 1: tin-foil surroundings, no surface term
    return p, xyz, mu, mus, ids, q


@pytest.mark.parametrize("terms", [7, 5, 4])
def test_energy_invariant_under_translation(terms):
    """Periodic Ewald energy does not depend on where the box origin sits."""
    p, xyz, mu, mus, ids, q = _tinfoil_system(terms)
    e0 = OracleDip(p, xyz, mu, mus, ids, q=q).total_energy()
    L = p.box[0]
    shifted = xyz + np.array([1.37, -2.91, 0.55])
    shifted -= L * np.round(shifted / L)
    e1 = OracleDip(p, shifted, mu, mus, ids, q=q).total_energy()
    np.testing.assert_allclose(e1, e0, rtol=0, atol=1e-9)


@pytest.mark.parametrize("terms", [7, 4])
def test_energy_invariant_under_cubic_rotation(terms):
    """A 90-degree turn of positions and dipoles about z maps the cubic box,
    the real-space pairs and the spherical k-set onto themselves."""
    p, xyz, mu, mus, ids, q = _tinfoil_system(terms)
    e0 = OracleDip(p, xyz, mu, mus, ids, q=q).total_energy()
    R = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    L = p.box[0]
    x1 = xyz @ R.T
    x1 -= L * np.round(x1 / L)
    e1 = OracleDip(p, x1, mu @ R.T, mus, ids, q=q).total_energy()
    np.testing.assert_allclose(e1, e0, rtol=0, atol=1e-9)
