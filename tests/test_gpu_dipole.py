"""Point dipoles under Ewald on the GPU (fg_dip_*) against the FP64 oracle
and the reference's own logs: AtomicRotation / AtomicTranslation trial by
trial (dU within 1e-9 kT, identical decisions), the published Ewald known
answers, the plain trial/commit API, batched launches and Q(k) rebuilds."""
import os

import numpy as np
import pytest

from beofaunus_gb300.params import FG_MODEL_EWALD_DIPOLE, FgParams, make_params
from beofaunus_gb300 import workloads
from oracle.oracle import OracleDip

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

DU_TOL = 1e-9   # kT, per trial


def gpu():
    from beofaunus_gb300 import gpu as g
    return g


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def dip_case(name, quirk=1):
    g = load(name)
    p = FgParams.from_buffer_copy(g["params"].tobytes())
    p.bjerrum = float(g["bjerrum"])
    p.ewald_dipole_quirk = quirk
    return g, p


def agree(du_a, acc_a, du_b, acc_b, u=None):
    np.testing.assert_allclose(du_a, du_b, rtol=0, atol=DU_TOL)
    bad = np.nonzero(acc_a != acc_b)[0]
    if u is not None:
        # a decision may differ only where u sits on exp(-dU) within the dU tolerance
        for t in bad:
            assert abs(np.log(u[t]) + du_b[t]) < 1e-8, t
    else:
        assert len(bad) == 0


@pytest.mark.parametrize("name", ["dip_fluid", "dip_mixture", "dip_mixture_id"])
def test_reference_stream(name):
    """The reference's own trials (regenerated draws) through fg_dip_sweep:
    dU and decisions as the reference logged them."""
    G = gpu()
    g, p = dip_case(name)
    s = G.DipoleSystem(p, g["xyz"], g["mu"], g["mus"], g["ids"], charges=g["q"])
    assert s.total_energy()[5] == pytest.approx(float(g["u0"]), abs=1e-9)
    st = G.dip_draw_stream(int(g["seed"]), len(g["ids"]), len(g["idx"]), dp=float(p.type_dp[0]),
                           dprot=float(g["dprot"]), kinds=g["kind"])
    np.testing.assert_array_equal(st["idx"], g["idx"])
    r = s.sweep(st)
    agree(r["du"], r["acc"], g["du"], g["acc"])
    assert r["energy_change"] == pytest.approx(float(g["u_move_sum"]), abs=1e-8)
    assert s.total_energy()[5] == pytest.approx(float(g["u1"]), abs=1e-8)
    assert s.running_energy() == pytest.approx(float(g["u1"]), abs=1e-8)


def known(terms_quirk, charges, mus):
    G = gpu()
    terms, quirk = terms_quirk
    p = make_params(FG_MODEL_EWALD_DIPOLE, 10.0, 1.0, [dict(q=1.0, sigma=0.0, eps=0.0)],
                    ewald_alpha=0.894427190999916, ewald_cutoff=5.0, ewald_cutoff_k=11.0, ewald_eps_surf=1.0,
                    ewald_update_frequency=10, ewald_terms=terms, ewald_dipole_quirk=quirk)
    xyz = np.array([[0.0, 0, 0], [1, 0, 0], [0, 0, 1], [1, 0, 1]])
    return G.DipoleSystem(p, xyz, np.tile([1.0, 0, 0], (4, 1)), np.array(mus), np.zeros(4, np.int32),
                          charges=np.array(charges))


def test_known_answers():
    # unittests.cpp:131-193 (doi:10.1063/1.481216), units of lB; Catch's Approx epsilon
    e = known((5, 0), [1.0, -1.0, 0, 0], [0.0, 0, 0, 0]).total_energy()
    assert e[0] == pytest.approx(-0.205903210732068, rel=1.2e-5)
    assert e[2] + e[4] == pytest.approx(0.215125076289333, rel=1.2e-5)
    assert e[3] == pytest.approx(-1.009253008808064, rel=1.2e-5)
    assert e[5] == pytest.approx(-1.0000311, rel=1.2e-5)
    e = known((5, 0), [0.0, 0, 0, 0], [0.0, 0, 1, 1]).total_energy()
    assert e[0] == pytest.approx(-2.044358213791836, rel=1.2e-5)
    assert e[2] + e[4] == pytest.approx(0.582251578315622, rel=1.2e-5)
    assert e[3] == pytest.approx(-0.538268271364301, rel=1.2e-5)
    assert e[5] == pytest.approx(-2.0003749, rel=1.2e-5)
    # the reference's live code on the same configuration
    g = load("dip_known")
    e = known((5, 1), [0.0, 0, 0, 0], [0.0, 0, 1, 1]).total_energy()
    assert e[0] == 0.0
    assert e[5] == pytest.approx(float(g["dd_total"][0]), rel=1e-11)


def fluid(terms=7, quirk=0, n=120, n_ions=40, seed=9, uf=1000, kc=6.0):
    p, xyz, mu, mus, ids, q = workloads.dipolar_fluid(n=n, seed=seed, n_ions=n_ions, terms=terms, quirk=quirk,
                                                      kc=kc, update_frequency=uf)
    p.bjerrum = 60.0
    return p, xyz, mu, mus, ids, q


@pytest.mark.parametrize("terms,quirk", [(7, 0), (7, 1), (4, 0), (3, 0)])
def test_stream_against_oracle(terms, quirk):
    G = gpu()
    p, xyz, mu, mus, ids, q = fluid(terms=terms, quirk=quirk, uf=50)
    s = G.DipoleSystem(p, xyz, mu, mus, ids, charges=q)
    o = OracleDip(p, xyz, mu, mus, ids, q=q)
    assert s.total_energy() == pytest.approx(o.total_energy(), abs=1e-8)
    st = G.dip_draw_stream(17 + terms, len(ids), 3000, p_rotate=0.5, dp=0.7, dprot=2.0)
    r = s.sweep(st)
    ro = o.run_stream(st)
    agree(r["du"], r["acc"], ro["du"], ro["acc"], st["u"])
    assert 0.2 < r["acc"].mean() < 0.9
    assert r["rebuilds"] == r["accepted"] // 50
    x, m = s.state()
    xo, mo = o.state()
    np.testing.assert_allclose(m, mo, rtol=0, atol=1e-12)
    d = x - xo
    d -= p.box[0] * np.round(d / p.box[0])
    assert np.abs(d).max() < 1e-9
    assert s.total_energy()[5] == pytest.approx(o.total_energy()[5], abs=1e-7)
    assert s.running_energy() == pytest.approx(s.total_energy()[5], abs=1e-7)


def test_plain_trial_commit():
    G = gpu()
    p, xyz, mu, mus, ids, q = fluid(uf=4)
    s = G.DipoleSystem(p, xyz, mu, mus, ids, charges=q)
    o = OracleDip(p, xyz, mu, mus, ids, q=q)
    rng = np.random.default_rng(2)
    for t in range(40):
        i = int(rng.integers(len(ids)))
        x, m = o.state()
        nx = x[i] + (rng.uniform(-0.6, 0.6, 3) if t % 2 else 0.0)
        nm = rng.normal(size=3) if t % 3 == 0 else m[i]
        nm = nm / np.linalg.norm(nm)
        du = s.trial_du(i, nx, nm)
        assert du == pytest.approx(o.trial_du(i, nx, nm), abs=DU_TOL)
        acc = bool(t % 4)
        c = s.commit(acc)
        assert c == pytest.approx(o.commit(acc), abs=1e-9)
    assert s.total_energy()[5] == pytest.approx(o.total_energy()[5], abs=1e-8)


def test_run_many_matches_single_systems():
    G = gpu()
    systems, singles, streams = [], [], []
    for k in range(6):
        p, xyz, mu, mus, ids, q = fluid(n=60 + 20 * k, n_ions=10 * k, seed=30 + k, uf=40)
        st = G.dip_draw_stream(100 + k, len(ids), 500 + 100 * k, p_rotate=0.5, dp=0.7, dprot=2.0)
        a = G.DipoleSystem(p, xyz, mu, mus, ids, charges=q)
        a.stream_upload(st)
        systems.append(a)
        b = G.DipoleSystem(p, xyz, mu, mus, ids, charges=q)
        singles.append(b.sweep(st))
        streams.append(st)
    per, tot = G.dip_run_many(systems)
    assert tot["trials"] == sum(len(st["idx"]) for st in streams)
    for k in range(6):
        assert per[k]["trials"] == len(streams[k]["idx"])
        assert per[k]["accepted"] == singles[k]["accepted"]
        assert per[k]["energy_change"] == singles[k]["energy_change"]   # same block size: same sums


def test_invalid_arguments():
    G = gpu()
    p, xyz, mu, mus, ids, q = fluid(n=20, n_ions=0)
    s = G.DipoleSystem(p, xyz, mu, mus, ids, charges=q)
    with pytest.raises(G.FgError):
        s.commit(True)   # nothing pending
    s.stream_upload(G.dip_draw_stream(2, 20, 5))
    with pytest.raises(G.FgError):
        s.trial_du(0, xyz[0], mu[0])   # the staged stream would be overwritten
    G.dip_run_many([s])
    st = G.dip_draw_stream(1, 20, 10)
    st["kind"][3] = 7
    with pytest.raises(G.FgError):
        s.sweep(st)
    bad = make_params(FG_MODEL_EWALD_DIPOLE, 10.0, 1.0, [dict(q=1.0, sigma=1.0, eps=0.1)], ewald_alpha=0.3,
                      ewald_cutoff=4.0, ewald_cutoff_k=40.0, ewald_terms=4)
    with pytest.raises(G.FgError):
        G.DipoleSystem(bad, xyz[:4], mu[:4], mus[:4], ids[:4])


def test_large_system_unstaged():
    """3000 particles: the sweep's arrays exceed the shared-memory staging
    limit, so the launch reads them from global memory; the near-pair queue
    spans many iterations per warp."""
    G = gpu()
    p, xyz, mu, mus, ids, q = workloads.dipolar_fluid(n=3000, seed=41, n_ions=600, terms=7, kc=5.0,
                                                      update_frequency=30)
    p.bjerrum = 60.0
    s = G.DipoleSystem(p, xyz, mu, mus, ids, charges=q)
    o = OracleDip(p, xyz, mu, mus, ids, q=q)
    st = G.dip_draw_stream(77, 3000, 300, p_rotate=0.5, dp=0.7, dprot=2.0)
    r = s.sweep(st)
    ro = o.run_stream(st)
    agree(r["du"], r["acc"], ro["du"], ro["acc"], st["u"])
    assert r["accepted"] > 30
    assert s.total_energy()[5] == pytest.approx(o.total_energy()[5], abs=1e-7)


@pytest.mark.parametrize("case", ["stockmayer_input", "two_particles", "no_dipoles"])
def test_edge_cases(case):
    """The reference's Stockmayer input as written (useDipoleDipole only, the
    live code, cutoffK 0: no k-vectors), the smallest system, and a system
    whose dipoles are all zero."""
    G = gpu()
    if case == "stockmayer_input":
        p, xyz, mu, mus, ids, q = workloads.dipolar_fluid(n=100, seed=5, kc=0.0, terms=4, quirk=1)
        dprot = 270.0 * np.pi / 180.0
    elif case == "two_particles":
        p, xyz, mu, mus, ids, q = workloads.dipolar_fluid(n=2, seed=6, box=8.0, kc=3.0, terms=7, n_ions=1)
        p.bjerrum = 60.0
        dprot = 2.0
    else:
        p, xyz, mu, mus, ids, q = workloads.dipolar_fluid(n=80, seed=7, kc=4.0, terms=7, n_ions=80)
        p.bjerrum = 20.0
        dprot = 2.0
    s = G.DipoleSystem(p, xyz, mu, mus, ids, charges=q)
    o = OracleDip(p, xyz, mu, mus, ids, q=q)
    assert s.num_kvectors == o.num_kvectors
    if case == "stockmayer_input":
        assert s.num_kvectors == 0
    assert s.total_energy() == pytest.approx(o.total_energy(), abs=1e-8)
    st = G.dip_draw_stream(3, len(ids), 1000, p_rotate=0.5, dp=0.7, dprot=dprot)
    r = s.sweep(st)
    ro = o.run_stream(st)
    agree(r["du"], r["acc"], ro["du"], ro["acc"], st["u"])
    assert r["accepted"] > 0


def test_translation_and_rotation_invariance():
    """With tin-foil surroundings the device energies and every trial's dU are
    the same for the system shifted through the box or turned by 90 degrees
    about z (the cubic box, the pairs and the spherical k-set map onto
    themselves)."""
    G = gpu()
    p, xyz, mu, mus, ids, q = fluid(n=90, n_ions=30, seed=12)
    p.ewald_eps_surf = 0.5
    L = p.box[0]
    R = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    variants = [(xyz, mu), (xyz + np.array([2.3, -1.1, 4.7]), mu), (xyz @ R.T, mu @ R.T)]
    st = G.dip_draw_stream(8, len(ids), 600, p_rotate=0.5, dp=0.7, dprot=2.0)
    energies, dus = [], []
    for k, (x, m) in enumerate(variants):
        x = x - L * np.round(x / L)
        s = G.DipoleSystem(p, x, m, mus, ids, charges=q)
        energies.append(s.total_energy()[5])
        sk = dict(st)
        if k == 2:   # the same moves, turned with the system
            sk["axis"] = st["axis"] @ R.T
            sk["disp"] = st["disp"] @ R.T
        dus.append(s.sweep(sk)["du"])
    for e, d in zip(energies[1:], dus[1:]):
        assert e == pytest.approx(energies[0], abs=1e-8)
        np.testing.assert_allclose(d, dus[0], rtol=0, atol=1e-8)
