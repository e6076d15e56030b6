"""Failures made on the host, never on the GPU: bad input is refused before
any device work, a job larger than the whole server budget is refused, a
client that goes away mid-job is dropped between rounds, and in every case
the library stays usable.

Reference behaviour these replace: a NaN energy only prints a warning
(move.h:495-497) and an overlap returns pc::infty for an early reject
(energy.h:195-196); here a non-finite coordinate is an error code
(FG_ERR_INVALID) at the boundary, so nothing non-finite reaches a kernel.
"""
import numpy as np
import pytest

from beofaunus_gb300 import workloads

pytestmark = pytest.mark.gpu


def test_non_finite_coordinates_are_refused_and_the_system_stays_usable():
    from beofaunus_gb300.gpu import FgError, System
    p, x, q, ids = workloads.rpm800(seed=3)
    for v in (np.nan, np.inf, -np.inf):
        bad = x.copy()
        bad[5, 1] = v
        with pytest.raises(FgError, match="non-finite"):
            System(p, bad, q, ids)
    s = System(p, x, q, ids)
    e0 = s.total_energy()["total"]
    bad = x.copy()
    bad[11, 2] = np.nan
    with pytest.raises(FgError, match="non-finite"):
        s.set_state(bad, q, ids)
    with pytest.raises(FgError, match="non-finite"):
        s.trial_du(3, [np.inf, 0.0, 0.0])
    # nothing was changed: the next trial and the total energy are as before
    s.set_state(x, q, ids)
    du = s.trial_du(3, x[3] + 0.25)
    assert np.isfinite(du)
    s.commit(False)
    assert s.total_energy()["total"] == pytest.approx(e0, abs=1e-9)
    s.close()


def test_non_finite_molecule_and_dipole_inputs_are_refused():
    from beofaunus_gb300.gpu import DipoleSystem, FgError, MolSystem
    p, x, mu, mus, ids = workloads.dipolar_molecules(8, seed=2, box=60.0)
    bad = x.copy()
    bad[7, 0] = np.nan
    with pytest.raises(FgError, match="non-finite"):
        MolSystem(p, bad, mu, mus, ids, 20)
    p, x, mu, mus, ids, q = workloads.dipolar_fluid(n=40, seed=3, n_ions=10, terms=7, kc=4.0)
    badmu = mu.copy()
    badmu[4, 1] = np.inf
    with pytest.raises(FgError, match="non-finite"):
        DipoleSystem(p, x, badmu, mus, ids, charges=q)


def test_server_refuses_a_job_larger_than_its_whole_budget():
    from beofaunus_gb300.gpu import FgError, Server
    budget = 256 << 10    # a 20000-ion job needs about 1 MB, a 300-ion one about 60 KB
    srv = Server(budget, threads=256, round_pairs=1 << 16)
    big = workloads.dh_lj_salt(20000, seed=5)
    with pytest.raises(FgError, match="budget"):
        srv.submit(*big, 5, 1000)
    assert srv.bytes_in_use == 0
    # the server goes on serving jobs that fit
    p, x, q, t = workloads.dh_lj_salt(300, seed=6)
    jid = srv.submit(p, x, q, t, 6, 900)
    for _ in range(1000):
        srv.step()
        if srv.poll(jid)["state"] == 2:
            break
    assert srv.poll(jid)["state"] == 2
    assert srv.bytes_in_use == 0
    srv.close()


def test_cancelled_job_frees_its_memory_and_leaves_the_others_unchanged():
    """A client that goes away while its job runs: the job is dropped between
    rounds, its bytes return to the budget, and the remaining jobs finish
    with the results they have alone."""
    from beofaunus_gb300.gpu import Server
    a = (workloads.dh_lj_salt(400, seed=7), 7, 2400)
    b = (workloads.dh_lj_salt(600, seed=8), 8, 6000)

    def serve(items, cancel_after=None):
        srv = Server(1 << 30, threads=256, round_pairs=1 << 16)
        ids = [srv.submit(*sysargs, seed, n) for sysargs, seed, n in items]
        rounds = 0
        while True:
            srv.step()
            rounds += 1
            if cancel_after is not None and rounds == cancel_after:
                st = srv.poll(ids[1])
                assert st["state"] == 1 and 0 < st["trials"] < items[1][2]
                before = srv.bytes_in_use
                srv.cancel(ids[1])
                assert srv.bytes_in_use < before
                ids = ids[:1]
            if all(srv.poll(j)["state"] == 2 for j in ids):
                break
            assert rounds < 10000
        out = srv.poll(ids[0], positions=True)
        assert srv.bytes_in_use == 0
        srv.close()
        return out

    alone = serve([a])
    mixed = serve([a, b], cancel_after=2)
    np.testing.assert_array_equal(mixed["xyz"], alone["xyz"])
    assert mixed["accepted"] == alone["accepted"]
