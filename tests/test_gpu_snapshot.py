"""Snapshots (fg_snapshot / fg_restore, fg_server_snapshot / fg_server_resume):
a run stopped and resumed from a snapshot continues exactly as the run that
never stopped, bit for bit.

The reference's counterparts are Space::save/load (space.h:376-377) and the
random state it writes to move_out.json (slump.h:111-124) without reading it
back; a resumed reference run therefore does not continue its random stream.
Here the comparison is against our own uninterrupted run, so every check is
exact equality (dU, decisions, positions, Q(k), running energy)."""
import numpy as np
import pytest

from beofaunus_gb300 import workloads

pytestmark = pytest.mark.gpu


def _systems():
    return {
        # Ewald, cell list, rebuild every 40 accepted trials (the snapshot
        # falls between two rebuilds: the accept counter must carry over)
        "ewald_cells": workloads.rpm_ewald(1500, 70.0, 6, seed=3, update_frequency=40, cutoff=14.0,
                                           use_cell_list=1),
        # Ewald, all pairs, with a surface term
        "ewald_surface": workloads.rpm_ewald(400, 40.0, 5, seed=4, update_frequency=25, cutoff=14.0,
                                             eps_surf=80.0),
        "dhlj": workloads.dh_lj_salt(600, seed=5),
    }


@pytest.mark.parametrize("name", ["ewald_cells", "ewald_surface", "dhlj"])
def test_restored_system_continues_bit_for_bit(name):
    from beofaunus_gb300.gpu import System
    p, xyz, q, ids = _systems()[name]
    a = System(p, xyz, q, ids)
    st1 = a.draw_translation_stream(11, 3001)
    a.sweep(*st1, log=False)
    blob = a.snapshot()
    st2 = a.draw_translation_stream(12, 4000)
    ra = a.sweep(*st2)
    b = System.from_snapshot(blob)
    rb = b.sweep(*st2)
    np.testing.assert_array_equal(rb["du"], ra["du"])
    np.testing.assert_array_equal(rb["acc"], ra["acc"])
    assert rb["stats"]["rebuilds"] == ra["stats"]["rebuilds"]
    np.testing.assert_array_equal(b.positions(), a.positions())
    if a.num_kvectors:
        assert ra["stats"]["rebuilds"] > 0
        np.testing.assert_array_equal(b.qk(), a.qk())
    assert b.running_energy() == a.running_energy()
    # the restored system's own bookkeeping agrees with a fresh FP64 total
    e64 = b.total_energy_fp64()["total"]
    assert abs(b.running_energy() - e64) < 1e-3
    # a snapshot of the restored system equals one of the original
    assert b.snapshot() == a.snapshot()
    a.close()
    b.close()


def test_restore_into_an_existing_system_and_device_streams():
    """fg_restore into a live system (same parameters) rewinds it; Philox
    streams drawn on the device run identically afterwards."""
    from beofaunus_gb300.gpu import System
    p, xyz, q, ids = _systems()["ewald_cells"]
    a = System(p, xyz, q, ids)
    blob = a.snapshot()
    a.stream_philox(5000, 21)
    r1 = a.stream_run()
    x1, q1, e1 = a.positions(), a.qk(), a.running_energy()
    a.restore(blob)
    np.testing.assert_array_equal(a.positions(), System.from_snapshot(blob).positions())
    a.stream_philox(5000, 21)
    r2 = a.stream_run()
    assert r2["accepted"] == r1["accepted"] and r2["rebuilds"] == r1["rebuilds"]
    np.testing.assert_array_equal(a.positions(), x1)
    np.testing.assert_array_equal(a.qk(), q1)
    assert a.running_energy() == e1


def test_restore_refuses_damaged_and_foreign_snapshots():
    from beofaunus_gb300.gpu import FgError, System
    p, xyz, q, ids = _systems()["ewald_surface"]
    a = System(p, xyz, q, ids)
    a.sweep(*a.draw_translation_stream(3, 500), log=False)
    blob = bytearray(a.snapshot())
    x0 = a.positions()
    bad = bytearray(blob)
    bad[-5] ^= 0x40                                   # one bit of the payload
    with pytest.raises(FgError, match="checksum"):
        a.restore(bytes(bad))
    with pytest.raises(FgError):
        a.restore(bytes(blob[:-8]))                   # truncated
    p2, xyz2, q2, ids2 = workloads.rpm_ewald(402, 40.0, 5, seed=4, update_frequency=25, cutoff=14.0, eps_surf=80.0)
    other = System(p2, xyz2, q2, ids2)
    with pytest.raises(FgError, match="another system"):
        other.restore(bytes(blob))
    p3, xyz3, q3, ids3 = workloads.rpm_ewald(400, 40.0, 5, seed=4, update_frequency=25, cutoff=14.0, eps_surf=70.0)
    third = System(p3, xyz3, q3, ids3)
    with pytest.raises(FgError, match="another system"):
        third.restore(bytes(blob))
    # the refused calls left the system as it was
    np.testing.assert_array_equal(a.positions(), x0)
    a.restore(bytes(blob))
    np.testing.assert_array_equal(a.positions(), x0)


def _server_job():
    p, x, q, ids = workloads.dh_lj_salt(400, seed=9, kT_scale=1.1)
    return p, x, q, ids, 9, 12000


def test_server_job_resumed_from_a_snapshot_finishes_as_if_never_stopped():
    """A job snapshotted between rounds, cancelled (its client went away) and
    resumed on a fresh server, next to another job, finishes with the same
    positions, accepted count and energy as the uninterrupted job."""
    from beofaunus_gb300.gpu import Server
    p, x, q, ids, seed, n = _server_job()

    def finish(srv, jid):
        for _ in range(100000):
            if srv.poll(jid)["state"] == 2:
                break
            srv.step()
        return srv.poll(jid, positions=True)

    srv = Server(1 << 30, threads=256, round_pairs=1 << 18)
    whole = finish(srv, srv.submit(p, x, q, ids, seed, n))

    srv1 = Server(1 << 30, threads=256, round_pairs=1 << 18)
    jid = srv1.submit(p, x, q, ids, seed, n)
    for _ in range(3):
        srv1.step()
    mid = srv1.poll(jid)
    assert mid["state"] == 1 and 0 < mid["trials"] < n
    blob = srv1.snapshot(jid)
    srv1.cancel(jid)
    srv1.close()

    srv2 = Server(1 << 30, threads=256, round_pairs=1 << 18)
    po, xo, qo, io = workloads.dh_lj_salt(700, seed=10)
    other = srv2.submit(po, xo, qo, io, 10, 5000)
    jid2 = srv2.resume(blob)
    assert srv2.poll(jid2)["trials"] == mid["trials"]
    res = finish(srv2, jid2)
    finish(srv2, other)
    np.testing.assert_array_equal(res["xyz"], whole["xyz"])
    assert res["accepted"] == whole["accepted"]
    assert res["energy"] == whole["energy"]
    assert res["trials"] == n
