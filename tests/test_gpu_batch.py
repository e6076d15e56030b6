"""Batched systems, parallel tempering and the job server on the GPU,
checked against individual runs and against the FP64 oracle."""
import numpy as np
import pytest

from beofaunus_gb300 import workloads
from oracle.oracle import OracleSystem, philox, philox_stream

pytestmark = pytest.mark.gpu


def test_batch_equals_individual_runs():
    """Three 800-ion Ewald systems in one launch give bit-identical results
    to the same systems run one at a time (same streams, same threads, one
    CTA each as in the batch)."""
    from beofaunus_gb300.gpu import Batch, System
    specs = [workloads.rpm800(seed=s, update_frequency=200) for s in (1, 2, 3)]
    alone = []
    for i, (p, x, q, ids) in enumerate(specs):
        s = System(p, x, q, ids, threads=256)
        s.cluster = 1
        s.stream_philox(1600, seed=9, stream_id=i)
        st = s.stream_run()
        alone.append((s.positions(), st["accepted"], st["rebuilds"], s.running_energy()))
    systems = [System(p, x, q, ids, threads=256) for (p, x, q, ids) in specs]
    b = Batch(systems, threads=256)
    b.stream_philox([1600] * 3, seed=9)
    per, tot = b.run()
    assert tot["trials"] == 4800
    for i, s in enumerate(systems):
        np.testing.assert_array_equal(s.positions(), alone[i][0])
        assert per[i]["accepted"] == alone[i][1]
        assert per[i]["rebuilds"] == alone[i][2]
        assert s.running_energy() == alone[i][3]


def test_parallel_tempering_matches_oracle():
    """Four DH+LJ replicas of uneven size on a temperature ladder: every
    sweep and every exchange decision reproduced by the oracle from the same
    Philox streams (findPartner pairing, move.h:6621-6633)."""
    from beofaunus_gb300.gpu import Batch, System
    sizes = [60, 80, 100, 120]
    temps = np.array([0.8, 1.1, 1.5, 2.0])
    specs = [workloads.dh_lj_salt(n, seed=100 + n, density=0.004) for n in sizes]
    systems = [System(p, x, q, ids, threads=128) for (p, x, q, ids) in specs]
    oracles = [OracleSystem(p, x, q, ids) for (p, x, q, ids) in specs]
    b = Batch(systems, threads=128)
    seed, rounds, sweeps = 5, 6, 3
    b.pt_setup(temps, seed)
    b.pt_run(rounds, sweeps)
    st = b.pt_state()
    # oracle replay
    perm = list(range(4))
    utot = [o.total_energy()["total"] for o in oracles]
    for rd in range(rounds):
        for s_, (o, (p, x, q, ids)) in enumerate(zip(oracles, specs)):
            rung = perm.index(s_)
            o.set_kT(temps[rung])
            n = sweeps * sizes[s_]
            idx, disp, u = philox_stream(seed, s_, rd * n, n, ids, [p.type_dp[t] for t in range(p.n_types)],
                                         list(p.box))
            r = o.mc_run_stream(idx, disp, u)
            utot[s_] += r["utot"]
        c = philox([rd & 0xFFFFFFFF, rd >> 32, 0, 0x50540000], [seed, 0x50545054])
        dr = 1 if c[0] / 4294967296.0 > 0.5 else -1
        for i in range(4):
            pp = i + dr if i % 2 == 0 else i - dr
            if pp <= i or pp >= 4:
                continue
            a, bb = perm[i], perm[pp]
            arg = (1.0 / temps[i] - 1.0 / temps[pp]) * (utot[a] - utot[bb])
            cq = philox([rd & 0xFFFFFFFF, rd >> 32, i, 0x50540001], [seed, 0x50545054])
            uu = (cq[0] + 0.5) / 4294967296.0
            if not (uu > np.exp(arg)):
                perm[i], perm[pp] = bb, a
    np.testing.assert_array_equal(st["perm"], perm)
    for s_, (sysg, o) in enumerate(zip(systems, oracles)):
        np.testing.assert_allclose(sysg.positions(), o.positions(), rtol=0, atol=1e-9)
        assert st["energies"][s_] == pytest.approx(o.total_energy()["total"], abs=1e-4)
    assert st["attempts"].sum() > 0


def _job(n, seed, kT):
    p, x, q, ids = workloads.dh_lj_salt(n, seed=seed, kT_scale=kT)
    return p, x, q, ids


def test_server_result_same_alone_and_mixed():
    """Continuous batching: a job's result does not depend on the other jobs
    sharing the GPU, and admission respects the memory budget."""
    from beofaunus_gb300.gpu import Server
    jobs = {"A": (_job(200, 11, 1.0), 11), "B": (_job(350, 12, 1.3), 12), "C": (_job(500, 13, 0.9), 13)}

    def run(order, budget):
        srv = Server(budget, threads=256, round_pairs=1 << 18)
        ids = {}
        for name in order:
            (p, x, q, t), seed = jobs[name]
            ids[name] = srv.submit(p, x, q, t, seed, 3 * len(x))
        max_running = 0
        for _ in range(10000):
            running, _, _ = srv.step()
            max_running = max(max_running, running)
            if all(srv.poll(j)["state"] == 2 for j in ids.values()):
                break
        out = {k: srv.poll(j, positions=True) for k, j in ids.items()}
        assert all(o["state"] == 2 for o in out.values())
        return out, max_running, srv

    alone, _, _ = run(["A"], 1 << 30)
    mixed, maxr, _ = run(["B", "A", "C"], 1 << 30)
    assert maxr == 3
    np.testing.assert_array_equal(mixed["A"]["xyz"], alone["A"]["xyz"])
    assert mixed["A"]["accepted"] == alone["A"]["accepted"]
    assert mixed["A"]["energy"] == alone["A"]["energy"]
    # a budget that holds one job at a time: jobs queue and still all finish,
    # with unchanged results
    from beofaunus_gb300.gpu import System
    one_job = 0
    for k in "ABC":
        (p, x, q, t), seed = jobs[k]
        n = len(x)
        stream = min(3 * n, min(max(32, (1 << 18) // n), 1 << 20)) * 40
        one_job = max(one_job, System(p, x, q, t, threads=256).device_bytes + stream)
    tight, maxr1, _ = run(["B", "A", "C"], int(1.3 * one_job))
    assert maxr1 == 1
    np.testing.assert_array_equal(tight["A"]["xyz"], alone["A"]["xyz"])


def test_server_job_matches_oracle():
    from beofaunus_gb300.gpu import Server
    (p, x, q, t), seed = _job(300, 21, 1.2), 21
    srv = Server(1 << 30, threads=256, round_pairs=1 << 16)
    jid = srv.submit(p, x, q, t, seed, 1500)
    while srv.poll(jid)["state"] != 2:
        srv.step()
    res = srv.poll(jid, positions=True)
    o = OracleSystem(p, x, q, t)
    idx, disp, u = philox_stream(seed, 0, 0, 1500, t, [p.type_dp[k] for k in range(p.n_types)], list(p.box))
    r = o.mc_run_stream(idx, disp, u)
    assert res["accepted"] == int(r["acc"].sum())
    np.testing.assert_allclose(res["xyz"], o.positions(), rtol=0, atol=1e-9)


def test_server_mixes_kernel_variants():
    """Jobs small enough for shared-memory coordinates and jobs that are not
    run in the same round (two launches side by side) with unchanged results."""
    from beofaunus_gb300.gpu import Server
    small, big = _job(300, 31, 1.1), _job(9000, 32, 1.0)

    def run(items):
        srv = Server(1 << 32, round_pairs=1 << 20)
        ids = [srv.submit(p, x, q, t, seed, n_trials) for (p, x, q, t), seed, n_trials in items]
        for _ in range(100000):
            srv.step()
            if all(srv.poll(j)["state"] == 2 for j in ids):
                break
        return [srv.poll(j, positions=True) for j in ids]

    alone = run([(small, 31, 3000)])
    mixed = run([(big, 32, 18000), (small, 31, 3000)])
    assert all(m["state"] == 2 for m in mixed)
    np.testing.assert_array_equal(mixed[1]["xyz"], alone[0]["xyz"])
    assert mixed[1]["accepted"] == alone[0]["accepted"]
