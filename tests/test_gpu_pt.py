"""Parallel tempering on the GPU, pinned to the reference and to the oracle.

1. The reference's own run (tests/golden/pt_dhlj.npz, made by the reference's
   Move::ParallelTempering over one process per rung, see
   tests/test_oracle_pt.py): the batch replays it with the reference's random
   streams uploaded to every member, FP64 system energies from the device and
   fg_pt_swap given the reference's uniforms. Every translation count, every
   exchange decision and the final configurations must agree.
2. The c3 ladder at full size: 64 DH+LJ replicas, N log-uniform in 500-4000,
   temperatures geometric from 0.8 to 2.0, device Philox streams and the
   captured exchange rounds (fg_pt_run), replayed by the oracle round by round
   from the same streams and the same exchange rule (move.h:6621-6722).
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

from beofaunus_gb300 import workloads
from beofaunus_gb300.params import FgParams
from oracle.oracle import OracleSystem, philox, philox_stream, pt_streams

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_gpu_parallel_tempering_reproduces_the_reference_run():
    from beofaunus_gb300.gpu import Batch, System
    g = np.load(os.path.join(GOLDEN, "pt_dhlj.npz"))
    p = FgParams.from_buffer_copy(g["params"].tobytes())
    p.bjerrum = float(g["bjerrum"])
    temps = g["temps"]
    R, N = g["xyz"].shape[:2]
    rounds, sweeps = int(g["rounds"]), int(g["sweeps"])
    dpp = np.array([p.type_dp[t] for t in g["ids"]])
    streams, ua, ud = pt_streams(int(g["seed"]), dpp, sweeps * N, rounds)
    systems = [System(p, g["xyz"][r], g["q"], g["ids"]) for r in range(R)]
    b = Batch(systems)
    b.pt_setup(temps, 1)
    for rd in range(rounds):
        for m in range(R):
            b.stream_upload(m, *streams[rd])   # every rank draws the same stream
        per, _ = b.run()
        perm = b.pt_state()["perm"]
        for i in range(R):
            assert per[perm[i]]["accepted"] == int(g["translations_accepted"][i][rd]), (rd, i)
        E = [s.total_energy_fp64()["total"] for s in systems]
        for i in range(R):
            assert E[perm[i]] / temps[i] == pytest.approx(g["uold"][i][rd], rel=1e-9, abs=1e-8)
        ex = b.pt_swap(ud[rd], ua[rd], E)
        np.testing.assert_array_equal(ex, g["acc"][:, rd], err_msg="round %d" % rd)
    perm = b.pt_state()["perm"]
    for i in range(R):
        np.testing.assert_allclose(systems[perm[i]].positions(), g["final_positions"][i], rtol=0, atol=1e-9)
    b.close()
    for s in systems:
        s.close()


# ------------------------------------------------------------------ c3 ladder
C3_SEED, C3_ROUNDS, C3_SWEEPS = 11, 2, 2


def c3_ladder():
    sizes = workloads.pt_ladder_sizes(64)
    temps = workloads.pt_temperatures(64, 0.8, 2.0)
    specs = [workloads.dh_lj_salt(int(n), seed=500 + i, start="scatter") for i, n in enumerate(sizes)]
    return sizes, temps, specs


def _replica_round(args):
    """Oracle: one replica's sweeps of one round from its Philox stream.
    Returns (positions, utot change, closest |dU/kT + ln u|)."""
    pb, xyz, q, ids, kT, seed, stream, first, n = args
    p = FgParams.from_buffer_copy(pb)
    o = OracleSystem(p, xyz, q, ids)
    o.set_kT(kT)
    idx, disp, u = philox_stream(seed, stream, first, n, ids, [p.type_dp[t] for t in range(p.n_types)], list(p.box))
    r = o.mc_run_stream(idx, disp, u)
    return o.positions(), r["utot"], float(np.min(np.abs(r["du"] / kT + np.log(u))))


def c3_oracle(sizes, temps, specs, seed, rounds, sweeps, pool):
    """The ladder replayed by the oracle: Philox streams of the device
    (stream id = system, counters continuing over rounds), exchange rule of
    pt_swap_kernel on the running totals. Returns perm, positions, energies
    and the smallest distance of any translation or exchange from its
    threshold."""
    n = len(sizes)
    pos = [s[1] for s in specs]
    utot = [OracleSystem(p, x, q, i).total_energy()["total"] for p, x, q, i in specs]
    perm = list(range(n))
    margin_t, margin_x = np.inf, np.inf
    for rd in range(rounds):
        jobs = []
        for s in range(n):
            p, _, q, ids = specs[s]
            cnt = sweeps * int(sizes[s])
            jobs.append((bytes(p), pos[s], q, ids, float(temps[perm.index(s)]), seed, s, rd * cnt, cnt))
        res = pool.map(_replica_round, jobs)
        for s in range(n):
            pos[s] = res[s][0]
            utot[s] += res[s][1]
            margin_t = min(margin_t, res[s][2])
        c = philox([rd & 0xFFFFFFFF, rd >> 32, 0, 0x50540000], [seed, 0x50545054])
        dr = 1 if c[0] / 4294967296.0 > 0.5 else -1
        for i in range(n):
            pp = i + dr if i % 2 == 0 else i - dr
            if pp <= i or pp >= n:
                continue
            a, bb = perm[i], perm[pp]
            arg = (1.0 / temps[i] - 1.0 / temps[pp]) * (utot[a] - utot[bb])
            cq = philox([rd & 0xFFFFFFFF, rd >> 32, i, 0x50540001], [seed, 0x50545054])
            uu = (cq[0] + 0.5) / 4294967296.0
            margin_x = min(margin_x, abs(np.log(uu) - arg))
            if not (uu > np.exp(arg)):
                perm[i], perm[pp] = bb, a
    return perm, pos, utot, margin_t, margin_x


def test_c3_ladder_matches_oracle():
    from beofaunus_gb300.gpu import Batch, System
    sizes, temps, specs = c3_ladder()
    assert len(sizes) == 64 and sizes.min() >= 500 and sizes.max() <= 4000
    systems = [System(p, x, q, i) for p, x, q, i in specs]
    b = Batch(systems)
    b.pt_setup(temps, C3_SEED)
    b.pt_run(C3_ROUNDS, C3_SWEEPS)
    st = b.pt_state()
    with mp.get_context("spawn").Pool(max(1, min(16, os.cpu_count() or 1))) as pool:
        perm, pos, utot, margin_t, margin_x = c3_oracle(sizes, temps, specs, C3_SEED, C3_ROUNDS, C3_SWEEPS, pool)
    print("c3 ladder: exchanges %d of %d, closest translation %.3g, closest exchange %.3g" %
          (int(st["accepts"].sum()), int(st["attempts"].sum()), margin_t, margin_x))
    # the seeds are such that no decision lies near its threshold: within the
    # 1e-6 kT tolerance (and the ~1e-4 kT FP32 offset of the running totals at
    # upload) the device must take every one the oracle takes
    assert margin_t > 2e-6 and margin_x > 1e-3
    np.testing.assert_array_equal(st["perm"], perm)
    for s in range(64):
        np.testing.assert_allclose(systems[s].positions(), pos[s], rtol=0, atol=1e-9)
        assert st["energies"][s] == pytest.approx(utot[s], abs=2e-3)
    assert st["attempts"].sum() > 0
    b.close()
    for s in systems:
        s.close()
