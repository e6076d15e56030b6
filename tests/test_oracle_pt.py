"""Parallel tempering pinned to the reference itself (CPU).

tests/golden/pt_dhlj.npz holds a run of the reference's own
Move::ParallelTempering (move.h:6520-6771): 8 ranks, one process per rung,
each sweeping a 240-ion DH+LJ salt with AtomicTranslation between exchange
attempts (oracle/ref/ref_harness_pt.cpp, MPI calls served by the stand-in of
oracle/ref/fakempi; made by tests/golden/make_golden.py).

The oracle replays it from the same starts: the reference's random streams
(oracle.pt_streams: every rank draws the same global sequence, and
findPartner's uniform comes from the MPI controller's own generator), one
OracleSystem per configuration at the temperature of the rung that holds
it, and the exchange rule restated in oracle.pt_exchange. Every translation
count, every exchange decision, every energy the reference's move computed
and the final configurations must agree.
"""
import os

import numpy as np
import pytest

from beofaunus_gb300.params import FgParams
from oracle.oracle import OracleSystem, pt_exchange, pt_streams

from conftest import GOLDEN


def load_pt():
    g = np.load(os.path.join(GOLDEN, "pt_dhlj.npz"))
    p = FgParams.from_buffer_copy(g["params"].tobytes())
    p.bjerrum = float(g["bjerrum"])
    return g, p


def test_reference_streams_are_replayed():
    g, p = load_pt()
    R, N = g["xyz"].shape[:2]
    rounds, sweeps = int(g["rounds"]), int(g["sweeps"])
    dpp = np.array([p.type_dp[t] for t in g["ids"]])
    _, ua, ud = pt_streams(int(g["seed"]), dpp, sweeps * N, rounds)
    for r in range(R):   # every rank drew the same uniforms
        np.testing.assert_array_equal(g["u_accept"][r], ua)
        np.testing.assert_array_equal(g["u_direction"][r], ud)


def test_oracle_parallel_tempering_reproduces_the_reference_run():
    g, p = load_pt()
    temps = g["temps"]
    R, N = g["xyz"].shape[:2]
    rounds, sweeps = int(g["rounds"]), int(g["sweeps"])
    dpp = np.array([p.type_dp[t] for t in g["ids"]])
    streams, ua, ud = pt_streams(int(g["seed"]), dpp, sweeps * N, rounds)
    systems = [OracleSystem(p, g["xyz"][r], g["q"], g["ids"]) for r in range(R)]
    for r in range(R):
        assert systems[r].total_energy()["total"] / temps[r] == pytest.approx(g["u0"][r], rel=1e-10)
    perm = list(range(R))   # perm[rung] = configuration
    margin = np.inf         # closest approach of a translation's dU / kT to its threshold -ln u
    for rd in range(rounds):
        for i in range(R):
            o = systems[perm[i]]
            o.set_kT(temps[i])
            res = o.mc_run_stream(*streams[rd])
            assert int(res["acc"].sum()) == int(g["translations_accepted"][i][rd])
            margin = min(margin, np.min(np.abs(res["du"] / temps[i] + np.log(streams[rd][2]))))
        E = [o.total_energy()["total"] for o in systems]
        for i in range(R):
            assert E[perm[i]] / temps[i] == pytest.approx(g["uold"][i][rd], rel=1e-10, abs=1e-9)
        new, swapped = pt_exchange(E, temps, perm, ud[rd], ua[rd])
        for i in range(R):
            if not np.isnan(g["unew"][i][rd]):
                # the partner's configuration in this rung's energy, as the reference's move computed it
                dr = 1 if ud[rd] > 0.5 else -1
                pp = i + dr if i % 2 == 0 else i - dr
                assert E[perm[pp]] / temps[i] == pytest.approx(g["unew"][i][rd], rel=1e-10, abs=1e-9)
        assert list(swapped) == [int(a) for a in g["acc"][:, rd]], "round %d" % rd
        perm = new
    for i in range(R):
        np.testing.assert_allclose(systems[perm[i]].positions(), g["final_positions"][i], rtol=0, atol=1e-9)
    assert 0 < g["acc"].mean() < 1
    # no decision of the run lies within twice the 1e-6 kT parity band: a
    # device replay within that tolerance must reproduce every one of them
    assert margin > 2e-6
