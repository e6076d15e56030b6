"""dU accuracy of the batched Ewald block kernel at the benchmarked size.

The bench's default workload runs 16384-ion Ewald systems (L = 163 A,
K = 2242, cell list, rebuild every 1000 accepted trials) many to a launch.
Here the same kernel and launch kind are checked against the FP64 oracle
trial by trial:

* a batch of 4 such systems in one launch, every trial logged on the device
  (fg_batch_set_log) and replayed by the oracle from the same start and the
  same Philox streams;
* the error tail of one chain over 10^5 trials: the device runs the chain in
  segments (host mt19937 draws as the reference makes them), the oracle
  replays each segment from the device's coordinates at its start, all
  segments at once in a process pool.

Tolerance (as every parity test): |dU_GPU - dU_FP64| <= 1e-6 kT, decisions
identical except inside that band around the threshold.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

from beofaunus_gb300 import workloads
from oracle.oracle import compare_chain, replay_chain

pytestmark = pytest.mark.gpu

TOL_DU = 1e-6


def _pool(n):
    return mp.get_context("spawn").Pool(max(1, min(n, os.cpu_count() or 1)))


def _check(res):
    assert res["divergence_in_band"], "decisions differ outside the tolerance band: %s" % res
    assert res["max_err"] <= TOL_DU, res


def _batched_run(cases, T, mode):
    """Run the cases as one batch with every trial logged; the rebuilds run
    inside the sweep launch (mode 1) or in the rebuild kernel (mode 2)."""
    from beofaunus_gb300.gpu import Batch, System
    systems = [System(p, x, q, i) for p, x, q, i in cases]
    batch = Batch(systems)
    batch.set_rebuild_mode(mode)
    for m in range(len(cases)):
        batch.set_log(m)
    batch.stream_philox([T] * len(cases), 4242)
    per, tot = batch.run()
    out = []
    for m, s in enumerate(systems):
        idx, disp, u = s.stream_get(0, T)
        du, acc = s.log_get(0, T)
        out.append(dict(idx=idx, disp=disp, u=u, du=du, acc=acc, pos=s.positions(), qk=s.qk(),
                        accepted=per[m]["accepted"]))
    batch.close()
    for s in systems:
        s.close()
    return out, tot


def test_batched_rpm16k_block_kernel_matches_oracle():
    """Both places of the Q(k) rebuild (inside the persistent sweep, as the
    bench's batch of one system per SM runs it, and the separate rebuild
    kernel) give bit-identical chains, and those match the oracle."""
    B, T = 4, 1500
    cases = [workloads.rpm16k(seed=300 + b, update_frequency=1000, start="scatter") for b in range(B)]
    inside, tot = _batched_run(cases, T, 1)
    outside, tot2 = _batched_run(cases, T, 2)
    assert tot["trials"] == B * T
    assert tot["rebuilds"] >= B and tot["rebuilds"] == tot2["rebuilds"]   # uf = 1000 accepted: every chain rebuilds
    assert tot["sweep_launches"] == 1
    for a, b in zip(inside, outside):
        np.testing.assert_array_equal(a["du"], b["du"])
        np.testing.assert_array_equal(a["acc"], b["acc"])
        np.testing.assert_array_equal(a["pos"], b["pos"])
        np.testing.assert_array_equal(a["qk"], b["qk"])
    jobs = [(bytes(p), x, q, i, r["idx"], r["disp"], r["u"]) for (p, x, q, i), r in zip(cases, inside)]
    with _pool(B) as pool:
        ref = pool.map(replay_chain, jobs)
    for m in range(B):
        r = inside[m]
        res = compare_chain(r["du"], r["acc"], ref[m][0], ref[m][1], r["u"], TOL_DU)
        print("member %d: max |dU err| %.3g rms %.3g over %d trials" % (m, res["max_err"], res["rms_err"],
                                                                         res["compared"]))
        _check(res)
        assert r["accepted"] == int(np.sum(r["acc"]))


def test_rpm16k_error_tail_over_1e5_trials():
    """One 16384-ion chain, 8 segments of 12800 trials (102400 in all)."""
    from beofaunus_gb300.gpu import System
    p, x, q, i = workloads.rpm16k(seed=777, update_frequency=1000, start="scatter")
    s = System(p, x, q, i)
    nseg, T = 8, 12800
    jobs, dev = [], []
    for g in range(nseg):
        start = s.positions()
        idx, disp, u = s.draw_translation_stream(9000 + g, T)
        r = s.sweep(idx, disp, u)
        dev.append((r["du"], r["acc"], u))
        jobs.append((bytes(p), start, q, i, idx, disp, u))
    s.close()
    with _pool(nseg) as pool:
        ref = pool.map(replay_chain, jobs)
    errs = []
    for g in range(nseg):
        du, acc, u = dev[g]
        res = compare_chain(du, acc, ref[g][0], ref[g][1], u, TOL_DU)
        _check(res)
        errs.append(np.abs(du[:res["compared"]] - ref[g][0][:res["compared"]]))
    e = np.concatenate(errs)
    q50, q99, q9999 = np.quantile(e, [0.5, 0.99, 0.9999])
    print("rpm16k tail over %d trials: max %.3g, rms %.3g, median %.3g, p99 %.3g, p99.99 %.3g, >5e-7: %d" %
          (len(e), e.max(), np.sqrt(np.mean(e ** 2)), q50, q99, q9999, int(np.sum(e > 5e-7))))
    assert len(e) > 0.9 * nseg * T
    assert e.max() <= TOL_DU
