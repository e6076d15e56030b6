"""Benchmark: Metropolis trial moves per second on 16384-ion Ewald systems.

Workload (per system): restricted primitive model, 16384 ions (+1/-1,
sigma 4 A) in a periodic cube L = 163 A, Bjerrum length 7.1 A, Ewald alpha
0.2/A, real-space cutoff 20 A with a cell list, spherical |n|^2 <= 100 (2242
k-vectors), WCA eps 0.1 kT, dp 2 A, Q(k) rebuilt from scratch every 1000
accepted trials. Seeded synthetic overlap-free starts (no dataset exists for
this path). One "step" = one sweep (16384 AtomicTranslation trials) of every
system.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value         batched: B independent systems (default B = number of SMs, one
              persistent CTA per system) advanced by the batched sweep; each
              system's Philox trial stream is staged in HBM before the timed
              region; time = CUDA events on the library's stream; the inputs
              (B systems' coordinates, cells and streams) exceed L2 and L2 is
              also flushed (256 MiB write) between timed steps.
e2e           the same batch through the C-ABI with host buffers: per step the
              reference's own mt19937 trial streams (drawn on the host before
              the step) are copied in (fg_batch_stream_upload) and every
              system's scalars are read back, all inside the wall-clock timed
              region.
single_chain  one system alone (one CTA), same kernel, same stream kind.
plain_per_trial_api  fg_trial_du + fg_commit per trial from a host loop: the
              plain drop-in Energybase path.
roofline      the sweep kernel against the FP32 pipe (pair and k-space terms
              are FP32 arithmetic, no dense contraction): algorithmic FLOP per
              trial (cost model below) x trials per launch / mean launch time.
cpu_baseline  the FP64 oracle port of the reference's per-trial work, one
              process per host core, on a time-bounded sample.
--impl reference   that CPU path alone, in the same units (its line is the
              reference arm).
"""
import argparse
import concurrent.futures as cf
import json
import multiprocessing as mp
import os
import re
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MC trial moves/s at dU err<=1e-6 kT vs FP64; batched/served vs plain; p99 latency"
UNIT = "trial moves/s"
N_IONS = 16384
BOX = 163.0
SIGMA = 4.0
WORKLOAD = "rpm16k_ewald_wca_cells_batched"
SYS_SCALARS_BYTES = 88          # sizeof(SysScalars): one system's per-step read-back

# Cost model of one trial (algorithmic work, FMA = 2 FLOP):
#   pairs: 2 x 127 ion pairs within the 20 A cutoff (old and new position),
#          40 FP32 FLOP and 3 MUFU ops each (Ewald real space + WCA);
#   k-space: per k-vector, e^{ik.r_old} (table + Taylor, 15), k.dr (5),
#          e^{ik.dr}-1 (Horner, 27), the complex products and the |Q|^2
#          difference (18): 65 FLOP;
#   commit (accepted trials only): per k-vector e^{ik.r_new} and the two
#          fixed-point contributions: 23 FLOP.
PAIRS_PER_TRIAL = 254
FLOP_PER_PAIR = 40
MUFU_PER_PAIR = 3
FLOP_PER_K = 65
FLOP_PER_K_COMMIT = 23


def workload_config(B, T):
    return {"workload": WORKLOAD, "systems": B, "n_particles_per_system": N_IONS, "box_A": BOX,
            "bjerrum_A": 7.1, "ewald": {"alpha": 0.2, "cutoff_A": 20.0, "kvectors": 2242, "n2_max": 100,
                                        "update_frequency": 1000, "cell_list": True},
            "wca_eps_kT": 0.1, "dp_A": 2.0, "trials_per_system_per_step": T,
            "l2": "inputs larger than L2 and flushed (256 MiB write) between timed steps",
            "rng": "Philox4x32-10 streams staged in HBM (value); reference mt19937 from host (e2e)"}


# ----------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev=0):
        self.p = None
        self.dev = dev
        self.path = os.path.join(ROOT, "gpurun_out", "clocks_bench_%d.csv" % dev)

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        busy = [x for x in sm if x > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------- start configurations
def _positions(seed):
    from beofaunus_gb300 import workloads
    return workloads.scatter_positions(N_IONS, BOX, SIGMA, seed)


def make_positions(seeds):
    """Overlap-free starts for every system, generated in a spawn pool."""
    procs = max(1, min(len(seeds), os.cpu_count() or 1))
    with mp.get_context("spawn").Pool(procs) as pool:
        return pool.map(_positions, seeds)


# ----------------------------------------------------------------- CPU path
_cpu_cache = {}


def _cpu_task(args):
    """Time-bounded sample of the oracle port on one core: trials in chunks of
    64 until ``seconds`` have passed. The system is built once per process."""
    seed, seconds = args
    import numpy as np
    from beofaunus_gb300 import workloads
    from oracle.oracle import OracleSystem, translation_stream
    if seed not in _cpu_cache:
        p, xyz, q, ids = workloads.rpm16k(seed=seed, update_frequency=1000, start="scatter")
        _cpu_cache[seed] = (OracleSystem(p, xyz, q, ids), np.array([p.type_dp[i] for i in ids]), [0])
    o, dpp, chunk = _cpu_cache[seed]
    n, t_run = 0, 0.0
    while t_run < seconds:
        idx, disp, u = translation_stream(seed * 100000 + chunk[0], dpp, 64)
        chunk[0] += 1
        t0 = time.perf_counter()
        o.mc_run_stream(idx, disp, u)
        t_run += time.perf_counter() - t0
        n += 64
    return n, t_run


class CpuPath:
    """The FP64 oracle port of the reference's per-trial work (all-pairs
    EwaldReal + WCA, 2K complex exponentials, self and surface sums, Q(k)
    rebuild every 1000 accepted) on every host core: one process per core,
    each its own system and seed, as independent reference runs would be."""

    def __init__(self, cores=None):
        from oracle import oracle
        oracle.build()
        self.cores = cores or os.cpu_count() or 1
        self.pool = mp.get_context("spawn").Pool(self.cores)

    def sample(self, seconds):
        res = self.pool.map(_cpu_task, [(1000 + c, seconds) for c in range(self.cores)], chunksize=1)
        rate = sum(n / t for n, t in res)
        trials = sum(n for n, _ in res)
        return rate, trials

    def close(self):
        self.pool.close()
        self.pool.join()

    def describe(self, seconds, trials):
        return ("%d processes (one per host core), each its own 16384-ion Ewald system, ~%.0f s of FP64 "
                "trials (%d in total); value = sum of per-process trial rates" % (self.cores, seconds, trials))


def cpu_baseline(seconds):
    cp = CpuPath()
    try:
        cp.sample(0.5)                      # build each process's system outside the sample
        rate, trials = cp.sample(seconds)
    finally:
        cp.close()
    return {"value": rate, "unit": UNIT, "cores": cp.cores, "kind": "port", "sample": cp.describe(seconds, trials)}


# ----------------------------------------------------------------- helpers
def fp32_gemm_tflops(torch, dev):
    """Measured FP32 peak: cuBLAS SGEMM 8192^3 with TF32 off, best of 5."""
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(8192, 8192, device=dev)
    b = torch.randn(8192, 8192, device=dev)
    c = torch.empty(8192, 8192, device=dev)
    for _ in range(2):
        torch.matmul(a, b, out=c)
    best = None
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del a, b, c
    return 2.0 * 8192 ** 3 / (best / 1e3) / 1e12


def profiled_traffic():
    """DRAM bytes per sweep-kernel launch from the committed ncu summary
    (a line 'dram_bytes_per_launch_full: <n>'), or None."""
    path = os.path.join(ROOT, "profiles", "sweep_kernel_rpm16k_batch.md")
    try:
        for line in open(path):
            m = re.match(r"\s*[-*]?\s*dram_bytes_per_launch_full:\s*([0-9.eE+]+)", line)
            if m:
                return float(m.group(1))
    except OSError:
        pass
    return None


# ----------------------------------------------------------------- our arm
def run_ours(args, rank, world):
    import numpy as np
    import torch

    from beofaunus_gb300 import build, workloads
    from beofaunus_gb300.gpu import Batch, System

    build.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    B = args.systems or sms
    T = args.trials
    steps, warm = args.steps, args.warmup

    # independent systems (replicas only across ranks: distinct seeds, no exchange)
    seeds = [1 + rank * 1000003 + b for b in range(B + 1)]
    xyzs = make_positions(seeds)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    fp32_peak = fp32_gemm_tflops(torch, dev)

    systems = []
    for b in range(B):
        p, xyz, q, ids = workloads.rpm16k(seed=seeds[b], update_frequency=1000, start=xyzs[b])
        systems.append(System(p, xyz, q, ids))
    batch = Batch(systems)

    def device_step(step_seed):
        batch.stream_philox([T] * B, step_seed)        # staged in HBM, untimed
        flush.fill_(step_seed & 0xFF)
        torch.cuda.synchronize()
        return batch.run()[1]

    for s in range(warm):
        device_step(10 + s)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    stats = [device_step(1000 + s) for s in range(steps)]
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    dev_ms = sum(st["device_ms"] for st in stats)
    sweep_ms = sum(st["sweep_kernel_ms"] for st in stats)
    launches = sum(st["sweep_launches"] for st in stats)
    kernels = sum(st["kernel_launches"] for st in stats)
    trials = sum(st["trials"] for st in stats)
    accepted = sum(st["accepted"] for st in stats)
    rebuilds = sum(st["rebuilds"] for st in stats)
    if dist:
        t = torch.tensor([float(trials), dev_ms], dtype=torch.float64, device=dev)
        tr = t[:1].clone()
        dist.all_reduce(tr)
        mx = t[1:].clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        all_trials, max_ms = tr.item(), mx.item()
    else:
        all_trials, max_ms = float(trials), dev_ms
    value = all_trials / (max_ms / 1e3)

    if args.value_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": max_ms / steps,
                              "sweep_kernel_ms": sweep_ms, "sweep_launches": launches, "trials": trials,
                              "systems": B}))
        if dist:
            dist.destroy_process_group()
        return

    # ---- e2e: host streams in, scalars out, wall clock around upload + run
    pool = cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1))
    e2e_s, e2e_trials, e2e_gathers = 0.0, 0, 0
    for s in range(steps):
        host = [systems[b].draw_translation_stream(50000 + 1000 * s + b, T) for b in range(B)]
        flush.fill_(s & 0xFF)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        list(pool.map(lambda b: batch.stream_upload(b, *host[b]), range(B)))
        _, tot = batch.run()
        e2e_s += time.perf_counter() - t0
        e2e_trials += tot["trials"]
        e2e_gathers += tot["kernel_launches"] - 1 - 3 * tot["sweep_launches"]
        del host
    pool.shutdown()
    e2e = e2e_trials / e2e_s
    if dist:
        t = torch.tensor([float(e2e_trials)], dtype=torch.float64, device=dev)
        dist.all_reduce(t)
        m = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        dist.all_reduce(m, op=dist.ReduceOp.MAX)
        e2e = t.item() / m.item()

    # ---- roofline of the dominant kernel (sweep kernel), FP32 pipe
    K = systems[0].num_kvectors
    acc_rate = accepted / max(trials, 1)
    flop_per_trial = PAIRS_PER_TRIAL * FLOP_PER_PAIR + K * FLOP_PER_K + acc_rate * K * FLOP_PER_K_COMMIT
    avg_launch_s = sweep_ms / max(launches, 1) / 1e3
    trials_per_launch = trials / max(launches, 1)
    achieved = flop_per_trial * trials_per_launch / avg_launch_s / 1e12
    sm_mhz = (clk or {}).get("sm_mhz") or 1900.0
    mufu_peak = sms * 16 * sm_mhz * 1e6
    mufu_frac = PAIRS_PER_TRIAL * MUFU_PER_PAIR * trials_per_launch / avg_launch_s / mufu_peak
    traffic = profiled_traffic()

    # ---- single chain: one system, one CTA
    p, xyz, q, ids = workloads.rpm16k(seed=seeds[B], update_frequency=1000, start=xyzs[B])
    one = System(p, xyz, q, ids)
    one.stream_philox(T, 7)
    one.stream_run()
    sc = []
    for s in range(2):
        one.stream_philox(T, 8 + s)
        flush.fill_(s)
        torch.cuda.synchronize()
        sc.append(one.stream_run())
    single = sum(st["trials"] for st in sc) / (sum(st["device_ms"] for st in sc) / 1e3)

    # ---- plain per-trial drop-in path (fg_trial_du + fg_commit per trial)
    idx, disp, u = one.draw_translation_stream(777, 300)
    pos = one.positions()
    t0 = time.perf_counter()
    for t in range(300):
        i = int(idx[t])
        new = pos[i] + disp[t]
        new -= BOX * np.round(new / BOX)
        du = one.trial_du(i, new)
        acc = not (u[t] > np.exp(-du))
        one.commit(acc)
        if acc:
            pos[i] = new
    plain = 300 / (time.perf_counter() - t0)
    one.close()

    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": steps,
        "warmup": warm,
        "ms_per_step": max_ms / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 pair and k terms; df (~48-bit) sums; int64 fixed-point Q(k)",
        "data": "synthetic (seeded overlap-free starts; Philox streams, reference mt19937 for e2e)",
        "config": workload_config(B, T),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": B * T * 40,
                "d2h_bytes_per_step": int(round(e2e_gathers / steps)) * B * SYS_SCALARS_BYTES},
        "gpu_launches": int(kernels),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": traffic,
                     "peak_source": "measured in this run: cuBLAS SGEMM 8192^3, TF32 off (best of 5)",
                     "flop_per_trial": flop_per_trial, "trials_per_launch": trials_per_launch,
                     "mean_launch_ms": avg_launch_s * 1e3, "mufu_frac": mufu_frac,
                     "note": "pair and k-space terms are FP32 arithmetic with no dense contraction; "
                             "each system is a sequential Markov chain on one SM"},
        "single_chain": {"value": single, "unit": UNIT, "us_per_trial": 1e6 / single},
        "plain_per_trial_api": {"value": plain, "unit": UNIT},
        "batched_over_plain": value / plain,
        "batched_over_single_chain": value / single,
        "acceptance": acc_rate,
        "qk_rebuilds": rebuilds,
        "clocks": clk,
    }
    batch.close()
    for s_ in systems:
        s_.close()
    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))


def run_reference(args):
    """The reference's CPU path on the host cores: the FP64 oracle port (the
    reference binary built from source is x86-only here and does not travel)."""
    warm, steps = args.warmup, args.steps
    cp = CpuPath()
    try:
        cp.sample(0.5)
        for _ in range(warm):
            cp.sample(args.ref_seconds)
        vals, trials = [], 0
        for _ in range(steps):
            r, n = cp.sample(args.ref_seconds)
            vals.append(r)
            trials += n
    finally:
        cp.close()
    value = statistics.mean(vals)
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": steps, "warmup": warm, "ms_per_step": 1e3 * args.ref_seconds,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded overlap-free starts, reference mt19937 stream)",
           "config": workload_config(cp.cores, "time-bounded sample per step"),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cp.cores, "kind": "port",
                            "sample": cp.describe(args.ref_seconds, trials // max(steps, 1))},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--systems", type=int, default=0, help="systems per GPU (default: SM count)")
    ap.add_argument("--trials", type=int, default=N_IONS, help="trials per system per step (default: one sweep)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample per core")
    ap.add_argument("--ref-seconds", type=float, default=3.0, help="reference arm: seconds per step")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--value-only", action="store_true", help="device-resident value only (profiling)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    run_ours(args, rank, world)


if __name__ == "__main__":
    main()
