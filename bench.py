"""Benchmark: Metropolis trial moves per second on the 16384-ion Ewald workload.

Workload (one "step" = one sweep = 16384 trials of AtomicTranslation):
restricted primitive model, 16384 ions (+1/-1, sigma 4 A) in a periodic cube
L = 163 A, Bjerrum length 7.1 A, Ewald alpha 0.2/A, real-space cutoff 20 A
with a cell list, spherical |n|^2 <= 100 (2242 k-vectors), WCA eps 0.1 kT,
dp 2 A, Q(k) rebuilt every 1000 accepted trials. Synthetic seeded RSA start
(no dataset exists for this path). The per-trial random stream is the
reference's own (std::mt19937 replayed exactly as the reference draws it).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value      device-resident throughput: trial streams staged in HBM before the
           timed region; per-step CUDA events on the library's stream; L2
           flushed (256 MiB write) between timed steps.
e2e        the same metric through the C-ABI call a user makes (fg_sweep with
           host buffers): host->device copy of the step's trial stream and
           device->host read of its per-trial results inside the timed region.
--impl reference   the reference's CPU path on all host cores (one process per
           core), reported in the same units.
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_IONS = 16384
WORKLOAD = "rpm16k_ewald_wca_cells"
METRIC = "MC trial moves/s at dU err<=1e-6 kT vs FP64 (16384-ion Ewald, single system)"


def workload_config():
    return {"workload": WORKLOAD, "n_particles": N_IONS, "box_A": 163.0, "bjerrum_A": 7.1,
            "ewald": {"alpha": 0.2, "cutoff_A": 20.0, "kvectors": 2242, "n2_max": 100,
                      "update_frequency": 1000},
            "wca_eps_kT": 0.1, "dp_A": 2.0, "trials_per_step": N_IONS,
            "l2": "flushed (256 MiB write) between timed steps", "rng": "reference mt19937 stream"}


# ----------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.p = None
        self.path = os.path.join(ROOT, "gpurun_out", "clocks_bench.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self, dev=0):
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
            if len(parts) < 9 or parts[0] != str(dev):
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


# ----------------------------------------------------------------- CPU baseline
def _cpu_worker(args):
    seed, n_trials = args
    from beofaunus_gb300 import workloads
    from oracle.oracle import OracleSystem, translation_stream
    import numpy as np
    p, xyz, q, ids = workloads.rpm16k(seed=seed, update_frequency=1000)
    o = OracleSystem(p, xyz, q, ids)
    dpp = np.array([p.type_dp[i] for i in ids])
    idx, disp, u = translation_stream(seed, dpp, n_trials)
    t0 = time.perf_counter()
    o.mc_run_stream(idx, disp, u)
    return n_trials, time.perf_counter() - t0


def cpu_baseline(trials_per_core=1024, cores=None):
    """The oracle port (FP64 restatement of the reference's per-trial work:
    all-pairs EwaldReal+WCA, 2K complex exponentials, self/surface sums,
    rebuild every 1000 accepted) on all host cores, one process per core."""
    cores = cores or os.cpu_count() or 1
    from oracle import oracle
    oracle.build()
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(1000 + c, trials_per_core) for c in range(cores)])
    rate = sum(n / t for n, t in res)
    return {"value": rate, "unit": "trials/s", "cores": cores, "kind": "port",
            "sample": "%d processes x %d trials of the 16384-ion Ewald system (oracle port of the "
                      "reference's per-trial FP64 work), aggregate of per-process rates" % (cores, trials_per_core),
            "per_core": rate / cores}


def reference_binary():
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
    if os.path.exists(exe) and os.access(exe, os.X_OK):
        try:
            r = subprocess.run([exe], capture_output=True, timeout=10)
            if r.returncode == 2:   # usage message: the binary runs on this machine
                return exe
        except Exception:
            return None
    return None


# ----------------------------------------------------------------- our arm
def run_ours(args):
    import numpy as np
    import torch

    from beofaunus_gb300 import build, workloads
    from beofaunus_gb300.gpu import System

    build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    p, xyz, q, ids = workloads.rpm16k(seed=1, update_frequency=1000)
    sys_ = System(p, xyz, q, ids)
    steps, warm = args.steps, args.warmup
    T = args.trials
    streams = [sys_.draw_translation_stream(100 + s, T) for s in range(warm + steps)]

    # warm-up (untimed): also the e2e path
    for s in range(warm):
        sys_.sweep(*streams[s], log=False)
    # ---- device-resident value: stage every timed step's stream first
    stats = []
    clocks = ClockSampler()
    clocks.start()
    torch.cuda.synchronize()
    for s in range(steps):
        sys_.stream_upload(*streams[warm + s])
        flush.fill_(s & 0xFF)
        torch.cuda.synchronize()
        st = sys_.stream_run()
        stats.append(st)
    torch.cuda.synchronize()
    clk = clocks.stop()
    dev_ms = sum(st["device_ms"] for st in stats)
    sweep_ms = sum(st["sweep_kernel_ms"] for st in stats)
    launches = sum(st["sweep_launches"] for st in stats)
    trials = sum(st["trials"] for st in stats)
    value = trials / (dev_ms / 1e3)

    if args.value_only:
        print(json.dumps({"metric": METRIC, "value": value, "unit": "trials/s", "ms_per_step": dev_ms / steps,
                          "sweep_kernel_ms": sweep_ms, "sweep_launches": launches, "trials": trials}))
        return
    # ---- e2e through fg_sweep with host buffers (H2D stream, D2H results)
    e2e_streams = [sys_.draw_translation_stream(5000 + s, T) for s in range(steps)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(steps):
        sys_.sweep(*e2e_streams[s], log=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e = steps * T / e2e_s

    # ---- roofline of the dominant kernel (sweep_kernel)
    # algorithmic bytes per trial (L1/L2-resident working set, what one trial
    # must touch): Q(k) + k-vector tables 36 B x 2242, candidate positions
    # 2 x 127 pairs x 20 B within the cutoff, the trial record 40 B.
    K = sys_.num_kvectors
    bytes_per_trial = 36 * K + 2 * 127 * 20 + 40
    flops_per_trial = 45 * K + 2 * 127 * 40
    avg_launch_ms = sweep_ms / max(launches, 1)
    trials_per_launch = trials / max(launches, 1)
    achieved_gbs = bytes_per_trial * trials_per_launch / (avg_launch_ms / 1e3) / 1e9
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    sm_mhz = (clk or {}).get("sm_mhz") or 1900.0
    fp32_peak_tflops = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    fp32_sm_peak = fp32_peak_tflops / 152
    achieved_tflops = flops_per_trial * trials_per_launch / (avg_launch_ms / 1e3) / 1e12

    # ---- plain per-trial drop-in path (fg_trial_du + fg_commit per trial)
    idx, disp, u = sys_.draw_translation_stream(777, 400)
    pos = sys_.positions()
    t0 = time.perf_counter()
    for t in range(400):
        i = int(idx[t])
        new = pos[i] + disp[t]
        new -= 163.0 * np.round(new / 163.0)
        du = sys_.trial_du(i, new)
        acc = not (u[t] > np.exp(-du))
        sys_.commit(acc)
        if acc:
            pos[i] = new
    plain_rate = 400 / (time.perf_counter() - t0)

    cfg = workload_config()
    cfg["trials_per_step"] = T
    out = {
        "metric": METRIC,
        "value": value,
        "unit": "trials/s",
        "n_gpus": 1,
        "steps": steps,
        "warmup": warm,
        "ms_per_step": dev_ms / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 pair/k terms, compensated df (~48-bit) sums and Q(k)",
        "data": "synthetic (seeded RSA start, reference RNG stream)",
        "config": cfg,
        "e2e": {"value": e2e, "unit": "trials/s", "h2d_bytes_per_step": T * 40,
                "d2h_bytes_per_step": T * (8 + 1) + 64},
        "gpu_launches": int(launches * 4),
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved_gbs / hbm_peak, "traffic": None,
                     "note": "sequential Markov chain on one SM: latency-bound; see fp32_one_sm"},
        "fp32_one_sm": {"achieved_tflops": achieved_tflops, "peak_tflops_one_sm": fp32_sm_peak,
                        "frac": achieved_tflops / fp32_sm_peak,
                        "peak": "nominal 128 FP32 lanes x 2 flop x measured SM clock"},
        "plain_per_trial_api": {"value": plain_rate, "unit": "trials/s"},
        "clocks": clk,
    }
    sys_.close()
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(trials_per_core=args.cpu_trials)
    print(json.dumps(out))


def run_reference(args):
    """The reference's CPU path on the host cores (oracle port: the compiled
    reference cannot travel to this machine's architecture)."""
    warm, steps = args.warmup, args.steps
    cb = None
    times = []
    for s in range(warm + steps):
        r = cpu_baseline(trials_per_core=args.cpu_trials)
        if s >= warm:
            times.append(r)
        cb = r
    value = statistics.mean(r["value"] for r in times)
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "trials/s", "n_gpus": args.gpus,
           "steps": steps, "warmup": warm, "ms_per_step": 1e3 * N_IONS / value, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
           "config": workload_config(),
           "cpu_baseline": {"value": value, "unit": "trials/s", "cores": cb["cores"], "kind": cb["kind"],
                            "sample": cb["sample"]},
           "e2e": {"value": value, "unit": "trials/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-trials", type=int, default=1024)
    ap.add_argument("--trials", type=int, default=N_IONS, help="trials per step (default: one sweep)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--value-only", action="store_true", help="device-resident value only (profiling)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        # replicas only: every rank runs its own independent system
    run_ours(args)


if __name__ == "__main__":
    main()
