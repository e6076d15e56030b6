"""Benchmark: Metropolis trial moves per second on 16384-ion Ewald systems.

Workload (per system): restricted primitive model, 16384 ions (+1/-1,
sigma 4 A) in a periodic cube L = 163 A, Bjerrum length 7.1 A, Ewald alpha
0.2/A, real-space cutoff 20 A with a cell list, spherical |n|^2 <= 100 (2242
k-vectors), WCA eps 0.1 kT, dp 2 A, Q(k) rebuilt from scratch every 1000
accepted trials. Seeded synthetic overlap-free starts (no dataset exists for
this path). One "step" = one sweep (16384 AtomicTranslation trials) of every
system.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload rpm16k|rpm800|pt64|molecules|serving|dipoles]

The default workload is the batched 16384-ion Ewald one below; the others
measure the remaining configurations of the path the same way (one JSON line
each): rpm800 = 800-ion Ewald systems (L = 60, |n|^2 <= 49), pt64 = 64-replica
Debye-Hueckel + LJ parallel tempering, molecules = 1000 rigid 20-site dipolar
molecules per system (TranslateRotate), serving = Poisson job stream through
the continuous-batching server with p50/p99 job latency, dipoles = point
dipoles under the dipolar Ewald sum (AtomicRotation + AtomicTranslation).

With N > 1 every rank runs its own replicas (distinct seeds, no data-path
exchange); value = all ranks' trials over the slowest rank's time
(reduce_sum_max / reduce_rate). Started without a launcher, bench.py --gpus N
starts its N ranks itself under torch.distributed.run (launch_ranks); a run
whose rank count differs from --gpus stops with an error.

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
single_chain  one system alone on a thread-block cluster of CTAs (the built-in
              size; the figure for every size up to the largest that fits
              is listed beside it), same stream kind.
plain_per_trial_api  fg_trial_du + fg_commit per trial from a host loop: the
              plain drop-in Energybase path.
roofline      the Ewald block kernel against the FP32 pipe (pair and k-space
              terms are FP32 arithmetic; the block's 32x32 Gram matrix is the
              only contraction, a tenth of the kernel, on the tensor cores):
              algorithmic FLOP per trial (cost model below) x trials per
              launch / mean launch time.
cpu_baseline  the reference's own CPU path, one process per host core, on a
              time-bounded sample: the reference built from its sources on
              this machine (oracle/_ref/ref_harness) for the Ewald and DH+LJ
              workloads, else the FP64 oracle port of its per-trial work.
--impl reference   that CPU path alone, in the same units (its line is the
              reference arm).
"""
import argparse
import math
import concurrent.futures as cf
import json
import multiprocessing as mp
import os
import re
import statistics
import subprocess
import sys
import tempfile
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
# what fg_stream_upload copies per trial: the caller's int32 index, three
# double displacements and one double uniform (the 40-byte trial records are
# built from them on the device)
UPLOAD_BYTES_PER_TRIAL = 4 + 3 * 8 + 8

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
#   rebuild (every 1000 accepted trials, inside the sweep launch): per
#          particle and k-vector one complex product w e_z (6 FLOP) of its
#          integer term (the per-axis tables and the w of a run of k-vectors
#          are not counted).
FLOP_PER_TERM_REBUILD = 6


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
        # raw samples; the summary goes into the JSON line
        self.path = os.path.join(os.environ.get("FG_CLOCKS_DIR", tempfile.gettempdir()), "clocks_bench_%d.csv" % dev)

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


def _cpu_system(kind, seed):
    """One FP64 oracle system of the given workload kind (built once per process)."""
    import numpy as np
    from beofaunus_gb300 import workloads
    from oracle.oracle import OracleDip, OracleMol, OracleSystem
    if kind == "dipoles":
        p, xyz, mu, mus, ids, q = dipole_fluid(seed)
        return OracleDip(p, xyz, mu, mus, ids, q=q), None
    if kind == "molecules":
        p, xyz, mu, mus, ids = workloads.dipolar_molecules(1000, seed=seed)
        return OracleMol(p, xyz, mu, mus, ids, 20), None
    if kind == "rpm16k":
        p, xyz, q, ids = workloads.rpm16k(seed=seed, update_frequency=1000, start="scatter")
    elif kind == "rpm800":
        p, xyz, q, ids = workloads.rpm800(seed=seed, update_frequency=1000)
    elif kind.startswith("dhlj"):
        n, kT = kind[4:].split("@") if "@" in kind else (kind[4:], "1.0")
        p, xyz, q, ids = workloads.dh_lj_salt(int(n), seed, kT_scale=float(kT), start="scatter")
    else:
        raise ValueError(kind)
    return OracleSystem(p, xyz, q, ids), np.array([p.type_dp[i] for i in ids])


def _cpu_task(args):
    """Time-bounded sample of the oracle port on one core: chunks of trials
    until ``seconds`` of trial time have passed. Returns (trials, seconds)."""
    kind, seed, seconds = args
    from oracle.oracle import dip_stream, mol_stream, translation_stream
    key = (kind, seed)
    if key not in _cpu_cache:
        _cpu_cache[key] = _cpu_system(kind, seed) + ([0],)
    o, dpp, chunk = _cpu_cache[key]
    n, t_run = 0, 0.0
    while t_run < seconds:
        if kind == "molecules":
            st = mol_stream(seed * 100000 + chunk[0], 1000, 1.0, 0.3, True, 4)
            t0 = time.perf_counter()
            o.run_stream(st)
            k = 4
        elif kind == "dipoles":
            k = 64
            st = dip_stream(seed * 100000 + chunk[0], DIP_N, k, 0.5, DIP_DP, DIP_DPROT)
            t0 = time.perf_counter()
            o.run_stream(st)
        else:
            k = 64 if kind == "rpm16k" else 256
            idx, disp, u = translation_stream(seed * 100000 + chunk[0], dpp, k)
            t0 = time.perf_counter()
            o.mc_run_stream(idx, disp, u)
        t_run += time.perf_counter() - t0
        chunk[0] += 1
        n += k
    return n, t_run


class CpuPath:
    """The FP64 oracle port of the reference's per-trial work on every host
    core: one process per core, each its own system and seed, as independent
    reference runs would be. ``kinds`` gives each process its workload kind
    (cycled)."""

    def __init__(self, kinds, weights=None, cores=None):
        from oracle import oracle
        oracle.build()
        self.cores = cores or os.cpu_count() or 1
        self.kinds = [kinds[c % len(kinds)] for c in range(self.cores)]
        self.weights = None if weights is None else [weights[c % len(weights)] for c in range(self.cores)]
        self.pool = mp.get_context("spawn").Pool(self.cores)

    def sample(self, seconds):
        """Trial rate of all cores. Identical systems: the sum of per-process
        rates. A mix of system sizes (weights = each kind's share of the
        workload's trials): cores / (weighted mean time per trial), i.e. the
        rate at which the cores clear that mix."""
        res = self.pool.map(_cpu_task, [(k, 1000 + c, seconds) for c, k in enumerate(self.kinds)], chunksize=1)
        trials = sum(n for n, _ in res)
        if self.weights is None:
            rate = sum(n / t for n, t in res)
        else:
            tau = [t / n for n, t in res]
            rate = self.cores * sum(self.weights) / sum(w * x for w, x in zip(self.weights, tau))
        return rate, trials

    def close(self):
        self.pool.close()
        self.pool.join()

    def describe(self, seconds, trials):
        ks = sorted(set(self.kinds))
        how = ("sum of per-process trial rates" if self.weights is None else
               "cores / trial-weighted mean time per trial over the workload's size mix")
        return ("%d processes (one per host core), each its own system (%s), ~%.0f s of FP64 trials (%d in total); "
                "value = %s" % (self.cores, ", ".join(ks[:6]) + (" ..." if len(ks) > 6 else ""), seconds, trials, how))


# ----------------------------------------------------------------- the reference itself on the host
REF_HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def _ref_input(kind, seed, seconds, steps, warmup):
    """Input of the reference harness for one host process: the reference's
    own Space, energy (NonbondedEwald<WCA> or Nonbonded<DH + LJ>) and
    AtomicTranslation on the workload kind's system, time-bounded samples.
    None where the kind has no reference run here (molecules, dipoles)."""
    from beofaunus_gb300 import workloads
    kT = 1.0
    if kind == "rpm16k":
        p, xyz, q, ids = workloads.rpm16k(seed=seed, update_frequency=1000, start="scatter")
    elif kind == "rpm800":
        p, xyz, q, ids = workloads.rpm800(seed=seed, update_frequency=1000)
    elif kind.startswith("dhlj"):
        n, t = kind[4:].split("@") if "@" in kind else (kind[4:], "1.0")
        kT = float(t)
        p, xyz, q, ids = workloads.dh_lj_salt(int(n), seed, start="scatter")
    else:
        return None
    ewald = p.model == 1
    # a temperature T scales every energy by 1/T: the Bjerrum length and the
    # LJ epsilons are given at T
    types = [dict(q=p.type_charge[t], sigma=p.type_sigma[t], eps=p.type_eps[t] / kT, dp=p.type_dp[t])
             for t in range(p.n_types)]
    d = dict(mode="bench", model="ewald_wca" if ewald else "dh_lj", box=p.box[0], bjerrum=p.bjerrum / kT,
             types=types, positions=xyz.tolist(), type_ids=[int(i) for i in ids], seed=seed, sweeps=0,
             seconds=seconds, steps=steps, warmup=warmup)
    if ewald:
        d.update(alpha=p.ewald_alpha, cutoff=p.ewald_cutoff, cutoffK=p.ewald_cutoff_k, eps_surf=p.ewald_eps_surf,
                 debyelength=p.ewald_debye_length, spherical_sum=bool(p.ewald_spherical_sum),
                 update_frequency=int(p.ewald_update_frequency))
    else:
        d.update(debyelength=p.dh_debye_length)
    return d


def ref_path_available(kinds):
    return os.path.exists(REF_HARNESS) and all(not k.startswith(("molecules", "dipoles")) for k in kinds)


def ref_cpu_rates(kinds, weights, seconds, steps, warmup, cores=None):
    """The reference's own CPU path (oracle/_ref/ref_harness, the reference
    built from its sources on this machine) on every host core: one process
    per core, each its own system and seed. Returns per timed step the rate
    of all cores (identical systems: the sum of the per-process rates; a size
    mix: cores / trial-weighted mean time per trial), the total trials and
    the core count."""
    cores = cores or os.cpu_count() or 1
    ks = [kinds[c % len(kinds)] for c in range(cores)]
    ws = None if weights is None else [weights[c % len(weights)] for c in range(cores)]
    with tempfile.TemporaryDirectory() as tmp:
        procs = []
        for c, k in enumerate(ks):
            fin, fout = os.path.join(tmp, "in%d.json" % c), os.path.join(tmp, "out%d.json" % c)
            with open(fin, "w") as f:
                json.dump(_ref_input(k, 1000 + c, seconds, steps, warmup), f)
            procs.append((subprocess.Popen([REF_HARNESS, fin, fout], cwd=tmp, stdout=subprocess.DEVNULL,
                                           stderr=subprocess.DEVNULL), fout))
        rates = []
        for pr, fout in procs:
            if pr.wait(timeout=600 + 2 * (steps + warmup) * seconds) != 0:
                raise RuntimeError("reference harness failed")
            with open(fout) as f:
                rates.append(json.load(f)["rates"])
    per_step = []
    for s in range(steps):
        r = [rates[c][s] for c in range(cores)]
        if ws is None:
            per_step.append(sum(r))
        else:
            per_step.append(cores * sum(ws) / sum(w / x for w, x in zip(ws, r)))
    trials = int(sum(sum(x) for x in rates) * seconds)
    return per_step, trials, cores, sorted(set(ks))


def cpu_baseline(seconds, kinds=("rpm16k",), weights=None):
    if ref_path_available(kinds):
        vals, trials, cores, ks = ref_cpu_rates(list(kinds), weights, seconds, 1, 0)
        return {"value": vals[0], "unit": UNIT, "cores": cores, "kind": "reference",
                "sample": "the reference built from its own sources on this machine (oracle/_ref/ref_harness: "
                          "Space, NonbondedEwald<WCA> or Nonbonded<DH+LJ>, AtomicTranslation), %d processes (one "
                          "per host core), each its own system (%s), %.0f s of trials each (%d in total)"
                          % (cores, ", ".join(ks[:6]), seconds, trials)}
    cp = CpuPath(list(kinds), weights)
    try:
        cp.sample(0.2)                      # build each process's system outside the sample
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
    """DRAM bytes per trial of the Ewald block kernel from the committed ncu
    summary (a line 'dram_bytes_per_trial: <n>'), or None."""
    path = os.path.join(ROOT, "profiles", "ewald_block_kernel_rpm16k_batch.md")
    try:
        for line in open(path):
            m = re.match(r"\s*[-*]?\s*dram_bytes_per_trial:\s*([0-9.eE+]+)", line)
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
    # accuracy inside the timed run: two members log every trial's dU on the
    # device (a store per trial for 2 of the B systems); the last timed step's
    # first trials are replayed by the FP64 oracle afterwards
    chk = sorted({0, B - 1})
    for m in chk:
        batch.set_log(m)
    e64_0 = [] if args.value_only else [s_.total_energy_fp64()["total"] for s_ in systems]
    run_0 = [] if args.value_only else [s_.running_energy() for s_ in systems]

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
    stats = []
    for s in range(steps):
        if s == steps - 1:
            # start of the checked step (a host read between device-timed steps)
            chk_start = {m: systems[m].positions() for m in chk}
        stats.append(device_step(1000 + s))
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
    all_trials, max_ms = reduce_sum_max(dist, trials, dev_ms, dev)
    value = all_trials / (max_ms / 1e3)

    if args.value_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": max_ms / steps,
                              "sweep_kernel_ms": sweep_ms, "sweep_launches": launches, "trials": trials,
                              "systems": B}))
        if dist:
            dist.destroy_process_group()
        return

    # ---- accuracy of the timed run (checker: the FP64 oracle, after timing)
    accuracy = accuracy_check(systems, chk, chk_start, min(T, args.check_trials), e64_0, run_0,
                              (warm + steps) * T)
    for m in chk:
        batch.set_log(m, False)

    # ---- e2e: host streams in, scalars out, wall clock around upload + run.
    # Each step's inputs (the reference's mt19937 draws, made on the host
    # before the step) sit in pinned host memory, from which the upload copies.
    pool = cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1))
    e2e_s, e2e_trials, e2e_gathers = 0.0, 0, 0

    def pinned(shape, dt):
        return torch.empty(shape, dtype=dt, pin_memory=True).numpy()

    pin = [(pinned(T, torch.int32), pinned((T, 3), torch.float64), pinned(T, torch.float64)) for _ in range(B)]

    def stage(seed0):
        for b in range(B):
            for dst, src in zip(pin[b], systems[b].draw_translation_stream(seed0 + b, T)):
                np.copyto(dst, src.reshape(dst.shape))

    # one untimed pass first: upload buffers are allocated on first use
    stage(40000)
    list(pool.map(lambda b: batch.stream_upload(b, *pin[b]), range(B)))
    batch.run()
    for s in range(steps):
        stage(50000 + 1000 * s)
        flush.fill_(s & 0xFF)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        list(pool.map(lambda b: batch.stream_upload(b, *pin[b]), range(B)))
        _, tot = batch.run()
        e2e_s += time.perf_counter() - t0
        e2e_trials += tot["trials"]
        # every member's scalars are read back before the run and after it
        # (one launch per run: the sweep kernel rebuilds Q(k) itself); a run
        # with external rebuilds reads them once more per host check
        e2e_gathers += 2 if tot["sweep_launches"] == 1 else tot["kernel_launches"] - 1 - 3 * tot["sweep_launches"]
    pool.shutdown()
    e2e = reduce_rate(dist, e2e_trials, e2e_s, dev)

    # ---- roofline of the dominant kernel (sweep kernel), FP32 pipe
    K = systems[0].num_kvectors
    acc_rate = accepted / max(trials, 1)
    flop_per_trial = PAIRS_PER_TRIAL * FLOP_PER_PAIR + K * FLOP_PER_K + acc_rate * K * FLOP_PER_K_COMMIT
    avg_launch_s = sweep_ms / max(launches, 1) / 1e3
    trials_per_launch = trials / max(launches, 1)
    rebuilds_per_launch = rebuilds / max(launches, 1)
    flop_rebuild = N_IONS * K * FLOP_PER_TERM_REBUILD   # one rebuild of one system
    flop_per_launch = flop_per_trial * trials_per_launch + flop_rebuild * rebuilds_per_launch
    achieved = flop_per_launch / avg_launch_s / 1e12
    sm_mhz = (clk or {}).get("sm_mhz") or 1900.0
    mufu_peak = sms * 16 * sm_mhz * 1e6
    mufu_frac = PAIRS_PER_TRIAL * MUFU_PER_PAIR * trials_per_launch / avg_launch_s / mufu_peak
    per_trial = profiled_traffic()
    traffic = per_trial * trials_per_launch if per_trial is not None else None

    # ---- single chain: one system alone, on a thread-block cluster of every
    # size up to what fits (the built-in choice is the headline figure)
    p, xyz, q, ids = workloads.rpm16k(seed=seeds[B], update_frequency=1000, start=xyzs[B])
    one = System(p, xyz, q, ids)
    default_c = one.cluster
    by_cluster = {}
    c = 1
    while c <= one.max_cluster:
        one.cluster = c
        one.stream_philox(T, 7)
        one.stream_run()
        sc = []
        for s in range(2):
            one.stream_philox(T, 8 + s)
            flush.fill_(s)
            torch.cuda.synchronize()
            sc.append(one.stream_run())
        by_cluster[c] = sum(st["trials"] for st in sc) / (sum(st["device_ms"] for st in sc) / 1e3)
        c *= 2
    one.cluster = 0
    single = by_cluster[default_c]

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
        "dtype": "f32",
        "precision": "f32 pair and k terms; df (~48-bit) sums; int64 fixed-point Q(k)",
        "data": "synthetic (seeded overlap-free starts; Philox streams, reference mt19937 for e2e)",
        "config": workload_config(B, T),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": B * T * UPLOAD_BYTES_PER_TRIAL,
                "d2h_bytes_per_step": int(round(e2e_gathers / steps)) * B * SYS_SCALARS_BYTES},
        "gpu_launches": int(kernels),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": traffic,
                     "peak_source": "measured in this run: cuBLAS SGEMM 8192^3, TF32 off (best of 5)",
                     "flop_per_trial": flop_per_trial, "trials_per_launch": trials_per_launch,
                     "flop_per_rebuild": flop_rebuild, "rebuilds_per_launch": rebuilds_per_launch,
                     "mean_launch_ms": avg_launch_s * 1e3, "mufu_frac": mufu_frac,
                     "note": "one launch per step runs every system's sweep, its Q(k) rebuilds included; "
                             "pair and k-space terms are FP32 arithmetic (the 32x32 Gram matrix of a "
                             "trial block runs on the tensor cores, mma.sync TF32 x3); each system is a "
                             "sequential Markov chain on one SM"},
        "single_chain": {"value": single, "unit": UNIT, "us_per_trial": 1e6 / single, "cluster_ctas": default_c,
                         "us_per_trial_by_cluster_ctas": {str(k): 1e6 / v for k, v in by_cluster.items()}},
        "plain_per_trial_api": {"value": plain, "unit": UNIT},
        "batched_over_plain": value / plain,
        "batched_over_single_chain": value / single,
        "acceptance": acc_rate,
        "qk_rebuilds": rebuilds,
        "max_du_err": accuracy["max_du_err"],
        "accuracy": accuracy,
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


def accuracy_check(systems, members, starts, n, e64_0, run_0, trials_per_system):
    """dU error of the timed batched run against the FP64 oracle.

    For each checked member the oracle replays the first n trials of the last
    timed step (the member's Philox stream as staged, read back) from the
    member's coordinates at the start of that step; the device's own logged
    dU values of those trials are compared one by one (decisions must agree
    except inside the 1e-6 kT band). Then every system's running energy is
    compared with fg_total_energy_fp64: the drift is the difference between
    the change of the running total (the sum of accepted dU and rebuild
    corrections) and the change of the FP64 system energy since set-up."""
    import numpy as np

    from oracle.oracle import compare_chain, replay_chain
    jobs, dev = [], []
    for m in members:
        s = systems[m]
        idx, disp, u = s.stream_get(0, n)
        du, acc = s.log_get(0, n)
        dev.append((du, acc, u))
        jobs.append((bytes(s.params), starts[m], s.charges, s.type_ids, idx, disp, u))
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        ref = pool.map(replay_chain, jobs)
    res = [compare_chain(d[0], d[1], r[0], r[1], d[2], 1e-6) for d, r in zip(dev, ref)]
    drift = []
    for s, e0, r0 in zip(systems, e64_0, run_0):
        drift.append(abs((s.running_energy() - r0) - (s.total_energy_fp64()["total"] - e0)))
    return {"max_du_err": max(r["max_err"] for r in res),
            "rms_du_err": float(np.sqrt(np.mean([r["rms_err"] ** 2 for r in res]))),
            "members_checked": members, "trials_checked_per_member": n,
            "trials_compared": sum(r["compared"] for r in res),
            "decisions_identical": all(r["decisions_identical"] for r in res),
            "divergence_in_band": all(r["divergence_in_band"] for r in res),
            "checked": "the device's own logged dU of the last timed step's first trials of each checked member, "
                       "against the FP64 oracle replaying the same Philox stream from the same start",
            "max_energy_drift_kT": max(drift), "drift_systems": len(drift),
            "drift_trials_per_system": trials_per_system,
            "drift": "|change of the running total energy - change of the FP64 system energy| since set-up"}


def _pt_sizes():
    from beofaunus_gb300 import workloads
    return [int(n) for n in workloads.pt_ladder_sizes(64)]


def _serving_sizes(n_jobs, seed=5):
    import numpy as np
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(math.log(256), math.log(16384), n_jobs))
    return [int(2 * round(x / 2)) for x in n], list(rng.uniform(0.8, 2.0, n_jobs))


def cpu_kinds(workload, cores=None):
    """(kinds, weights) of the CPU path for a workload: the systems the host
    processes run and, for size mixes, each one's share of the trials (16
    quantiles of the mix; a size's trials are proportional to its N)."""
    cores = cores or os.cpu_count() or 1
    if workload in ("rpm16k", "rpm800", "molecules", "dipoles"):
        return [workload], None
    if workload == "pt64":
        sizes = sorted(_pt_sizes())
        temps = [1.0] * len(sizes)
    elif workload == "serving":
        s_, t_ = _serving_sizes(200)
        order = sorted(range(len(s_)), key=lambda i: s_[i])
        sizes, temps = [s_[i] for i in order], [t_[i] for i in order]
    else:
        raise ValueError(workload)
    k = min(cores, len(sizes))
    picks = [int((q + 0.5) * len(sizes) / k) for q in range(k)]
    kinds = ["dhlj%d@%.3f" % (sizes[i], temps[i]) for i in picks]
    # each pick stands for len(sizes)/k systems; trials per system ~ N
    weights = [float(sizes[i]) for i in picks]
    return kinds, weights


WORKLOAD_NAMES = {"rpm16k": WORKLOAD, "rpm800": "rpm800_ewald_wca_batched", "pt64": "pt64_dh_lj_ladder",
                  "molecules": "dipolar_molecules_1000x20_batched", "serving": "serving_dh_lj_poisson",
                  "dipoles": "stockmayer100_dipolar_ewald_batched"}


def base_line(metric_value, steps, warm, ms_per_step, world, config, dtype, data):
    return {"metric": METRIC, "value": metric_value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": warm,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": dtype.split()[0], "precision": dtype, "data": data, "config": config}


def gpu_setup(args):
    import torch
    from beofaunus_gb300 import build
    build.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    return torch, dev, local, torch.cuda.get_device_properties(dev).multi_processor_count


def reduce_sum_max(dist, total, slowest, device):
    """(sum over ranks of total, max over ranks of slowest); dist None = one process."""
    if dist is None:
        return float(total), float(slowest)
    import torch
    t = torch.tensor([float(total)], dtype=torch.float64, device=device)
    dist.all_reduce(t)
    m = torch.tensor([float(slowest)], dtype=torch.float64, device=device)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return t.item(), m.item()


def reduce_rate(dist, trials, seconds, device):
    """Whole-job rate over ranks (replicas only: no data-path exchange): all
    ranks' trials over the slowest rank's time."""
    n, t = reduce_sum_max(dist, trials, seconds, device)
    return n / t


def launch_ranks(n, argv):
    """bench.py --gpus N started without a launcher: run the same command as
    N ranks under torch.distributed.run on this node (rendezvous on
    127.0.0.1, a free port). Returns the launcher's exit status, which is
    non-zero when any rank failed or did not come up."""
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=%d" % n,
           "--master-addr=127.0.0.1", "--master-port=%d" % port, os.path.abspath(__file__)] + list(argv)
    return subprocess.call(cmd)


def job_dist():
    """torch.distributed when this run has more than one rank, else None."""
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1 else None


# ----------------------------------------------------------------- 800-ion Ewald
def run_rpm800(args, rank, world):
    import numpy as np
    from beofaunus_gb300 import workloads
    from beofaunus_gb300.gpu import Batch, System
    torch, dev, local, sms = gpu_setup(args)
    B = args.systems or sms
    T = args.trials or 800
    steps, warm = args.steps, args.warmup
    systems = []
    for b in range(B):
        p, xyz, q, ids = workloads.rpm_ewald(800, 60.0, 7, seed=1 + rank * 1000003 + b, update_frequency=1000,
                                             start="scatter")
        systems.append(System(p, xyz, q, ids))
    batch = Batch(systems)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def step(seed):
        batch.stream_philox([T] * B, seed)
        flush.fill_(seed & 0xFF)
        torch.cuda.synchronize()
        return batch.run()[1]

    for s_ in range(warm):
        step(10 + s_)
    clocks = ClockSampler(local)
    clocks.start()
    stats = [step(1000 + s_) for s_ in range(steps)]
    clk = clocks.stop()
    ms = sum(st["device_ms"] for st in stats)
    trials = sum(st["trials"] for st in stats)
    value = reduce_rate(job_dist(), trials, ms / 1e3, dev)
    # e2e: host mt19937 streams in, scalars out (800-trial streams: a thread
    # pool costs more than it saves here)
    e2e_s, e2e_t = 0.0, 0
    for b in range(B):   # one untimed pass first: upload buffers are allocated on first use
        batch.stream_upload(b, *systems[b].draw_translation_stream(6000 + b, T))
    batch.run()
    for s_ in range(steps):
        host = [systems[b].draw_translation_stream(7000 + 100 * s_ + b, T) for b in range(B)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for b in range(B):
            batch.stream_upload(b, *host[b])
        _, tot = batch.run()
        e2e_s += time.perf_counter() - t0
        e2e_t += tot["trials"]
    one = systems[0]
    one.stream_philox(4 * T, 5)
    r1 = one.stream_run()
    single = r1["trials"] / (r1["device_ms"] / 1e3)
    idx, disp, u = one.draw_translation_stream(777, 300)
    pos = one.positions()
    t0 = time.perf_counter()
    for t in range(300):
        i = int(idx[t])
        new = pos[i] + disp[t]
        new -= 60.0 * np.round(new / 60.0)
        du = one.trial_du(i, new)
        acc = not (u[t] > np.exp(-du))
        one.commit(acc)
        if acc:
            pos[i] = new
    plain = 300 / (time.perf_counter() - t0)
    cfg = {"workload": WORKLOAD_NAMES["rpm800"], "systems": B, "n_particles_per_system": 800, "box_A": 60.0,
           "ewald": {"alpha": 0.2, "cutoff_A": 20.0, "kvectors": systems[0].num_kvectors, "n2_max": 49,
                     "update_frequency": 1000}, "trials_per_system_per_step": T,
           "l2": "L2 flushed (256 MiB write) between timed steps"}
    out = base_line(value, steps, warm, ms / steps, world, cfg, "f32 pair and k terms; df sums; int64 Q(k)",
                    "synthetic (seeded overlap-free starts)")
    out.update({"e2e": {"value": reduce_rate(job_dist(), e2e_t, e2e_s, dev), "unit": UNIT, "h2d_bytes_per_step": B * T * UPLOAD_BYTES_PER_TRIAL,
                        "d2h_bytes_per_step": B * SYS_SCALARS_BYTES * 2},
                "gpu_launches": int(sum(st["kernel_launches"] for st in stats)),
                "single_chain": {"value": single, "unit": UNIT}, "plain_per_trial_api": {"value": plain, "unit": UNIT},
                "batched_over_plain": value / plain, "clocks": clk})
    batch.close()
    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds, *cpu_kinds("rpm800"))
    if rank == 0:
        print(json.dumps(out))


# ----------------------------------------------------------------- parallel tempering
def run_pt(args, rank, world):
    from beofaunus_gb300 import workloads
    from beofaunus_gb300.gpu import Batch, System
    torch, dev, local, sms = gpu_setup(args)
    sizes = _pt_sizes()
    temps = workloads.pt_temperatures(64)
    sweeps = args.pt_sweeps
    systems = []
    for r, n in enumerate(sizes):
        p, xyz, q, ids = workloads.dh_lj_salt(n, 100 + r + rank * 1000003, start="scatter")
        systems.append(System(p, xyz, q, ids))
    batch = Batch(systems)
    # the schedule (least particles per CTA) chosen by the autotuner on
    # clones of the 64 replicas, before any timing
    tune = batch.autotune(args.tune_trials) if args.tune_trials else None
    batch.pt_setup(temps, 1234 + rank)
    steps, warm = args.steps, args.warmup
    for _ in range(warm):
        batch.pt_run(1, sweeps)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    stats = [batch.pt_run(1, sweeps) for _ in range(steps)]
    clk = clocks.stop()
    ms = sum(st["device_ms"] for st in stats)
    trials = sum(st["trials"] for st in stats)
    value = reduce_rate(job_dist(), trials, ms / 1e3, dev)
    state = batch.pt_state()
    acc_swaps = [int(a) for a in state["accepts"][:63]]
    att_swaps = [int(a) for a in state["attempts"][:63]]
    # largest replica alone: the bound of one fused launch over uneven sizes
    big = int(max(range(64), key=lambda r: sizes[r]))
    cfg = {"workload": WORKLOAD_NAMES["pt64"], "replicas": 64, "n_min": min(sizes), "n_max": max(sizes),
           "n_total": sum(sizes), "density_per_A3": 0.002, "debye_length_A": 10.0, "lj_sigma_A": 4.0,
           "lj_eps_kT": 0.2, "temperatures": [0.8, 2.0], "sweeps_per_swap": sweeps,
           "launch": "one graph per round: Philox draws, persistent sweep over all replicas, swap kernel",
           "autotune": tune}
    out = base_line(value, steps, warm, ms / steps, world, cfg, "f32 pair terms; df sums",
                    "synthetic (seeded overlap-free starts, Philox streams)")
    out.update({"gpu_launches": int(sum(st["kernel_launches"] for st in stats)),
                "swap_acceptance": sum(acc_swaps) / max(sum(att_swaps), 1),
                "largest_replica": sizes[big], "clocks": clk,
                "e2e": None})
    # e2e: the same rounds driven through the host stream path are the batch
    # e2e of the other workloads; for PT every input is generated on the
    # device, so the end-to-end line is the round plus the state read-back.
    t0 = time.perf_counter()
    for _ in range(steps):
        batch.pt_run(1, sweeps)
        batch.pt_state()
    e2e_s = time.perf_counter() - t0
    out["e2e"] = {"value": trials / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 0,
                  "d2h_bytes_per_step": 64 * (4 + 8 + 8 + 8)}
    batch.close()
    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds, *cpu_kinds("pt64"))
    if rank == 0:
        print(json.dumps(out))


# ----------------------------------------------------------------- rigid dipolar molecules
def _mol_system(seed):
    from beofaunus_gb300 import workloads
    return workloads.dipolar_molecules(1000, seed=seed)


# Cost model of one molecule trial (algorithmic FP32 work, FMA = 2 FLOP), per
# position (old and new) of each of the 20 moved sites:
#   LJ against every other site (no cutoff in LennardJonesLB): distance,
#     r^2, 1/r^2, (s/r)^6, 4eps(x^2 - x): 15 FLOP;
#   ion-dipole (no cutoff in IonDipole) for pairs with a dipole: the moved
#     molecule's dipole against every other site plus every moved site
#     against every other dipole: 20 FLOP more;
#   inside rc = 15 A (about 84 sites per moved site at this density):
#     Coulomb Q5/r and the reaction-field dipole-dipole: 40 FLOP more.
MOL_LJ_FLOP, MOL_ID_FLOP, MOL_NEAR_FLOP, MOL_NEAR_SITES = 15, 20, 40, 84


def mol_flop_per_trial(n_sites=20000, n_dipoles=1000, gs=20):
    lj = 2 * gs * (n_sites - gs) * MOL_LJ_FLOP
    idp = 2 * ((n_sites - gs) + gs * (n_dipoles - 1)) * MOL_ID_FLOP
    near = 2 * gs * MOL_NEAR_SITES * MOL_NEAR_FLOP
    return lj + idp + near


def run_molecules(args, rank, world):
    import numpy as np
    from beofaunus_gb300.gpu import MolSystem, mol_draw_stream, mol_run_many
    torch, dev, local, sms = gpu_setup(args)
    C = args.cluster
    B = args.systems or max(1, sms // C)
    T = args.trials or 1000
    steps, warm = args.steps, args.warmup
    with mp.get_context("spawn").Pool(min(B, os.cpu_count() or 1)) as pool:
        data = pool.map(_mol_system, [11 + rank * 1000003 + b for b in range(B)])
    systems = []
    for b, (p, xyz, mu, mus, ids) in enumerate(data):
        s_ = MolSystem(p, xyz, mu, mus, ids, 20, cluster=C)
        systems.append(s_)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def step(seed):
        for b, s_ in enumerate(systems):
            s_.stream_upload(mol_draw_stream(seed * 1000 + b, 1000, T, 1.0, 0.3, True))
        flush.fill_(seed & 0xFF)
        torch.cuda.synchronize()
        return mol_run_many(systems)[1]

    for s_ in range(warm):
        step(10 + s_)
    clocks = ClockSampler(local)
    clocks.start()
    stats = [step(1000 + s_) for s_ in range(steps)]
    clk = clocks.stop()
    ms = sum(st["device_ms"] for st in stats)
    trials = sum(st["trials"] for st in stats)
    value = reduce_rate(job_dist(), trials, ms / 1e3, dev)
    # e2e: host draws (the reference's mt19937) uploaded inside the timed region
    e2e_s, e2e_t = 0.0, 0
    for s_ in range(steps):
        host = [mol_draw_stream(50000 + 100 * s_ + b, 1000, T, 1.0, 0.3, True) for b in range(B)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for b, s2 in enumerate(systems):
            s2.stream_upload(host[b])
        _, tot = mol_run_many(systems)
        e2e_s += time.perf_counter() - t0
        e2e_t += tot["trials"]
    # one system alone on the largest cluster: the single-system latency
    one = systems[0]
    single = {}
    for c in sorted({one.max_cluster, C}):
        one.cluster = c
        st = mol_draw_stream(99, 1000, 2000, 1.0, 0.3, True)
        one.sweep(st, log=False)
        r = one.sweep(mol_draw_stream(98, 1000, 2000, 1.0, 0.3, True), log=False)
        single["cluster_%d" % c] = {"value": r["trials"] / (r["device_ms"] / 1e3), "unit": UNIT,
                                    "us_per_trial": r["device_ms"] * 1e3 / r["trials"]}
    one.cluster = C
    # plain per-trial path: host-computed rotation + fg_mol_trial_du + fg_mol_commit
    xyz, mu, cm = one.state()
    L = 150.0
    st = mol_draw_stream(77, 1000, 200, 1.0, 0.3, True)
    t0 = time.perf_counter()
    for k in range(200):
        g = int(st["group"][k])
        sl = slice(20 * g, 20 * g + 20)
        ax, ang = st["axis"][k], st["angle"][k]
        K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
        R = np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K
        off = xyz[sl] - cm[g]
        off -= L * np.round(off / L)
        new = cm[g] + off @ R.T + st["trans"][k]
        new -= L * np.round(new / L)
        newmu = mu[sl] @ R.T
        newcm = cm[g] + st["trans"][k]
        newcm -= L * np.round(newcm / L)
        du = one.trial_du(g, new, newmu, newcm)
        acc = not (st["u"][k] > np.exp(-du))
        one.commit(acc)
        if acc:
            xyz[sl], mu[sl], cm[g] = new, newmu, newcm
    plain = 200 / (time.perf_counter() - t0)
    # roofline (FP32): algorithmic FLOP per trial (cost model above)
    flop = mol_flop_per_trial()
    achieved = flop * value / 1e12
    fp32_peak = fp32_gemm_tflops(torch, dev)
    cfg = {"workload": WORKLOAD_NAMES["molecules"], "systems": B, "ctas_per_system": C, "molecules_per_system": 1000,
           "sites_per_molecule": 20, "box_A": 150.0, "site_sigma_A": 3.5, "lj_eps_kT": 0.2, "dipole_eA": 1.5,
           "rf_cutoff_A": 15.0, "eps_rf": 1e11, "dp_A": 1.0, "drot_rad": 0.3, "trials_per_system_per_step": T,
           "l2": "L2 flushed (256 MiB write) between timed steps"}
    out = base_line(value, steps, warm, ms / steps, world, cfg,
                    "f32 pair terms; exact int64 r^2 differences near; FP64 rigid rotation; df sums",
                    "synthetic (seeded molecules, reference mt19937 TranslateRotate draws)")
    out.update({"e2e": {"value": reduce_rate(job_dist(), e2e_t, e2e_s, dev), "unit": UNIT, "h2d_bytes_per_step": B * T * 80,
                        "d2h_bytes_per_step": B * 48},
                "gpu_launches": int(sum(st["kernel_launches"] for st in stats)),
                "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                             "frac": achieved / fp32_peak, "traffic": None,
                             "peak_source": "measured in this run: cuBLAS SGEMM 8192^3, TF32 off (best of 5)",
                             "flop_per_trial": flop,
                             "note": "whole-launch rate over all systems; each system is one sequential chain"},
                "single_system": single, "plain_per_trial_api": {"value": plain, "unit": UNIT},
                "batched_over_plain": value / plain, "clocks": clk})
    for s_ in systems:
        s_.close()
    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds, *cpu_kinds("molecules"))
    if rank == 0:
        print(json.dumps(out))


# ----------------------------------------------------------------- point dipoles under Ewald
# The reference's Stockmayer example's shape (stockmayer.json): 100 LJ point
# dipoles, |mu| 1.652 e A, sigma 2.8863 A, eps 1.97 kJ/mol, L 29.6336 A,
# T 315.8 K (lB 529 A), dp 0.7 A, dprot 270 deg, AtomicRotation and
# AtomicTranslation with equal probability; full dipolar Ewald (alpha
# 0.25 / A, real-space cutoff 14.42 A, spherical kc 7: 783 k-vectors,
# tin-foil surroundings).
DIP_N, DIP_DP, DIP_DPROT = 100, 0.7, 270.0 * math.pi / 180.0


def dipole_fluid(seed):
    from beofaunus_gb300 import workloads
    from beofaunus_gb300.params import FG_EWALD_DIPOLE_DIPOLE
    return workloads.dipolar_fluid(n=DIP_N, seed=seed, kc=7.0, terms=FG_EWALD_DIPOLE_DIPOLE, quirk=0)


# Cost model of one trial (algorithmic FP64 work, FMA = 2 FLOP; erfc and exp
# counted as 20 FLOP each), old and new position of the moved particle:
#   every other particle: distance and LJ, 15 FLOP;
#   inside rc (the fraction 4/3 pi rc^3 / V of pairs): erfc, exp, sqrt and
#     the T1/T2 dipole-dipole terms, 80 FLOP more;
#   per k-vector: two three-factor phase products (24), k.mu twice (12), the
#     Q increments (8) and the energy change (12): 56 FLOP.
DIP_PAIR_FLOP, DIP_NEAR_FLOP, DIP_K_FLOP = 15, 80, 56


def dip_flop_per_trial(n, K, rc, box):
    near = min(1.0, 4.0 / 3.0 * math.pi * rc ** 3 / box ** 3)
    return 2 * (n - 1) * (DIP_PAIR_FLOP + near * DIP_NEAR_FLOP) + K * DIP_K_FLOP


def fp64_gemm_tflops(torch, dev):
    """Measured FP64 peak: cuBLAS DGEMM 4096^3, best of 5."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    best = 0.0
    for _ in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * 4096 ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12)
    return best


def run_dipoles(args, rank, world):
    from beofaunus_gb300.gpu import DipoleSystem, dip_autotune, dip_draw_stream, dip_run_many
    torch, dev, local, sms = gpu_setup(args)
    B = args.systems or 4 * sms
    T = args.trials or 2000
    steps, warm = args.steps, args.warmup
    with mp.get_context("spawn").Pool(min(B, os.cpu_count() or 1)) as pool:
        data = pool.map(dipole_fluid, [21 + rank * 1000003 + b for b in range(B)])
    systems = [DipoleSystem(p, xyz, mu, mus, ids, charges=q, threads=args.dip_threads or None)
               for (p, xyz, mu, mus, ids, q) in data]
    # threads per system: the autotuner's choice on clones of these systems
    # (untimed), unless given
    tune = dip_autotune(systems, 256) if not args.dip_threads else None
    threads = tune["chosen"] if tune else args.dip_threads
    p0 = data[0][0]
    K = systems[0].num_kvectors
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def draws(seed, b):
        return dip_draw_stream(seed * 1000 + b, DIP_N, T, 0.5, DIP_DP, DIP_DPROT)

    def step(seed):
        for b, s_ in enumerate(systems):
            s_.stream_upload(draws(seed, b))
        flush.fill_(seed & 0xFF)
        torch.cuda.synchronize()
        return dip_run_many(systems)[1]

    for s_ in range(warm):
        step(10 + s_)
    clocks = ClockSampler(local)
    clocks.start()
    stats = [step(1000 + s_) for s_ in range(steps)]
    clk = clocks.stop()
    ms = sum(st["device_ms"] for st in stats)
    trials = sum(st["trials"] for st in stats)
    value = reduce_rate(job_dist(), trials, ms / 1e3, dev)
    acc = sum(st["accepted"] for st in stats) / trials
    # e2e: the reference's draws made on the host and uploaded inside the
    # timed region (trial records built and copied from a thread pool)
    e2e_s, e2e_t = 0.0, 0
    pool = cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1))
    for s_ in range(steps):
        host = [draws(50000 + s_, b) for b in range(B)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        list(pool.map(lambda b: systems[b].stream_upload(host[b]), range(B)))
        _, tot = dip_run_many(systems)
        e2e_s += time.perf_counter() - t0
        e2e_t += tot["trials"]
    pool.shutdown()
    # one system alone: the single-chain latency (a whole CTA of 256 threads)
    one = systems[0]
    one.set_threads(256)
    one.sweep(dip_draw_stream(99, DIP_N, 2000, 0.5, DIP_DP, DIP_DPROT), log=False)
    r = one.sweep(dip_draw_stream(98, DIP_N, 4000, 0.5, DIP_DP, DIP_DPROT), log=False)
    single = {"value": r["trials"] / (r["device_ms"] / 1e3), "unit": UNIT,
              "us_per_trial": r["device_ms"] * 1e3 / r["trials"], "threads": 256}
    # plain per-trial API: fg_dip_trial_du + fg_dip_commit per trial
    import numpy as np
    xyz, mu = one.state()
    st = dip_draw_stream(77, DIP_N, 300, 0.5, DIP_DP, DIP_DPROT)
    L = p0.box[0]
    t0 = time.perf_counter()
    for k in range(300):
        i = int(st["idx"][k])
        nx, nm = xyz[i].copy(), mu[i].copy()
        if st["kind"][k] == 1:
            ax, ang = st["axis"][k], st["angle"][k]
            Km = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
            nm = (np.eye(3) + np.sin(ang) * Km + (1 - np.cos(ang)) * Km @ Km) @ nm
        else:
            nx = nx + st["disp"][k]
            nx -= L * np.round(nx / L)
        du = one.trial_du(i, nx, nm)
        a = not (st["u"][k] > np.exp(-du))
        one.commit(a)
        if a:
            xyz[i], mu[i] = nx, nm
    plain = 300 / (time.perf_counter() - t0)
    flop = dip_flop_per_trial(DIP_N, K, p0.ewald_cutoff, L)
    achieved = flop * value / 1e12
    fp32_peak = fp32_gemm_tflops(torch, dev)
    fp64_peak = fp64_gemm_tflops(torch, dev)
    cfg = {"workload": WORKLOAD_NAMES["dipoles"], "systems": B, "threads_per_system": threads, "autotune": tune,
           "particles_per_system": DIP_N, "box_A": L,
           "dipole_eA": 1.652, "sigma_A": 2.8863, "lj_eps_kT": float(p0.type_eps[0]), "bjerrum_A": p0.bjerrum,
           "ewald_alpha": p0.ewald_alpha, "ewald_cutoff_A": p0.ewald_cutoff, "ewald_cutoff_k": p0.ewald_cutoff_k,
           "k_vectors": K, "terms": "dipole-dipole (real + reciprocal + surface + self)",
           "dp_A": DIP_DP, "dprot_rad": DIP_DPROT, "p_rotate": 0.5, "trials_per_system_per_step": T,
           "acceptance": acc, "l2": "L2 flushed (256 MiB write) between timed steps"}
    out = base_line(value, steps, warm, ms / steps, world, cfg, "f64 near pairs, double-float k-space, f32 far pairs",
                    "synthetic (seeded dipolar fluid, reference mt19937 AtomicRotation/AtomicTranslation draws)")
    out.update({"e2e": {"value": reduce_rate(job_dist(), e2e_t, e2e_s, dev), "unit": UNIT, "h2d_bytes_per_step": B * T * 72,
                        "d2h_bytes_per_step": B * 2 * 96},
                "gpu_launches": int(sum(st["kernel_launches"] for st in stats)),
                "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                             "frac": achieved / fp32_peak, "traffic": None,
                             "peak_source": "measured in this run: cuBLAS SGEMM 8192^3, TF32 off (best of 5)",
                             "flop_per_trial": flop, "fp64_peak_dgemm": fp64_peak,
                             "achieved_over_fp64_peak": achieved / fp64_peak,
                             "note": "mixed precision: near pairs FP64, phase tables and k-space in double-float "
                                     "and far pairs in FP32; whole-launch rate over all systems, each system one "
                                     "sequential chain"},
                "single_system": single, "plain_per_trial_api": {"value": plain, "unit": UNIT},
                "batched_over_plain": value / plain, "clocks": clk})
    for s_ in systems:
        s_.close()
    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds, *cpu_kinds("dipoles"))
    if rank == 0:
        print(json.dumps(out))


# ----------------------------------------------------------------- serving
def _serving_job(args):
    n, temp, seed = args
    from beofaunus_gb300 import workloads
    return workloads.dh_lj_salt(n, seed, kT_scale=temp, start="scatter")


def run_serving(args, rank, world):
    """Poisson job stream through the continuous-batching server. Each job is
    a DH+LJ salt with N log-uniform in [256, 16384], its own temperature in
    [0.8, 2.0] and seed, running ``--job-sweeps`` sweeps. The named 2000
    sweeps per job cost about 2000 x 200 x E[N^2] = 1.3e13 pair terms for the
    200-job mix (hours of GPU time), so the default is 20 and a run with
    fewer than 2000 carries the job length in config.workload.
    Capacity is measured first with every job submitted at once; the timed
    run then feeds the same job mix at 80 % of that capacity."""
    import numpy as np
    from beofaunus_gb300.gpu import Server
    torch, dev, local, sms = gpu_setup(args)
    n_jobs = args.jobs
    sizes, temps = _serving_sizes(n_jobs, seed=5 + rank)
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        jobs = pool.map(_serving_job, [(n, t, 100 + i) for i, (n, t) in enumerate(zip(sizes, temps))])
    sweeps = args.job_sweeps
    budget = int(args.serve_gib * (1 << 30))
    # the server's schedule threshold comes from the autotuner, timed on a
    # batch of clones of the first 64 jobs (the process keeps the choice)
    tune = None
    if args.tune_trials:
        from beofaunus_gb300.gpu import Batch, System
        sample = [System(*jobs[j]) for j in range(min(64, n_jobs))]
        tb = Batch(sample)
        tune = tb.autotune(args.tune_trials)
        tb.close()
        for x in sample:
            x.close()

    def run_stream(arrivals):
        srv = Server(budget, round_pairs=args.round_pairs)
        t0 = time.perf_counter()
        submitted, finish, ids = 0, {}, {}
        order = list(range(n_jobs))
        dev_ms = 0.0
        while len(finish) < n_jobs:
            now = time.perf_counter() - t0
            while submitted < n_jobs and arrivals[submitted] <= now:
                j = order[submitted]
                p, xyz, q, ids_ = jobs[j]
                ids[srv.submit(p, xyz, q, ids_, 1000 + j, sweeps * len(ids_))] = j
                submitted += 1
            if len(ids) == len(finish):
                time.sleep(max(0.0, min(arrivals[submitted] - now, 0.01)) if submitted < n_jobs else 0)
                continue
            running, fin, ms = srv.step()
            dev_ms += ms
            tnow = time.perf_counter() - t0
            for jid, j in ids.items():
                if j in finish:
                    continue
                if srv.poll(jid)["state"] >= 2:
                    finish[j] = tnow
                    srv.release(jid)
        srv.close()
        return finish, time.perf_counter() - t0, dev_ms

    total_trials = sweeps * sum(sizes)
    # capacity: everything submitted at t = 0; the sustained completion rate
    # between 10 % and 70 % of the jobs done (the start-up and the drain, where
    # the GPU holds few jobs, are left out)
    fin0, span0, _ = run_stream([0.0] * n_jobs)
    f = sorted(fin0.values())
    i10, i70 = int(0.1 * n_jobs), int(0.7 * n_jobs)
    capacity = (i70 - i10) / max(f[i70] - f[i10], 1e-9)
    rate = 0.8 * capacity
    rng = np.random.default_rng(11)
    arrivals = list(np.cumsum(rng.exponential(1.0 / rate, n_jobs)))
    clocks = ClockSampler(local)
    clocks.start()
    finish, span, dev_ms = run_stream(arrivals)
    clk = clocks.stop()
    lat = np.array([finish[j] - arrivals[j] for j in range(n_jobs)])
    value = total_trials / span
    # the named job length is 2000 sweeps; a run with fewer says so in its name
    wname = WORKLOAD_NAMES["serving"] + ("" if sweeps == 2000 else "_%dsweeps_per_job" % sweeps)
    cfg = {"workload": wname, "jobs": n_jobs, "n_range": [256, 16384],
           "temperature_range": [0.8, 2.0], "sweeps_per_job": sweeps, "sweeps_per_job_named": 2000,
           "arrival": "Poisson at 0.8 x measured capacity", "capacity_jobs_per_s": capacity,
           "capacity_definition": "completions per s between 10% and 70% of jobs done, all submitted at t=0",
           "all_at_once_makespan_s": span0,
           "device_budget_GiB": args.serve_gib, "round_pairs": args.round_pairs, "autotune": tune}
    out = base_line(value, 1, 1, 1e3 * span, world, cfg, "f32 pair terms; df sums",
                    "synthetic (seeded overlap-free starts, Philox streams per job)")
    out.update({"latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                              "mean": float(lat.mean()), "max": float(lat.max())},
                "device_busy_frac": dev_ms / 1e3 / span, "clocks": clk,
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": int(sum(24 * n + 16 for n in sizes)),
                        "d2h_bytes_per_step": int(sum(24 * n for n in sizes))}})
    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds, *cpu_kinds("serving"))
    if rank == 0:
        print(json.dumps(out))


def run_reference(args):
    """The reference's CPU path on the host cores: the reference itself,
    built from its sources on this machine (oracle/_ref/ref_harness) where
    the workload has a reference run here, else the FP64 oracle port."""
    warm, steps = args.warmup, args.steps
    kinds, weights = cpu_kinds(args.workload)
    if ref_path_available(kinds):
        vals, trials, cores, ks = ref_cpu_rates(kinds, weights, args.ref_seconds, steps, warm)
        value = statistics.mean(vals)
        cfg = workload_config(cores, "time-bounded sample per step") if args.workload == "rpm16k" else \
            {"workload": WORKLOAD_NAMES[args.workload], "systems": cores, "per_step": "time-bounded sample"}
        out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
               "steps": steps, "warmup": warm, "ms_per_step": 1e3 * args.ref_seconds,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic (seeded overlap-free starts, the reference's own mt19937 stream)",
               "config": cfg,
               "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "reference",
                                "sample": "the reference built from its own sources on this machine "
                                          "(oracle/_ref/ref_harness), %d processes (one per host core), each "
                                          "its own system (%s); per step %.1f s of trials per process, %d "
                                          "trials in all" % (cores, ", ".join(ks[:6]), args.ref_seconds, trials)},
               "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return
    cp = CpuPath(*cpu_kinds(args.workload))
    try:
        cp.sample(0.2)
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
    cfg = workload_config(cp.cores, "time-bounded sample per step") if args.workload == "rpm16k" else \
        {"workload": WORKLOAD_NAMES[args.workload], "systems": cp.cores, "per_step": "time-bounded sample"}
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": steps, "warmup": warm, "ms_per_step": 1e3 * args.ref_seconds,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded overlap-free starts, reference mt19937 stream)",
           "config": cfg,
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
    ap.add_argument("--workload", default="rpm16k", choices=["rpm16k", "rpm800", "pt64", "molecules", "serving",
                                                                 "dipoles"])
    ap.add_argument("--systems", type=int, default=0, help="systems per GPU (default: SM count, or SMs / cluster)")
    ap.add_argument("--trials", type=int, default=0, help="trials per system per step (default: one sweep)")
    ap.add_argument("--cluster", type=int, default=4, help="molecules: CTAs per system")
    ap.add_argument("--pt-sweeps", type=int, default=100, help="pt64: sweeps between swaps")
    ap.add_argument("--jobs", type=int, default=200, help="serving: jobs in the stream")
    ap.add_argument("--job-sweeps", type=int, default=20, help="serving: sweeps per job")
    ap.add_argument("--serve-gib", type=float, default=8.0, help="serving: device budget for jobs")
    ap.add_argument("--round-pairs", type=int, default=1 << 24, help="serving: pair evaluations per job per round")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample per core")
    ap.add_argument("--ref-seconds", type=float, default=3.0, help="reference arm: seconds per step")
    ap.add_argument("--dip-threads", type=int, default=0,
                    help="dipoles: threads per system (one CTA); 0 = the autotuner's choice")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--tune-trials", type=int, default=512,
                    help="pt64/serving: trials per member per autotuner candidate (0: no tuning)")
    ap.add_argument("--value-only", action="store_true", help="device-resident value only (profiling)")
    ap.add_argument("--check-trials", type=int, default=3000,
                    help="rpm16k: trials per checked member replayed by the FP64 oracle after timing")
    args = ap.parse_args()
    if args.gpus < 1:
        raise SystemExit("--gpus must be at least 1")
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # outside a launcher: start the N ranks here (one process per GPU)
        sys.exit(launch_ranks(args.gpus, sys.argv[1:]))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world != args.gpus:
        raise SystemExit("bench.py --gpus %d is running with %d ranks" % (args.gpus, world))
    if args.impl == "reference":
        if world > 1:
            # every rank must have come up; rank 0 alone then runs the host path
            import torch.distributed as dist
            dist.init_process_group("gloo")
            dist.barrier()
        if rank == 0:
            run_reference(args)
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return
    if args.workload == "rpm16k":
        args.trials = args.trials or N_IONS
        run_ours(args, rank, world)
    else:
        if world > 1:
            import torch.distributed as dist
            import torch
            dist.init_process_group("nccl", device_id=torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0"))))
        {"rpm800": run_rpm800, "pt64": run_pt, "molecules": run_molecules, "serving": run_serving,
         "dipoles": run_dipoles}[args.workload](
            args, rank, world)


if __name__ == "__main__":
    main()
