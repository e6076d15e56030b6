"""Generate the golden fixtures in this folder from the reference itself.

Runs the reference harness (oracle/ref/ref_harness.cpp, linked against the
reference library built from its own sources by oracle/ref/Makefile) on
seeded synthetic systems and stores what the reference computed: per-trial
particle index, trial position, dU and acceptance, plus the total energies
before and after. Needs the reference checkout; the committed .npz files are
what the tests read.

    python tests/golden/make_golden.py [--ref /root/reference]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from beofaunus_gb300 import workloads  # noqa: E402


def harness_input(mode, params, xyz, ids, seed, sweeps, model):
    types = []
    for t in range(params.n_types):
        types.append(dict(q=params.type_charge[t], sigma=params.type_sigma[t], eps=params.type_eps[t],
                          dp=params.type_dp[t]))
    d = dict(mode=mode, model=model, box=params.box[0], bjerrum=params.bjerrum, types=types,
             positions=xyz.tolist(), type_ids=[int(i) for i in ids], seed=seed, sweeps=sweeps)
    if model == "ewald_wca":
        d.update(alpha=params.ewald_alpha, cutoff=params.ewald_cutoff, cutoffK=params.ewald_cutoff_k,
                 eps_surf=params.ewald_eps_surf, debyelength=params.ewald_debye_length,
                 spherical_sum=bool(params.ewald_spherical_sum),
                 update_frequency=int(params.ewald_update_frequency))
    else:
        d.update(debyelength=params.dh_debye_length)
    return d


def run_harness(exe, d):
    with tempfile.TemporaryDirectory() as tmp:
        fin, fout = os.path.join(tmp, "in.json"), os.path.join(tmp, "out.json")
        with open(fin, "w") as f:
            json.dump(d, f)
        subprocess.check_call([exe, fin, fout], cwd=tmp, stdout=subprocess.DEVNULL)
        with open(fout) as f:
            return json.load(f)


CASES = {
    # name: (builder, model, seed, sweeps)
    "ewald_small_uf1": (lambda: workloads.rpm_ewald(64, 20.0, 5, seed=11, update_frequency=-1, alpha=0.35,
                                                    cutoff=9.5), "ewald_wca", 101, 2),
    "ewald_surface_uf5": (lambda: workloads.rpm_ewald(200, 32.0, 6, seed=12, update_frequency=5,
                                                      eps_surf=1.0, cutoff=15.0), "ewald_wca", 102, 1),
    "ewald_rpm800": (lambda: workloads.rpm800(seed=13, update_frequency=1000), "ewald_wca", 103, 1),
    "dhlj_small": (lambda: workloads.dh_lj_salt(300, seed=14, density=0.004), "dh_lj", 104, 2),
    "dhlj_500": (lambda: workloads.dh_lj_salt(500, seed=15), "dh_lj", 105, 1),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "REF=" + a.ref])
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_harness")

    known = run_harness(exe, dict(mode="ewald_known"))
    np.savez_compressed(os.path.join(HERE, "ewald_known.npz"),
                        **{k: np.asarray(v, dtype=np.float64) for k, v in known.items()})
    print("ewald_known", {k: v[0] for k, v in known.items()})

    for name, (builder, model, seed, sweeps) in CASES.items():
        if a.only and name != a.only:
            continue
        params, xyz, q, ids = builder()
        out = run_harness(exe, harness_input("mc", params, xyz, ids, seed, sweeps, model))
        n = len(out["idx"])
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            params=np.frombuffer(bytes(params), dtype=np.uint8), xyz=xyz, q=q, ids=ids,
            seed=np.int64(seed), sweeps=np.int64(sweeps), bjerrum=np.float64(out["bjerrum"][0]),
            u0=np.float64(out["u0"][0]), u1=np.float64(out["u1"][0]),
            u_move_sum=np.float64(out["u_move_sum"][0]),
            idx=np.asarray(out["idx"], dtype=np.int32),
            trial_xyz=np.asarray(out["trial_xyz"]).reshape(n, 3),
            du=np.asarray(out["du"]), acc=np.asarray(out["acc"], dtype=np.uint8),
            final_positions=np.asarray(out["final_positions"]).reshape(-1, 3))
        print(name, "trials", n, "acceptance %.3f" % np.mean(out["acc"]), "u0 %.6f" % out["u0"][0])


if __name__ == "__main__":
    main()
