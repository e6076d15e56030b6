"""Generate the golden fixtures in this folder from the reference itself.

Runs the reference harnesses (oracle/ref/ref_harness.cpp,
ref_harness_mol.cpp, ref_harness_dip.cpp and ref_harness_pt.cpp, linked against the reference library built from its own
sources by oracle/ref/Makefile) on seeded synthetic systems and stores what
the reference computed: per-trial particle (or molecule) index, trial
position, dU and acceptance, plus the total energies before and after. Needs
the reference checkout; the committed .npz files are what the tests read.

    python tests/golden/make_golden.py [--ref <reference checkout>]

(default: oracle/refdir.py's lookup: $FG_REFERENCE_DIR, else the staged copy
in baseline/_ref/faunus)
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
                 isotropic_pbc=bool(params.ewald_isotropic_pbc),
                 update_frequency=int(params.ewald_update_frequency))
    else:
        d.update(debyelength=params.dh_debye_length)
    return d


def isotropic(spec):
    """The same system with NonbondedEwald's isotropic_pbc on."""
    params, xyz, q, ids = spec
    params.ewald_isotropic_pbc = 1
    return params, xyz, q, ids


def run_harness(exe, d, files=()):
    """Run a harness on input d; with files, also return the contents of
    those files the harness wrote in its working directory."""
    with tempfile.TemporaryDirectory() as tmp:
        fin, fout = os.path.join(tmp, "in.json"), os.path.join(tmp, "out.json")
        with open(fin, "w") as f:
            json.dump(d, f)
        subprocess.check_call([exe, fin, fout], cwd=tmp, stdout=subprocess.DEVNULL)
        with open(fout) as f:
            out = json.load(f)
        if not files:
            return out
        return out, [open(os.path.join(tmp, x), "rb").read() for x in files]


CASES = {
    # name: (builder, model, seed, sweeps)
    "ewald_small_uf1": (lambda: workloads.rpm_ewald(64, 20.0, 5, seed=11, update_frequency=-1, alpha=0.35,
                                                    cutoff=9.5), "ewald_wca", 101, 2),
    "ewald_surface_uf5": (lambda: workloads.rpm_ewald(200, 32.0, 6, seed=12, update_frequency=5,
                                                      eps_surf=1.0, cutoff=15.0), "ewald_wca", 102, 1),
    "ewald_rpm800": (lambda: workloads.rpm800(seed=13, update_frequency=1000), "ewald_wca", 103, 1),
    "ewald_iso": (lambda: isotropic(workloads.rpm_ewald(120, 24.0, 5, seed=17, update_frequency=7, cutoff=10.0,
                                                        eps_surf=1.0)), "ewald_wca", 109, 2),
    "dhlj_small": (lambda: workloads.dh_lj_salt(300, seed=14, density=0.004), "dh_lj", 104, 2),
    "dhlj_500": (lambda: workloads.dh_lj_salt(500, seed=15), "dh_lj", 105, 1),
    "dhlj_rdf": (lambda: workloads.dh_lj_salt(400, seed=16, density=0.004), "dh_lj", 106, 4),
}
# Isobaric volume moves (ExternalPressure + Isobaric): name -> (builder, model,
# seed, volume dp, pressure in mM, moves)
ISO_CASES = {
    "iso_dhlj": (lambda: workloads.dh_lj_salt(200, seed=21, density=0.004), "dh_lj", 107, 0.1, 100.0, 30),
    "iso_ewald": (lambda: workloads.rpm_ewald(100, 25.0, 5, seed=22, update_frequency=4, cutoff=10.0),
                  "ewald_wca", 108, 0.1, 100.0, 30),
}
# AtomRDF sampled by the reference after every sweep: name -> (type1, type2, dr)
RDF = {"dhlj_rdf": (0, 1, 0.5)}


# rigid dipolar molecules: (n_molecules, workload seed, RNG seed, sweeps, center_rotation)
MOL_CASES = {
    "mol_small": (40, 21, 201, 3, True),
    "mol_endrot": (27, 22, 202, 3, False),
    "mol_125": (125, 23, 203, 1, True),
}


def mol_input(mode, params, xyz, mu, mus, ids, seed, sweeps, center_rotation, molsize=20, dp=1.0, dprot=0.3):
    types = [dict(q=params.type_charge[t], sigma=params.type_sigma[t], eps=params.type_eps[t])
             for t in range(params.n_types)]
    return dict(mode=mode, box=params.box[0], temperature=298.0, bjerrum=params.bjerrum, cutoff=params.rf_cutoff,
                eps_rf=params.rf_eps_rf, types=types, molsize=molsize, n_mol=len(ids) // molsize,
                type_ids=[int(i) for i in ids], positions=xyz.tolist(), mu=mu.tolist(),
                muscalar=[float(m) for m in mus], dp=dp, dprot=dprot, center_rotation=center_rotation,
                seed=seed, sweeps=sweeps)


def make_mol(exe, name, n_mol, wseed, seed, sweeps, center_rotation):
    params, xyz, mu, mus, ids = workloads.dipolar_molecules(n_mol, seed=wseed)
    out = run_harness(exe, mol_input("mol_mc", params, xyz, mu, mus, ids, seed, sweeps, center_rotation))
    n = len(out["du"])
    extra = {}
    if name == "mol_small":
        # pair energies on chosen site pairs: random ones, every dipole site
        # against sites within 16 A, near contacts
        rng = np.random.default_rng(5)
        N = len(ids)
        pairs = set()
        while len(pairs) < 300:
            a, b = rng.integers(0, N, 2)
            if a // 20 != b // 20:
                pairs.add((int(a), int(b)))
        L = params.box[0]
        d = xyz[:, None, :] - xyz[None, :, :]
        d -= L * np.round(d / L)
        r = np.sqrt((d ** 2).sum(-1))
        for a in np.nonzero(mus)[0]:
            for b in np.nonzero((r[a] < 16.0) & (np.arange(N) // 20 != a // 20))[0]:
                pairs.add((int(a), int(b)))
        close = np.argwhere((r < 4.0) & ((np.arange(N)[:, None] // 20) != (np.arange(N)[None, :] // 20)))
        for a, b in close[:100]:
            pairs.add((int(a), int(b)))
        pairs = sorted(pairs)
        pu = run_harness(exe, dict(mol_input("mol_pairs", params, xyz, mu, mus, ids, seed, 0, center_rotation),
                                   pairs=pairs))
        extra = dict(pairs=np.asarray(pairs, dtype=np.int32), pair_u=np.asarray(pu["u"]),
                     pair_total=np.float64(pu["total"][0]))
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        params=np.frombuffer(bytes(params), dtype=np.uint8), xyz=xyz, mu=mu, mus=mus, ids=ids,
        seed=np.int64(seed), sweeps=np.int64(sweeps), center_rotation=np.int64(center_rotation),
        dp=np.float64(1.0), dprot=np.float64(0.3), cm0=np.asarray(out["cm0"]).reshape(-1, 3),
        u0=np.float64(out["u0"][0]), u1=np.float64(out["u1"][0]), u_move_sum=np.float64(out["u_move_sum"][0]),
        group=np.asarray(out["group"], dtype=np.int32), first_xyz=np.asarray(out["first_xyz"]).reshape(n, 3),
        first_mu=np.asarray(out["first_mu"]).reshape(n, 3), du=np.asarray(out["du"]),
        acc=np.asarray(out["acc"], dtype=np.uint8), final_positions=np.asarray(out["final_positions"]).reshape(-1, 3),
        final_mu=np.asarray(out["final_mu"]).reshape(-1, 3), final_cm=np.asarray(out["final_cm"]).reshape(-1, 3),
        **extra)
    print(name, "trials", n, "acceptance %.3f" % np.mean(out["acc"]), "u0 %.6f" % out["u0"][0])


# point dipoles: name -> (workload kwargs, harness template flags, seed, sweeps, dprot in radians)
DIP_CASES = {
    "dip_fluid": (dict(n=100, seed=3, kc=5.0), "ii_dd", 21, 4, 1.5),
    "dip_mixture": (dict(n=60, seed=4, kc=5.0, n_ions=20, update_frequency=7), "ii_dd", 22, 4, 1.0),
    "dip_mixture_id": (dict(n=60, seed=5, kc=5.0, n_ions=20, terms=7), "ii_id_dd", 23, 4, 1.0),
}


def dip_input(mode, params, xyz, mu, mus, ids, q, seed, sweeps, terms, dprot):
    types = [dict(q=params.type_charge[t], sigma=params.type_sigma[t], eps=params.type_eps[t],
                  dp=params.type_dp[t], dprot=dprot) for t in range(params.n_types)]
    return dict(mode=mode, terms=terms, box=params.box[0], bjerrum=params.bjerrum, types=types,
                positions=xyz.tolist(), type_ids=[int(i) for i in ids], charges=[float(c) for c in q],
                mu=mu.tolist(), mus=[float(m) for m in mus], seed=seed, sweeps=sweeps,
                alpha=params.ewald_alpha, cutoff=params.ewald_cutoff, cutoffK=params.ewald_cutoff_k,
                eps_surf=params.ewald_eps_surf, debyelength=params.ewald_debye_length,
                spherical_sum=bool(params.ewald_spherical_sum),
                update_frequency=int(params.ewald_update_frequency))


def make_dip(exe):
    # the unit test's configurations on the live code (bjerrum 1: energies in units of lB)
    p = workloads.make_params(workloads.FG_MODEL_EWALD_DIPOLE, 10.0, 1.0, [dict(q=1.0, sigma=0.0, eps=0.0)],
                              ewald_alpha=0.894427190999916, ewald_cutoff=5.0, ewald_cutoff_k=11.0,
                              ewald_eps_surf=1.0, ewald_update_frequency=10, ewald_terms=5)
    xyz = np.array([[0.0, 0, 0], [1, 0, 0], [0, 0, 1], [1, 0, 1]])
    known = run_harness(exe, dip_input("known", p, xyz, np.tile([1.0, 0, 0], (4, 1)), np.zeros(4),
                                       np.zeros(4, np.int32), np.zeros(4), 0, 0, "ii_dd", 0.0))
    np.savez_compressed(os.path.join(HERE, "dip_known.npz"),
                        **{k: np.asarray(v, dtype=np.float64) for k, v in known.items()})
    print("dip_known", {k: v[0] for k, v in known.items()})
    for name, (kw, terms, seed, sweeps, dprot) in DIP_CASES.items():
        params, xyz, mu, mus, ids, q = workloads.dipolar_fluid(quirk=1, **kw)
        params.bjerrum = 60.0   # acceptance near one half at these step sizes
        d = dip_input("mc", params, xyz, mu, mus, ids, q, seed, sweeps, terms, dprot)
        extra = {}
        if name == "dip_fluid":
            d["state_file"] = "final.state"
            out, (state,) = run_harness(exe, d, files=["final.state"])
            extra = dict(state_text=np.frombuffer(state, dtype=np.uint8))
        else:
            out = run_harness(exe, d)
        n = len(out["idx"])
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            params=np.frombuffer(bytes(params), dtype=np.uint8), xyz=xyz, mu=mu, mus=mus, ids=ids, q=q,
            seed=np.int64(seed), sweeps=np.int64(sweeps), dprot=np.float64(dprot),
            bjerrum=np.float64(out["bjerrum"][0]), u0=np.float64(out["u0"][0]), u1=np.float64(out["u1"][0]),
            u_move_sum=np.float64(out["u_move_sum"][0]), kind=np.asarray(out["kind"], dtype=np.int32),
            idx=np.asarray(out["idx"], dtype=np.int32), trial_xyz=np.asarray(out["trial_xyz"]).reshape(n, 3),
            trial_mu=np.asarray(out["trial_mu"]).reshape(n, 3), du=np.asarray(out["du"]),
            acc=np.asarray(out["acc"], dtype=np.uint8),
            final_positions=np.asarray(out["final_positions"]).reshape(-1, 3),
            final_mu=np.asarray(out["final_mu"]).reshape(-1, 3), **extra)
        print(name, "trials", n, "acceptance %.3f" % np.mean(out["acc"]), "u0 %.6f" % out["u0"][0])


# Parallel tempering: ranks (rungs), ions per rank, seed, rounds, sweeps per
# round, temperature ladder (geometric, reduced units)
PT_CASE = dict(ranks=8, n=240, density=0.006, seed=7, rounds=16, sweeps=4, t_min=0.6, t_max=3.0)


def make_pt(exe):
    """The reference's own ParallelTempering (move.h:6520-6771) over one
    process per rung (oracle/ref/ref_harness_pt.cpp with the stand-in MPI of
    oracle/ref/fakempi), DH+LJ salt, AtomicTranslation sweeps between the
    exchange attempts. Stores what each rank computed."""
    c = PT_CASE
    R, N = c["ranks"], c["n"]
    temps = workloads.pt_temperatures(R, c["t_min"], c["t_max"])
    cases = [workloads.dh_lj_salt(N, seed=100 + r, density=c["density"]) for r in range(R)]
    params, _, q, ids = cases[0]
    types = [dict(q=params.type_charge[t], sigma=params.type_sigma[t], eps=params.type_eps[t],
                  dp=params.type_dp[t]) for t in range(params.n_types)]
    d = dict(box=params.box[0], bjerrum=params.bjerrum, debyelength=params.dh_debye_length, types=types,
             type_ids=[int(i) for i in ids], seed=c["seed"], rounds=c["rounds"], sweeps_per_round=c["sweeps"],
             ranks=[dict(temperature=float(temps[r]), positions=cases[r][1].tolist()) for r in range(R)])
    with tempfile.TemporaryDirectory() as tmp:
        fin = os.path.join(tmp, "in.json")
        with open(fin, "w") as f:
            json.dump(d, f)
        procs = []
        for r in range(R):
            env = dict(os.environ, FAKEMPI_RANK=str(r), FAKEMPI_SIZE=str(R), FAKEMPI_DIR=tmp,
                       FAKEMPI_TIMEOUT="120")
            procs.append(subprocess.Popen([exe, fin, os.path.join(tmp, "out")], cwd=tmp, env=env,
                                          stdout=subprocess.DEVNULL))
        rcs = [p.wait(timeout=600) for p in procs]
        if any(rcs):
            raise RuntimeError("parallel tempering ranks failed: %s" % rcs)
        outs = []
        for r in range(R):
            with open(os.path.join(tmp, "out%d.json" % r)) as f:
                outs.append(json.load(f))
    stack = lambda k: np.asarray([o[k] for o in outs], dtype=np.float64)
    # the base Bjerrum length (unit temperature) as the reference rounds it
    lB = outs[0]["bjerrum"][0] * temps[0]
    np.savez_compressed(
        os.path.join(HERE, "pt_dhlj.npz"), params=np.frombuffer(bytes(params), dtype=np.uint8),
        bjerrum=np.float64(lB), temps=np.asarray(temps), xyz=np.stack([cs[1] for cs in cases]), q=q, ids=ids,
        seed=np.int64(c["seed"]), rounds=np.int64(c["rounds"]), sweeps=np.int64(c["sweeps"]),
        u_direction=stack("u_direction"), u_accept=stack("u_accept"), uold=stack("uold"), unew=stack("unew"),
        acc=stack("acc").astype(np.uint8), translations_accepted=stack("translations_accepted"),
        u0=stack("u0")[:, 0], u1=stack("u1")[:, 0],
        final_positions=stack("final_positions").reshape(R, N, 3))
    acc = stack("acc")
    print("pt_dhlj ranks", R, "rounds", c["rounds"], "exchange acceptance by rung", acc.mean(axis=1).round(2))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    if a.ref is None:
        from oracle.refdir import reference_dir
        a.ref = reference_dir()
    if not a.ref:
        sys.exit("no reference checkout: pass --ref or set FG_REFERENCE_DIR")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), "REF=" + a.ref])
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
    exe_mol = os.path.join(ROOT, "oracle", "_ref", "ref_harness_mol")
    if a.only in (None, "pt"):
        make_pt(os.path.join(ROOT, "oracle", "_ref", "ref_harness_pt"))
        if a.only:
            return
    if a.only in (None, "dip"):
        make_dip(os.path.join(ROOT, "oracle", "_ref", "ref_harness_dip"))
        if a.only:
            return
    for name, case in MOL_CASES.items():
        if a.only and name != a.only:
            continue
        make_mol(exe_mol, name, *case)
    if a.only and a.only in MOL_CASES:
        return

    for name, (builder, model, seed, vdp, pmm, moves) in ISO_CASES.items():
        if a.only and name != a.only:
            continue
        params, xyz, q, ids = builder()
        d = harness_input("isobaric", params, xyz, ids, seed, 0, model)
        d.update(volume_dp=vdp, pressure_mM=pmm, moves=moves)
        out = run_harness(exe, d)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            params=np.frombuffer(bytes(params), dtype=np.uint8), xyz=xyz, q=q, ids=ids,
            seed=np.int64(seed), volume_dp=np.float64(vdp), pressure_mM=np.float64(pmm), moves=np.int64(moves),
            bjerrum=np.float64(out["bjerrum"][0]), v0=np.float64(out["v0"][0]), du=np.asarray(out["du"]),
            acc=np.asarray(out["acc"], dtype=np.uint8), volume=np.asarray(out["volume"]),
            u_move_sum=np.float64(out["u_move_sum"][0]),
            final_positions=np.asarray(out["final_positions"]).reshape(-1, 3))
        print(name, "moves", moves, "acceptance %.3f" % np.mean(out["acc"]))
    if a.only and a.only in ISO_CASES:
        return

    if a.only in (None, "ewald_known"):
        known = run_harness(exe, dict(mode="ewald_known"))
        np.savez_compressed(os.path.join(HERE, "ewald_known.npz"),
                            **{k: np.asarray(v, dtype=np.float64) for k, v in known.items()})
        print("ewald_known", {k: v[0] for k, v in known.items()})

    for name, (builder, model, seed, sweeps) in CASES.items():
        if a.only and name != a.only:
            continue
        params, xyz, q, ids = builder()
        d = harness_input("mc", params, xyz, ids, seed, sweeps, model)
        extra = {}
        if name in RDF:
            t1, t2, dr = RDF[name]
            d["rdf"] = dict(t1=t1, t2=t2, dr=dr)
            d["state_file"] = "final.state"
            out, (state,) = run_harness(exe, d, files=["final.state"])
            extra = dict(rdf_types=np.asarray(RDF[name][:2], dtype=np.int32), rdf_dr=np.float64(RDF[name][2]),
                         rdf_key=np.asarray(out["rdf_key"]), rdf_count=np.asarray(out["rdf_count"]),
                         rdf_volume=np.float64(out["rdf_volume"][0]),
                         state_text=np.frombuffer(state, dtype=np.uint8))
        else:
            out = run_harness(exe, d)
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
            final_positions=np.asarray(out["final_positions"]).reshape(-1, 3), **extra)
        print(name, "trials", n, "acceptance %.3f" % np.mean(out["acc"]), "u0 %.6f" % out["u0"][0])


if __name__ == "__main__":
    main()
