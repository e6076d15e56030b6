"""The launch-shape autotuner (fg_autotune, fg_batch_autotune,
fg_mol_autotune): it times candidates on clones, leaves the caller's chains
where they were, and the tuned shapes keep parity with the FP64 oracle and
the reference's own molecule log."""
import os

import numpy as np
import pytest

from beofaunus_gb300 import workloads
from beofaunus_gb300.params import FgParams
from oracle.oracle import OracleSystem, philox_stream

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
TOL_DU = 1e-6


@pytest.fixture(autouse=True)
def fresh_tuning():
    from beofaunus_gb300.gpu import tune_reset
    tune_reset()
    yield
    tune_reset()


def test_dh_system_tuning_keeps_state_and_parity():
    from beofaunus_gb300.gpu import System
    p, xyz, q, ids = workloads.dh_lj_salt(4000, seed=41)
    s = System(p, xyz, q, ids)
    x0, e0 = s.positions(), s.running_energy()
    rep = s.autotune(512)
    vals = [v for v, _ in rep["candidates"]]
    assert len(vals) >= 2 and vals[0] == 1 and all(b == 2 * a for a, b in zip(vals, vals[1:]))
    assert rep["chosen"] in vals and all(us > 0 for _, us in rep["candidates"])
    # tuning ran on a clone
    np.testing.assert_array_equal(s.positions(), x0)
    assert s.running_energy() == e0
    # the tuned shape still reproduces the oracle trial by trial
    o = OracleSystem(p, xyz, q, ids)
    idx, disp, u = s.draw_translation_stream(7, 3000)
    r = s.sweep(idx, disp, u)
    ro = o.mc_run_stream(idx, disp, u)
    n = len(idx)
    mism = np.nonzero(r["acc"] != ro["acc"])[0]
    upto = n
    if len(mism):
        t = mism[0]
        assert abs(ro["du"][t] + np.log(u[t])) < TOL_DU
        upto = t + 1
    assert np.abs(r["du"][:upto] - ro["du"][:upto]).max() < TOL_DU
    if upto == n:
        np.testing.assert_allclose(s.positions(), o.positions(), rtol=0, atol=1e-9)


def test_ewald_block_kernel_tunes_its_cluster():
    """An Ewald system alone: the candidates are the cluster sizes 1, 2, 4, ...
    up to what fits; tuning runs on a clone, and the chosen size applies."""
    from beofaunus_gb300.gpu import System
    p, xyz, q, ids = workloads.rpm800(seed=5, update_frequency=200)
    s = System(p, xyz, q, ids)
    x0 = s.positions()
    rep = s.autotune(256)
    vals = [v for v, _ in rep["candidates"]]
    assert vals[0] == 1 and vals[-1] == s.max_cluster and all(b == 2 * a for a, b in zip(vals, vals[1:]))
    assert rep["chosen"] in vals and s.cluster == rep["chosen"]
    np.testing.assert_array_equal(s.positions(), x0)


def test_batch_tuning_keeps_oracle_parity():
    """A tuned schedule for uneven DH+LJ members: states untouched by the
    tuning, and the following batch run reproduces the oracle."""
    from beofaunus_gb300.gpu import Batch, System
    sizes = [500, 1200, 3000]
    specs = [workloads.dh_lj_salt(n, seed=200 + n) for n in sizes]
    systems = [System(p, x, q, ids) for (p, x, q, ids) in specs]
    b = Batch(systems)
    x0 = [s.positions() for s in systems]
    rep = b.autotune(256)
    assert [v for v, _ in rep["candidates"]] == [128, 256, 512, 1024, 2048]
    assert rep["chosen"] in (128, 256, 512, 1024, 2048)
    for s, x in zip(systems, x0):
        np.testing.assert_array_equal(s.positions(), x)
    seed, n = 77, 2 * max(sizes)
    b.stream_philox([n] * len(sizes), seed)
    per, tot = b.run()
    for i, (s, (p, x, q, ids)) in enumerate(zip(systems, specs)):
        o = OracleSystem(p, x, q, ids)
        idx, disp, u = philox_stream(seed, i, 0, n, ids, [p.type_dp[t] for t in range(p.n_types)], list(p.box))
        ro = o.mc_run_stream(idx, disp, u)
        assert per[i]["accepted"] == int(ro["acc"].sum())
        np.testing.assert_allclose(s.positions(), o.positions(), rtol=0, atol=1e-9)


def test_mol_tuning_keeps_reference_log():
    """Cluster size chosen by timing; the reference's TranslateRotate log
    is then reproduced at that size."""
    from beofaunus_gb300.gpu import MolSystem, mol_draw_stream
    g = np.load(os.path.join(GOLDEN, "mol_125.npz"))
    p = FgParams.from_buffer_copy(g["params"].tobytes())
    s = MolSystem(p, g["xyz"], g["mu"], g["mus"], g["ids"], 20, mass_centers=g["cm0"])
    before = s.state()
    rep = s.autotune(64)
    vals = [v for v, _ in rep["candidates"]]
    assert vals and rep["chosen"] in vals and s.cluster == rep["chosen"]
    for a, b in zip(s.state(), before):
        np.testing.assert_array_equal(a, b)
    n = len(g["group"])
    st = mol_draw_stream(int(g["seed"]), s.m, n, float(g["dp"]), float(g["dprot"]), bool(g["center_rotation"]))
    r = s.sweep(st)
    assert np.abs(r["du"] - g["du"]).max() < TOL_DU
    np.testing.assert_array_equal(r["acc"], g["acc"])


def test_dh_batch_mixes_one_cta_variants():
    """Members whose one-CTA sweep would differ (positions in shared memory
    or not) batch together: DH+LJ members all run the block kernel."""
    from beofaunus_gb300.gpu import Batch, System
    specs = [workloads.dh_lj_salt(n, seed=300 + n, start="scatter") for n in (256, 12000)]
    systems = [System(p, x, q, ids) for (p, x, q, ids) in specs]
    b = Batch(systems)
    rep = b.autotune(64)
    assert rep["chosen"] is not None
    b.stream_philox([512, 512], 3)
    per, tot = b.run()
    assert tot["trials"] == 1024 and tot["error_flags"] == 0
    p, x, q, ids = specs[0]
    o = OracleSystem(p, x, q, ids)
    idx, disp, u = philox_stream(3, 0, 0, 512, ids, [p.type_dp[t] for t in range(p.n_types)], list(p.box))
    ro = o.mc_run_stream(idx, disp, u)
    assert per[0]["accepted"] == int(ro["acc"].sum())
    np.testing.assert_allclose(systems[0].positions(), o.positions(), rtol=0, atol=1e-9)


def test_dipole_autotune_threads():
    """fg_dip_autotune times 32..256 threads per system on clones run together,
    applies the fastest to the caller's systems (whose chains do not advance)
    and makes it the default for new dipole systems."""
    from beofaunus_gb300 import gpu, workloads
    systems = []
    for k in range(6):
        p, xyz, mu, mus, ids, q = workloads.dipolar_fluid(n=80, seed=50 + k, kc=4.0)
        systems.append(gpu.DipoleSystem(p, xyz, mu, mus, ids, charges=q))
    e0 = [s.total_energy()[5] for s in systems]
    x0 = [s.state()[0] for s in systems]
    r = gpu.dip_autotune(systems, 128)
    assert [c[0] for c in r["candidates"]] == [32, 64, 128, 256]
    assert all(c[1] > 0 for c in r["candidates"])
    assert r["chosen"] == min(r["candidates"], key=lambda c: c[1])[0]
    for s, e, x in zip(systems, e0, x0):
        assert s.total_energy()[5] == e
        assert (s.state()[0] == x).all()
    # the tuned threads run the caller's systems, and new systems start from them
    st = gpu.dip_draw_stream(1, 80, 200)
    assert systems[0].sweep(st)["trials"] == 200
    gpu.tune_reset()
