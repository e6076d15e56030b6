"""The drop-in adapter (include/faunus_gb300_energy.hpp, NonbondedGPU behind
the reference's Energybase interface, energy.h:54-224) running inside the
reference's own, unmodified AtomicTranslation and Movebase::move
(move.h:515-555, 818-901): oracle/_ref/adapter_run, built from the
reference's sources and linked against this library. On the inputs and seeds
of the golden fixtures it reproduces the reference's own per-trial logs (made
by the reference with NonbondedEwald<WCA> or Nonbonded<DH+LJ>): the same
particles, trial positions and decisions, dU within 1e-6 kT, final positions
within 1e-9 Angstrom. "movebase" runs every trial through updateChange ->
energyChange -> update (fg_trial_du / fg_commit); "device" draws the same
random numbers and runs them as one device sweep (translateOnDevice)."""
import importlib.util
import os

import numpy as np
import pytest

from beofaunus_gb300.params import FgParams

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu

TOL_DU = 1e-6
EXE = os.path.join(ROOT, "oracle", "_ref", "adapter_run")


def _golden_tools():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.skipif(not os.path.exists(EXE), reason="adapter_run not built (reference sources absent)")
@pytest.mark.parametrize("mode", ["movebase", "device"])
@pytest.mark.parametrize("name", ["ewald_surface_uf5", "ewald_small_uf1", "ewald_rpm800", "dhlj_small"])
def test_adapter_inside_reference_moves_reproduces_reference_log(name, mode):
    mg = _golden_tools()
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    p = FgParams.from_buffer_copy(g["params"].tobytes())   # the input the fixture was made from
    model = "ewald_wca" if name.startswith("ewald") else "dh_lj"
    d = mg.harness_input(mode, p, g["xyz"], g["ids"], int(g["seed"]), int(g["sweeps"]), model)
    out = mg.run_harness(EXE, d)
    assert float(out["u0"][0]) == pytest.approx(float(g["u0"]), rel=1e-9, abs=1e-6)
    if mode == "movebase":
        np.testing.assert_array_equal(np.array(out["idx"], dtype=int), g["idx"])
        np.testing.assert_allclose(np.array(out["trial_xyz"]).reshape(-1, 3), g["trial_xyz"], rtol=0, atol=1e-12)
        np.testing.assert_array_equal(np.array(out["acc"], dtype=int), g["acc"])
        err = np.abs(np.array(out["du"]) - g["du"])
        assert err.max() <= TOL_DU, err.max()
    np.testing.assert_allclose(np.array(out["final_positions"]).reshape(-1, 3), g["final_positions"], rtol=0,
                               atol=1e-9)
    assert float(out["u_move_sum"][0]) == pytest.approx(float(g["u_move_sum"]), abs=1e-5)
    assert float(out["u1"][0]) == pytest.approx(float(g["u1"]), rel=1e-9, abs=1e-5)
