"""Isobaric volume moves on the device (fg_volume_move) and the FP64 system
energy behind them (fg_total_energy_fp64): against the reference's own
Isobaric logs (tests/golden/iso_*.npz) and the FP64 oracle."""
import os

import numpy as np
import pytest

from beofaunus_gb300 import workloads
from beofaunus_gb300.params import FG_MODEL_EWALD_WCA, FgParams
from oracle.oracle import MILLIMOLAR, OracleSystem, volume_move

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", ["rpm800", "dhlj"])
def test_fp64_total_energy_matches_oracle(which):
    from beofaunus_gb300.gpu import System
    if which == "rpm800":
        p, xyz, q, ids = workloads.rpm800(seed=31)
    else:
        p, xyz, q, ids = workloads.dh_lj_salt(700, seed=32)
    s = System(p, xyz, q, ids)
    o = OracleSystem(p, xyz, q, ids)
    eg, eo = s.total_energy_fp64(), o.total_energy()
    for k in ("pairs", "reciprocal", "self", "surface", "total"):
        assert eg[k] == pytest.approx(eo[k], rel=1e-10, abs=1e-9), k


@pytest.mark.parametrize("name", ["iso_dhlj", "iso_ewald"])
def test_volume_moves_match_reference_log(name):
    from beofaunus_gb300.gpu import System, slump_uniforms
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    p = FgParams.from_buffer_copy(g["params"].tobytes())
    p.bjerrum = float(g["bjerrum"])
    s = System(p, g["xyz"], g["q"], g["ids"])
    moves = int(g["moves"])
    u = slump_uniforms(int(g["seed"]), 2 * moves)
    P = float(g["pressure_mM"]) * MILLIMOLAR
    quirk = p.model == FG_MODEL_EWALD_WCA
    for m in range(moves):
        du, acc = s.volume_move(u[2 * m] - 0.5, float(g["volume_dp"]), P, u[2 * m + 1], reference_quirk=quirk)
        assert du == pytest.approx(float(g["du"][m]), abs=1e-8), m
        assert acc == bool(g["acc"][m]), m
        assert np.prod(s.box) == pytest.approx(float(g["volume"][m]), rel=1e-13), m
    np.testing.assert_allclose(s.positions(), g["final_positions"], rtol=0, atol=1e-9)


def test_translations_after_volume_moves_match_oracle():
    """After accepted volume moves every box-dependent table (k-vector
    weights, cells, displacement steps) follows the new box: a translation
    sweep then reproduces the oracle built at that box."""
    from beofaunus_gb300.gpu import System, slump_uniforms
    p, xyz, q, ids = workloads.rpm_ewald(400, 40.0, 6, seed=41, update_frequency=50, cutoff=12.0)
    s = System(p, xyz, q, ids)
    x = np.asarray(xyz)
    po = p
    u = slump_uniforms(9, 16)
    n_acc = 0
    for m in range(8):
        du, acc = s.volume_move(u[2 * m] - 0.5, 0.08, 60.0 * MILLIMOLAR, u[2 * m + 1])
        du_o, acc_o, po, x = volume_move(po, x, q, ids, u[2 * m] - 0.5, 0.08, 60.0 * MILLIMOLAR, u[2 * m + 1])
        assert du == pytest.approx(du_o, abs=1e-8) and acc == acc_o
        n_acc += acc
    assert n_acc > 0
    np.testing.assert_allclose(s.positions(), x, rtol=0, atol=1e-9)
    o = OracleSystem(po, x, q, ids)
    idx, disp, uu = s.draw_translation_stream(77, 1200)
    r = s.sweep(idx, disp, uu)
    ro = o.mc_run_stream(idx, disp, uu)
    upto = len(idx)
    mism = np.nonzero(r["acc"] != ro["acc"])[0]
    if len(mism):
        t = mism[0]
        assert abs(ro["du"][t] + np.log(uu[t])) < 1e-6
        upto = t + 1
    assert np.abs(r["du"][:upto] - ro["du"][:upto]).max() < 1e-6


def test_volume_move_inside_a_batch():
    """A batch member takes volume moves between batch runs (in place: its
    cell grid stays); the batch's next run then runs it in the new box,
    exactly as the same system alone does."""
    from beofaunus_gb300.gpu import Batch, System
    p, xyz, q, ids = workloads.dh_lj_salt(300, seed=5)
    a, alone = System(p, xyz, q, ids), System(p, xyz, q, ids)
    p2, xyz2, q2, ids2 = workloads.dh_lj_salt(300, seed=6)
    other = System(p2, xyz2, q2, ids2)
    b = Batch([a, other])
    for h, uacc in ((0.3, 0.0), (-0.2, 0.0)):
        d1, a1 = a.volume_move(h, 0.05, 1e-5, uacc)
        d2, a2 = alone.volume_move(h, 0.05, 1e-5, uacc)
        assert d1 == d2 and a1 and a2
    np.testing.assert_array_equal(a.box, alone.box)
    b.stream_philox([2000, 2000], 91, stream_ids=[7, 8])
    b.run()
    alone.stream_philox(2000, 91, 7)
    alone.stream_run()
    np.testing.assert_array_equal(a.positions(), alone.positions())
    b.close()
