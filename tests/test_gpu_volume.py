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


def test_volume_move_refused_inside_a_batch():
    from beofaunus_gb300.gpu import Batch, FgError, System
    p, xyz, q, ids = workloads.dh_lj_salt(300, seed=5)
    s = System(p, xyz, q, ids)
    b = Batch([s])
    with pytest.raises(FgError):
        s.volume_move(0.1, 0.05, 1e-5, 0.5)
    b.close()
    s.volume_move(0.1, 0.05, 1e-5, 0.5)   # allowed again once the batch is gone


def test_volume_moves_with_cells_in_place_and_across_a_cell_grid_change():
    """A cell-list system: moves that keep the cell grid run in place (the
    fixed-point positions stay, Q(k) stays exact, the box-dependent tables
    follow), a move that changes how many cells fit the box takes the
    general path; dU, decisions, positions and a translation sweep afterwards
    all match the FP64 oracle at each box."""
    from beofaunus_gb300.gpu import System
    p, xyz, q, ids = workloads.rpm_ewald(3600, 100.3, 6, seed=43, update_frequency=3, cutoff=20.0,
                                         use_cell_list=1)
    s = System(p, xyz, q, ids)
    x = np.asarray(xyz)
    po = p
    # half-steps: small growth and shrink inside the 5-cell grid, then a
    # shrink below 5 x 20 A (4 cells per axis), then a growth back over it
    halves = [0.2, -0.1, 0.15, -0.45, 0.3, 0.4]
    grids = []
    for m, h in enumerate(halves):
        # uniform 0: every move is accepted (reject only if u > exp(-dU))
        du, acc = s.volume_move(h, 0.08, 60.0 * MILLIMOLAR, 0.0)
        du_o, acc_o, po, x = volume_move(po, x, q, ids, h, 0.08, 60.0 * MILLIMOLAR, 0.0)
        assert du == pytest.approx(du_o, abs=1e-8) and acc and acc_o, m
        assert np.prod(s.box) == pytest.approx(po.box[0] * po.box[1] * po.box[2], rel=1e-13)
        grids.append(int(np.floor(s.box[0] / 20.0)))
    assert 4 in grids and 5 in grids          # both paths ran
    np.testing.assert_allclose(s.positions(), x, rtol=0, atol=1e-9)
    e64, eo = s.total_energy_fp64()["total"], OracleSystem(po, x, q, ids).total_energy()["total"]
    assert e64 == pytest.approx(eo, rel=1e-10, abs=1e-8)
    assert s.running_energy() == pytest.approx(e64, abs=1e-2)
    o = OracleSystem(po, x, q, ids)
    idx, disp, uu = s.draw_translation_stream(78, 600)
    r = s.sweep(idx, disp, uu)
    ro = o.mc_run_stream(idx, disp, uu)
    upto = len(idx)
    mism = np.nonzero(r["acc"] != ro["acc"])[0]
    if len(mism):
        t = mism[0]
        assert abs(ro["du"][t] + np.log(uu[t])) < 1e-6
        upto = t + 1
    assert np.abs(r["du"][:upto] - ro["du"][:upto]).max() < 1e-6
