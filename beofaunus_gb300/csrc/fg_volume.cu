// Isobaric volume move (included by fg_api.cu).
//
// Restates Move::Isobaric (move.h:5529-5624) with Energy::ExternalPressure
// (energy.h:1817-1890) for one atomic group, as the reference's bulk example
// wires them (pair energy + ExternalPressure):
//   V' = exp(ln V + half dp), half = slump.half() (move.h:5533);
//   every position scaled by (V'/V)^(1/3) about the origin (Cuboid::scale,
//   geometry.cpp:325-332, through Group::scale, group.h:318-330);
//   dU = E(V') - E(V) + P (V' - V) - (N + 1) ln(V'/V), E the system energy
//   (pairs + reciprocal + surface; the self term does not depend on V), the
//   pressure terms from ExternalPressure::external (P V - ln V) and
//   g_external (-N ln V for N atoms);
//   Metropolis as Movebase::metropolis (move.h:567-573): reject iff u > exp(-dU/kT).
//
// On the device and in place: with positions in fixed point relative to the
// box (X = x / L 2^64), scaling every position about the origin leaves every
// X as it is, so the trial configuration is the current one read in the new
// box. Both boxes' energies come from one FP64 pass over the fixed-point
// positions (Q(k) once: its exact phases depend on X only; the pair sum at
// each box's scale); an accepted move then changes only the box and what
// follows from it (apply_box), and Q(k) stays exact and unchanged, where the
// reference rebuilds it from scratch for the new geometry
// (NonbondedEwald::updateChange, ewald.h:651-659). The running energy
// continues by E(V') - E(V); the accepted-move counter of the Q(k) rebuild
// cadence advances as NonbondedEwald::update counts (ewald.h:633). A trial
// box with another cell grid (the cutoff fits a different number of times)
// takes the general path instead: a second system at the trial box, swapped
// in on acceptance (volume_move_rebuilt).
//
// Reference quirk (Ewald only). During the reference's energyChange for a
// geometry change, NonbondedEwald::setSpace -> setGeometry rebuilds Q(k)
// from spc->p, the positions before scaling, with the new box's k-vectors
// (ewald.h:731-756 via energy.h:3589-3593), and undo() hands that Q(k) to the
// trial (ewald.h:566-583): the trial's reciprocal energy is that of the
// unscaled positions in the new box. With reference_quirk set, dU takes that
// term (evaluated here in FP64 on the host), so dU and decisions follow the
// reference's; unset, dU is the energy difference of the scaled
// configurations. (Ours keeps the exact Q(k) of the scaled positions after
// an accepted move either way; the reference carries the unscaled one until
// its next update_frequency rebuild.)
double recip_unscaled(const fg_system *h, const fg_params &Pn, double recip_c, const std::vector<double> &xyz_old) {
    std::vector<int> n3;
    std::vector<double> ak, kv3;
    enumerate_k(Pn, n3, ak, kv3);
    double rec = 0;
    for (size_t k = 0; k < ak.size(); k++) {
        double re = 0, im = 0;
        for (int j = 0; j < h->N; j++) {
            const double qe = h->charges[j] * (double)h->desc.eff[h->types[j]];
            const double ph = kv3[3 * k] * xyz_old[3 * j] + kv3[3 * k + 1] * xyz_old[3 * j + 1] +
                              kv3[3 * k + 2] * xyz_old[3 * j + 2];
            re += qe * std::cos(ph);
            im += qe * std::sin(ph);
        }
        rec += ak[k] * (re * re + im * im);
    }
    return rec * recip_c;
}

namespace {

// The system in a new box, in place. The fixed-point positions X = x / L 2^64
// are the scaled positions in the new box as they are, and Q(k) = sum q eff
// e^{2 pi i n.X / 2^64} does not change at all; what changes are the box
// lengths and everything derived from them: the units of a coordinate word,
// the k-vectors and their weights A_k and prefactor 2 pi lB / V
// (kVectorChange, ewald.h:330-378), the surface prefactor, and the
// displacement steps in fixed point. Requires the same cell grid.
int apply_box(fg_system *h, const double box[3]) {
    fg_params &P = h->P;
    for (int a = 0; a < 3; a++) P.box[a] = box[a];
    SysDesc &d = h->desc;
    for (int a = 0; a < 3; a++) {
        d.L[a] = (float)P.box[a];
        d.s32[a] = (float)(P.box[a] / 4294967296.0);
        d.dl32[a] = (float)(P.box[a] / TWO64);
        d.s48_df[a] = split_df(P.box[a] / 281474976710656.0);
    }
    d.s32sq = (float)((P.box[0] / 4294967296.0) * (P.box[0] / 4294967296.0));
    if (h->K > 0) {
        std::vector<int> n3;
        std::vector<double> ak, kv3;
        enumerate_k(P, n3, ak, kv3);
        if ((int)ak.size() != h->K) return fail(FG_ERR_INVALID, "the k-vector set changes with the box");
        const double V = P.box[0] * P.box[1] * P.box[2];
        h->ak = ak;
        h->recip_c = 2 * PI / V * P.bjerrum;
        const double const_inf = (P.ewald_eps_surf < 1) ? 0.0 : 1.0;
        h->surf_c = const_inf * (2 * PI / ((2 * P.ewald_eps_surf + 1) * V)) * P.bjerrum;
        d.surf_c = (float)h->surf_c;
        std::vector<float4> kv(h->K);
        for (int k = 0; k < h->K; k++)
            kv[k] = make_float4((float)kv3[3 * k], (float)kv3[3 * k + 1], (float)kv3[3 * k + 2],
                                (float)(h->ak[k] * h->recip_c));
        CK(cudaMemcpyAsync(h->kvec, kv.data(), h->K * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    std::vector<int64_t> dpf(FG_MAX_TYPES * 3, 0);
    for (int t = 0; t < P.n_types; t++)
        for (int a = 0; a < 3; a++) dpf[3 * t + a] = (int64_t)llrint(P.type_dp[t] / P.box[a] * 4294967296.0);
    CK(cudaMemcpyAsync(h->dp_fix, dpf.data(), dpf.size() * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
    return push_desc(h);
}

// The move with the trial box as a complete second system (k-vectors, cell
// grid and displacement steps from it; Q(k) rebuilt there), swapped in on
// acceptance: for a trial box with another cell grid.
int volume_move_rebuilt(fg_system *h, double Vn, double f, double pressure, double u, int32_t reference_quirk,
                        double *du, int32_t *accepted) {
    const int N = h->N;
    const double V = h->P.box[0] * h->P.box[1] * h->P.box[2];
    std::vector<double> xyz(3 * (size_t)N);
    int rc = fg_get_state(h, xyz.data());
    if (rc) return rc;
    std::vector<double> xyz_old;
    if (reference_quirk && h->K > 0) xyz_old = xyz;
    for (double &x : xyz) x *= f;
    fg_params Pn = h->P;
    for (int a = 0; a < 3; a++) Pn.box[a] = h->P.box[a] * f;
    fg_system *t = nullptr;
    rc = fg_create(&Pn, N, &t);
    if (rc) return rc;
    auto drop = [&](int code) {
        fg_destroy(t);
        return code;
    };
    rc = fg_set_state(t, xyz.data(), h->charges.data(), h->types.data());
    if (rc) return drop(rc);
    double e0[5], e1[5];
    rc = total_energy_fp64(h, e0);
    if (!rc) rc = total_energy_fp64(t, e1);
    if (rc) return drop(rc);
    const double dE = e1[4] - e0[4];
    double d = dE + pressure * (Vn - V) - (N + 1) * std::log(Vn / V);
    if (reference_quirk && h->K > 0) d += recip_unscaled(h, t->P, t->recip_c, xyz_old) - e1[1];
    *du = d;
    const double kT = h->desc.kT;
    const bool acc = !(u > std::exp(-d / kT));   // NaN dU: accepted, as the reference's comparison
    *accepted = acc ? 1 : 0;
    if (!acc) return drop(FG_OK);
    SysScalars s0, s1;
    rc = read_scalars(h, s0);
    if (!rc) rc = read_scalars(t, s1);
    if (rc) return drop(rc);
    const float2 ut = split_df(df_val(s0.utot_hi, s0.utot_lo) + dE);
    s1.utot_hi = ut.x;
    s1.utot_lo = ut.y;
    s1.n_accepted = s0.n_accepted;
    s1.n_rebuilds = s0.n_rebuilds;
    int cnt = h->cnt_accepted_host;
    if (h->K > 0) {
        cnt = s0.cnt_accepted + 1;
        if (cnt > h->P.ewald_update_frequency - 1) cnt = 0;   // the rebuild is the one t just did
        s1.cnt_accepted = cnt;
    }
    rc = write_scalars(t, s1);
    if (rc) return drop(rc);
    t->threads = h->threads;
    t->ctas = h->ctas;
    t->eb_ctas = h->eb_ctas;
    t->cnt_accepted_host = cnt;
    if (h->desc.skip_rebuild) {
        rc = fg_set_rebuild_policy(t, 1);
        if (rc) return drop(rc);
    }
    if (h->desc.kT != 1.0f) {
        t->desc.kT = h->desc.kT;
        rc = push_desc(t);
        if (rc) return drop(rc);
    }
    std::swap(*h, *t);
    fg_destroy(t);   // the old box's arrays
    return FG_OK;
}

}  // namespace

extern "C" int fg_volume_move(fg_system *h, double half, double dp, double pressure, double u,
                              int32_t reference_quirk, double *du, int32_t *accepted) {
    if (!h || !du || !accepted) return fail(FG_ERR_INVALID, "null argument");
    if (h->types.empty()) return fail(FG_ERR_STATE, "fg_set_state first");
    if (h->trial_pending) return fail(FG_ERR_STATE, "a trial is pending: commit it first");
    if (!(pressure >= 0.0) || !std::isfinite(half) || !std::isfinite(dp))
        return fail(FG_ERR_INVALID, "bad volume move arguments");
    const int N = h->N;
    const double V = h->P.box[0] * h->P.box[1] * h->P.box[2];
    const double Vn = std::exp(std::log(V) + half * dp);
    const double f = std::cbrt(Vn / V);
    const double box1[3] = {h->P.box[0] * f, h->P.box[1] * f, h->P.box[2] * f};
    bool same_grid = true;
    if (h->use_cells)
        for (int a = 0; a < 3; a++)
            if ((int)std::floor(box1[a] / h->P.ewald_cutoff) != h->nc[a]) same_grid = false;
    // a batch holds its members' launch shape (cell grid, shared memory),
    // so a member moves only within its grid; between batch runs its
    // descriptor, and with it the new box, reaches the next launch
    if (!same_grid && h->batches > 0)
        return fail(FG_ERR_STATE, "this volume move changes the cell grid: not for a system in a batch");
    if (!same_grid) return volume_move_rebuilt(h, Vn, f, pressure, u, reference_quirk, du, accepted);
    // both boxes' FP64 energies of the same fixed-point configuration
    const double boxes[2][3] = {{h->P.box[0], h->P.box[1], h->P.box[2]}, {box1[0], box1[1], box1[2]}};
    double e[2][5];
    int rc = total_energy_fp64_boxes(h, 2, boxes, e);
    if (rc) return rc;
    const double dE = e[1][4] - e[0][4];
    double d = dE + pressure * (Vn - V) - (N + 1) * std::log(Vn / V);
    if (reference_quirk && h->K > 0) {
        std::vector<double> xyz_old(3 * (size_t)N);
        rc = fg_get_state(h, xyz_old.data());
        if (rc) return rc;
        fg_params Pn = h->P;
        for (int a = 0; a < 3; a++) Pn.box[a] = box1[a];
        d += recip_unscaled(h, Pn, 2 * PI / Vn * h->P.bjerrum, xyz_old) - e[1][1];
    }
    *du = d;
    const double kT = h->desc.kT;
    const bool acc = !(u > std::exp(-d / kT));   // NaN dU: accepted, as the reference's comparison
    *accepted = acc ? 1 : 0;
    if (!acc) return FG_OK;
    rc = apply_box(h, box1);
    if (rc) return rc;
    SysScalars s0;
    rc = read_scalars(h, s0);
    if (rc) return rc;
    const float2 ut = split_df(df_val(s0.utot_hi, s0.utot_lo) + dE);
    s0.utot_hi = ut.x;
    s0.utot_lo = ut.y;
    for (int a = 0; a < 3; a++) {   // the surface dipole sum q eff x scales with the positions
        const float2 m = split_df(df_val(s0.m[a][0], s0.m[a][1]) * f);
        s0.m[a][0] = m.x;
        s0.m[a][1] = m.y;
    }
    bool rebuild = false;
    if (h->K > 0) {
        // NonbondedEwald::update counts the accepted move (ewald.h:633);
        // Q(k) is unchanged and exact, so a rebuild due here only verifies it
        int cnt = s0.cnt_accepted + 1;
        if (cnt > h->P.ewald_update_frequency - 1) {
            cnt = 0;
            rebuild = !h->desc.skip_rebuild;
        }
        s0.cnt_accepted = cnt;
        h->cnt_accepted_host = cnt;
    }
    rc = write_scalars(h, s0);
    if (rc) return rc;
    if (rebuild) {
        double corr = 0;
        rc = fg_rebuild_qk(h, &corr);
        if (rc) return rc;
    }
    return FG_OK;
}

// The reference's global slump() sequence (RandomTwister::operator(),
// slump.h:62-95: uniform_real_distribution<double>(0, 1) on std::mt19937
// seeded with seed), for replaying the draws of moves driven from the host:
// Isobaric takes slump.half() = u - 0.5 and then the Metropolis uniform.
extern "C" int fg_slump_uniforms(uint32_t seed, int64_t n, double *u) {
    if (n < 0 || (n > 0 && !u)) return fail(FG_ERR_INVALID, "bad argument");
    std::mt19937 eng(seed);
    for (int64_t i = 0; i < n; i++) {
        std::uniform_real_distribution<double> uni(0, 1);   // one distribution object per call, as slump does
        u[i] = uni(eng);
    }
    return FG_OK;
}

// The system's current box lengths (they change with accepted volume moves).
extern "C" int fg_get_box(fg_system *h, double *box) {
    if (!h || !box) return fail(FG_ERR_INVALID, "null argument");
    for (int a = 0; a < 3; a++) box[a] = h->P.box[a];
    return FG_OK;
}
