// Isobaric volume move (included by fg_api.cu; host driven).
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
// The trial box is a complete second system built with the new box (k-vector
// weights, cell grid and displacement steps all follow from it; Q(k) is
// rebuilt there from scratch, as NonbondedEwald::updateChange does for a
// geometry change, ewald.h:651-659). An accepted move swaps the two systems'
// contents, so the caller's handle keeps working. The running energy
// continues by E(V') - E(V); the accepted-move counter of the Q(k) rebuild
// cadence advances as NonbondedEwald::update counts (ewald.h:633).
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
double recip_unscaled(const fg_system *h, const fg_system *t, const std::vector<double> &xyz_old) {
    std::vector<int> n3;
    std::vector<double> ak, kv3;
    enumerate_k(t->P, n3, ak, kv3);
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
    return rec * t->recip_c;
}

extern "C" int fg_volume_move(fg_system *h, double half, double dp, double pressure, double u,
                              int32_t reference_quirk, double *du, int32_t *accepted) {
    if (!h || !du || !accepted) return fail(FG_ERR_INVALID, "null argument");
    if (h->types.empty()) return fail(FG_ERR_STATE, "fg_set_state first");
    if (h->trial_pending) return fail(FG_ERR_STATE, "a trial is pending: commit it first");
    if (h->batches > 0) return fail(FG_ERR_STATE, "the system is in a batch: destroy the batch first");
    if (!(pressure >= 0.0) || !std::isfinite(half) || !std::isfinite(dp))
        return fail(FG_ERR_INVALID, "bad volume move arguments");
    const int N = h->N;
    const double V = h->P.box[0] * h->P.box[1] * h->P.box[2];
    const double Vn = std::exp(std::log(V) + half * dp);
    const double f = std::cbrt(Vn / V);
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
    // whole-system energies in FP64: the move's dU is their difference
    double e0[5], e1[5];
    rc = total_energy_fp64(h, e0);
    if (!rc) rc = total_energy_fp64(t, e1);
    if (rc) return drop(rc);
    const double dE = e1[4] - e0[4];
    double d = dE + pressure * (Vn - V) - (N + 1) * std::log(Vn / V);
    if (reference_quirk && h->K > 0) d += recip_unscaled(h, t, xyz_old) - e1[1];
    *du = d;
    const double kT = h->desc.kT;
    const bool acc = !(u > std::exp(-d / kT));   // NaN dU: accepted, as the reference's comparison
    *accepted = acc ? 1 : 0;
    if (!acc) return drop(FG_OK);
    // carry the running energy, counters and settings over to the new box
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
