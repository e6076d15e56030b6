// Point charges and point dipoles under Ewald summation: the AtomicRotation
// (move.h:976-1072) and AtomicTranslation (move.h:818-901) trials on
// DipoleParticle (point.h:591-680) with the energy change of
// NonbondedEwald<Tspace, LennardJonesLB, useIonIon, useIonDipole,
// useDipoleDipole> (ewald.h:228-757):
//   real space   EwaldReal (ewald.h:97-129) + LennardJonesLB (no cutoff);
//   k space      Q_ion(k) = sum q eff e^{ik.r}, Q_dip(k) = sum (k.mu) mu_s i e^{ik.r}
//                (ewald.h:388-415, 651-705), energy ewald.h:298-311;
//   surface      ewald.h:277-291 (running sums of q r and mu);
//   self         ewald.h:259-270 (unchanged by either move).
// fg_params.ewald_dipole_quirk selects the reading: 0 = the sum as ewald.h
// states it (real-space ion-dipole and dipole-dipole terms, reciprocal
// |Q_ion + Q_dip|^2); 1 = the reference's live code (EwaldReal returns after
// its ion-ion line, ewald.h:109-110; cross term 2 Re(Q_ion Q_dip),
// ewald.h:304-305; Q_dip rebuilt only with useDipoleDipole, ewald.h:400).
//
// Included by fg_api.cu (one translation unit).
//
// Work split. One system per CTA (128 threads by default, compiled for at
// most 128 registers so that four systems, sixteen warps, share an SM;
// fg_dip_autotune times the choices); a launch runs many systems (replicas,
// independent chains) side by side, with each system's k-vectors, A_k, Q(k)
// and particle records staged in shared memory for the launch when they fit.
// A trial is a block-wide pass: lanes 0..2 of warp 0 form the trial, one axis
// each (the quaternion rotation of mu or the fixed-point translation; the
// next trial's record is already loaded), the threads build the moved
// particle's per-axis phase tables e^{2 pi i n x_a / L_a}, n = 0..kcc, old and
// new (axis_entry_df: the exact 64-bit phase n X mod 2^64 split into a table
// angle and a short Taylor series, in df) and the (n_y, n_z) products the
// k-vectors use; then the pair loop and the k loop: far pairs are summed where
// they are found, near pairs are queued per warp in order and evaluated
// afterwards by consecutive threads, a translation's old and new position on
// two threads; a k-vector's phase is one product of a table entry with an
// (n_y, n_z) entry. The block reduces in a fixed order, thread 0 decides, and
// on acceptance the threads that computed a k-vector's Q increments add them
// to Q(k). A rotation keeps the position: one phase per k-vector and only the
// pair terms linear in the moved dipole; a translation keeps the dipole:
// dQ_dip = i (k.mu) mu_s (e_new - e_old).
//
// Precision. The per-trial dU must match the FP64 oracle to 1e-9 kT at Bjerrum
// lengths of hundreds of Angstrom, where single dipole pairs carry tens of kT.
// Near pairs (inside the radius beyond which no pair term of the state can
// exceed 1e-4 kT) are FP64, their radial functions from degree-5 tables on
// r^2 checked to 1e-13 against erfc/exp; far pairs are FP32, summed in
// double-float. The k loop, K terms per trial, runs in double-float (df: an
// unevaluated sum of two floats, ~48 significant bits) on the FP32 pipe, which
// on this part issues far more operations per clock than the FP64 pipe: Q(k),
// its increments, A_k, the phases and k.mu are all df; its sums take one
// TwoSum each (qadd), its error budget being absolute per k-vector. Surface
// sums and decisions are FP64. Positions are 64-bit fixed point (X = x/L
// 2^64): minimum image is the wrapped integer difference and every
// translation is exact.
namespace fgd {

constexpr int kDipMaxThreads = 256;
constexpr int kDipMaxKcc = 31;   // axis tables hold n = 0..kcc

constexpr int kDipErrNonFinite = 8;
constexpr int kDipErrLaunch = 64;

struct DipTrial {
    int32_t idx;   // particle
    int32_t kind;  // 1 rotation (q), 2 translation (t), 3 explicit: position t (absolute), dipole q[1..3]
    double thr;    // -ln u of the Metropolis uniform u: reject iff dU > kT thr, i.e. u > exp(-dU / kT)
                   // (Movebase::metropolis, move.h:567-573); +inf for u = 0
    double q[4];   // rotation quaternion (w, x, y, z)
    int64_t t[3];  // translation (fixed point)
};

struct DipScalars {
    int64_t cursor;       // next trial of the staged stream
    int64_t n_trials;     // end of the stream for this launch
    int64_t n_accepted;   // cumulative
    int64_t n_rebuilds;   // cumulative Q(k) rebuilds
    int32_t error;
    int32_t cnt_accepted; // NonbondedEwald::cnt_accepted (ewald.h:633)
    int32_t pad[2];
    double usum;          // accepted dU + rebuild corrections of the current stream
    double utot;          // running total energy
    double drift;         // NonbondedEwald::update_drift
    double pend_du;       // dU of an evaluated explicit trial
    double M[6];          // surface sums: sum q eff r (3), sum mu_s mu (3)
};

struct DipDesc {
    int32_t N, K, kcc, nt;
    int32_t ion_q;        // Q_ion kept (useIonIon || useIonDipole)
    int32_t dip_q;        // Q_dip kept by trials (useIonDipole || useDipoleDipole)
    int32_t dip_q_build;  // Q_dip built by rebuilds (quirk: useDipoleDipole only)
    int32_t ii, id, dd, quirk, uf, small_kappa, any_term;
    double L[3], s64[3], tpl[3];   // box, L / 2^64, 2 pi / L
    double alpha, alpha2, rc2, kappa, lB, kT;
    double recip_c;       // 2 pi lB / V
    double surf_c;        // 2 pi lB / ((2 eps_surf + 1) V), 0 with tin-foil surroundings
    double t1c, t2c;      // 2 alpha / sqrt(pi), 4 alpha^3 / (3 sqrt(pi))
    double eff[FG_MAX_TYPES];
    double qeqe[FG_MAX_TYPES * FG_MAX_TYPES], s2[FG_MAX_TYPES * FG_MAX_TYPES], eps4[FG_MAX_TYPES * FG_MAX_TYPES];
    // far pairs in FP32: beyond rf (rf2f = rf^2) no pair term exceeds the far
    // bound, so the FP32 rounding of a far pair stays below 1e-10 kT
    float rf2f, rc2f, alphaf, alpha2f, kappaf, lBf, t1cf, t2cf;
    float qeqef[FG_MAX_TYPES * FG_MAX_TYPES], s2f[FG_MAX_TYPES * FG_MAX_TYPES], eps4f[FG_MAX_TYPES * FG_MAX_TYPES];
    int64_t *pos;         // [3N] fixed point
    double *mu;           // [3N] dipole unit vectors
    double *mus;          // [N] dipole scalars
    double *q;            // [N] charges
    int32_t *type;        // [N]
    float4 *pf;           // [N] mu_s mu (x, y, z) and q as floats (far pairs)
    int32_t *nearq;       // [N + kDipMaxThreads] near-pair queue of the trial in flight
    // radial functions A, B, C of the real-space sum (see radial()) on
    // s = r^2 in [ts0, rc^2]: tn intervals of width 1 / tinv, six
    // coefficients per function per interval in the local variable
    // t = (s - s_k) tinv; null: evaluated directly
    const double *rtab;
    double ts0, tinv;
    int32_t tn, pad_tab;
    const float4 *sctab;
    const int16_t *yzl;   // the (n_y, n_z) table entries some k-vector uses ((n_y + kcc) W + n_z + kcc)
    int32_t nyz, pad_yz;
    char4 *kn;            // [K] n-vector of k
    double *ak;           // [K] A_k with the half-space factor
    double2 *qi, *qd;     // [K] FP64 accumulators of a rebuild
    float4 *fqi, *fqd;    // [K] Q_ion, Q_dip as df complex {re.hi, re.lo, im.hi, im.lo}
    float4 *dqi, *dqd;    // [K] increments of the trial in flight (df complex)
    float2 *akf;          // [K] A_k as df
    DipTrial *trials;
    double *log_du;       // [trials] or null
    uint8_t *log_acc;
    DipScalars *sc;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 conj_if(double2 a, bool c) { return c ? make_double2(a.x, -a.y) : a; }

// ---- double-float arithmetic (FP32 pipe)
using fg::df;
using fg::fast_two_sum;
__device__ __forceinline__ df dsplit(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ double dval(df a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ df dneg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df dadd(df a, df b) { return fg::df_add(a, b); }
__device__ __forceinline__ df dsub(df a, df b) { return fg::df_add(a, dneg(b)); }
__device__ __forceinline__ df dtwice(df a) { return {2.0f * a.hi, 2.0f * a.lo}; }
// a * b: the exact product of the high words by FMA plus the cross terms
__device__ __forceinline__ df dmul(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}
// a * n for a small integer n (exact in float)
__device__ __forceinline__ df dmul_i(df a, int n) {
    const float f = (float)n;
    const float p = __fmul_rn(a.hi, f);
    float e = __fmaf_rn(a.hi, f, -p);
    e = __fmaf_rn(a.lo, f, e);
    return fast_two_sum(p, e);
}
struct dc {
    df re, im;
};
__device__ __forceinline__ dc dc_load(float4 v) { return {{v.x, v.y}, {v.z, v.w}}; }
__device__ __forceinline__ float4 dc_pack(dc a) { return make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo); }
__device__ __forceinline__ dc dc_split(double2 a) { return {dsplit(a.x), dsplit(a.y)}; }
__device__ __forceinline__ double2 dc_val(float4 v) { return make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w); }
__device__ __forceinline__ dc dc_mul(dc a, dc b) {
    return {dsub(dmul(a.re, b.re), dmul(a.im, b.im)), dadd(dmul(a.re, b.im), dmul(a.im, b.re))};
}
__device__ __forceinline__ dc dc_conj_if(dc a, bool c) { return c ? dc{a.re, dneg(a.im)} : a; }
// The k loop's forms: Re(a conj(b)) (dc_dotq), Re(a b) (dc_rprodq), n . m
// for a small integer vector n (dkdotq), with sums of one TwoSum each
// (fg::df_add_quick), whose error (~2^-47 of the larger operand) is of the
// size of the operands' own rounding; the loop's error budget is absolute
// (each term against the scale |Q| |dQ| A_k of its k-vector), so the exact
// renormalisation of dadd buys nothing there.
__device__ __forceinline__ df qadd(df a, df b) { return fg::df_add_quick(a, b); }
__device__ __forceinline__ df qsub(df a, df b) { return fg::df_add_quick(a, dneg(b)); }
// a * b left as the rounded product of the high words and its error (not
// renormalised): only as an operand of qadd/qsub, whose TwoSum of the high
// parts is exact for any pair of floats
__device__ __forceinline__ df dmul_u(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    return {p, __fmaf_rn(a.lo, b.hi, e)};
}
__device__ __forceinline__ df dmul_iu(df a, int n) {
    const float f = (float)n;
    const float p = __fmul_rn(a.hi, f);
    return {p, __fmaf_rn(a.lo, f, __fmaf_rn(a.hi, f, -p))};
}
__device__ __forceinline__ dc dc_mulq(dc a, dc b) {
    return {qsub(dmul_u(a.re, b.re), dmul_u(a.im, b.im)), qadd(dmul_u(a.re, b.im), dmul_u(a.im, b.re))};
}
__device__ __forceinline__ df dc_dotq(dc a, dc b) { return qadd(dmul_u(a.re, b.re), dmul_u(a.im, b.im)); }
__device__ __forceinline__ df dc_rprodq(dc a, dc b) { return qsub(dmul_u(a.re, b.re), dmul_u(a.im, b.im)); }
__device__ __forceinline__ df dkdotq(char4 n, const df *m) {
    return qadd(qadd(dmul_iu(m[0], n.x), dmul_iu(m[1], n.y)), dmul_iu(m[2], n.z));
}

// e^{i k.r} from one particle's axis tables (tab[axis * (kcc+1) + |n|]);
// negative components take the conjugate
__device__ __forceinline__ double2 kphase(const double2 *tab, int stride, char4 n) {
    const double2 ex = tab[n.x];
    const double2 ey = conj_if(tab[stride + (n.y < 0 ? -n.y : n.y)], n.y < 0);
    const double2 ez = conj_if(tab[2 * stride + (n.z < 0 ? -n.z : n.z)], n.z < 0);
    return cmul(cmul(ex, ey), ez);
}

// Dynamic shared memory of the sweep kernel: e^{i (ny k_y y + nz k_z z)} of
// the moved particle for ny, nz in [-kcc, kcc], old then new; a k-vector's
// phase is then one product with the x-axis entry.
__host__ __device__ constexpr size_t dip_yz_bytes(int kcc) {
    return (size_t)2 * (2 * kcc + 1) * (2 * kcc + 1) * sizeof(double2);
}

// The arrays one sweep touches per trial. A sweep launch stages them in
// shared memory (dip_stage_layout, after the yz table) when they fit, so the
// k loop and the pair loop read no global memory; Q(k) goes back to global
// memory at the end of the launch, positions and pf on every acceptance.
struct DipArrays {
    const char4 *kn;
    const float2 *akf;
    float4 *fqi, *fqd, *dqi, *dqd;
    int64_t *pos;
    float4 *pf;
    const int32_t *type;
    double *mu;
    const double *mus, *q;
};

__host__ __device__ inline size_t dip_al16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline size_t dip_stage_layout(int K, int N, int kcc, int ion_q, int dip_q, size_t off[12]) {
    size_t b = dip_yz_bytes(kcc);
    off[0] = b;                               // kn
    b = dip_al16(b + (size_t)K * 4);
    off[1] = b;                               // akf
    b = dip_al16(b + (size_t)K * 8);
    off[2] = b;                               // fqi
    if (ion_q) b += (size_t)K * 16;
    off[3] = b;                               // fqd
    if (dip_q) b += (size_t)K * 16;
    off[4] = b;                               // dqi
    if (ion_q) b += (size_t)K * 16;
    off[5] = b;                               // dqd
    if (dip_q) b += (size_t)K * 16;
    off[6] = b;                               // pos
    b = dip_al16(b + (size_t)N * 24);
    off[7] = b;                               // pf
    b += (size_t)N * 16;
    off[8] = b;                               // type
    b = dip_al16(b + (size_t)N * 4);
    off[9] = b;                               // mu
    b += (size_t)N * 24;
    off[10] = b;                              // mus
    b += (size_t)N * 8;
    off[11] = b;                              // q
    return dip_al16(b + (size_t)N * 8);
}

// cos, sin of 2 pi n X / 2^64: the phase reduced exactly in integers
__device__ __forceinline__ double2 axis_entry(int n, int64_t X) {
    const int64_t ph = (int64_t)((uint64_t)(int64_t)n * (uint64_t)X);
    double s, c;
    sincospi((double)ph * 1.0842021724855044e-19, &s, &c);   // 2^-63
    return make_double2(c, s);
}

__device__ __forceinline__ double horner6(const double *c, double t) {
    return fma(fma(fma(fma(fma(c[5], t, c[4]), t, c[3]), t, c[2]), t, c[1]), t, c[0]);
}

// Radial functions of the real-space sum at s = r^2 (r <= rc):
//   A = ion-ion: erfc(a r) / r, or the kappa-screened form (ewald.h:109);
//   B = T1f(r) / r^3, C = T2f(r) / r^5 (ewald.h:46-47),
// from the interpolation table where it covers s, else from erfc and exp.
__device__ __forceinline__ void radial(const DipDesc &d, double s, double &A, double &B, double &C) {
    if (d.rtab && s >= d.ts0) {
        const double u = (s - d.ts0) * d.tinv;
        int k = (int)u;
        k = k < d.tn - 1 ? k : d.tn - 1;
        const double t = u - (double)k;
        const double *c = d.rtab + 18 * k;
        A = (d.quirk || d.ii) ? horner6(c, t) : 0.0;   // the ion-ion function only where a term uses it
        B = horner6(c + 6, t);
        C = horner6(c + 12, t);
        return;
    }
    const double r1 = sqrt(s), ir1 = 1.0 / r1, ir2 = ir1 * ir1;
    const double ar = d.alpha * r1, ec = erfc(ar), ex = exp(-d.alpha2 * s);
    if (d.small_kappa) {
        A = ec * ir1;
    } else {
        const double h = d.kappa / 2.0 / d.alpha;
        A = (erfc(ar + h) * exp(d.kappa * r1) + erfc(ar - h) * exp(-d.kappa * r1)) / (2.0 * r1);
    }
    const double T1f = r1 * d.t1c * ex + ec;
    B = T1f * ir1 * ir2;
    C = 3.0 * (T1f + d.t2c * r1 * r1 * r1 * ex) * (ir2 * ir2 * ir1);
}

// Pair energy of particles a (moved) and b at r = a - b: EwaldReal + LJ
// (CombinedPairPotential, potentials.h:3768-3771). real/lj split for totals.
__device__ __forceinline__ void dip_pair(const DipDesc &d, double rx, double ry, double rz, double qa, int ta,
                                         double mas, const double *ma, double qb, int tb, double mbs,
                                         const double *mb, double &real, double &lj) {
    const double r2 = rx * rx + ry * ry + rz * rz;
    const int tt = ta * d.nt + tb;
    // LennardJonesMixed (potentials.h:2036-2040): s2 / r2 through 1 / r2 from
    // its float value and two Newton steps (relative error ~1e-16, against
    // the ~20 FP64 operations of a correctly rounded division)
    double ir2 = (double)__frcp_rn((float)r2);
    ir2 = ir2 * fma(-r2, ir2, 2.0);
    ir2 = ir2 * fma(-r2, ir2, 2.0);
    double x = d.s2[tt] * ir2;
    x = x * x * x;
    lj = d.eps4[tt] * (x * x - x);
    real = 0.0;
    if (!d.any_term || r2 > d.rc2) return;
    double A, B, C;
    radial(d, r2, A, B, C);
    if (d.quirk || d.ii) real = qa * qb * A * d.qeqe[tt] * d.lB;
    if (d.quirk || !(d.id || d.dd)) return;
    double Ed = 0.0;
    if (d.id) {
        Ed += qa * (rx * mb[0] + ry * mb[1] + rz * mb[2]) * mbs * B;
        Ed -= qb * (rx * ma[0] + ry * ma[1] + rz * ma[2]) * mas * B;
    }
    if (d.dd) {
        const double t3 = -(mb[0] * ma[0] + mb[1] * ma[1] + mb[2] * ma[2]) * B;
        const double t5 = (mb[0] * rx + mb[1] * ry + mb[2] * rz) * (ma[0] * rx + ma[1] * ry + ma[2] * rz) * C;
        Ed += -(t5 + t3) * mbs * mas;
    }
    real += d.lB * Ed;
}

// Far pair (r beyond rf) in FP32: EwaldReal + LJ of a and b, with
// ma, mb = (mu_s mu, q). Same terms as dip_pair.
__device__ __forceinline__ float far_pair(const DipDesc &d, float rx, float ry, float rz, int ta, float4 ma, int tb,
                                          float4 mb) {
    const float r2 = rx * rx + ry * ry + rz * rz;
    const int tt = ta * d.nt + tb;
    const float ir2 = 1.0f / r2;
    float x = d.s2f[tt] * ir2;
    x = x * x * x;
    float e = d.eps4f[tt] * (x * x - x);
    if (!d.any_term || r2 > d.rc2f) return e;
    const float r1 = sqrtf(r2), ir1 = 1.0f / r1;
    const float ar = d.alphaf * r1, ec = erfcf(ar);
    if (d.quirk || d.ii) {
        float t;
        if (d.small_kappa) {
            t = ec * ir1;
        } else {
            const float h = d.kappaf / (2.0f * d.alphaf);
            t = (erfcf(ar + h) * expf(d.kappaf * r1) + erfcf(ar - h) * expf(-d.kappaf * r1)) * 0.5f * ir1;
        }
        e += ma.w * mb.w * t * d.qeqef[tt] * d.lBf;
    }
    if (d.quirk || !(d.id || d.dd)) return e;
    const float ex = expf(-d.alpha2f * r2);
    const float T1f = r1 * d.t1cf * ex + ec, T1 = T1f * ir1 * ir2;
    float Ed = 0.0f;
    if (d.id) Ed += (ma.w * (rx * mb.x + ry * mb.y + rz * mb.z) - mb.w * (rx * ma.x + ry * ma.y + rz * ma.z)) * T1;
    if (d.dd) {
        const float T2f = 3.0f * (T1f + d.t2cf * r1 * r1 * r1 * ex);
        Ed += (ma.x * mb.x + ma.y * mb.y + ma.z * mb.z) * T1 -
              (mb.x * rx + mb.y * ry + mb.z * rz) * (ma.x * rx + ma.y * ry + ma.z * rz) * T2f * (ir2 * ir2 * ir1);
    }
    return e + d.lBf * Ed;
}

// Far pair when only a's dipole turns by dm (= mu_s dmu), FP32.
__device__ __forceinline__ float far_turn(const DipDesc &d, float rx, float ry, float rz, float3 dm, float4 mb) {
    const float r2 = rx * rx + ry * ry + rz * rz;
    if (d.quirk || !(d.id || d.dd) || r2 > d.rc2f) return 0.0f;
    const float r1 = sqrtf(r2), ir1 = 1.0f / r1, ir2 = ir1 * ir1;
    const float ex = expf(-d.alpha2f * r2);
    const float T1f = r1 * d.t1cf * ex + erfcf(d.alphaf * r1), T1 = T1f * ir1 * ir2;
    float Ed = 0.0f;
    if (d.id) Ed -= mb.w * (rx * dm.x + ry * dm.y + rz * dm.z) * T1;
    if (d.dd) {
        const float T2f = 3.0f * (T1f + d.t2cf * r1 * r1 * r1 * ex);
        Ed += (dm.x * mb.x + dm.y * mb.y + dm.z * mb.z) * T1 -
              (mb.x * rx + mb.y * ry + mb.z * rz) * (dm.x * rx + dm.y * ry + dm.z * rz) * T2f * (ir2 * ir2 * ir1);
    }
    return d.lBf * Ed;
}

// float of the high word of a 64-bit fixed-point difference (units of L / 2^32)
__device__ __forceinline__ float hi_diff(int64_t a, int64_t b) {
    return (float)(int32_t)((uint64_t)(a - b) >> 32);
}

// Change of the pair energy when only a's dipole turns (mu_a -> mu_a + dmu,
// the positions fixed): the terms linear in mu_a with dmu in its place; LJ,
// ion-ion and the q_a mu_b term do not change.
__device__ __forceinline__ double dip_turn(const DipDesc &d, double rx, double ry, double rz, double mas,
                                           const double *dmu, double qb, double mbs, const double *mb) {
    const double r2 = rx * rx + ry * ry + rz * rz;
    if (d.quirk || !(d.id || d.dd) || r2 > d.rc2) return 0.0;
    double A, B, C;
    radial(d, r2, A, B, C);
    double Ed = 0.0;
    if (d.id) Ed -= qb * (rx * dmu[0] + ry * dmu[1] + rz * dmu[2]) * mas * B;
    if (d.dd) {
        const double t3 = -(mb[0] * dmu[0] + mb[1] * dmu[1] + mb[2] * dmu[2]) * B;
        const double t5 = (mb[0] * rx + mb[1] * ry + mb[2] * rz) * (dmu[0] * rx + dmu[1] * ry + dmu[2] * rz) * C;
        Ed += -(t5 + t3) * mbs * mas;
    }
    return d.lB * Ed;
}

__device__ __forceinline__ df dsqr(df a) { return dmul(a, a); }
// cos, sin of 2 pi n X / 2^64 as df without the FP64 pipe: the phase reduced
// exactly in integers to the nearest of kDipScTab table angles plus a rest
// |theta| <= pi / kDipScTab, whose sine and cosine come from their Taylor
// series (sin: theta - theta^3/6 + theta^5/120, the last two in FP32; cos:
// 1 - theta^2/2 in df + theta^4/24), rotated by the table entry.
constexpr int kDipScTab = 1024;
__device__ __forceinline__ float4 axis_entry_df(int n, int64_t X, const float4 *__restrict__ tab) {
    const uint64_t ph = (uint64_t)(int64_t)n * (uint64_t)X;
    const uint32_t idx = (uint32_t)((ph + (1ull << 53)) >> 54);   // mod 2^64: 0 .. kDipScTab - 1
    const int64_t rem = (int64_t)(ph - ((uint64_t)idx << 54));    // |rem| <= 2^53
    const float h = (float)rem, l = (float)(rem - (int64_t)h);
    const df th = dmul(df{h, l}, df{0x1.921fb6p-62f, -0x1.777a5cp-87f});   // 2 pi / 2^64 as df
    const float t2f = th.hi * th.hi;
    const df sn = fg::df_add_f(th, th.hi * t2f * __fmaf_rn(t2f, 1.0f / 120.0f, -1.0f / 6.0f));
    const df t2 = dsqr(th);
    const df cs = fg::df_add_f(dsub(df{1.0f, 0.0f}, df{0.5f * t2.hi, 0.5f * t2.lo}), t2f * t2f * (1.0f / 24.0f));
    const float4 e = __ldg(tab + (idx & (kDipScTab - 1)));
    return dc_pack(dc_mul(dc{{e.x, e.y}, {e.z, e.w}}, dc{cs, sn}));
}

// Block sum in a fixed order (result valid in thread 0).
__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < nw; w++) s += red[w];
    return s;
}

// c (|Mq|^2 + 2 Mq.Mmu + |Mmu|^2) = c |Mq + Mmu|^2: its change when the sum
// S = Mq + Mmu moves by D is c (2 S.D + D.D)
__device__ __forceinline__ double surface_change(const DipDesc &d, const double *M, const double *D) {
    const double s0 = M[0] + M[3], s1 = M[1] + M[4], s2 = M[2] + M[5];
    return d.surf_c * (2.0 * (s0 * D[0] + s1 * D[1] + s2 * D[2]) + D[0] * D[0] + D[1] * D[1] + D[2] * D[2]);
}

// Reciprocal energy sum_k A_k Q2(k) of this thread's k-vectors (before recip_c)
__device__ __forceinline__ double q2(const DipDesc &d, double2 a, double2 b) {
    double s = 0.0;
    if (d.ii) s += a.x * a.x + a.y * a.y;
    if (d.id) s += 2.0 * (d.quirk ? a.x * b.x - a.y * b.y : a.x * b.x + a.y * b.y);
    if (d.dd) s += b.x * b.x + b.y * b.y;
    return s;
}

struct DipShared {
    int64_t po[3], pn[3];
    double muo[3], mun[3];
    double ro[3], rn[3];
    double qa, qeff, mas, thr, du;
    double M[6];
    int idx, ta, accept, rebuild, fixed, same_mu;
    int qcnt[kDipMaxThreads / 32];
    double red[kDipMaxThreads / 32];
    float4 tab[2][3 * (kDipMaxKcc + 1)];    // moved particle, old and new (df complex)
    df mo[3], mn[3], md[3];                 // 2 pi / L_a mu_s times mu_old, mu_new, mu_new - mu_old
    df qeffd;
    double2 rtab[3 * (kDipMaxKcc + 1)];     // rebuild: one particle at a time
    double rq, rmu[3];
};

// Q(k) from scratch (updateAllComplexNumbers, ewald.h:388-415). Returns the
// reciprocal energy before and after in thread 0.
__device__ void dip_rebuild(const DipDesc &d, const DipArrays &A, DipShared &S, double &before, double &after) {
    const int tid = threadIdx.x, T = blockDim.x, st = d.kcc + 1;
    double e = 0.0;
    for (int k = tid; k < d.K; k += T) {
        e += d.ak[k] * q2(d, dc_val(A.fqi[k]), dc_val(A.fqd[k]));
        d.qi[k] = make_double2(0.0, 0.0);
        d.qd[k] = make_double2(0.0, 0.0);
    }
    before = block_sum(e, S.red) * d.recip_c;
    for (int j = 0; j < d.N; j++) {
        __syncthreads();   // previous particle's table consumed
        for (int e = tid; e < 3 * st; e += T) {
            const int a = e / st, n = e - a * st;
            S.rtab[e] = axis_entry(n, A.pos[3 * j + a]);
        }
        if (tid == 0) {
            S.rq = A.q[j] * d.eff[A.type[j]];
            for (int a = 0; a < 3; a++) S.rmu[a] = A.mu[3 * j + a] * A.mus[j];
        }
        __syncthreads();
        for (int k = tid; k < d.K; k += T) {
            const char4 n = A.kn[k];
            const double2 ph = kphase(S.rtab, st, n);
            if (d.ion_q) {
                double2 v = d.qi[k];
                v.x += S.rq * ph.x;
                v.y += S.rq * ph.y;
                d.qi[k] = v;
            }
            if (d.dip_q_build) {
                const double km = n.x * d.tpl[0] * S.rmu[0] + n.y * d.tpl[1] * S.rmu[1] + n.z * d.tpl[2] * S.rmu[2];
                double2 v = d.qd[k];
                v.x -= km * ph.y;
                v.y += km * ph.x;
                d.qd[k] = v;
            }
        }
    }
    e = 0.0;
    for (int k = tid; k < d.K; k += T) {
        const double2 a = d.qi[k], b = d.qd[k];
        e += d.ak[k] * q2(d, a, b);
        A.fqi[k] = dc_pack(dc_split(a));
        A.fqd[k] = dc_pack(dc_split(b));
    }
    after = block_sum(e, S.red) * d.recip_c;
}

// Q(k) of the uploaded state (setSpace -> setGeometry, ewald.h:731-756)
__global__ void __launch_bounds__(kDipMaxThreads, 1) dip_build_kernel(const DipDesc *dp) {
    __shared__ DipShared S;
    double before, after;
    const DipDesc &d = *dp;
    const DipArrays A = {d.kn, d.akf, d.fqi, d.fqd, d.dqi, d.dqd, d.pos, d.pf, d.type, d.mu, d.mus, d.q};
    dip_rebuild(d, A, S, before, after);
}

// mode 0: run the staged stream [cursor, n_trials) with Metropolis decisions;
// mode 1: evaluate trials[0] (explicit) and keep it pending;
// mode 2: apply the pending trials[0] as accepted.
// MAXT: the launch bound. 128 threads per system at most 128 registers
// (four systems, sixteen warps on an SM) or up to kDipMaxThreads at one CTA
// per SM.
template <int MAXT>
__global__ void __launch_bounds__(MAXT, MAXT <= 128 ? 4 : 1) dip_sweep_kernel(const DipDesc *__restrict__ descs, int mode,
                                                                               int stage) {
    const DipDesc &d = descs[blockIdx.x];
    __shared__ DipShared S;
    extern __shared__ __align__(16) unsigned char dsm[];
    float4 *eyz = reinterpret_cast<float4 *>(dsm);   // df complex
    const int tid = threadIdx.x, T = blockDim.x, st = d.kcc + 1;
    const int W = 2 * d.kcc + 1, W2 = W * W;
    if (T > MAXT || (T & 31)) {
        if (tid == 0) atomicOr(&d.sc->error, kDipErrLaunch);
        return;
    }
    DipArrays A = {d.kn, d.akf, d.fqi, d.fqd, d.dqi, d.dqd, d.pos, d.pf, d.type, d.mu, d.mus, d.q};
    if (stage) {
        size_t off[12];
        dip_stage_layout(d.K, d.N, d.kcc, d.ion_q, d.dip_q, off);
        char4 *kn = reinterpret_cast<char4 *>(dsm + off[0]);
        float2 *akf = reinterpret_cast<float2 *>(dsm + off[1]);
        float4 *fqi = reinterpret_cast<float4 *>(dsm + off[2]), *fqd = reinterpret_cast<float4 *>(dsm + off[3]);
        int64_t *pos = reinterpret_cast<int64_t *>(dsm + off[6]);
        float4 *pf = reinterpret_cast<float4 *>(dsm + off[7]);
        int32_t *typ = reinterpret_cast<int32_t *>(dsm + off[8]);
        double *smu = reinterpret_cast<double *>(dsm + off[9]), *smus = reinterpret_cast<double *>(dsm + off[10]),
               *sq = reinterpret_cast<double *>(dsm + off[11]);
        for (int k = tid; k < d.K; k += T) {
            kn[k] = A.kn[k];
            akf[k] = A.akf[k];
            if (d.ion_q) fqi[k] = A.fqi[k];
            if (d.dip_q) fqd[k] = A.fqd[k];
        }
        for (int j = tid; j < d.N; j += T) {
            pos[3 * j] = A.pos[3 * j];
            pos[3 * j + 1] = A.pos[3 * j + 1];
            pos[3 * j + 2] = A.pos[3 * j + 2];
            pf[j] = A.pf[j];
            typ[j] = A.type[j];
            for (int a = 0; a < 3; a++) smu[3 * j + a] = A.mu[3 * j + a];
            smus[j] = A.mus[j];
            sq[j] = A.q[j];
        }
        A = {kn, akf, fqi, fqd, reinterpret_cast<float4 *>(dsm + off[4]), reinterpret_cast<float4 *>(dsm + off[5]), pos,
             pf, typ, smu, smus, sq};
        __syncthreads();
    }
    DipScalars sc;
    if (tid == 0) {
        sc = *d.sc;
        for (int a = 0; a < 6; a++) S.M[a] = sc.M[a];
    }
    int64_t t0 = 0, t1 = 1;
    if (mode == 0) {
        t0 = d.sc->cursor;
        t1 = d.sc->n_trials;
    }
    DipTrial nxt;   // lanes 0..2: the next trial's record, loaded one trial ahead
    if (tid < 3 && t0 < t1) nxt = d.trials[mode == 0 ? t0 : 0];
    for (int64_t t = t0; t < t1; t++) {
        // ---- the trial: lane a of warp 0 takes axis a (a < 3), lane 0 the
        // particle's scalars; a rotation is Eigen's quaternion-vector
        // product (QuaternionRotate, geometry.cpp:753-766) one component per
        // lane: uv = 2 v x p, mu' = p + w uv + v x uv
        if (tid < 32) {
            const int lane = tid;
            const DipTrial tr = nxt;
            if (lane < 3 && mode == 0 && t + 1 < t1) nxt = d.trials[t + 1];   // in flight during this trial
            const int i = __shfl_sync(0xffffffffu, tr.idx, 0), kind = __shfl_sync(0xffffffffu, tr.kind, 0);
            const int a = lane < 3 ? lane : 0, a1 = a == 2 ? 0 : a + 1, a2 = a == 0 ? 2 : a - 1;
            const int64_t po = A.pos[3 * i + a];
            const double muo = A.mu[3 * i + a];
            const double p1 = __shfl_sync(0xffffffffu, muo, a1), p2 = __shfl_sync(0xffffffffu, muo, a2);
            int64_t pn = po;
            double mun = muo;
            if (kind == 1) {
                const double w = tr.q[0], v1 = tr.q[1 + a1], v2 = tr.q[1 + a2];
                double u = v1 * p2 - v2 * p1;
                u += u;
                const double u1 = __shfl_sync(0xffffffffu, u, a1), u2 = __shfl_sync(0xffffffffu, u, a2);
                mun = muo + w * u + (v1 * u2 - v2 * u1);
            } else if (kind == 2) {
                pn = (int64_t)((uint64_t)po + (uint64_t)tr.t[a]);
            } else if (kind == 3) {
                pn = tr.t[a];
                mun = tr.q[1 + a];
            }
            if (lane < 3) {
                S.po[a] = po;
                S.pn[a] = pn;
                S.muo[a] = muo;
                S.mun[a] = mun;
                if (d.surf_c != 0.0) {   // positions in Angstrom for the surface sums only
                    S.ro[a] = (double)po * d.s64[a];
                    S.rn[a] = (double)pn * d.s64[a];
                }
            }
            const bool fixed = __all_sync(0xffffffffu, lane >= 3 || pn == po);
            const bool same_mu = __all_sync(0xffffffffu, lane >= 3 || mun == muo);
            if (lane == 0) {
                S.idx = i;
                S.thr = tr.thr;
                S.ta = A.type[i];
                S.qa = A.q[i];
                S.qeff = A.q[i] * d.eff[S.ta];
                S.mas = A.mus[i];
                S.fixed = fixed ? 1 : 0;
                S.same_mu = same_mu ? 1 : 0;
            }
        }
        __syncthreads();
        if (mode != 2) {
            // ---- axis tables of the moved particle, old (w = 0) and new (w = 1;
            // a rotation keeps the position: old only)
            const bool fixed = S.fixed;
            const int nw = fixed ? 1 : 2;
            for (int e = tid; e < nw * 3 * st; e += T) {
                const int w = e / (3 * st), r = e - w * 3 * st, a = r / st, n = r - a * st;
                S.tab[w][r] = axis_entry_df(n, w ? S.pn[a] : S.po[a], d.sctab);
            }
            const int sl = tid - (T - 32);   // the last warp, beside the axis tables
            if (sl >= 0 && sl < 10) {   // one value per lane
                if (sl == 9) {
                    S.qeffd = dsplit(S.qeff);
                } else {
                    const int a = sl % 3, w = sl / 3;
                    const double f = d.tpl[a] * S.mas;
                    const double v = w == 0 ? S.muo[a] : (w == 1 ? S.mun[a] : S.mun[a] - S.muo[a]);
                    (w == 0 ? S.mo : (w == 1 ? S.mn : S.md))[a] = dsplit(v * f);
                }
            }
            __syncthreads();
            for (int e = tid; e < nw * d.nyz; e += T) {   // the entries the k-vectors use
                const int w = e >= d.nyz ? 1 : 0, r = __ldg(d.yzl + (e - w * d.nyz));
                const int ny = r / W - d.kcc, nz = r - (ny + d.kcc) * W - d.kcc;
                const dc ey = dc_conj_if(dc_load(S.tab[w][st + (ny < 0 ? -ny : ny)]), ny < 0);
                const dc ez = dc_conj_if(dc_load(S.tab[w][2 * st + (nz < 0 ? -nz : nz)]), nz < 0);
                eyz[w * W2 + r] = dc_pack(dc_mulq(ey, ez));
            }
            __syncthreads();
            const int i = S.idx, ta = S.ta;
            const double qa = S.qa, mas = S.mas;
            const double muo[3] = {S.muo[0], S.muo[1], S.muo[2]}, mun[3] = {S.mun[0], S.mun[1], S.mun[2]};
            double acc = 0.0;
            // ---- real space: the moved particle against every other one. Far
            // pairs (both distances beyond rf) in FP32 where they are found;
            // near pairs queued per warp in order and evaluated afterwards in
            // FP64 by consecutive threads, so only the warps they fill run FP64.
            const double dmu[3] = {mun[0] - muo[0], mun[1] - muo[1], mun[2] - muo[2]};
            const float4 mao = make_float4((float)(muo[0] * mas), (float)(muo[1] * mas), (float)(muo[2] * mas), (float)qa);
            const float4 man = make_float4((float)(mun[0] * mas), (float)(mun[1] * mas), (float)(mun[2] * mas), (float)qa);
            const float3 dmf = make_float3((float)(dmu[0] * mas), (float)(dmu[1] * mas), (float)(dmu[2] * mas));
            const float sx = (float)(d.L[0] * 2.3283064365386963e-10), sy = (float)(d.L[1] * 2.3283064365386963e-10),
                        sz = (float)(d.L[2] * 2.3283064365386963e-10);   // L / 2^32
            const int warp = tid >> 5, lane = tid & 31, iters = (d.N + T - 1) / T;
            int32_t *wq = d.nearq + warp * iters * 32;
            int nq = 0;
            df accf = {0.0f, 0.0f};
            for (int it = 0; it < iters; it++) {
                const int j = it * T + tid;
                bool nearp = false;
                if (j < d.N && j != i) {
                    const int64_t pj0 = A.pos[3 * j], pj1 = A.pos[3 * j + 1], pj2 = A.pos[3 * j + 2];
                    const float ox = hi_diff(S.po[0], pj0) * sx, oy = hi_diff(S.po[1], pj1) * sy,
                                oz = hi_diff(S.po[2], pj2) * sz;
                    const float r2o = ox * ox + oy * oy + oz * oz;
                    if (fixed) {
                        nearp = r2o < d.rf2f;
                        if (!nearp) accf = fg::df_add_f(accf, far_turn(d, ox, oy, oz, dmf, A.pf[j]));
                    } else {
                        const float nx = hi_diff(S.pn[0], pj0) * sx, ny = hi_diff(S.pn[1], pj1) * sy,
                                    nz = hi_diff(S.pn[2], pj2) * sz;
                        nearp = r2o < d.rf2f || nx * nx + ny * ny + nz * nz < d.rf2f;
                        if (!nearp) {
                            const float4 mb = A.pf[j];
                            const int tb = A.type[j];
                            accf = fg::df_add_f(accf, far_pair(d, nx, ny, nz, ta, man, tb, mb) -
                                                          far_pair(d, ox, oy, oz, ta, mao, tb, mb));
                        }
                    }
                }
                const unsigned b = __ballot_sync(0xffffffffu, nearp);
                if (nearp) wq[nq + __popc(b & ((1u << lane) - 1u))] = j;
                nq += __popc(b);
            }
            if (lane == 0) S.qcnt[warp] = nq;
            __syncthreads();
            int total = 0;
            for (int w = 0; w < (T >> 5); w++) total += S.qcnt[w];
            // a translation's pair takes two threads, one for the old position
            // (subtracted) and one for the new
            const int ne = fixed ? total : 2 * total;
            for (int e = tid; e < ne; e += T) {
                const int pi = fixed ? e : (e >> 1);
                const bool at_new = !fixed && (e & 1);
                int w = 0, r = pi;
                while (r >= S.qcnt[w]) {
                    r -= S.qcnt[w];
                    w++;
                }
                const int j = d.nearq[w * iters * 32 + r];
                int64_t pj[3];
                double mb[3];
                for (int a = 0; a < 3; a++) {
                    pj[a] = A.pos[3 * j + a];
                    mb[a] = A.mu[3 * j + a];
                }
                const double qb = A.q[j], mbs = A.mus[j];
                double rv[3];
                for (int a = 0; a < 3; a++)
                    rv[a] = (double)(int64_t)((uint64_t)(at_new ? S.pn[a] : S.po[a]) - (uint64_t)pj[a]) * d.s64[a];
                if (fixed) {
                    acc += dip_turn(d, rv[0], rv[1], rv[2], mas, dmu, qb, mbs, mb);
                    continue;
                }
                const int tb = A.type[j];
                double ev, lv;
                dip_pair(d, rv[0], rv[1], rv[2], qa, ta, mas, at_new ? mun : muo, qb, tb, mbs, mb, ev, lv);
                acc += at_new ? ev + lv : -(ev + lv);
            }
            acc += (double)accf.hi + (double)accf.lo;
            // ---- k space (df): increments of Q_ion and Q_dip and the energy change.
            // A translation keeps the dipole (k.mu_new = k.mu_old): dQ_dip =
            // i (k.mu) mu_s (e_new - e_old), dQ_ion = q eff (e_new - e_old).
            df ek = {0.0f, 0.0f};
            const df qeffd = S.qeffd;
            const bool same_mu = S.same_mu;
            const df mo[3] = {S.mo[0], S.mo[1], S.mo[2]}, mn[3] = {S.mn[0], S.mn[1], S.mn[2]},
                     md[3] = {S.md[0], S.md[1], S.md[2]};
            for (int k = tid; k < d.K; k += T) {
                const char4 n = A.kn[k];
                const int yz = (n.y + d.kcc) * W + n.z + d.kcc;
                const dc eo = dc_mulq(dc_load(S.tab[0][n.x]), dc_load(eyz[yz]));
                dc dci = {{0.0f, 0.0f}, {0.0f, 0.0f}}, dcd = dci;
                if (fixed) {
                    // the dipole turns in place: dQ_dip = i (k.dmu) mu_s e^{ik.r}
                    if (d.dip_q) {
                        const df kmd = dkdotq(n, md);
                        dcd = {dneg(dmul(kmd, eo.im)), dmul(kmd, eo.re)};
                    }
                } else {
                    const dc en = dc_mulq(dc_load(S.tab[1][n.x]), dc_load(eyz[W2 + yz]));
                    const dc de = {qsub(en.re, eo.re), qsub(en.im, eo.im)};
                    if (d.ion_q) dci = {dmul(qeffd, de.re), dmul(qeffd, de.im)};
                    if (d.dip_q) {
                        if (same_mu) {
                            const df km = dkdotq(n, mo);
                            dcd = {dneg(dmul(km, de.im)), dmul(km, de.re)};
                        } else {
                            const df kmo = dkdotq(n, mo), kmn = dkdotq(n, mn);
                            dcd = {qsub(dmul(kmo, eo.im), dmul(kmn, en.im)), qsub(dmul(kmn, en.re), dmul(kmo, eo.re))};
                        }
                    }
                }
                df sum = {0.0f, 0.0f};
                if (d.ii) {
                    const dc Qi = dc_load(A.fqi[k]);
                    sum = qadd(dtwice(dc_dotq(Qi, dci)), dc_dotq(dci, dci));
                }
                if (d.id) {
                    const dc Qi = dc_load(A.fqi[k]), Qd = dc_load(A.fqd[k]);
                    if (d.quirk)
                        sum = qadd(sum, dtwice(qadd(qadd(dc_rprodq(Qi, dcd), dc_rprodq(dci, Qd)), dc_rprodq(dci, dcd))));
                    else
                        sum = qadd(sum, dtwice(qadd(qadd(dc_dotq(Qi, dcd), dc_dotq(dci, Qd)), dc_dotq(dci, dcd))));
                }
                if (d.dd) {
                    const dc Qd = dc_load(A.fqd[k]);
                    const df t = qadd(dtwice(dc_dotq(Qd, dcd)), dc_dotq(dcd, dcd));
                    sum = (d.ii || d.id) ? qadd(sum, t) : t;
                }
                const float2 a = A.akf[k];
                ek = qadd(ek, dmul_u(df{a.x, a.y}, sum));
                if (d.ion_q) A.dqi[k] = dc_pack(dci);
                if (d.dip_q) A.dqd[k] = dc_pack(dcd);
            }
            acc += dval(ek) * d.recip_c;
            // the block sum without its leading barrier: red was last read
            // before the previous trial's decision barrier
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0) S.red[warp] = acc;
            __syncthreads();
            double sum = 0.0;
            if (tid == 0)
                for (int w = 0; w < (T >> 5); w++) sum += S.red[w];
            if (tid == 0) {
                // surface term from the running sums (nothing with tin-foil surroundings)
                double du = sum;
                if (d.surf_c != 0.0) {
                    double D[3];
                    for (int a = 0; a < 3; a++)
                        D[a] = (d.ion_q ? S.qeff * (S.rn[a] - S.ro[a]) : 0.0) +
                               ((d.id || d.dd) ? S.mas * (S.mun[a] - S.muo[a]) : 0.0);
                    du += surface_change(d, S.M, D);
                }
                S.du = du;
                if (!isfinite(du)) sc.error |= kDipErrNonFinite;
                if (mode == 0) {
                    const double kT = d.kT;
                    S.accept = !(du > kT * S.thr) ? 1 : 0;   // NaN dU accepts, as u > exp(NaN) is false
                    if (d.log_du) {
                        d.log_du[t] = du;
                        d.log_acc[t] = (uint8_t)S.accept;
                    }
                } else {
                    S.accept = 0;
                    sc.pend_du = du;
                }
            }
        } else if (tid == 0) {
            S.accept = 1;
            S.du = sc.pend_du;
        }
        __syncthreads();
        if (!S.accept) continue;
        // ---- accepted: Q(k), the particle, the sums
        for (int k = tid; k < d.K; k += T) {
            if (d.ion_q) {
                const dc a = dc_load(A.fqi[k]), b = dc_load(A.dqi[k]);
                A.fqi[k] = dc_pack({dadd(a.re, b.re), dadd(a.im, b.im)});
            }
            if (d.dip_q) {
                const dc a = dc_load(A.fqd[k]), b = dc_load(A.dqd[k]);
                A.fqd[k] = dc_pack({dadd(a.re, b.re), dadd(a.im, b.im)});
            }
        }
        if (tid < 3) {   // lane a: axis a of the particle and of the sums
            const int i = S.idx, a = tid;
            const float pa = (float)(S.mun[a] * S.mas);
            reinterpret_cast<float *>(&A.pf[i])[a] = pa;
            A.pos[3 * i + a] = S.pn[a];
            A.mu[3 * i + a] = S.mun[a];
            if (stage) {
                reinterpret_cast<float *>(&d.pf[i])[a] = pa;
                d.pos[3 * i + a] = S.pn[a];
                d.mu[3 * i + a] = S.mun[a];
            }
            if (d.ion_q && d.surf_c != 0.0) S.M[a] += S.qeff * (S.rn[a] - S.ro[a]);
            if (d.id || d.dd) S.M[3 + a] += S.mas * (S.mun[a] - S.muo[a]);
        }
        if (tid == 0) {
            sc.n_accepted++;
            sc.usum += S.du;
            sc.utot += S.du;
            S.rebuild = 0;
            if (++sc.cnt_accepted > d.uf - 1) {   // NonbondedEwald::update (ewald.h:633)
                sc.cnt_accepted = 0;
                S.rebuild = 1;
            }
        }
        __syncthreads();
        if (S.rebuild) {
            double before, after;
            dip_rebuild(d, A, S, before, after);
            if (tid == 0) {
                sc.n_rebuilds++;
                sc.drift += fabs(after - before);
                sc.usum += after - before;
                sc.utot += after - before;
            }
        }
    }
    if (stage)   // Q(k) back to global memory (each thread its own k-vectors)
        for (int k = tid; k < d.K; k += T) {
            if (d.ion_q) d.fqi[k] = A.fqi[k];
            if (d.dip_q) d.fqd[k] = A.fqd[k];
        }
    if (tid == 0) {
        if (mode == 0) sc.cursor = t1;
        for (int a = 0; a < 6; a++) sc.M[a] = S.M[a];
        // the host may have moved the stream end while this kernel was queued
        sc.n_trials = d.sc->n_trials;
        *d.sc = sc;
    }
}

// Whole-system pair sums for the total energy: row i against j > i, one
// block per row; out[2 i] = EwaldReal, out[2 i + 1] = LJ.
__global__ void __launch_bounds__(kDipMaxThreads) dip_pairs_kernel(const DipDesc *dp, double *out) {
    const DipDesc &d = *dp;
    __shared__ double red[kDipMaxThreads / 32];
    const int i = blockIdx.x;
    double er = 0.0, el = 0.0;
    double ma[3];
    for (int a = 0; a < 3; a++) ma[a] = d.mu[3 * i + a];
    for (int j = i + 1 + threadIdx.x; j < d.N; j += blockDim.x) {
        double r[3], mb[3];
        for (int a = 0; a < 3; a++) {
            r[a] = (double)(int64_t)((uint64_t)d.pos[3 * i + a] - (uint64_t)d.pos[3 * j + a]) * d.s64[a];
            mb[a] = d.mu[3 * j + a];
        }
        double e, l;
        dip_pair(d, r[0], r[1], r[2], d.q[i], d.type[i], d.mus[i], ma, d.q[j], d.type[j], d.mus[j], mb, e, l);
        er += e;
        el += l;
    }
    const double s0 = block_sum(er, red);
    const double s1 = block_sum(el, red);
    if (threadIdx.x == 0) {
        out[2 * i] = s0;
        out[2 * i + 1] = s1;
    }
}

}  // namespace fgd

struct fg_dipsys {
    fg_params P{};
    int N = 0, K = 0, kcc = 0;
    int device = 0;
    int threads = 128;   // four warps per system at <= 128 registers: four systems share an SM
    cudaStream_t stream = nullptr;
    fgd::DipDesc desc{};
    fgd::DipDesc *d_desc = nullptr;
    int64_t *pos = nullptr;
    double *mu = nullptr, *mus = nullptr, *q = nullptr, *ak = nullptr, *pairs = nullptr;
    int32_t *type = nullptr, *nearq = nullptr;
    float4 *pf = nullptr, *sctab = nullptr;
    int16_t *yzl = nullptr;
    char4 *kn = nullptr;
    double2 *qi = nullptr, *qd = nullptr;
    float4 *fqi = nullptr, *fqd = nullptr, *dqi = nullptr, *dqd = nullptr;
    float2 *akf = nullptr;
    fgd::DipTrial *trials = nullptr;
    int64_t trials_cap = 0;
    double *log_du = nullptr;
    uint8_t *log_acc = nullptr;
    int64_t log_cap = 0;
    fgd::DipScalars *sc = nullptr;
    int64_t n_stream = 0;
    int64_t acc0 = 0;
    bool pending = false;
    bool state_set = false;
    std::vector<double> ak_h, charges_h, mus_h;
    std::vector<int32_t> types_h;
    std::vector<char4> kn_h;
    std::vector<double> rtab_key;   // shared radial table in use
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    size_t device_bytes = 0;
};

namespace {

void dip_radial_release(fg_dipsys *h);

void dip_free(fg_dipsys *h) {
    dip_radial_release(h);
    void *ptrs[] = {h->d_desc, h->pos, h->mu, h->mus, h->q, h->ak, h->pairs, h->type, h->nearq, h->pf, h->sctab, h->yzl, h->kn,
                    h->qi, h->qd,
                    h->fqi, h->fqd, h->dqi, h->dqd, h->akf, h->trials, h->log_du, h->log_acc, h->sc};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
}

int dip_dmalloc(fg_dipsys *h, void **p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    h->device_bytes += bytes;
    return FG_OK;
}

int dip_push_desc(fg_dipsys *h) {
    CK(cudaMemcpyAsync(h->d_desc, &h->desc, sizeof(fgd::DipDesc), cudaMemcpyHostToDevice, h->stream));
    return FG_OK;
}

// Squared far radius: beyond rf no pair term of this state (largest charge,
// dipole, LJ and effective-charge factors) exceeds 1e-4 kT, so the FP32
// rounding of a far pair (a few ulp) is below 1e-10 kT. Ewald terms end at
// rc, LJ has no cutoff. Bisection on the decreasing bound.
float dip_far_radius2(const fg_dipsys *h) {
    const fgd::DipDesc &d = h->desc;
    const int nt = d.nt;
    double qm = 0.0, mm = 0.0, e4 = 0.0, s2 = 0.0, qq = 0.0;
    for (int i = 0; i < h->N; i++) {
        qm = std::max(qm, std::fabs(h->charges_h[i]));
        mm = std::max(mm, std::fabs(h->mus_h[i]));
    }
    for (int k = 0; k < nt * nt; k++) {
        e4 = std::max(e4, std::fabs(d.eps4[k]));
        s2 = std::max(s2, d.s2[k]);
        qq = std::max(qq, std::fabs(d.qeqe[k]));
    }
    auto bound = [&](double r) {
        const double r2 = r * r, x = s2 / r2, x3 = x * x * x;
        double b = e4 * (x3 * x3 + x3);
        if (!d.any_term || r2 > d.rc2) return b;
        const double ar = d.alpha * r, ec = std::erfc(ar), ex = std::exp(-d.alpha2 * r2);
        if (d.quirk || d.ii) {
            const double h2 = d.kappa / 2.0 / d.alpha;
            const double t = d.small_kappa ? ec / r
                                           : (std::erfc(ar + h2) * std::exp(d.kappa * r) +
                                              std::erfc(ar - h2) * std::exp(-d.kappa * r)) / (2.0 * r);
            b += d.lB * qm * qm * qq * t;
        }
        if (!d.quirk) {
            const double T1f = r * d.t1c * ex + ec, T2f = 3.0 * (T1f + d.t2c * r * r * r * ex);
            if (d.id) b += d.lB * 2.0 * qm * mm * T1f / r2;
            if (d.dd) b += d.lB * mm * mm * (T1f + T2f) / (r2 * r);
        }
        return b;
    };
    const double eps = 1e-4;
    double hi = 0.5 * std::sqrt(d.L[0] * d.L[0] + d.L[1] * d.L[1] + d.L[2] * d.L[2]) + 1.0, lo = 1e-3;
    if (bound(hi) > eps) return 3.0e38f;   // nothing is far
    for (int it = 0; it < 60; it++) {
        const double mid = 0.5 * (lo + hi);
        if (bound(mid) > eps) lo = mid;
        else hi = mid;
    }
    const double rf = hi + 1e-3;   // covers the float distance of the high words
    return (float)(rf * rf);
}

// ---- interpolation tables of the radial functions, shared by every system
// with the same (alpha, kappa, rc): a degree-5 polynomial per interval,
// interpolating at the six Chebyshev points of the interval (computed in long
// double), checked against the functions before use.
struct RadialTab {
    double *dev = nullptr;
    int refs = 0;
};
std::mutex g_rtab_mu;
std::map<std::vector<double>, RadialTab> g_rtab;

constexpr int kRadialIntervals = 4096;

void radial_exact(long double alpha, long double kappa, bool small_kappa, long double s, long double f[3]) {
    const long double r = std::sqrt(s), ar = alpha * r;
    const long double ec = std::erfc(ar), ex = std::exp(-alpha * alpha * s);
    if (small_kappa) {
        f[0] = ec / r;
    } else {
        const long double h = kappa / 2 / alpha;
        f[0] = (std::erfc(ar + h) * std::exp(kappa * r) + std::erfc(ar - h) * std::exp(-kappa * r)) / (2 * r);
    }
    const long double pi = 3.141592653589793238462643383279502884L;
    const long double T1f = r * 2 * alpha / std::sqrt(pi) * ex + ec;
    f[1] = T1f / (r * s);
    f[2] = 3 * (T1f + 4 * alpha * alpha * alpha / 3 / std::sqrt(pi) * r * s * ex) / (s * s * r);
}

// Builds (or finds) the table for h's parameters; returns 0 and sets the
// descriptor fields, or leaves them null when the check fails.
int dip_radial_table(fg_dipsys *h) {
    fgd::DipDesc &d = h->desc;
    d.rtab = nullptr;
    if (!d.any_term) return FG_OK;
    const double ts0 = 4.0;   // r >= 2 A from the table, closer pairs directly
    if (!(d.rc2 > ts0 * 1.01)) return FG_OK;
    std::vector<double> key = {d.alpha, d.kappa, d.rc2, (double)d.small_kappa};
    std::lock_guard<std::mutex> lk(g_rtab_mu);
    RadialTab &t = g_rtab[key];
    const double w = (d.rc2 - ts0) / kRadialIntervals;
    if (!t.dev) {
        const int n = kRadialIntervals;
        std::vector<double> c((size_t)n * 18);
        const long double pi = 3.141592653589793238462643383279502884L;
        bool ok = true;
        for (int k = 0; k < n && ok; k++) {
            // Chebyshev points of [0, 1], Newton divided differences, then monomial coefficients
            long double tx[6], fy[3][6];
            for (int j = 0; j < 6; j++) {
                tx[j] = (1 - std::cos((2 * j + 1) * pi / 12)) / 2;
                long double f[3];
                radial_exact(d.alpha, d.kappa, d.small_kappa, ts0 + (k + tx[j]) * (long double)w, f);
                for (int m = 0; m < 3; m++) fy[m][j] = f[m];
            }
            for (int m = 0; m < 3; m++) {
                long double dd[6];
                for (int j = 0; j < 6; j++) dd[j] = fy[m][j];
                for (int o = 1; o < 6; o++)
                    for (int j = 5; j >= o; j--) dd[j] = (dd[j] - dd[j - 1]) / (tx[j] - tx[j - o]);
                long double poly[6] = {0, 0, 0, 0, 0, 0};
                for (int j = 5; j >= 0; j--) {   // poly = poly * (t - tx[j]) + dd[j]
                    for (int o = 5; o >= 1; o--) poly[o] = poly[o - 1] - tx[j] * poly[o];
                    poly[0] = -tx[j] * poly[0] + dd[j];
                }
                for (int o = 0; o < 6; o++) c[(size_t)k * 18 + 6 * m + o] = (double)poly[o];
            }
            for (long double tt : {0.0L, 0.29L, 0.61L, 0.97L}) {
                long double f[3];
                radial_exact(d.alpha, d.kappa, d.small_kappa, ts0 + (k + tt) * (long double)w, f);
                for (int m = 0; m < 3; m++) {
                    const double *cc = &c[(size_t)k * 18 + 6 * m];
                    const double tv = (double)tt;
                    const double v = ((((cc[5] * tv + cc[4]) * tv + cc[3]) * tv + cc[2]) * tv + cc[1]) * tv + cc[0];
                    if (std::fabs((long double)v - f[m]) > 1e-13L * std::fabs(f[m])) ok = false;
                }
            }
        }
        if (!ok) {
            g_rtab.erase(key);
            return FG_OK;   // direct evaluation
        }
        CK(cudaMalloc(&t.dev, c.size() * sizeof(double)));
        CK(cudaMemcpy(t.dev, c.data(), c.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    t.refs++;
    h->rtab_key = key;
    d.rtab = t.dev;
    d.ts0 = ts0;
    d.tinv = 1.0 / w;
    d.tn = kRadialIntervals;
    return FG_OK;
}

void dip_radial_release(fg_dipsys *h) {
    if (h->rtab_key.empty()) return;
    std::lock_guard<std::mutex> lk(g_rtab_mu);
    auto it = g_rtab.find(h->rtab_key);
    if (it != g_rtab.end() && --it->second.refs <= 0) {
        cudaFree(it->second.dev);
        g_rtab.erase(it);
    }
    h->rtab_key.clear();
}

int dip_read_scalars(fg_dipsys *h, fgd::DipScalars &s) {
    CK(cudaMemcpyAsync(&s, h->sc, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

int dip_write_scalars(fg_dipsys *h, const fgd::DipScalars &s) {
    CK(cudaMemcpyAsync(h->sc, &s, sizeof(s), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

int dip_ensure_trials(fg_dipsys *h, int64_t n, bool log) {
    if (n > h->trials_cap) {
        if (h->trials) cudaFree(h->trials);
        h->trials = nullptr;
        const int64_t cap = std::max<int64_t>(n, 1024);
        int rc = dip_dmalloc(h, (void **)&h->trials, (size_t)cap * sizeof(fgd::DipTrial));
        if (rc) return rc;
        h->trials_cap = cap;
        h->desc.trials = h->trials;
    }
    if (log && n > h->log_cap) {
        if (h->log_du) cudaFree(h->log_du);
        if (h->log_acc) cudaFree(h->log_acc);
        h->log_du = nullptr;
        h->log_acc = nullptr;
        int rc = dip_dmalloc(h, (void **)&h->log_du, (size_t)n * sizeof(double));
        if (!rc) rc = dip_dmalloc(h, (void **)&h->log_acc, (size_t)n);
        if (rc) return rc;
        h->log_cap = n;
    }
    h->desc.log_du = log ? h->log_du : nullptr;
    h->desc.log_acc = log ? h->log_acc : nullptr;
    return dip_push_desc(h);
}

// The reciprocal, self and surface energies from the host copies and Q(k).
int dip_host_energies(fg_dipsys *h, const std::vector<double> &xyz, const std::vector<double> &mu, double &rec,
                      double &self, double &surf) {
    const fgd::DipDesc &d = h->desc;
    std::vector<float4> fi(h->K), fd(h->K);
    std::vector<double2> qi(h->K), qd(h->K);
    if (h->K) {
        CK(cudaMemcpyAsync(fi.data(), h->fqi, h->K * sizeof(float4), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(fd.data(), h->fqd, h->K * sizeof(float4), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    for (int k = 0; k < h->K; k++) {
        qi[k] = make_double2((double)fi[k].x + (double)fi[k].y, (double)fi[k].z + (double)fi[k].w);
        qd[k] = make_double2((double)fd[k].x + (double)fd[k].y, (double)fd[k].z + (double)fd[k].w);
    }
    rec = 0.0;
    for (int k = 0; k < h->K; k++) {
        double s = 0.0;
        if (d.ii) s += qi[k].x * qi[k].x + qi[k].y * qi[k].y;
        if (d.id) s += 2.0 * (d.quirk ? qi[k].x * qd[k].x - qi[k].y * qd[k].y : qi[k].x * qd[k].x + qi[k].y * qd[k].y);
        if (d.dd) s += qd[k].x * qd[k].x + qd[k].y * qd[k].y;
        rec += h->ak_h[k] * s;
    }
    rec *= d.recip_c;
    double Eq = 0.0, Emu = 0.0, M[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < h->N; i++) {
        const double qe = h->charges_h[i] * d.eff[h->types_h[i]];
        if (d.ion_q) {
            Eq += qe * qe;
            for (int a = 0; a < 3; a++) M[a] += qe * xyz[3 * i + a];
        }
        if (d.id || d.dd) {
            Emu += h->mus_h[i] * h->mus_h[i];
            for (int a = 0; a < 3; a++) M[3 + a] += mu[3 * i + a] * h->mus_h[i];
        }
    }
    self = (-d.alpha * (Eq + d.alpha2 * (2.0 / 3.0) * Emu) / std::sqrt(PI)) * d.lB;
    surf = d.surf_c * (M[0] * M[0] + M[1] * M[1] + M[2] * M[2] + 2.0 * (M[0] * M[3] + M[1] * M[4] + M[2] * M[5]) +
                       M[3] * M[3] + M[4] * M[4] + M[5] * M[5]);
    return FG_OK;
}

int dip_get_state(fg_dipsys *h, std::vector<double> &xyz, std::vector<double> &mu) {
    std::vector<int64_t> X(3 * (size_t)h->N);
    mu.resize(3 * (size_t)h->N);
    CK(cudaMemcpyAsync(X.data(), h->pos, X.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(mu.data(), h->mu, mu.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    xyz.resize(X.size());
    for (size_t k = 0; k < X.size(); k++) xyz[k] = from_fix(X[k], h->P.box[k % 3]);
    return FG_OK;
}

// comp = {EwaldReal pairs, LJ pairs, reciprocal, self, surface, total}
int dip_total(fg_dipsys *h, double *comp) {
    fgd::dip_pairs_kernel<<<h->N, 128, 0, h->stream>>>(h->d_desc, h->pairs);
    CK(cudaGetLastError());
    std::vector<double> rows(2 * (size_t)h->N);
    CK(cudaMemcpyAsync(rows.data(), h->pairs, rows.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    double er = 0.0, el = 0.0;
    for (int i = 0; i < h->N; i++) {
        er += rows[2 * i];
        el += rows[2 * i + 1];
    }
    std::vector<double> xyz, mu;
    int rc = dip_get_state(h, xyz, mu);
    if (rc) return rc;
    double rec, self, surf;
    rc = dip_host_energies(h, xyz, mu, rec, self, surf);
    if (rc) return rc;
    comp[0] = er;
    comp[1] = el;
    comp[2] = rec;
    comp[3] = self;
    comp[4] = surf;
    comp[5] = er + el + rec + self + surf;
    return FG_OK;
}

// Shared memory of a sweep launch over these systems: the staged layout
// when every system's fits in kDipStageMax (two or more CTAs per SM), else
// the yz table alone.
constexpr size_t kDipStageMax = 110 * 1024;

size_t dip_launch_smem(fg_dipsys *const *sys, int n, int &stage) {
    size_t yz = 0, st = 0;
    for (int i = 0; i < n; i++) {
        const fgd::DipDesc &d = sys[i]->desc;
        size_t off[12];
        yz = std::max(yz, fgd::dip_yz_bytes(d.kcc));
        st = std::max(st, fgd::dip_stage_layout(d.K, d.N, d.kcc, d.ion_q, d.dip_q, off));
    }
    stage = st <= kDipStageMax ? 1 : 0;
    return stage ? st : yz;
}

int dip_launch(fg_dipsys *const *sys, const fgd::DipDesc *descs, int n, int mode, cudaStream_t st) {
    int stage = 0;
    size_t smem = dip_launch_smem(sys, n, stage);
    if (mode != 0) {
        stage = 0;
        smem = fgd::dip_yz_bytes(sys[0]->kcc);
    }
    const int T = sys[0]->threads;
    const void *fn = T <= 128 ? (const void *)fgd::dip_sweep_kernel<128> : (const void *)fgd::dip_sweep_kernel<fgd::kDipMaxThreads>;
    CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (T <= 128)
        fgd::dip_sweep_kernel<128><<<n, T, smem, st>>>(descs, mode, stage);
    else
        fgd::dip_sweep_kernel<fgd::kDipMaxThreads><<<n, T, smem, st>>>(descs, mode, stage);
    CK(cudaGetLastError());
    return FG_OK;
}

int dip_run(fg_dipsys *const *sys, int n, fg_sweep_stats *per, fg_sweep_stats *total) {
    if (!sys || n < 1) return fail(FG_ERR_INVALID, "bad argument");
    fg_dipsys *h0 = sys[0];
    int64_t maxn = 0;
    for (int i = 0; i < n; i++) {
        fg_dipsys *h = sys[i];
        if (!h || !h->state_set) return fail(FG_ERR_STATE, "system %d has no state", i);
        if (h->pending) return fail(FG_ERR_STATE, "system %d has a pending trial: commit it first", i);
        if (h->device != h0->device) return fail(FG_ERR_INVALID, "systems must share the device");
        if (h->threads != h0->threads) return fail(FG_ERR_INVALID, "systems must share the block size");
        maxn = std::max(maxn, h->n_stream);
        CK(cudaStreamSynchronize(h->stream));
    }
    cudaStream_t st = h0->stream;
    const fgd::DipDesc *descs = h0->d_desc;
    fgd::DipDesc *tmp = nullptr;
    if (n > 1) {
        std::vector<fgd::DipDesc> v(n);
        for (int i = 0; i < n; i++) v[i] = sys[i]->desc;
        CK(cudaMalloc(&tmp, n * sizeof(fgd::DipDesc)));
        CK(cudaMemcpyAsync(tmp, v.data(), n * sizeof(fgd::DipDesc), cudaMemcpyHostToDevice, st));
        descs = tmp;
    }
    // launches of at most kChunk trials per system keep each kernel short
    const int64_t kChunk = 16384;
    const int64_t nl = (maxn + kChunk - 1) / kChunk;
    std::vector<int64_t> ends((size_t)std::max<int64_t>(nl, 1) * n);
    CK(cudaEventRecord(h0->ev0, st));
    int rc = FG_OK;
    for (int64_t c = 0; c < nl && !rc; c++) {
        for (int i = 0; i < n; i++) {
            int64_t &e = ends[(size_t)c * n + i];
            e = std::min(sys[i]->n_stream, (c + 1) * kChunk);
            CK(cudaMemcpyAsync(&sys[i]->sc->n_trials, &e, sizeof(int64_t), cudaMemcpyHostToDevice, st));
        }
        rc = dip_launch(sys, descs, n, 0, st);
    }
    CK(cudaEventRecord(h0->ev1, st));
    CK(cudaEventSynchronize(h0->ev1));
    if (tmp) cudaFree(tmp);
    if (rc) return rc;
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, h0->ev0, h0->ev1));
    std::vector<fgd::DipScalars> s1(n);
    for (int i = 0; i < n; i++)
        CK(cudaMemcpyAsync(&s1[i], sys[i]->sc, sizeof(fgd::DipScalars), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    fg_sweep_stats tot{};
    int errs = 0;
    for (int i = 0; i < n; i++) {
        fg_sweep_stats x{};
        x.trials = s1[i].cursor;
        x.accepted = s1[i].n_accepted - sys[i]->acc0;
        x.energy_change = s1[i].usum;
        x.device_ms = ms;
        x.sweep_kernel_ms = ms;
        x.sweep_launches = (int32_t)nl;
        x.error_flags = s1[i].error;
        x.kernel_launches = nl;
        x.rebuilds = s1[i].n_rebuilds;
        errs |= s1[i].error;
        if (per) per[i] = x;
        tot.trials += x.trials;
        tot.accepted += x.accepted;
        tot.rebuilds += x.rebuilds;
        tot.energy_change += x.energy_change;
        sys[i]->n_stream = 0;
    }
    tot.device_ms = ms;
    tot.sweep_kernel_ms = ms;
    tot.sweep_launches = (int32_t)nl;
    tot.kernel_launches = nl;
    tot.error_flags = errs;
    if (total) *total = tot;
    if (errs) return fail(FG_ERR_DEVICE, "device error flags 0x%x", errs);
    return FG_OK;
}

int dip_upload(fg_dipsys *h, int64_t n, const int32_t *kind, const int32_t *idx, const double *axis,
               const double *angle, const double *disp, const double *u, bool log) {
    if (!h || n < 0 || (n > 0 && (!kind || !idx || !u))) return fail(FG_ERR_INVALID, "bad argument");
    if (!h->state_set) return fail(FG_ERR_STATE, "fg_dip_set_state first");
    if (h->pending) return fail(FG_ERR_STATE, "a trial is pending: commit it first");
    std::vector<fgd::DipTrial> tr(n);
    for (int64_t k = 0; k < n; k++) {
        fgd::DipTrial &t = tr[k];
        t = fgd::DipTrial{};
        if (idx[k] < 0 || idx[k] >= h->N) return fail(FG_ERR_INVALID, "trial %lld: particle out of range", (long long)k);
        t.idx = idx[k];
        t.kind = kind[k];
        t.thr = u[k] > 0.0 ? -std::log(u[k]) : INFINITY;
        t.q[0] = 1.0;
        if (kind[k] == 1) {
            if (!axis || !angle) return fail(FG_ERR_INVALID, "rotations need axis and angle");
            double ax = axis[3 * k], ay = axis[3 * k + 1], az = axis[3 * k + 2];
            const double nrm = std::sqrt(ax * ax + ay * ay + az * az);
            if (!(nrm > 0)) return fail(FG_ERR_INVALID, "trial %lld: zero rotation axis", (long long)k);
            ax /= nrm;
            ay /= nrm;
            az /= nrm;
            // Eigen::AngleAxisd(angle, u) as a quaternion (geometry.cpp:762)
            const double ha = 0.5 * angle[k], sh = std::sin(ha);
            t.q[0] = std::cos(ha);
            t.q[1] = sh * ax;
            t.q[2] = sh * ay;
            t.q[3] = sh * az;
        } else if (kind[k] == 2) {
            if (!disp) return fail(FG_ERR_INVALID, "translations need disp");
            for (int a = 0; a < 3; a++) t.t[a] = to_fix(disp[3 * k + a], h->P.box[a]);
        } else {
            return fail(FG_ERR_INVALID, "trial %lld: kind must be 1 (rotation) or 2 (translation)", (long long)k);
        }
    }
    int rc = dip_ensure_trials(h, n, log);
    if (rc) return rc;
    if (n) CK(cudaMemcpyAsync(h->trials, tr.data(), n * sizeof(fgd::DipTrial), cudaMemcpyHostToDevice, h->stream));
    fgd::DipScalars s;
    rc = dip_read_scalars(h, s);
    if (rc) return rc;
    s.cursor = 0;
    s.n_trials = 0;
    s.usum = 0.0;
    s.error = 0;
    h->acc0 = s.n_accepted;
    h->n_stream = n;
    return dip_write_scalars(h, s);
}

}  // namespace

extern "C" {

int fg_dip_create(const fg_params *params, int32_t n_particles, fg_dipsys **out) {
    if (!params || !out) return fail(FG_ERR_INVALID, "null argument");
    *out = nullptr;
    const fg_params &P = *params;
    if (P.model != FG_MODEL_EWALD_DIPOLE) return fail(FG_ERR_INVALID, "fg_dip_create needs FG_MODEL_EWALD_DIPOLE");
    if (n_particles < 2 || n_particles >= (1 << 24)) return fail(FG_ERR_INVALID, "particle count must be 2..2^24");
    if (P.n_types < 1 || P.n_types > FG_MAX_TYPES) return fail(FG_ERR_INVALID, "bad type count");
    if ((P.ewald_terms & ~7) != 0) return fail(FG_ERR_INVALID, "bad ewald_terms");
    if (P.ewald_isotropic_pbc) return fail(FG_ERR_INVALID, "isotropic_pbc is built for FG_MODEL_EWALD_WCA only");
    if (!(P.bjerrum > 0) || !(P.ewald_alpha > 0) || !(P.ewald_cutoff > 0) || !(P.ewald_debye_length > 0))
        return fail(FG_ERR_INVALID, "bad Ewald parameters");
    for (int a = 0; a < 3; a++)
        if (!(P.box[a] > 0)) return fail(FG_ERR_INVALID, "bad box");
    const int kcc = (int)std::ceil(P.ewald_cutoff_k);
    if (kcc < 0 || kcc > fgd::kDipMaxKcc) return fail(FG_ERR_INVALID, "cutoffK must be 0..%d", fgd::kDipMaxKcc);
    fg_dipsys *h = new fg_dipsys();
    h->P = P;
    h->N = n_particles;
    h->kcc = kcc;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (g_tune_dip_threads) h->threads = g_tune_dip_threads;
    }
    auto bail = [&](int rc) {
        dip_free(h);
        delete h;
        return rc;
    };
    if (cudaGetDevice(&h->device) != cudaSuccess) return bail(fail(FG_ERR_CUDA, "no CUDA device"));
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(FG_ERR_CUDA, "stream"));
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);
    // k-vectors as kVectorChange enumerates them (ewald.h:330-378), n-vectors kept
    std::vector<int> n3;
    std::vector<double> ak, kv3;
    enumerate_k(P, n3, ak, kv3);
    h->K = (int)ak.size();
    h->ak_h = ak;
    h->kn_h.resize(h->K);
    for (int k = 0; k < h->K; k++)
        h->kn_h[k] = make_char4((signed char)n3[3 * k], (signed char)n3[3 * k + 1], (signed char)n3[3 * k + 2], 0);
    fgd::DipDesc &d = h->desc;
    d.N = h->N;
    d.K = h->K;
    d.kcc = kcc;
    d.nt = P.n_types;
    d.ii = (P.ewald_terms & FG_EWALD_ION_ION) ? 1 : 0;
    d.id = (P.ewald_terms & FG_EWALD_ION_DIPOLE) ? 1 : 0;
    d.dd = (P.ewald_terms & FG_EWALD_DIPOLE_DIPOLE) ? 1 : 0;
    d.quirk = P.ewald_dipole_quirk ? 1 : 0;
    d.any_term = (d.ii || d.id || d.dd) ? 1 : 0;
    d.ion_q = (d.ii || d.id) ? 1 : 0;
    d.dip_q = (d.id || d.dd) ? 1 : 0;
    d.dip_q_build = d.quirk ? d.dd : d.dip_q;
    d.uf = P.ewald_update_frequency;
    const double V = P.box[0] * P.box[1] * P.box[2];
    for (int a = 0; a < 3; a++) {
        d.L[a] = P.box[a];
        d.s64[a] = P.box[a] / TWO64;
        d.tpl[a] = 2.0 * PI / P.box[a];
    }
    d.alpha = P.ewald_alpha;
    d.alpha2 = d.alpha * d.alpha;
    d.rc2 = P.ewald_cutoff * P.ewald_cutoff;
    d.kappa = 1.0 / P.ewald_debye_length;
    // kappa / 2 alpha and kappa rc below 1e-20: erfc(ar +- h) = erfc(ar) and
    // e^{+-kappa r} = 1 in FP64, so the screened form is erfc(ar) / r exactly
    d.small_kappa = (d.kappa / (2.0 * d.alpha) < 1e-20 && d.kappa * P.ewald_cutoff < 1e-20) ? 1 : 0;
    d.lB = P.bjerrum;
    d.kT = P.kT_scale > 0 ? P.kT_scale : 1.0;
    d.recip_c = 2.0 * PI / V * d.lB;
    d.surf_c = (P.ewald_eps_surf < 1) ? 0.0 : 2.0 * PI / ((2.0 * P.ewald_eps_surf + 1.0) * V) * d.lB;
    d.t1c = 2.0 * d.alpha / std::sqrt(PI);
    d.t2c = 4.0 * d.alpha2 * d.alpha / 3.0 / std::sqrt(PI);
    const int nt = P.n_types;
    auto qs = [&](int t) {   // effective charge (ewald.h:532-549)
        const double r = 0.5 * P.type_sigma[t];
        double q = P.type_charge[t];
        if (std::fabs(d.kappa * r) > 1e-9) q *= std::sinh(r * d.kappa) / r / d.kappa;
        return q;
    };
    for (int i = 0; i < nt; i++) {
        // a neutral type has no effective charge (the reference's 0/0 is
        // never used when no ion term is on)
        d.eff[i] = P.type_charge[i] != 0.0 ? qs(i) / P.type_charge[i] : 0.0;
        for (int j = 0; j < nt; j++) {
            const double sig = 0.5 * (P.type_sigma[i] + P.type_sigma[j]);
            d.s2[i * nt + j] = sig * sig;
            d.eps4[i * nt + j] = 4 * std::sqrt(P.type_eps[i] * P.type_eps[j]);
            d.qeqe[i * nt + j] = (P.type_charge[i] != 0.0 && P.type_charge[j] != 0.0)
                                     ? qs(i) * qs(j) / P.type_charge[i] / P.type_charge[j] : 0.0;
        }
    }
    d.rc2f = (float)d.rc2;
    d.alphaf = (float)d.alpha;
    d.alpha2f = (float)d.alpha2;
    d.kappaf = (float)d.kappa;
    d.lBf = (float)d.lB;
    d.t1cf = (float)d.t1c;
    d.t2cf = (float)d.t2c;
    for (int k = 0; k < nt * nt; k++) {
        d.qeqef[k] = (float)d.qeqe[k];
        d.s2f[k] = (float)d.s2[k];
        d.eps4f[k] = (float)d.eps4[k];
    }
    d.rf2f = 3.0e38f;   // set with the state
    if (int rc0 = dip_radial_table(h)) return bail(rc0);
    int rc_;
#define TRY(x)                     \
    do {                           \
        rc_ = (x);                 \
        if (rc_) return bail(rc_); \
    } while (0)
    const size_t N = h->N, K = std::max(h->K, 1);
    TRY(dip_dmalloc(h, (void **)&h->d_desc, sizeof(fgd::DipDesc)));
    TRY(dip_dmalloc(h, (void **)&h->pos, 3 * N * sizeof(int64_t)));
    TRY(dip_dmalloc(h, (void **)&h->mu, 3 * N * sizeof(double)));
    TRY(dip_dmalloc(h, (void **)&h->mus, N * sizeof(double)));
    TRY(dip_dmalloc(h, (void **)&h->q, N * sizeof(double)));
    TRY(dip_dmalloc(h, (void **)&h->type, N * sizeof(int32_t)));
    TRY(dip_dmalloc(h, (void **)&h->nearq, (N + fgd::kDipMaxThreads) * sizeof(int32_t)));
    TRY(dip_dmalloc(h, (void **)&h->pf, N * sizeof(float4)));
    TRY(dip_dmalloc(h, (void **)&h->sctab, fgd::kDipScTab * sizeof(float4)));
    {   // the (n_y, n_z) entries of the phase table that some k-vector uses
        const int W = 2 * h->kcc + 1;
        std::vector<char> used((size_t)W * W, 0);
        for (const char4 &n : h->kn_h) used[(size_t)(n.y + h->kcc) * W + n.z + h->kcc] = 1;
        std::vector<int16_t> yz;
        for (int r = 0; r < W * W; r++)
            if (used[r]) yz.push_back((int16_t)r);
        if (yz.empty()) yz.push_back(0);
        TRY(dip_dmalloc(h, (void **)&h->yzl, yz.size() * sizeof(int16_t)));
        if (cudaMemcpy(h->yzl, yz.data(), yz.size() * sizeof(int16_t), cudaMemcpyHostToDevice))
            return bail(fail(FG_ERR_CUDA, "upload of the phase-table list failed"));
        d.yzl = h->yzl;
        d.nyz = (int)yz.size();
    }
    TRY(dip_dmalloc(h, (void **)&h->pairs, 2 * N * sizeof(double)));
    TRY(dip_dmalloc(h, (void **)&h->kn, K * sizeof(char4)));
    TRY(dip_dmalloc(h, (void **)&h->ak, K * sizeof(double)));
    TRY(dip_dmalloc(h, (void **)&h->qi, K * sizeof(double2)));
    TRY(dip_dmalloc(h, (void **)&h->qd, K * sizeof(double2)));
    TRY(dip_dmalloc(h, (void **)&h->fqi, K * sizeof(float4)));
    TRY(dip_dmalloc(h, (void **)&h->fqd, K * sizeof(float4)));
    TRY(dip_dmalloc(h, (void **)&h->dqi, K * sizeof(float4)));
    TRY(dip_dmalloc(h, (void **)&h->dqd, K * sizeof(float4)));
    TRY(dip_dmalloc(h, (void **)&h->akf, K * sizeof(float2)));
    TRY(dip_dmalloc(h, (void **)&h->sc, sizeof(fgd::DipScalars)));
    d.pos = h->pos;
    d.mu = h->mu;
    d.mus = h->mus;
    d.q = h->q;
    d.type = h->type;
    d.nearq = h->nearq;
    d.pf = h->pf;
    d.sctab = h->sctab;
    d.kn = h->kn;
    d.ak = h->ak;
    d.qi = h->qi;
    d.qd = h->qd;
    d.fqi = h->fqi;
    d.fqd = h->fqd;
    d.dqi = h->dqi;
    d.dqd = h->dqd;
    d.akf = h->akf;
    d.sc = h->sc;
    if (h->K) {
        std::vector<float2> akf(h->K);
        for (int k = 0; k < h->K; k++) akf[k] = split_df(ak[k]);
        if (cudaMemcpyAsync(h->kn, h->kn_h.data(), h->K * sizeof(char4), cudaMemcpyHostToDevice, h->stream) ||
            cudaMemcpyAsync(h->ak, ak.data(), h->K * sizeof(double), cudaMemcpyHostToDevice, h->stream) ||
            cudaMemcpyAsync(h->akf, akf.data(), h->K * sizeof(float2), cudaMemcpyHostToDevice, h->stream) ||
            cudaStreamSynchronize(h->stream))
            return bail(fail(FG_ERR_CUDA, "upload of the k-vectors failed"));
    }
    {   // cos, sin of 2 pi i / kDipScTab as df (axis_entry_df)
        std::vector<float4> sct(fgd::kDipScTab);
        for (int i = 0; i < fgd::kDipScTab; i++) {
            const long double th = 2.0L * 3.141592653589793238462643383279502884L * i / fgd::kDipScTab;
            const float2 c = split_df((double)std::cos(th)), sn = split_df((double)std::sin(th));
            sct[i] = make_float4(c.x, c.y, sn.x, sn.y);
        }
        if (cudaMemcpyAsync(h->sctab, sct.data(), sct.size() * sizeof(float4), cudaMemcpyHostToDevice, h->stream) ||
            cudaStreamSynchronize(h->stream))
            return bail(fail(FG_ERR_CUDA, "upload of the phase table failed"));
    }
    TRY(dip_ensure_trials(h, 1, false));
    fgd::DipScalars s{};
    TRY(dip_write_scalars(h, s));
#undef TRY
    *out = h;
    return FG_OK;
}

int fg_dip_destroy(fg_dipsys *h) {
    if (!h) return FG_OK;
    cudaStreamSynchronize(h->stream);
    dip_free(h);
    delete h;
    return FG_OK;
}

int fg_dip_num_kvectors(fg_dipsys *h) { return h ? h->K : 0; }

int fg_dip_set_state(fg_dipsys *h, const double *xyz, const double *mu_unit, const double *mu_scalar,
                     const double *charges, const int32_t *type_ids) {
    if (!h || !xyz || !mu_unit || !mu_scalar || !type_ids) return fail(FG_ERR_INVALID, "null argument");
    const int N = h->N;
    std::vector<int64_t> X(3 * (size_t)N);
    h->types_h.assign(type_ids, type_ids + N);
    h->charges_h.resize(N);
    h->mus_h.assign(mu_scalar, mu_scalar + N);
    for (int i = 0; i < N; i++) {
        if (type_ids[i] < 0 || type_ids[i] >= h->P.n_types) return fail(FG_ERR_INVALID, "particle %d: bad type", i);
        h->charges_h[i] = charges ? charges[i] : h->P.type_charge[type_ids[i]];
        for (int a = 0; a < 3; a++) {
            if (!std::isfinite(xyz[3 * i + a]) || !std::isfinite(mu_unit[3 * i + a]))
                return fail(FG_ERR_INVALID, "particle %d: non-finite input", i);
            X[3 * i + a] = to_fix(xyz[3 * i + a], h->P.box[a]);
        }
    }
    CK(cudaMemcpyAsync(h->pos, X.data(), X.size() * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->mu, mu_unit, 3 * (size_t)N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->mus, mu_scalar, (size_t)N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->q, h->charges_h.data(), (size_t)N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->type, type_ids, (size_t)N * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    std::vector<float4> pf(N);
    for (int i = 0; i < N; i++)
        pf[i] = make_float4((float)(mu_unit[3 * i] * mu_scalar[i]), (float)(mu_unit[3 * i + 1] * mu_scalar[i]),
                            (float)(mu_unit[3 * i + 2] * mu_scalar[i]), (float)h->charges_h[i]);
    CK(cudaMemcpyAsync(h->pf, pf.data(), (size_t)N * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
    h->desc.rf2f = dip_far_radius2(h);
    int rc = dip_push_desc(h);
    if (rc) return rc;
    fgd::DipScalars s{};
    std::vector<double> xyzw, muw;
    rc = dip_write_scalars(h, s);
    if (rc) return rc;
    h->state_set = true;
    h->pending = false;
    // surface sums and energies on the host from the uploaded (wrapped) state
    rc = dip_get_state(h, xyzw, muw);
    if (rc) return rc;
    for (int i = 0; i < N; i++) {
        const double qe = h->charges_h[i] * h->desc.eff[h->types_h[i]];
        for (int a = 0; a < 3; a++) {
            if (h->desc.ion_q) s.M[a] += qe * xyzw[3 * i + a];
            if (h->desc.id || h->desc.dd) s.M[3 + a] += muw[3 * i + a] * h->mus_h[i];
        }
    }
    rc = dip_write_scalars(h, s);
    if (rc) return rc;
    fgd::dip_build_kernel<<<1, h->threads, 0, h->stream>>>(h->d_desc);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    double comp[6];
    rc = dip_total(h, comp);
    if (rc) return rc;
    rc = dip_read_scalars(h, s);
    if (rc) return rc;
    s.utot = comp[5];
    s.n_accepted = 0;
    s.n_rebuilds = 0;
    s.cnt_accepted = 0;
    return dip_write_scalars(h, s);
}

int fg_dip_get_state(fg_dipsys *h, double *xyz, double *mu_unit) {
    if (!h) return fail(FG_ERR_INVALID, "null argument");
    if (!h->state_set) return fail(FG_ERR_STATE, "no state");
    std::vector<double> x, m;
    int rc = dip_get_state(h, x, m);
    if (rc) return rc;
    if (xyz) std::copy(x.begin(), x.end(), xyz);
    if (mu_unit) std::copy(m.begin(), m.end(), mu_unit);
    return FG_OK;
}

int fg_dip_set_threads(fg_dipsys *h, int32_t threads) {
    if (!h) return fail(FG_ERR_INVALID, "null argument");
    if (threads < 32 || threads > fgd::kDipMaxThreads || threads % 32)
        return fail(FG_ERR_INVALID, "threads must be a multiple of 32 in 32..%d", fgd::kDipMaxThreads);
    h->threads = threads;
    return FG_OK;
}

int fg_dip_trial_du(fg_dipsys *h, int32_t i, const double *new_xyz, const double *new_mu_unit, double *du) {
    if (!h || !new_xyz || !du) return fail(FG_ERR_INVALID, "null argument");
    if (!h->state_set) return fail(FG_ERR_STATE, "fg_dip_set_state first");
    if (h->pending) return fail(FG_ERR_STATE, "a trial is pending: commit it first");
    if (h->n_stream > 0) return fail(FG_ERR_STATE, "a staged stream is waiting: run it first");
    if (i < 0 || i >= h->N) return fail(FG_ERR_INVALID, "particle out of range");
    fgd::DipTrial t{};
    t.idx = i;
    t.kind = 3;
    for (int a = 0; a < 3; a++) t.t[a] = to_fix(new_xyz[a], h->P.box[a]);
    if (new_mu_unit) {
        for (int a = 0; a < 3; a++) t.q[1 + a] = new_mu_unit[a];
    } else {
        CK(cudaMemcpyAsync(&t.q[1], h->mu + 3 * (size_t)i, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    int rc = dip_ensure_trials(h, 1, false);
    if (rc) return rc;
    CK(cudaMemcpyAsync(h->trials, &t, sizeof(t), cudaMemcpyHostToDevice, h->stream));
    rc = dip_launch(&h, h->d_desc, 1, 1, h->stream);
    if (rc) return rc;
    fgd::DipScalars s;
    rc = dip_read_scalars(h, s);
    if (rc) return rc;
    if (s.error) return fail(FG_ERR_DEVICE, "device error flags 0x%x", s.error);
    *du = s.pend_du;
    h->pending = true;
    return FG_OK;
}

int fg_dip_commit(fg_dipsys *h, int32_t accepted, double *correction) {
    if (!h) return fail(FG_ERR_INVALID, "null argument");
    if (!h->pending) return fail(FG_ERR_STATE, "no pending trial");
    h->pending = false;
    if (correction) *correction = 0.0;
    if (!accepted) return FG_OK;
    fgd::DipScalars s0, s1;
    int rc = dip_read_scalars(h, s0);
    if (!rc) rc = dip_launch(&h, h->d_desc, 1, 2, h->stream);
    if (!rc) rc = dip_read_scalars(h, s1);
    if (rc) return rc;
    // what update() returns: the reciprocal-energy change of a Q(k) rebuild
    if (correction) *correction = s1.n_rebuilds > s0.n_rebuilds ? (s1.usum - s0.usum) - s0.pend_du : 0.0;
    return FG_OK;
}

int fg_dip_stream_upload(fg_dipsys *h, int64_t n, const int32_t *kind, const int32_t *idx, const double *axis,
                         const double *angle, const double *disp, const double *u) {
    return dip_upload(h, n, kind, idx, axis, angle, disp, u, false);
}

int fg_dip_run_many(fg_dipsys *const *systems, int32_t n_systems, fg_sweep_stats *per_system, fg_sweep_stats *total) {
    return dip_run(systems, n_systems, per_system, total);
}

int fg_dip_sweep(fg_dipsys *h, int64_t n, const int32_t *kind, const int32_t *idx, const double *axis,
                 const double *angle, const double *disp, const double *u, uint8_t *acc, double *du,
                 fg_sweep_stats *stats) {
    const bool log = acc || du;
    int rc = dip_upload(h, n, kind, idx, axis, angle, disp, u, log);
    if (rc) return rc;
    fg_sweep_stats st{};
    rc = dip_run(&h, 1, nullptr, &st);
    if (stats) *stats = st;
    if (rc) return rc;
    if (log && n > 0) {
        std::vector<double> l(n);
        std::vector<uint8_t> a(n);
        CK(cudaMemcpyAsync(l.data(), h->log_du, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(a.data(), h->log_acc, n, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (du) std::copy(l.begin(), l.end(), du);
        if (acc) std::copy(a.begin(), a.end(), acc);
    }
    return FG_OK;
}

int fg_dip_total_energy(fg_dipsys *h, double *comp) {
    if (!h || !comp) return fail(FG_ERR_INVALID, "null argument");
    if (!h->state_set) return fail(FG_ERR_STATE, "no state");
    return dip_total(h, comp);
}

int fg_dip_running_energy(fg_dipsys *h, double *u) {
    if (!h || !u) return fail(FG_ERR_INVALID, "null argument");
    fgd::DipScalars s;
    int rc = dip_read_scalars(h, s);
    if (rc) return rc;
    *u = s.utot;
    return FG_OK;
}

// Draws of n AtomicRotation / AtomicTranslation trials on one atomic group of
// n_particles, as the reference takes them from slump (std::mt19937 seeded
// with seed): per trial the move (rotation when a uniform falls below
// p_rotate; with p_rotate < 0 the caller's kind[] says), then
// slump.element over the one group, the particle (Group::random,
// group.h:129-134), for a rotation a ranunit axis (point.h:74-88) and the
// angle dprot * half() (move.h:1020-1030), for a translation three
// dp * half() (move.h:830-840), and the Metropolis uniform.
int fg_dip_draw_stream(uint32_t seed, int32_t n_particles, int64_t n, double p_rotate, double dp, double dprot,
                       int32_t *kind, int32_t *idx, double *axis, double *angle, double *disp, double *u) {
    if (n_particles < 1 || n < 0 || (n > 0 && (!kind || !idx || !axis || !angle || !disp || !u)))
        return fail(FG_ERR_INVALID, "bad argument");
    std::mt19937 eng(seed);
    auto uni = [&]() {
        std::uniform_real_distribution<double> U(0, 1);
        return U(eng);
    };
    auto range = [&](int a, int b) {
        std::uniform_int_distribution<int> D(a, b);
        return D(eng);
    };
    for (int64_t t = 0; t < n; t++) {
        const bool rot = p_rotate < 0 ? kind[t] == 1 : uni() < p_rotate;
        kind[t] = rot ? 1 : 2;
        range(0, 0);
        idx[t] = range(0, n_particles - 1);
        double v[3] = {0, 0, 0}, an = 0.0, d[3] = {0, 0, 0};
        if (rot) {
            double r2;
            do {
                for (int a = 0; a < 3; a++) v[a] = 2 * uni() - 1;
                r2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
            } while (r2 > 1);
            const double s = std::sqrt(r2);
            for (int a = 0; a < 3; a++) v[a] /= s;
            an = dprot * (uni() - 0.5);
        } else {
            for (int a = 0; a < 3; a++) d[a] = dp * (uni() - 0.5);
        }
        u[t] = uni();
        for (int a = 0; a < 3; a++) {
            axis[3 * t + a] = v[a];
            disp[3 * t + a] = d[a];
        }
        angle[t] = an;
    }
    return FG_OK;
}

int64_t fg_dip_device_bytes(fg_dipsys *h) { return h ? (int64_t)h->device_bytes : 0; }

// Threads per system (32, 64, 128, 256) timed on clones of the caller's
// systems run side by side, the way fg_dip_run_many runs them: every clone
// takes the same host-drawn stream of n_trials (half rotations, half
// translations) per candidate; the fastest aggregate rate is applied to the
// caller's systems and recorded for systems created afterwards. The caller's
// chains do not advance.
int fg_dip_autotune(fg_dipsys *const *systems, int32_t n_systems, int64_t n_trials, fg_tune_report *report) {
    if (!systems || n_systems < 1) return fail(FG_ERR_INVALID, "no systems");
    if (n_trials < 32) return fail(FG_ERR_INVALID, "n_trials must be >= 32");
    if (report) *report = fg_tune_report{};
    std::vector<fg_dipsys *> c(n_systems, nullptr);
    auto drop = [&](int rc) {
        for (fg_dipsys *x : c)
            if (x) fg_dip_destroy(x);
        return rc;
    };
    for (int i = 0; i < n_systems; i++) {
        fg_dipsys *h = systems[i];
        if (!h || !h->state_set) return drop(fail(FG_ERR_STATE, "system %d has no state", i));
        std::vector<double> xyz, mu;
        int rc = dip_get_state(h, xyz, mu);
        if (!rc) rc = fg_dip_create(&h->P, h->N, &c[i]);
        if (!rc) rc = fg_dip_set_state(c[i], xyz.data(), mu.data(), h->mus_h.data(), h->charges_h.data(),
                                       h->types_h.data());
        if (rc) return drop(rc);
    }
    std::vector<std::pair<int, double>> t;
    const int cand[4] = {32, 64, 128, 256};
    for (int ci = 0; ci < 4; ci++) {
        const int T = cand[ci];
        int rc = FG_OK;
        for (int pass = 0; pass < 2 && !rc; pass++) {   // warm-up, then timed
            for (int i = 0; i < n_systems && !rc; i++) {
                const int N = c[i]->N;
                const int64_t n = pass ? n_trials : std::max<int64_t>(32, n_trials / 4);
                std::vector<int32_t> kind(n), idx(n);
                std::vector<double> axis(3 * n), angle(n), disp(3 * n), u(n);
                rc = fg_dip_draw_stream(0x7e57u + 977u * (uint32_t)i + (uint32_t)pass, N, n, 0.5, 0.5, 1.0,
                                        kind.data(), idx.data(), axis.data(), angle.data(), disp.data(), u.data());
                if (!rc) rc = fg_dip_set_threads(c[i], T);
                if (!rc) rc = fg_dip_stream_upload(c[i], n, kind.data(), idx.data(), axis.data(), angle.data(),
                                                   disp.data(), u.data());
            }
            fg_sweep_stats st{};
            if (!rc) rc = fg_dip_run_many(c.data(), n_systems, nullptr, &st);
            if (!rc && pass) {
                const double us = st.trials > 0 ? st.device_ms * 1e3 / (double)st.trials : 0.0;
                t.push_back({T, us});
                report_add(report, T, us);
            }
        }
        if (rc) return drop(rc);
    }
    const int best = report_pick(report, t);
    const int T = t[best].first;
    for (int i = 0; i < n_systems; i++) systems[i]->threads = T;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_dip_threads = T;
    }
    return drop(FG_OK);
}

}  // extern "C"
