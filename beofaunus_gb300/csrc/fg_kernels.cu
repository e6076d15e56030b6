// Energy-change kernels for atomic systems (one particle moved per trial).
//
//   sweep_kernel      persistent, one CTA per system (a batch is a grid of
//                     systems): runs the trial stream (trial -> dU ->
//                     Metropolis -> accept/reject -> update) and stops early
//                     when the Ewald update_frequency asks for a Q(k) rebuild
//   trial_kernel /    the plain drop-in path, one call per trial, mirroring
//   commit_kernel     Energy::energyChange and Movebase::update
//   qk_rebuild_*      Q(k) from scratch (updateAllComplexNumbers)
//   pair_total_kernel systemEnergy's pair sum
//   philox_stream     device-generated trial streams
//
// Reference path restated here: Movebase::move (move.h:515-555),
// AtomicTranslation::_trialMove/_acceptMove/_rejectMove (move.h:818-889),
// Energy::energyChangeConfiguration (energy.h:3521-3572), EwaldReal
// (ewald.h:97-110), WeeksChandlerAndersen (potentials.h:2186-2193),
// DebyeHuckel (potentials.h:3314-3323), LennardJonesMixed
// (potentials.h:2036-2040), NonbondedEwald::updateChange/update/external
// (ewald.h:613-729), getSurfaceEnergy (ewald.h:277-291).
//
// Q(k) bookkeeping. Each particle contributes the complex integer
// c_k(j) = (rint(w.x e.x) - rint(w.y e.y), rint(w.x e.y) + rint(w.y e.x)),
// the product w_j(nx, ny) e_z(nz) with each of its four real products rounded
// to the nearest integer, where w_j = (s q_j eff_j e_x(nx)) e_y(ny),
// s = 2^g c (c = 4095/4096), and e_a(n) = e^{i n 2 pi x_a / L_a} comes from
// sincos_turns on the exact integer phase n h_a (its conjugate for n < 0),
// every product rounded in a fixed order (qk_w, qk_term_bits): a
// deterministic function of the particle's fixed-point position. g is chosen
// so that every |w e_z| < 2^22, where one FMA with 1.5 2^23 as addend rounds
// a product to the nearest integer on the FMA pipe (qk_rint_bits). Q(k) is
// kept as the exact int64 sum of these contributions in units of 2^-28 / c
// (each shifted by 28 - g), and an accepted move adds c_k(new) - c_k(old).
// So Q(k) never drifts: a rebuild from scratch reproduces it bit for bit (the
// rebuilds check that), where the reference's FP64 running sum needs the
// rebuild to undo accumulated error. The factorised form lets a rebuild share
// one w per particle across the k-vectors with the same (nx, ny); since the
// rounding is symmetric, the four rounded products for e_z(n) also give the
// contribution to -n (e_z(-n) = conj e_z(n)), so a rebuild forms them once
// for both.
// The energy change itself uses the increment in the form
// q e^{ik.r_old}(e^{ik.d} - 1), whose FP32 error is relative to |d|.
#include <cstdint>
#include <cuda_runtime.h>

#include "fg_device.cuh"
#include "fg_system.cuh"

namespace fg {

constexpr int MODEL_EWALD = 1;
constexpr int MODEL_DHLJ = 2;
constexpr int kSweepThreads = 512;

// ------------------------------------------------------------------ df arithmetic
__device__ __forceinline__ df two_prod(float a, float b) {
    float p = a * b;
    return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ df dfm(df a, df b) {
    df p = two_prod(a.hi, b.hi);
    p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df dfm_f(df a, float b) {
    df p = two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_from_i64(int64_t v) {
    float h = __ll2float_rn(v);
    float l = __ll2float_rn(v - __float2ll_rn(h));
    return fast_two_sum(h, l);
}
__device__ __forceinline__ df df_sqrt(df a) {
    float r0 = sqrtf(a.hi);
    df p = two_prod(r0, r0);
    float diff = ((a.hi - p.hi) - p.lo) + a.lo;
    return fast_two_sum(r0, diff * (0.5f / r0));
}
__device__ __forceinline__ df df_recip(df a) {
    float i0 = 1.0f / a.hi;
    df p = two_prod(a.hi, i0);
    float e = ((1.0f - p.hi) - p.lo) - a.lo * i0;
    return fast_two_sum(i0, i0 * e);
}
__device__ __forceinline__ df df_div(df a, df b) {
    float q1 = a.hi / b.hi;
    df r = df_add(a, df_neg(dfm_f(b, q1)));
    return fast_two_sum(q1, r.hi / b.hi);
}

// ------------------------------------------------------------------ pairs (FP32)
// 1/sqrt(r2) to FP32 accuracy: hardware estimate plus one Newton step.
__device__ __forceinline__ float rsqrt_nr(float r2) {
    const float y = rsqrtf(r2);
    return y * fmaf(-0.5f * r2 * y, y, 1.5f);
}

// erfc for x >= 0: the Chebyshev fit of Press, Teukolsky, Vetterling and
// Flannery (Numerical Recipes in C, 2nd ed., section 6.2, "erfcc"),
// fractional error below 1.2e-7 everywhere.
__device__ __forceinline__ float erfc_nr(float z) {
    const float t = __frcp_rn(fmaf(0.5f, z, 1.0f));
    float p = fmaf(t, 0.17087277f, -0.82215223f);
    p = fmaf(t, p, 1.48851587f);
    p = fmaf(t, p, -1.13520398f);
    p = fmaf(t, p, 0.27886807f);
    p = fmaf(t, p, -0.18628806f);
    p = fmaf(t, p, 0.09678418f);
    p = fmaf(t, p, 0.37409196f);
    p = fmaf(t, p, 1.00002368f);
    p = fmaf(t, p, -1.26551223f);
    return t * expf(fmaf(-z, z, p));
}

// EwaldReal (kappa-screened form, ewald.h:109) + WCA; qq = qa qb QeQe lB.
// NEAR: correctly rounded sqrt/divide and erfcf for the few pairs close to
// contact, whose energies are largest; otherwise reciprocal square root and
// the Chebyshev erfc.
template <bool NEAR>
__device__ __forceinline__ float pair_ewald_wca(float r2, float qq, float s2, float wca2, float eps4,
                                                const SysDesc &d) {
    float u = 0.0f;
    const float ri = NEAR ? 1.0f / sqrtf(r2) : rsqrt_nr(r2);
    if (r2 <= d.rc2) {
        const float r = NEAR ? sqrtf(r2) : r2 * ri;
        float e;
        if (d.kappa == 0.0f) {
            e = NEAR ? erfcf(d.alpha * r) : erfc_nr(d.alpha * r);
        } else {
            const float k2a = d.kappa / (2.0f * d.alpha);
            e = 0.5f * (erfcf(d.alpha * r + k2a) * expf(d.kappa * r) + erfcf(d.alpha * r - k2a) * expf(-d.kappa * r));
        }
        u = NEAR ? qq * e / r : qq * e * ri;
    }
    if (r2 <= wca2) {
        float x = NEAR ? s2 / r2 : s2 * ri * ri;
        x = x * x * x;
        u += eps4 * (x * x - x + 0.25f);
    }
    return u;
}

// DebyeHuckel + LennardJonesMixed; qq = qa qb lB.
__device__ __forceinline__ float pair_dh_lj(float r2, float qq, float s2, float eps4, const SysDesc &d) {
    const float r = sqrtf(r2);
    const float u = qq * expf(-d.kappa * r) / r;
    float x = s2 / r2;
    x = x * x * x;
    return u + eps4 * (x * x - x);
}

template <int MODEL, bool NEAR = true>
__device__ __forceinline__ float pair_u(float r2, float qi, float qj, int t, const SysDesc &d) {
    if (MODEL == MODEL_EWALD)
        return pair_ewald_wca<NEAR>(r2, qi * qj * d.qeqe[t] * d.lB, d.s2[t], d.wca2[t], d.eps4[t], d);
    return pair_dh_lj(r2, qi * qj * d.lB, d.s2[t], d.eps4[t], d);
}

// Minimum-image squared distance from high-word fixed-point coordinates.
__device__ __forceinline__ float dist2(int4 a, int xb, int yb, int zb, const SysDesc &d) {
    float dx = (float)(a.x - xb) * d.s32[0];
    float dy = (float)(a.y - yb) * d.s32[1];
    float dz = (float)(a.z - zb) * d.s32[2];
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// ------------------------------------------------------------------ core pairs
// Pairs inside the repulsive core (r < sigma_ij) carry large, steep energies
// (WCA/LJ ~ r^-12) where FP32 rounding and 32-bit coordinates would exceed
// the 1e-6 kT budget. They are rare, so they are evaluated in df from 48-bit
// coordinate differences: the Coulomb-like part from a Taylor table of g(y)
// (erfc for Ewald, exp(-y) for Debye-Hueckel) at spacing 1/128, the
// r^-12/r^-6 part by df division and products.
__device__ __forceinline__ int16_t ext16(int64_t X) {
    int32_t h = hi32(X);
    int32_t rem = (int32_t)((uint64_t)X - ((uint64_t)(uint32_t)h << 32));
    return (int16_t)(rem >> 16);
}

template <int MODEL>
__device__ __noinline__ df pair_core_df(int dh0, int dh1, int dh2, int de0, int de1, int de2, float qi, float qj,
                                        int t, const SysDesc &d) {
    df r2 = {0.0f, 0.0f};
    const int dhs[3] = {dh0, dh1, dh2}, des[3] = {de0, de1, de2};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        int64_t v = ((int64_t)dhs[a] << 16) + (int64_t)des[a];
        df x = dfm(df_from_i64(v), df{d.s48_df[a].x, d.s48_df[a].y});
        r2 = df_add(r2, dfm(x, x));
    }
    df r = df_sqrt(r2);
    df inv = df_recip(r);
    df y = dfm(df{d.coef_df.x, d.coef_df.y}, r);
    int j = (int)(y.hi * 128.0f + 0.5f);
    j = min(max(j, 0), d.core_tab_n - 1);
    float dl = (y.hi - (float)j * (1.0f / 128.0f)) + y.lo;
    float4 c0 = d.core_tab[j];
    float4 c1 = d.core_tab2[j];
    df g = df_add(df{c0.x, c0.y}, dfm_f(df{c0.z, c0.w}, dl));
    g = df_add_f(g, dl * dl * fmaf(dl, fmaf(dl, c1.z, c1.y), c1.x));
    df u = dfm(dfm(dfm(df{d.pref_df[t].x, d.pref_df[t].y}, two_prod(qi, qj)), g), inv);
    df x = df_div(df{d.s2_df[t].x, d.s2_df[t].y}, r2);
    df x3 = dfm(dfm(x, x), x);
    df w = df_add(dfm(x3, x3), df_neg(x3));
    if (MODEL == MODEL_EWALD) w = df_add_f(w, 0.25f);
    return df_add(u, dfm(w, df{d.eps4_df[t].x, d.eps4_df[t].y}));
}

// ------------------------------------------------------------------ move
struct Move {
    int i, ti;        // particle and its type
    float q;          // its charge
    int64_t xo[3];    // old fixed-point coordinates
    int64_t xn[3];    // new
    int ho[3], hn[3]; // high words
    int eo[3], en[3]; // 16-bit extensions
    float dxf[3];     // displacement (Angstrom, minimum image)
    int co, cn;       // old / new cell
};

__device__ __forceinline__ int cell_of(const int h[3], const SysDesc &d) {
    int c[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        uint32_t u = (uint32_t)h[a] + 0x80000000u;
        c[a] = (int)(((uint64_t)u * (uint32_t)d.nc[a]) >> 32);
    }
    return (c[2] * d.nc[1] + c[1]) * d.nc[0] + c[0];
}

__device__ __forceinline__ void move_setup(Move &m, int i, const int64_t xo[3], const int64_t xn[3], float q,
                                           int ti, const SysDesc &d) {
    m.i = i;
    m.ti = ti;
    m.q = q;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        m.xo[a] = xo[a];
        m.xn[a] = xn[a];
        m.ho[a] = hi32(xo[a]);
        m.hn[a] = hi32(xn[a]);
        m.eo[a] = ext16(xo[a]);
        m.en[a] = ext16(xn[a]);
        int64_t dd = (int64_t)((uint64_t)xn[a] - (uint64_t)xo[a]);
        m.dxf[a] = i64_to_float(dd) * d.dl32[a];
    }
    if (d.use_cells) {
        m.co = cell_of(m.ho, d);
        m.cn = cell_of(m.hn, d);
    }
}

// One candidate j against the moved particle: adds u(new) - u(old) to the
// float accumulator, or to the df accumulator for core pairs.
template <int MODEL>
__device__ __forceinline__ void pair_candidate(const Move &m, int4 pj, int tj, const short4 *ext, const SysDesc &d,
                                               float &accf, df &accd) {
    const float qj = __int_as_float(pj.w);
    const float r2n = dist2(pj, m.hn[0], m.hn[1], m.hn[2], d);
    const float r2o = dist2(pj, m.ho[0], m.ho[1], m.ho[2], d);
    const int t = d.uniform_types ? 0 : m.ti * d.n_types + tj;
    const float s2 = d.core_tab_n > 0 ? d.s2[t] : 0.0f;   // no core table: FP32 throughout
    const bool cn = r2n < s2, co = r2o < s2;
    // near: within 2 sigma (DH) or 1.5 sigma (Ewald) of either position
    const float near2 = d.s2[t] * (MODEL == MODEL_DHLJ ? 4.0f : 2.25f);
    const bool near = r2n < near2 || r2o < near2;
    if (MODEL == MODEL_DHLJ && !cn && !co && near) {
        // accurate difference form: u_o expm1(-kappa dr - log1p(dr / r_o))
        long long S = 0;
        const int pjv[3] = {pj.x, pj.y, pj.z};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            long long dn = (int)(pjv[a] - m.hn[a]), dO = (int)(pjv[a] - m.ho[a]);
            S += (dn - dO) * (dn + dO);
        }
        const float dR2 = i64_to_float(S) * d.s32sq;
        const float ro = sqrtf(r2o), rn = sqrtf(r2n);
        const float dr = dR2 / (rn + ro);
        const float z = fmaf(-d.kappa, dr, -log1pf(dr / ro));
        const float uo = m.q * qj * d.lB * expf(-d.kappa * ro) / ro;
        const float xo = d.s2[t] / r2o;
        const float xo3 = xo * xo * xo;
        const float tau = -dR2 / r2n;
        const float t3m1 = tau * fmaf(tau, tau + 3.0f, 3.0f);
        accf += fmaf(uo, expm1f(z), d.eps4[t] * xo3 * t3m1 * fmaf(xo3, t3m1 + 2.0f, -1.0f));
        return;
    }
    if (MODEL == MODEL_DHLJ && !cn && !co) {
        // Difference form, so the rounding error scales with |u(new) - u(old)|
        // and not with |u| (no cutoff: every pair contributes). With
        // r_n^2 - r_o^2 = sum_a (dn_a - do_a)(dn_a + do_a) exact in integers
        // (minimum images taken separately, as the reference's sqdist does):
        //   LJ: 4eps x_o^3 (t^3 - 1)(x_o^3 (t^3 + 1) - 1), t = r_o^2 / r_n^2
        long long S = 0;
        const int pjv[3] = {pj.x, pj.y, pj.z};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            long long dn = (int)(pjv[a] - m.hn[a]), dO = (int)(pjv[a] - m.ho[a]);
            S += (dn - dO) * (dn + dO);
        }
        // DH: u_n/u_o - 1 = (expm1(-kappa dr) - t)/(1 + t), t = dr/r_o, with
        // expm1 by its Taylor series (|kappa dr| is small) or expm1f.
        const float dR2 = i64_to_float(S) * d.s32sq;
        const float rio = rsqrt_nr(r2o), rin = rsqrt_nr(r2n);
        const float ro = r2o * rio, rn = r2n * rin;
        const float dr = dR2 * __frcp_rn(rn + ro);
        const float tt = dr * rio;
        const float y = -d.kappa * dr;
        float em1;
        if (fabsf(y) < 0.25f) {
            em1 = fmaf(y, 1.0f / 5040.0f, 1.0f / 720.0f);
            em1 = fmaf(y, em1, 1.0f / 120.0f);
            em1 = fmaf(y, em1, 1.0f / 24.0f);
            em1 = fmaf(y, em1, 1.0f / 6.0f);
            em1 = fmaf(y, em1, 0.5f);
            em1 = fmaf(y * y, em1, y);
        } else {
            em1 = expm1f(y);
        }
        const float uo = m.q * qj * d.lB * expf(-d.kappa * ro) * rio;
        const float ddh = uo * (em1 - tt) * __frcp_rn(1.0f + tt);
        const float xo = d.s2[t] * rio * rio;
        const float xo3 = xo * xo * xo;
        const float tau = -dR2 * (rin * rin);
        const float t3m1 = tau * fmaf(tau, tau + 3.0f, 3.0f);
        accf += fmaf(d.eps4[t] * xo3, t3m1 * fmaf(xo3, t3m1 + 2.0f, -1.0f), ddh);
        return;
    }
    float un, uo;
    if (near) {
        un = cn ? 0.0f : pair_u<MODEL, true>(r2n, m.q, qj, t, d);
        uo = co ? 0.0f : pair_u<MODEL, true>(r2o, m.q, qj, t, d);
    } else {
        un = pair_u<MODEL, false>(r2n, m.q, qj, t, d);
        uo = pair_u<MODEL, false>(r2o, m.q, qj, t, d);
    }
    accf += un - uo;
    if (cn || co) {
        const short4 e = *ext;
        if (cn)
            accd = df_add(accd, pair_core_df<MODEL>(pj.x - m.hn[0], pj.y - m.hn[1], pj.z - m.hn[2], e.x - m.en[0],
                                                    e.y - m.en[1], e.z - m.en[2], m.q, qj, t, d));
        if (co)
            accd = df_add(accd, df_neg(pair_core_df<MODEL>(pj.x - m.ho[0], pj.y - m.ho[1], pj.z - m.ho[2],
                                                           e.x - m.eo[0], e.y - m.eo[1], e.z - m.eo[2], m.q, qj,
                                                           t, d)));
    }
}

// ------------------------------------------------------------------ shared memory
struct Smem {
    float2 *sc_tab;     // 256 cos/sin entries
    float2 *red;        // 32 warp partials (df)
    float4 *kvec;       // K: kx, ky, kz, A'
    uint32_t *kpack;    // K: n vector
    longlong2 *qfix;    // K: Q(k), exact fixed point
    float2 *qf;         // K: Q(k) rounded to float (energy)
    float2 *ktab;       // axis tables (qk_tab_len) of a committed move: new, then old position
    int4 *pos;          // N (positions in shared memory)
    short4 *pos_ext;    // N
    uint8_t *ptype;     // N
    int *ccount;        // cells: particles per cell
    uint32_t *pcs;      // cells: particle -> cell << 12 | slot
};

__host__ __device__ __forceinline__ size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

// Byte layout of the dynamic shared memory; the host sizes launches with it.
// Entries of the per-position axis tables: e_x(0..kcc), e_y(-kcc..kcc), e_z(-kcc..kcc).
__host__ __device__ __forceinline__ int qk_tab_len(int kcc) { return 5 * kcc + 3; }

__host__ __device__ __forceinline__ size_t smem_layout(int N, int K, int kcc, int ncell, bool kspace, bool pos_smem,
                                                       bool cells, size_t off[8]) {
    size_t b = 256 * 8 + 32 * 8;
    off[0] = b;                                   // kvec
    if (kspace) b += (size_t)K * 16;
    off[1] = b;                                   // qfix
    if (kspace) b += (size_t)K * 16;
    off[2] = b;                                   // qf, ktab
    if (kspace) b = align16(b + (size_t)K * 8 + (size_t)2 * qk_tab_len(kcc) * 8);
    off[3] = b;                                   // kpack
    if (kspace) b = align16(b + (size_t)K * 4);
    off[4] = b;                                   // pos, pos_ext, ptype
    if (pos_smem) b = align16(b + (size_t)N * 25);
    off[5] = b;                                   // ccount
    if (cells) b = align16(b + (size_t)ncell * 4);
    off[6] = b;                                   // pcs
    if (cells) b = align16(b + (size_t)N * 4);
    off[7] = b;
    return b;
}

__device__ __forceinline__ Smem carve(char *base, const SysDesc &d, bool kspace, bool pos_smem, bool cells) {
    size_t off[8];
    smem_layout(d.N, d.K, d.kcc, d.nc[0] * d.nc[1] * d.nc[2], kspace, pos_smem, cells, off);
    Smem s;
    s.sc_tab = (float2 *)base;
    s.red = (float2 *)(base + 256 * 8);
    s.kvec = (float4 *)(base + off[0]);
    s.qfix = (longlong2 *)(base + off[1]);
    s.qf = (float2 *)(base + off[2]);
    s.ktab = (float2 *)(base + off[2] + (size_t)d.K * 8);
    s.kpack = (uint32_t *)(base + off[3]);
    s.pos = (int4 *)(base + off[4]);
    s.pos_ext = (short4 *)(base + off[4] + (size_t)d.N * 16);
    s.ptype = (uint8_t *)(base + off[4] + (size_t)d.N * 24);
    s.ccount = (int *)(base + off[5]);
    s.pcs = (uint32_t *)(base + off[6]);
    return s;
}

// Copy a system descriptor into shared memory (all threads participate).
__device__ __forceinline__ void load_desc(SysDesc &dst, const SysDesc *__restrict__ src) {
    const int4 *s4 = reinterpret_cast<const int4 *>(src);
    int4 *d4 = reinterpret_cast<int4 *>(&dst);
    for (int t = threadIdx.x; t < (int)(sizeof(SysDesc) / 16); t += blockDim.x) d4[t] = s4[t];
    __syncthreads();
}

// Q(k) fixed point (units of 2^-28 / c, c = 4095/4096) to float, by 32-bit
// halves.
constexpr float kQkInvC = 4096.0f / 4095.0f;
__device__ __forceinline__ float fix28_to_float(long long v) {
    const int hi = (int)(v >> 32);
    const unsigned lo = (unsigned)v;
    return fmaf((float)hi, 16.0f * kQkInvC, (float)lo * (3.7252902984619141e-09f * kQkInvC));
}
__device__ __forceinline__ float2 q_to_float(longlong2 q) { return make_float2(fix28_to_float(q.x), fix28_to_float(q.y)); }

__device__ __forceinline__ void load_smem(const SysDesc &d, const Smem &s, bool kspace, bool pos_smem, bool cells,
                                          const float2 *sc_tab) {
    for (int t = threadIdx.x; t < 256; t += blockDim.x) s.sc_tab[t] = sc_tab[t];
    if (kspace)
        for (int k = threadIdx.x; k < d.K; k += blockDim.x) {
            s.kvec[k] = d.kvec[k];
            s.kpack[k] = d.kpack[k];
            longlong2 q = d.qfix[k];
            s.qfix[k] = q;
            s.qf[k] = q_to_float(q);
        }
    if (pos_smem)
        for (int j = threadIdx.x; j < d.N; j += blockDim.x) {
            s.pos[j] = d.pos4[j];
            s.pos_ext[j] = d.pos_ext[j];
            s.ptype[j] = d.ptype[j];
        }
    if (cells) {
        const int ncell = d.nc[0] * d.nc[1] * d.nc[2];
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) s.ccount[c] = d.cell_count[c];
        for (int j = threadIdx.x; j < d.N; j += blockDim.x)
            s.pcs[j] = ((uint32_t)d.p_cell[j] << 12) | (uint32_t)d.p_slot[j];
    }
    __syncthreads();
}

// ------------------------------------------------------------------ pair loops
template <int MODEL>
__device__ __forceinline__ void pairs_cells_warp(const Move &m, const SysDesc &d, const Smem &s, float &accf,
                                                 df &accd) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    int co[3], cn[3], lo[3], len[3];
    co[0] = m.co % d.nc[0]; co[1] = (m.co / d.nc[0]) % d.nc[1]; co[2] = m.co / (d.nc[0] * d.nc[1]);
    cn[0] = m.cn % d.nc[0]; cn[1] = (m.cn / d.nc[0]) % d.nc[1]; cn[2] = m.cn / (d.nc[0] * d.nc[1]);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        int delta = cn[a] - co[a];
        if (delta > 1) delta -= d.nc[a];
        if (delta < -1) delta += d.nc[a];
        if ((delta > 1 || delta < -1) && threadIdx.x == 0) d.sc->error |= kErrStencil;
        lo[a] = co[a] + min(delta, 0) - 1;
        len[a] = 3 + (delta != 0 ? 1 : 0);
    }
    const int ncell = len[0] * len[1] * len[2];
    for (int k = warp; k < ncell; k += nwarp) {
        const int ix = k % len[0], iy = (k / len[0]) % len[1], iz = k / (len[0] * len[1]);
        int cx = lo[0] + ix, cy = lo[1] + iy, cz = lo[2] + iz;
        cx += (cx < 0) ? d.nc[0] : 0; cx -= (cx >= d.nc[0]) ? d.nc[0] : 0;
        cy += (cy < 0) ? d.nc[1] : 0; cy -= (cy >= d.nc[1]) ? d.nc[1] : 0;
        cz += (cz < 0) ? d.nc[2] : 0; cz -= (cz >= d.nc[2]) ? d.nc[2] : 0;
        const int cid = (cz * d.nc[1] + cy) * d.nc[0] + cx;
        const int cnt = s.ccount[cid];
        for (int slot = lane; slot < cnt; slot += 32) {
            const int idx = cid * d.cap + slot;
            const int pid = d.cell_pid[idx];
            if ((pid & 0xFFFFFF) == m.i) continue;
            pair_candidate<MODEL>(m, d.cell_pos[idx], pid >> 24, &d.cell_ext[idx], d, accf, accd);
        }
    }
}

template <int MODEL, bool POS_SMEM>
__device__ __forceinline__ void pairs_all_strided(const Move &m, const SysDesc &d, const Smem &s, float &accf,
                                                  df &accd) {
    for (int j = threadIdx.x; j < d.N; j += blockDim.x) {
        if (j == m.i) continue;
        const int4 pj = POS_SMEM ? s.pos[j] : d.pos4[j];
        const int tj = POS_SMEM ? s.ptype[j] : d.ptype[j];
        pair_candidate<MODEL>(m, pj, tj, POS_SMEM ? &s.pos_ext[j] : &d.pos_ext[j], d, accf, accd);
    }
}

// ------------------------------------------------------------------ k-space
__device__ __forceinline__ void unpack_n(uint32_t p, int &nx, int &ny, int &nz) {
    nx = (int)(int8_t)(p & 0xFF);
    ny = (int)(int8_t)((p >> 8) & 0xFF);
    nz = (int)(int8_t)(p >> 16);
}
__device__ __forceinline__ uint32_t phase(int nx, int ny, int nz, const int h[3]) {
    return (uint32_t)nx * (uint32_t)h[0] + (uint32_t)ny * (uint32_t)h[1] + (uint32_t)nz * (uint32_t)h[2];
}

// isotropic_pbc (ewald.h:669-675): D_k = q (c'_x c'_y c'_z - c_x c_y c_z),
// c_a = cos(n_a 2 pi x_a / L_a), each axis difference taken as
// cos a' - cos a = -2 sin((a' + a) / 2) sin((a' - a) / 2) so that a short
// step keeps its relative accuracy.
__device__ __forceinline__ float iso_delta(int nx, int ny, int nz, const Move &m, const float2 *__restrict__ tab) {
    const int nn[3] = {nx, ny, nz};
    float co[3], cn[3], dc[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const uint32_t po = (uint32_t)nn[a] * (uint32_t)m.ho[a], pn = (uint32_t)nn[a] * (uint32_t)m.hn[a];
        const int32_t dp = (int32_t)(pn - po);
        co[a] = sincos_turns(po, tab).x;
        cn[a] = sincos_turns(pn, tab).x;
        const float sm = sincos_turns(po + (uint32_t)(dp >> 1), tab).y;
        const float sh = sinf((float)dp * (3.14159265f / 4294967296.0f));   // pi / 2^32 per unit
        dc[a] = -2.0f * sm * sh;
    }
    return fmaf(dc[0], cn[1] * cn[2], co[0] * fmaf(dc[1], cn[2], co[1] * dc[2]));
}

// Reciprocal-space energy change of the trial for this thread's k-vectors:
// A'_k (2 Re(conj(Q_k) D_k) + |D_k|^2), D_k = q e^{ik.r_old}(e^{ik.d} - 1)
// (isotropic_pbc: Q and D real, iso_delta).
__device__ __forceinline__ float kspace_energy(const Move &m, const SysDesc &d, const Smem &s) {
    float acc = 0.0f;
    const float qe = m.q * d.eff[m.ti];
    for (int k = threadIdx.x; k < d.K; k += blockDim.x) {
        int nx, ny, nz;
        unpack_n(s.kpack[k], nx, ny, nz);
        if (d.iso) {
            const float D = qe * iso_delta(nx, ny, nz, m, s.sc_tab);
            acc = fmaf(s.kvec[k].w, fmaf(2.0f, s.qf[k].x * D, D * D), acc);
            continue;
        }
        const uint32_t ph = phase(nx, ny, nz, m.ho);
        const float2 e = sincos_turns(ph, s.sc_tab);
        const float4 kv = s.kvec[k];
        const float phi = fmaf(kv.x, m.dxf[0], fmaf(kv.y, m.dxf[1], kv.z * m.dxf[2]));
        float2 w;
        if (fabsf(phi) <= 1.6f) {
            w = expm1_i_horner(phi);
        } else {
            const float2 en = sincos_turns(phase(nx, ny, nz, m.hn) - ph, s.sc_tab);
            w = make_float2(en.x - 1.0f, en.y);
        }
        float2 dd = cmul(e, w);
        dd.x *= qe;
        dd.y *= qe;
        const float2 q = s.qf[k];
        acc = fmaf(kv.w, fmaf(2.0f, fmaf(q.x, dd.x, q.y * dd.y), fmaf(dd.x, dd.x, dd.y * dd.y)), acc);
    }
    return acc;
}

// cos/sin of a turn fraction as sincos_turns, with every operation an
// explicit round-to-nearest intrinsic so that no call site can contract or
// reorder it: Q(k) contributions must come out bit-identical in the
// rebuild, the sweeps and the plain commit.
__device__ __forceinline__ float2 sincos_turns_rn(uint32_t ph, const float2 *__restrict__ tab) {
    const uint32_t i = (ph + (1u << 23)) >> 24;
    const int32_t h = (int32_t)(ph << 8) >> 9;
    const float d = __fmaf_rn(__int_as_float(0x4B400000 + h), 2.0f * kRadPerTurnUnit,
                              -12582912.0f * (2.0f * kRadPerTurnUnit));
    const float d2 = __fmul_rn(d, d);
    const float sn = __fmaf_rn(__fmul_rn(d2, -1.0f / 6.0f), d, d);
    const float cs = __fmaf_rn(d2, __fmaf_rn(d2, 1.0f / 24.0f, -0.5f), 1.0f);
    const float2 t = tab[i & 255u];
    return make_float2(__fmaf_rn(t.x, cs, -__fmul_rn(t.y, sn)), __fmaf_rn(t.x, sn, __fmul_rn(t.y, cs)));
}

// Entry t of the axis tables of fixed-point position h (high words):
// [0, kcc] e_x(n), [kcc+1, 3kcc+1] e_y(n - kcc), [3kcc+2, 5kcc+2] e_z(n - kcc).
// iso (isotropic_pbc): the cosine alone, (cos, 0); the integer terms built on
// it (qk_w, qk_term_bits) are then those of q cos cos cos with a zero
// imaginary part, by the same roundings.
__device__ __forceinline__ float2 qk_tab_entry(int t, int kcc, const int h[3], const float2 *__restrict__ tab,
                                               bool iso = false) {
    int axis = 0, n = t;
    if (t > 3 * kcc + 1) {
        axis = 2;
        n = t - (4 * kcc + 2);
    } else if (t > kcc) {
        axis = 1;
        n = t - (2 * kcc + 1);
    }
    const int an = n < 0 ? -n : n;
    const int ha = axis == 0 ? h[0] : (axis == 1 ? h[1] : h[2]);   // no dynamic register indexing
    const float2 e = sincos_turns_rn((uint32_t)an * (uint32_t)ha, tab);
    if (iso) return make_float2(e.x, 0.0f);
    return n < 0 ? make_float2(e.x, -e.y) : e;
}

// w = (s q eff e_x) e_y, then the integer term round(w e_z), as one
// fixed sequence of roundings.
__device__ __forceinline__ float2 qk_w(float q2g, float2 ex, float2 ey) {
    const float ax = __fmul_rn(q2g, ex.x), ay = __fmul_rn(q2g, ex.y);
    return make_float2(__fmaf_rn(ax, ey.x, -__fmul_rn(ay, ey.y)), __fmaf_rn(ax, ey.y, __fmul_rn(ay, ey.x)));
}
// For |x| < 2^22, x + 1.5 2^23 lies in [2^23, 2^24), where floats are the
// integers: fma(a, b, 1.5 2^23) is 1.5 2^23 + rint(a b) (to nearest, ties to
// even, as __float2int_rn rounds), and its bit pattern is that of 1.5 2^23
// plus rint(a b). One FMA instead of a multiply and a conversion on the XU
// pipe. Ties to even is symmetric, rint(-x) = -rint(x), which makes the
// contribution of e_z(-n) = conj e_z(n) the same four rounded products.
constexpr float kQkMagic = 12582912.0f;
constexpr uint32_t kQkMagicBits = 0x4B400000u;
__device__ __forceinline__ uint32_t qk_rint_bits(float a, float b) { return __float_as_uint(__fmaf_rn(a, b, kQkMagic)); }
// (real, imaginary) contribution of w e_z, each plus kQkMagicBits: sums of n
// of them minus n kQkMagicBits are sums of contributions, exactly in 32-bit
// wrap-around
__device__ __forceinline__ uint2 qk_term_bits(float2 w, float2 ez) {
    const uint32_t a = qk_rint_bits(w.x, ez.x), r = qk_rint_bits(w.y, ez.y);
    const uint32_t b = qk_rint_bits(w.x, ez.y), c = qk_rint_bits(w.y, ez.x);
    return make_uint2(a - r + kQkMagicBits, b + c - kQkMagicBits);
}
__device__ __forceinline__ int2 qk_term(float2 w, float2 ez) {
    const uint2 b = qk_term_bits(w, ez);
    return make_int2((int)(b.x - kQkMagicBits), (int)(b.y - kQkMagicBits));
}
// an integer contribution in units of 2^-28 / c
__device__ __forceinline__ long long qk_widen(int c, int shift) { return (long long)c * (1LL << shift); }
// s q eff of a particle (s = 2^g c: products exact in the exponent and c's
// 12-bit mantissa, then one rounding)
__device__ __forceinline__ float qk_charge(float q, float eff, const SysDesc &d) {
    return __fmul_rn(__fmul_rn(q, eff), d.qk_scale);
}
// c_k(new) - c_k(old) for k-vector n from the two positions' axis tables
// (the two terms' offsets cancel in the difference of their bit patterns)
__device__ __forceinline__ int2 qk_delta(int nx, int ny, int nz, float q2g, const float2 *__restrict__ tn,
                                        const float2 *__restrict__ to, int kcc) {
    const int iy = 2 * kcc + 1 + ny, iz = 4 * kcc + 2 + nz;
    const uint2 cn = qk_term_bits(qk_w(q2g, tn[nx], tn[iy]), tn[iz]);
    const uint2 co = qk_term_bits(qk_w(q2g, to[nx], to[iy]), to[iz]);
    return make_int2((int)(cn.x - co.x), (int)(cn.y - co.y));
}
// Axis tables of a move's new and old positions into tn and to (all threads
// of the block; the caller synchronises before use).
__device__ __forceinline__ void qk_move_tables(const int hn[3], const int ho[3], int kcc, float2 *tn, float2 *to,
                                               const float2 *__restrict__ tab, bool iso) {
    const int T = qk_tab_len(kcc);
    for (int t = threadIdx.x; t < 2 * T; t += blockDim.x) {
        if (t < T) tn[t] = qk_tab_entry(t, kcc, hn, tab, iso);
        else to[t - T] = qk_tab_entry(t - T, kcc, ho, tab, iso);
    }
}

// Accepted move: Q(k) += c_k(new) - c_k(old) for this thread's k-vectors.
// Block-wide (uniform call): the axis tables go through shared memory.
__device__ __forceinline__ void kspace_commit(const Move &m, const SysDesc &d, const Smem &s) {
    const int T = qk_tab_len(d.kcc);
    qk_move_tables(m.hn, m.ho, d.kcc, s.ktab, s.ktab + T, s.sc_tab, d.iso != 0);
    __syncthreads();
    const float q2g = qk_charge(m.q, d.eff[m.ti], d);
    for (int k = threadIdx.x; k < d.K; k += blockDim.x) {
        int nx, ny, nz;
        unpack_n(s.kpack[k], nx, ny, nz);
        const int2 c = qk_delta(nx, ny, nz, q2g, s.ktab, s.ktab + T, d.kcc);
        longlong2 q = s.qfix[k];
        q.x += qk_widen(c.x, d.qk_shift);
        q.y += qk_widen(c.y, d.qk_shift);
        s.qfix[k] = q;
        s.qf[k] = q_to_float(q);
    }
}

// Surface term change (getSurfaceEnergy, ewald.h:277-291) from a thread's
// copy of M = sum q eff r over wrapped positions: dE = c (2 M.dM + |dM|^2).
__device__ __forceinline__ df surface_delta(const Move &m, const SysDesc &d, const df M[3], float dM[3]) {
    const float qe = m.q * d.eff[m.ti];
    df acc = {0.0f, 0.0f};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float rn = (float)m.hn[a] * d.s32[a];
        const float ro = (float)m.ho[a] * d.s32[a];
        dM[a] = qe * (rn - ro);
        if (d.surf_c != 0.0f) acc = df_add_f(acc, d.surf_c * fmaf(2.0f * (M[a].hi + M[a].lo), dM[a], dM[a] * dM[a]));
    }
    return acc;
}

// Accept: master and pair coordinates; for cell systems the membership kept
// in shared memory (counts, particle -> cell/slot) and the slot arrays.
__device__ __forceinline__ void commit_position(const Move &m, const SysDesc &d, const Smem &s, bool pos_smem,
                                                bool cells) {
    const int4 rec = make_int4(m.hn[0], m.hn[1], m.hn[2], __float_as_int(m.q));
    const short4 ext = make_short4((short)m.en[0], (short)m.en[1], (short)m.en[2], 0);
    d.pos64[3 * m.i + 0] = m.xn[0];
    d.pos64[3 * m.i + 1] = m.xn[1];
    d.pos64[3 * m.i + 2] = m.xn[2];
    d.pos4[m.i] = rec;
    d.pos_ext[m.i] = ext;
    if (pos_smem) {
        s.pos[m.i] = rec;
        s.pos_ext[m.i] = ext;
    }
    if (cells) {
        const int slot = (int)(s.pcs[m.i] & 0xFFFu);
        if (m.cn == m.co) {
            d.cell_pos[m.co * d.cap + slot] = rec;
            d.cell_ext[m.co * d.cap + slot] = ext;
        } else {
            const int last = s.ccount[m.co] - 1;
            if (last != slot) {
                const int src = m.co * d.cap + last, dst = m.co * d.cap + slot;
                const int pid = d.cell_pid[src];
                d.cell_pos[dst] = d.cell_pos[src];
                d.cell_ext[dst] = d.cell_ext[src];
                d.cell_pid[dst] = pid;
                s.pcs[pid & 0xFFFFFF] = ((uint32_t)m.co << 12) | (uint32_t)slot;
            }
            s.ccount[m.co] = last;
            int ns = s.ccount[m.cn];
            if (ns >= d.cap) {
                d.sc->error |= kErrCellOverflow;
                ns = d.cap - 1;
            } else {
                s.ccount[m.cn] = ns + 1;
            }
            d.cell_pos[m.cn * d.cap + ns] = rec;
            d.cell_ext[m.cn * d.cap + ns] = ext;
            d.cell_pid[m.cn * d.cap + ns] = m.i | (m.ti << 24);
            s.pcs[m.i] = ((uint32_t)m.cn << 12) | (uint32_t)ns;
        }
    }
}

__device__ __forceinline__ void store_back(const SysDesc &d, const Smem &s, bool kspace, bool cells) {
    if (kspace)
        for (int k = threadIdx.x; k < d.K; k += blockDim.x) d.qfix[k] = s.qfix[k];
    if (cells) {
        const int ncell = d.nc[0] * d.nc[1] * d.nc[2];
        for (int c = threadIdx.x; c < ncell; c += blockDim.x) d.cell_count[c] = s.ccount[c];
        for (int j = threadIdx.x; j < d.N; j += blockDim.x) {
            d.p_cell[j] = (int)(s.pcs[j] >> 12);
            d.p_slot[j] = (int)(s.pcs[j] & 0xFFFu);
        }
    }
}

// ------------------------------------------------------------------ sweep
// Persistent sweep. Per trial t, with no single-thread section on the
// critical path:
//   k-space(t)  each thread owns fixed k-vectors and their Q(k), so the
//               commit of t-1 needs no barrier there
//   barrier B   the coordinate/cell commit of t-1 (warp 0, lane 0) is visible
//   prefetch    the particle of t+1 and the trial record of t+2
//   pairs(t)    cell list: one warp per stencil cell; else strided over j
//   barrier A   per-warp partial sums published
//   decide      every warp reduces the partials itself (same order, same
//               bits) and applies the Metropolis test: no broadcast
//   commit      Q(k) by their owner threads; coordinates/cells by warp 0,
//               lane 0, overlapping the next trial's k-space work
// Stops after an accepted trial that makes a Q(k) rebuild due
// (NonbondedEwald::update, ewald.h:633: ++cnt_accepted > update_frequency-1)
// unless the system skips rebuilds (they reproduce Q(k) exactly).
template <int MODEL, bool CELLS, bool POS_SMEM>
__global__ void __launch_bounds__(kSweepThreads, 1) sweep_kernel(const SysDesc *__restrict__ descs, int64_t end,
                                                                 const float2 *__restrict__ sc_tab) {
    extern __shared__ __align__(16) char smem_raw[];
    __shared__ __align__(16) SysDesc sd;
    load_desc(sd, descs + blockIdx.x);
    const SysDesc &d = sd;
    constexpr bool KSPACE = (MODEL == MODEL_EWALD);
    const Smem s = carve(smem_raw, d, KSPACE, POS_SMEM, CELLS);
    SysScalars *sc = d.sc;
    if (sc->rebuild_pending || sc->cursor >= min(end, sc->n_trials)) return;
    load_smem(d, s, KSPACE, POS_SMEM, CELLS, sc_tab);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    int64_t cur = sc->cursor;
    const int64_t stop = min(end, sc->n_trials);
    df U = {sc->u_hi, sc->u_lo};
    df Ut = {sc->utot_hi, sc->utot_lo};
    df M[3];
#pragma unroll
    for (int a = 0; a < 3; a++) M[a] = {sc->m[a][0], sc->m[a][1]};
    int cnt_acc = sc->cnt_accepted;
    int64_t nacc = sc->n_accepted;
    const int uf = d.update_frequency;
    bool rebuild = false;
    Trial tr = d.trials[cur];
    Trial trn = (cur + 1 < stop) ? d.trials[cur + 1] : tr;
    int64_t xo[3];
#pragma unroll
    for (int a = 0; a < 3; a++) xo[a] = d.pos64[3 * tr.idx + a];
    float qi = __int_as_float(d.pos4[tr.idx].w);
    int ti = d.ptype[tr.idx];
    while (true) {
        Move m;
        {
            int64_t xn[3];
#pragma unroll
            for (int a = 0; a < 3; a++) xn[a] = (int64_t)((uint64_t)xo[a] + (uint64_t)tr.d[a]);
            move_setup(m, tr.idx, xo, xn, qi, ti, d);
        }
        float accf = 0.0f;
        df accd = {0.0f, 0.0f};
        if (KSPACE) accf = kspace_energy(m, d, s);
        __syncthreads();   // B
        const bool has_next = cur + 1 < stop;
        int64_t xo_next[3] = {0, 0, 0};
        float q_next = 0.0f;
        int t_next = 0;
        if (has_next) {
#pragma unroll
            for (int a = 0; a < 3; a++) xo_next[a] = d.pos64[3 * trn.idx + a];
            q_next = __int_as_float(d.pos4[trn.idx].w);
            t_next = d.ptype[trn.idx];
        }
        const Trial trnn = (cur + 2 < stop) ? d.trials[cur + 2] : trn;
        if (CELLS) pairs_cells_warp<MODEL>(m, d, s, accf, accd);
        else pairs_all_strided<MODEL, POS_SMEM>(m, d, s, accf, accd);
        const df part = warp_sum_df(df_add_f(accd, accf));
        if (lane == 0) s.red[warp] = make_float2(part.hi, part.lo);
        __syncthreads();   // A
        df du = {0.0f, 0.0f};
        if (lane < nwarp) du = {s.red[lane].x, s.red[lane].y};
        du = warp_sum_df(du);
        float dM[3] = {0.0f, 0.0f, 0.0f};
        if (KSPACE) du = df_add(du, surface_delta(m, d, M, dM));
        df thr = {tr.thr_hi, tr.thr_lo};
        if (d.kT != 1.0f) thr = dfm_f(thr, d.kT);
        const bool nan = !(du.hi == du.hi);
        // Movebase::metropolis (move.h:567-573): reject iff u > exp(-dU/kT),
        // i.e. dU > kT (-ln u); a NaN dU compares false there: accepted.
        const bool accept = nan || !df_gt(du, thr);
        if (warp == 0 && lane == 0) {
            if (nan) sc->error |= kErrNonFinite;
            if (d.log_trials) {
                d.trial_du[cur] = make_float2(du.hi, du.lo);
                d.trial_acc[cur] = accept ? 1 : 0;
            }
            if (accept) commit_position(m, d, s, POS_SMEM, CELLS);
        }
        if (accept) {
            U = df_add(U, du);
            Ut = df_add(Ut, du);
            nacc++;
            if (KSPACE) {
#pragma unroll
                for (int a = 0; a < 3; a++) M[a] = df_add_f(M[a], dM[a]);
                kspace_commit(m, d, s);
                if (++cnt_acc > uf - 1) {
                    cnt_acc = 0;
                    rebuild = !d.skip_rebuild;
                }
            }
        }
        cur++;
        if (rebuild || cur >= stop) break;
        const bool same = accept && trn.idx == m.i;
#pragma unroll
        for (int a = 0; a < 3; a++) xo[a] = same ? m.xn[a] : xo_next[a];
        qi = q_next;
        ti = t_next;
        tr = trn;
        trn = trnn;
    }
    __syncthreads();
    store_back(d, s, KSPACE, CELLS);
    if (threadIdx.x == 0) {
        sc->cursor = cur;
        sc->u_hi = U.hi;
        sc->u_lo = U.lo;
        sc->utot_hi = Ut.hi;
        sc->utot_lo = Ut.lo;
        sc->n_accepted = nacc;
        for (int a = 0; a < 3; a++) {
            sc->m[a][0] = M[a].hi;
            sc->m[a][1] = M[a].lo;
        }
        sc->cnt_accepted = cnt_acc;
        if (rebuild) sc->rebuild_pending = 1;
    }
}

// ------------------------------------------------------------------ plain path
// dU of moving particle req[0] to fixed-point req[1..3] (Energy::energyChange
// after updateChange). out[0] = dU (df), out[1..2] = dM (surface).
template <int MODEL, bool CELLS>
__global__ void __launch_bounds__(kSweepThreads) trial_kernel(const SysDesc *__restrict__ dsc,
                                                              const int64_t *__restrict__ req,
                                                              float2 *__restrict__ out,
                                                              const float2 *__restrict__ sc_tab) {
    extern __shared__ __align__(16) char smem_raw[];
    __shared__ __align__(16) SysDesc sd;
    load_desc(sd, dsc);
    const SysDesc &d = sd;
    constexpr bool KSPACE = (MODEL == MODEL_EWALD);
    const Smem s = carve(smem_raw, d, KSPACE, false, CELLS);
    load_smem(d, s, KSPACE, false, CELLS, sc_tab);
    const int i = (int)req[0];
    int64_t xo[3], xn[3];
    for (int a = 0; a < 3; a++) {
        xo[a] = d.pos64[3 * i + a];
        xn[a] = req[1 + a];
    }
    Move m;
    move_setup(m, i, xo, xn, __int_as_float(d.pos4[i].w), d.ptype[i], d);
    float accf = KSPACE ? kspace_energy(m, d, s) : 0.0f;
    df accd = {0.0f, 0.0f};
    if (CELLS) pairs_cells_warp<MODEL>(m, d, s, accf, accd);
    else pairs_all_strided<MODEL, false>(m, d, s, accf, accd);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    const df part = warp_sum_df(df_add_f(accd, accf));
    if (lane == 0) s.red[warp] = make_float2(part.hi, part.lo);
    __syncthreads();
    if (warp == 0) {
        df du = {0.0f, 0.0f};
        if (lane < nwarp) du = {s.red[lane].x, s.red[lane].y};
        du = warp_sum_df(du);
        if (lane == 0) {
            float dM[3] = {0, 0, 0};
            df M[3];
            for (int a = 0; a < 3; a++) M[a] = {d.sc->m[a][0], d.sc->m[a][1]};
            if (KSPACE) du = df_add(du, surface_delta(m, d, M, dM));
            out[0] = make_float2(du.hi, du.lo);
            out[1] = make_float2(dM[0], dM[1]);
            out[2] = make_float2(dM[2], 0.0f);
        }
    }
}

// Movebase acceptMove + NonbondedEwald::update for the last plain trial: one
// CTA (it reuses the sweep's cell bookkeeping in shared memory).
template <int MODEL, bool CELLS>
__global__ void __launch_bounds__(kSweepThreads) commit_kernel(const SysDesc *__restrict__ dsc,
                                                               const int64_t *__restrict__ req,
                                                               const float2 *__restrict__ trial_out,
                                                               const float2 *__restrict__ sc_tab) {
    extern __shared__ __align__(16) char smem_raw[];
    __shared__ __align__(16) SysDesc sd;
    load_desc(sd, dsc);
    const SysDesc &d = sd;
    constexpr bool KSPACE = (MODEL == MODEL_EWALD);
    const Smem s = carve(smem_raw, d, KSPACE, false, CELLS);
    load_smem(d, s, KSPACE, false, CELLS, sc_tab);
    const int i = (int)req[0];
    int64_t xo[3], xn[3];
    for (int a = 0; a < 3; a++) {
        xo[a] = d.pos64[3 * i + a];
        xn[a] = req[1 + a];
    }
    Move m;
    move_setup(m, i, xo, xn, __int_as_float(d.pos4[i].w), d.ptype[i], d);
    __syncthreads();   // everyone has read the old coordinates
    if (KSPACE) kspace_commit(m, d, s);
    if (threadIdx.x == 0) {
        commit_position(m, d, s, false, CELLS);
        SysScalars *sc = d.sc;
        const df du = {trial_out[0].x, trial_out[0].y};
        df U = df_add(df{sc->u_hi, sc->u_lo}, du);
        df Ut = df_add(df{sc->utot_hi, sc->utot_lo}, du);
        sc->u_hi = U.hi;
        sc->u_lo = U.lo;
        sc->utot_hi = Ut.hi;
        sc->utot_lo = Ut.lo;
        sc->n_accepted++;
        if (KSPACE) {
            const float dM[3] = {trial_out[1].x, trial_out[1].y, trial_out[2].x};
            for (int a = 0; a < 3; a++) {
                const df ma = df_add_f(df{sc->m[a][0], sc->m[a][1]}, dM[a]);
                sc->m[a][0] = ma.hi;
                sc->m[a][1] = ma.lo;
            }
        }
    }
    __syncthreads();
    store_back(d, s, KSPACE, CELLS);
}

// ------------------------------------------------------------------ Q(k) rebuild
// updateAllComplexNumbers (ewald.h:388-415) as the exact integer sum of the
// per-particle contributions. One thread per run of k-vectors sharing
// (nx, ny) (at most kQkRun of them, consecutive nz): per staged particle it
// forms w once and one term per k. Terms (|c| < 2^22) are summed exactly in
// 32 bits over a pass of `stage` <= 64 particles, then added to the thread's
// int64 totals in shared memory. Per pass the block stages the particles'
// axis tables (stage x qk_tab_len) from positions prefetched during the
// previous pass, one particle per thread (stage <= blockDim.x). blockIdx.x
// covers a chunk of particles, blockIdx.y selects the system of a batch;
// only systems with rebuild_pending set do work.
constexpr int kQkRun = 8;
constexpr int kQkMaxThreads = 512;
// One pass over nb staged particles for runs of (at most) L k-vectors.
// Sums of the terms' bit patterns (qk_term_bits); the caller subtracts
// nb kQkMagicBits per sum.
template <int L>
__device__ __forceinline__ void qk_pass(const float2 *et, int T, const float *q2g, int nb, int ix, int iy, int iz,
                                        unsigned ax[kQkRun], unsigned ay[kQkRun]) {
    for (int jj = 0; jj < nb; jj++) {
        const float2 *e = et + jj * T;
        const float2 w = qk_w(q2g[jj], e[ix], e[iy]);
#pragma unroll
        for (int u = 0; u < L; u++) {
            const uint2 c = qk_term_bits(w, e[iz + u]);
            ax[u] += c.x;
            ay[u] += c.y;
        }
    }
}
constexpr int kQkMaxStage = 64;
__host__ __device__ __forceinline__ size_t qk_rebuild_smem(int stage, int T, int threads) {
    return (size_t)stage * T * 8 + (size_t)2 * kQkRun * threads * 8 + (size_t)stage * (16 + 4);
}
__global__ void __launch_bounds__(kQkMaxThreads) qk_rebuild_kernel(const SysDesc *__restrict__ descs, int chunk, int stage) {
    extern __shared__ __align__(16) char qk_smem[];
    __shared__ float2 tab[256];
    const SysDesc &d = descs[blockIdx.y];
    if (d.K == 0 || d.sc->rebuild_pending == 0) return;
    const int j0 = blockIdx.x * chunk, j1 = min(d.N, j0 + chunk);
    if (j0 >= d.N) return;
    const int kcc = d.kcc, T = qk_tab_len(kcc), tid = threadIdx.x, nt = blockDim.x;
    float2 *et = (float2 *)qk_smem;                                          // stage x T
    long long *tot = (long long *)(qk_smem + (size_t)stage * T * 8);          // [2 kQkRun][nt]
    int4 *sp = (int4 *)(qk_smem + (size_t)stage * T * 8 + (size_t)2 * kQkRun * nt * 8);   // stage
    float *q2g = (float *)(sp + stage);                                        // stage
    for (int t = tid; t < 256; t += nt) tab[t] = d.sc_tab[t];
    const int shift = d.qk_shift;
    for (int r0 = 0; r0 < d.nseg; r0 += nt) {   // uniform over the block
        const int r = r0 + tid;
        int k0 = 0, len = 0, ix = 0, iy = 0, iz = 0;
        if (r < d.nseg) {
            const int2 sg = d.kseg[r];
            k0 = sg.x & 0xFFFFFF;
            len = sg.x >> 24;
            ix = (int)(int8_t)(sg.y & 0xFF);
            iy = 2 * kcc + 1 + (int)(int8_t)((sg.y >> 8) & 0xFF);
            iz = 4 * kcc + 2 + (int)(int8_t)((sg.y >> 16) & 0xFF);
        }
#pragma unroll
        for (int u = 0; u < 2 * kQkRun; u++) tot[u * nt + tid] = 0;
        const int wl = __reduce_max_sync(0xffffffffu, len);   // warp-uniform run length
        int4 pn = make_int4(0, 0, 0, 0);
        float qn = 0.0f;
        if (tid < stage && j0 + tid < j1) {
            pn = d.pos4[j0 + tid];
            qn = d.eff[d.ptype[j0 + tid]];
        }
        for (int b = j0; b < j1; b += stage) {
            const int nb = min(stage, j1 - b);
            __syncthreads();   // the previous pass is done with sp, q2g and et
            if (tid < nb) {
                sp[tid] = pn;
                q2g[tid] = qk_charge(__int_as_float(pn.w), qn, d);
            }
            if (tid < stage && b + stage + tid < j1) {   // prefetch the next pass
                pn = d.pos4[b + stage + tid];
                qn = d.eff[d.ptype[b + stage + tid]];
            }
            __syncthreads();
            {
                int jj = tid / T, e = tid - jj * T;
                const int djj = nt / T, de = nt - djj * T;
                while (jj < nb) {
                    const int4 p = sp[jj];
                    const int h[3] = {p.x, p.y, p.z};
                    et[jj * T + e] = qk_tab_entry(e, kcc, h, tab, d.iso != 0);
                    jj += djj;
                    e += de;
                    if (e >= T) {
                        e -= T;
                        jj++;
                    }
                }
            }
            __syncthreads();
            if (len > 0) {
                // unsigned sums: the dropped lanes may wrap, harmlessly
                unsigned ax[kQkRun], ay[kQkRun];
#pragma unroll
                for (int u = 0; u < kQkRun; u++) ax[u] = ay[u] = 0u;
                // the warp's longest run sets the trip count (runs are sorted
                // by length, so warps are nearly uniform); terms past a lane's
                // len read entries further along the buffer (at most
                // kQkRun - 1 past the last record, still inside the shared
                // allocation) and are dropped below
                switch (wl) {
                    case 1: qk_pass<1>(et, T, q2g, nb, ix, iy, iz, ax, ay); break;
                    case 2: qk_pass<2>(et, T, q2g, nb, ix, iy, iz, ax, ay); break;
                    case 3: qk_pass<3>(et, T, q2g, nb, ix, iy, iz, ax, ay); break;
                    case 4: qk_pass<4>(et, T, q2g, nb, ix, iy, iz, ax, ay); break;
                    case 5: qk_pass<5>(et, T, q2g, nb, ix, iy, iz, ax, ay); break;
                    case 6: qk_pass<6>(et, T, q2g, nb, ix, iy, iz, ax, ay); break;
                    case 7: qk_pass<7>(et, T, q2g, nb, ix, iy, iz, ax, ay); break;
                    default: qk_pass<8>(et, T, q2g, nb, ix, iy, iz, ax, ay); break;
                }
                const unsigned off = (unsigned)nb * kQkMagicBits;
#pragma unroll
                for (int u = 0; u < kQkRun; u++)
                    if (u < len) {
                        tot[(2 * u) * nt + tid] += qk_widen((int)(ax[u] - off), shift);
                        tot[(2 * u + 1) * nt + tid] += qk_widen((int)(ay[u] - off), shift);
                    }
            }
        }
#pragma unroll
        for (int u = 0; u < kQkRun; u++)
            if (u < len) {
                atomicAdd((unsigned long long *)&d.qnew[k0 + u].x, (unsigned long long)tot[(2 * u) * nt + tid]);
                atomicAdd((unsigned long long *)&d.qnew[k0 + u].y, (unsigned long long)tot[(2 * u + 1) * nt + tid]);
            }
        __syncthreads();   // tot and the staging buffers are reused by the next round
    }
}

// Compare the rebuilt Q(k) with the running one, adopt it, and record the
// reciprocal-energy change (update()'s drift correction: zero when the two
// agree, as they must) in corr[system] and the running energies.
__global__ void __launch_bounds__(1024) qk_rebuild_finish(const SysDesc *__restrict__ descs,
                                                          float2 *__restrict__ corr) {
    __shared__ float2 red[32];
    __shared__ int pending, mism;
    const SysDesc &d = descs[blockIdx.x];
    if (threadIdx.x == 0) {
        pending = d.K > 0 && d.sc->rebuild_pending;
        mism = 0;
    }
    __syncthreads();
    if (!pending) {
        if (threadIdx.x == 0) corr[blockIdx.x] = make_float2(0.0f, 0.0f);
        return;
    }
    df e = {0.0f, 0.0f};
    int bad = 0;
    for (int k = threadIdx.x; k < d.K; k += blockDim.x) {
        const longlong2 qo = d.qfix[k], qn = d.qnew[k];
        if (qo.x != qn.x || qo.y != qn.y) {
            bad = 1;
            const float2 fo = q_to_float(qo), fn = q_to_float(qn);
            const float dre = fix28_to_float(qn.x - qo.x);
            const float dim = fix28_to_float(qn.y - qo.y);
            e = df_add_f(e, d.kvec[k].w * fmaf(dre, fo.x + fn.x, dim * (fo.y + fn.y)));
        }
        d.qfix[k] = qn;
        d.qnew[k] = make_longlong2(0, 0);
    }
    if (bad) atomicOr(&mism, 1);
    e = warp_sum_df(e);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[w] = make_float2(e.hi, e.lo);
    __syncthreads();
    if (w == 0) {
        df t = {0.0f, 0.0f};
        if (lane < (int)(blockDim.x >> 5)) t = {red[lane].x, red[lane].y};
        t = warp_sum_df(t);
        if (lane == 0) {
            corr[blockIdx.x] = make_float2(t.hi, t.lo);
            SysScalars *sc = d.sc;
            const df U = df_add(df{sc->u_hi, sc->u_lo}, t);
            const df Ut = df_add(df{sc->utot_hi, sc->utot_lo}, t);
            sc->u_hi = U.hi;
            sc->u_lo = U.lo;
            sc->utot_hi = Ut.hi;
            sc->utot_lo = Ut.lo;
            if (mism && sc->verify_rebuild) sc->error |= kErrQkMismatch;
            sc->rebuild_pending = 0;
            sc->n_rebuilds++;
        }
    }
}

// ------------------------------------------------------------------ total energy
// Sum over all pairs i<j (g_internal, energy.h:1207-1216); block partials (df).
template <int MODEL>
__global__ void __launch_bounds__(256) pair_total_kernel(const SysDesc *__restrict__ dsc, float2 *__restrict__ part) {
    __shared__ float2 red[32];
    __shared__ __align__(16) SysDesc sd;
    load_desc(sd, dsc);
    const SysDesc &d = sd;
    df acc = {0, 0};
    for (int64_t i = blockIdx.x; i < d.N; i += gridDim.x) {
        const int4 pi = d.pos4[i];
        const int ti = d.ptype[i];
        const float qi = __int_as_float(pi.w);
        const short4 ei = d.pos_ext[i];
        float a = 0.0f;
        for (int j = (int)i + 1 + threadIdx.x; j < d.N; j += blockDim.x) {
            const int4 pj = d.pos4[j];
            const int t = d.uniform_types ? 0 : ti * d.n_types + d.ptype[j];
            const float r2 = dist2(pj, pi.x, pi.y, pi.z, d);
            if (d.core_tab_n > 0 && r2 < d.s2[t]) {
                const short4 ej = d.pos_ext[j];
                acc = df_add(acc, pair_core_df<MODEL>(pj.x - pi.x, pj.y - pi.y, pj.z - pi.z, ej.x - ei.x,
                                                      ej.y - ei.y, ej.z - ei.z, qi, __int_as_float(pj.w), t, d));
            } else {
                a += pair_u<MODEL>(r2, qi, __int_as_float(pj.w), t, d);
            }
        }
        acc = df_add_f(acc, a);
    }
    acc = warp_sum_df(acc);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[w] = make_float2(acc.hi, acc.lo);
    __syncthreads();
    if (w == 0) {
        df t = {0, 0};
        if (lane < (int)(blockDim.x >> 5)) t = {red[lane].x, red[lane].y};
        t = warp_sum_df(t);
        if (lane == 0) part[blockIdx.x] = make_float2(t.hi, t.lo);
    }
}

// ------------------------------------------------------------------ trial streams
// Device-generated stream: Philox4x32-10 with key = (seed, stream id) and
// counters (trial, 0) and (trial, 1). Per trial: particle floor(r.x N / 2^32);
// displacement (r_a - 2^31) DP_a for r.y, r.z, r.w with DP_a = round(dp/L_a
// 2^32); u = (r2.x + 0.5) / 2^32 and threshold -ln(u) (scaled by kT in the
// sweep).
__global__ void philox_stream_kernel(const SysDesc *__restrict__ dsc, uint32_t seed, uint32_t sys, int64_t first,
                                     int64_t n, const int64_t *__restrict__ dp_fix, Trial *__restrict__ out) {
    const SysDesc &d = *dsc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g = first + t;
        const u4 r = philox4x32_10(u4{(uint32_t)g, (uint32_t)(g >> 32), 0u, 0u}, seed, sys);
        const u4 r2 = philox4x32_10(u4{(uint32_t)g, (uint32_t)(g >> 32), 1u, 0u}, seed, sys);
        Trial tr;
        tr.idx = (int32_t)(((uint64_t)r.x * (uint32_t)d.N) >> 32);
        tr.pad = 0;
        const int ty = d.ptype[tr.idx];
        tr.d[0] = (int64_t)(int32_t)(r.y - 0x80000000u) * dp_fix[3 * ty + 0];
        tr.d[1] = (int64_t)(int32_t)(r.z - 0x80000000u) * dp_fix[3 * ty + 1];
        tr.d[2] = (int64_t)(int32_t)(r.w - 0x80000000u) * dp_fix[3 * ty + 2];
        const double u = ((double)r2.x + 0.5) * (1.0 / 4294967296.0);
        const double thr = -log(u);
        const float h = (float)thr;
        tr.thr_hi = h;
        tr.thr_lo = (float)(thr - (double)h);
        out[t] = tr;
    }
}

// Trial records from the host's arrays (fg_stream_upload): x/L wrapped to [-1/2, 1/2), rounded to 2^-62 and
// shifted to the 64-bit fixed point; the Metropolis threshold -ln u split
// into a float pair (+inf for u = 0).
__global__ void make_trials_kernel(int64_t n, const int32_t *idx, const double *disp, const double *u, double Lx,
                                   double Ly, double Lz, Trial *out) {
    const double L[3] = {Lx, Ly, Lz};
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        Trial tr;
        tr.idx = idx[t];
        tr.pad = 0;
        for (int a = 0; a < 3; a++) {
            double f = disp[3 * t + a] / L[a];
            f -= floor(f + 0.5);
            tr.d[a] = (int64_t)((uint64_t)(int64_t)llrint(f * 4611686018427387904.0) << 2);
        }
        const double ut = u[t];
        const double thr = ut > 0.0 ? -log(ut) : __longlong_as_double(0x7ff0000000000000LL);   // +inf
        const float hi = (float)thr;
        tr.thr_hi = hi;
        tr.thr_lo = isfinite(thr) ? (float)(thr - (double)hi) : 0.0f;
        out[t] = tr;
    }
}

}  // namespace fg
