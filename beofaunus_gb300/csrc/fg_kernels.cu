// Energy-change kernels for atomic systems (one particle moved per trial):
//   * sweep_kernel  : persistent, one CTA per system; runs the trial stream
//                     (trial -> dU -> Metropolis -> accept/reject -> update),
//                     stopping early when an Ewald Q(k) rebuild is due.
//   * trial_kernel / commit_kernel : the plain drop-in path, one call per
//                     trial, mirroring Energy::energyChange + Movebase::update.
//   * qk_rebuild_*  : full Q(k) = sum_j q_j e^{ik.r_j} (updateAllComplexNumbers).
//   * total energy  : systemEnergy for one atomic group.
//
// Reference path restated here: Movebase::move (move.h:515-555),
// AtomicTranslation::_trialMove/_acceptMove/_rejectMove (move.h:818-889),
// Energy::energyChangeConfiguration (energy.h:3521-3572), EwaldReal
// (ewald.h:97-110), WeeksChandlerAndersen (potentials.h:2186-2193),
// DebyeHuckel (potentials.h:3314-3323), LennardJonesMixed
// (potentials.h:2036-2040), NonbondedEwald::updateChange/update/external
// (ewald.h:613-729).
#include <cstdint>
#include <cuda_runtime.h>

#include "fg_device.cuh"
#include "fg_system.cuh"

namespace fg {

constexpr int MODEL_EWALD = 1;
constexpr int MODEL_DHLJ = 2;

// df product (Dekker/FMA two-product plus cross terms).
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float &rh, float &rl) {
    float p = ah * bh;
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, fmaf(al, bh, e));
    df r = fast_two_sum(p, e);
    rh = r.hi;
    rl = r.lo;
}

// ------------------------------------------------------------------ pairs
// EwaldReal (kappa-screened form, ewald.h:109) + WCA. qq = qa*qb*QeQe*lB.
__device__ __forceinline__ float pair_ewald_wca(float r2, float qq, float s2, float wca2, float eps4,
                                                const SysDesc &d) {
    float u = 0.0f;
    if (r2 <= d.rc2) {
        float r = sqrtf(r2);
        float e;
        if (d.kappa == 0.0f) {
            e = erfcf(d.alpha * r);
        } else {
            float k2a = d.kappa / (2.0f * d.alpha);
            e = 0.5f * (erfcf(d.alpha * r + k2a) * expf(d.kappa * r) +
                        erfcf(d.alpha * r - k2a) * expf(-d.kappa * r));
        }
        u = qq * e / r;
    }
    if (r2 <= wca2) {
        float x = s2 / r2;
        x = x * x * x;
        u += eps4 * (x * x - x + 0.25f);
    }
    return u;
}

// DebyeHuckel + LennardJonesMixed. qq = qa*qb*lB.
__device__ __forceinline__ float pair_dh_lj(float r2, float qq, float s2, float eps4, const SysDesc &d) {
    float r = sqrtf(r2);
    float u = qq * expf(-d.kappa * r) / r;
    float x = s2 / r2;
    x = x * x * x;
    return u + eps4 * (x * x - x);
}

template <int MODEL>
__device__ __forceinline__ float pair_u(float r2, float qi, float qj, int ti, int tj, const SysDesc &d,
                                        bool uniform) {
    int t = uniform ? 0 : ti * d.n_types + tj;
    float s2 = d.s2[t], eps4 = d.eps4[t];
    if (MODEL == MODEL_EWALD) {
        float qq = qi * qj * d.qeqe[t] * d.lB;
        return pair_ewald_wca(r2, qq, s2, d.wca2[t], eps4, d);
    } else {
        return pair_dh_lj(r2, qi * qj * d.lB, s2, eps4, d);
    }
}


// ------------------------------------------------------------------ core pairs
// Pairs inside the repulsive core (r < sigma_ij) carry large, steep energies
// (WCA/LJ ~ r^-12): there FP32 rounding and 32-bit coordinate resolution
// would exceed the 1e-6 kT budget. They are rare, so they are evaluated in df
// from 48-bit coordinate differences: Coulomb-like part from a Taylor table
// of g(y) (erfc for Ewald, exp(-y) for Debye-Hueckel) at spacing 1/128, and
// the r^-12/r^-6 part by df division and products.
__device__ __forceinline__ int16_t ext16(int64_t X) {
    int32_t h = hi32(X);
    int32_t rem = (int32_t)((uint64_t)X - ((uint64_t)(uint32_t)h << 32));
    return (int16_t)(rem >> 16);
}

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
    df p = dfm_f(b, q1);
    df r = df_add(a, df_neg(p));
    float q2 = r.hi / b.hi;
    return fast_two_sum(q1, q2);
}

// Energy of one core pair as df. dh: high-word differences (j - i), de:
// differences of the 16-bit extensions; t: type-pair index.
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
    // Coulomb-like part: pref * qi qj * g(coef r) / r
    df y = dfm(df{d.coef_df.x, d.coef_df.y}, r);
    int j = (int)(y.hi * 128.0f + 0.5f);
    j = min(max(j, 0), d.core_tab_n - 1);
    float dl = (y.hi - (float)j * (1.0f / 128.0f)) + y.lo;
    float4 c0 = d.core_tab[j];
    float4 c1 = d.core_tab2[j];
    df g = df_add(df{c0.x, c0.y}, dfm_f(df{c0.z, c0.w}, dl));
    g = df_add_f(g, dl * dl * fmaf(dl, fmaf(dl, c1.z, c1.y), c1.x));
    df qq = two_prod(qi, qj);
    df u = dfm(dfm(dfm(df{d.pref_df[t].x, d.pref_df[t].y}, qq), g), inv);
    // r^-12 / r^-6 part
    df x = df_div(df{d.s2_df[t].x, d.s2_df[t].y}, r2);
    df x3 = dfm(dfm(x, x), x);
    df w = df_add(dfm(x3, x3), df_neg(x3));
    if (MODEL == MODEL_EWALD) w = df_add_f(w, 0.25f);
    w = dfm(w, df{d.eps4_df[t].x, d.eps4_df[t].y});
    return df_add(u, w);
}

// Minimum-image squared distance from high-word fixed-point coordinates.
__device__ __forceinline__ float dist2(int4 a, int xb, int yb, int zb, const SysDesc &d) {
    float dx = (float)(a.x - xb) * d.s32[0];
    float dy = (float)(a.y - yb) * d.s32[1];
    float dz = (float)(a.z - zb) * d.s32[2];
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// ------------------------------------------------------------------ move
struct Move {
    int i;            // particle
    int ti;           // its type
    float q;          // its charge
    int64_t xo[3];    // old fixed-point coordinates
    int64_t xn[3];    // new
    int ho[3], hn[3]; // high words
    int eo[3], en[3]; // 16-bit extensions
    float dxf[3];     // displacement (Angstrom, minimum image) in float
    int co, cn;       // old / new cell (cell systems)
};

__device__ __forceinline__ int cell_of(const int h[3], const SysDesc &d) {
    int c[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        // high word as unsigned offset from -L/2: [0, 2^32)
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
        // minimum-image displacement; |d| < L/2 always for a trial move
        int64_t dd = (int64_t)((uint64_t)xn[a] - (uint64_t)xo[a]);
        m.dxf[a] = (float)dd * d.dl32[a];
    }
    if (d.use_cells) {
        m.co = cell_of(m.ho, d);
        m.cn = cell_of(m.hn, d);
    }
}

// ------------------------------------------------------------------ shared state
struct Smem {
    float2 *sc_tab;    // 256 cos/sin entries
    float4 *kvec;      // K
    uint32_t *kpack;   // K
    float4 *qk;        // K df complex
    int4 *pos;         // N (POS_SMEM)
    short4 *pos_ext;   // N (POS_SMEM)
    uint8_t *ptype;    // N (POS_SMEM)
    float2 *red;       // 32 warp partials (df)
    int *cells;        // stencil scan: 64 cell ids + 65 offsets
    int *bcast;        // decision broadcast
};

// One candidate j against the moved particle: adds u(new) - u(old) to the
// float accumulator (outside the core) or the df accumulator (core pairs).
template <int MODEL>
__device__ __forceinline__ void pair_candidate(const Move &m, int4 pj, int tj, const short4 *ext, const SysDesc &d,
                                               bool uni, float &accf, df &accd) {
    float qj = __int_as_float(pj.w);
    float r2n = dist2(pj, m.hn[0], m.hn[1], m.hn[2], d);
    float r2o = dist2(pj, m.ho[0], m.ho[1], m.ho[2], d);
    int t = uni ? 0 : m.ti * d.n_types + tj;
    float s2 = d.core_tab_n > 0 ? d.s2[t] : 0.0f;   // no core table: FP32 throughout
    bool cn = r2n < s2, co = r2o < s2;
    if (MODEL == MODEL_DHLJ && !cn && !co) {
        // Difference form, so the rounding error scales with |u(new) - u(old)|
        // and not with |u|: r_n^2 - r_o^2 = sum_a (dn_a - do_a)(dn_a + do_a)
        // exactly in integers, then
        //   DH: u_o * expm1(-kappa (r_n - r_o) - log1p((r_n - r_o)/r_o))
        //   LJ: 4eps x_o^3 (t^3 - 1) (x_o^3 (t^3 + 1) - 1), t = r_o^2/r_n^2.
        // (minimum images taken separately, as the reference's sqdist does:
        // near r = L/2 the image of new and old may differ)
        long long S = 0;
        {
            const int pjv[3] = {pj.x, pj.y, pj.z};
#pragma unroll
            for (int a = 0; a < 3; a++) {
                long long dn = (int)(pjv[a] - m.hn[a]), dO = (int)(pjv[a] - m.ho[a]);
                S += (dn - dO) * (dn + dO);
            }
        }
        float dR2 = (float)S * d.s32sq;
        float ro = sqrtf(r2o), rn = sqrtf(r2n);
        float dr = dR2 / (rn + ro);
        float z = fmaf(-d.kappa, dr, -log1pf(dr / ro));
        float uo = m.q * qj * d.lB * expf(-d.kappa * ro) / ro;
        float xo = d.s2[t] / r2o;
        float xo3 = xo * xo * xo;
        float tau = -dR2 / r2n;
        float t3m1 = tau * fmaf(tau, tau + 3.0f, 3.0f);
        accf += fmaf(uo, expm1f(z), d.eps4[t] * xo3 * t3m1 * fmaf(xo3, t3m1 + 2.0f, -1.0f));
        return;
    }
    float un = cn ? 0.0f : pair_u<MODEL>(r2n, m.q, qj, m.ti, tj, d, uni);
    float uo = co ? 0.0f : pair_u<MODEL>(r2o, m.q, qj, m.ti, tj, d, uni);
    accf += un - uo;
    if (cn || co) {
        short4 e = *ext;
        if (cn)
            accd = df_add(accd, pair_core_df<MODEL>(pj.x - m.hn[0], pj.y - m.hn[1], pj.z - m.hn[2], e.x - m.en[0],
                                                    e.y - m.en[1], e.z - m.en[2], m.q, qj, t, d));
        if (co)
            accd = df_add(accd, df_neg(pair_core_df<MODEL>(pj.x - m.ho[0], pj.y - m.ho[1], pj.z - m.ho[2],
                                                           e.x - m.eo[0], e.y - m.eo[1], e.z - m.eo[2], m.q, qj,
                                                           t, d)));
    }
}

// Per-thread partial of the real-space sum (new - old) over all particles.
template <int MODEL, bool POS_SMEM>
__device__ __forceinline__ void pair_partial_all(const Move &m, const SysDesc &d, const Smem &s, float &accf,
                                                 df &accd) {
    const bool uni = d.uniform_types != 0;
    for (int j = threadIdx.x; j < d.N; j += blockDim.x) {
        if (j == m.i) continue;
        int4 pj = POS_SMEM ? s.pos[j] : d.pos4[j];
        int tj = uni ? 0 : (POS_SMEM ? s.ptype[j] : d.ptype[j]);
        pair_candidate<MODEL>(m, pj, tj, POS_SMEM ? &s.pos_ext[j] : &d.pos_ext[j], d, uni, accf, accd);
    }
}

// Cell-list variant: visits the union of the 27-cell stencils of the old and
// new cell (cells are at least one cutoff wide, so every pair within the
// cutoff of either position is seen; farther pairs contribute zero).
template <int MODEL>
__device__ __forceinline__ void pair_partial_cells(const Move &m, const SysDesc &d, const Smem &s, float &accf,
                                                   df &accd) {
    // warp 0 builds the cell list and a prefix sum of counts
    if (threadIdx.x < 32) {
        int lane = threadIdx.x;
        int co[3], cn[3], lo[3], len[3];
        int c = m.co;
        co[0] = c % d.nc[0]; co[1] = (c / d.nc[0]) % d.nc[1]; co[2] = c / (d.nc[0] * d.nc[1]);
        c = m.cn;
        cn[0] = c % d.nc[0]; cn[1] = (c / d.nc[0]) % d.nc[1]; cn[2] = c / (d.nc[0] * d.nc[1]);
#pragma unroll
        for (int a = 0; a < 3; a++) {
            int delta = cn[a] - co[a];
            if (delta > 1) delta -= d.nc[a];
            if (delta < -1) delta += d.nc[a];
            if (delta > 1 || delta < -1) d.sc->error |= kErrStencil;
            lo[a] = co[a] + min(delta, 0) - 1;
            len[a] = 3 + (delta != 0 ? 1 : 0);
        }
        int ncell = len[0] * len[1] * len[2];
        int my_cnt[2] = {0, 0}, my_id[2] = {0, 0};
#pragma unroll
        for (int r = 0; r < 2; r++) {
            int k = lane + 32 * r;
            if (k < ncell) {
                int ix = k % len[0], iy = (k / len[0]) % len[1], iz = k / (len[0] * len[1]);
                int cx = lo[0] + ix, cy = lo[1] + iy, cz = lo[2] + iz;
                cx += (cx < 0) ? d.nc[0] : 0; cx -= (cx >= d.nc[0]) ? d.nc[0] : 0;
                cy += (cy < 0) ? d.nc[1] : 0; cy -= (cy >= d.nc[1]) ? d.nc[1] : 0;
                cz += (cz < 0) ? d.nc[2] : 0; cz -= (cz >= d.nc[2]) ? d.nc[2] : 0;
                int cid = (cz * d.nc[1] + cy) * d.nc[0] + cx;
                my_id[r] = cid;
                my_cnt[r] = d.cell_count[cid];
            }
        }
        // inclusive scan over 64 entries (two rounds of 32)
        int base = 0;
#pragma unroll
        for (int r = 0; r < 2; r++) {
            int v = my_cnt[r];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += t;
            }
            s.cells[lane + 32 * r] = my_id[r];
            s.cells[64 + 1 + lane + 32 * r] = base + v;   // end offset
            base += __shfl_sync(0xffffffffu, v, 31);
        }
        if (lane == 0) { s.cells[64] = 0; s.bcast[1] = min(ncell, 64); }
    }
    __syncthreads();
    const int ncell = s.bcast[1];
    const int total = s.cells[64 + ncell];
    const bool uni = d.uniform_types != 0;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        // find the cell holding candidate t (offsets are increasing)
        int lo = 0, hi = ncell - 1;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (s.cells[64 + 1 + mid] > t) hi = mid; else lo = mid + 1;
        }
        int slot = t - s.cells[64 + lo];
        int cid = s.cells[lo];
        int idx = cid * d.cap + slot;
        int pid = d.cell_pid[idx];
        if ((pid & 0xFFFFFF) == m.i) continue;
        int4 pj = d.cell_pos[idx];
        int tj = uni ? 0 : (pid >> 24);
        pair_candidate<MODEL>(m, pj, tj, &d.cell_ext[idx], d, uni, accf, accd);
    }
}

// Reciprocal-space change for this thread's k-vectors (k = tid + r*blockDim).
// Delta_k = q e^{ik.r_old} (e^{ik.d} - 1): relative (not absolute) FP32 error.
// Energy: A'_k (2 Re(conj(Q_k) Delta_k) + |Delta_k|^2), A'_k = A_k 2 pi lB / V.
__device__ __forceinline__ float kspace_partial(const Move &m, const SysDesc &d, const Smem &s,
                                                const float4 *__restrict__ qk, float2 dq[kMaxKPerThread]) {
    float acc = 0.0f;
    const float qe = m.q * d.eff[m.ti];
#pragma unroll
    for (int r = 0; r < kMaxKPerThread; r++) {
        int k = threadIdx.x + r * blockDim.x;
        dq[r] = make_float2(0.0f, 0.0f);
        if (k < d.K) {
            uint32_t p = s.kpack[k];
            int nx = (int)(int8_t)(p & 0xFF), ny = (int)(int8_t)((p >> 8) & 0xFF), nz = (int)(int8_t)(p >> 16);
            uint32_t ph = (uint32_t)nx * (uint32_t)m.ho[0] + (uint32_t)ny * (uint32_t)m.ho[1] +
                          (uint32_t)nz * (uint32_t)m.ho[2];
            float2 e = sincos_turns(ph, s.sc_tab);
            float4 kv = s.kvec[k];
            float phi = fmaf(kv.x, m.dxf[0], fmaf(kv.y, m.dxf[1], kv.z * m.dxf[2]));
            float2 w;
            if (fabsf(phi) <= 1.6f) {
                w = expm1_i(phi);
            } else {
                uint32_t phn = (uint32_t)nx * (uint32_t)m.hn[0] + (uint32_t)ny * (uint32_t)m.hn[1] +
                               (uint32_t)nz * (uint32_t)m.hn[2];
                float2 en = sincos_turns(phn - ph, s.sc_tab);
                w = make_float2(en.x - 1.0f, en.y);
            }
            float2 dd = cmul(e, w);
            dd.x *= qe;
            dd.y *= qe;
            dq[r] = dd;
            float4 q = qk[k];
            acc = fmaf(kv.w, fmaf(2.0f, fmaf(q.x, dd.x, q.z * dd.y), fmaf(dd.x, dd.x, dd.y * dd.y)), acc);
        }
    }
    return acc;
}

// Surface term change (getSurfaceEnergy, ewald.h:277-291) for thread 0:
// M = sum q eff r over wrapped positions; dE = c (2 M.dM + |dM|^2).
__device__ __forceinline__ df surface_delta(const Move &m, const SysDesc &d, float dM[3]) {
    const float qe = m.q * d.eff[m.ti];
    df acc = {0.0f, 0.0f};
    if (d.surf_c == 0.0f) {
        dM[0] = dM[1] = dM[2] = 0.0f;
        return acc;
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        // wrapped-coordinate difference (a boundary crossing changes r by L)
        float rn = (float)m.hn[a] * d.s32[a];
        float ro = (float)m.ho[a] * d.s32[a];
        dM[a] = qe * (rn - ro);
        float M = d.sc->m[a][0] + d.sc->m[a][1];
        acc = df_add_f(acc, d.surf_c * fmaf(2.0f * M, dM[a], dM[a] * dM[a]));
    }
    return acc;
}

// Block-wide df sum of per-thread partials; result valid in warp 0.
__device__ __forceinline__ df block_sum(df x, const Smem &s) {
    x = warp_sum_df(x);
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) s.red[w] = make_float2(x.hi, x.lo);
    __syncthreads();
    df t = {0.0f, 0.0f};
    if (w == 0) {
        int nw = (blockDim.x + 31) >> 5;
        if (lane < nw) t = {s.red[lane].x, s.red[lane].y};
        t = warp_sum_df(t);
    }
    return t;
}

// Accept: positions (master, pair copy, cell list) -- thread 0 only.
__device__ __forceinline__ void commit_position(const Move &m, const SysDesc &d, const Smem &s, bool pos_smem) {
    int4 rec = make_int4(m.hn[0], m.hn[1], m.hn[2], __float_as_int(m.q));
    d.pos64[3 * m.i + 0] = m.xn[0];
    d.pos64[3 * m.i + 1] = m.xn[1];
    d.pos64[3 * m.i + 2] = m.xn[2];
    short4 ext = make_short4((short)m.en[0], (short)m.en[1], (short)m.en[2], 0);
    d.pos4[m.i] = rec;
    d.pos_ext[m.i] = ext;
    if (pos_smem) {
        s.pos[m.i] = rec;
        s.pos_ext[m.i] = ext;
    }
    if (d.use_cells) {
        int slot = d.p_slot[m.i];
        if (m.cn == m.co) {
            d.cell_pos[m.co * d.cap + slot] = rec;
            d.cell_ext[m.co * d.cap + slot] = ext;
        } else {
            // remove from old cell: move its last entry into our slot
            int last = d.cell_count[m.co] - 1;
            int src = m.co * d.cap + last;
            if (last != slot) {
                int pid = d.cell_pid[src];
                d.cell_pos[m.co * d.cap + slot] = d.cell_pos[src];
                d.cell_ext[m.co * d.cap + slot] = d.cell_ext[src];
                d.cell_pid[m.co * d.cap + slot] = pid;
                d.p_slot[pid & 0xFFFFFF] = slot;
            }
            d.cell_count[m.co] = last;
            int ns = d.cell_count[m.cn];
            if (ns >= d.cap) {
                d.sc->error |= kErrCellOverflow;
                ns = d.cap - 1;   // keep indices in bounds; result flagged invalid
            } else {
                d.cell_count[m.cn] = ns + 1;
            }
            d.cell_pos[m.cn * d.cap + ns] = rec;
            d.cell_ext[m.cn * d.cap + ns] = ext;
            d.cell_pid[m.cn * d.cap + ns] = m.i | (m.ti << 24);
            d.p_cell[m.i] = m.cn;
            d.p_slot[m.i] = ns;
        }
    }
}

// Copy a system descriptor into shared memory (all threads participate).
__device__ __forceinline__ void load_desc(SysDesc &dst, const SysDesc *__restrict__ src) {
    const int4 *s4 = reinterpret_cast<const int4 *>(src);
    int4 *d4 = reinterpret_cast<int4 *>(&dst);
    for (int t = threadIdx.x; t < (int)(sizeof(SysDesc) / 16); t += blockDim.x) d4[t] = s4[t];
    __syncthreads();
}

// ------------------------------------------------------------------ smem carve
__device__ __forceinline__ Smem carve(char *base, const SysDesc &d, bool pos_smem, bool kspace) {
    Smem s;
    char *p = base;
    s.sc_tab = (float2 *)p; p += 256 * sizeof(float2);
    s.red = (float2 *)p; p += 32 * sizeof(float2);
    s.cells = (int *)p; p += 160 * sizeof(int);
    s.bcast = (int *)p; p += 8 * sizeof(int);
    if (kspace) {
        s.kvec = (float4 *)p; p += d.K * sizeof(float4);
        s.qk = (float4 *)p; p += d.K * sizeof(float4);
        s.kpack = (uint32_t *)p; p += ((d.K + 3) & ~3) * sizeof(uint32_t);
    } else {
        s.kvec = nullptr; s.qk = nullptr; s.kpack = nullptr;
    }
    if (pos_smem) {
        s.pos = (int4 *)p; p += d.N * sizeof(int4);
        s.pos_ext = (short4 *)p; p += d.N * sizeof(short4);
        s.ptype = (uint8_t *)p;
    } else {
        s.pos = nullptr; s.pos_ext = nullptr; s.ptype = nullptr;
    }
    return s;
}

__device__ __forceinline__ void load_smem(const SysDesc &d, const Smem &s, bool pos_smem, bool kspace,
                                          const float2 *sc_tab) {
    for (int t = threadIdx.x; t < 256; t += blockDim.x) s.sc_tab[t] = sc_tab[t];
    if (kspace)
        for (int k = threadIdx.x; k < d.K; k += blockDim.x) {
            s.kvec[k] = d.kvec[k];
            s.qk[k] = d.qk[k];
            s.kpack[k] = d.kpack[k];
        }
    if (pos_smem)
        for (int j = threadIdx.x; j < d.N; j += blockDim.x) {
            s.pos[j] = d.pos4[j];
            s.pos_ext[j] = d.pos_ext[j];
            s.ptype[j] = d.ptype[j];
        }
    __syncthreads();
}

// ------------------------------------------------------------------ sweep
// Runs trials [cursor, end) of each system's stream; one CTA per system.
// Stops after an accepted trial that makes a Q(k) rebuild due
// (NonbondedEwald::update, ewald.h:633: ++cnt_accepted > update_frequency-1).
template <int MODEL, bool CELLS, bool POS_SMEM>
__global__ void __launch_bounds__(kMaxThreads) sweep_kernel(const SysDesc *__restrict__ descs, int64_t end,
                                                            const float2 *__restrict__ sc_tab) {
    extern __shared__ __align__(16) char smem_raw[];
    __shared__ __align__(16) SysDesc sd;
    load_desc(sd, descs + blockIdx.x);
    const SysDesc &d = sd;
    constexpr bool KSPACE = (MODEL == MODEL_EWALD);
    Smem s = carve(smem_raw, d, POS_SMEM, KSPACE);
    SysScalars *sc = d.sc;
    if (sc->rebuild_pending) return;   // the host runs the rebuild first
    load_smem(d, s, POS_SMEM, KSPACE, sc_tab);
    int64_t cur = sc->cursor;
    const int64_t stop = min(end, sc->n_trials);
    df U = {sc->u_hi, sc->u_lo};
    int cnt_acc = sc->cnt_accepted;
    int64_t nacc = sc->n_accepted;
    const int uf = d.update_frequency;
    bool rebuild = false;
    while (cur < stop && !rebuild) {
        const Trial tr = d.trials[cur];
        Move m;
        int64_t xo[3], xn[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            xo[a] = d.pos64[3 * tr.idx + a];
            xn[a] = (int64_t)((uint64_t)xo[a] + (uint64_t)tr.d[a]);
        }
        int4 rec = POS_SMEM ? s.pos[tr.idx] : d.pos4[tr.idx];
        int ti = POS_SMEM ? s.ptype[tr.idx] : d.ptype[tr.idx];
        move_setup(m, tr.idx, xo, xn, __int_as_float(rec.w), ti, d);
        float part = 0.0f;
        df partd = {0.0f, 0.0f};
        if (CELLS) pair_partial_cells<MODEL>(m, d, s, part, partd);
        else pair_partial_all<MODEL, POS_SMEM>(m, d, s, part, partd);
        float2 dq[kMaxKPerThread];
        if (KSPACE) part += kspace_partial(m, d, s, s.qk, dq);
        df du = block_sum(df_add_f(partd, part), s);
        if (threadIdx.x == 0) {
            float dM[3];
            if (KSPACE) du = df_add(du, surface_delta(m, d, dM));
            df thr = {tr.thr_hi, tr.thr_lo};
            if (d.kT != 1.0f) df_mul(thr.hi, thr.lo, d.kT, 0.0f, thr.hi, thr.lo);
            bool nan = !(du.hi == du.hi);
            // Movebase::metropolis (move.h:567-573): reject iff u > exp(-dU/kT),
            // i.e. dU > kT * (-ln u). A NaN dU compares false there: accepted.
            bool accept = nan || !df_gt(du, thr);
            if (nan) sc->error |= kErrNonFinite;
            if (d.log_trials) {
                d.trial_du[cur] = make_float2(du.hi, du.lo);
                d.trial_acc[cur] = accept ? 1 : 0;
            }
            if (accept) {
                commit_position(m, d, s, POS_SMEM);
                U = df_add(U, du);
                nacc++;
                if (KSPACE) {
#pragma unroll
                    for (int a = 0; a < 3; a++) {
                        df ma = {sc->m[a][0], sc->m[a][1]};
                        ma = df_add_f(ma, dM[a]);
                        sc->m[a][0] = ma.hi;
                        sc->m[a][1] = ma.lo;
                    }
                    if (++cnt_acc > uf - 1) rebuild = true;
                }
            }
            s.bcast[0] = (accept ? 1 : 0) | (rebuild ? 2 : 0);
        }
        __syncthreads();
        const int flag = s.bcast[0];
        if (KSPACE && (flag & 1)) {
            // Q(k) += Delta_k (df, exact accumulation of the FP32 increments)
#pragma unroll
            for (int r = 0; r < kMaxKPerThread; r++) {
                int k = threadIdx.x + r * blockDim.x;
                if (k < d.K) {
                    float4 q = s.qk[k];
                    df re = df_add_f(df{q.x, q.y}, dq[r].x);
                    df im = df_add_f(df{q.z, q.w}, dq[r].y);
                    s.qk[k] = make_float4(re.hi, re.lo, im.hi, im.lo);
                }
            }
        }
        rebuild = (flag & 2) != 0;
        cur++;
    }
    // write back
    if (KSPACE)
        for (int k = threadIdx.x; k < d.K; k += blockDim.x) d.qk[k] = s.qk[k];
    if (threadIdx.x == 0) {
        sc->cursor = cur;
        sc->u_hi = U.hi;
        sc->u_lo = U.lo;
        sc->n_accepted = nacc;
        if (KSPACE) {
            if (rebuild) { sc->rebuild_pending = 1; cnt_acc = 0; }
            sc->cnt_accepted = cnt_acc;
        }
    }
}

// ------------------------------------------------------------------ plain path
// dU for moving particle `idx` to fixed-point xn (Energy::energyChange after
// updateChange). Writes dU (df) to out[0] and Delta Q(k) to d.pending_dq.
template <int MODEL, bool CELLS>
__global__ void __launch_bounds__(kMaxThreads) trial_kernel(const SysDesc *__restrict__ dsc,
                                                            const int64_t *__restrict__ req,
                                                            float2 *__restrict__ out,
                                                            const float2 *__restrict__ sc_tab) {
    extern __shared__ __align__(16) char smem_raw[];
    __shared__ __align__(16) SysDesc sd;
    load_desc(sd, dsc);
    const SysDesc &d = sd;
    constexpr bool KSPACE = (MODEL == MODEL_EWALD);
    Smem s = carve(smem_raw, d, false, KSPACE);
    load_smem(d, s, false, KSPACE, sc_tab);
    int i = (int)req[0];
    int64_t xo[3], xn[3];
    for (int a = 0; a < 3; a++) {
        xo[a] = d.pos64[3 * i + a];
        xn[a] = req[1 + a];
    }
    int4 rec = d.pos4[i];
    Move m;
    move_setup(m, i, xo, xn, __int_as_float(rec.w), d.ptype[i], d);
    float part = 0.0f;
    df partd = {0.0f, 0.0f};
    if (CELLS) pair_partial_cells<MODEL>(m, d, s, part, partd);
    else pair_partial_all<MODEL, false>(m, d, s, part, partd);
    float2 dq[kMaxKPerThread];
    if (KSPACE) {
        part += kspace_partial(m, d, s, s.qk, dq);
        for (int r = 0; r < kMaxKPerThread; r++) {
            int k = threadIdx.x + r * blockDim.x;
            if (k < d.K) d.pending_dq[k] = dq[r];
        }
    }
    df du = block_sum(df_add_f(partd, part), s);
    if (threadIdx.x == 0) {
        float dM[3] = {0, 0, 0};
        if (KSPACE) du = df_add(du, surface_delta(m, d, dM));
        out[0] = make_float2(du.hi, du.lo);
        out[1] = make_float2(dM[0], dM[1]);
        out[2] = make_float2(dM[2], 0.0f);
    }
}

// Movebase acceptMove/rejectMove + NonbondedEwald::update for the last trial.
// flags[0] = accepted; returns flags[1] = 1 if a Q(k) rebuild is now due.
template <int MODEL>
__global__ void commit_kernel(const SysDesc *__restrict__ dsc, const int64_t *__restrict__ req,
                              const float2 *__restrict__ trial_out, int accepted, int32_t *__restrict__ flags) {
    const SysDesc &d = *dsc;
    constexpr bool KSPACE = (MODEL == MODEL_EWALD);
    if (!accepted) {
        if (threadIdx.x == 0 && blockIdx.x == 0) flags[1] = 0;
        return;
    }
    if (KSPACE)
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < d.K; k += gridDim.x * blockDim.x) {
            float4 q = d.qk[k];
            float2 dd = d.pending_dq[k];
            df re = df_add_f(df{q.x, q.y}, dd.x);
            df im = df_add_f(df{q.z, q.w}, dd.y);
            d.qk[k] = make_float4(re.hi, re.lo, im.hi, im.lo);
        }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int i = (int)req[0];
        int64_t xo[3], xn[3];
        for (int a = 0; a < 3; a++) {
            xo[a] = d.pos64[3 * i + a];
            xn[a] = req[1 + a];
        }
        int4 rec = d.pos4[i];
        Move m;
        move_setup(m, i, xo, xn, __int_as_float(rec.w), d.ptype[i], d);
        Smem s{};
        commit_position(m, d, s, false);
        SysScalars *sc = d.sc;
        df U = {sc->u_hi, sc->u_lo};
        U = df_add(U, df{trial_out[0].x, trial_out[0].y});
        sc->u_hi = U.hi;
        sc->u_lo = U.lo;
        sc->n_accepted++;
        int due = 0;
        if (KSPACE) {
            float dM[3] = {trial_out[1].x, trial_out[1].y, trial_out[2].x};
            for (int a = 0; a < 3; a++) {
                df ma = {sc->m[a][0], sc->m[a][1]};
                ma = df_add_f(ma, dM[a]);
                sc->m[a][0] = ma.hi;
                sc->m[a][1] = ma.lo;
            }
            if (++sc->cnt_accepted > d.update_frequency - 1) {
                sc->cnt_accepted = 0;
                sc->rebuild_pending = 1;
                due = 1;
            }
        }
        flags[1] = due;
    }
}

// ------------------------------------------------------------------ Q(k) rebuild
// updateAllComplexNumbers (ewald.h:388-415) to ~1e-13: per particle and axis
// the factors e^{i n theta_a}, theta_a = 2 pi X_a / 2^64, from FP64
// sincospi of the exact integer phase (n X mod 2^64), stored as df pairs;
// then Q_k = sum_j q_j eff_j ex[nx] ey[ny] ez[nz] accumulated in df.
__global__ void axis_phase_kernel(const SysDesc *__restrict__ dsc, int kc, float4 *__restrict__ tab) {
    const SysDesc &d = *dsc;
    if (d.sc->rebuild_pending == 0) return;
    // tab layout: particle-major, (kc+1) x-entries, (2kc+1) y, (2kc+1) z
    const int per = (kc + 1) + 2 * (2 * kc + 1);
    int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t total = (int64_t)d.N * per;
    for (; tid < total; tid += (int64_t)gridDim.x * blockDim.x) {
        int j = (int)(tid / per), e = (int)(tid % per);
        int axis, n;
        if (e <= kc) { axis = 0; n = e; }
        else if (e <= kc + 2 * kc + 1) { axis = 1; n = e - (kc + 1) - kc; }
        else { axis = 2; n = e - (kc + 1) - (2 * kc + 1) - kc; }
        uint64_t ph = (uint64_t)(int64_t)n * (uint64_t)d.pos64[3 * j + axis];
        // turns in [-1/2, 1/2) -> sincospi argument in [-1, 1)
        double t = (double)(int64_t)ph * (1.0 / 9223372036854775808.0);
        double sn, cs;
        sincospi(t, &sn, &cs);
        float ch = (float)cs, sh = (float)sn;
        tab[tid] = make_float4(ch, (float)(cs - (double)ch), sh, (float)(sn - (double)sh));
    }
}

// (a + ib)(c + id) in df
__device__ __forceinline__ float4 df_cmul(float4 a, float4 b) {
    float r1h, r1l, r2h, r2l, i1h, i1l, i2h, i2l;
    df_mul(a.x, a.y, b.x, b.y, r1h, r1l);
    df_mul(a.z, a.w, b.z, b.w, r2h, r2l);
    df_mul(a.x, a.y, b.z, b.w, i1h, i1l);
    df_mul(a.z, a.w, b.x, b.y, i2h, i2l);
    df re = df_add(df{r1h, r1l}, df{-r2h, -r2l});
    df im = df_add(df{i1h, i1l}, df{i2h, i2l});
    return make_float4(re.hi, re.lo, im.hi, im.lo);
}

// One block per group of 128 k-vectors x one particle chunk; partial sums to
// part[chunk][k] (df complex). A second kernel reduces over chunks.
__global__ void __launch_bounds__(128) qk_partial_kernel(const SysDesc *__restrict__ dsc, int kc,
                                                         const float4 *__restrict__ tab, int chunk,
                                                         float4 *__restrict__ part) {
    const SysDesc &d = *dsc;
    if (d.sc->rebuild_pending == 0) return;
    const int per = (kc + 1) + 2 * (2 * kc + 1);
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int c = blockIdx.y;
    int j0 = c * chunk, j1 = min(d.N, j0 + chunk);
    if (k >= d.K) return;
    uint32_t p = d.kpack[k];
    int nx = (int)(int8_t)(p & 0xFF), ny = (int)(int8_t)((p >> 8) & 0xFF), nz = (int)(int8_t)(p >> 16);
    int ex = nx, ey = (kc + 1) + (ny + kc), ez = (kc + 1) + (2 * kc + 1) + (nz + kc);
    df re = {0, 0}, im = {0, 0};
    for (int j = j0; j < j1; j++) {
        const float4 *t = tab + (int64_t)j * per;
        float4 e = df_cmul(df_cmul(t[ex], t[ey]), t[ez]);
        float qe = __int_as_float(d.pos4[j].w) * d.eff[d.ptype[j]];
        float h, l;
        df_mul(e.x, e.y, qe, 0.0f, h, l);
        re = df_add(re, df{h, l});
        df_mul(e.z, e.w, qe, 0.0f, h, l);
        im = df_add(im, df{h, l});
    }
    part[(int64_t)c * d.K + k] = make_float4(re.hi, re.lo, im.hi, im.lo);
}

// Reduce partials, replace Q(k), and return in energy[1] the change of the
// reciprocal energy caused by the rebuild (update()'s drift correction).
__global__ void __launch_bounds__(1024) qk_finish_kernel(const SysDesc *__restrict__ dsc,
                                                         const float4 *__restrict__ part, int nchunk,
                                                         float2 *__restrict__ energy) {
    __shared__ float2 red[64];
    __shared__ int pending;
    const SysDesc &d = *dsc;
    if (threadIdx.x == 0) pending = d.sc->rebuild_pending;
    __syncthreads();
    if (pending == 0) {
        if (threadIdx.x == 0) energy[1] = make_float2(0.0f, 0.0f);
        return;
    }
    df eb = {0, 0}, ea = {0, 0};
    for (int k = threadIdx.x; k < d.K; k += blockDim.x) {
        df re = {0, 0}, im = {0, 0};
        for (int c = 0; c < nchunk; c++) {
            float4 v = part[(int64_t)c * d.K + k];
            re = df_add(re, df{v.x, v.y});
            im = df_add(im, df{v.z, v.w});
        }
        float4 old = d.qk[k];
        float a = d.kvec[k].w;
        // A'(|Qn|^2 - |Qo|^2) = A' ((Qn-Qo).(Qn+Qo)) with the difference
        // taken in df, so the (tiny) drift correction keeps its digits
        df dre = df_add(re, df{-old.x, -old.y}), dim = df_add(im, df{-old.z, -old.w});
        float sre = (re.hi + old.x) + (re.lo + old.y), sim = (im.hi + old.z) + (im.lo + old.w);
        eb = df_add_f(eb, 0.0f);
        ea = df_add_f(ea, a * fmaf(dre.hi + dre.lo, sre, (dim.hi + dim.lo) * sim));
        d.qk[k] = make_float4(re.hi, re.lo, im.hi, im.lo);
    }
    eb = warp_sum_df(eb);
    ea = warp_sum_df(ea);
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { red[w] = make_float2(eb.hi, eb.lo); red[32 + w] = make_float2(ea.hi, ea.lo); }
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        df b = {0, 0}, a = {0, 0};
        if (lane < nw) { b = {red[lane].x, red[lane].y}; a = {red[32 + lane].x, red[32 + lane].y}; }
        b = warp_sum_df(b);
        a = warp_sum_df(a);
        if (lane == 0) {
            energy[0] = make_float2(b.hi, b.lo);
            energy[1] = make_float2(a.hi, a.lo);
            // the correction (after - before) joins the running energy, as
            // Movebase::move adds update()'s return value to utot
            SysScalars *sc = d.sc;
            df U = {sc->u_hi, sc->u_lo};
            U = df_add(U, a);
            sc->u_hi = U.hi;
            sc->u_lo = U.lo;
            sc->rebuild_pending = 0;
            sc->n_rebuilds++;
        }
    }
}

// ------------------------------------------------------------------ total energy
// Sum over all pairs i<j (g_internal, energy.h:1207-1216); block partials (df).
template <int MODEL>
__global__ void __launch_bounds__(256) pair_total_kernel(const SysDesc *__restrict__ dsc,
                                                         float2 *__restrict__ part) {
    __shared__ float2 red[32];
    __shared__ __align__(16) SysDesc sd;
    load_desc(sd, dsc);
    const SysDesc &d = sd;
    const bool uni = d.uniform_types != 0;
    df acc = {0, 0};
    int64_t npair_rows = d.N;
    for (int64_t i = blockIdx.x; i < npair_rows; i += gridDim.x) {
        int4 pi = d.pos4[i];
        int ti = uni ? 0 : d.ptype[i];
        float qi = __int_as_float(pi.w);
        short4 ei = d.pos_ext[i];
        float a = 0.0f;
        for (int j = (int)i + 1 + threadIdx.x; j < d.N; j += blockDim.x) {
            int4 pj = d.pos4[j];
            int tj = uni ? 0 : d.ptype[j];
            float r2 = dist2(pj, pi.x, pi.y, pi.z, d);
            int t = uni ? 0 : ti * d.n_types + tj;
            if (d.core_tab_n > 0 && r2 < d.s2[t]) {
                short4 ej = d.pos_ext[j];
                acc = df_add(acc, pair_core_df<MODEL>(pj.x - pi.x, pj.y - pi.y, pj.z - pi.z, ej.x - ei.x,
                                                      ej.y - ei.y, ej.z - ei.z, qi, __int_as_float(pj.w), t, d));
            } else {
                a += pair_u<MODEL>(r2, qi, __int_as_float(pj.w), ti, tj, d, uni);
            }
        }
        acc = df_add_f(acc, a);
    }
    acc = warp_sum_df(acc);
    int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
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
// Device-generated stream (batched / served systems): Philox4x32-10 with
// key = (seed, system), counters (trial, 0) and (trial, 1). Per trial:
// particle = floor(r.x * N / 2^32); displacement_a = (r_a - 2^31) * DP_a for
// r.y, r.z, r.w with DP_a = round(dp/L_a * 2^32); u = (r2.x + 0.5) / 2^32,
// threshold -ln(u) (the kernel scales it by the system's kT).
__global__ void philox_stream_kernel(const SysDesc *__restrict__ dsc, uint32_t seed, uint32_t sys, int64_t first,
                                     int64_t n, const int64_t *__restrict__ dp_fix, Trial *__restrict__ out) {
    const SysDesc &d = *dsc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t g = first + t;
        u4 r = philox4x32_10(u4{(uint32_t)g, (uint32_t)(g >> 32), 0u, 0u}, seed, sys);
        u4 r2 = philox4x32_10(u4{(uint32_t)g, (uint32_t)(g >> 32), 1u, 0u}, seed, sys);
        Trial tr;
        tr.idx = (int32_t)(((uint64_t)r.x * (uint32_t)d.N) >> 32);
        tr.pad = 0;
        int ty = d.ptype[tr.idx];
        tr.d[0] = (int64_t)(int32_t)(r.y - 0x80000000u) * dp_fix[3 * ty + 0];
        tr.d[1] = (int64_t)(int32_t)(r.z - 0x80000000u) * dp_fix[3 * ty + 1];
        tr.d[2] = (int64_t)(int32_t)(r.w - 0x80000000u) * dp_fix[3 * ty + 2];
        double u = ((double)r2.x + 0.5) * (1.0 / 4294967296.0);
        double thr = -log(u);
        float h = (float)thr;
        tr.thr_hi = h;
        tr.thr_lo = (float)(thr - (double)h);
        out[t] = tr;
    }
}

}  // namespace fg
