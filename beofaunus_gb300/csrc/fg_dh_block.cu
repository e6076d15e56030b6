// Debye-Hueckel + Lennard-Jones sweeps in blocks of trials (all-pairs systems).
//
// Included by fg_api.cu after fg_kernels.cu (one translation unit).
//
// The Metropolis chain is sequential: trial t+1 sees the configuration that
// trial t left. For a pair potential that dependence is small and exact to
// undo: if trial a (particle i_a, old o_a -> new n_a) was accepted, the energy
// change of a later trial m (particle i_m != i_a, o_m -> n_m) differs from its
// value in the configuration before trial a by exactly
//     c(a, m) = [u(n_m, n_a) - u(o_m, n_a)] - [u(n_m, o_a) - u(o_m, o_a)].
// So a block of up to 32 trials is evaluated in parallel against the
// configuration at the start of the block (each warp sums two trials over all
// particles), the 32 x 32 corrections c(a, m) are evaluated in parallel, and
// one warp then walks the block in order: lane m keeps dU_m = base_m +
// sum of c(a, m) over accepted a < m, decides, and on acceptance every later
// lane adds its correction. A trial whose particle was already moved by an
// accepted trial of the block ends the block there; it is evaluated again at
// the start of the next one. Decisions, dU values and the acceptance sequence
// are those of the one-trial-at-a-time chain (Movebase::move, move.h:515-555).
//
// Large systems spread one block over a thread-block cluster: CTA r sums the
// particles of slice r, the per-trial partial sums meet through distributed
// shared memory after one cluster barrier per block, and every CTA resolves
// the block identically (same numbers, same order) and applies the accepted
// moves to the shared master coordinates and its own slice.
namespace fg {

constexpr int kBlkTrials = 32;
constexpr int kBlkThreads = 512;

__device__ __forceinline__ unsigned blk_cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned blk_cluster_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void blk_cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ float2 blk_ld_cluster(const float2 *p, unsigned rank) {
    unsigned a = (unsigned)__cvta_generic_to_shared(p), ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(ra) : "memory");
    return v;
}

struct BlkSmem {
    int4 *spos;      // slice: high words, .w = charge bits
    short4 *sext;    // slice: 16 more bits
    uint8_t *stype;  // slice: types
    Move *mv;        // [32] trials of the block
    float2 *thr;     // [32] threshold (df, already times kT)
    uint32_t *col;   // [32] earlier trials of the block on the same particle
    float2 *corr;    // [32][32] c(a, m) as df
    float2 *part;    // [2][32] this CTA's partial sums (double-buffered)
    int *info;       // [4]: trials resolved in the block, decisions bitmask, queue length
    uint32_t *queue; // near pairs (trial << 24 | slice index), evaluated densely after the sums
    unsigned long long *fix;  // [32] near-pair sums per trial, fixed point 2^-40
};

constexpr int kBlkQueue = 2048;

__host__ __device__ inline size_t blk_align(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline size_t blk_smem_bytes(int ns, bool slice) {
    size_t o = 0;
    if (slice) o += blk_align((size_t)ns * 16) + blk_align((size_t)ns * 8) + blk_align((size_t)ns);
    o += blk_align(sizeof(Move) * kBlkTrials);
    o += blk_align(8 * kBlkTrials) + blk_align(4 * kBlkTrials);
    o += blk_align(8 * kBlkTrials * kBlkTrials) + blk_align(8 * 2 * kBlkTrials) + 16;
    o += blk_align(4 * 2048) + blk_align(8 * kBlkTrials);
    return o;
}

__device__ inline BlkSmem blk_carve(unsigned char *b, int ns, bool slice) {
    BlkSmem s;
    size_t o = 0;
    if (slice) {
        s.spos = (int4 *)(b + o); o += blk_align((size_t)ns * 16);
        s.sext = (short4 *)(b + o); o += blk_align((size_t)ns * 8);
        s.stype = (uint8_t *)(b + o); o += blk_align((size_t)ns);
    } else {
        s.spos = nullptr; s.sext = nullptr; s.stype = nullptr;
    }
    s.mv = (Move *)(b + o); o += blk_align(sizeof(Move) * kBlkTrials);
    s.thr = (float2 *)(b + o); o += blk_align(8 * kBlkTrials);
    s.col = (uint32_t *)(b + o); o += blk_align(4 * kBlkTrials);
    s.corr = (float2 *)(b + o); o += blk_align(8 * kBlkTrials * kBlkTrials);
    s.part = (float2 *)(b + o); o += blk_align(8 * 2 * kBlkTrials);
    s.info = (int *)(b + o); o += 16;
    s.queue = (uint32_t *)(b + o); o += blk_align(4 * 2048);
    s.fix = (unsigned long long *)(b + o);
    return s;
}

// df -> fixed point (2^-40) and back, for order-independent sums of near pairs
__device__ __forceinline__ unsigned long long blk_to_fix(df v) {
    const long long a = __float2ll_rn(v.hi * 1099511627776.0f);
    const long long b = __float2ll_rn(v.lo * 1099511627776.0f);
    return (unsigned long long)(a + b);
}
__device__ __forceinline__ df blk_from_fix(unsigned long long u) {
    const long long v = (long long)u;
    const float h = i64_to_float(v);
    const long long r = v - __float2ll_rn(h);
    return fast_two_sum(h * 9.094947017729282e-13f, i64_to_float(r) * 9.094947017729282e-13f);
}

__device__ __forceinline__ float blk_rcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float blk_ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// One partner j of trial m beyond 2 sigma of both positions (the bulk of the
// all-pairs sum): u(new) - u(old) of Debye-Hueckel + LJ in difference form,
// r_n^2 - r_o^2 exact from integers (cubic box), the DH ratio as
// (expm1(-kappa dr) - dr/r_o) / (1 + dr/r_o); rounding scales with the
// difference. Reciprocal and exponential use the approximate SFU forms: their
// ~2 ulp enter only as relative errors of the (small) difference. Returns
// false (and nothing) for pairs that need the careful path.
__device__ __forceinline__ bool blk_far(const Move &m, int4 pj, int tj, const SysDesc &d, float kl2e, float &acc) {
    const float r2n = dist2(pj, m.hn[0], m.hn[1], m.hn[2], d);
    const float r2o = dist2(pj, m.ho[0], m.ho[1], m.ho[2], d);
    const int t = d.uniform_types ? 0 : m.ti * d.n_types + tj;
    const float s2 = d.s2[t];
    const float near2 = 4.0f * s2;
    if (r2n < near2 || r2o < near2) return false;
    long long S = 0;
    {
        const int pjv[3] = {pj.x, pj.y, pj.z};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const long long dn = (int)((uint32_t)pjv[a] - (uint32_t)m.hn[a]);
            const long long dO = (int)((uint32_t)pjv[a] - (uint32_t)m.ho[a]);
            S += (dn - dO) * (dn + dO);
        }
    }
    const float dR2 = i64_to_float(S) * d.s32sq;
    const float rio = rsqrt_nr(r2o), rin = rsqrt_nr(r2n);
    const float ro = r2o * rio, rn = r2n * rin;
    const float dr = dR2 * blk_rcp(rn + ro);
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
    const float qj = __int_as_float(pj.w);
    const float uo = m.q * qj * d.lB * blk_ex2(kl2e * ro) * rio;
    const float ddh = uo * (em1 - tt) * blk_rcp(1.0f + tt);
    const float xo = s2 * rio * rio;
    const float xo3 = xo * xo * xo;
    const float tau = -dR2 * (rin * rin);
    const float t3m1 = tau * fmaf(tau, tau + 3.0f, 3.0f);
    acc += fmaf(d.eps4[t] * xo3, t3m1 * fmaf(xo3, t3m1 + 2.0f, -1.0f), ddh);
    return true;
}

// dU contribution of one partner (high words pj with charge bits, type tj,
// extension e) for trial m, as a df number.
__device__ __forceinline__ df blk_pair(const Move &m, int4 pj, int tj, const short4 *e, const SysDesc &d) {
    float a = 0.0f;
    df ad = {0.0f, 0.0f};
    pair_candidate<MODEL_DHLJ>(m, pj, tj, e, d, a, ad);
    return df_add_f(ad, a);
}

// Warp-aggregated append to the near-pair queue; true = the queue is full and
// the lane evaluates its pair in place.
__device__ __forceinline__ bool blk_enqueue(const BlkSmem &s, bool near, uint32_t code) {
    const unsigned active = __activemask();
    const unsigned m = __ballot_sync(active, near);
    if (!m) return false;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&s.info[2], __popc(m));
    base = __shfl_sync(active, base, leader);
    if (!near) return false;
    const int slot = base + __popc(m & ((1u << lane) - 1u));
    if (slot < kBlkQueue) {
        s.queue[slot] = code;
        return false;
    }
    return true;
}

// One cluster of C CTAs per system; system members[blockIdx.x / C] of descs
// (members == nullptr: blockIdx.x / C). C == 1 runs without a cluster.
template <bool SLICE, bool CLUSTER>
__global__ void __launch_bounds__(kBlkThreads, 1) dh_block_kernel(const SysDesc *__restrict__ descs,
                                                                  const int *__restrict__ members, int C,
                                                                  int64_t end) {
    extern __shared__ __align__(16) unsigned char blk_smem_raw[];
    __shared__ __align__(16) SysDesc sd;
    const int sys = members ? members[blockIdx.x / C] : (int)(blockIdx.x / C);
    // launch-shape check: the partial sums are read from C CTAs of this
    // cluster; anything else records an error and touches no other CTA
    if (CLUSTER ? (int)blk_cluster_size() != C : C != 1) {
        if (threadIdx.x == 0) atomicOr(&descs[sys].sc->error, kErrLaunch);
        return;
    }
    const int rank = CLUSTER ? (int)blk_cluster_rank() : 0;
    load_desc(sd, descs + sys);
    const SysDesc &d = sd;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
    const int N = d.N;
    const int ns_full = (N + C - 1) / C;
    const int j0 = min(rank * ns_full, N), j1 = min(j0 + ns_full, N), ns = j1 - j0;
    BlkSmem s = blk_carve(blk_smem_raw, ns_full, SLICE);
    SysScalars *sc = d.sc;
    int64_t cur = sc->cursor;
    const int64_t stop = min(end, sc->n_trials);
    if (SLICE)
        for (int jj = tid; jj < ns; jj += blockDim.x) {
            s.spos[jj] = d.pos4[j0 + jj];
            s.sext[jj] = d.pos_ext[j0 + jj];
            s.stype[jj] = d.ptype[j0 + jj];
        }
    df U = {sc->u_hi, sc->u_lo};
    df Ut = {sc->utot_hi, sc->utot_lo};
    int64_t nacc = sc->n_accepted;
    int err = 0;
    if (CLUSTER) blk_cluster_barrier();
    else __syncthreads();
    int64_t nblock = 0;
    while (cur < stop) {
        const int kb = (int)((stop - cur) < (int64_t)kBlkTrials ? (stop - cur) : (int64_t)kBlkTrials);
        const int slot = (int)(nblock & 1);
        // ---- set up the block's trials (old coordinates: the block start)
        if (tid < kb) {
            const Trial tr = d.trials[cur + tid];
            int64_t xo[3], xn[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                xo[a] = d.pos64[3 * tr.idx + a];
                xn[a] = (int64_t)((uint64_t)xo[a] + (uint64_t)tr.d[a]);
            }
            Move m;
            move_setup(m, tr.idx, xo, xn, __int_as_float(d.pos4[tr.idx].w), d.ptype[tr.idx], d);
            s.mv[tid] = m;
            df thr = {tr.thr_hi, tr.thr_lo};
            if (d.kT != 1.0f) thr = dfm_f(thr, d.kT);
            s.thr[tid] = make_float2(thr.hi, thr.lo);
        }
        if (tid < kBlkTrials) s.fix[tid] = 0ull;
        if (tid == 0) s.info[2] = 0;
        __syncthreads();
        if (tid < kb) {
            uint32_t c = 0;
            const int i = s.mv[tid].i;
            for (int a = 0; a < tid; a++)
                if (s.mv[a].i == i) c |= 1u << a;
            s.col[tid] = c;
        }
        // ---- corrections c(a, m), a < m (identical in every CTA of a cluster)
        for (int e = tid; e < kBlkTrials * kBlkTrials; e += blockDim.x) {
            const int a = e / kBlkTrials, m = e - a * kBlkTrials;
            float2 out = make_float2(0.0f, 0.0f);
            if (a < m && m < kb && s.mv[a].i != s.mv[m].i) {
                const Move &A = s.mv[a];
                const Move &Mm = s.mv[m];
                const int4 pn = make_int4(A.hn[0], A.hn[1], A.hn[2], __float_as_int(A.q));
                const int4 po = make_int4(A.ho[0], A.ho[1], A.ho[2], __float_as_int(A.q));
                const short4 en = make_short4((short)A.en[0], (short)A.en[1], (short)A.en[2], 0);
                const short4 eo = make_short4((short)A.eo[0], (short)A.eo[1], (short)A.eo[2], 0);
                const df c = df_add(blk_pair(Mm, pn, A.ti, &en, d), df_neg(blk_pair(Mm, po, A.ti, &eo, d)));
                out = make_float2(c.hi, c.lo);
            }
            s.corr[e] = out;
        }
        // ---- base sums: warp w takes trials w, w + nwarp, ... over this slice
        const float kl2e = -d.kappa * 1.4426950408889634f;   // exp(-kappa r) = 2^(kl2e r)
        for (int m = warp; m < kb; m += nwarp) {
            const Move mv = s.mv[m];
            float accf = 0.0f, accf2 = 0.0f;
            df accd = {0.0f, 0.0f};
            // two partners per iteration: independent chains for the scheduler
            for (int jj = lane; jj < ns; jj += 64) {
                const int ja = j0 + jj, jb = ja + 32;
                const bool vb = jj + 32 < ns;
                const int4 pa = SLICE ? s.spos[jj] : d.pos4[ja];
                const int ta = SLICE ? s.stype[jj] : d.ptype[ja];
                const int4 pb = vb ? (SLICE ? s.spos[jj + 32] : d.pos4[jb]) : pa;
                const int tb = vb ? (SLICE ? s.stype[jj + 32] : d.ptype[jb]) : ta;
                // pairs inside 2 sigma go to the queue (evaluated densely below)
                const bool na = ja != mv.i && !blk_far(mv, pa, ta, d, kl2e, accf);
                const bool nb = vb && jb != mv.i && !blk_far(mv, pb, tb, d, kl2e, accf2);
                if (blk_enqueue(s, na, ((uint32_t)m << 24) | (uint32_t)jj))
                    pair_candidate<MODEL_DHLJ>(mv, pa, ta, SLICE ? &s.sext[jj] : &d.pos_ext[ja], d, accf, accd);
                if (blk_enqueue(s, nb, ((uint32_t)m << 24) | (uint32_t)(jj + 32)))
                    pair_candidate<MODEL_DHLJ>(mv, pb, tb, SLICE ? &s.sext[jj + 32] : &d.pos_ext[jb], d, accf2,
                                               accd);
            }
            const df p = warp_sum_df(df_add_f(df_add_f(accd, accf), accf2));
            if (lane == 0) s.part[slot * kBlkTrials + m] = make_float2(p.hi, p.lo);
        }
        __syncthreads();
        {
            const int nq = min(s.info[2], kBlkQueue);
            for (int e = tid; e < nq; e += blockDim.x) {
                const uint32_t q = s.queue[e];
                const int m = (int)(q >> 24), jj = (int)(q & 0xFFFFFF);
                const int j = j0 + jj;
                const int4 pj = SLICE ? s.spos[jj] : d.pos4[j];
                const int tj = SLICE ? s.stype[jj] : d.ptype[j];
                const df v = blk_pair(s.mv[m], pj, tj, SLICE ? &s.sext[jj] : &d.pos_ext[j], d);
                atomicAdd(&s.fix[m], blk_to_fix(v));
            }
        }
        __syncthreads();
        if (tid < kb) {
            const float2 p = s.part[slot * kBlkTrials + tid];
            const df v = df_add(df{p.x, p.y}, blk_from_fix(s.fix[tid]));
            s.part[slot * kBlkTrials + tid] = make_float2(v.hi, v.lo);
        }
        if (CLUSTER) blk_cluster_barrier();
        else __syncthreads();
        // ---- resolve the block in order (warp 0; lane m = trial m)
        if (warp == 0) {
            df S = {0.0f, 0.0f};
            if (lane < kb) {
                for (int r = 0; r < C; r++) {
                    const float2 p = CLUSTER ? blk_ld_cluster(&s.part[slot * kBlkTrials + lane], (unsigned)r)
                                             : s.part[slot * kBlkTrials + lane];
                    S = df_add(S, df{p.x, p.y});
                }
            }
            const uint32_t colm = lane < kb ? s.col[lane] : 0u;
            const float2 th = lane < kb ? s.thr[lane] : make_float2(0.0f, 0.0f);
            uint32_t accm = 0;
            int done = kb;
            for (int a = 0; a < kb; a++) {
                const bool coll = __shfl_sync(0xffffffffu, (colm & accm) != 0u ? 1 : 0, a) != 0;
                if (coll) {
                    done = a;
                    break;
                }
                const float dh = __shfl_sync(0xffffffffu, S.hi, a);
                const float dl = __shfl_sync(0xffffffffu, S.lo, a);
                const float t_hi = __shfl_sync(0xffffffffu, th.x, a);
                const float t_lo = __shfl_sync(0xffffffffu, th.y, a);
                const df du = {dh, dl};
                const bool nan = !(dh == dh);
                // Movebase::metropolis (move.h:567-573): reject iff dU > kT (-ln u);
                // a NaN dU compares false there: accepted
                const bool acc = nan || !df_gt(du, df{t_hi, t_lo});
                if (nan) err |= kErrNonFinite;
                if (lane == 0 && rank == 0 && d.log_trials) {
                    d.trial_du[cur + a] = make_float2(dh, dl);
                    d.trial_acc[cur + a] = acc ? 1 : 0;
                }
                if (acc) {
                    accm |= 1u << a;
                    U = df_add(U, du);
                    Ut = df_add(Ut, du);
                    nacc++;
                    if (lane > a && lane < kb) {
                        const float2 c = s.corr[a * kBlkTrials + lane];
                        S = df_add(S, df{c.x, c.y});
                    }
                }
            }
            if (lane == 0) {
                s.info[0] = done;
                s.info[1] = (int)accm;
            }
        }
        __syncthreads();
        // ---- apply the accepted moves (at most one per particle per block)
        const int done = s.info[0];
        const uint32_t accm = (uint32_t)s.info[1];
        if (tid < done && (accm >> tid) & 1u) {
            const Move &m = s.mv[tid];
            const int4 rec = make_int4(m.hn[0], m.hn[1], m.hn[2], __float_as_int(m.q));
            const short4 ext = make_short4((short)m.en[0], (short)m.en[1], (short)m.en[2], 0);
            // every CTA writes the same values to the master arrays; each reads
            // them only after its own write
            d.pos64[3 * m.i + 0] = m.xn[0];
            d.pos64[3 * m.i + 1] = m.xn[1];
            d.pos64[3 * m.i + 2] = m.xn[2];
            d.pos4[m.i] = rec;
            d.pos_ext[m.i] = ext;
            if (SLICE && m.i >= j0 && m.i < j1) {
                s.spos[m.i - j0] = rec;
                s.sext[m.i - j0] = ext;
            }
        }
        cur += done;
        nblock++;
        __syncthreads();
    }
    if (rank == 0 && tid == 0) {
        sc->cursor = cur;
        sc->u_hi = U.hi;
        sc->u_lo = U.lo;
        sc->utot_hi = Ut.hi;
        sc->utot_lo = Ut.lo;
        sc->n_accepted = nacc;
        sc->error |= err;
    }
    if (CLUSTER) blk_cluster_barrier();   // no CTA leaves while another may read its shared memory
}

}  // namespace fg
