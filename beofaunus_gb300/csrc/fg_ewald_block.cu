// Ewald + WCA sweeps in blocks of trials (one CTA per system).
//
// Included by fg_api.cu after fg_kernels.cu (one translation unit).
//
// Same idea as the Debye-Hueckel block kernel (fg_dh_block.cu): a block of up
// to 32 trials is evaluated against the configuration at the block start, and
// one warp resolves it in order with exact corrections for the trials it
// accepts. For Ewald the correction of trial m after an accepted trial a has
// three parts:
//   real space   [u(n_m,n_a) - u(o_m,n_a)] - [u(n_m,o_a) - u(o_m,o_a)]
//   surface      2 c dM_a . dM_m                 (E_surf = c |M|^2)
//   reciprocal   sum_k A'_k 2 Re(conj(D_a,k) D_m,k)
// with D_m,k = q e^{ik.r_old}(e^{ik.d} - 1) the same increment the energy uses.
// The reciprocal parts of all pairs of the block form a 32 x 32 Gram matrix
// over k of the trials' increments; it is accumulated in 4 x 4 register tiles
// while the increments stream through shared memory in chunks of k-vectors.
// Q(k) itself stays the exact fixed-point sum: after the block each accepted
// trial's integer contributions are applied in order. A trial whose particle
// an accepted trial of the block already moved ends the block, and so does
// the accepted trial that makes a Q(k) rebuild due. In a batch that fills the
// GPU the CTA then rebuilds its system's Q(k) from scratch in place
// (eb_rebuild) and carries on, so one launch runs every system's whole
// stream; a system running alone exits instead and leaves the rebuild to the
// rebuild kernel, which spreads it over all SMs.
namespace fg {

constexpr int kEbTrials = 32;
constexpr int kEbThreads = 512;
constexpr int kEbKc = 128;   // scratch buffer rows (of 32 float2)
constexpr int kEbMaxCluster = 16;
constexpr int kEbGramN = 6 * 32 * 4;   // floats of one Gram accumulator set (eb_gram_regs' layout)

struct EbSmem {
    Smem b;          // sc_tab, qfix, kpack, cells as in the one-trial kernel; kvec here holds
                     // {A'_k, Q(k) as float (re, im), sqrt(A'_k)}: k itself comes from the integer n
    Move *mv;        // [32]
    float2 *thr;     // [32] threshold (df, times kT)
    uint32_t *col;   // [32] earlier trials on the same particle
    int *info;       // [8] resolved count, accepted mask, rebuild
    float2 *partR;   // [32] real-space base (df)
    float2 *kbase;   // [32] reciprocal base (df)
    float2 *corr;    // [32][32] real-space + surface corrections (df)
    float *G;        // [32][32] reciprocal cross terms
    float2 *delta;   // [kEbKc x 32] scratch: real-space queues and k-space trial records, then
                     // the Gram and reciprocal-base partials, then the commit's axis tables
    float2 *Mdf;     // [3] surface dipole M (df)
    // cluster only (written by the other CTAs into the leader's copy): per
    // rank its Gram sums [C][kEbGramN] and reciprocal bases [C][32], per trial
    // and part the real-space partial sums [32][parts]
    float *xgram;
    float2 *xkbase;
    float2 *xreal;
};

// Shared memory of one CTA holding Kl k-vectors, in a cluster of C CTAs.
__host__ __device__ inline size_t eb_layout(int N, int Kl, int ncell, bool cells, int C, size_t off[19]) {
    size_t b = 256 * 8 + 32 * 8;            // sc_tab, red
    off[0] = b; b += (size_t)Kl * 16;       // kvec
    off[1] = b; b += (size_t)Kl * 16;       // qfix
    off[2] = b; b = align16(b + (size_t)Kl * 4);           // kpack
    off[3] = b; if (cells) b = align16(b + (size_t)ncell * 4);   // ccount
    off[4] = b; if (cells) b = align16(b + (size_t)N * 4);       // pcs
    off[5] = b; b = align16(b + sizeof(Move) * kEbTrials);      // mv
    off[6] = b; b = align16(b + 8 * kEbTrials);                 // thr
    off[7] = b; b = align16(b + 4 * kEbTrials);                 // col
    off[8] = b; b = align16(b + 4 * 8);                         // info
    off[9] = b; b = align16(b + 8 * kEbTrials);                 // partR
    off[10] = b; b = align16(b + 8 * kEbTrials);                // kbase
    off[11] = b; b = align16(b + 8 * kEbTrials * kEbTrials);    // corr
    off[12] = b; b = align16(b + 4 * kEbTrials * kEbTrials);    // G
    off[13] = b; b = align16(b + 8 * kEbKc * kEbTrials);        // delta
    off[14] = b; b = align16(b + 8 * 3);                        // Mdf
    const int cx = C > 1 ? C : 0;
    off[15] = b; b = align16(b + (size_t)4 * kEbGramN * cx);    // xgram
    off[16] = b; b = align16(b + (size_t)8 * kEbTrials * cx);   // xkbase
    off[17] = b; b = align16(b + (size_t)8 * kEbTrials * (C > 1 ? (C + 1) / 2 : 0));   // xreal
    off[18] = b;
    return b;
}

__device__ inline EbSmem eb_carve(char *base, const SysDesc &d, bool cells) {
    size_t off[19];
    const int ncell = d.nc[0] * d.nc[1] * d.nc[2];
    eb_layout(d.N, d.eb_kmax, ncell, cells, d.eb_ctas, off);
    EbSmem s;
    s.b.sc_tab = (float2 *)base;
    s.b.red = (float2 *)(base + 256 * 8);
    s.b.kvec = (float4 *)(base + off[0]);
    s.b.qfix = (longlong2 *)(base + off[1]);
    s.b.qf = nullptr;
    s.b.ktab = nullptr;
    s.b.kpack = (uint32_t *)(base + off[2]);
    s.b.pos = nullptr;
    s.b.pos_ext = nullptr;
    s.b.ptype = nullptr;
    s.b.ccount = (int *)(base + off[3]);
    s.b.pcs = (uint32_t *)(base + off[4]);
    s.mv = (Move *)(base + off[5]);
    s.thr = (float2 *)(base + off[6]);
    s.col = (uint32_t *)(base + off[7]);
    s.info = (int *)(base + off[8]);
    s.partR = (float2 *)(base + off[9]);
    s.kbase = (float2 *)(base + off[10]);
    s.corr = (float2 *)(base + off[11]);
    s.G = (float *)(base + off[12]);
    s.delta = (float2 *)(base + off[13]);
    s.Mdf = (float2 *)(base + off[14]);
    s.xgram = (float *)(base + off[15]);
    s.xkbase = (float2 *)(base + off[16]);
    s.xreal = (float2 *)(base + off[17]);
    return s;
}

// Real-space sum of one trial by one warp: every stencil cell (cell list) or
// every particle (no cell list), lanes over the slots.
// One k-step of the Gram matrix on the tensor cores: components c = the real
// and imaginary parts of 4 consecutive k-vectors of X = sqrt(A') D. mma.sync
// m16n8k8 TF32 with the three-product split (hi hi + hi lo + lo hi, each
// operand split into a TF32 high part and the TF32 rounding of the rest)
// keeps FP32-level accuracy. Lane (gq = lane / 4, gt = lane % 4) holds the
// components gt and gt + 4 of trials gq + 8 r; these are the A fragments of
// the two 16-row tiles and, G being X X^T, the B fragments of the four
// 8-column tiles. Accumulated tiles (row tile, column tile): (0,0) (0,1)
// (0,2) (0,3) (1,2) (1,3), every pair a < m lies in one of them.
__device__ __forceinline__ uint32_t eb_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ void eb_mma(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ void eb_gram_regs(const float xf[4][2], float gc[6][4]) {
    uint32_t hi[4][2], lo[4][2];
#pragma unroll
    for (int r = 0; r < 4; r++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
            hi[r][h] = eb_tf32(xf[r][h]);
            lo[r][h] = eb_tf32(xf[r][h] - __uint_as_float(hi[r][h]));
        }
#pragma unroll
    for (int t = 0; t < 6; t++) {
        const int mi = t < 4 ? 0 : 1, nj = t < 4 ? t : t - 2;
        const uint32_t ah[4] = {hi[2 * mi][0], hi[2 * mi + 1][0], hi[2 * mi][1], hi[2 * mi + 1][1]};
        const uint32_t al[4] = {lo[2 * mi][0], lo[2 * mi + 1][0], lo[2 * mi][1], lo[2 * mi + 1][1]};
        eb_mma(gc[t], al, hi[nj][0], hi[nj][1]);
        eb_mma(gc[t], ah, lo[nj][0], lo[nj][1]);
        eb_mma(gc[t], ah, hi[nj][0], hi[nj][1]);
    }
}

// Barrier 1 over the block's warps 1.. (nthreads = blockDim - 32 threads).
__device__ __forceinline__ void eb_qbar(int nthreads) {
    asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

// Stores into CTA `rank`'s copy of a shared-memory variable (the cluster's
// distributed shared memory).
__device__ __forceinline__ uint32_t eb_remote(const void *p, unsigned rank) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    return ra;
}
__device__ __forceinline__ void eb_st_remote(float2 *p, unsigned rank, float2 v) {
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(eb_remote(p, rank)), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ void eb_st_remote(float *p, unsigned rank, float v) {
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(eb_remote(p, rank)), "f"(v) : "memory");
}
__device__ __forceinline__ void eb_st_remote(int *p, unsigned rank, int v) {
    asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(eb_remote(p, rank)), "r"(v) : "memory");
}

// Real-space base of one trial by one warp (or part `part` of `nparts`: the
// candidate batches part, part + nparts, ...). Candidates (cell stencil, or all
// particles) are screened by distance first: only those that may lie within
// reach2 of the old or the new position (all particles: either distance; cell
// stencil: the distance to the step's midpoint against reach + |d|/2) enter a
// 32-entry warp queue in shared memory (qp, qm), which is evaluated with all
// lanes busy when the next batch would overflow it. Skipped candidates
// contribute exactly zero (every pair term is zero beyond reach2), so the sum
// is that of the full loop, in another order.
template <bool CELLS>
__device__ __forceinline__ void eb_flush(int qn, const int4 *qp, const int2 *qm, const Move &m, const SysDesc &d,
                                         float &accf, df &accd) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    if (lane < qn) {
        const int2 e = qm[lane];
        pair_candidate<MODEL_EWALD>(m, qp[lane], e.y, (CELLS ? d.cell_ext : d.pos_ext) + e.x, d, accf, accd);
    }
    __syncwarp();
}
template <bool CELLS>
__device__ __forceinline__ void eb_push(bool f, int4 pos, int idx, int t, int &qn, int4 *qp, int2 *qm,
                                        const Move &m, const SysDesc &d, float &accf, df &accd) {
    const int lane = threadIdx.x & 31;
    const uint32_t mask = __ballot_sync(0xffffffffu, f);
    const int c = __popc(mask);
    if (qn + c > 32) {
        eb_flush<CELLS>(qn, qp, qm, m, d, accf, accd);
        qn = 0;
    }
    if (f) {
        const int r = qn + __popc(mask & ((1u << lane) - 1u));
        qp[r] = pos;
        qm[r] = make_int2(idx, t);
    }
    qn += c;
}
__device__ __forceinline__ bool eb_in_reach(int4 p, const Move &m, const SysDesc &d) {
    return dist2(p, m.hn[0], m.hn[1], m.hn[2], d) <= d.reach2 || dist2(p, m.ho[0], m.ho[1], m.ho[2], d) <= d.reach2;
}

template <bool CELLS>
__device__ __forceinline__ void eb_pairs_warp(const Move &m, const SysDesc &d, const Smem &s, int4 *qp, int2 *qm,
                                              int part, int nparts, float &accf, df &accd) {
    const int lane = threadIdx.x & 31;
    int qn = 0;
    if (!CELLS) {
        for (int b = 32 * part; b < d.N; b += 32 * nparts) {   // warp-uniform trip count
            const int j = b + lane;
            const bool v = j < d.N && j != m.i;
            const int4 p = v ? d.pos4[j] : make_int4(0, 0, 0, 0);
            const int t = v ? d.ptype[j] : 0;
            eb_push<CELLS>(v && eb_in_reach(p, m, d), p, j, t, qn, qp, qm, m, d, accf, accd);
        }
        eb_flush<CELLS>(qn, qp, qm, m, d, accf, accd);
        return;
    }
    // The stencil: the cells around the old cell, widened by one along each
    // axis where the particle changed cells (at most 4 x 4 x 4). Lane c (and
    // c + 32) takes stencil cell c: it drops the cell when no point of the
    // cell box lies within reach of the old or the new position, so that the
    // cell's particles cannot contribute, and the warp's prefix sum over the
    // remaining cells' counts flattens their slots into one candidate list,
    // which the warp then screens 32 candidates at a time with all lanes busy.
    int co[3], cn[3], lo[3], len[3];
    co[0] = m.co % d.nc[0]; co[1] = (m.co / d.nc[0]) % d.nc[1]; co[2] = m.co / (d.nc[0] * d.nc[1]);
    cn[0] = m.cn % d.nc[0]; cn[1] = (m.cn / d.nc[0]) % d.nc[1]; cn[2] = m.cn / (d.nc[0] * d.nc[1]);
#pragma unroll
    for (int a = 0; a < 3; a++) {
        int delta = cn[a] - co[a];
        if (delta > 1) delta -= d.nc[a];
        if (delta < -1) delta += d.nc[a];
        if ((delta > 1 || delta < -1) && lane == 0) atomicOr(&d.sc->error, kErrStencil);
        lo[a] = co[a] + min(delta, 0) - 1;
        len[a] = 3 + (delta != 0 ? 1 : 0);
    }
    const int ncell = len[0] * len[1] * len[2];   // <= 64
    // reach of a cell box: squared distance (Angstrom^2) from the old and the
    // new position, on unwrapped coordinates u = h + 2^31 (the new one as the
    // old plus the minimum-image step, so that both lie on the stencil's side
    // of the box edge); a small margin covers the float rounding of the box
    // bounds (units of 2^32 / L carry ~2^8 units of rounding here)
    const float reach2m = d.reach2 * 1.0001f + 1e-3f;
    float uo[3], un[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        uo[a] = (float)((uint32_t)m.ho[a] + 0x80000000u);
        un[a] = uo[a] + (float)(int)(m.hn[a] - m.ho[a]);
    }
    int cidv[2], cntv[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int c = lane + 32 * h;
        cidv[h] = 0;
        cntv[h] = 0;
        if (c < ncell) {
            const int i0 = c % len[0], i1 = (c / len[0]) % len[1], i2 = c / (len[0] * len[1]);
            const int cu[3] = {lo[0] + i0, lo[1] + i1, lo[2] + i2};
            float d2o = 0.0f, d2n = 0.0f;
            int w[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float W = 4294967296.0f / (float)d.nc[a];
                const float A = (float)cu[a] * W, B = A + W;
                const float xo = fmaxf(fmaxf(A - uo[a], uo[a] - B), 0.0f) * d.s32[a];
                const float xn = fmaxf(fmaxf(A - un[a], un[a] - B), 0.0f) * d.s32[a];
                d2o = fmaf(xo, xo, d2o);
                d2n = fmaf(xn, xn, d2n);
                w[a] = cu[a] + (cu[a] < 0 ? d.nc[a] : 0) - (cu[a] >= d.nc[a] ? d.nc[a] : 0);
            }
            cidv[h] = (w[2] * d.nc[1] + w[1]) * d.nc[0] + w[0];
            if (fminf(d2o, d2n) <= reach2m) cntv[h] = s.ccount[cidv[h]];
        }
    }
    // inclusive prefix sums of the two halves; start = exclusive
    int inc0 = cntv[0], inc1 = cntv[1];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v0 = __shfl_up_sync(0xffffffffu, inc0, o), v1 = __shfl_up_sync(0xffffffffu, inc1, o);
        if (lane >= o) {
            inc0 += v0;
            inc1 += v1;
        }
    }
    const int tot0 = __shfl_sync(0xffffffffu, inc0, 31);
    const int st0 = inc0 - cntv[0], st1 = tot0 + inc1 - cntv[1];
    const int total = tot0 + __shfl_sync(0xffffffffu, inc1, 31);
    // screening against the midpoint hm of the step: a partner within reach
    // of the old or the new position lies within reach + |d|/2 of hm
    const int hm[3] = {m.ho[0] + ((int)(m.hn[0] - m.ho[0]) >> 1), m.ho[1] + ((int)(m.hn[1] - m.ho[1]) >> 1),
                       m.ho[2] + ((int)(m.hn[2] - m.ho[2]) >> 1)};
    const float hd = 0.5f * sqrtf(fmaf(m.dxf[0], m.dxf[0], fmaf(m.dxf[1], m.dxf[1], m.dxf[2] * m.dxf[2])));
    const float rm = sqrtf(reach2m) + hd + 1e-3f, rm2 = rm * rm;
    int c = 0;   // warp-uniform: the cell holding candidate b
    for (int b = 32 * part; b < total; b += 32 * nparts) {
        // the first stencil cell whose slots reach past b
        while (true) {
            const int e = (c < 32 ? __shfl_sync(0xffffffffu, st0, c) + __shfl_sync(0xffffffffu, cntv[0], c)
                                  : __shfl_sync(0xffffffffu, st1, c - 32) + __shfl_sync(0xffffffffu, cntv[1], c - 32));
            if (e > b) break;
            c++;
        }
        const int g = b + lane;
        int mc = c;
        for (int cc = c + 1; cc < ncell; cc++) {   // warp-uniform
            const int sc0 = cc < 32 ? __shfl_sync(0xffffffffu, st0, cc) : __shfl_sync(0xffffffffu, st1, cc - 32);
            if (sc0 > b + 31) break;
            if (sc0 <= g) mc = cc;
        }
        const int sA = __shfl_sync(0xffffffffu, st0, mc & 31), sB = __shfl_sync(0xffffffffu, st1, mc & 31);
        const int cA = __shfl_sync(0xffffffffu, cidv[0], mc & 31), cB = __shfl_sync(0xffffffffu, cidv[1], mc & 31);
        const int cid = mc < 32 ? cA : cB, slot = g - (mc < 32 ? sA : sB);
        const bool in = g < total;
        const int idx = cid * d.cap + slot;
        const int pid = in ? d.cell_pid[idx] : -1;
        const int4 pos = in ? d.cell_pos[idx] : make_int4(0, 0, 0, 0);
        const bool v = pid >= 0 && (pid & 0xFFFFFF) != m.i && dist2(pos, hm[0], hm[1], hm[2], d) <= rm2;
        eb_push<CELLS>(v, pos, idx, pid >> 24, qn, qp, qm, m, d, accf, accd);
    }
    eb_flush<CELLS>(qn, qp, qm, m, d, accf, accd);
}

// dU of trial m from one partner at high words p (charge bits in .w), type t,
// extension e, as a df number.
__device__ __forceinline__ df eb_pair(const Move &m, int4 p, int t, const short4 *e, const SysDesc &d) {
    float a = 0.0f;
    df ad = {0.0f, 0.0f};
    pair_candidate<MODEL_EWALD>(m, p, t, e, d, a, ad);
    return df_add_f(ad, a);
}

// updateAllComplexNumbers (ewald.h:388-415) inside the sweep, every
// update_frequency accepted trials (NonbondedEwald::update, ewald.h:633-640):
// Q(k) from scratch as the exact sum of every particle's integer
// contributions, compared with the running Q(k) in shared memory and adopted.
// The two agree bit for bit unless the device misbehaved (a contribution is a
// deterministic function of the fixed-point position), so the energy
// correction is zero; a difference is recorded (kErrQkMismatch where the
// system verifies) and its energy is added to the running sums, as the
// reference adds the drift it removes.
//   work split: thread t owns items t, t + blockDim, ... of the system's
//   rebuild list (rb_items: up to kRbLen values n of one (nx, ny) column, each
//   giving the k-vectors +n and -n). Per particle it forms w once (qk_w) and
//   per n the four rounded products a, r, b, c of w e_z(n) (qk_rint_bits),
//   whose sums give both contributions: (a - r, b + c) to +n and, e_z(-n)
//   being the conjugate and the rounding symmetric, (a + r, c - b) to -n;
//   term by term these are qk_term_bits' values. Particles pass through the
//   increment buffer in stages of 64 with their axis tables (8 threads build
//   one particle's table: e_x(0..kcc), e_y(-kcc..kcc), e_z(0..kcc)), stored
//   for pairs of particles so that one 16-byte load serves two; the four
//   sums run in 32 bits over a stage, then in int64 registers. The same items
//   carry the per-block Q(k) update (eb_commit_qk).
// All threads call it (block-uniform). Returns the energy correction
// (valid in thread 0) and whether any Q(k) differed.
constexpr int kRbLen = 4;
__host__ __device__ __forceinline__ int rb_tab_len(int kcc) { return 4 * kcc + 3; }
// entry t of the rebuild's axis tables: the e_x and e_y parts of qk_tab_len's
// layout, then e_z for n >= 0 only
__device__ __forceinline__ float2 rb_tab_entry(int t, int kcc, const int h[3], const float2 *__restrict__ tab) {
    return qk_tab_entry(t <= 3 * kcc + 1 ? t : t + kcc, kcc, h, tab);
}
// One stage of the rebuild for this thread's item: np particle pairs, whose
// axis tables sit as float4 {e_2p(t), e_2p+1(t)} at tab[p * T + t] (one
// 16-byte load gives an entry of both particles) and whose charges are
// q2[p]. The four sums carry 2 np kQkMagicBits (a padding particle has
// charge 0 and zero tables and adds exactly that).
template <int L>
__device__ __forceinline__ void rb_pass(const float4 *tab, int T, const float2 *q2, int np, int ix, int iy, int iz,
                                        unsigned sa[kRbLen], unsigned sr[kRbLen], unsigned sb[kRbLen],
                                        unsigned sc[kRbLen]) {
    for (int p = 0; p < np; p++) {
        const float4 *e = tab + p * T;
        const float2 q = q2[p];
        const float4 ex = e[ix], ey = e[iy];
        const float2 w0 = qk_w(q.x, make_float2(ex.x, ex.y), make_float2(ey.x, ey.y));
        const float2 w1 = qk_w(q.y, make_float2(ex.z, ex.w), make_float2(ey.z, ey.w));
#pragma unroll
        for (int u = 0; u < L; u++) {
            const float4 z = e[iz + u];
            sa[u] += qk_rint_bits(w0.x, z.x) + qk_rint_bits(w1.x, z.z);
            sr[u] += qk_rint_bits(w0.y, z.y) + qk_rint_bits(w1.y, z.w);
            sb[u] += qk_rint_bits(w0.x, z.y) + qk_rint_bits(w1.x, z.w);
            sc[u] += qk_rint_bits(w0.y, z.x) + qk_rint_bits(w1.y, z.z);
        }
    }
}
// Compare one rebuilt Q(k) (its total in the k-vector table's slot, see
// eb_rebuild) with the running value and adopt it; energy of the difference
// into e; the slot gets back its {A', Q as float, sqrt A'} from the k-vector
// array in global memory.
__device__ __forceinline__ void rb_adopt(const SysDesc &d, const EbSmem &s, int k, df &e, int &bad) {
    const longlong2 qn = reinterpret_cast<const longlong2 *>(s.b.kvec)[k];
    const longlong2 qo = s.b.qfix[k];
    const float A = d.kvec[k].w;
    const float2 fn = q_to_float(qn);
    if (qo.x != qn.x || qo.y != qn.y) {
        bad = 1;
        const float2 fo = q_to_float(qo);
        const float dre = fix28_to_float(qn.x - qo.x), dim = fix28_to_float(qn.y - qo.y);
        e = df_add_f(e, A * fmaf(dre, fo.x + fn.x, dim * (fo.y + fn.y)));
        s.b.qfix[k] = qn;
    }
    s.b.kvec[k] = make_float4(A, fn.x, fn.y, sqrtf(A));
}
__device__ __forceinline__ void rb_add(const EbSmem &s, int k, long long x, long long y) {
    longlong2 *t = reinterpret_cast<longlong2 *>(s.b.kvec) + k;
    longlong2 v = *t;
    v.x += x;
    v.y += y;
    *t = v;
}
// The int64 totals of the rebuilt Q(k) live in the k-vector table's own
// 16-byte slots (kvec[k], free while the rebuild runs: nothing else reads it
// until rb_adopt restores it), each owned by the thread of its item, so the
// thread's registers hold only the 32-bit sums of a stage.
__device__ __noinline__ bool eb_rebuild(const SysDesc &d, const EbSmem &s, df &corr) {
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31;
    const int kcc = d.kcc, T = rb_tab_len(kcc);
    // the increment buffer holds the stage's tables (pairs of particles) plus
    // kRbLen entries of headroom for the unused tail reads of rb_pass
    float4 *tab = reinterpret_cast<float4 *>(s.delta);
    const int npair = min(kEbThreads / 16, (kEbKc * kEbTrials / 2 - kRbLen) / T), stage = 2 * npair;
    float2 *q2 = reinterpret_cast<float2 *>(s.G);   // [npair], free between blocks
    const int shift = d.qk_shift;
    df e = {0.0f, 0.0f};
    int bad = 0;
    __syncthreads();   // every thread is past its last read of kvec
    for (int r0 = 0; r0 < d.n_rb_items; r0 += nt) {   // uniform over the block
        const int r = r0 + tid;
        int kp0 = 0, kn0 = 0, len = 0, n0 = 0, ix = 0, iy = 0, iz = 0;
        if (r < d.n_rb_items) {
            const int4 it = d.rb_items[r];
            kp0 = it.x & 0xFFFFFF;
            len = it.x >> 24;
            kn0 = it.y & 0xFFFFFF;
            n0 = it.y >> 24;
            ix = (int)(int8_t)(it.z & 0xFF);
            iy = 2 * kcc + 1 + (int)(int8_t)((it.z >> 8) & 0xFF);
            iz = 3 * kcc + 2 + n0;
        }
        const int wl = __reduce_max_sync(0xffffffffu, len);   // warp-uniform (items sorted by length)
        for (int u = 0; u < len; u++) {
            reinterpret_cast<longlong2 *>(s.b.kvec)[kp0 + u] = make_longlong2(0, 0);
            reinterpret_cast<longlong2 *>(s.b.kvec)[kn0 - u] = make_longlong2(0, 0);
        }
        // 8 threads per particle build its table (stage <= nt / 8); each
        // thread's particle record of the next stage is loaded during this
        // stage's sums
        const int jj = tid >> 3;
        int4 pn = make_int4(0, 0, 0, 0);
        int tn = 0;
        if (jj < min(stage, d.N)) {
            pn = d.pos4[jj];
            tn = d.ptype[jj];
        }
        for (int j0 = 0; j0 < d.N; j0 += stage) {
            const int nb = min(stage, d.N - j0), np = (nb + 1) >> 1;
            __syncthreads();   // the previous stage's tables are consumed
            float2 *tf = reinterpret_cast<float2 *>(tab);
            if (jj < 2 * np) {
                const bool live = jj < nb;
                const float qv = live ? qk_charge(__int_as_float(pn.w), d.eff[tn], d) : 0.0f;
                const int hp[3] = {pn.x, pn.y, pn.z};
                if ((tid & 7) == 0) reinterpret_cast<float *>(q2)[jj] = qv;
                for (int t = tid & 7; t < T; t += 8)
                    tf[((jj >> 1) * T + t) * 2 + (jj & 1)] =
                        live ? rb_tab_entry(t, kcc, hp, s.b.sc_tab) : make_float2(0.0f, 0.0f);
            }
            if (jj < stage && j0 + stage + jj < d.N) {
                pn = d.pos4[j0 + stage + jj];
                tn = d.ptype[j0 + stage + jj];
            }
            __syncthreads();
            if (wl > 0) {
                unsigned sa[kRbLen], sr[kRbLen], sb[kRbLen], sc[kRbLen];
#pragma unroll
                for (int u = 0; u < kRbLen; u++) sa[u] = sr[u] = sb[u] = sc[u] = 0u;
                switch (wl) {
                    case 1: rb_pass<1>(tab, T, q2, np, ix, iy, iz, sa, sr, sb, sc); break;
                    case 2: rb_pass<2>(tab, T, q2, np, ix, iy, iz, sa, sr, sb, sc); break;
                    case 3: rb_pass<3>(tab, T, q2, np, ix, iy, iz, sa, sr, sb, sc); break;
                    default: rb_pass<4>(tab, T, q2, np, ix, iy, iz, sa, sr, sb, sc); break;
                }
                // each of the four sums carries 2 np kQkMagicBits
                const unsigned off2 = 4u * (unsigned)np * kQkMagicBits;
#pragma unroll
                for (int u = 0; u < kRbLen; u++) {
                    if (u >= len) continue;
                    rb_add(s, kp0 + u, qk_widen((int)(sa[u] - sr[u]), shift),
                           qk_widen((int)(sb[u] + sc[u] - off2), shift));
                    if (n0 + u > 0)
                        rb_add(s, kn0 - u, qk_widen((int)(sa[u] + sr[u] - off2), shift),
                               qk_widen((int)(sc[u] - sb[u]), shift));
                }
            }
        }
        // compare with the running sums and adopt
        for (int u = 0; u < len; u++) {
            rb_adopt(d, s, kp0 + u, e, bad);
            if (n0 + u > 0) rb_adopt(d, s, kn0 - u, e, bad);
        }
    }
    // energy correction: warp sums, then warp 0 over the warps (fixed order)
    e = warp_sum_df(e);
    const int anybad = __syncthreads_or(bad);   // also: every thread is done with the buffers
    if (lane == 0) s.b.red[tid >> 5] = make_float2(e.hi, e.lo);
    __syncthreads();
    if (tid < 32) {
        df t = {0.0f, 0.0f};
        if (lane < (nt >> 5)) t = {s.b.red[lane].x, s.b.red[lane].y};
        corr = warp_sum_df(t);
    }
    __syncthreads();   // red is free again
    return anybad != 0;
}

// Q(k) after a block: every accepted trial a adds c_k(new_a) - c_k(old_a)
// (ewald.h:665-705). Threads qt = 0..nq-1 (warps 1.. of the CTA, which
// synchronise among themselves on named barrier 1) own the rebuild's items
// (rb_items): per accepted trial they form w once for the new and the old
// position and, per n of the item, the four rounded products of each (the
// same integers the rebuild sums), accumulate the differences in 32 bits over
// the block's trials (at most 32 x 2^23) and add them to the exact int64 Q(k)
// of the item's (+n, -n) k-vectors at the end; integer sums, so the order of
// the trials does not matter. The axis tables of the accepted trials'
// new and old positions sit in the increment buffer as float4
// {new.re, new.im, old.re, old.im}, trial-major (tab[g * T + t]).
// On a cluster the CTA takes its own items [i0, i1), whose k-vectors it holds
// from k0 on (shared-memory index = k - k0).
__device__ __noinline__ void eb_commit_qk(const SysDesc &d, const EbSmem &s, uint32_t live, int qt, int nq, int i0,
                                          int i1, int k0) {
    int *alist = reinterpret_cast<int *>(s.corr);   // free after the resolution
    float *qg = s.G;                                // [32], free after the resolution
    if (qt < kEbTrials && ((live >> qt) & 1u)) {
        const int g = __popc(live & ((1u << qt) - 1u));
        alist[g] = qt;
        const Move &A = s.mv[qt];
        qg[g] = qk_charge(A.q, d.eff[A.ti], d);
    }
    const int na = __popc(live);
    const int kcc = d.kcc, T = rb_tab_len(kcc);
    float4 *tab = reinterpret_cast<float4 *>(s.delta);
    const int gmax = min(kEbTrials, (kEbKc * kEbTrials / 2 - kRbLen) / T);
    const int shift = d.qk_shift;
    for (int g0 = 0; g0 < na; g0 += gmax) {
        const int ng = min(gmax, na - g0);
        eb_qbar(nq);   // list written; the previous group's tables consumed
        for (int e = qt; e < ng * T; e += nq) {
            const int g = e / T, t = e - g * T;
            const Move &A = s.mv[alist[g0 + g]];
            const float2 en = rb_tab_entry(t, kcc, A.hn, s.b.sc_tab), eo = rb_tab_entry(t, kcc, A.ho, s.b.sc_tab);
            tab[e] = make_float4(en.x, en.y, eo.x, eo.y);
        }
        eb_qbar(nq);
        for (int r = i0 + qt; r < i1; r += nq) {
            const int4 it = d.rb_items[r];
            const int kp0 = (it.x & 0xFFFFFF) - k0, len = it.x >> 24, kn0 = (it.y & 0xFFFFFF) - k0, n0 = it.y >> 24;
            const int ix = (int)(int8_t)(it.z & 0xFF), iy = 2 * kcc + 1 + (int)(int8_t)((it.z >> 8) & 0xFF);
            const int iz = 3 * kcc + 2 + n0;
            unsigned da[kRbLen], dr[kRbLen], db[kRbLen], dc[kRbLen];
#pragma unroll
            for (int u = 0; u < kRbLen; u++) da[u] = dr[u] = db[u] = dc[u] = 0u;
            for (int g = 0; g < ng; g++) {
                const float4 *e = tab + g * T;
                const float q2g = qg[g0 + g];
                const float4 ex = e[ix], ey = e[iy];
                const float2 wn = qk_w(q2g, make_float2(ex.x, ex.y), make_float2(ey.x, ey.y));
                const float2 wo = qk_w(q2g, make_float2(ex.z, ex.w), make_float2(ey.z, ey.w));
#pragma unroll
                for (int u = 0; u < kRbLen; u++) {
                    if (u < len) {
                        const float4 z = e[iz + u];
                        da[u] += qk_rint_bits(wn.x, z.x) - qk_rint_bits(wo.x, z.z);
                        dr[u] += qk_rint_bits(wn.y, z.y) - qk_rint_bits(wo.y, z.w);
                        db[u] += qk_rint_bits(wn.x, z.y) - qk_rint_bits(wo.x, z.w);
                        dc[u] += qk_rint_bits(wn.y, z.x) - qk_rint_bits(wo.y, z.z);
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < kRbLen; u++) {
                if (u >= len) continue;
                // +n: (a - r, b + c); -n: (a + r, c - b)
                longlong2 q = s.b.qfix[kp0 + u];
                q.x += qk_widen((int)(da[u] - dr[u]), shift);
                q.y += qk_widen((int)(db[u] + dc[u]), shift);
                s.b.qfix[kp0 + u] = q;
                float2 qf = q_to_float(q);
                s.b.kvec[kp0 + u].y = qf.x;
                s.b.kvec[kp0 + u].z = qf.y;
                if (n0 + u > 0) {
                    q = s.b.qfix[kn0 - u];
                    q.x += qk_widen((int)(da[u] + dr[u]), shift);
                    q.y += qk_widen((int)(dc[u] - db[u]), shift);
                    s.b.qfix[kn0 - u] = q;
                    qf = q_to_float(q);
                    s.b.kvec[kn0 - u].y = qf.x;
                    s.b.kvec[kn0 - u].z = qf.y;
                }
            }
        }
    }
}

// Accepted trial: master and pair coordinates, and (in_cell: the particle
// stays in its cell) its record in the cell's slot array. Independent for
// distinct particles.
__device__ __forceinline__ void eb_commit_position(const Move &m, const SysDesc &d, const Smem &s, bool in_cell) {
    const int4 rec = make_int4(m.hn[0], m.hn[1], m.hn[2], __float_as_int(m.q));
    const short4 ext = make_short4((short)m.en[0], (short)m.en[1], (short)m.en[2], 0);
    d.pos64[3 * m.i + 0] = m.xn[0];
    d.pos64[3 * m.i + 1] = m.xn[1];
    d.pos64[3 * m.i + 2] = m.xn[2];
    d.pos4[m.i] = rec;
    d.pos_ext[m.i] = ext;
    if (d.use_cells && in_cell) {
        const int slot = (int)(s.pcs[m.i] & 0xFFFu);
        d.cell_pos[m.co * d.cap + slot] = rec;
        d.cell_ext[m.co * d.cap + slot] = ext;
    }
}
// A particle that changed cells: out of the old cell (the cell's last slot
// fills the hole) and into the next free slot of the new one, as
// commit_position does. One thread, accepted trials in order.
__device__ __forceinline__ void eb_cell_move(const Move &m, const SysDesc &d, const Smem &s) {
    const int4 rec = make_int4(m.hn[0], m.hn[1], m.hn[2], __float_as_int(m.q));
    const short4 ext = make_short4((short)m.en[0], (short)m.en[1], (short)m.en[2], 0);
    const int slot = (int)(s.pcs[m.i] & 0xFFFu);
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

// The cell counts alone of eb_cell_move: the other CTAs of a cluster keep
// their own copy for their stencil walks.
__device__ __forceinline__ void eb_cell_count_move(const Move &m, const SysDesc &d, const Smem &s) {
    s.ccount[m.co] -= 1;
    const int ns = s.ccount[m.cn];
    if (ns < d.cap) s.ccount[m.cn] = ns + 1;
}

// Surface dipole change of a trial (Angstrom e), as surface_delta computes it.
__device__ __forceinline__ void eb_dM(const Move &m, const SysDesc &d, float dM[3]) {
    const float qe = m.q * d.eff[m.ti];
#pragma unroll
    for (int a = 0; a < 3; a++) dM[a] = qe * ((float)m.hn[a] * d.s32[a] - (float)m.ho[a] * d.s32[a]);
}

// CLUSTER: one system on a thread-block cluster of C = eb_ctas CTAs (a
// system alone, where one CTA would leave the other SMs idle). CTA r holds
// the k-vectors [k0, k1) and their Q(k) (eb_ranges[r]) and runs the k-steps of
// its own k-vectors, a 1/C share of the correction pairs and the real-space
// walks of its warps (trial m in C/2 parts over the cluster's 16 C warps);
// its partial sums go into CTA 0's shared memory (remote stores), and after a
// cluster barrier CTA 0 alone completes the sums and resolves the block, and
// hands the outcome to every CTA. Then CTA 0 writes the positions and cell
// lists to global memory, every CTA updates its own Q(k) and cell counts, and
// a cluster barrier makes the new positions visible to the whole cluster
// before the next block reads them. A rebuild ends the launch (the rebuild
// kernel takes it, as for any system alone). The sums run in another order
// than on one CTA, so the dU agree to rounding, not bit for bit.
template <bool CELLS, bool CLUSTER>
__global__ void __launch_bounds__(kEbThreads, 1) ewald_block_kernel(const SysDesc *__restrict__ descs, int64_t end,
                                                                    const float2 *__restrict__ sc_tab) {
    extern __shared__ __align__(16) char eb_smem_raw[];
    __shared__ __align__(16) SysDesc sd;
    const int C = CLUSTER ? (int)blk_cluster_size() : 1;
    const int rank = CLUSTER ? (int)blk_cluster_rank() : 0;
    load_desc(sd, descs + (CLUSTER ? blockIdx.x / C : blockIdx.x));
    const SysDesc &d = sd;
    EbSmem s = eb_carve(eb_smem_raw, d, CELLS);
    SysScalars *sc = d.sc;
    // the work split (16 threads per trial, two Gram k-steps per warp) is
    // written for exactly kEbThreads threads; a cluster must match the
    // system's k-vector split (the same for every CTA of the cluster)
    if (blockDim.x != kEbThreads || (CLUSTER ? C != d.eb_ctas || C > kEbMaxCluster : d.eb_ctas != 1)) {
        if (threadIdx.x == 0) atomicOr(&sc->error, kErrLaunch);
        return;
    }
    if (sc->rebuild_pending || sc->cursor >= min(end, sc->n_trials)) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
    // this CTA's k-vectors [k0, k0 + K) and rebuild items [i0, i1)
    int k0 = 0, K = d.K, i0 = 0, i1 = d.n_rb_items;
    if (CLUSTER) {
        const int4 rg = d.eb_ranges[rank];
        k0 = rg.x;
        K = rg.y - rg.x;
        i0 = rg.z;
        i1 = rg.w;
    }
    // tables
    for (int t = tid; t < 256; t += blockDim.x) s.b.sc_tab[t] = sc_tab[t];
    for (int k = tid; k < K; k += blockDim.x) {
        const longlong2 q = d.qfix[k0 + k];
        const float2 qf = q_to_float(q);
        const float A = d.kvec[k0 + k].w;
        s.b.kvec[k] = make_float4(A, qf.x, qf.y, sqrtf(A));
        s.b.kpack[k] = d.kpack[k0 + k];
        s.b.qfix[k] = q;
    }
    // 2 pi / L per axis: k.d = sum_a n_a (2 pi / L_a) d_a
    const float tpl[3] = {6.283185307179586f / d.L[0], 6.283185307179586f / d.L[1], 6.283185307179586f / d.L[2]};
    if (CELLS) {
        const int ncell = d.nc[0] * d.nc[1] * d.nc[2];
        for (int c = tid; c < ncell; c += blockDim.x) s.b.ccount[c] = d.cell_count[c];
        for (int j = tid; j < d.N; j += blockDim.x)
            s.b.pcs[j] = ((uint32_t)d.p_cell[j] << 12) | (uint32_t)d.p_slot[j];
    }
    if (tid < 3) s.Mdf[tid] = make_float2(sc->m[tid][0], sc->m[tid][1]);
    if (CLUSTER) blk_cluster_barrier();   // every CTA of the cluster runs before any remote store
    else __syncthreads();
    int64_t cur = sc->cursor;
    const int64_t stop = min(end, sc->n_trials);
    df U = {sc->u_hi, sc->u_lo};
    df Ut = {sc->utot_hi, sc->utot_lo};
    int cnt_acc = sc->cnt_accepted;
    int64_t nacc = sc->n_accepted;
    const int uf = d.update_frequency;
    bool rebuild = false;
    int err = 0;
    // k space: warp w takes the k-steps (4 k-vectors) w, w + 16, ...; lane
    // (gq, gt) holds the Gram fragments of trials gq + 8 r, components gt and
    // gt + 4 of the step (eb_gram_regs)
    const int gq = lane >> 2, gt = lane & 3, gh = gt & 1, gk = gt >> 1;
    // per-trial records of the k-space phase (in the increment buffer, past
    // the real-space queues): {d 2pi/L, q eff}, {old high words, fast}, {new high words}
    float4 *rA = reinterpret_cast<float4 *>(reinterpret_cast<char *>(s.delta) + 16384);
    int4 *rB = reinterpret_cast<int4 *>(rA + kEbTrials);
    int4 *rC = rB + kEbTrials;
    while (cur < stop) {
        const int kb = (int)((stop - cur) < (int64_t)kEbTrials ? (stop - cur) : (int64_t)kEbTrials);
        // ---- trials of the block (old coordinates: the block start)
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
        __syncthreads();
        if (tid < kb) {
            uint32_t c = 0;
            const int i = s.mv[tid].i;
            for (int a = 0; a < tid; a++)
                if (s.mv[a].i == i) c |= 1u << a;
            s.col[tid] = c;
        }
        if (tid < kEbTrials) {
            float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            int4 b = make_int4(0, 0, 0, 1), c = make_int4(0, 0, 0, 0);
            if (tid < kb) {
                const Move &M = s.mv[tid];
                a = make_float4(M.dxf[0] * tpl[0], M.dxf[1] * tpl[1], M.dxf[2] * tpl[2], M.q * d.eff[M.ti]);
                // |k.d| <= kcc (|d_x| + |d_y| + |d_z|) 2pi/L: within the Taylor
                // range of expm1_i_horner every k takes the branch-free path
                const bool fast = (float)d.kcc * (fabsf(a.x) + fabsf(a.y) + fabsf(a.z)) <= 1.6f;
                b = make_int4(M.ho[0], M.ho[1], M.ho[2], fast ? 1 : 0);
                c = make_int4(M.hn[0], M.hn[1], M.hn[2], 0);
            }
            rA[tid] = a;
            rB[tid] = b;
            rC[tid] = c;
        }
        // the k-space records are the last shared input of the phases below:
        // from here each warp runs its corrections, its real-space walks and
        // its k-steps back to back, with no barrier between them (a warp
        // done walking early starts on k space)
        __syncthreads();
        // ---- real-space and surface corrections c(a, m), a < m (cluster: a
        // 1/C share per CTA, into CTA 0's table)
        const int e_lo = CLUSTER ? rank * (kEbTrials * kEbTrials / C) : 0;
        const int e_hi = CLUSTER ? e_lo + kEbTrials * kEbTrials / C : kEbTrials * kEbTrials;
        for (int e = e_lo + tid; e < e_hi; e += blockDim.x) {
            const int a = e / kEbTrials, m = e - a * kEbTrials;
            float2 out = make_float2(0.0f, 0.0f);
            if (a < m && m < kb && s.mv[a].i != s.mv[m].i) {
                const Move &A = s.mv[a];
                const Move &Mm = s.mv[m];
                const int4 pn = make_int4(A.hn[0], A.hn[1], A.hn[2], __float_as_int(A.q));
                const int4 po = make_int4(A.ho[0], A.ho[1], A.ho[2], __float_as_int(A.q));
                const short4 en = make_short4((short)A.en[0], (short)A.en[1], (short)A.en[2], 0);
                const short4 eo = make_short4((short)A.eo[0], (short)A.eo[1], (short)A.eo[2], 0);
                df c = df_add(eb_pair(Mm, pn, A.ti, &en, d), df_neg(eb_pair(Mm, po, A.ti, &eo, d)));
                if (d.surf_c != 0.0f) {
                    float da[3], dm[3];
                    eb_dM(A, d, da);
                    eb_dM(Mm, d, dm);
                    c = df_add_f(c, 2.0f * d.surf_c * fmaf(da[0], dm[0], fmaf(da[1], dm[1], da[2] * dm[2])));
                }
                out = make_float2(c.hi, c.lo);
            }
            if (CLUSTER) eb_st_remote(&s.corr[e], 0, out);
            else s.corr[e] = out;
        }
        // ---- real-space base: warp w sums trials w, w + nwarp, ...; its
        // candidate queue lives in the (not yet used) increment buffer. On a
        // cluster warp g = 16 r + w of the cluster takes part g % P of trial
        // g / P (P = C / 2 parts per trial), into CTA 0's part table.
        {
            const int P = CLUSTER ? (C + 1) / 2 : 1;
            const int u0 = CLUSTER ? rank * nwarp + warp : warp, du = CLUSTER ? C * nwarp : nwarp;
            for (int u = u0; u < kb * P; u += du) {
                const int m = u / P, part = u - m * P;
                const Move mv = s.mv[m];
                float accf = 0.0f;
                df accd = {0.0f, 0.0f};
                int4 *qp = reinterpret_cast<int4 *>(s.delta) + warp * 48;
                int2 *qm = reinterpret_cast<int2 *>(qp + 32);
                eb_pairs_warp<CELLS>(mv, d, s.b, qp, qm, part, P, accf, accd);
                const df p = warp_sum_df(df_add_f(accd, accf));
                if (lane == 0) {
                    if (CLUSTER) eb_st_remote(&s.xreal[m * P + part], 0, make_float2(p.hi, p.lo));
                    else s.partR[m] = make_float2(p.hi, p.lo);
                }
            }
        }
        // ---- reciprocal base and Gram matrix. Lane (gq, gt) and its partner
        // lane ^ 1 need the same increments sqrt(A') D[trial][k] (trials
        // gq + 8 r, k-vectors 4 st + gk and 4 st + 2 + gk), one the real and
        // one the imaginary part: each computes half (r = 2 gh, 2 gh + 1) and
        // they swap the other part. No chunk buffer, no barriers in the loop.
        float kac[2] = {0.0f, 0.0f};   // reciprocal base of trials gq + 8 (2 gh + rr)
        float gc[6][4];
#pragma unroll
        for (int x = 0; x < 6; x++)
#pragma unroll
            for (int y = 0; y < 4; y++) gc[x][y] = 0.0f;
        for (int st = warp; 4 * st < K; st += kEbThreads / 32) {
            float xf[4][2];   // component gh of sqrt(A') D[gq + 8 r][k_j]
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const int kraw = 4 * st + 2 * j + gk;
                const int k = min(kraw, K - 1);
                int nx, ny, nz;
                unpack_n(s.b.kpack[k], nx, ny, nz);
                const float4 kv = s.b.kvec[k];   // {A', Re Q, Im Q, sqrt A'}
                const float fx = small_int_to_float(nx), fy = small_int_to_float(ny), fz = small_int_to_float(nz);
#pragma unroll
                for (int rr = 0; rr < 2; rr++) {
                    const int t = gq + 8 * (2 * gh + rr);
                    const float4 a = rA[t];
                    const int4 b = rB[t];
                    const int ho[3] = {b.x, b.y, b.z};
                    const uint32_t ph = phase(nx, ny, nz, ho);
                    const float2 e = sincos_turns(ph, s.b.sc_tab);
                    const float phi = fmaf(fx, a.x, fmaf(fy, a.y, fz * a.z));
                    float2 w;
                    if (b.w || fabsf(phi) <= 1.6f) {
                        w = expm1_i_horner(phi);
                    } else {
                        const int4 c = rC[t];
                        const int hn[3] = {c.x, c.y, c.z};
                        const float2 en = sincos_turns(phase(nx, ny, nz, hn) - ph, s.b.sc_tab);
                        w = make_float2(en.x - 1.0f, en.y);
                    }
                    const float live = kraw < K ? a.w : 0.0f;   // q eff; 0 past K and for idle trials
                    float2 dd = cmul(e, w);
                    dd.x *= live;
                    dd.y *= live;
                    kac[rr] = fmaf(kv.x, fmaf(2.0f, fmaf(kv.y, dd.x, kv.z * dd.y), fmaf(dd.x, dd.x, dd.y * dd.y)),
                                   kac[rr]);
                    const float own = (gh ? dd.y : dd.x) * kv.w, other = (gh ? dd.x : dd.y) * kv.w;
                    const float recv = __shfl_xor_sync(0xffffffffu, other, 1);
                    xf[rr][j] = gh ? recv : own;
                    xf[2 + rr][j] = gh ? own : recv;
                }
            }
            eb_gram_regs(xf, gc);
        }
        // reciprocal base per trial: partials of (warp, lane, rr) summed in a
        // fixed order in df
        float *KP = reinterpret_cast<float *>(reinterpret_cast<char *>(s.delta) + 28672);   // [16][32][2]
        KP[(warp * 32 + lane) * 2] = kac[0];
        KP[(warp * 32 + lane) * 2 + 1] = kac[1];
        // Gram: the 16 warps' partial tiles meet in the (now free) increment
        // buffer in two rounds and are summed in a fixed order, so the result
        // does not depend on timing
        __syncthreads();
        float *P = reinterpret_cast<float *>(s.delta);   // [8 slots][6 tiles][32 lanes][4]
        {
            const int nw = kEbThreads / 32, slot = warp % (nw / 2);
            float *q = P + slot * (6 * 32 * 4) + lane * 4;
            if (warp < nw / 2) {
#pragma unroll
                for (int x = 0; x < 6; x++)
                    *reinterpret_cast<float4 *>(q + x * 128) = make_float4(gc[x][0], gc[x][1], gc[x][2], gc[x][3]);
            }
            if (tid < kEbTrials) {
                // trial t = gq' + 8 r': lanes gq' * 4 + (r' >> 1) + 2 gk', slot rr = r' & 1
                const int tq = tid & 7, tr = tid >> 3;
                df v = {0.0f, 0.0f};
                for (int w = 0; w < nw; w++)
                    for (int g2 = 0; g2 < 2; g2++)
                        v = df_add_f(v, KP[(w * 32 + tq * 4 + (tr >> 1) + 2 * g2) * 2 + (tr & 1)]);
                if (CLUSTER) eb_st_remote(&s.xkbase[rank * kEbTrials + tid], 0, make_float2(v.hi, v.lo));
                else s.kbase[tid] = make_float2(v.hi, v.lo);
            }
            __syncthreads();
            if (warp >= nw / 2) {
#pragma unroll
                for (int x = 0; x < 6; x++) {
                    float4 v = *reinterpret_cast<float4 *>(q + x * 128);
                    v.x += gc[x][0];
                    v.y += gc[x][1];
                    v.z += gc[x][2];
                    v.w += gc[x][3];
                    *reinterpret_cast<float4 *>(q + x * 128) = v;
                }
            }
            __syncthreads();
            // element e = (tile, lane, j) of the accumulator layout
            for (int e = tid; e < kEbGramN; e += blockDim.x) {
                float v = 0.0f;
                for (int sl = 0; sl < nw / 2; sl++) v += P[sl * kEbGramN + e];
                if (CLUSTER) {   // CTA 0 adds the ranks' sums up below
                    eb_st_remote(&s.xgram[rank * kEbGramN + e], 0, v);
                    continue;
                }
                const int x = e >> 7, ln = (e >> 2) & 31, j = e & 3;
                const int mi = x < 4 ? 0 : 1, nj = x < 4 ? x : x - 2;
                const int row = 16 * mi + (ln >> 2) + ((j & 2) ? 8 : 0);
                const int col = 8 * nj + 2 * (ln & 3) + (j & 1);
                // one correction per pair (a, m): real space + surface + reciprocal
                const float2 c = s.corr[row * kEbTrials + col];
                const df cs = df_add_f(df{c.x, c.y}, 2.0f * v);
                s.corr[row * kEbTrials + col] = make_float2(cs.hi, cs.lo);
            }
        }
        if (CLUSTER) {
            // every CTA's partial sums are in CTA 0: it completes them in a
            // fixed order (ranks, parts)
            blk_cluster_barrier();
            if (rank == 0) {
                for (int e = tid; e < kEbGramN; e += blockDim.x) {
                    float v = 0.0f;
                    for (int r = 0; r < C; r++) v += s.xgram[r * kEbGramN + e];
                    const int x = e >> 7, ln = (e >> 2) & 31, j = e & 3;
                    const int mi = x < 4 ? 0 : 1, nj = x < 4 ? x : x - 2;
                    const int row = 16 * mi + (ln >> 2) + ((j & 2) ? 8 : 0);
                    const int col = 8 * nj + 2 * (ln & 3) + (j & 1);
                    const float2 c = s.corr[row * kEbTrials + col];
                    const df cs = df_add_f(df{c.x, c.y}, 2.0f * v);
                    s.corr[row * kEbTrials + col] = make_float2(cs.hi, cs.lo);
                }
                if (tid < kEbTrials) {
                    const int P = (C + 1) / 2;
                    df kv = {0.0f, 0.0f}, rv = {0.0f, 0.0f};
                    for (int r = 0; r < C; r++) {
                        const float2 x = s.xkbase[r * kEbTrials + tid];
                        kv = df_add(kv, df{x.x, x.y});
                    }
                    for (int p = 0; p < P; p++) {
                        const float2 x = s.xreal[tid * P + p];
                        rv = df_add(rv, df{x.x, x.y});
                    }
                    s.kbase[tid] = make_float2(kv.hi, kv.lo);
                    s.partR[tid] = make_float2(rv.hi, rv.lo);
                }
            }
        }
        __syncthreads();
        // ---- resolve the block in order (warp 0 of CTA 0; lane m = trial m)
        if (warp == 0 && rank == 0) {
            df S = {0.0f, 0.0f};
            float dMl[3] = {0.0f, 0.0f, 0.0f};
            if (lane < kb) {
                const float2 r = s.partR[lane], kk = s.kbase[lane];
                S = df_add(df{r.x, r.y}, df{kk.x, kk.y});
                const df Mb[3] = {{s.Mdf[0].x, s.Mdf[0].y}, {s.Mdf[1].x, s.Mdf[1].y}, {s.Mdf[2].x, s.Mdf[2].y}};
                S = df_add(S, surface_delta(s.mv[lane], d, Mb, dMl));
            }
            const uint32_t colm = lane < kb ? s.col[lane] : 0u;
            const float2 th = lane < kb ? s.thr[lane] : make_float2(0.0f, 0.0f);
            uint32_t accm = 0;
            int done = kb;
            for (int a = 0; a < kb; a++) {
                // lane a decides: its S already holds the corrections of every
                // accepted trial before it in the block. Movebase::metropolis
                // (move.h:567-573): reject iff dU > kT (-ln u); a NaN dU
                // compares false there: accepted
                const float2 c = s.corr[a * kEbTrials + lane];   // loaded ahead of the decision
                // every lane forms its own flags; lane a's are the ones used
                const bool nan = !(S.hi == S.hi);
                const int fl = ((colm & accm) != 0u ? 1 : 0) | (nan || !df_gt(S, df{th.x, th.y}) ? 2 : 0) | (nan ? 4 : 0);
                const int f = __shfl_sync(0xffffffffu, fl, a);
                if (f & 1) {   // its particle was moved by an accepted trial of this block
                    done = a;
                    break;
                }
                if (f & 4) err |= kErrNonFinite;
                if (f & 2) {
                    accm |= 1u << a;
                    nacc++;
                    const df Sc = df_add_quick(S, df{c.x, c.y});
                    const bool later = lane > a && lane < kb;
                    S.hi = later ? Sc.hi : S.hi;
                    S.lo = later ? Sc.lo : S.lo;
                    // NonbondedEwald::update (ewald.h:633): a rebuild after
                    // update_frequency accepted trials ends the block here
                    if (++cnt_acc > uf - 1) {
                        cnt_acc = 0;
                        if (!d.skip_rebuild) {
                            rebuild = true;
                            done = a + 1;
                            break;
                        }
                    }
                }
            }
            // lane m's S is trial m's dU as decided: log it, and add the
            // accepted ones to the running sums (a fixed-order warp sum)
            const bool take = lane < done && ((accm >> lane) & 1u);
            if (d.log_trials && lane < done) {
                d.trial_du[cur + lane] = make_float2(S.hi, S.lo);
                d.trial_acc[cur + lane] = take ? 1 : 0;
            }
            const df sum = warp_sum_df(take ? S : df{0.0f, 0.0f});
            U = df_add(U, sum);
            Ut = df_add(Ut, sum);
            if (lane == 0) {
                s.info[0] = done;
                s.info[1] = (int)accm;
                s.info[2] = rebuild ? 1 : 0;
                s.info[3] = cnt_acc;
            }
            if (CLUSTER && lane > 0 && lane < C) {   // the outcome, to the other CTAs
                eb_st_remote(&s.info[0], lane, done);
                eb_st_remote(&s.info[1], lane, (int)accm);
                eb_st_remote(&s.info[2], lane, rebuild ? 1 : 0);
                eb_st_remote(&s.info[3], lane, cnt_acc);
            }
        }
        if (CLUSTER) blk_cluster_barrier();
        else __syncthreads();
        const int done = s.info[0];
        const uint32_t accm = (uint32_t)s.info[1];
        rebuild = s.info[2] != 0;
        cnt_acc = s.info[3];
        // ---- apply the accepted trials. Warp 0 commits the positions and
        // cell lists while warps 1.. update Q(k), synchronising among
        // themselves on named barrier 1; the block barrier below joins the two.
        const uint32_t live = accm & ((done >= 32) ? 0xffffffffu : ((1u << done) - 1u));
        if (warp == 0 && rank != 0) {
            // the other CTAs of a cluster: their cell counts alone
            if (CELLS && lane == 0)
                for (int a = 0; a < done; a++)
                    if (((accm >> a) & 1u) && s.mv[a].cn != s.mv[a].co) eb_cell_count_move(s.mv[a], d, s.b);
        } else if (warp == 0) {
            // positions (and, for a particle that stays in its
            // cell record) of the accepted trials, one lane each: the
            // particles are distinct; then lane 0 moves, in order, the
            // particles that changed cells
            const bool mine = (live >> lane) & 1u;
            bool mover = false;
            if (mine) {
                const Move &A = s.mv[lane];
                mover = CELLS && A.cn != A.co;
                eb_commit_position(A, d, s.b, !mover);
            }
            const uint32_t movers = __ballot_sync(0xffffffffu, mover);
            __syncwarp();   // the lanes' records are visible to lane 0
            if (lane == 0) {
                df M[3] = {{s.Mdf[0].x, s.Mdf[0].y}, {s.Mdf[1].x, s.Mdf[1].y}, {s.Mdf[2].x, s.Mdf[2].y}};
                for (int a = 0; a < done; a++) {
                    if (!((accm >> a) & 1u)) continue;
                    if ((movers >> a) & 1u) eb_cell_move(s.mv[a], d, s.b);
                    float dm[3];
                    eb_dM(s.mv[a], d, dm);
#pragma unroll
                    for (int x = 0; x < 3; x++) M[x] = df_add_f(M[x], dm[x]);
                }
#pragma unroll
                for (int x = 0; x < 3; x++) s.Mdf[x] = make_float2(M[x].hi, M[x].lo);
            }
        } else if (tid >= 32 && live) {
            // Q(k) += sum over accepted trials of c_k(new) - c_k(old), over
            // the rebuild's items (eb_commit_qk): each thread owns items of
            // (+n, -n) k-vector pairs and adds every accepted trial's change
            eb_commit_qk(d, s, live, tid - 32, blockDim.x - 32, i0, i1, k0);
        }
        cur += done;
        if (CLUSTER) {
            // CTA 0's positions and cell lists are visible to the cluster
            blk_cluster_barrier();
            if (rebuild) break;   // the rebuild kernel takes it (rebuild_pending)
            continue;
        }
        __syncthreads();
        if (rebuild && !d.rebuild_in_kernel) break;   // the rebuild kernel takes it (rebuild_pending)
        if (rebuild) {
            df corr;
            const bool mism = eb_rebuild(d, s, corr);
            if (tid == 0) {
                U = df_add(U, corr);
                Ut = df_add(Ut, corr);
                sc->n_rebuilds++;
                if (mism && sc->verify_rebuild) err |= kErrQkMismatch;
            }
            rebuild = false;
        }
    }
    // write back Q(k), cells and the scalars (a cluster: every CTA its own
    // Q(k), CTA 0 the rest)
    if (CLUSTER) {
        for (int k = tid; k < K; k += blockDim.x) d.qfix[k0 + k] = s.b.qfix[k];
        if (rank == 0) store_back(d, s.b, false, CELLS);
    } else {
        store_back(d, s.b, true, CELLS);
    }
    if (tid == 0 && rank == 0) {
        sc->cursor = cur;
        sc->u_hi = U.hi;
        sc->u_lo = U.lo;
        sc->utot_hi = Ut.hi;
        sc->utot_lo = Ut.lo;
        sc->n_accepted = nacc;
        for (int a = 0; a < 3; a++) {
            sc->m[a][0] = s.Mdf[a].x;
            sc->m[a][1] = s.Mdf[a].y;
        }
        sc->cnt_accepted = cnt_acc;
        if (rebuild) sc->rebuild_pending = 1;
        sc->error |= err;
    }
}

}  // namespace fg
