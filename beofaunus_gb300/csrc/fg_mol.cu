// Rigid dipolar molecules on the device: the TranslateRotate trial
// (move.h:1620-1705) and the whole-molecule energy change of
// NonbondedVector::g2All/g2g (energy.h:182-215, 1156-1196) over
//     CoulombGalore (multipole.h:569-598, the live operator: lB q q Q5(r/rc)/r)
//   + LennardJonesLB (potentials.h:2036-2040, no cutoff)
//   + IonDipole (multipole.h:993-996 -> q2mu 269-277, no cutoff)
//   + DipoleDipoleGalore reaction field (multipole.h:767-782, 910-920).
//
// Included by fg_api.cu (one translation unit).
//
// Work split. One system runs on a thread-block cluster of C CTAs (C <= 16,
// one per SM). A trial moves one molecule of gs sites; its energy change is a
// sum over the gs moved sites against all N - gs other sites. CTA r owns the
// site slice [r N/C, (r+1) N/C) and the dipole-site slice [r D/C, (r+1) D/C),
// kept in its shared memory, and sums its part; the C partial sums meet
// through distributed shared memory after one cluster barrier per trial, and
// every CTA then makes the same Metropolis decision from the same numbers.
// Each CTA keeps its own replica of the FP64-exact state (64-bit fixed-point
// positions, FP64 dipole vectors, mass centres) in global memory, so no CTA
// ever reads what another CTA wrote during the sweep.
//
// Precision. Positions are 64-bit fixed point (X = x/L 2^64). The rotation
// of a trial runs in FP64 on offsets from the rotation centre (20 sites per
// trial). Pair terms are FP32 except where that would exceed the 1e-6 kT
// budget:
//  * far pairs (both r_old, r_new >= rc): LJ and ion-dipole are small; LJ
//    uses 22-bit-truncated coordinate differences converted without the
//    conversion pipe, ion-dipole exact 32-bit differences;
//  * near pairs (r_old or r_new < rc) are queued and evaluated afterwards,
//    densely: LJ and Coulomb as differences u(r_new) - u(r_old) whose
//    rounding error scales with the difference, from r_new^2 - r_old^2
//    computed in FP64 from exact 48-bit coordinate differences; terms with a
//    dipole in FP64 (a few per trial);
//  * per-trial sums are double-float (df).
// The image convention is the reference's minimum image (Cuboid::vdist),
// taken on exact integer differences.
namespace fgm {

using fg::df;
using fg::df_add;
using fg::df_add_f;
using fg::df_gt;
using fg::hi32;
using fg::warp_sum_df;

constexpr int kMolThreads = 512;
constexpr int kMaxGroupSites = 31;   // lane gs of the setup warp computes the mass centre
constexpr int kQueueCap = 3072;
constexpr int kMaxCluster = 16;

// Error bits
constexpr int kMolErrNonFinite = 8;
constexpr int kMolErrLaunch = 64;   // launched with another cluster shape than requested

struct MolTrial {
    int32_t g;       // molecule index
    int32_t flags;   // 1 rotate, 2 translate, 4 explicit new coordinates (expl_*)
    int32_t center;  // rotation centre: 0 mass centre, 1 first site, 2 last site
    float thr_hi, thr_lo;  // -ln u as df: reject iff dU > threshold
    int32_t pad;
    double qw, qx, qy, qz;  // rotation quaternion (w, v)
    int64_t t[3];           // translation, fixed point
};

struct MolScalars {
    int64_t cursor;      // next trial
    int64_t n_trials;    // trials in the stream
    int64_t n_accepted;  // accepted so far (cumulative)
    int32_t error;
    int32_t pad;
    float u_hi, u_lo;        // sum of accepted dU of the current stream
    float utot_hi, utot_lo;  // running total energy
};

struct alignas(16) MolDesc {
    int32_t N, gs, M, D, nt, C, uniform_lj, cubic;
    float s32[3];       // L / 2^32 (one unit of the high word)
    float sc9[3];       // 512 L / 2^32 (unit of the high word >> 9)
    double s64d[3];     // L / 2^64
    double inv64d[3];   // 2^64 / L
    float lB, rc2, rc2near, rc1i, A5, B5, kT, rfB;
    float s32sq, pad2[3];  // (L / 2^32)^2 for cubic boxes
    double lBd, rcd, rfBd, pad3;
    long long rc2int;  // ceil(rc^2) in squared high-word units (cubic boxes)
    long long pad4;
    double s32sqd[3];
    float s2[256], eps4[256], lbqq[256];
    float qtype[16];
    double s2d[256], eps4d[256];  // FP64 copies for the total energy
    int64_t *rep_pos;  // C replicas x N x 3, fixed point
    double *rep_mu;    // C replicas x N x 3, dipole unit vectors
    int64_t *rep_cm;   // C replicas x M x 3, mass centres
    int4 *pos4;        // N: rounded high words (x, y, z), type
    int32_t *site_dip; // N: index in the dipole list, or -1
    int32_t *dip_site; // D: site of each dipole
    double *mus;       // N: dipole scalars (e Angstrom)
    float4 *dip4;      // D: mu-hat * mu (x, y, z), mu
    int4 *dip_pos4;    // D: positions of the dipole sites, .w = site << 8 | type
    const MolTrial *trials;
    float2 *log_du;
    uint8_t *log_acc;
    MolScalars *sc;
    const int64_t *expl_pos;  // gs x 3 new positions (explicit trials)
    const double *expl_mu;    // gs x 3 new dipole unit vectors
    const int64_t *expl_cm;   // 3, new mass centre
    double *eval_du;          // dU of an evaluated (not decided) trial
};

// ---------------------------------------------------------------- cluster PTX
__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Load a float2 from the shared memory of CTA `rank` of this cluster.
__device__ __forceinline__ float2 ld_cluster_f2(const float2 *p, unsigned rank) {
    unsigned a = (unsigned)__cvta_generic_to_shared(p), ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(ra) : "memory");
    return v;
}

// ---------------------------------------------------------------- helpers
// a - b with two's-complement wrap (the minimum image of high words).
__device__ __forceinline__ int wsub(int a, int b) { return (int)((uint32_t)a - (uint32_t)b); }

// Exact float of |m| < 2^22 without the conversion pipe.
__device__ __forceinline__ float small_to_float(int m) { return __int_as_float(0x4B400000 + m) - 12582912.0f; }

struct D3 {
    double x, y, z;
};
__device__ __forceinline__ double dot3(const D3 &a, const D3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 cross3(const D3 &a, const D3 &b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// Quaternion rotation as Eigen applies it: uv = v x p; uv += uv; p + w uv + v x uv.
__device__ __forceinline__ D3 qrot(double w, const D3 &v, const D3 &p) {
    D3 uv = cross3(v, p);
    uv = {uv.x + uv.x, uv.y + uv.y, uv.z + uv.z};
    D3 c = cross3(v, uv);
    return {p.x + w * uv.x + c.x, p.y + w * uv.y + c.y, p.z + w * uv.z + c.z};
}

// ---------------------------------------------------------------- shared memory
// Moved-molecule data, double-buffered: while the CTA sums trial t, the last
// warp prepares trial t+1 (its rotation runs in FP64 and is latency-bound).
struct GroupBuf {
    int4 *go, *gn;    // old/new high words; .w = type | dipole flag (go) / site << 8 | type (gn)
    float4 *gfo;      // old dipole vector mu-hat * mu (x, y, z), mu
    float4 *gfn;      // new dipole vector
    double *gmu;      // [gs][3] new unit dipole (FP64, for the replica)
    int64_t *gX;      // [gs][3] new fixed-point positions
    int64_t *gcm;     // [3] new mass centre
};

struct MolSmem {
    int4 *spos;     // site slice: high words, .w = type
    float4 *sdip;   // dipole slice: mu-hat * mu, mu
    int4 *sdpos;    // dipole slice positions, .w = site << 8 | type
    GroupBuf buf[2];
    uint32_t *queue;
    int *qcount;
    float2 *red;   // [32]
    float2 *part;  // [2] cluster partial sums (double-buffered by trial parity)
    int *flag;     // [4]: decision, speculation invalid
};

__host__ __device__ inline size_t mol_align16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline size_t mol_group_bytes(int gs) {
    return mol_align16((size_t)gs * 16 * 4) + mol_align16((size_t)gs * 3 * 8 * 2 + 3 * 8);
}

__host__ __device__ inline void mol_smem_layout(int ns, int nd, int gs, bool slice_smem, size_t off[16]) {
    size_t o = 0;
    off[0] = o; o += mol_align16(slice_smem ? (size_t)ns * 16 : 0);   // spos
    off[1] = o; o += mol_align16((size_t)nd * 16);                    // sdip
    off[2] = o; o += mol_align16((size_t)nd * 16);                    // sdpos
    off[3] = o; o += 2 * mol_group_bytes(gs);                         // group buffers
    off[4] = o; o += mol_align16((size_t)kQueueCap * 4 + 16);         // queue, qcount
    off[5] = o; o += mol_align16(32 * 8 + 2 * 8 + 16);                // red, part, flag
    off[6] = o;
}

__device__ inline MolSmem mol_carve(unsigned char *base, int ns, int nd, int gs, bool slice_smem) {
    size_t off[16];
    mol_smem_layout(ns, nd, gs, slice_smem, off);
    MolSmem s;
    s.spos = (int4 *)(base + off[0]);
    s.sdip = (float4 *)(base + off[1]);
    s.sdpos = (int4 *)(base + off[2]);
    for (int b = 0; b < 2; b++) {
        unsigned char *g = base + off[3] + b * mol_group_bytes(gs);
        GroupBuf &B = s.buf[b];
        B.go = (int4 *)g;
        B.gn = B.go + gs;
        B.gfo = (float4 *)(B.gn + gs);
        B.gfn = B.gfo + gs;
        B.gmu = (double *)(g + mol_align16((size_t)gs * 16 * 4));
        B.gX = (int64_t *)(B.gmu + 3 * gs);
        B.gcm = B.gX + 3 * gs;
    }
    s.queue = (uint32_t *)(base + off[4]);
    s.qcount = (int *)(s.queue + kQueueCap);
    s.red = (float2 *)(base + off[5]);
    s.part = s.red + 32;
    s.flag = (int *)(s.part + 2);
    return s;
}

// ---------------------------------------------------------------- pair terms
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Far pairs: squared distance from the high-word differences rounded to
// float (relative error < 1e-7; one conversion per axis, which measured
// faster than a shift-and-add conversion on the integer pipe).
__device__ __forceinline__ float far_r2(int4 a, int4 b, float3 sc9) {
    // the 32-bit minimum-image difference rounded to float (sc9 / 512 = L / 2^32)
    const float dx = (float)wsub(a.x, b.x) * (sc9.x * (1.0f / 512.0f));
    const float dy = (float)wsub(a.y, b.y) * (sc9.y * (1.0f / 512.0f));
    const float dz = (float)wsub(a.z, b.z) * (sc9.z * (1.0f / 512.0f));
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}
__device__ __forceinline__ float lj_r2(float r2, float s2, float e4) {
    const float x = s2 * rcp_approx(r2);
    const float x3 = x * x * x;
    return e4 * fmaf(x3, x3, -x3);
}

// Exact 32-bit difference vector a - b in Angstrom (FP32).
__device__ __forceinline__ float3 diff32(int4 a, int4 b, float3 s32) {
    return make_float3((float)wsub(a.x, b.x) * s32.x, (float)wsub(a.y, b.y) * s32.y, (float)wsub(a.z, b.z) * s32.z);
}
__device__ __forceinline__ float dot3f(float3 a, float3 b) { return fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)); }

// Coulomb part f(r) = Q5(r/rc) / r with Q5(q) = (q-1)^3 (A5 q^2 + B5 q - 1).
__device__ __forceinline__ float coul_f(float r, float rc1i, float A5, float B5) {
    const float q = r * rc1i;
    const float qm = q - 1.0f;
    return qm * qm * qm * fmaf(fmaf(A5, q, B5), q, -1.0f) / r;
}

// r_new^2 - r_old^2 (Angstrom^2) from exact integer arithmetic on the high
// words: sum_a (dn_a - do_a)(dn_a + do_a), each minimum image taken
// separately as Cuboid::vdist does; |product| < 2^62 always.
__device__ __forceinline__ float dr2_exact(int4 pn, int4 po, int4 pj, const MolDesc &d) {
    const int dn[3] = {wsub(pn.x, pj.x), wsub(pn.y, pj.y), wsub(pn.z, pj.z)};
    const int dO[3] = {wsub(po.x, pj.x), wsub(po.y, pj.y), wsub(po.z, pj.z)};
    if (d.cubic) {
        long long S = 0;
#pragma unroll
        for (int a = 0; a < 3; a++) S += ((long long)dn[a] - dO[a]) * ((long long)dn[a] + dO[a]);
        return fg::i64_to_float(S) * d.s32sq;
    }
    double S = 0.0;
#pragma unroll
    for (int a = 0; a < 3; a++)
        S += (double)(((long long)dn[a] - dO[a]) * ((long long)dn[a] + dO[a])) * d.s32sqd[a];
    return (float)S;
}

// Near pair, kind A: moved site i (old po, new pn) against site j: LJ and
// Coulomb as differences whose rounding scales with the difference, and the
// ion-dipole term of i's dipole with j's charge (FP32, a few per trial).
__device__ __noinline__ float near_pair_a(int4 po, int4 pn, float4 fo, float4 fn, int4 pj, const MolDesc &d) {
    const float3 s32 = make_float3(d.s32[0], d.s32[1], d.s32[2]);
    const float3 ro = diff32(po, pj, s32), rn = diff32(pn, pj, s32);
    const float ro2 = dot3f(ro, ro), rn2 = dot3f(rn, rn);
    const float dR2 = dr2_exact(pn, po, pj, d);
    const int ti = po.w & 0xFF, tj = pj.w & 0xFF;
    const int t = ti * d.nt + tj;
    // LJ: 4eps x_o^3 (t^3 - 1)(x_o^3 (t^3 + 1) - 1), t^3 - 1 from tau = -dR2 / r_n^2
    const float xo = d.s2[t] / ro2;
    const float xo3 = xo * xo * xo;
    const float tau = -dR2 / rn2;
    const float t3m1 = tau * fmaf(tau, tau + 3.0f, 3.0f);
    float acc = d.eps4[t] * xo3 * t3m1 * fmaf(xo3, t3m1 + 2.0f, -1.0f);
    // Coulomb (CoulombGalore)
    const float A = d.lbqq[t];
    if (A != 0.0f) {
        const bool io = ro2 < d.rc2, in_ = rn2 < d.rc2;
        const float r_o = sqrtf(ro2), r_n = sqrtf(rn2);
        if (io && in_) {
            // f_n - f_o = [Q5(q_n) - Q5(q_o)] / r_n - Q5(q_o) dr / (r_n r_o)
            const float dr = dR2 / (r_n + r_o);
            const float qo = r_o * d.rc1i, qn = r_n * d.rc1i, dq = dr * d.rc1i;
            const float mo = qo - 1.0f, mn = qn - 1.0f;
            const float Po = fmaf(fmaf(d.A5, qo, d.B5), qo, -1.0f);
            const float Pn = fmaf(fmaf(d.A5, qn, d.B5), qn, -1.0f);
            const float dcube = dq * fmaf(mn, mn + mo, mo * mo);   // (q_n-1)^3 - (q_o-1)^3
            const float dP = dq * fmaf(d.A5, qn + qo, d.B5);       // P(q_n) - P(q_o)
            const float dQ = fmaf(dcube, Pn, mo * mo * mo * dP);
            acc += A * (dQ / r_n - mo * mo * mo * Po * dr / (r_n * r_o));
        } else if (io) {
            acc -= A * coul_f(r_o, d.rc1i, d.A5, d.B5);
        } else if (in_) {
            acc += A * coul_f(r_n, d.rc1i, d.A5, d.B5);
        }
    }
    if (po.w & 0x100) {
        // W2 of IonDipole(a = i, b = j): -lB q_j (mu_i . r) / r^3
        const float qj = d.qtype[tj];
        const float io = rsqrtf(ro2), in_ = rsqrtf(rn2);
        const float w = dot3f(make_float3(fn.x, fn.y, fn.z), rn) * in_ * in_ * in_ -
                        dot3f(make_float3(fo.x, fo.y, fo.z), ro) * io * io * io;
        acc -= d.lB * qj * w;
    }
    return acc;
}

// Near pair, kind B: moved site i against dipole k: ion-dipole with i's charge
// and, when i carries a dipole, dipole-dipole with the reaction field; the
// cutoff test is exact on the integer squared distance.
__device__ __noinline__ float near_pair_b(int4 po, int4 pn, float4 fo, float4 fn, int4 pk, float4 vk,
                                          const MolDesc &d) {
    const float3 s32 = make_float3(d.s32[0], d.s32[1], d.s32[2]);
    const float3 ro = diff32(po, pk, s32), rn = diff32(pn, pk, s32);
    const float ro2 = dot3f(ro, ro), rn2 = dot3f(rn, rn);
    const float io = rsqrtf(ro2), in_ = rsqrtf(rn2);
    const float3 v = make_float3(vk.x, vk.y, vk.z);
    const float qi = d.qtype[po.w & 0xFF];
    float acc = d.lB * qi * (dot3f(v, rn) * in_ * in_ * in_ - dot3f(v, ro) * io * io * io);
    if (po.w & 0x100) {
        auto dd = [&](float4 f, float3 r, float r2, float ri, int4 p) {
            const int dx = wsub(p.x, pk.x), dy = wsub(p.y, pk.y), dz = wsub(p.z, pk.z);
            bool inside;
            if (d.cubic) {
                // exact: |r|^2 < rc^2 on integers (rc2int = ceil(rc^2) in high-word units)
                inside = (long long)dx * dx + (long long)dy * dy + (long long)dz * dz < d.rc2int;
            } else {
                inside = (double)dx * dx * d.s32sqd[0] + (double)dy * dy * d.s32sqd[1] +
                             (double)dz * dz * d.s32sqd[2] < d.rcd * d.rcd;
            }
            if (!inside) return 0.0f;
            const float3 u = make_float3(f.x, f.y, f.z);
            const float r1 = r2 * ri;
            const float q = r1 * d.rc1i;
            const float dt = dot3f(u, v);
            // mu2mu with A = 1, B = rfB q^3: -(3 (u.r)(v.r)/r^2 - u.v + u.v B) / r^3
            const float T = fmaf(3.0f * dot3f(u, r), dot3f(v, r) * (ri * ri), -dt) + dt * (d.rfB * q * q * q);
            return -d.lB * T * ri * ri * ri;
        };
        acc += dd(fn, rn, rn2, in_, pn) - dd(fo, ro, ro2, io, po);
    }
    return acc;
}

// ---------------------------------------------------------------- trial setup
// New coordinates of the moved molecule: FP64 rotation of offsets from the
// centre, then translation, one lane per site; lane gs does the mass centre.
// Old data come from this CTA's replica. Called by one warp.
__device__ __forceinline__ void setup_trial(const MolTrial &tr, const MolDesc &d, const GroupBuf &B, int rank,
                                            int lane) {
    const int gs = d.gs, g = tr.g;
    const int64_t *P = d.rep_pos + (size_t)rank * d.N * 3;
    const double *MU = d.rep_mu + (size_t)rank * d.N * 3;
    const int64_t *CM = d.rep_cm + (size_t)rank * d.M * 3;
    if (lane > gs) return;
    const bool explicit_ = tr.flags & 4;
    int64_t c[3] = {0, 0, 0};
    if (!explicit_) {
        if (tr.center == 0) {
            for (int a = 0; a < 3; a++) c[a] = CM[3 * g + a];
        } else {
            const int cs = g * gs + (tr.center == 1 ? 0 : gs - 1);
            for (int a = 0; a < 3; a++) c[a] = P[3 * cs + a];
        }
    }
    const D3 qv = {tr.qx, tr.qy, tr.qz};
    auto move_point = [&](const int64_t X[3], int64_t out[3]) {
        int64_t Y[3] = {X[0], X[1], X[2]};
        if (tr.flags & 1) {
            const D3 a = {(double)(int64_t)((uint64_t)X[0] - (uint64_t)c[0]) * d.s64d[0],
                          (double)(int64_t)((uint64_t)X[1] - (uint64_t)c[1]) * d.s64d[1],
                          (double)(int64_t)((uint64_t)X[2] - (uint64_t)c[2]) * d.s64d[2]};
            const D3 b = qrot(tr.qw, qv, a);
            Y[0] = (int64_t)((uint64_t)c[0] + (uint64_t)__double2ll_rn(b.x * d.inv64d[0]));
            Y[1] = (int64_t)((uint64_t)c[1] + (uint64_t)__double2ll_rn(b.y * d.inv64d[1]));
            Y[2] = (int64_t)((uint64_t)c[2] + (uint64_t)__double2ll_rn(b.z * d.inv64d[2]));
        }
        if (tr.flags & 2)
            for (int a = 0; a < 3; a++) Y[a] = (int64_t)((uint64_t)Y[a] + (uint64_t)tr.t[a]);
        for (int a = 0; a < 3; a++) out[a] = Y[a];
    };
    if (lane == gs) {
        int64_t cn[3];
        if (explicit_) {
            for (int a = 0; a < 3; a++) cn[a] = d.expl_cm ? d.expl_cm[a] : CM[3 * g + a];
        } else {
            const int64_t co[3] = {CM[3 * g], CM[3 * g + 1], CM[3 * g + 2]};
            move_point(co, cn);
        }
        for (int a = 0; a < 3; a++) B.gcm[a] = cn[a];
        return;
    }
    const int site = g * gs + lane;
    const int64_t Xo[3] = {P[3 * site], P[3 * site + 1], P[3 * site + 2]};
    int64_t Xn[3];
    const D3 uo = {MU[3 * site], MU[3 * site + 1], MU[3 * site + 2]};
    D3 un;
    if (explicit_) {
        for (int a = 0; a < 3; a++) Xn[a] = d.expl_pos[3 * lane + a];
        un = d.expl_mu ? D3{d.expl_mu[3 * lane], d.expl_mu[3 * lane + 1], d.expl_mu[3 * lane + 2]} : uo;
    } else {
        move_point(Xo, Xn);
        un = (tr.flags & 1) ? qrot(tr.qw, qv, uo) : uo;  // DipoleParticle::rotate (point.h:672-679)
    }
    const int type = d.pos4[site].w & 0xFF;
    const bool has_dip = d.site_dip[site] >= 0;
    const double m = d.mus[site];
    B.go[lane] = make_int4(hi32(Xo[0]), hi32(Xo[1]), hi32(Xo[2]), type | (has_dip ? 0x100 : 0));
    B.gn[lane] = make_int4(hi32(Xn[0]), hi32(Xn[1]), hi32(Xn[2]), type | (site << 8));
    B.gfo[lane] = make_float4((float)(uo.x * m), (float)(uo.y * m), (float)(uo.z * m), (float)m);
    B.gfn[lane] = make_float4((float)(un.x * m), (float)(un.y * m), (float)(un.z * m), (float)m);
    B.gmu[3 * lane] = un.x;
    B.gmu[3 * lane + 1] = un.y;
    B.gmu[3 * lane + 2] = un.z;
    for (int a = 0; a < 3; a++) B.gX[3 * lane + a] = Xn[a];
}

// ---------------------------------------------------------------- energy change
// Warp-aggregated append of near pairs to the queue; a full queue makes the
// lanes evaluate their pair in place (returned in `inplace`).
__device__ __forceinline__ bool enqueue(const MolSmem &s, bool near, uint32_t code) {
    const unsigned active = __activemask();
    const unsigned m = __ballot_sync(active, near);
    if (!m) return false;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(s.qcount, __popc(m));
    base = __shfl_sync(active, base, leader);
    if (!near) return false;
    const int slot = base + __popc(m & ((1u << lane) - 1u));
    if (slot < kQueueCap) {
        s.queue[slot] = code;
        return false;
    }
    return true;
}

// This CTA's part of dU for the trial in buffer B. Pair loops use threads
// [0, nwork); the queue is drained by all threads.
template <bool SLICE_SMEM>
__device__ float mol_partial_loops(const MolDesc &d, const MolSmem &s, const GroupBuf &B, int g, int j0, int ns,
                                   int nd, int nwork) {
    const int tid = threadIdx.x, gs = d.gs;
    const int g_lo = g * gs, g_hi = g_lo + gs;
    const float3 sc9 = make_float3(d.sc9[0], d.sc9[1], d.sc9[2]);
    const float3 s32 = make_float3(d.s32[0], d.s32[1], d.s32[2]);
    const float rc2near = d.rc2near, lB = d.lB;
    const int nt = d.nt;
    const bool uni = d.uniform_lj != 0;
    const float s2u = d.s2[0], e4u = d.eps4[0];
    float acc = 0.0f;
    if (tid >= nwork) return 0.0f;
    // loop A: slice sites j (one per thread) against every moved site i;
    // whole warps iterate together so the queue appends stay warp-wide
    for (int jb = tid - (tid & 31); jb < ns; jb += nwork) {
        const int jj = jb + (tid & 31);
        const int j = j0 + jj;
        const bool valid = jj < ns && !(j >= g_lo && j < g_hi);
        const int4 pj = SLICE_SMEM ? s.spos[min(jj, ns - 1)] : d.pos4[j0 + min(jj, ns - 1)];
        const int tj = pj.w & 0xFF;
        const float qj = d.qtype[tj];
#pragma unroll 2
        for (int i = 0; i < gs; i++) {
            const int4 po = B.go[i], pn = B.gn[i];
            const int t = (po.w & 0xFF) * nt + tj;
            const float s2 = uni ? s2u : d.s2[t], e4 = uni ? e4u : d.eps4[t];
            const float r2o = far_r2(po, pj, sc9), r2n = far_r2(pn, pj, sc9);
            const bool near = valid && ((r2o < rc2near) | (r2n < rc2near));
            if (enqueue(s, near, ((uint32_t)i << 24) | (uint32_t)jj))
                acc += near_pair_a(po, pn, B.gfo[i], B.gfn[i], pj, d);
            if (valid && !near) {
                acc += lj_r2(r2n, s2, e4) - lj_r2(r2o, s2, e4);
                if ((po.w & 0x100) && qj != 0.0f) {
                    // W2 of IonDipole(a = i, b = j): -lB q_j (mu_i . r) / r^3
                    const float3 ro = diff32(po, pj, s32), rn = diff32(pn, pj, s32);
                    const float4 fo = B.gfo[i], fn = B.gfn[i];
                    const float ro2 = dot3f(ro, ro), rn2 = dot3f(rn, rn);
                    const float io = rsqrtf(ro2), in_ = rsqrtf(rn2);
                    const float w = dot3f(make_float3(fn.x, fn.y, fn.z), rn) * in_ * in_ * in_ -
                                    dot3f(make_float3(fo.x, fo.y, fo.z), ro) * io * io * io;
                    acc -= lB * qj * w;
                }
            }
        }
    }
    // loop B: (dipole k of this slice, moved site i) items spread over threads
    const int nitems = nd * gs;
    for (int eb = tid - (tid & 31); eb < nitems; eb += nwork) {
        const int e = eb + (tid & 31);
        const int kk = min(e, nitems - 1) / gs, i = min(e, nitems - 1) - kk * gs;
        const int4 pk = s.sdpos[kk];
        const int ksite = pk.w >> 8;
        const bool valid = e < nitems && !(ksite >= g_lo && ksite < g_hi);
        const int4 po = B.go[i], pn = B.gn[i];
        const float3 ro = diff32(po, pk, s32), rn = diff32(pn, pk, s32);
        const float ro2 = dot3f(ro, ro), rn2 = dot3f(rn, rn);
        const bool near = valid && ((ro2 < rc2near) | (rn2 < rc2near));
        if (enqueue(s, near, 0x800000u | ((uint32_t)i << 24) | (uint32_t)kk))
            acc += near_pair_b(po, pn, B.gfo[i], B.gfn[i], pk, s.sdip[kk], d);
        if (valid && !near) {
            const float qi = d.qtype[po.w & 0xFF];
            if (qi != 0.0f) {
                // W1 of IonDipole(a = i, b = k): lB q_i (mu_k . r) / r^3 (dipole-dipole is 0 beyond rc)
                const float4 vk = s.sdip[kk];
                const float3 v = make_float3(vk.x, vk.y, vk.z);
                const float io = rsqrtf(ro2), in_ = rsqrtf(rn2);
                acc += lB * qi * (dot3f(v, rn) * in_ * in_ * in_ - dot3f(v, ro) * io * io * io);
            }
        }
    }
    return acc;
}

template <bool SLICE_SMEM>
__device__ float mol_partial_queue(const MolDesc &d, const MolSmem &s, const GroupBuf &B, int j0) {
    const int nq = min(*s.qcount, kQueueCap);
    float acc = 0.0f;
    for (int e = threadIdx.x; e < nq; e += blockDim.x) {
        const uint32_t q = s.queue[e];
        const int i = (int)((q >> 24) & 0x7F);
        const int idx = (int)(q & 0x7FFFFF);
        if (q & 0x800000u) {
            acc += near_pair_b(B.go[i], B.gn[i], B.gfo[i], B.gfn[i], s.sdpos[idx], s.sdip[idx], d);
        } else {
            const int4 pj = SLICE_SMEM ? s.spos[idx] : d.pos4[j0 + idx];
            acc += near_pair_a(B.go[i], B.gn[i], B.gfo[i], B.gfn[i], pj, d);
        }
    }
    return acc;
}

// ---------------------------------------------------------------- the sweep
// One cluster of C CTAs per system (blockIdx.x / C). EVAL: evaluate trial 0
// only, write its dU to eval_du, decide and commit nothing. The last warp
// prepares the next trial's coordinates while the others sum pairs; the
// prepared buffer is discarded when an accepted trial moved the same molecule.
template <bool SLICE_SMEM, bool CLUSTER, bool EVAL>
__global__ void __launch_bounds__(kMolThreads, 1) mol_sweep_kernel(const MolDesc *__restrict__ descs) {
    extern __shared__ __align__(16) unsigned char mol_smem_raw[];
    const int C = CLUSTER ? (int)descs[0].C : 1;
    const int sys = blockIdx.x / C;
    // launch-shape check: partial sums are read from C CTAs of this cluster
    if (CLUSTER && (int)cluster_size() != C) {
        if (threadIdx.x == 0) atomicOr(&descs[sys].sc->error, kMolErrLaunch);
        return;
    }
    const int rank = CLUSTER ? (int)cluster_rank() : 0;
    const MolDesc &d = descs[sys];
    const int tid = threadIdx.x, lane = tid & 31;
    const int nwork = (int)blockDim.x - 32;           // threads on the pair loops
    const bool setup_warp = tid >= nwork;
    const int ns_full = (d.N + C - 1) / C, nd_full = (d.D + C - 1) / C;
    const int j0 = min(rank * ns_full, d.N), j1 = min(j0 + ns_full, d.N), ns = j1 - j0;
    const int k0 = min(rank * nd_full, d.D), k1 = min(k0 + nd_full, d.D), nd = k1 - k0;
    MolSmem s = mol_carve(mol_smem_raw, ns_full, nd_full, d.gs, SLICE_SMEM);
    if (SLICE_SMEM)
        for (int jj = tid; jj < ns; jj += blockDim.x) s.spos[jj] = d.pos4[j0 + jj];
    for (int kk = tid; kk < nd; kk += blockDim.x) {
        s.sdip[kk] = d.dip4[k0 + kk];
        s.sdpos[kk] = d.dip_pos4[k0 + kk];
    }
    int64_t cursor = EVAL ? 0 : d.sc->cursor;
    const int64_t n = EVAL ? 1 : d.sc->n_trials;
    df usum = {d.sc->u_hi, d.sc->u_lo};
    df utot = {d.sc->utot_hi, d.sc->utot_lo};
    int64_t nacc = d.sc->n_accepted;
    int err = 0;
    if (tid == 0) {
        s.part[0] = s.part[1] = make_float2(0.0f, 0.0f);
        s.flag[0] = s.flag[1] = 0;
    }
    if (cursor < n && setup_warp) setup_trial(d.trials[cursor], d, s.buf[cursor & 1], rank, lane);
    if (CLUSTER) cluster_barrier();
    else __syncthreads();
    for (; cursor < n; cursor++) {
        const int b = (int)(cursor & 1);
        const MolTrial tr = d.trials[cursor];
        if (s.flag[1]) {   // the prepared buffer is stale (same molecule, accepted)
            __syncthreads();
            if (setup_warp) setup_trial(tr, d, s.buf[b], rank, lane);
            if (tid == 0) s.flag[1] = 0;
        }
        if (tid == 0) *s.qcount = 0;
        __syncthreads();
        float part;
        if (!setup_warp) {
            part = mol_partial_loops<SLICE_SMEM>(d, s, s.buf[b], tr.g, j0, ns, nd, nwork);
        } else {
            part = 0.0f;
            if (!EVAL && cursor + 1 < n) setup_trial(d.trials[cursor + 1], d, s.buf[b ^ 1], rank, lane);
        }
        __syncthreads();
        part += mol_partial_queue<SLICE_SMEM>(d, s, s.buf[b], j0);
        df pd = warp_sum_df(df{part, 0.0f});
        if (lane == 0) s.red[tid >> 5] = make_float2(pd.hi, pd.lo);
        __syncthreads();
        const int slot = b;
        if (tid < 32) {
            df v = {0.0f, 0.0f};
            if (tid < (int)(blockDim.x >> 5)) v = df{s.red[tid].x, s.red[tid].y};
            v = warp_sum_df(v);
            if (tid == 0) s.part[slot] = make_float2(v.hi, v.lo);
        }
        if (CLUSTER) cluster_barrier();
        else __syncthreads();
        if (tid < 32) {
            df v = {0.0f, 0.0f};
            if (tid < C) {
                const float2 p = CLUSTER ? ld_cluster_f2(&s.part[slot], (unsigned)tid) : s.part[slot];
                v = df{p.x, p.y};
            }
            v = warp_sum_df(v);
            v.hi = __shfl_sync(0xffffffffu, v.hi, 0);
            v.lo = __shfl_sync(0xffffffffu, v.lo, 0);
            if (tid == 0) {
                int dec;
                if (!isfinite(v.hi)) dec = 2;
                else dec = df_gt(v, df{tr.thr_hi, tr.thr_lo}) ? 0 : 1;
                s.flag[0] = dec;
                s.red[0] = make_float2(v.hi, v.lo);
                if (dec == 1 && cursor + 1 < n && d.trials[cursor + 1].g == tr.g) s.flag[1] = 1;
            }
        }
        __syncthreads();
        const int dec = s.flag[0];
        const df du = {s.red[0].x, s.red[0].y};
        if (EVAL) {
            if (rank == 0 && tid == 0) *d.eval_du = (double)du.hi + (double)du.lo;
            break;
        }
        if (dec == 2) {
            err |= kMolErrNonFinite;
            break;
        }
        if (rank == 0 && tid == 0) {
            if (d.log_du) d.log_du[cursor] = make_float2(du.hi, du.lo);
            if (d.log_acc) d.log_acc[cursor] = (uint8_t)dec;
        }
        if (dec == 1) {
            nacc++;
            usum = df_add(usum, du);
            utot = df_add(utot, du);
            const int gs = d.gs, g = tr.g;
            const GroupBuf &B = s.buf[b];
            if (tid < gs) {
                const int site = g * gs + tid;
                int64_t *P = d.rep_pos + ((size_t)rank * d.N + site) * 3;
                double *MU = d.rep_mu + ((size_t)rank * d.N + site) * 3;
                for (int a = 0; a < 3; a++) {
                    P[a] = B.gX[3 * tid + a];
                    MU[a] = B.gmu[3 * tid + a];
                }
                const int4 pn = make_int4(B.gn[tid].x, B.gn[tid].y, B.gn[tid].z, B.go[tid].w & 0xFF);
                if (site >= j0 && site < j1) {
                    if (SLICE_SMEM) s.spos[site - j0] = pn;
                    else d.pos4[site] = pn;
                }
                const int k = d.site_dip[site];
                if (k >= k0 && k < k1) {
                    s.sdpos[k - k0] = make_int4(pn.x, pn.y, pn.z, (site << 8) | (pn.w & 0xFF));
                    s.sdip[k - k0] = B.gfn[tid];
                }
            } else if (tid == gs) {
                int64_t *CM = d.rep_cm + ((size_t)rank * d.M + g) * 3;
                for (int a = 0; a < 3; a++) CM[a] = B.gcm[a];
            }
        }
        __syncthreads();
    }
    // write the slices back (each CTA its own range) and the scalars
    if (!EVAL) {
        if (SLICE_SMEM)
            for (int jj = tid; jj < ns; jj += blockDim.x) d.pos4[j0 + jj] = s.spos[jj];
        for (int kk = tid; kk < nd; kk += blockDim.x) {
            d.dip4[k0 + kk] = s.sdip[kk];
            d.dip_pos4[k0 + kk] = s.sdpos[kk];
        }
        if (rank == 0 && tid == 0) {
            MolScalars *sc = d.sc;
            sc->cursor = cursor;
            sc->n_accepted = nacc;
            sc->u_hi = usum.hi;
            sc->u_lo = usum.lo;
            sc->utot_hi = utot.hi;
            sc->utot_lo = utot.lo;
            sc->error |= err;
        }
    }
    if (CLUSTER) cluster_barrier();   // no CTA leaves while another may read its shared memory
}

// Apply an evaluated explicit trial (fg_mol_commit): new positions, dipoles
// and mass centre into every replica, the site/dipole records and the
// running energy. One block of >= gs + 1 threads.
__global__ void mol_commit_kernel(const MolDesc *__restrict__ descs, int g, int accepted, int nrep) {
    const MolDesc &d = descs[0];
    const int tid = threadIdx.x, gs = d.gs;
    if (!accepted) return;
    if (tid < gs) {
        const int site = g * gs + tid;
        int64_t X[3];
        for (int a = 0; a < 3; a++) X[a] = d.expl_pos[3 * tid + a];
        for (int r = 0; r < nrep; r++) {
            int64_t *P = d.rep_pos + ((size_t)r * d.N + site) * 3;
            double *MU = d.rep_mu + ((size_t)r * d.N + site) * 3;
            for (int a = 0; a < 3; a++) {
                P[a] = X[a];
                if (d.expl_mu) MU[a] = d.expl_mu[3 * tid + a];
            }
        }
        const int type = d.pos4[site].w & 0xFF;
        const int4 p4 = make_int4(hi32(X[0]), hi32(X[1]), hi32(X[2]), type);
        d.pos4[site] = p4;
        const int k = d.site_dip[site];
        if (k >= 0) {
            const double m = d.mus[site];
            const double *u = d.rep_mu + (size_t)site * 3;
            d.dip_pos4[k] = make_int4(p4.x, p4.y, p4.z, (site << 8) | type);
            d.dip4[k] = make_float4((float)(u[0] * m), (float)(u[1] * m), (float)(u[2] * m), (float)m);
        }
    } else if (tid == gs && d.expl_cm) {
        for (int r = 0; r < nrep; r++)
            for (int a = 0; a < 3; a++) d.rep_cm[((size_t)r * d.M + g) * 3 + a] = d.expl_cm[a];
    }
}

// IonDipole (q2mu, multipole.h:269-277) in FP64 with r = r_a - r_b:
// lB [qa mub (mub.r) - qb mua (mua.r)] / r^3, mu vectors already scaled.
__device__ __forceinline__ double ion_dipole64(double qa, const D3 &mua, double qb, const D3 &mub, const D3 &r,
                                               double lB) {
    const double r2i = 1.0 / dot3(r, r);
    const double r3i = sqrt(r2i) * r2i;
    return lB * (qa * dot3(mub, r) * r3i - qb * dot3(mua, r) * r3i);
}
// DipoleDipoleGalore with the reaction field (multipole.h:287-299, 767-782, 910-920).
__device__ __forceinline__ double dipole_dipole64(const D3 &ua, double ma, const D3 &ub, double mb, const D3 &r,
                                                  const MolDesc &d) {
    const double r2 = dot3(r, r);
    const double r1 = sqrt(r2);
    if (!(r1 < d.rcd)) return 0.0;
    const double q = r1 / d.rcd;
    const double bf = d.rfBd * q * q * q;
    const double r2i = 1.0 / r2;
    const double dt = dot3(ua, ub);
    const double T = (3.0 * dot3(ua, r) * dot3(ub, r) * r2i - dt) + dt * bf;
    return d.lBd * (-(ma * mb) * T * sqrt(r2i) * r2i);
}

// Total energy in FP64, as Energybase::systemEnergy sums it (energy.h:169-180):
// out[0] += intermolecular pairs, out[1] += intramolecular pairs
// (NonbondedVector::g_internal, energy.h:1207-1216). Grid: x over sites i
// (256 per block), y over chunks of j.
__global__ void mol_total_kernel(const MolDesc *__restrict__ descs, int chunk, double *out) {
    const MolDesc &d = descs[0];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int jb = blockIdx.y * chunk, je = min(jb + chunk, d.N);
    double inter = 0.0, intra = 0.0;
    if (i < d.N) {
        const int64_t *P = d.rep_pos;
        const int ti = d.pos4[i].w & 0xFF;
        const double qi = d.qtype[ti], mi = d.mus[i];
        const D3 ui = {d.rep_mu[3 * i], d.rep_mu[3 * i + 1], d.rep_mu[3 * i + 2]};
        const D3 vi = {ui.x * mi, ui.y * mi, ui.z * mi};
        for (int j = max(jb, i + 1); j < je; j++) {
            const int tj = d.pos4[j].w & 0xFF;
            const D3 r = {(double)(int64_t)((uint64_t)P[3 * i] - (uint64_t)P[3 * j]) * d.s64d[0],
                          (double)(int64_t)((uint64_t)P[3 * i + 1] - (uint64_t)P[3 * j + 1]) * d.s64d[1],
                          (double)(int64_t)((uint64_t)P[3 * i + 2] - (uint64_t)P[3 * j + 2]) * d.s64d[2]};
            const double r2 = dot3(r, r);
            double u = 0.0;
            // CoulombGalore (kappa = 0)
            const int t = ti * d.nt + tj;
            if (r2 < (double)d.rc2) {
                const double rr = sqrt(r2);
                const double q = rr / d.rcd, q2 = q * q;
                const double a2 = -66.0 * 1494.0 / 56916.0;
                const double Q = (q - 1.0) * (q - 1.0) * (q - 1.0) *
                                 (5.0 / 22.0 * q2 * a2 + 9.0 / 22.0 * q * a2 - 0.6 * q2 - 1.2 * q - 1.0);
                u += d.lBd * (double)d.qtype[ti] * (double)d.qtype[tj] / rr * Q;
            }
            // LennardJonesLB
            {
                double x = d.s2d[t] / r2;
                x = x * x * x;
                u += d.eps4d[t] * (x * x - x);
            }
            const double mj = d.mus[j];
            if (mi != 0.0 || mj != 0.0) {
                const D3 uj = {d.rep_mu[3 * j], d.rep_mu[3 * j + 1], d.rep_mu[3 * j + 2]};
                const D3 vj = {uj.x * mj, uj.y * mj, uj.z * mj};
                u += ion_dipole64(qi, vi, (double)d.qtype[tj], vj, r, d.lBd);
                if (mi != 0.0 && mj != 0.0) u += dipole_dipole64(ui, mi, uj, mj, r, d);
            }
            if (i / d.gs == j / d.gs) intra += u;
            else inter += u;
        }
    }
    // block sums, then one atomic per block
    __shared__ double red[2][32];
    for (int o = 16; o > 0; o >>= 1) {
        inter += __shfl_xor_sync(0xffffffffu, inter, o);
        intra += __shfl_xor_sync(0xffffffffu, intra, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = inter;
        red[1][threadIdx.x >> 5] = intra;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            a += red[0][w];
            b += red[1][w];
        }
        atomicAdd(&out[0], a);
        atomicAdd(&out[1], b);
    }
}

}  // namespace fgm

// ==================================================================== host side
struct fg_molsys {
    fg_params P{};
    int N = 0, gs = 0, M = 0, D = 0;
    int device = 0;
    int C = 1;          // CTAs per system (thread-block cluster)
    int max_cluster = 1;
    cudaStream_t stream = nullptr;
    fgm::MolDesc desc{};
    fgm::MolDesc *d_desc = nullptr;
    int64_t *rep_pos = nullptr, *rep_cm = nullptr;
    double *rep_mu = nullptr, *mus = nullptr;
    int4 *pos4 = nullptr, *dip_pos4 = nullptr;
    int32_t *site_dip = nullptr, *dip_site = nullptr;
    float4 *dip4 = nullptr;
    fgm::MolTrial *trials = nullptr;
    int64_t trials_cap = 0;
    float2 *log_du = nullptr;
    uint8_t *log_acc = nullptr;
    int64_t log_cap = 0;
    fgm::MolScalars *sc = nullptr;
    int64_t *expl_pos = nullptr;
    double *expl_mu = nullptr, *eval_du = nullptr, *tot = nullptr;
    int64_t *expl_cm = nullptr;
    int pending = -1;   // molecule of an evaluated explicit trial awaiting fg_mol_commit
    double pending_du = 0.0;
    int64_t n_stream = 0;   // trials in the staged stream
    bool staged = false;    // a stream is staged and not yet run (it occupies the trial buffer)
    int64_t acc0 = 0;       // accepted count when the stream was staged
    bool has_cm = false;
    bool state_set = false;
    std::vector<int32_t> types;
    std::vector<double> mus_h;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    size_t device_bytes = 0;
};

namespace {

int mol_dmalloc(fg_molsys *h, void **p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    h->device_bytes += bytes;
    return FG_OK;
}
#define MOL_DMALLOC(ptr, bytes)                                        \
    do {                                                               \
        int rc_ = mol_dmalloc(h, (void **)&(ptr), (size_t)(bytes));    \
        if (rc_) return rc_;                                           \
    } while (0)

void mol_free(fg_molsys *h) {
    void *ptrs[] = {h->d_desc, h->rep_pos, h->rep_cm, h->rep_mu, h->mus, h->pos4, h->dip_pos4,
                    h->site_dip, h->dip_site, h->dip4, h->trials, h->log_du, h->log_acc, h->sc,
                    h->expl_pos, h->expl_mu, h->eval_du, h->tot, h->expl_cm};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
}

// Geometry::anyCenter with equal masses (geometry.h:714-738) in fixed point:
// origin at the middle site, minimum-image offsets, mean, wrapped.
void mol_mass_center(const int64_t *X, int front, int gs, int64_t out[3]) {
    const int o = front + (int)((gs - 1) * 0.5);
    for (int a = 0; a < 3; a++) {
        long double s = 0;
        for (int i = front; i < front + gs; i++) s += (long double)(int64_t)((uint64_t)X[3 * i + a] - (uint64_t)X[3 * o + a]);
        out[a] = (int64_t)((uint64_t)X[3 * o + a] + (uint64_t)(int64_t)llroundl(s / gs));
    }
}

size_t mol_smem_bytes(const fg_molsys *h, int C, bool slice_smem) {
    size_t off[16];
    fgm::mol_smem_layout((h->N + C - 1) / C, (h->D + C - 1) / C, h->gs, slice_smem, off);
    return off[6];
}

struct MolLaunch {
    void (*fn)(const fgm::MolDesc *);
    size_t smem;
    bool cluster;
};

template <bool EVAL>
int mol_pick(const fg_molsys *h, MolLaunch &L) {
    const bool slice = mol_smem_bytes(h, h->C, true) <= 200 * 1024;
    const bool cl = h->C > 1;
    L.smem = mol_smem_bytes(h, h->C, slice);
    L.cluster = cl;
    if (slice) L.fn = cl ? fgm::mol_sweep_kernel<true, true, EVAL> : fgm::mol_sweep_kernel<true, false, EVAL>;
    else L.fn = cl ? fgm::mol_sweep_kernel<false, true, EVAL> : fgm::mol_sweep_kernel<false, false, EVAL>;
    cudaError_t e = cudaFuncSetAttribute((const void *)L.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, "shared memory attribute: %s", cudaGetErrorString(e));
    if (cl) {
        e = cudaFuncSetAttribute((const void *)L.fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return fail(FG_ERR_CUDA, "cluster attribute: %s", cudaGetErrorString(e));
    }
    return FG_OK;
}

int mol_launch(const fg_molsys *h, const MolLaunch &L, const fgm::MolDesc *descs, int n_systems, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(n_systems * h->C));
    cfg.blockDim = dim3(fgm::kMolThreads);
    cfg.dynamicSmemBytes = L.smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    if (L.cluster) {
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)h->C;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    cudaError_t e = cudaLaunchKernelEx(&cfg, L.fn, descs);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, "molecule sweep launch: %s", cudaGetErrorString(e));
    return FG_OK;
}

// Largest cluster the device runs for this kernel's shared memory (<= 16).
int mol_max_cluster(fg_molsys *h) {
    int best = 1;
    for (int c : {16, 8, 4, 2}) {
        const int saved = h->C;
        h->C = c;
        MolLaunch L;
        int rc = mol_pick<false>(h, L);
        h->C = saved;
        if (rc) continue;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)c);
        cfg.blockDim = dim3(fgm::kMolThreads);
        cfg.dynamicSmemBytes = L.smem;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)c;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, (const void *)L.fn, &cfg) == cudaSuccess && n > 0) {
            best = c;
            break;
        }
        cudaGetLastError();
    }
    return best;
}

int mol_alloc_replicas(fg_molsys *h, int C) {
    if (h->rep_pos) cudaFree(h->rep_pos);
    if (h->rep_mu) cudaFree(h->rep_mu);
    if (h->rep_cm) cudaFree(h->rep_cm);
    h->rep_pos = nullptr;
    h->rep_mu = nullptr;
    h->rep_cm = nullptr;
    MOL_DMALLOC(h->rep_pos, (size_t)C * h->N * 3 * sizeof(int64_t));
    MOL_DMALLOC(h->rep_mu, (size_t)C * h->N * 3 * sizeof(double));
    MOL_DMALLOC(h->rep_cm, (size_t)C * h->M * 3 * sizeof(int64_t));
    h->desc.rep_pos = h->rep_pos;
    h->desc.rep_mu = h->rep_mu;
    h->desc.rep_cm = h->rep_cm;
    return FG_OK;
}

int mol_push_desc(fg_molsys *h) {
    h->desc.C = h->C;
    CK(cudaMemcpyAsync(h->d_desc, &h->desc, sizeof(fgm::MolDesc), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

int mol_ensure_trials(fg_molsys *h, int64_t n, bool log) {
    n = std::max<int64_t>(n, 1);
    if (n > h->trials_cap) {
        if (h->trials) cudaFree(h->trials);
        h->trials = nullptr;
        MOL_DMALLOC(h->trials, n * sizeof(fgm::MolTrial));
        h->trials_cap = n;
    }
    if (log && n > h->log_cap) {
        if (h->log_du) cudaFree(h->log_du);
        if (h->log_acc) cudaFree(h->log_acc);
        h->log_du = nullptr;
        h->log_acc = nullptr;
        MOL_DMALLOC(h->log_du, n * sizeof(float2));
        MOL_DMALLOC(h->log_acc, n);
        h->log_cap = n;
    }
    h->desc.trials = h->trials;
    return FG_OK;
}

int mol_read_scalars(fg_molsys *h, fgm::MolScalars &s) {
    CK(cudaMemcpyAsync(&s, h->sc, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FG_OK;
}
int mol_write_scalars(fg_molsys *h, const fgm::MolScalars &s) {
    CK(cudaMemcpyAsync(h->sc, &s, sizeof(s), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

// Copy replica 0 into replicas 1..C-1 (after the state changed through it).
int mol_sync_replicas(fg_molsys *h) {
    for (int r = 1; r < h->C; r++) {
        CK(cudaMemcpyAsync(h->rep_pos + (size_t)r * h->N * 3, h->rep_pos, (size_t)h->N * 3 * sizeof(int64_t),
                           cudaMemcpyDeviceToDevice, h->stream));
        CK(cudaMemcpyAsync(h->rep_mu + (size_t)r * h->N * 3, h->rep_mu, (size_t)h->N * 3 * sizeof(double),
                           cudaMemcpyDeviceToDevice, h->stream));
        CK(cudaMemcpyAsync(h->rep_cm + (size_t)r * h->M * 3, h->rep_cm, (size_t)h->M * 3 * sizeof(int64_t),
                           cudaMemcpyDeviceToDevice, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

int mol_total(fg_molsys *h, double out[2]) {
    CK(cudaMemsetAsync(h->tot, 0, 2 * sizeof(double), h->stream));
    const int chunk = 2048;
    dim3 grid((unsigned)((h->N + 255) / 256), (unsigned)((h->N + chunk - 1) / chunk));
    fgm::mol_total_kernel<<<grid, 256, 0, h->stream>>>(h->d_desc, chunk, h->tot);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, h->tot, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

// MolTrial records from the reference's draws (or any explicit stream).
void mol_make_trials(const fg_molsys *h, int64_t n, const int32_t *mol, const double *axis, const double *angle,
                     const int32_t *center, const double *trans, const double *u, int rotate, int translate,
                     std::vector<fgm::MolTrial> &out) {
    out.resize(n);
    for (int64_t k = 0; k < n; k++) {
        fgm::MolTrial &t = out[k];
        t = fgm::MolTrial{};
        t.g = mol[k];
        t.flags = (rotate ? 1 : 0) | (translate ? 2 : 0);
        t.center = center ? center[k] : 0;
        t.qw = 1.0;
        if (rotate) {
            double ax = axis[3 * k], ay = axis[3 * k + 1], az = axis[3 * k + 2];
            const double nrm = std::sqrt(ax * ax + ay * ay + az * az);
            ax /= nrm; ay /= nrm; az /= nrm;
            const double ha = 0.5 * angle[k], sh = std::sin(ha);
            t.qw = std::cos(ha);
            t.qx = sh * ax; t.qy = sh * ay; t.qz = sh * az;
        }
        if (translate)
            for (int a = 0; a < 3; a++) t.t[a] = to_fix(trans[3 * k + a], h->P.box[a]);
        // Movebase::metropolis (move.h:567-573): reject iff u > exp(-dU)
        const double thr = -std::log(u[k]);
        const float2 f = split_df(thr);
        t.thr_hi = f.x;
        t.thr_lo = f.y;
        if (u[k] <= 0.0) { t.thr_hi = INFINITY; t.thr_lo = 0.0f; }
    }
}

// Stage a trial stream: validate, build MolTrial records, upload, reset the
// stream cursor and per-stream sums.
int mol_upload(fg_molsys *h, int64_t n, const int32_t *mol, const double *axis, const double *angle,
               const int32_t *center, const double *trans, const double *u, int rotate, int translate, bool log) {
    if (!h || n < 0 || (n > 0 && (!mol || !u))) return fail(FG_ERR_INVALID, "bad argument");
    if (rotate && n > 0 && (!axis || !angle)) return fail(FG_ERR_INVALID, "rotation needs axis and angle");
    if (translate && n > 0 && !trans) return fail(FG_ERR_INVALID, "translation needs trans");
    if (!h->state_set) return fail(FG_ERR_STATE, "fg_mol_set_state first");
    if (h->pending >= 0) return fail(FG_ERR_STATE, "a trial is pending: call fg_mol_commit");
    for (int64_t k = 0; k < n; k++) {
        if (mol[k] < 0 || mol[k] >= h->M) return fail(FG_ERR_INVALID, "molecule index out of range at %lld", (long long)k);
        if (center && (center[k] < 0 || center[k] > 2)) return fail(FG_ERR_INVALID, "bad centre kind");
    }
    int rc = mol_ensure_trials(h, n, log);
    if (rc) return rc;
    std::vector<fgm::MolTrial> tr;
    mol_make_trials(h, n, mol, axis, angle, center, trans, u, rotate, translate, tr);
    if (n > 0) CK(cudaMemcpyAsync(h->trials, tr.data(), n * sizeof(fgm::MolTrial), cudaMemcpyHostToDevice, h->stream));
    fgm::MolScalars s0;
    rc = mol_read_scalars(h, s0);
    if (rc) return rc;
    h->acc0 = s0.n_accepted;
    fgm::MolScalars s = s0;
    s.cursor = 0;
    s.n_trials = n;
    s.u_hi = s.u_lo = 0.0f;
    s.error = 0;
    rc = mol_write_scalars(h, s);
    if (rc) return rc;
    h->n_stream = n;
    h->staged = true;
    h->desc.log_du = log ? h->log_du : nullptr;
    h->desc.log_acc = log ? h->log_acc : nullptr;
    h->desc.expl_pos = nullptr;
    h->desc.expl_mu = nullptr;
    h->desc.expl_cm = nullptr;
    return mol_push_desc(h);
}

// Run the staged streams of several systems in one launch per chunk (one
// cluster of C CTAs per system); launches hold at most kChunk trials each.
int mol_run(fg_molsys *const *sys, int n, fg_sweep_stats *per, fg_sweep_stats *total) {
    if (!sys || n < 1) return fail(FG_ERR_INVALID, "bad argument");
    fg_molsys *h0 = sys[0];
    size_t smem_slice = 0, smem_flat = 0;
    bool all_slice = true;
    int64_t maxn = 0;
    for (int i = 0; i < n; i++) {
        fg_molsys *h = sys[i];
        if (!h || !h->state_set) return fail(FG_ERR_STATE, "system %d has no state", i);
        if (h->C != h0->C) return fail(FG_ERR_INVALID, "systems must share the cluster size");
        if (h->device != h0->device) return fail(FG_ERR_INVALID, "systems must share the device");
        const size_t a = mol_smem_bytes(h, h->C, true);
        if (a > 200 * 1024) all_slice = false;
        smem_slice = std::max(smem_slice, a);
        smem_flat = std::max(smem_flat, mol_smem_bytes(h, h->C, false));
        maxn = std::max(maxn, h->n_stream);
        CK(cudaStreamSynchronize(h->stream));
    }
    MolLaunch L;
    L.cluster = h0->C > 1;
    L.smem = all_slice ? smem_slice : smem_flat;
    if (all_slice) L.fn = L.cluster ? fgm::mol_sweep_kernel<true, true, false> : fgm::mol_sweep_kernel<true, false, false>;
    else L.fn = L.cluster ? fgm::mol_sweep_kernel<false, true, false> : fgm::mol_sweep_kernel<false, false, false>;
    CK(cudaFuncSetAttribute((const void *)L.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
    if (L.cluster) CK(cudaFuncSetAttribute((const void *)L.fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaStream_t st = h0->stream;
    const fgm::MolDesc *descs = h0->d_desc;
    fgm::MolDesc *tmp = nullptr;
    if (n > 1) {
        std::vector<fgm::MolDesc> v(n);
        for (int i = 0; i < n; i++) v[i] = sys[i]->desc;
        CK(cudaMalloc(&tmp, n * sizeof(fgm::MolDesc)));
        CK(cudaMemcpyAsync(tmp, v.data(), n * sizeof(fgm::MolDesc), cudaMemcpyHostToDevice, st));
        descs = tmp;
    }
    std::vector<fgm::MolScalars> s0(n), s1(n);
    for (int i = 0; i < n; i++) {
        CK(cudaMemcpyAsync(&s0[i], sys[i]->sc, sizeof(fgm::MolScalars), cudaMemcpyDeviceToHost, st));
    }
    const int64_t kChunk = 65536;
    const int64_t nl = (maxn + kChunk - 1) / kChunk;
    std::vector<int64_t> ends((size_t)nl * n);
    CK(cudaEventRecord(h0->ev0, st));
    int rc = FG_OK;
    for (int64_t c = 0; c < nl && !rc; c++) {
        for (int i = 0; i < n; i++) {
            int64_t &e = ends[(size_t)c * n + i];
            e = std::min(sys[i]->n_stream, (c + 1) * kChunk);
            CK(cudaMemcpyAsync(&sys[i]->sc->n_trials, &e, sizeof(int64_t), cudaMemcpyHostToDevice, st));
        }
        rc = mol_launch(h0, L, descs, n, st);
    }
    CK(cudaEventRecord(h0->ev1, st));
    CK(cudaEventSynchronize(h0->ev1));
    for (int i = 0; i < n; i++) sys[i]->staged = false;
    if (tmp) cudaFree(tmp);
    if (rc) return rc;
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, h0->ev0, h0->ev1));
    for (int i = 0; i < n; i++)
        CK(cudaMemcpyAsync(&s1[i], sys[i]->sc, sizeof(fgm::MolScalars), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    fg_sweep_stats tot{};
    int errs = 0;
    for (int i = 0; i < n; i++) {
        fg_sweep_stats x{};
        x.trials = s1[i].cursor;
        x.accepted = s1[i].n_accepted - sys[i]->acc0;
        x.energy_change = df_val(s1[i].u_hi, s1[i].u_lo);
        x.device_ms = ms;
        x.sweep_kernel_ms = ms;
        x.sweep_launches = (int32_t)nl;
        x.error_flags = s1[i].error;
        x.kernel_launches = nl;
        errs |= s1[i].error;
        if (per) per[i] = x;
        tot.trials += x.trials;
        tot.accepted += x.accepted;
        tot.energy_change += x.energy_change;
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

}  // namespace

extern "C" {

int fg_mol_create(const fg_params *params, int32_t n_sites, int32_t sites_per_molecule, fg_molsys **out) {
    if (!params || !out) return fail(FG_ERR_INVALID, "null argument");
    *out = nullptr;
    const fg_params &P = *params;
    if (P.model != FG_MODEL_MULTIPOLE_RF) return fail(FG_ERR_INVALID, "fg_mol_create needs FG_MODEL_MULTIPOLE_RF");
    if (sites_per_molecule < 1 || sites_per_molecule > fgm::kMaxGroupSites)
        return fail(FG_ERR_INVALID, "sites per molecule must be 1..%d", fgm::kMaxGroupSites);
    if (n_sites < 2 * sites_per_molecule || n_sites % sites_per_molecule)
        return fail(FG_ERR_INVALID, "site count must be a multiple (>= 2) of the molecule size");
    if (n_sites >= (1 << 23)) return fail(FG_ERR_CAPACITY, "at most 2^23 sites");
    if (P.n_types < 1 || P.n_types > FG_MAX_TYPES) return fail(FG_ERR_INVALID, "bad type count");
    const double Lmin = std::min(P.box[0], std::min(P.box[1], P.box[2]));
    if (!(P.rf_cutoff > 0) || !(P.rf_cutoff < 0.5 * Lmin)) return fail(FG_ERR_INVALID, "cutoff must be in (0, L/2)");
    if (!(P.bjerrum > 0) || !(P.rf_eps_r > 0) || !(P.rf_eps_rf > 0)) return fail(FG_ERR_INVALID, "bad dielectric");
    fg_molsys *h = new fg_molsys();
    h->P = P;
    h->N = n_sites;
    h->gs = sites_per_molecule;
    h->M = n_sites / sites_per_molecule;
    auto bail = [&](int rc) {
        mol_free(h);
        delete h;
        return rc;
    };
    if (cudaGetDevice(&h->device) != cudaSuccess) return bail(fail(FG_ERR_CUDA, "no CUDA device"));
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(FG_ERR_CUDA, "stream"));
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);
    fgm::MolDesc &d = h->desc;
    d.N = h->N;
    d.gs = h->gs;
    d.M = h->M;
    d.nt = P.n_types;
    bool uniform = true;
    for (int i = 0; i < P.n_types; i++)
        if (P.type_sigma[i] != P.type_sigma[0] || P.type_eps[i] != P.type_eps[0]) uniform = false;
    d.uniform_lj = uniform ? 1 : 0;
    for (int a = 0; a < 3; a++) {
        d.s32[a] = (float)(P.box[a] / 4294967296.0);
        d.sc9[a] = (float)(512.0 * P.box[a] / 4294967296.0);
        d.s32sqd[a] = (P.box[a] / 4294967296.0) * (P.box[a] / 4294967296.0);
        d.s64d[a] = P.box[a] / TWO64;
        d.inv64d[a] = TWO64 / P.box[a];
    }
    const double rc = P.rf_cutoff;
    d.lB = (float)P.bjerrum;
    d.lBd = P.bjerrum;
    d.rc2 = (float)(rc * rc);
    d.rc2near = (float)((rc + 0.05) * (rc + 0.05));
    d.rc1i = (float)(1.0 / rc);
    d.rcd = rc;
    const double a2 = -66.0 * 1494.0 / 56916.0;   // CoulombGalore Q5 coefficient at kappa = 0
    d.A5 = (float)(5.0 / 22.0 * a2 - 0.6);
    d.B5 = (float)(9.0 / 22.0 * a2 - 1.2);
    d.rfBd = -(2 * (P.rf_eps_rf - P.rf_eps_r) / (2 * P.rf_eps_rf + P.rf_eps_r)) / P.rf_eps_r;
    d.rfB = (float)d.rfBd;
    d.cubic = (P.box[0] == P.box[1] && P.box[1] == P.box[2]) ? 1 : 0;
    d.s32sq = (float)((P.box[0] / 4294967296.0) * (P.box[0] / 4294967296.0));
    {
        const double u = rc / (P.box[0] / 4294967296.0);   // rc in high-word units
        d.rc2int = (long long)std::ceil(u * u);
    }
    d.kT = (float)(P.kT_scale > 0 ? P.kT_scale : 1.0);
    const int nt = P.n_types;
    for (int i = 0; i < nt; i++) {
        d.qtype[i] = (float)P.type_charge[i];
        for (int j = 0; j < nt; j++) {
            const double sig = 0.5 * (P.type_sigma[i] + P.type_sigma[j]);
            const double e4 = 4 * std::sqrt(P.type_eps[i] * P.type_eps[j]);
            d.s2[i * nt + j] = (float)(sig * sig);
            d.eps4[i * nt + j] = (float)e4;
            d.s2d[i * nt + j] = sig * sig;
            d.eps4d[i * nt + j] = e4;
            d.lbqq[i * nt + j] = (float)(P.bjerrum * P.type_charge[i] * P.type_charge[j]);
        }
    }
    if (uniform) {
        d.s2[0] = (float)(P.type_sigma[0] * P.type_sigma[0]);
        d.eps4[0] = (float)(4 * P.type_eps[0]);
    }
    int rc_;
#define TRY(x)                 \
    do {                       \
        rc_ = (x);             \
        if (rc_) return bail(rc_); \
    } while (0)
    TRY(mol_dmalloc(h, (void **)&h->d_desc, sizeof(fgm::MolDesc)));
    TRY(mol_dmalloc(h, (void **)&h->mus, (size_t)h->N * sizeof(double)));
    TRY(mol_dmalloc(h, (void **)&h->pos4, (size_t)h->N * sizeof(int4)));
    TRY(mol_dmalloc(h, (void **)&h->site_dip, (size_t)h->N * sizeof(int32_t)));
    TRY(mol_dmalloc(h, (void **)&h->sc, sizeof(fgm::MolScalars)));
    TRY(mol_dmalloc(h, (void **)&h->expl_pos, (size_t)h->gs * 3 * sizeof(int64_t)));
    TRY(mol_dmalloc(h, (void **)&h->expl_mu, (size_t)h->gs * 3 * sizeof(double)));
    TRY(mol_dmalloc(h, (void **)&h->expl_cm, 3 * sizeof(int64_t)));
    TRY(mol_dmalloc(h, (void **)&h->eval_du, sizeof(double)));
    TRY(mol_dmalloc(h, (void **)&h->tot, 2 * sizeof(double)));
    d.mus = h->mus;
    d.pos4 = h->pos4;
    d.site_dip = h->site_dip;
    d.sc = h->sc;
    d.eval_du = h->eval_du;
    h->max_cluster = mol_max_cluster(h);
    // default: enough CTAs that each owns <= ~1250 sites, within what the device runs
    int C = 1;
    while (C < h->max_cluster && (h->N + C - 1) / C > 1250) C *= 2;
    h->C = C;
    TRY(mol_alloc_replicas(h, C));
    TRY(mol_ensure_trials(h, 1, false));
    fgm::MolScalars s{};
    TRY(mol_write_scalars(h, s));
#undef TRY
    *out = h;
    return FG_OK;
}

int fg_mol_destroy(fg_molsys *h) {
    if (!h) return FG_OK;
    cudaStreamSynchronize(h->stream);
    mol_free(h);
    delete h;
    return FG_OK;
}

int fg_mol_set_state(fg_molsys *h, const double *xyz, const double *mu_unit, const double *mu_scalar,
                     const int32_t *type_ids, const double *mass_centers) {
    if (!h || !xyz || !type_ids) return fail(FG_ERR_INVALID, "null argument");
    const int N = h->N;
    std::vector<int64_t> X(3 * (size_t)N), CM(3 * (size_t)h->M);
    std::vector<double> MU(3 * (size_t)N, 0.0);
    std::vector<int4> p4(N);
    std::vector<int32_t> sd(N, -1), ds;
    h->types.assign(type_ids, type_ids + N);
    h->mus_h.assign(N, 0.0);
    for (int i = 0; i < N; i++) {
        if (type_ids[i] < 0 || type_ids[i] >= h->P.n_types) return fail(FG_ERR_INVALID, "bad type id at %d", i);
        for (int a = 0; a < 3; a++) {
            if (!std::isfinite(xyz[3 * i + a])) return fail(FG_ERR_INVALID, "non-finite position at %d", i);
            X[3 * i + a] = to_fix(xyz[3 * i + a], h->P.box[a]);
        }
        const double m = mu_scalar ? mu_scalar[i] : 0.0;
        if (m != 0.0) {
            if (!mu_unit) return fail(FG_ERR_INVALID, "dipole scalars need unit vectors");
            for (int a = 0; a < 3; a++) MU[3 * i + a] = mu_unit[3 * i + a];
            sd[i] = (int32_t)ds.size();
            ds.push_back(i);
        } else if (mu_unit) {
            for (int a = 0; a < 3; a++) MU[3 * i + a] = mu_unit[3 * i + a];
        }
        h->mus_h[i] = m;
        p4[i] = make_int4(hi32h(X[3 * i]), hi32h(X[3 * i + 1]), hi32h(X[3 * i + 2]), type_ids[i]);
    }
    for (int g = 0; g < h->M; g++) {
        if (mass_centers)
            for (int a = 0; a < 3; a++) CM[3 * g + a] = to_fix(mass_centers[3 * g + a], h->P.box[a]);
        else
            mol_mass_center(X.data(), g * h->gs, h->gs, &CM[3 * g]);
    }
    const int D = (int)ds.size();
    if (D != h->D || !h->dip4) {
        if (h->dip4) cudaFree(h->dip4);
        if (h->dip_pos4) cudaFree(h->dip_pos4);
        if (h->dip_site) cudaFree(h->dip_site);
        h->dip4 = nullptr;
        h->dip_pos4 = nullptr;
        h->dip_site = nullptr;
        MOL_DMALLOC(h->dip4, (size_t)std::max(D, 1) * sizeof(float4));
        MOL_DMALLOC(h->dip_pos4, (size_t)std::max(D, 1) * sizeof(int4));
        MOL_DMALLOC(h->dip_site, (size_t)std::max(D, 1) * sizeof(int32_t));
        h->D = D;
    }
    std::vector<float4> d4(std::max(D, 1));
    std::vector<int4> dp4(std::max(D, 1));
    for (int k = 0; k < D; k++) {
        const int i = ds[k];
        const double m = h->mus_h[i];
        d4[k] = make_float4((float)(MU[3 * i] * m), (float)(MU[3 * i + 1] * m), (float)(MU[3 * i + 2] * m), (float)m);
        dp4[k] = make_int4(p4[i].x, p4[i].y, p4[i].z, (i << 8) | type_ids[i]);
    }
    fgm::MolDesc &d = h->desc;
    d.D = D;
    d.dip4 = h->dip4;
    d.dip_pos4 = h->dip_pos4;
    d.dip_site = h->dip_site;
    cudaStream_t st = h->stream;
    for (int r = 0; r < h->C; r++) {
        CK(cudaMemcpyAsync(h->rep_pos + (size_t)r * N * 3, X.data(), X.size() * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(h->rep_mu + (size_t)r * N * 3, MU.data(), MU.size() * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(h->rep_cm + (size_t)r * h->M * 3, CM.data(), CM.size() * 8, cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemcpyAsync(h->mus, h->mus_h.data(), (size_t)N * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(h->pos4, p4.data(), (size_t)N * sizeof(int4), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(h->site_dip, sd.data(), (size_t)N * 4, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(h->dip4, d4.data(), (size_t)std::max(D, 1) * sizeof(float4), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(h->dip_pos4, dp4.data(), (size_t)std::max(D, 1) * sizeof(int4), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(h->dip_site, ds.empty() ? sd.data() : ds.data(), (size_t)std::max(D, 1) * 4,
                       cudaMemcpyHostToDevice, st));
    int rc = mol_push_desc(h);
    if (rc) return rc;
    double tot[2];
    rc = mol_total(h, tot);
    if (rc) return rc;
    fgm::MolScalars s{};
    const float2 u = split_df(tot[0] + tot[1]);
    s.utot_hi = u.x;
    s.utot_lo = u.y;
    rc = mol_write_scalars(h, s);
    if (rc) return rc;
    h->pending = -1;
    h->state_set = true;
    return FG_OK;
}

int fg_mol_get_state(fg_molsys *h, double *xyz, double *mu_unit, double *mass_centers) {
    if (!h || !h->state_set) return fail(FG_ERR_STATE, "no state");
    const int N = h->N;
    std::vector<int64_t> X(3 * (size_t)N), CM(3 * (size_t)h->M);
    std::vector<double> MU(3 * (size_t)N);
    CK(cudaMemcpyAsync(X.data(), h->rep_pos, X.size() * 8, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(MU.data(), h->rep_mu, MU.size() * 8, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(CM.data(), h->rep_cm, CM.size() * 8, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < N; i++)
        for (int a = 0; a < 3; a++) {
            if (xyz) xyz[3 * i + a] = from_fix(X[3 * i + a], h->P.box[a]);
            if (mu_unit) mu_unit[3 * i + a] = MU[3 * i + a];
        }
    if (mass_centers)
        for (int g = 0; g < h->M; g++)
            for (int a = 0; a < 3; a++) mass_centers[3 * g + a] = from_fix(CM[3 * g + a], h->P.box[a]);
    return FG_OK;
}

int fg_mol_set_cluster(fg_molsys *h, int32_t ctas) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (ctas < 1 || ctas > h->max_cluster || (ctas & (ctas - 1)))
        return fail(FG_ERR_INVALID, "cluster size must be a power of two in 1..%d", h->max_cluster);
    if (ctas == h->C) return FG_OK;
    std::vector<int64_t> X, CM;
    std::vector<double> MU;
    if (h->state_set) {
        X.resize(3 * (size_t)h->N);
        MU.resize(3 * (size_t)h->N);
        CM.resize(3 * (size_t)h->M);
        CK(cudaMemcpyAsync(X.data(), h->rep_pos, X.size() * 8, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(MU.data(), h->rep_mu, MU.size() * 8, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(CM.data(), h->rep_cm, CM.size() * 8, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    int rc = mol_alloc_replicas(h, ctas);
    if (rc) return rc;
    h->C = ctas;
    if (h->state_set) {
        for (int r = 0; r < ctas; r++) {
            CK(cudaMemcpyAsync(h->rep_pos + (size_t)r * h->N * 3, X.data(), X.size() * 8, cudaMemcpyHostToDevice,
                               h->stream));
            CK(cudaMemcpyAsync(h->rep_mu + (size_t)r * h->N * 3, MU.data(), MU.size() * 8, cudaMemcpyHostToDevice,
                               h->stream));
            CK(cudaMemcpyAsync(h->rep_cm + (size_t)r * h->M * 3, CM.data(), CM.size() * 8, cudaMemcpyHostToDevice,
                               h->stream));
        }
        CK(cudaStreamSynchronize(h->stream));
    }
    return mol_push_desc(h);
}

int fg_mol_get_cluster(fg_molsys *h, int32_t *ctas, int32_t *max_ctas) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (ctas) *ctas = h->C;
    if (max_ctas) *max_ctas = h->max_cluster;
    return FG_OK;
}

int fg_mol_trial_du(fg_molsys *h, int32_t molecule, const double *new_xyz, const double *new_mu_unit,
                    const double *new_mass_center, double *du) {
    if (!h || !new_xyz || !du) return fail(FG_ERR_INVALID, "null argument");
    if (!h->state_set) return fail(FG_ERR_STATE, "fg_mol_set_state first");
    if (h->pending >= 0) return fail(FG_ERR_STATE, "a trial is pending: call fg_mol_commit");
    if (h->staged) return fail(FG_ERR_STATE, "a staged stream is waiting: run it first");
    if (molecule < 0 || molecule >= h->M) return fail(FG_ERR_INVALID, "molecule index out of range");
    std::vector<int64_t> X(3 * (size_t)h->gs);
    for (int s = 0; s < h->gs; s++)
        for (int a = 0; a < 3; a++) X[3 * s + a] = to_fix(new_xyz[3 * s + a], h->P.box[a]);
    CK(cudaMemcpyAsync(h->expl_pos, X.data(), X.size() * 8, cudaMemcpyHostToDevice, h->stream));
    if (new_mu_unit)
        CK(cudaMemcpyAsync(h->expl_mu, new_mu_unit, (size_t)h->gs * 3 * 8, cudaMemcpyHostToDevice, h->stream));
    int64_t cm[3];
    if (new_mass_center) {
        for (int a = 0; a < 3; a++) cm[a] = to_fix(new_mass_center[a], h->P.box[a]);
        CK(cudaMemcpyAsync(h->expl_cm, cm, sizeof(cm), cudaMemcpyHostToDevice, h->stream));
    }
    fgm::MolTrial t{};
    t.g = molecule;
    t.flags = 4;
    t.qw = 1.0;
    CK(cudaMemcpyAsync(h->trials, &t, sizeof(t), cudaMemcpyHostToDevice, h->stream));
    h->desc.expl_pos = h->expl_pos;
    h->desc.expl_mu = new_mu_unit ? h->expl_mu : nullptr;
    h->desc.expl_cm = new_mass_center ? h->expl_cm : nullptr;
    h->desc.trials = h->trials;
    int rc = mol_push_desc(h);
    if (rc) return rc;
    MolLaunch L;
    rc = mol_pick<true>(h, L);
    if (rc) return rc;
    rc = mol_launch(h, L, h->d_desc, 1, h->stream);
    if (rc) return rc;
    CK(cudaMemcpyAsync(du, h->eval_du, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->pending = molecule;
    h->pending_du = *du;
    return FG_OK;
}

int fg_mol_commit(fg_molsys *h, int32_t accepted) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (h->pending < 0) return fail(FG_ERR_STATE, "no pending trial");
    const int g = h->pending;
    h->pending = -1;
    if (!accepted) return FG_OK;
    fgm::mol_commit_kernel<<<1, 64, 0, h->stream>>>(h->d_desc, g, 1, h->C);
    CK(cudaGetLastError());
    fgm::MolScalars s;
    int rc = mol_read_scalars(h, s);
    if (rc) return rc;
    s.n_accepted++;
    const double ut = df_val(s.utot_hi, s.utot_lo) + h->pending_du;
    const float2 f = split_df(ut);
    s.utot_hi = f.x;
    s.utot_lo = f.y;
    return mol_write_scalars(h, s);
}

// Reference draws for n TranslateRotate trials on one molecule kind
// ("permol"), consuming the global slump as move.h:1624-1685 and 567-573 do.
int fg_mol_draw_stream(uint32_t seed, int32_t n_molecules, int64_t n, double dp, double dprot,
                       int32_t center_rotation, int32_t *mol, double *axis, int32_t *center, double *angle,
                       double *trans, double *u) {
    if (n_molecules < 1 || n < 0 || (n > 0 && (!mol || !u))) return fail(FG_ERR_INVALID, "bad argument");
    std::mt19937 eng(seed);
    std::uniform_real_distribution<double> U(0, 1);
    for (int64_t k = 0; k < n; k++) {
        std::uniform_int_distribution<int> pick(0, n_molecules - 1);
        mol[k] = pick(eng);                                     // slump.element(gvec)
        double v[3] = {0, 0, 0}, ang = 0.0, t[3] = {0, 0, 0};
        int c = 0;
        if (dprot > 1e-6) {
            double r2;
            do {                                                // Point::ranunit (point.h:74-88)
                for (int a = 0; a < 3; a++) v[a] = (2 * U(eng) - 1) * 1.0;
                r2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
            } while (r2 > 1);
            const double s = std::sqrt(r2);
            for (int a = 0; a < 3; a++) v[a] /= s;
            if (!center_rotation) c = (U(eng) < 0.5) ? 1 : 2;
            ang = dprot * (U(eng) - 0.5);                       // slump.half()
        }
        if (dp > 1e-6)
            for (int a = 0; a < 3; a++) t[a] = 1.0 * dp * (U(eng) - 0.5);
        const double um = U(eng);                               // Movebase::metropolis
        for (int a = 0; a < 3; a++) {
            if (axis) axis[3 * k + a] = v[a];
            if (trans) trans[3 * k + a] = t[a];
        }
        if (center) center[k] = c;
        if (angle) angle[k] = ang;
        u[k] = um;
    }
    return FG_OK;
}

// n TranslateRotate trials on the device. rotate/translate say whether the
// move has dprot/dp above 1e-6 (move.h:1642, 1671); the arrays are the draws
// (fg_mol_draw_stream). acc/du (may be NULL) receive per-trial results.
int fg_mol_stream_upload(fg_molsys *h, int64_t n, const int32_t *mol, const double *axis, const double *angle,
                         const int32_t *center, const double *trans, const double *u, int32_t rotate,
                         int32_t translate) {
    return mol_upload(h, n, mol, axis, angle, center, trans, u, rotate, translate, false);
}

int fg_mol_run_many(fg_molsys *const *systems, int32_t n_systems, fg_sweep_stats *per_system, fg_sweep_stats *total) {
    return mol_run(systems, n_systems, per_system, total);
}

int fg_mol_sweep(fg_molsys *h, int64_t n, const int32_t *mol, const double *axis, const double *angle,
                 const int32_t *center, const double *trans, const double *u, int32_t rotate, int32_t translate,
                 uint8_t *acc, double *du, fg_sweep_stats *stats) {
    const bool log = acc || du;
    int rc = mol_upload(h, n, mol, axis, angle, center, trans, u, rotate, translate, log);
    if (rc) return rc;
    fg_sweep_stats st{};
    rc = mol_run(&h, 1, nullptr, &st);
    if (stats) *stats = st;
    if (rc) return rc;
    if (log && n > 0) {
        std::vector<float2> l(n);
        std::vector<uint8_t> a(n);
        CK(cudaMemcpyAsync(l.data(), h->log_du, n * sizeof(float2), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(a.data(), h->log_acc, n, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        for (int64_t k = 0; k < n; k++) {
            if (du) du[k] = df_val(l[k].x, l[k].y);
            if (acc) acc[k] = a[k];
        }
    }
    return FG_OK;
}

// comp = {intermolecular, intramolecular, total} in FP64 (systemEnergy).
int fg_mol_total_energy(fg_molsys *h, double *comp) {
    if (!h || !comp) return fail(FG_ERR_INVALID, "null argument");
    if (!h->state_set) return fail(FG_ERR_STATE, "no state");
    double t[2];
    int rc = mol_total(h, t);
    if (rc) return rc;
    comp[0] = t[0];
    comp[1] = t[1];
    comp[2] = t[1] + t[0];
    return FG_OK;
}

// Running total energy (initial total + accepted dU since fg_mol_set_state).
int fg_mol_running_energy(fg_molsys *h, double *u) {
    if (!h || !u) return fail(FG_ERR_INVALID, "null argument");
    fgm::MolScalars s;
    int rc = mol_read_scalars(h, s);
    if (rc) return rc;
    *u = df_val(s.utot_hi, s.utot_lo);
    return FG_OK;
}

int64_t fg_mol_device_bytes(fg_molsys *h) { return h ? (int64_t)h->device_bytes : 0; }

}  // extern "C"
