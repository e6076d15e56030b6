// C-ABI implementation, single systems: handle lifetime, uploads, launches
// and the host-side replay of the reference's random stream. Batches,
// parallel tempering and the job server are in fg_batch.cu (same
// translation unit). See include/faunus_gb300.h.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "faunus_gb300.h"
#include "fg_kernels.cu"
#include "fg_dh_block.cu"
#include "fg_ewald_block.cu"

using fg::SysDesc;
using fg::SysScalars;
using fg::Trial;

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(FG_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));     \
    } while (0)

const double TWO64 = 18446744073709551616.0;
const double TWO62 = 4611686018427387904.0;
const double PI = 3.14159265358979323846;

// x (Angstrom) -> 64-bit fixed point of the periodic box [-L/2, L/2)
int64_t to_fix(double x, double L) {
    double f = x / L;
    f -= std::floor(f + 0.5);
    return (int64_t)((uint64_t)(int64_t)llrint(f * TWO62) << 2);
}
double from_fix(int64_t X, double L) { return (double)X * (L / TWO64); }
int32_t hi32h(int64_t X) { return (int32_t)((uint64_t)(X + 0x80000000LL) >> 32); }
int16_t ext16h(int64_t X) {
    int32_t h = hi32h(X);
    int32_t rem = (int32_t)((uint64_t)X - ((uint64_t)(uint32_t)h << 32));
    return (int16_t)(rem >> 16);
}
float2 split_df(double v) {
    float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}
double df_val(float hi, float lo) { return (double)hi + (double)lo; }

int cell_of_h(const int64_t X[3], const int nc[3]) {
    int c[3];
    for (int a = 0; a < 3; a++) {
        uint32_t u = (uint32_t)hi32h(X[a]) + 0x80000000u;
        c[a] = (int)(((uint64_t)u * (uint32_t)nc[a]) >> 32);
    }
    return (c[2] * nc[1] + c[1]) * nc[0] + c[0];
}

}  // namespace

struct fg_system {
    fg_params P{};
    int N = 0, K = 0, kc = 0, model = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    SysDesc desc{};
    SysDesc *d_desc = nullptr;
    // device arrays
    int64_t *pos64 = nullptr;
    int4 *pos4 = nullptr;
    short4 *pos_ext = nullptr, *cell_ext = nullptr;
    uint8_t *ptype = nullptr;
    int32_t *cell_count = nullptr, *cell_pid = nullptr, *p_cell = nullptr, *p_slot = nullptr;
    int4 *cell_pos = nullptr;
    float4 *kvec = nullptr, *core_tab = nullptr, *core_tab2 = nullptr;
    uint32_t *kpack = nullptr;
    int2 *kseg = nullptr;
    int4 *rb_items = nullptr;
    int nseg = 0, n_rb_items = 0;
    longlong2 *qfix = nullptr, *qnew = nullptr;
    SysScalars *sc = nullptr;
    float2 *trial_out = nullptr, *corr = nullptr, *pair_part = nullptr;
    int64_t *req = nullptr, *dp_fix = nullptr;
    float2 *sc_tab = nullptr;
    Trial *trials = nullptr;
    int64_t trials_cap = 0, n_trials = 0;
    int32_t *raw_idx = nullptr;          // host trial arrays as uploaded (converted on the device)
    double *raw_disp = nullptr, *raw_u = nullptr;
    int64_t raw_cap = 0;
    float2 *log_du = nullptr;
    uint8_t *log_acc = nullptr;
    int64_t log_cap = 0;
    int64_t log_n = 0;             // trials of the last logged run (fg_log_get)
    bool log_batch = false;        // log this member's trials in batch runs (fg_batch_set_log)
    // host-side values
    std::vector<double> ak;
    std::vector<int32_t> types;
    double self_energy = 0, surf_c = 0, recip_c = 0;
    int threads = 0;
    int ctas = 0;                  // block-kernel CTAs per system (0: tuned cache / heuristic)
    // Ewald block kernel of a system alone on a cluster (fg_set_cluster)
    std::vector<int> n3;           // n-vectors of the k-vectors (3 per k)
    int eb_ctas = 0;               // requested cluster size (0: built-in choice)
    int4 *eb_ranges = nullptr;     // [1 + kEbMaxCluster]: one CTA's range, then the cluster's per rank
    int4 *cl_items = nullptr;      // rebuild items grouped by cluster rank
    int cl_c = 0;                  // cluster size the two above are built for
    int cl_kmax = 0;               // most k-vectors of one rank
    int cl_n_items = 0;
    int cl_max = 0;                // largest cluster that fits (0: not yet known)
    SysDesc *d_desc_cl = nullptr;  // the descriptor of cluster launches
    int batches = 0;               // live batches holding this system
    std::vector<double> charges;   // host copy of the uploaded charges (clones for tuning)
    bool use_cells = false, pos_smem = false;
    int nc[3] = {0, 0, 0};
    int cap = 0;
    bool trial_pending = false;
    bool state_set = false;
    int cnt_accepted_host = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    size_t device_bytes = 0;
};

namespace {

void free_all(fg_system *h) {
    void *ptrs[] = {h->d_desc, h->pos64, h->pos4, h->pos_ext, h->cell_ext, h->ptype, h->cell_count, h->cell_pid,
                    h->p_cell, h->p_slot, h->cell_pos, h->kvec, h->core_tab, h->core_tab2, h->kpack, h->qfix,
                    h->qnew, h->sc, h->trial_out, h->corr, h->pair_part, h->req, h->dp_fix, h->sc_tab, h->trials,
                    h->log_du, h->log_acc, h->kseg, h->rb_items, h->raw_idx, h->raw_disp, h->raw_u,
                    h->eb_ranges, h->cl_items, h->d_desc_cl};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
}

int dmalloc(fg_system *h, void **p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    h->device_bytes += bytes;
    return FG_OK;
}
#define DMALLOC(ptr, bytes)                                        \
    do {                                                           \
        int rc_ = dmalloc(h, (void **)&(ptr), (size_t)(bytes));    \
        if (rc_) return rc_;                                       \
    } while (0)

// k-vectors exactly as NonbondedEwald::kVectorChange (ewald.h:330-378), with
// its isotropic_pbc branch (n_y, n_z from 0, a factor 2 per positive
// component); returns n-vectors, k and A_k.
void enumerate_k(const fg_params &P, std::vector<int> &n3, std::vector<double> &ak, std::vector<double> &kv3) {
    double kc = P.ewald_cutoff_k, kc2 = kc * kc;
    int kcc = (int)std::ceil(kc);
    double maxL = std::max(P.box[0], std::max(P.box[1], P.box[2]));
    double check = 0.1 * (4 * PI * PI) / (maxL * maxL);
    double kappa = 1.0 / P.ewald_debye_length, alpha2 = P.ewald_alpha * P.ewald_alpha;
    const bool iso = P.ewald_isotropic_pbc != 0;
    const int lo = iso ? 0 : -kcc;
    for (int kx = 0; kx <= kcc; kx++)
        for (int ky = lo; ky <= kcc; ky++)
            for (int kz = lo; kz <= kcc; kz++) {
                double factor = kx > 0 ? 2.0 : 1.0;
                if (iso && ky > 0) factor *= 2.0;
                if (iso && kz > 0) factor *= 2.0;
                double k[3] = {2 * PI * (kx / P.box[0]), 2 * PI * (ky / P.box[1]), 2 * PI * (kz / P.box[2])};
                double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
                if (k2 < check) continue;
                if (P.ewald_spherical_sum && (kx * kx / kc2 + ky * ky / kc2 + kz * kz / kc2 > 1.0)) continue;
                n3.push_back(kx); n3.push_back(ky); n3.push_back(kz);
                kv3.push_back(k[0]); kv3.push_back(k[1]); kv3.push_back(k[2]);
                ak.push_back(factor * std::exp(-(k2 + kappa * kappa) / (4.0 * alpha2)) / (k2 + kappa * kappa));
            }
}

// Threads of the per-system CTA (multiple of 32, <= kSweepThreads).
// rb_item_list for items of at most L values of n.
bool rb_item_list_len(const std::vector<int> &n3, int kbeg, int kend, int L, std::vector<int4> &items) {
    items.clear();
    for (int k = kbeg; k < kend;) {
        int e = k + 1;
        while (e < kend && n3[3 * e] == n3[3 * k] && n3[3 * e + 1] == n3[3 * k + 1]) e++;
        // column [k, e): nz ascending
        std::map<int, int> kz;
        for (int q = k; q < e; q++) kz[n3[3 * q + 2]] = q;
        const int m = kz.rbegin()->first;
        for (auto &z : kz)
            if (!kz.count(-z.first)) return false;
        for (int n = 1; n <= m; n++)
            if (!kz.count(n)) return false;
        if (kz.size() != (size_t)(2 * m + (kz.count(0) ? 1 : 0))) return false;
        const int nlo = kz.count(0) ? 0 : 1;
        for (int n0 = nlo; n0 <= m; n0 += L) {
            const int len = std::min(L, m - n0 + 1);
            const int kp0 = kz[n0], kn0 = kz[-n0];
            // k(+n) and k(-n) run contiguously in the column
            for (int u = 0; u < len; u++)
                if (kz[n0 + u] != kp0 + u || kz[-(n0 + u)] != kn0 - u) return false;
            items.push_back(make_int4(kp0 | (len << 24), kn0 | (n0 << 24),
                                      (n3[3 * k] & 0xFF) | ((n3[3 * k + 1] & 0xFF) << 8), 0));
        }
        k = e;
    }
    std::stable_sort(items.begin(), items.end(), [](const int4 &a, const int4 &b) {
        const int la = a.x >> 24, lb = b.x >> 24;
        if (la != lb) return la > lb;
        return (a.y >> 24) < (b.y >> 24);
    });
    return true;
}

// Items of the block kernel's in-kernel rebuild (eb_rebuild). The k-vectors
// of one (nx, ny) form a contiguous run of nz = -m..m in enumeration order
// (kVectorChange's loop order, with nz = 0 missing from (0, 0)). An item
// takes up to kRbLen values n = n0, n0 + 1, ... of one such column and both
// k-vectors (nx, ny, +n) and (nx, ny, -n) of each (one for n = 0): e_z(-n) is
// the conjugate of e_z(n), so the four rounded products of a contribution
// serve both. The item length is the smallest (at most kRbLen) whose item
// count fits `slots` threads, so that the most warps take a share. Encoded as
// {kp0 | len << 24, kn0 | n0 << 24, nx & 0xFF | (ny & 0xFF) << 8, 0}:
// k(+n) = kp0 + (n - n0), k(-n) = kn0 - (n - n0). Sorted by length (longest
// first), then n0, so that warps run equal trip counts and read the same e_z
// entries. Returns false if a column is not symmetric in nz.
bool rb_item_list(const std::vector<int> &n3, int kbeg, int kend, int slots, std::vector<int4> &items) {
    for (int L = 1; L <= fg::kRbLen; L++) {
        if (!rb_item_list_len(n3, kbeg, kend, L, items)) return false;
        if ((int)items.size() <= slots) break;
    }
    return true;
}

// The k-vectors of a cluster of C CTAs: whole (nx, ny) columns (an item's
// +n and -n lie in one column), contiguous in enumeration order, cut where
// the running count comes nearest to r K / C; per rank its rebuild items
// (rb_item_list over its columns). ranges[r] = {k0, k1, i0, i1}. False if
// there are fewer columns than CTAs.
bool eb_cluster_plan(const std::vector<int> &n3, int K, int C, std::vector<int4> &ranges, std::vector<int4> &items,
                     int &kmax) {
    std::vector<int> starts;   // column starts
    for (int k = 0; k < K; k++)
        if (k == 0 || n3[3 * k] != n3[3 * (k - 1)] || n3[3 * k + 1] != n3[3 * (k - 1) + 1]) starts.push_back(k);
    const int ncol = (int)starts.size();
    if (ncol < C) return false;
    starts.push_back(K);
    std::vector<int> cut(C + 1, 0);   // column index where rank r starts
    cut[C] = ncol;
    for (int r = 1; r < C; r++) {
        const double target = (double)K * r / C;
        int best = cut[r - 1] + 1;
        for (int c = best; c <= ncol - (C - r); c++)
            if (std::fabs(starts[c] - target) < std::fabs(starts[best] - target)) best = c;
        cut[r] = best;
    }
    ranges.assign(C, make_int4(0, 0, 0, 0));
    items.clear();
    kmax = 0;
    for (int r = 0; r < C; r++) {
        const int k0 = starts[cut[r]], k1 = starts[cut[r + 1]];
        std::vector<int4> it;
        if (!rb_item_list(n3, k0, k1, fg::kEbThreads - 32, it)) return false;
        ranges[r] = make_int4(k0, k1, (int)items.size(), (int)(items.size() + it.size()));
        items.insert(items.end(), it.begin(), it.end());
        kmax = std::max(kmax, k1 - k0);
    }
    return true;
}
int sweep_threads(const fg_system *h) {
    int t = h->threads;
    if (t <= 0) {
        if (h->model == FG_MODEL_EWALD_WCA) t = (h->K + 3) / 4;   // ~4 k-vectors per thread
        else t = h->N / 8;                                      // ~8 particles per thread
        t = ((t + 31) / 32) * 32;
        t = std::max(128, std::min(fg::kSweepThreads, t));
    }
    return t;
}

size_t sweep_smem(const fg_system *h, bool pos_smem) {
    size_t off[8];
    return fg::smem_layout(h->N, h->K, h->kc, h->nc[0] * h->nc[1] * h->nc[2], h->model == FG_MODEL_EWALD_WCA, pos_smem,
                           h->use_cells, off);
}

using SweepFn = void (*)(const SysDesc *, int64_t, const float2 *);
using TrialFn = void (*)(const SysDesc *, const int64_t *, float2 *, const float2 *);
using CommitFn = void (*)(const SysDesc *, const int64_t *, const float2 *, const float2 *);

// Ewald systems run the block-of-trials kernel (fg_ewald_block.cu) when its
// shared memory fits; 512 threads per system.
size_t ewald_block_smem(const fg_system *h) {
    size_t off[19];
    return fg::eb_layout(h->N, h->K, h->nc[0] * h->nc[1] * h->nc[2], h->use_cells, 1, off);
}
bool ewald_block_ok(const fg_system *h) {
    return h->model == FG_MODEL_EWALD_WCA && h->K > 0 && h->N < (1 << 24) && !h->P.ewald_isotropic_pbc &&
           ewald_block_smem(h) + sizeof(SysDesc) + 1024 <= 227 * 1024;
}

SweepFn sweep_fn(const fg_system *h) {
    if (ewald_block_ok(h))
        return h->use_cells ? fg::ewald_block_kernel<true, false> : fg::ewald_block_kernel<false, false>;
    if (h->model == FG_MODEL_EWALD_WCA) {
        if (h->use_cells) return fg::sweep_kernel<fg::MODEL_EWALD, true, false>;
        if (h->pos_smem) return fg::sweep_kernel<fg::MODEL_EWALD, false, true>;
        return fg::sweep_kernel<fg::MODEL_EWALD, false, false>;
    }
    if (h->pos_smem) return fg::sweep_kernel<fg::MODEL_DHLJ, false, true>;
    return fg::sweep_kernel<fg::MODEL_DHLJ, false, false>;
}
TrialFn trial_fn(const fg_system *h) {
    if (h->model == FG_MODEL_EWALD_WCA)
        return h->use_cells ? fg::trial_kernel<fg::MODEL_EWALD, true> : fg::trial_kernel<fg::MODEL_EWALD, false>;
    return fg::trial_kernel<fg::MODEL_DHLJ, false>;
}
CommitFn commit_fn(const fg_system *h) {
    if (h->model == FG_MODEL_EWALD_WCA)
        return h->use_cells ? fg::commit_kernel<fg::MODEL_EWALD, true> : fg::commit_kernel<fg::MODEL_EWALD, false>;
    return fg::commit_kernel<fg::MODEL_DHLJ, false>;
}

int set_smem_attr(const void *fn, size_t bytes) {
    CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return FG_OK;
}

// ---------------------------------------------------------------- Ewald block sweeps on a cluster
// A system alone runs the Ewald block kernel on a thread-block cluster of C
// CTAs (fg_ewald_block.cu, CLUSTER): the k-vectors are split by columns
// (eb_cluster_plan), each CTA holding its share in shared memory.
SweepFn eb_cluster_fn(const fg_system *h) {
    return h->use_cells ? fg::ewald_block_kernel<true, true> : fg::ewald_block_kernel<false, true>;
}
size_t eb_cluster_smem(const fg_system *h, int C, int kmax) {
    size_t off[19];
    return fg::eb_layout(h->N, kmax, h->nc[0] * h->nc[1] * h->nc[2], h->use_cells, C, off);
}
int eb_cluster_attrs(const fg_system *h, size_t smem) {
    const void *fn = (const void *)eb_cluster_fn(h);
    CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CK(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    return FG_OK;
}
void eb_cluster_cfg(cudaLaunchConfig_t &cfg, cudaLaunchAttribute *attr, int C, size_t smem, cudaStream_t st) {
    cfg = cudaLaunchConfig_t{};
    cfg.gridDim = dim3((unsigned)C);
    cfg.blockDim = dim3(fg::kEbThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
}

// Largest cluster (power of two, <= kEbMaxCluster) whose shared memory fits
// and that the device co-schedules for this system; 1 where none does.
int eb_cluster_max(fg_system *h) {
    if (h->model != FG_MODEL_EWALD_WCA || h->K <= 0 || !ewald_block_ok(h)) return 1;
    if (h->cl_max > 0) return h->cl_max;
    h->cl_max = 1;
    for (int C = fg::kEbMaxCluster; C >= 2; C /= 2) {
        std::vector<int4> ranges, items;
        int kmax = 0;
        if (!eb_cluster_plan(h->n3, h->K, C, ranges, items, kmax)) continue;
        const size_t smem = eb_cluster_smem(h, C, kmax);
        if (smem + sizeof(SysDesc) + 1024 > 227 * 1024) continue;
        if (eb_cluster_attrs(h, smem)) {
            cudaGetLastError();
            continue;
        }
        cudaLaunchConfig_t cfg;
        cudaLaunchAttribute attr[1];
        eb_cluster_cfg(cfg, attr, C, smem, h->stream);
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, (const void *)eb_cluster_fn(h), &cfg) == cudaSuccess && n > 0) {
            h->cl_max = C;
            break;
        }
        cudaGetLastError();
    }
    return h->cl_max;
}

// CTAs of the cluster a system alone runs on: the requested size, or the
// built-in choice (as many as fit, with no fewer than 128 k-vectors per CTA;
// 16 on 16384 ions with K = 2242 runs 0.89 us per trial against 1.03 on 8
// and 3.23 on one), capped by what fits.
int eb_cluster_ctas(fg_system *h) {
    if (h->model != FG_MODEL_EWALD_WCA || h->K <= 0 || !ewald_block_ok(h)) return 1;
    const int want = h->eb_ctas > 0 ? h->eb_ctas : std::max(1, std::min(fg::kEbMaxCluster, h->K / 128));
    const int maxc = eb_cluster_max(h);
    int C = 1;
    while (2 * C <= std::min(want, maxc)) C *= 2;
    return C;
}

// The k-vector split and descriptor of a C-CTA cluster (built once per C).
int eb_cluster_prepare(fg_system *h, int C) {
    if (h->cl_c != C) {
        std::vector<int4> ranges, items;
        int kmax = 0;
        if (!eb_cluster_plan(h->n3, h->K, C, ranges, items, kmax))
            return fail(FG_ERR_INVALID, "k-vectors do not split over %d CTAs", C);
        if (!h->cl_items) {   // at most one item per k-vector
            int rc = dmalloc(h, (void **)&h->cl_items, (size_t)h->K * sizeof(int4));
            if (rc) return rc;
        }
        if ((int)items.size() > h->K) return fail(FG_ERR_INVALID, "cluster item list longer than K");
        CK(cudaMemcpy(h->cl_items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->eb_ranges + 1, ranges.data(), ranges.size() * sizeof(int4), cudaMemcpyHostToDevice));
        h->cl_c = C;
        h->cl_kmax = kmax;
        h->cl_n_items = (int)items.size();
    }
    if (!h->d_desc_cl) {
        int rc = dmalloc(h, (void **)&h->d_desc_cl, sizeof(SysDesc));
        if (rc) return rc;
    }
    SysDesc dc = h->desc;
    dc.eb_ctas = C;
    dc.eb_kmax = h->cl_kmax;
    dc.eb_ranges = h->eb_ranges + 1;
    dc.rb_items = h->cl_items;
    dc.n_rb_items = h->cl_n_items;
    CK(cudaMemcpyAsync(h->d_desc_cl, &dc, sizeof(SysDesc), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return eb_cluster_attrs(h, eb_cluster_smem(h, C, h->cl_kmax));
}

int eb_cluster_launch(fg_system *h, int C, int64_t end) {
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    eb_cluster_cfg(cfg, attr, C, eb_cluster_smem(h, C, h->cl_kmax), h->stream);
    cudaError_t e = cudaLaunchKernelEx(&cfg, eb_cluster_fn(h), (const SysDesc *)h->d_desc_cl, end,
                                       (const float2 *)h->sc_tab);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, "cluster sweep launch: %s", cudaGetErrorString(e));
    return FG_OK;
}

// ---------------------------------------------------------------- DH block sweeps
// Debye-Hueckel systems without a cell list run the block-of-trials kernel
// (fg_dh_block.cu), large ones on a cluster of CTAs.
using BlkFn = void (*)(const SysDesc *, const int *, int, int64_t);

bool dh_block_ok(const fg_system *h) { return h->model == FG_MODEL_DH_LJ && !h->use_cells; }

// Shared memory of the block kernel for N particles on C CTAs; slice = the
// CTA's particles are staged in shared memory.
size_t dh_block_smem(int N, int C, bool *slice) {
    const int ns = (N + C - 1) / C;
    const size_t with = fg::blk_smem_bytes(ns, true);
    const bool fits = with + sizeof(SysDesc) + 1024 <= 227 * 1024;
    if (slice) *slice = fits;
    return fits ? with : fg::blk_smem_bytes(ns, false);
}

BlkFn dh_block_fn(bool slice, bool cluster) {
    if (slice) return cluster ? fg::dh_block_kernel<true, true> : fg::dh_block_kernel<true, false>;
    return cluster ? fg::dh_block_kernel<false, true> : fg::dh_block_kernel<false, false>;
}

int dh_block_attrs(BlkFn fn, size_t smem, bool cluster) {
    CK(cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (cluster) CK(cudaFuncSetAttribute((const void *)fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    return FG_OK;
}

// Largest cluster (<= 16) the device co-schedules for the block kernel.
int dh_block_max_cluster() {
    static int cached[64];
    static bool init[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    dev = std::min(std::max(dev, 0), 63);
    if (init[dev]) return cached[dev];
    int best = 1;
    for (int c : {16, 8, 4, 2}) {
        bool slice;
        const size_t smem = dh_block_smem(16384, c, &slice);
        BlkFn fn = dh_block_fn(slice, true);
        if (dh_block_attrs(fn, smem, true)) continue;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)c);
        cfg.blockDim = dim3(fg::kBlkThreads);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)c;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, (const void *)fn, &cfg) == cudaSuccess && n > 0) {
            best = c;
            break;
        }
        cudaGetLastError();
    }
    cached[dev] = best;
    init[dev] = true;
    return best;
}

// Launch shapes chosen by the autotuner (fg_tune.cu), process-wide:
// CTAs per system for a DH+LJ system alone, per power-of-two size class, and
// the least particles per CTA when a batch or the server shares the SMs out.
std::mutex g_tune_mu;
std::map<int, int> g_tune_dh_ctas;   // floor(log2 N) -> CTAs
int g_tune_min_per_cta = 256;
int g_tune_dip_threads = 0;          // threads per point-dipole system (0: built-in default)

int size_class(int N) {
    int c = 0;
    while ((2 << c) <= N) c++;
    return c;
}

// CTAs for one system alone: the tuned choice for its size class, else about
// 2048 particles per CTA.
int dh_block_ctas(int N) {
    const int maxc = dh_block_max_cluster();
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_dh_ctas.find(size_class(N));
        if (it != g_tune_dh_ctas.end()) return std::max(1, std::min(it->second, maxc));
    }
    int C = 1;
    while (C < maxc && (N + C - 1) / C > 2048) C <<= 1;
    return C;
}
int tuned_min_per_cta() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return g_tune_min_per_cta;
}

int dh_sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return std::max(n, 1);
}

// CTAs per system for systems run side by side: start at one each, then keep
// doubling the system with the most work per CTA (weight / CTAs) while the
// SMs hold every CTA at once, the device allows the cluster and each CTA keeps
// at least min_per_cta particles. weight ~ pair evaluations of the launch.
std::vector<int> dh_block_ctas_many(const std::vector<int> &N, const std::vector<double> &w, int min_per_cta) {
    const int n = (int)N.size();
    std::vector<int> C(n, 1);
    const int maxc = dh_block_max_cluster();
    long spare = (long)dh_sm_count() - n;
    while (spare > 0) {
        int best = -1;
        double bw = 0;
        for (int i = 0; i < n; i++) {
            if (2 * C[i] > maxc || N[i] / (2 * C[i]) < min_per_cta || C[i] > spare) continue;
            const double x = w[i] / C[i];
            if (x > bw) {
                bw = x;
                best = i;
            }
        }
        if (best < 0) break;
        spare -= C[best];
        C[best] *= 2;
    }
    return C;
}

// One launch of the block kernel over n systems (members: indices into descs,
// device memory, or nullptr for 0..n-1) with C CTAs each.
int dh_block_launch(const SysDesc *descs, const int *members, int n, int C, int maxN, int64_t end, cudaStream_t st) {
    bool slice;
    const size_t smem = dh_block_smem(maxN, C, &slice);
    BlkFn fn = dh_block_fn(slice, C > 1);
    int rc = dh_block_attrs(fn, smem, C > 1);
    if (rc) return rc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(n * C));
    cfg.blockDim = dim3(fg::kBlkThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    if (C > 1) {
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)C;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    cudaError_t e = cudaLaunchKernelEx(&cfg, fn, descs, members, C, end);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, "block sweep launch: %s", cudaGetErrorString(e));
    return FG_OK;
}

// Systems grouped by their CTA count, each group one launch; groups after the
// first run on side streams forked from and joined back into `st`.
struct DhGroups {
    std::vector<int> C;                 // per group
    std::vector<std::vector<int>> mem;  // per group: member indices
    std::vector<int> maxN;
    int *d_members = nullptr;           // all groups' members, concatenated
    std::vector<int> offset;
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> ev;        // fork + one join per side stream
    void release() {
        if (d_members) cudaFree(d_members);
        d_members = nullptr;
        for (auto x : side) cudaStreamDestroy(x);
        for (auto x : ev) cudaEventDestroy(x);
        side.clear();
        ev.clear();
        C.clear();
        mem.clear();
        maxN.clear();
        offset.clear();
    }
};

int dh_groups_build_c(DhGroups &g, const std::vector<int> &N, const std::vector<int> &C);

int dh_groups_build(DhGroups &g, const std::vector<int> &N, const std::vector<double> &w, int min_per_cta) {
    return dh_groups_build_c(g, N, dh_block_ctas_many(N, w, min_per_cta));
}

// Largest CTA count a system of N particles is given (>= min_per_cta particles per CTA).
int dh_block_ctas_cap(int N, int min_per_cta) {
    const int maxc = dh_block_max_cluster();
    int C = 1;
    while (2 * C <= maxc && N / (2 * C) >= min_per_cta) C *= 2;
    return C;
}

int dh_groups_build_c(DhGroups &g, const std::vector<int> &N, const std::vector<int> &C) {
    if (g.d_members) cudaFree(g.d_members);
    g.d_members = nullptr;
    g.C.clear();
    g.mem.clear();
    g.maxN.clear();
    g.offset.clear();
    for (size_t i = 0; i < N.size(); i++) {
        size_t k = 0;
        while (k < g.C.size() && g.C[k] != C[i]) k++;
        if (k == g.C.size()) {
            g.C.push_back(C[i]);
            g.mem.emplace_back();
            g.maxN.push_back(0);
        }
        g.mem[k].push_back((int)i);
        g.maxN[k] = std::max(g.maxN[k], N[i]);
    }
    std::vector<int> all;
    for (auto &m : g.mem) {
        g.offset.push_back((int)all.size());
        all.insert(all.end(), m.begin(), m.end());
    }
    CK(cudaMalloc(&g.d_members, std::max<size_t>(all.size(), 1) * sizeof(int)));
    CK(cudaMemcpy(g.d_members, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice));
    while (g.side.size() + 1 < g.C.size()) {   // side streams and events are kept across rebuilds
        cudaStream_t x;
        CK(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
        g.side.push_back(x);
    }
    while (g.ev.size() < g.C.size()) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        g.ev.push_back(e);
    }
    return FG_OK;
}

int dh_groups_launch(const DhGroups &g, const SysDesc *descs, int64_t end, cudaStream_t st) {
    if (g.C.size() > 1) CK(cudaEventRecord(g.ev[0], st));
    for (size_t k = 0; k < g.C.size(); k++) {
        cudaStream_t s = k == 0 ? st : g.side[k - 1];
        if (k > 0) CK(cudaStreamWaitEvent(s, g.ev[0], 0));
        int rc = dh_block_launch(descs, g.d_members + g.offset[k], (int)g.mem[k].size(), g.C[k], g.maxN[k], end, s);
        if (rc) return rc;
        if (k > 0) CK(cudaEventRecord(g.ev[k], s));
    }
    for (size_t k = 1; k < g.C.size(); k++) CK(cudaStreamWaitEvent(st, g.ev[k], 0));
    return FG_OK;
}

// Rebuild kernels for n systems whose descriptors are at `descs` (device):
// maxN particles, maxSeg k-vector runs and axis bound maxKcc at most.
int launch_rebuild(const SysDesc *descs, int n, int maxN, int maxSeg, int maxKcc, float2 *corr, cudaStream_t st) {
    if (maxSeg == 0) return FG_OK;
    const int T = fg::qk_tab_len(maxKcc);
    const int threads = std::min(fg::kQkMaxThreads, ((maxSeg + 31) / 32) * 32);
    // each thread stages (and prefetches) one particle of a pass: a pass holds
    // at most as many particles as the block has threads
    const int stage = std::max(1, std::min({fg::kQkMaxStage, 40960 / (T * 8), threads}));
    const size_t smem = fg::qk_rebuild_smem(stage, T, threads);
    int rc = set_smem_attr((const void *)fg::qk_rebuild_kernel, smem);
    if (rc) return rc;
    // about four blocks per SM over all systems, at least 256 particles each
    const long long want = 4LL * dh_sm_count();
    int chunk = (int)std::max<long long>(256, ((long long)maxN * n + want - 1) / want);
    chunk = ((chunk + stage - 1) / stage) * stage;
    dim3 g((maxN + chunk - 1) / chunk, n);
    fg::qk_rebuild_kernel<<<g, threads, smem, st>>>(descs, chunk, stage);
    fg::qk_rebuild_finish<<<n, 1024, 0, st>>>(descs, corr);
    CK(cudaGetLastError());
    return FG_OK;
}

int read_scalars(fg_system *h, SysScalars &s) {
    CK(cudaMemcpyAsync(&s, h->sc, sizeof(SysScalars), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FG_OK;
}
int write_scalars(fg_system *h, const SysScalars &s) {
    CK(cudaMemcpyAsync(h->sc, &s, sizeof(SysScalars), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

int ensure_trials(fg_system *h, int64_t n, bool log) {
    n = std::max<int64_t>(n, 1);
    if (n > h->trials_cap) {
        if (h->trials) cudaFree(h->trials);
        h->trials = nullptr;
        DMALLOC(h->trials, n * sizeof(Trial));
        h->trials_cap = n;
    }
    if (log && n > h->log_cap) {
        if (h->log_du) cudaFree(h->log_du);
        if (h->log_acc) cudaFree(h->log_acc);
        h->log_du = nullptr;
        h->log_acc = nullptr;
        DMALLOC(h->log_du, n * sizeof(float2));
        DMALLOC(h->log_acc, n);
        h->log_cap = n;
    }
    return FG_OK;
}

int push_desc(fg_system *h) {
    CK(cudaMemcpyAsync(h->d_desc, &h->desc, sizeof(SysDesc), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

// Host -> device trial records: fixed-point displacement and -ln(u) as df.
// Pair part of the total energy (device) in kT.
int pair_energy(fg_system *h, double &out) {
    const int nb = 1024;
    using PairFn = void (*)(const SysDesc *, float2 *);
    PairFn fn = h->model == FG_MODEL_EWALD_WCA ? fg::pair_total_kernel<fg::MODEL_EWALD>
                                                : fg::pair_total_kernel<fg::MODEL_DHLJ>;
    fn<<<nb, 256, 0, h->stream>>>(h->d_desc, h->pair_part);
    CK(cudaGetLastError());
    std::vector<float2> part(nb);
    CK(cudaMemcpyAsync(part.data(), h->pair_part, nb * sizeof(float2), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    double s = 0;
    for (auto &p : part) s += df_val(p.x, p.y);
    out = s;
    return FG_OK;
}

int get_qk_host(fg_system *h, std::vector<double> &q) {
    q.assign(2 * (size_t)h->K, 0.0);
    if (h->K == 0) return FG_OK;
    std::vector<longlong2> v(h->K);
    CK(cudaMemcpyAsync(v.data(), h->qfix, v.size() * sizeof(longlong2), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    // units of 2^-28 / c, c = 4095/4096 (set_qk_scale)
    const double unit = (1.0 / 268435456.0) * (4096.0 / 4095.0);
    for (int k = 0; k < h->K; k++) {
        q[2 * k] = (double)v[k].x * unit;
        q[2 * k + 1] = (double)v[k].y * unit;
    }
    return FG_OK;
}

// {pairs, reciprocal, self, surface, total} in kT
int total_energy(fg_system *h, double *c) {
    double pairs = 0;
    int rc = pair_energy(h, pairs);
    if (rc) return rc;
    double rec = 0, self = 0, surf = 0;
    if (h->K > 0) {
        std::vector<double> q;
        rc = get_qk_host(h, q);
        if (rc) return rc;
        for (int k = 0; k < h->K; k++) rec += h->ak[k] * (q[2 * k] * q[2 * k] + q[2 * k + 1] * q[2 * k + 1]);
        rec *= h->recip_c;
        self = h->self_energy;
        SysScalars s;
        rc = read_scalars(h, s);
        if (rc) return rc;
        double M2 = 0;
        for (int a = 0; a < 3; a++) {
            double m = df_val(s.m[a][0], s.m[a][1]);
            M2 += m * m;
        }
        surf = h->surf_c * M2;
    }
    c[0] = pairs;
    c[1] = rec;
    c[2] = self;
    c[3] = surf;
    c[4] = (surf + rec) + (self + pairs);
    return FG_OK;
}

// Launch config for the sweep of one system (and its batch peers).
struct LaunchCfg {
    SweepFn fn;
    int threads;
    size_t smem;
};
// Threads and shared memory of the sweep launch (the per-trial kernels keep
// sweep_threads / sweep_smem).
int sweep_launch_threads(const fg_system *h) { return ewald_block_ok(h) ? fg::kEbThreads : sweep_threads(h); }
size_t sweep_launch_smem(const fg_system *h) {
    return ewald_block_ok(h) ? ewald_block_smem(h) : sweep_smem(h, h->pos_smem);
}

int sweep_config(const fg_system *h, LaunchCfg &c) {
    c.fn = sweep_fn(h);
    c.threads = sweep_launch_threads(h);
    c.smem = sweep_launch_smem(h);
    return set_smem_attr((const void *)c.fn, c.smem);
}

// Run trials [0, n) of the staged stream (sweep + rebuild until done).
int run_stream(fg_system *h, int64_t n, bool log, fg_sweep_stats *stats) {
    SysScalars s0;
    int rc = read_scalars(h, s0);
    if (rc) return rc;
    s0.cursor = 0;
    s0.n_trials = n;
    const int64_t acc0 = s0.n_accepted;
    const int rb0 = s0.n_rebuilds;
    s0.u_hi = 0.0f;
    s0.u_lo = 0.0f;
    rc = write_scalars(h, s0);
    if (rc) return rc;
    h->desc.trials = h->trials;
    h->desc.log_trials = log ? 1 : 0;
    h->desc.trial_du = h->log_du;
    h->desc.trial_acc = h->log_acc;
    h->desc.rebuild_in_kernel = 0;   // a system alone leaves its rebuilds to the rebuild kernel (all SMs)
    h->log_n = log ? n : 0;
    rc = push_desc(h);
    if (rc) return rc;
    LaunchCfg cfg;
    rc = sweep_config(h, cfg);
    if (rc) return rc;
    const int ebc = eb_cluster_ctas(h);   // > 1: the Ewald block kernel on a cluster
    if (ebc > 1) {
        rc = eb_cluster_prepare(h, ebc);
        if (rc) return rc;
    }
    const bool rebuilds = h->K > 0 && !h->desc.skip_rebuild;
    const int uf = std::max(h->P.ewald_update_frequency, 1);
    int launches = 0;
    std::vector<cudaEvent_t> evs;
    CK(cudaEventRecord(h->ev0, h->stream));
    SysScalars s = s0;
    while (true) {
        // enough sweep/rebuild pairs for the worst case (every trial accepted)
        const int pairs = rebuilds ? (int)std::min<int64_t>((n - s.cursor) / uf + 1, 64) : 1;
        for (int p = 0; p < pairs; p++) {
            cudaEvent_t a, b;
            CK(cudaEventCreate(&a));
            CK(cudaEventCreate(&b));
            evs.push_back(a);
            evs.push_back(b);
            CK(cudaEventRecord(a, h->stream));
            if (dh_block_ok(h)) {
                rc = dh_block_launch(h->d_desc, nullptr, 1, h->ctas > 0 ? h->ctas : dh_block_ctas(h->N), h->N, n,
                                     h->stream);
                if (rc) return rc;
            } else if (ebc > 1) {
                rc = eb_cluster_launch(h, ebc, n);
                if (rc) return rc;
            } else {
                cfg.fn<<<1, cfg.threads, cfg.smem, h->stream>>>(h->d_desc, n, h->sc_tab);
            }
            CK(cudaGetLastError());
            CK(cudaEventRecord(b, h->stream));
            launches++;
            if (rebuilds) {
                rc = launch_rebuild(h->d_desc, 1, h->N, h->nseg, h->kc, h->corr, h->stream);
                if (rc) return rc;
            }
        }
        const int64_t before = s.cursor;
        rc = read_scalars(h, s);
        if (rc) return rc;
        if (s.error) break;
        if (s.cursor >= n && !s.rebuild_pending) break;
        if (s.cursor == before && !s.rebuild_pending)
            return fail(FG_ERR_DEVICE, "sweep made no progress at trial %lld", (long long)s.cursor);
    }
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaEventSynchronize(h->ev1));
    float total_ms = 0.0f, sweep_ms = 0.0f;
    CK(cudaEventElapsedTime(&total_ms, h->ev0, h->ev1));
    for (size_t e = 0; e + 1 < evs.size(); e += 2) {
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, evs[e], evs[e + 1]));
        sweep_ms += ms;
        cudaEventDestroy(evs[e]);
        cudaEventDestroy(evs[e + 1]);
    }
    h->cnt_accepted_host = s.cnt_accepted;
    if (stats) {
        stats->trials = s.cursor;
        stats->accepted = s.n_accepted - acc0;
        stats->rebuilds = s.n_rebuilds - rb0;
        stats->energy_change = df_val(s.u_hi, s.u_lo);
        stats->device_ms = total_ms;
        stats->sweep_kernel_ms = sweep_ms;
        stats->sweep_launches = launches;
        stats->error_flags = s.error;
        stats->kernel_launches = (int64_t)launches * (rebuilds ? 3 : 1);
    }
    if (s.error) return fail(FG_ERR_DEVICE, "device error flags 0x%x", s.error);
    return FG_OK;
}

}  // namespace

extern "C" {

int fg_version(void) { return 200; }

const char *fg_last_error(void) { return g_err.c_str(); }

void fg_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    fg::u4 r = fg::philox4x32_10(fg::u4{ctr[0], ctr[1], ctr[2], ctr[3]}, key[0], key[1]);
    out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}

// Largest |q eff| of the particles (charges, or the type charges when null).
double qk_charge_bound(const fg_system *h, const double *charge) {
    double qmax = 0;
    if (charge) {
        for (int i = 0; i < h->N; i++)
            qmax = std::max(qmax, std::fabs(charge[i] * h->desc.eff[h->types[i]]));
    } else {
        for (int t = 0; t < h->P.n_types; t++)
            qmax = std::max(qmax, std::fabs(h->P.type_charge[t] * h->desc.eff[t]));
    }
    return qmax;
}

// Scale s = 2^g c of the Q(k) contributions (grid 1/s): g is the largest
// value <= 28 with 2^g max|q eff| <= 2^22 and c = 4095/4096, so every term
// |s q eff e_x e_y e_z| stays below 2^22 - 2^9 whatever the few-ulp rounding
// of the unit factors, inside the range where qk_term rounds with one FP32
// addition; 256 terms sum exactly in int32. Q(k) is held in units of
// 2^-28 / c (each term shifted left by 28 - g).
int set_qk_scale(SysDesc &d, double qmax) {
    if (!(qmax <= 4194304.0)) return FG_ERR_INVALID;
    int g = 28;
    while (g > 0 && std::ldexp(qmax, g) > 4194304.0) g--;
    d.qk_scale = (float)std::ldexp(4095.0 / 4096.0, g);
    d.qk_shift = 28 - g;
    return FG_OK;
}

int fg_create(const fg_params *params, int32_t n_particles, fg_system **out) {
    if (!params || !out) return fail(FG_ERR_INVALID, "null argument");
    *out = nullptr;
    const fg_params &P = *params;
    if (P.model != FG_MODEL_EWALD_WCA && P.model != FG_MODEL_DH_LJ)
        return fail(FG_ERR_INVALID, "model %d not supported by the atomic path", P.model);
    if (n_particles < 2 || n_particles >= (1 << 24)) return fail(FG_ERR_INVALID, "bad particle count %d", n_particles);
    if (P.n_types < 1 || P.n_types > FG_MAX_TYPES) return fail(FG_ERR_INVALID, "bad n_types %d", P.n_types);
    for (int a = 0; a < 3; a++)
        if (!(P.box[a] > 0)) return fail(FG_ERR_INVALID, "box must be positive");
    if (P.model == FG_MODEL_DH_LJ && (P.box[1] != P.box[0] || P.box[2] != P.box[0]))
        return fail(FG_ERR_INVALID, "Debye-Hueckel systems need a cubic box");
    if (P.model == FG_MODEL_EWALD_WCA) {
        if (!(P.ewald_alpha > 0) || !(P.ewald_cutoff > 0) || !(P.ewald_debye_length > 0))
            return fail(FG_ERR_INVALID, "Ewald needs alpha, cutoff and debye_length > 0");
        if (std::ceil(P.ewald_cutoff_k) > 127) return fail(FG_ERR_INVALID, "cutoffK too large");
    } else if (!(P.dh_debye_length > 0)) {
        return fail(FG_ERR_INVALID, "dh_debye_length must be > 0");
    }
    fg_system *h = new fg_system();
    h->P = P;
    h->N = n_particles;
    h->model = P.model;
    auto bail = [&](int code) {
        free_all(h);
        delete h;
        return code;
    };
    if (cudaGetDevice(&h->device) != cudaSuccess) return bail(fail(FG_ERR_CUDA, "no CUDA device"));
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(FG_ERR_CUDA, "stream create failed"));
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);

    SysDesc &d = h->desc;
    std::memset(&d, 0, sizeof(d));
    d.model = P.model;
    d.N = n_particles;
    d.n_types = P.n_types;
    for (int a = 0; a < 3; a++) {
        d.L[a] = (float)P.box[a];
        d.s32[a] = (float)(P.box[a] / 4294967296.0);
        d.dl32[a] = (float)(P.box[a] / TWO64);
    }
    d.s32sq = (float)((P.box[0] / 4294967296.0) * (P.box[0] / 4294967296.0));
    d.lB = (float)P.bjerrum;
    d.kT = (float)(P.kT_scale > 0 ? P.kT_scale : 1.0);
    d.update_frequency = P.ewald_update_frequency;
    const int nt = P.n_types;
    double kappa = 0;
    if (P.model == FG_MODEL_EWALD_WCA) {
        kappa = 1.0 / P.ewald_debye_length;
        d.alpha = (float)P.ewald_alpha;
        d.rc2 = (float)(P.ewald_cutoff * P.ewald_cutoff);
        d.kappa = (kappa * P.ewald_cutoff < 1e-7) ? 0.0f : (float)kappa;
    } else {
        d.kappa = (float)(1.0 / P.dh_debye_length);
        d.rc2 = 3.0e38f;
    }
    // type tables: LorentzBerthelot mixing, eps x4 (potentials.h:2003-2023);
    // effective charges and QeQe (ewald.h:532-549)
    std::vector<double> eff(nt, 1.0);
    for (int i = 0; i < nt; i++) {
        double ri = 0.5 * P.type_sigma[i], qis = P.type_charge[i];
        // a neutral type's ratio is 0/0 in the reference (ewald.h:539); its
        // particles carry no charge (fg_set_state), so any value serves: 1
        if (P.model == FG_MODEL_EWALD_WCA && P.type_charge[i] != 0.0) {
            if (std::fabs(kappa * ri) > 1e-9) qis *= std::sinh(ri * kappa) / ri / kappa;
            eff[i] = qis / P.type_charge[i];
        }
        d.eff[i] = (float)eff[i];
    }
    bool uniform = true;
    for (int i = 0; i < nt; i++)
        for (int j = 0; j < nt; j++) {
            double sig = 0.5 * (P.type_sigma[i] + P.type_sigma[j]);
            double s2 = sig * sig, e4 = 4 * std::sqrt(P.type_eps[i] * P.type_eps[j]);
            int t = i * nt + j;
            d.s2[t] = (float)s2;
            d.eps4[t] = (float)e4;
            d.wca2[t] = (float)(s2 * std::pow(2, 2 / 6.));
            d.qeqe[t] = (float)(eff[i] * eff[j]);
            d.pref_df[t] = split_df(P.model == FG_MODEL_EWALD_WCA ? eff[i] * eff[j] * P.bjerrum : P.bjerrum);
            d.s2_df[t] = split_df(s2);
            d.eps4_df[t] = split_df(e4);
            if (d.s2[t] != d.s2[0] || d.eps4[t] != d.eps4[0] || d.qeqe[t] != d.qeqe[0]) uniform = false;
        }
    d.uniform_types = uniform ? 1 : 0;
    d.reach2 = d.rc2;
    for (int t = 0; t < nt * nt; t++) d.reach2 = std::max(d.reach2, std::max(d.wca2[t], d.s2[t]));

    // Ewald k-space
    std::vector<int> n3;
    std::vector<double> kv3;
    const double V = P.box[0] * P.box[1] * P.box[2];
    if (P.model == FG_MODEL_EWALD_WCA) {
        enumerate_k(P, n3, h->ak, kv3);
        h->K = (int)h->ak.size();
        h->kc = (int)std::ceil(P.ewald_cutoff_k);
        if (h->kc > 127 || h->K >= (1 << 24)) return bail(fail(FG_ERR_INVALID, "k-space cutoff too large"));
        h->recip_c = 2 * PI / V * P.bjerrum;
        const double const_inf = (P.ewald_eps_surf < 1) ? 0.0 : 1.0;
        h->surf_c = const_inf * (2 * PI / ((2 * P.ewald_eps_surf + 1) * V)) * P.bjerrum;
        d.surf_c = (float)h->surf_c;
    }
    d.K = h->K;
    // cells (auto: cutoff systems with >= 4 cells per axis and many particles)
    if (P.model == FG_MODEL_EWALD_WCA) {
        int nc[3];
        for (int a = 0; a < 3; a++) nc[a] = (int)std::floor(P.box[a] / P.ewald_cutoff);
        // a stencil spans up to 4 cells per axis, so 4 distinct cells are needed
        bool can = nc[0] >= 4 && nc[1] >= 4 && nc[2] >= 4 && (long)nc[0] * nc[1] * nc[2] < (1 << 20);
        bool want = (P.use_cell_list == 1) || (P.use_cell_list == 0 && n_particles >= 4096);
        if (P.use_cell_list == 1 && !can) return bail(fail(FG_ERR_INVALID, "cell list needs >= 4 cells per axis"));
        h->use_cells = can && want;
        if (h->use_cells)
            for (int a = 0; a < 3; a++) h->nc[a] = nc[a];
    }
    d.use_cells = h->use_cells ? 1 : 0;
    for (int a = 0; a < 3; a++) d.nc[a] = h->nc[a];
    // positions in shared memory when they fit next to the k-space tables
    h->pos_smem = !h->use_cells && sweep_smem(h, true) <= 200 * 1024;

    const int N = n_particles;
    int rc;
#define ALLOC(ptr, bytes)                          \
    do {                                           \
        rc = dmalloc(h, (void **)&(ptr), (bytes)); \
        if (rc) return bail(rc);                   \
    } while (0)
    ALLOC(h->d_desc, sizeof(SysDesc));
    ALLOC(h->pos64, (size_t)N * 3 * sizeof(int64_t));
    ALLOC(h->pos4, (size_t)N * sizeof(int4));
    ALLOC(h->pos_ext, (size_t)N * sizeof(short4));
    ALLOC(h->ptype, (size_t)N);
    ALLOC(h->sc, sizeof(SysScalars));
    ALLOC(h->req, 8 * sizeof(int64_t));
    ALLOC(h->trial_out, 4 * sizeof(float2));
    ALLOC(h->corr, 4 * sizeof(float2));
    ALLOC(h->sc_tab, 256 * sizeof(float2));
    ALLOC(h->dp_fix, FG_MAX_TYPES * 3 * sizeof(int64_t));
    ALLOC(h->pair_part, 1024 * sizeof(float2));
    if (h->K > 0) {
        ALLOC(h->kvec, (size_t)h->K * sizeof(float4));
        ALLOC(h->kpack, (size_t)h->K * sizeof(uint32_t));
        ALLOC(h->qfix, (size_t)h->K * sizeof(longlong2));
        ALLOC(h->qnew, (size_t)h->K * sizeof(longlong2));
        std::vector<float4> kv(h->K);
        std::vector<uint32_t> kp(h->K);
        for (int k = 0; k < h->K; k++) {
            kv[k] = make_float4((float)kv3[3 * k], (float)kv3[3 * k + 1], (float)kv3[3 * k + 2],
                                (float)(h->ak[k] * h->recip_c));
            kp[k] = (uint32_t)(n3[3 * k] & 0xFF) | ((uint32_t)(n3[3 * k + 1] & 0xFF) << 8) |
                    ((uint32_t)(n3[3 * k + 2] & 0xFF) << 16);
        }
        cudaMemcpy(h->kvec, kv.data(), h->K * sizeof(float4), cudaMemcpyHostToDevice);
        cudaMemcpy(h->kpack, kp.data(), h->K * sizeof(uint32_t), cudaMemcpyHostToDevice);
        // runs of consecutive k-vectors with the same (nx, ny) and consecutive
        // nz, each cut into near-equal pieces of at most kQkRun, longest
        // first (warps of the rebuild then run equal trip counts)
        std::vector<int2> seg;
        for (int k = 0; k < h->K;) {
            int run = 1;
            while (k + run < h->K && n3[3 * (k + run)] == n3[3 * k] && n3[3 * (k + run) + 1] == n3[3 * k + 1] &&
                   n3[3 * (k + run) + 2] == n3[3 * k + 2] + run)
                run++;
            const int pieces = (run + fg::kQkRun - 1) / fg::kQkRun;
            for (int p = 0, k0 = k; p < pieces; p++) {
                const int len = run / pieces + (p < run % pieces ? 1 : 0);
                seg.push_back(make_int2(k0 | (len << 24), (n3[3 * k0] & 0xFF) | ((n3[3 * k0 + 1] & 0xFF) << 8) |
                                                              ((n3[3 * k0 + 2] & 0xFF) << 16)));
                k0 += len;
            }
            k += run;
        }
        std::stable_sort(seg.begin(), seg.end(), [](const int2 &a, const int2 &b) { return (a.x >> 24) > (b.x >> 24); });
        h->nseg = (int)seg.size();
        ALLOC(h->kseg, seg.size() * sizeof(int2));
        cudaMemcpy(h->kseg, seg.data(), seg.size() * sizeof(int2), cudaMemcpyHostToDevice);
        // the block kernel's in-kernel rebuild: pairs (+n, -n) of k-vectors
        // (the isotropic k-set holds n_z >= 0 only: no block kernel, no items)
        std::vector<int4> rb;
        if (!P.ewald_isotropic_pbc && !rb_item_list(n3, 0, h->K, fg::kEbThreads - 32, rb))
            return bail(fail(FG_ERR_INVALID, "k-vector set is not symmetric in nz"));
        h->n_rb_items = (int)rb.size();
        ALLOC(h->rb_items, rb.size() * sizeof(int4));
        cudaMemcpy(h->rb_items, rb.data(), rb.size() * sizeof(int4), cudaMemcpyHostToDevice);
        // one CTA holds every k-vector and item
        ALLOC(h->eb_ranges, (1 + fg::kEbMaxCluster) * sizeof(int4));
        const int4 one = make_int4(0, h->K, 0, h->n_rb_items);
        cudaMemcpy(h->eb_ranges, &one, sizeof(int4), cudaMemcpyHostToDevice);
        h->n3 = n3;
        cudaMemset(h->qfix, 0, h->K * sizeof(longlong2));
        cudaMemset(h->qnew, 0, h->K * sizeof(longlong2));
    }
    if (h->use_cells) {
        const int ncell = h->nc[0] * h->nc[1] * h->nc[2];
        const double avg = (double)N / ncell;
        h->cap = std::min(4095, std::max(64, (((int)(2.5 * avg) + 32 + 31) / 32) * 32));
        ALLOC(h->cell_count, (size_t)ncell * sizeof(int32_t));
        ALLOC(h->cell_pid, (size_t)ncell * h->cap * sizeof(int32_t));
        ALLOC(h->cell_pos, (size_t)ncell * h->cap * sizeof(int4));
        ALLOC(h->cell_ext, (size_t)ncell * h->cap * sizeof(short4));
        ALLOC(h->p_cell, (size_t)N * sizeof(int32_t));
        ALLOC(h->p_slot, (size_t)N * sizeof(int32_t));
    }
    // Taylor table of g(y) for core pairs: erfc (Ewald, kappa = 0) or exp(-y)
    // (Debye-Hueckel) at y0 = j/128; entries f0, f1 as df, f2/2, f3/6, f4/24
    {
        const double coef = P.model == FG_MODEL_EWALD_WCA ? P.ewald_alpha : 1.0 / P.dh_debye_length;
        const bool ok = P.model == FG_MODEL_DH_LJ || d.kappa == 0.0f;
        double smax = 0;
        for (int i = 0; i < nt; i++) smax = std::max(smax, P.type_sigma[i]);
        const int ntab = ok && smax > 0 ? (int)std::ceil(coef * smax * 128.0) + 4 : 0;
        if (ntab > 0) {
            ALLOC(h->core_tab, (size_t)ntab * sizeof(float4));
            ALLOC(h->core_tab2, (size_t)ntab * sizeof(float4));
            std::vector<float4> t0(ntab), t1(ntab);
            const double k = 2.0 / std::sqrt(PI);
            for (int j = 0; j < ntab; j++) {
                const double y = j / 128.0;
                double f0, f1, f2, f3, f4;
                if (P.model == FG_MODEL_EWALD_WCA) {
                    const double e = std::exp(-y * y);
                    f0 = std::erfc(y);
                    f1 = -k * e;
                    f2 = 2 * k * y * e;
                    f3 = 2 * k * (1 - 2 * y * y) * e;
                    f4 = 2 * k * (4 * y * y * y - 6 * y) * e;
                } else {
                    f0 = std::exp(-y);
                    f1 = -f0; f2 = f0; f3 = -f0; f4 = f0;
                }
                const float2 a = split_df(f0), b = split_df(f1);
                t0[j] = make_float4(a.x, a.y, b.x, b.y);
                t1[j] = make_float4((float)(f2 / 2), (float)(f3 / 6), (float)(f4 / 24), 0.0f);
            }
            cudaMemcpy(h->core_tab, t0.data(), ntab * sizeof(float4), cudaMemcpyHostToDevice);
            cudaMemcpy(h->core_tab2, t1.data(), ntab * sizeof(float4), cudaMemcpyHostToDevice);
        }
        d.core_tab_n = ntab;
        d.core_tab = h->core_tab;
        d.core_tab2 = h->core_tab2;
        d.coef_df = split_df(coef);
        for (int a = 0; a < 3; a++) d.s48_df[a] = split_df(P.box[a] / 281474976710656.0);
    }
#undef ALLOC
    d.cap = h->cap;
    d.pos64 = h->pos64;
    d.pos4 = h->pos4;
    d.pos_ext = h->pos_ext;
    d.ptype = h->ptype;
    d.cell_count = h->cell_count;
    d.cell_pos = h->cell_pos;
    d.cell_ext = h->cell_ext;
    d.cell_pid = h->cell_pid;
    d.p_cell = h->p_cell;
    d.p_slot = h->p_slot;
    d.kvec = h->kvec;
    d.kpack = h->kpack;
    d.kseg = h->kseg;
    d.nseg = h->nseg;
    d.rb_items = h->rb_items;
    d.n_rb_items = h->n_rb_items;
    d.eb_ctas = 1;
    d.eb_kmax = h->K;
    d.eb_ranges = h->eb_ranges;
    d.iso = P.ewald_isotropic_pbc ? 1 : 0;
    d.kcc = h->kc;
    if (set_qk_scale(d, qk_charge_bound(h, nullptr)))
        return bail(fail(FG_ERR_INVALID, "charges too large for the Q(k) fixed point"));
    d.qfix = h->qfix;
    d.qnew = h->qnew;
    d.sc = h->sc;
    d.sc_tab = h->sc_tab;
    d.dp_fix = h->dp_fix;
    // cos/sin table at multiples of 2*pi/256
    std::vector<float2> tab(256);
    for (int i = 0; i < 256; i++) tab[i] = make_float2((float)std::cos(2 * PI * i / 256), (float)std::sin(2 * PI * i / 256));
    cudaMemcpy(h->sc_tab, tab.data(), sizeof(float2) * 256, cudaMemcpyHostToDevice);
    // displacement parameters in fixed point (device-generated streams)
    std::vector<int64_t> dpf(FG_MAX_TYPES * 3, 0);
    for (int t = 0; t < nt; t++)
        for (int a = 0; a < 3; a++) dpf[3 * t + a] = (int64_t)llrint(P.type_dp[t] / P.box[a] * 4294967296.0);
    cudaMemcpy(h->dp_fix, dpf.data(), dpf.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
    SysScalars s0{};
    s0.verify_rebuild = 1;
    cudaMemcpy(h->sc, &s0, sizeof(s0), cudaMemcpyHostToDevice);
    rc = push_desc(h);
    if (rc) return bail(rc);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return bail(fail(FG_ERR_CUDA, "setup failed"));
    *out = h;
    return FG_OK;
}

int fg_destroy(fg_system *h) {
    if (!h) return FG_OK;
    cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return FG_OK;
}

int fg_set_state(fg_system *h, const double *xyz, const double *charge, const int32_t *type_ids) {
    if (!h || !xyz || !type_ids) return fail(FG_ERR_INVALID, "null argument");
    const int N = h->N;
    const fg_params &P = h->P;
    std::vector<int64_t> p64(3 * (size_t)N);
    std::vector<int4> p4(N);
    std::vector<short4> pe(N);
    std::vector<uint8_t> pt(N);
    h->types.assign(type_ids, type_ids + N);
    h->charges.resize(N);
    double self = 0, M[3] = {0, 0, 0};
    for (int i = 0; i < N; i++) {
        const int t = type_ids[i];
        if (t < 0 || t >= P.n_types) return fail(FG_ERR_INVALID, "type id %d out of range", t);
        const double q = charge ? charge[i] : P.type_charge[t];
        if (P.model == FG_MODEL_EWALD_WCA && P.type_charge[t] == 0.0 && q != 0.0)
            return fail(FG_ERR_INVALID, "particle %d carries charge but its atom type is neutral: its Ewald effective "
                                        "charge is 0/0 (ewald.h:539)", i);
        h->charges[i] = q;
        int32_t hw[3];
        for (int a = 0; a < 3; a++) {
            if (!std::isfinite(xyz[3 * i + a])) return fail(FG_ERR_INVALID, "non-finite coordinate");
            p64[3 * i + a] = to_fix(xyz[3 * i + a], P.box[a]);
            hw[a] = hi32h(p64[3 * i + a]);
            // surface dipole over wrapped positions (ewald.h:277-291)
            M[a] += q * h->desc.eff[t] * from_fix(p64[3 * i + a], P.box[a]);
        }
        const float qf = (float)q;
        p4[i] = make_int4(hw[0], hw[1], hw[2], 0);
        std::memcpy(&p4[i].w, &qf, 4);
        pe[i] = make_short4(ext16h(p64[3 * i]), ext16h(p64[3 * i + 1]), ext16h(p64[3 * i + 2]), 0);
        pt[i] = (uint8_t)t;
        const double e = h->desc.eff[t];
        self += q * q * e * e;
    }
    h->self_energy = (-P.ewald_alpha * self / std::sqrt(PI)) * P.bjerrum;
    CK(cudaMemcpyAsync(h->pos64, p64.data(), p64.size() * 8, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->pos4, p4.data(), p4.size() * 16, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->ptype, pt.data(), pt.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->pos_ext, pe.data(), pe.size() * sizeof(short4), cudaMemcpyHostToDevice, h->stream));
    if (h->use_cells) {
        const int ncell = h->nc[0] * h->nc[1] * h->nc[2];
        std::vector<int32_t> cnt(ncell, 0), pid((size_t)ncell * h->cap, -1), pc(N), ps(N);
        std::vector<int4> cp((size_t)ncell * h->cap, make_int4(0, 0, 0, 0));
        std::vector<short4> ce((size_t)ncell * h->cap, make_short4(0, 0, 0, 0));
        for (int i = 0; i < N; i++) {
            const int c = cell_of_h(&p64[3 * i], h->nc);
            if (cnt[c] >= h->cap) return fail(FG_ERR_CAPACITY, "cell %d over capacity %d", c, h->cap);
            const int s = cnt[c]++;
            cp[(size_t)c * h->cap + s] = p4[i];
            ce[(size_t)c * h->cap + s] = pe[i];
            pid[(size_t)c * h->cap + s] = i | (type_ids[i] << 24);
            pc[i] = c;
            ps[i] = s;
        }
        CK(cudaMemcpyAsync(h->cell_count, cnt.data(), cnt.size() * 4, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->cell_pid, pid.data(), pid.size() * 4, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->cell_pos, cp.data(), cp.size() * 16, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->cell_ext, ce.data(), ce.size() * sizeof(short4), cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->p_cell, pc.data(), pc.size() * 4, cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->p_slot, ps.data(), ps.size() * 4, cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    SysScalars s0{};
    for (int a = 0; a < 3; a++) {
        const float2 m = split_df(M[a]);
        s0.m[a][0] = m.x;
        s0.m[a][1] = m.y;
    }
    int rc;
    if (h->K > 0) {
        // contribution grid for these charges, then Q(k) from scratch: adopt
        // the rebuild without the equality check
        if (set_qk_scale(h->desc, qk_charge_bound(h, charge)))
            return fail(FG_ERR_INVALID, "charges too large for the Q(k) fixed point");
        rc = push_desc(h);
        if (rc) return rc;
        CK(cudaMemsetAsync(h->qfix, 0, (size_t)h->K * sizeof(longlong2), h->stream));
        CK(cudaMemsetAsync(h->qnew, 0, (size_t)h->K * sizeof(longlong2), h->stream));
        s0.rebuild_pending = 1;
        s0.verify_rebuild = 0;
        rc = write_scalars(h, s0);
        if (rc) return rc;
        rc = launch_rebuild(h->d_desc, 1, h->N, h->nseg, h->kc, h->corr, h->stream);
        if (rc) return rc;
    }
    s0.rebuild_pending = 0;
    s0.verify_rebuild = 1;
    s0.n_rebuilds = 0;
    rc = write_scalars(h, s0);
    if (rc) return rc;
    // running total energy starts at systemEnergy of the uploaded state
    double c[5];
    rc = total_energy(h, c);
    if (rc) return rc;
    const float2 ut = split_df(c[4]);
    s0.utot_hi = ut.x;
    s0.utot_lo = ut.y;
    rc = write_scalars(h, s0);
    if (rc) return rc;
    h->cnt_accepted_host = 0;
    h->trial_pending = false;
    h->state_set = true;
    return FG_OK;
}

int fg_get_state(fg_system *h, double *xyz) {
    if (!h || !xyz) return fail(FG_ERR_INVALID, "null argument");
    std::vector<int64_t> p64(3 * (size_t)h->N);
    CK(cudaMemcpyAsync(p64.data(), h->pos64, p64.size() * 8, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < h->N; i++)
        for (int a = 0; a < 3; a++) xyz[3 * i + a] = from_fix(p64[3 * i + a], h->P.box[a]);
    return FG_OK;
}

int fg_num_kvectors(fg_system *h) { return h ? h->K : 0; }

int fg_set_threads(fg_system *h, int32_t threads) {
    if (!h || threads < 0 || threads > fg::kSweepThreads || (threads % 32) != 0)
        return fail(FG_ERR_INVALID, "threads must be a multiple of 32 in [0, %d]", fg::kSweepThreads);
    h->threads = threads;
    return FG_OK;
}

int fg_get_threads(fg_system *h) { return h ? sweep_threads(h) : 0; }

int fg_set_cluster(fg_system *h, int32_t ctas) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (ctas < 0 || ctas > fg::kEbMaxCluster || (ctas & (ctas - 1)) != 0)
        return fail(FG_ERR_INVALID, "ctas must be 0 or a power of two up to %d", fg::kEbMaxCluster);
    h->eb_ctas = ctas;
    return FG_OK;
}

int fg_get_cluster(fg_system *h, int32_t *ctas, int32_t *max_ctas) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (ctas) *ctas = eb_cluster_ctas(h);
    if (max_ctas) *max_ctas = eb_cluster_max(h);
    return FG_OK;
}

int fg_set_rebuild_policy(fg_system *h, int32_t skip) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    h->desc.skip_rebuild = skip ? 1 : 0;
    return push_desc(h);
}

int fg_trial_du(fg_system *h, int32_t n_moved, const int32_t *idx, const double *new_xyz, double *du) {
    if (!h || !idx || !new_xyz || !du) return fail(FG_ERR_INVALID, "null argument");
    if (!h->state_set) return fail(FG_ERR_STATE, "fg_set_state first");
    if (n_moved != 1) return fail(FG_ERR_INVALID, "atomic systems move one particle per trial");
    if (idx[0] < 0 || idx[0] >= h->N) return fail(FG_ERR_INVALID, "particle index out of range");
    for (int a = 0; a < 3; a++)
        if (!std::isfinite(new_xyz[a])) return fail(FG_ERR_INVALID, "non-finite coordinate");
    const int64_t req[4] = {idx[0], to_fix(new_xyz[0], h->P.box[0]), to_fix(new_xyz[1], h->P.box[1]),
                            to_fix(new_xyz[2], h->P.box[2])};
    CK(cudaMemcpyAsync(h->req, req, sizeof(req), cudaMemcpyHostToDevice, h->stream));
    const int T = sweep_threads(h);
    const size_t sm = sweep_smem(h, false);
    TrialFn fn = trial_fn(h);
    int rc = set_smem_attr((const void *)fn, sm);
    if (rc) return rc;
    fn<<<1, T, sm, h->stream>>>(h->d_desc, h->req, h->trial_out, h->sc_tab);
    CK(cudaGetLastError());
    float2 out[3];
    CK(cudaMemcpyAsync(out, h->trial_out, sizeof(out), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    *du = df_val(out[0].x, out[0].y);
    h->trial_pending = true;
    return FG_OK;
}

int fg_commit(fg_system *h, int32_t accepted, double *correction) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (!h->trial_pending) return fail(FG_ERR_STATE, "no pending trial");
    h->trial_pending = false;
    if (correction) *correction = 0.0;
    if (!accepted) return FG_OK;
    const int T = sweep_threads(h);
    const size_t sm = sweep_smem(h, false);
    CommitFn fn = commit_fn(h);
    int rc = set_smem_attr((const void *)fn, sm);
    if (rc) return rc;
    fn<<<1, T, sm, h->stream>>>(h->d_desc, h->req, h->trial_out, h->sc_tab);
    CK(cudaGetLastError());
    if (h->model == FG_MODEL_EWALD_WCA && !h->desc.skip_rebuild) {
        // the host mirrors the rebuild counter (NonbondedEwald::update, ewald.h:633)
        if (++h->cnt_accepted_host > h->P.ewald_update_frequency - 1) {
            h->cnt_accepted_host = 0;
            const int one = 1;
            CK(cudaMemcpyAsync(&h->sc->rebuild_pending, &one, sizeof(int), cudaMemcpyHostToDevice, h->stream));
            rc = launch_rebuild(h->d_desc, 1, h->N, h->nseg, h->kc, h->corr, h->stream);
            if (rc) return rc;
            float2 e;
            CK(cudaMemcpyAsync(&e, h->corr, sizeof(e), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            if (correction) *correction = df_val(e.x, e.y);
            SysScalars s;
            rc = read_scalars(h, s);
            if (rc) return rc;
            if (s.error) return fail(FG_ERR_DEVICE, "device error flags 0x%x", s.error);
        }
    }
    return FG_OK;
}

int fg_rebuild_qk(fg_system *h, double *correction) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (correction) *correction = 0.0;
    if (h->K == 0) return FG_OK;
    const int one = 1;
    CK(cudaMemcpyAsync(&h->sc->rebuild_pending, &one, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    int rc = launch_rebuild(h->d_desc, 1, h->N, h->nseg, h->kc, h->corr, h->stream);
    if (rc) return rc;
    float2 e;
    CK(cudaMemcpyAsync(&e, h->corr, sizeof(e), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (correction) *correction = df_val(e.x, e.y);
    SysScalars s;
    rc = read_scalars(h, s);
    if (rc) return rc;
    if (s.error) return fail(FG_ERR_DEVICE, "device error flags 0x%x", s.error);
    return FG_OK;
}

int fg_get_qk(fg_system *h, double *qk) {
    if (!h || !qk) return fail(FG_ERR_INVALID, "null argument");
    std::vector<double> q;
    int rc = get_qk_host(h, q);
    if (rc) return rc;
    std::copy(q.begin(), q.end(), qk);
    return FG_OK;
}

int fg_total_energy(fg_system *h, double *c) {
    if (!h || !c) return fail(FG_ERR_INVALID, "null argument");
    return total_energy(h, c);
}

int fg_running_energy(fg_system *h, double *u) {
    if (!h || !u) return fail(FG_ERR_INVALID, "null argument");
    SysScalars s;
    int rc = read_scalars(h, s);
    if (rc) return rc;
    *u = df_val(s.utot_hi, s.utot_lo);
    return FG_OK;
}

int fg_draw_translation_stream(fg_system *h, uint32_t seed, int64_t n, int32_t *idx, double *disp, double *u) {
    if (!h || !idx || !disp || !u || n < 0) return fail(FG_ERR_INVALID, "bad argument");
    if (h->types.empty()) return fail(FG_ERR_STATE, "fg_set_state first");
    // RandomTwister (slump.h:24-126): mt19937, uniform_int_distribution per
    // call, uniform_real_distribution<double>(0,1)
    std::mt19937 eng(seed);
    std::uniform_real_distribution<double> uni(0, 1);
    for (int64_t t = 0; t < n; t++) {
        { std::uniform_int_distribution<int> g(0, 0); g(eng); }            // slump.element(groups)
        int i;
        { std::uniform_int_distribution<int> g(0, h->N - 1); i = g(eng); } // Group::random
        const double dp = h->P.type_dp[h->types[i]];
        double tx = dp, ty = dp, tz = dp;                                   // dir * dp, dir = (1,1,1)
        tx *= uni(eng) - 0.5;
        ty *= uni(eng) - 0.5;
        tz *= uni(eng) - 0.5;
        idx[t] = i;
        disp[3 * t] = tx;
        disp[3 * t + 1] = ty;
        disp[3 * t + 2] = tz;
        u[t] = uni(eng);                                                    // Movebase::metropolis
    }
    return FG_OK;
}

// The caller's arrays are copied as they are and turned into trial records
// on the device (make_trials_kernel: to_fix for the displacement, -ln u as a
// float pair for the threshold), so the host does no per-trial work. The call
// returns when the records are in place: batches and parallel tempering run
// them from their own stream, and the caller may reuse its arrays.
int fg_stream_upload(fg_system *h, int64_t n, const int32_t *idx, const double *disp, const double *u) {
    if (!h || n < 0 || (n > 0 && (!idx || !disp || !u))) return fail(FG_ERR_INVALID, "bad argument");
    for (int64_t t = 0; t < n; t++)
        if (idx[t] < 0 || idx[t] >= h->N) return fail(FG_ERR_INVALID, "particle index out of range at %lld", (long long)t);
    int rc = ensure_trials(h, n, false);
    if (rc) return rc;
    if (n > h->raw_cap) {
        void *ptrs[] = {h->raw_idx, h->raw_disp, h->raw_u};
        for (void *p : ptrs)
            if (p) cudaFree(p);
        h->raw_idx = nullptr;
        h->raw_disp = h->raw_u = nullptr;
        h->raw_cap = 0;
        DMALLOC(h->raw_idx, n * sizeof(int32_t));
        DMALLOC(h->raw_disp, 3 * n * sizeof(double));
        DMALLOC(h->raw_u, n * sizeof(double));
        h->raw_cap = n;
    }
    if (n > 0) {
        CK(cudaMemcpyAsync(h->raw_idx, idx, n * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->raw_disp, disp, 3 * n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(h->raw_u, u, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)dh_sm_count() * 8);
        fg::make_trials_kernel<<<blocks, 256, 0, h->stream>>>(n, h->raw_idx, h->raw_disp, h->raw_u, h->P.box[0],
                                                              h->P.box[1], h->P.box[2], h->trials);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(h->stream));
    }
    h->n_trials = n;
    return FG_OK;
}

int fg_stream_philox(fg_system *h, int64_t n, uint32_t seed, uint32_t stream_id) {
    if (!h || n < 0) return fail(FG_ERR_INVALID, "bad argument");
    int rc = ensure_trials(h, n, false);
    if (rc) return rc;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)dh_sm_count() * 8));
    if (n > 0)
        fg::philox_stream_kernel<<<blocks, 256, 0, h->stream>>>(h->d_desc, seed, stream_id, 0, n, h->dp_fix, h->trials);
    CK(cudaGetLastError());
    // as fg_stream_upload: the records are in place on return, because
    // batches and parallel tempering read them from their own stream
    CK(cudaStreamSynchronize(h->stream));
    h->n_trials = n;
    return FG_OK;
}

int fg_stream_get(fg_system *h, int64_t first, int64_t n, int32_t *idx, double *disp, double *u) {
    if (!h || first < 0 || n < 0 || first + n > h->n_trials) return fail(FG_ERR_INVALID, "range outside the stream");
    if (n == 0) return FG_OK;
    std::vector<Trial> tr(n);
    CK(cudaMemcpyAsync(tr.data(), h->trials + first, n * sizeof(Trial), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int64_t t = 0; t < n; t++) {
        if (idx) idx[t] = tr[t].idx;
        for (int a = 0; a < 3; a++)
            if (disp) disp[3 * t + a] = from_fix(tr[t].d[a], h->P.box[a]);
        if (u) u[t] = std::exp(-df_val(tr[t].thr_hi, tr[t].thr_lo));
    }
    return FG_OK;
}

int fg_stream_run(fg_system *h, fg_sweep_stats *stats) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (!h->state_set) return fail(FG_ERR_STATE, "fg_set_state first");
    if (h->trial_pending) return fail(FG_ERR_STATE, "commit the pending trial first");
    return run_stream(h, h->n_trials, false, stats);
}

int fg_sweep(fg_system *h, int64_t n, const int32_t *idx, const double *disp, const double *u, uint8_t *accepted,
             double *du, fg_sweep_stats *stats) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (!h->state_set) return fail(FG_ERR_STATE, "fg_set_state first");
    if (h->trial_pending) return fail(FG_ERR_STATE, "commit the pending trial first");
    int rc = fg_stream_upload(h, n, idx, disp, u);
    if (rc) return rc;
    const bool log = accepted || du;
    rc = ensure_trials(h, n, log);
    if (rc) return rc;
    rc = run_stream(h, n, log, stats);
    if (rc) return rc;
    if (log && n > 0) {
        std::vector<float2> d(n);
        std::vector<uint8_t> a(n);
        CK(cudaMemcpyAsync(d.data(), h->log_du, n * sizeof(float2), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(a.data(), h->log_acc, n, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        for (int64_t t = 0; t < n; t++) {
            if (du) du[t] = df_val(d[t].x, d[t].y);
            if (accepted) accepted[t] = a[t];
        }
    }
    return FG_OK;
}

int fg_log_get(fg_system *h, int64_t first, int64_t n, double *du, uint8_t *accepted) {
    if (!h || first < 0 || n < 0) return fail(FG_ERR_INVALID, "bad argument");
    if (first + n > h->log_n) return fail(FG_ERR_INVALID, "range outside the last logged run (%lld trials)",
                                          (long long)h->log_n);
    if (n == 0) return FG_OK;
    std::vector<float2> d(n);
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(d.data(), h->log_du + first, n * sizeof(float2), cudaMemcpyDeviceToHost));
    if (accepted) CK(cudaMemcpy(accepted, h->log_acc + first, n, cudaMemcpyDeviceToHost));
    if (du)
        for (int64_t t = 0; t < n; t++) du[t] = df_val(d[t].x, d[t].y);
    return FG_OK;
}

int fg_synchronize(fg_system *h) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    CK(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

int64_t fg_device_bytes(fg_system *h) { return h ? (int64_t)h->device_bytes : 0; }

}  // extern "C"

#include "fg_batch.cu"
#include "fg_snapshot.cu"
#include "fg_noalloc.cu"
#include "fg_mol.cu"
#include "fg_tune.cu"
#include "fg_rdf.cu"
#include "fg_state.cu"
#include "fg_energy64.cu"
#include "fg_volume.cu"
#include "fg_dip.cu"
