// Pair energy without any device allocation (included by fg_api.cu).
//
// Some callers cannot call cudaMalloc: a plugin running inside a host
// application that owns the whole GPU memory pool and hands out only
// buffers it allocated itself, or a time-critical loop that must not call
// the allocator because cudaMalloc/cudaFree may synchronize the device and
// stall other work. fg_pair_energy_noalloc serves them: the caller passes
// device buffers for the inputs and the output, and every temporary lives in
// one file-scope __device__ array of fixed size (about 1.7 MB, held by every
// GPU that loads this library until the process exits).
//
// The array is shared by all calls: calls that overlap on the GPU (on
// different streams, or from different host threads) race on it and give
// wrong results. Nothing in it has to start at zero: every call writes all of
// it that it later reads, and clears its error word first.
//
// Type ids cannot be checked on the host (they are in device memory): the
// conversion kernel checks 0 <= t < n_types, records a bad id in the error
// word and stores type 0 in its place, so no table is read out of range;
// the final kernel then writes NaN instead of the energy.

namespace fg {

constexpr size_t noalloc_align16(size_t b) { return (b + 15) & ~(size_t)15; }
constexpr int kNoallocMaxParticles = FG_NOALLOC_MAX_PARTICLES;
constexpr int kNoallocMaxTab = 2048;       // Taylor-table entries for core pairs
constexpr int kNoallocBlocks = 1024;       // pair_total_kernel grid (one partial each)
constexpr size_t kNoallocDesc = 0;
constexpr size_t kNoallocTab0 = noalloc_align16(sizeof(SysDesc));
constexpr size_t kNoallocTab1 = kNoallocTab0 + (size_t)kNoallocMaxTab * 16;
constexpr size_t kNoallocPos4 = kNoallocTab1 + (size_t)kNoallocMaxTab * 16;
constexpr size_t kNoallocExt = kNoallocPos4 + (size_t)kNoallocMaxParticles * 16;
constexpr size_t kNoallocType = kNoallocExt + (size_t)kNoallocMaxParticles * 8;
constexpr size_t kNoallocQtype = noalloc_align16(kNoallocType + (size_t)kNoallocMaxParticles);
constexpr size_t kNoallocPart = kNoallocQtype + (size_t)FG_MAX_TYPES * 4;
constexpr size_t kNoallocErr = kNoallocPart + (size_t)kNoallocBlocks * 8;
constexpr size_t kNoallocBytes = kNoallocErr + 16;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// Caller coordinates (double, Angstrom) -> the fixed-point records the pair
// kernels read, with the same rounding as the host upload (fg_set_state).
// The box comes in double precision (the descriptor holds it as float).
__global__ void noalloc_convert_kernel(int n, int n_types, double3 box, const double *__restrict__ xyz,
                                       const double *__restrict__ charge, const int32_t *__restrict__ types) {
    int4 *pos4 = reinterpret_cast<int4 *>(g_noalloc_scratch + kNoallocPos4);
    short4 *ext = reinterpret_cast<short4 *>(g_noalloc_scratch + kNoallocExt);
    uint8_t *pt = reinterpret_cast<uint8_t *>(g_noalloc_scratch + kNoallocType);
    const float *qtype = reinterpret_cast<const float *>(g_noalloc_scratch + kNoallocQtype);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int h[3], e[3];
        for (int a = 0; a < 3; a++) {
            const double L = a == 0 ? box.x : (a == 1 ? box.y : box.z);
            double f = xyz[3 * i + a] / L;
            f -= floor(f + 0.5);
            const int64_t X = (int64_t)((uint64_t)(int64_t)__double2ll_rn(f * 4611686018427387904.0) << 2);
            h[a] = hi32(X);
            e[a] = ext16(X);
        }
        int t = types[i];
        if (t < 0 || t >= n_types) {
            atomicOr(reinterpret_cast<int *>(g_noalloc_scratch + kNoallocErr), 1);
            t = 0;
        }
        const float q = charge ? (float)charge[i] : qtype[t];
        pos4[i] = make_int4(h[0], h[1], h[2], __float_as_int(q));
        ext[i] = make_short4((short)e[0], (short)e[1], (short)e[2], 0);
        pt[i] = (uint8_t)t;
    }
}

__global__ void noalloc_finish_kernel(double *__restrict__ out) {
    __shared__ float2 red[32];
    const float2 *part = reinterpret_cast<const float2 *>(g_noalloc_scratch + kNoallocPart);
    df acc = {0.0f, 0.0f};
    for (int b = threadIdx.x; b < kNoallocBlocks; b += blockDim.x) acc = df_add(acc, df{part[b].x, part[b].y});
    acc = warp_sum_df(acc);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) red[w] = make_float2(acc.hi, acc.lo);
    __syncthreads();
    if (w == 0) {
        df t = {0.0f, 0.0f};
        if (lane < (int)(blockDim.x >> 5)) t = {red[lane].x, red[lane].y};
        t = warp_sum_df(t);
        const int bad = *reinterpret_cast<const int *>(g_noalloc_scratch + kNoallocErr);
        if (lane == 0) out[0] = bad ? __longlong_as_double(0x7ff8000000000000LL) : (double)t.hi + (double)t.lo;
    }
}

}  // namespace fg

namespace {

std::mutex g_noalloc_mu;
void *g_noalloc_addr[64] = {nullptr};

// Device address of the scratch array for the current device: taken once per
// device, with that device current, on the first call there.
int noalloc_scratch(unsigned char **out) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(FG_ERR_CUDA, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, fg::g_noalloc_scratch);
        if (e != cudaSuccess) return fail(FG_ERR_CUDA, "cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        g_noalloc_addr[dev] = p;
    }
    *out = (unsigned char *)g_noalloc_addr[dev];
    return FG_OK;
}

}  // namespace

extern "C" {

int fg_pair_energy_noalloc(const fg_params *params, int32_t n, const double *d_xyz, const double *d_charge,
                           const int32_t *d_types, double *d_energy, void *stream) {
    if (!params || !d_xyz || !d_types || !d_energy) return fail(FG_ERR_INVALID, "null argument");
    const fg_params &P = *params;
    if (P.model != FG_MODEL_EWALD_WCA && P.model != FG_MODEL_DH_LJ)
        return fail(FG_ERR_INVALID, "model %d not supported", P.model);
    if (n < 2) return fail(FG_ERR_INVALID, "need at least two particles");
    if (n > fg::kNoallocMaxParticles)
        return fail(FG_ERR_CAPACITY, "%d particles exceed the no-allocation limit of %d", n, fg::kNoallocMaxParticles);
    if (P.n_types < 1 || P.n_types > FG_MAX_TYPES) return fail(FG_ERR_INVALID, "bad n_types %d", P.n_types);
    for (int a = 0; a < 3; a++)
        if (!(P.box[a] > 0)) return fail(FG_ERR_INVALID, "box must be positive");
    if (P.model == FG_MODEL_DH_LJ && (P.box[1] != P.box[0] || P.box[2] != P.box[0]))
        return fail(FG_ERR_INVALID, "Debye-Hueckel systems need a cubic box");
    if (P.model == FG_MODEL_EWALD_WCA) {
        if (!(P.ewald_alpha > 0) || !(P.ewald_cutoff > 0) || !(P.ewald_debye_length > 0))
            return fail(FG_ERR_INVALID, "Ewald needs alpha, cutoff and debye_length > 0");
        for (int i = 0; i < P.n_types; i++)
            if (P.type_charge[i] == 0.0)
                return fail(FG_ERR_INVALID, "Ewald effective charges need non-zero type charges (ewald.h:539)");
    } else if (!(P.dh_debye_length > 0)) {
        return fail(FG_ERR_INVALID, "dh_debye_length must be > 0");
    }
    const int nt = P.n_types;
    // the same tables fg_create builds (type pairs, effective charges, core-pair Taylor table)
    SysDesc d;
    std::memset(&d, 0, sizeof(d));
    d.model = P.model;
    d.N = n;
    d.n_types = nt;
    for (int a = 0; a < 3; a++) {
        d.L[a] = (float)P.box[a];
        d.s32[a] = (float)(P.box[a] / 4294967296.0);
        d.dl32[a] = (float)(P.box[a] / TWO64);
        d.s48_df[a] = split_df(P.box[a] / 281474976710656.0);
    }
    d.s32sq = (float)((P.box[0] / 4294967296.0) * (P.box[0] / 4294967296.0));
    d.lB = (float)P.bjerrum;
    d.kT = 1.0f;
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
    std::vector<double> eff(nt, 1.0);
    for (int i = 0; i < nt; i++) {
        const double ri = 0.5 * P.type_sigma[i];
        double qis = P.type_charge[i];
        if (P.model == FG_MODEL_EWALD_WCA) {
            if (std::fabs(kappa * ri) > 1e-9) qis *= std::sinh(ri * kappa) / ri / kappa;
            eff[i] = qis / P.type_charge[i];
        }
        d.eff[i] = (float)eff[i];
    }
    bool uniform = true;
    for (int i = 0; i < nt; i++)
        for (int j = 0; j < nt; j++) {
            const double sig = 0.5 * (P.type_sigma[i] + P.type_sigma[j]);
            const double s2 = sig * sig, e4 = 4 * std::sqrt(P.type_eps[i] * P.type_eps[j]);
            const int t = i * nt + j;
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
    float qtype[FG_MAX_TYPES] = {0};
    for (int i = 0; i < nt; i++) qtype[i] = (float)P.type_charge[i];
    unsigned char *base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc) return rc;
    const double coef = P.model == FG_MODEL_EWALD_WCA ? P.ewald_alpha : 1.0 / P.dh_debye_length;
    const bool ok = P.model == FG_MODEL_DH_LJ || d.kappa == 0.0f;
    double smax = 0;
    for (int i = 0; i < nt; i++) smax = std::max(smax, P.type_sigma[i]);
    const int ntab = ok && smax > 0 ? (int)std::ceil(coef * smax * 128.0) + 4 : 0;
    if (ntab > fg::kNoallocMaxTab) return fail(FG_ERR_CAPACITY, "core table of %d entries exceeds %d", ntab, fg::kNoallocMaxTab);
    std::vector<float4> t0(std::max(ntab, 1)), t1(std::max(ntab, 1));
    const double kk = 2.0 / std::sqrt(PI);
    for (int j = 0; j < ntab; j++) {
        const double y = j / 128.0;
        double f0, f1, f2, f3, f4;
        if (P.model == FG_MODEL_EWALD_WCA) {
            const double e = std::exp(-y * y);
            f0 = std::erfc(y);
            f1 = -kk * e;
            f2 = 2 * kk * y * e;
            f3 = 2 * kk * (1 - 2 * y * y) * e;
            f4 = 2 * kk * (4 * y * y * y - 6 * y) * e;
        } else {
            f0 = std::exp(-y);
            f1 = -f0; f2 = f0; f3 = -f0; f4 = f0;
        }
        const float2 a = split_df(f0), b = split_df(f1);
        t0[j] = make_float4(a.x, a.y, b.x, b.y);
        t1[j] = make_float4((float)(f2 / 2), (float)(f3 / 6), (float)(f4 / 24), 0.0f);
    }
    d.core_tab_n = ntab;
    d.coef_df = split_df(coef);
    d.core_tab = (const float4 *)(base + fg::kNoallocTab0);
    d.core_tab2 = (const float4 *)(base + fg::kNoallocTab1);
    d.pos4 = (int4 *)(base + fg::kNoallocPos4);
    d.pos_ext = (short4 *)(base + fg::kNoallocExt);
    d.ptype = (uint8_t *)(base + fg::kNoallocType);
    cudaStream_t st = (cudaStream_t)stream;
    CK(cudaMemcpyAsync(base + fg::kNoallocDesc, &d, sizeof(SysDesc), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(base + fg::kNoallocQtype, qtype, sizeof(qtype), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(base + fg::kNoallocErr, 0, 16, st));
    if (ntab > 0) {
        CK(cudaMemcpyAsync(base + fg::kNoallocTab0, t0.data(), ntab * sizeof(float4), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(base + fg::kNoallocTab1, t1.data(), ntab * sizeof(float4), cudaMemcpyHostToDevice, st));
    }
    fg::noalloc_convert_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, nt, make_double3(P.box[0], P.box[1], P.box[2]),
                                                                 d_xyz, d_charge, d_types);
    using PairFn = void (*)(const SysDesc *, float2 *);
    PairFn fn = P.model == FG_MODEL_EWALD_WCA ? fg::pair_total_kernel<fg::MODEL_EWALD>
                                               : fg::pair_total_kernel<fg::MODEL_DHLJ>;
    fn<<<fg::kNoallocBlocks, 256, 0, st>>>((const SysDesc *)(base + fg::kNoallocDesc),
                                           (float2 *)(base + fg::kNoallocPart));
    fg::noalloc_finish_kernel<<<1, 1024, 0, st>>>(d_energy);
    CK(cudaGetLastError());
    return FG_OK;
}

}  // extern "C"
