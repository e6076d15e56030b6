// Pair distribution sampling on the device (included by fg_api.cu).
//
// Restates AtomRDF::update (analysis.h:2116-2134): every unordered pair
// i < j whose atom ids are {id1, id2} adds one count at the minimum-image
// distance r (Cuboid::sqdist, geometry.h:507-515, and dist = sqrt of it),
// binned as Table2D::round does (auxiliary.h:831): bin = int(r / dr + 0.5).
// The distance is formed in FP64 from the exact 64-bit fixed-point
// difference (its wrap is the minimum image), so a bin differs from the
// reference's only where r / dr + 0.5 lies within ~1e-15 of an integer.
namespace fg {

constexpr int kRdfThreads = 256;
constexpr int kRdfTile = 256;        // j positions staged per pass
constexpr int kRdfMaxBins = 8192;    // shared-memory histogram (uint32)

__global__ void __launch_bounds__(kRdfThreads) rdf_kernel(const SysDesc *__restrict__ dsc, int t1, int t2,
                                                        double3 sc, double inv_dr, int n_bins,
                                                        unsigned long long *__restrict__ hist,
                                                        unsigned long long *__restrict__ n_pairs) {
    __shared__ uint32_t h[kRdfMaxBins];
    __shared__ long long pj[kRdfTile][3];
    __shared__ uint8_t tj[kRdfTile];
    __shared__ unsigned long long cnt;
    const SysDesc &d = *dsc;
    for (int b = threadIdx.x; b < n_bins; b += blockDim.x) h[b] = 0u;
    if (threadIdx.x == 0) cnt = 0ull;
    const int N = d.N;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    long long xi[3] = {0, 0, 0};
    int ti = -1;
    if (i < N) {
#pragma unroll
        for (int a = 0; a < 3; a++) xi[a] = d.pos64[3 * i + a];
        ti = d.ptype[i];
    }
    const bool want = ti == t1 || ti == t2;
    const int other = ti == t1 ? t2 : t1;
    unsigned long long mine = 0;
    const int j_first = blockIdx.x * blockDim.x;   // pairs j > i only
    for (int j0 = j_first; j0 < N; j0 += kRdfTile) {
        __syncthreads();
        for (int t = threadIdx.x; t < kRdfTile; t += blockDim.x) {
            const int j = j0 + t;
            if (j < N) {
#pragma unroll
                for (int a = 0; a < 3; a++) pj[t][a] = d.pos64[3 * j + a];
                tj[t] = d.ptype[j];
            }
        }
        __syncthreads();
        if (!want) continue;
        const int nj = min(kRdfTile, N - j0);
        for (int t = 0; t < nj; t++) {
            const int j = j0 + t;
            if (j <= i || tj[t] != other) continue;
            double r2 = 0.0;
            const double s3[3] = {sc.x, sc.y, sc.z};   // L / 2^64 per axis (FP64 box lengths)
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const double x = (double)(long long)((unsigned long long)xi[a] - (unsigned long long)pj[t][a]) * s3[a];
                r2 = fma(x, x, r2);
            }
            const double fb = sqrt(r2) * inv_dr + 0.5;   // >= 0.5: compared before the integer cast
            mine++;
            if (fb < (double)n_bins) atomicAdd(&h[(int)fb], 1u);
        }
    }
    atomicAdd(&cnt, mine);
    __syncthreads();
    for (int b = threadIdx.x; b < n_bins; b += blockDim.x)
        if (h[b]) atomicAdd(&hist[b], (unsigned long long)h[b]);
    if (threadIdx.x == 0 && cnt) atomicAdd(n_pairs, cnt);
}

}  // namespace fg

extern "C" int fg_rdf_sample(fg_system *h, int32_t type1, int32_t type2, double dr, int32_t n_bins, int64_t *hist,
                             int64_t *n_pairs) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (h->types.empty()) return fail(FG_ERR_STATE, "fg_set_state first");
    if (!(dr > 0.0) || n_bins < 1 || n_bins > fg::kRdfMaxBins || !hist)
        return fail(FG_ERR_INVALID, "need dr > 0, 1 <= n_bins <= %d and a histogram", fg::kRdfMaxBins);
    if (type1 < 0 || type2 < 0 || type1 >= h->P.n_types || type2 >= h->P.n_types)
        return fail(FG_ERR_INVALID, "type id out of range");
    unsigned long long *d_buf = nullptr;
    const size_t bytes = ((size_t)n_bins + 1) * sizeof(unsigned long long);
    if (cudaMalloc(&d_buf, bytes) != cudaSuccess) return fail(FG_ERR_CUDA, "rdf buffer allocation failed");
    std::vector<unsigned long long> out((size_t)n_bins + 1);
    cudaError_t e = cudaMemsetAsync(d_buf, 0, bytes, h->stream);
    if (e == cudaSuccess) {
        fg::rdf_kernel<<<(h->N + fg::kRdfThreads - 1) / fg::kRdfThreads, fg::kRdfThreads, 0, h->stream>>>(
            h->d_desc, type1, type2,
            make_double3(std::ldexp(h->P.box[0], -64), std::ldexp(h->P.box[1], -64), std::ldexp(h->P.box[2], -64)),
            1.0 / dr, n_bins, d_buf, d_buf + n_bins);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out.data(), d_buf, bytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d_buf);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, "rdf: %s", cudaGetErrorString(e));
    for (int b = 0; b < n_bins; b++) hist[b] += (int64_t)out[b];
    if (n_pairs) *n_pairs += (int64_t)out[n_bins];
    return FG_OK;
}
