// FP64 system energy on the device (included by fg_api.cu): the reference's
// systemEnergy (energy.h:169-180) with every term in double precision, for
// moves whose dU is a difference of whole-system energies (the isobaric
// volume move) and for energy reports that need more than the FP32 pair
// path's ~1e-4 kT.
//
//   pairs: EwaldReal (ewald.h:97-110: the kappa-screened erfc form with the
//          effective charges' QeQe) + WeeksChandlerAndersen
//          (potentials.h:2186-2193), or DebyeHuckel (potentials.h:3314-3323)
//          + LennardJonesMixed (potentials.h:2036-2040), over all pairs i < j
//          with the minimum-image distance from the 64-bit fixed-point
//          difference;
//   Q(k):  sum_j q_j eff_j e^{i k.r_j} (ewald.h:388-415) with the phase
//          2 pi (n . X mod 2^64) / 2^64 taken exactly in integers, then sincos
//          in FP64; the reciprocal, self and surface terms are formed on the
//          host (ewald.h:259-311).
// Partial sums come back per block and are added on the host in a fixed
// order, so the result does not depend on timing.
namespace fg {

constexpr int kE64Threads = 256;
constexpr int kE64Tile = 256;

struct E64Pair {       // per type pair (row-major nt x nt)
    double s2, eps4, qeqe, wca2;
};

__global__ void __launch_bounds__(kE64Threads) energy64_pairs_kernel(const SysDesc *__restrict__ dsc,
                                                                   const double *__restrict__ q,
                                                                   const E64Pair *__restrict__ tp, int nt,
                                                                   double3 sc, double lB, double alpha,
                                                                   double kappa, double rc2, int ewald,
                                                                   double *__restrict__ part) {
    __shared__ long long pj[kE64Tile][3];
    __shared__ double qj[kE64Tile];
    __shared__ int tj[kE64Tile];
    __shared__ double red[kE64Threads / 32];
    const SysDesc &d = *dsc;
    const int N = d.N;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    long long xi[3] = {0, 0, 0};
    double qi = 0.0;
    int ti = 0;
    if (i < N) {
        for (int a = 0; a < 3; a++) xi[a] = d.pos64[3 * i + a];
        qi = q[i];
        ti = d.ptype[i];
    }
    const double s3[3] = {sc.x, sc.y, sc.z};
    const double k2a = ewald && kappa > 0.0 ? kappa / (2.0 * alpha) : 0.0;
    double acc = 0.0;
    for (int j0 = blockIdx.x * blockDim.x; j0 < N; j0 += kE64Tile) {
        __syncthreads();
        for (int t = threadIdx.x; t < kE64Tile; t += blockDim.x) {
            const int j = j0 + t;
            if (j < N) {
                for (int a = 0; a < 3; a++) pj[t][a] = d.pos64[3 * j + a];
                qj[t] = q[j];
                tj[t] = d.ptype[j];
            }
        }
        __syncthreads();
        if (i >= N) continue;
        const int nj = min(kE64Tile, N - j0);
        for (int t = 0; t < nj; t++) {
            if (j0 + t <= i) continue;
            double r2 = 0.0;
            for (int a = 0; a < 3; a++) {
                const double x = (double)(long long)((unsigned long long)xi[a] - (unsigned long long)pj[t][a]) * s3[a];
                r2 = fma(x, x, r2);
            }
            const E64Pair P = tp[ti * nt + tj[t]];
            const double r = sqrt(r2);
            double u = 0.0;
            if (ewald) {
                if (r2 <= rc2) {
                    const double qq = qi * qj[t] * P.qeqe * lB;
                    if (k2a == 0.0) {
                        u = qq * erfc(alpha * r) / r;
                    } else {
                        u = qq * 0.5 * (erfc(alpha * r + k2a) * exp(kappa * r) + erfc(alpha * r - k2a) * exp(-kappa * r)) / r;
                    }
                }
                if (r2 <= P.wca2) {
                    double x = P.s2 / r2;
                    x = x * x * x;
                    u += P.eps4 * (x * x - x + 0.25);
                }
            } else {
                double x = P.s2 / r2;
                x = x * x * x;
                u = lB * qi * qj[t] * exp(-kappa * r) / r + P.eps4 * (x * x - x);
            }
            acc += u;
        }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
        part[blockIdx.x] = s;
    }
}

// Partial Q(k) of particle chunk blockIdx.y for k = blockIdx.x * blockDim.x + tid.
__global__ void __launch_bounds__(kE64Threads) energy64_qk_kernel(const SysDesc *__restrict__ dsc,
                                                                const double *__restrict__ qe, int chunk,
                                                                double2 *__restrict__ part) {
    __shared__ long long pj[kE64Tile][3];
    __shared__ double qj[kE64Tile];
    const SysDesc &d = *dsc;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int nx = 0, ny = 0, nz = 0;
    if (k < d.K) unpack_n(d.kpack[k], nx, ny, nz);
    const int j0 = blockIdx.y * chunk, j1 = min(d.N, j0 + chunk);
    double re = 0.0, im = 0.0;
    for (int b = j0; b < j1; b += kE64Tile) {
        __syncthreads();
        for (int t = threadIdx.x; t < kE64Tile; t += blockDim.x) {
            const int j = b + t;
            if (j < j1) {
                for (int a = 0; a < 3; a++) pj[t][a] = d.pos64[3 * j + a];
                qj[t] = qe[j];
            }
        }
        __syncthreads();
        if (k >= d.K) continue;
        const int nb = min(kE64Tile, j1 - b);
        for (int t = 0; t < nb && d.iso; t++) {   // isotropic_pbc: q eff cos cos cos, real
            double c = qj[t];
            const int nn[3] = {nx, ny, nz};
            for (int a = 0; a < 3; a++)
                c *= cos((double)(long long)((unsigned long long)(long long)nn[a] * (unsigned long long)pj[t][a]) *
                         3.4061215800865545e-19);
            re += c;
        }
        for (int t = 0; t < nb && !d.iso; t++) {
            const unsigned long long ph = (unsigned long long)(long long)nx * (unsigned long long)pj[t][0] +
                                          (unsigned long long)(long long)ny * (unsigned long long)pj[t][1] +
                                          (unsigned long long)(long long)nz * (unsigned long long)pj[t][2];
            // 2 pi / 2^64 times the signed turn fraction
            const double ang = (double)(long long)ph * 3.4061215800865545e-19;
            double s, c;
            sincos(ang, &s, &c);
            re = fma(qj[t], c, re);
            im = fma(qj[t], s, im);
        }
    }
    if (k < d.K) part[(size_t)blockIdx.y * d.K + k] = make_double2(re, im);
}

}  // namespace fg

namespace {

// {pairs, reciprocal, self, surface, total} in kT, FP64 throughout, of the
// current configuration in each of nbox boxes: boxes[b] (box b's lengths;
// the fixed-point positions X = x / L 2^64 stand for x = X L / 2^64 in any
// box, so scaling every position with the box is the same X). Q(k) comes
// from one pass (its exact phases depend on X only), the pair sum from one
// pass per box at that box's scale, and the k-vector weights, reciprocal
// prefactor and surface term are those of each box (ewald.h:330-378, 277-311).
int total_energy_fp64_boxes(fg_system *h, int nbox, const double (*boxes)[3], double (*c)[5]) {
    const int N = h->N, nt = h->P.n_types;
    const fg_params &P = h->P;
    const bool ewald = h->model == FG_MODEL_EWALD_WCA;
    std::vector<fg::E64Pair> tp((size_t)nt * nt);
    std::vector<double> eff(nt, 1.0);
    const double kappa = ewald ? 1.0 / P.ewald_debye_length : 1.0 / P.dh_debye_length;
    for (int i = 0; i < nt; i++) {
        const double ri = 0.5 * P.type_sigma[i];
        if (ewald && P.type_charge[i] != 0.0 && std::fabs(kappa * ri) > 1e-9) eff[i] = std::sinh(ri * kappa) / ri / kappa;
    }
    for (int i = 0; i < nt; i++)
        for (int j = 0; j < nt; j++) {
            const double sig = 0.5 * (P.type_sigma[i] + P.type_sigma[j]);
            fg::E64Pair &e = tp[(size_t)i * nt + j];
            e.s2 = sig * sig;
            e.eps4 = 4 * std::sqrt(P.type_eps[i] * P.type_eps[j]);
            e.qeqe = eff[i] * eff[j];
            e.wca2 = e.s2 * std::pow(2, 2 / 6.);
        }
    std::vector<double> qe(N);
    for (int j = 0; j < N; j++) qe[j] = h->charges[j] * eff[h->types[j]];
    const int nb = (N + fg::kE64Threads - 1) / fg::kE64Threads;
    const int chunk = 1024, nchunk = (N + chunk - 1) / chunk;
    const int K = h->K;
    double *d_q = nullptr, *d_qe = nullptr, *d_part = nullptr;
    double2 *d_qk = nullptr;
    fg::E64Pair *d_tp = nullptr;
    auto release = [&]() {
        cudaFree(d_q);
        cudaFree(d_qe);
        cudaFree(d_part);
        cudaFree(d_qk);
        cudaFree(d_tp);
    };
    if (cudaMalloc(&d_q, N * sizeof(double)) != cudaSuccess || cudaMalloc(&d_qe, N * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&d_part, (size_t)nbox * nb * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&d_tp, tp.size() * sizeof(fg::E64Pair)) != cudaSuccess ||
        (K > 0 && cudaMalloc(&d_qk, (size_t)nchunk * K * sizeof(double2)) != cudaSuccess)) {
        release();
        return fail(FG_ERR_CUDA, "FP64 energy buffers");
    }
    cudaError_t e = cudaMemcpyAsync(d_q, h->charges.data(), N * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_qe, qe.data(), N * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_tp, tp.data(), tp.size() * sizeof(fg::E64Pair), cudaMemcpyHostToDevice, h->stream);
    for (int b = 0; b < nbox && e == cudaSuccess; b++) {
        const double3 sc = make_double3(std::ldexp(boxes[b][0], -64), std::ldexp(boxes[b][1], -64),
                                        std::ldexp(boxes[b][2], -64));
        fg::energy64_pairs_kernel<<<nb, fg::kE64Threads, 0, h->stream>>>(
            h->d_desc, d_q, d_tp, nt, sc, P.bjerrum, ewald ? P.ewald_alpha : 0.0, kappa,
            ewald ? P.ewald_cutoff * P.ewald_cutoff : 0.0, ewald ? 1 : 0, d_part + (size_t)b * nb);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && K > 0) {
        fg::energy64_qk_kernel<<<dim3((K + fg::kE64Threads - 1) / fg::kE64Threads, nchunk), fg::kE64Threads, 0,
                                 h->stream>>>(h->d_desc, d_qe, chunk, d_qk);
        e = cudaGetLastError();
    }
    std::vector<double> part((size_t)nbox * nb);
    std::vector<double2> qk(K > 0 ? (size_t)nchunk * K : 0);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(part.data(), d_part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && K > 0)
        e = cudaMemcpyAsync(qk.data(), d_qk, qk.size() * sizeof(double2), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    release();
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, "FP64 energy: %s", cudaGetErrorString(e));
    std::vector<double> q2;   // |Q(k)|^2
    double M0[3] = {0, 0, 0};  // sum q eff x in the current box
    if (K > 0) {
        q2.resize(K);
        for (int k = 0; k < K; k++) {
            double re = 0, im = 0;
            for (int b = 0; b < nchunk; b++) {
                re += qk[(size_t)b * K + k].x;
                im += qk[(size_t)b * K + k].y;
            }
            q2[k] = re * re + im * im;
        }
        std::vector<double> xyz(3 * (size_t)N);
        int rc = fg_get_state(h, xyz.data());
        if (rc) return rc;
        for (int j = 0; j < N; j++)
            for (int a = 0; a < 3; a++) M0[a] += qe[j] * xyz[3 * j + a];
    }
    for (int b = 0; b < nbox; b++) {
        double pairs = 0;
        for (int i = 0; i < nb; i++) pairs += part[(size_t)b * nb + i];
        double rec = 0, self = 0, surf = 0;
        if (K > 0) {
            fg_params Pb = P;
            for (int a = 0; a < 3; a++) Pb.box[a] = boxes[b][a];
            const double V = Pb.box[0] * Pb.box[1] * Pb.box[2];
            std::vector<int> n3;
            std::vector<double> ak, kv3;
            enumerate_k(Pb, n3, ak, kv3);
            if ((int)ak.size() != K) return fail(FG_ERR_INVALID, "the k-vector set changes with the box");
            for (int k = 0; k < K; k++) rec += ak[k] * q2[k];
            rec *= 2 * PI / V * P.bjerrum;
            self = h->self_energy;
            const double const_inf = (P.ewald_eps_surf < 1) ? 0.0 : 1.0;
            const double surf_c = const_inf * (2 * PI / ((2 * P.ewald_eps_surf + 1) * V)) * P.bjerrum;
            double M2 = 0;
            for (int a = 0; a < 3; a++) {
                const double m = M0[a] * (boxes[b][a] / P.box[a]);
                M2 += m * m;
            }
            surf = surf_c * M2;
        }
        c[b][0] = pairs;
        c[b][1] = rec;
        c[b][2] = self;
        c[b][3] = surf;
        c[b][4] = (surf + rec) + (self + pairs);
    }
    return FG_OK;
}

int total_energy_fp64(fg_system *h, double *c) {
    const double box[1][3] = {{h->P.box[0], h->P.box[1], h->P.box[2]}};
    double out[1][5];
    int rc = total_energy_fp64_boxes(h, 1, box, out);
    if (rc) return rc;
    for (int i = 0; i < 5; i++) c[i] = out[0][i];
    return FG_OK;
}

}  // namespace

extern "C" int fg_total_energy_fp64(fg_system *h, double *components5) {
    if (!h || !components5) return fail(FG_ERR_INVALID, "null argument");
    if (h->types.empty()) return fail(FG_ERR_STATE, "fg_set_state first");
    return total_energy_fp64(h, components5);
}
