// Batches, parallel tempering and the job server (included by fg_api.cu).
//
// A batch is a set of independent systems advanced by one launch of the
// persistent sweep kernel (one CTA per system). Parallel tempering runs a
// batch whose systems sit on a temperature ladder and exchanges temperatures
// between neighbours on the device (the configuration exchange of
// Move::ParallelTempering, move.h:6542-6771, as a label swap). The job
// server admits Monte Carlo jobs by device-memory footprint and advances all
// admitted jobs together in rounds (continuous batching).

namespace fg {

// Reset per-system scalars for a new stream of counts[s] trials.
__global__ void batch_reset_kernel(const SysDesc *__restrict__ descs, int n, const int64_t *__restrict__ counts) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    SysScalars *sc = descs[s].sc;
    sc->cursor = 0;
    sc->n_trials = counts[s];
    sc->u_hi = 0.0f;
    sc->u_lo = 0.0f;
}

// Philox trial streams for all systems of a batch: system s gets counts[s]
// trials with counters starting at descs[s].stream_first + round * counts[s]
// (round read from the device, so a captured graph can be replayed).
__global__ void batch_philox_kernel(const SysDesc *__restrict__ descs, const int64_t *__restrict__ counts,
                                    const int64_t *__restrict__ round) {
    const SysDesc &d = descs[blockIdx.y];
    const int64_t n = counts[blockIdx.y];
    const int64_t first = d.stream_first + (round ? *round : 0) * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t g = first + t;
        const u4 r = philox4x32_10(u4{(uint32_t)g, (uint32_t)(g >> 32), 0u, 0u}, d.seed, d.stream_id);
        const u4 r2 = philox4x32_10(u4{(uint32_t)g, (uint32_t)(g >> 32), 1u, 0u}, d.seed, d.stream_id);
        Trial tr;
        tr.idx = (int32_t)(((uint64_t)r.x * (uint32_t)d.N) >> 32);
        tr.pad = 0;
        const int ty = d.ptype[tr.idx];
        tr.d[0] = (int64_t)(int32_t)(r.y - 0x80000000u) * d.dp_fix[3 * ty + 0];
        tr.d[1] = (int64_t)(int32_t)(r.z - 0x80000000u) * d.dp_fix[3 * ty + 1];
        tr.d[2] = (int64_t)(int32_t)(r.w - 0x80000000u) * d.dp_fix[3 * ty + 2];
        const double u = ((double)r2.x + 0.5) * (1.0 / 4294967296.0);
        const double thr = -log(u);
        const float h = (float)thr;
        tr.thr_hi = h;
        tr.thr_lo = (float)(thr - (double)h);
        const_cast<Trial *>(d.trials)[t] = tr;
    }
}

__global__ void gather_scalars_kernel(const SysDesc *__restrict__ descs, int n, SysScalars *__restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) out[s] = *descs[s].sc;
}

// Temperature exchange between neighbouring rungs (findPartner, move.h:6621-6633:
// one uniform picks the pairing (0,1)(2,3).. or (1,2)(3,4)..; then per pair
// the Metropolis test of _energyChange, move.h:6700-6722: the total
// dU = [U_i(x_b) - U_i(x_a)] + [U_p(x_a) - U_p(x_b)] = (beta_i - beta_p)(E_b - E_a)
// with E_a the energy of the system a at rung i, exchanged iff not u > exp(-dU)).
// perm[rung] = system; the swap exchanges perm entries and the systems' kT
// (the configurations stay where they are). By default the uniforms come from
// Philox (counter = the round) and E from the systems' running totals; with
// `given` = {u_direction, u_accept} every pair takes that one acceptance
// uniform (the reference's ranks all draw the same one from their global
// generator) and with `energies` E comes from that array (per system).
// One thread; n is small.
__global__ void pt_swap_kernel(SysDesc *__restrict__ descs, int n, int *__restrict__ perm,
                               const double *__restrict__ temps, uint32_t seed, int64_t *__restrict__ round,
                               long long *__restrict__ attempts, long long *__restrict__ accepts,
                               const double *__restrict__ given, const double *__restrict__ energies) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int64_t rd = *round;
    const u4 r = philox4x32_10(u4{(uint32_t)rd, (uint32_t)(rd >> 32), 0u, 0x50540000u}, seed, 0x50545054u);
    const double udir = given ? given[0] : (double)r.x * (1.0 / 4294967296.0);
    const int dr = udir > 0.5 ? 1 : -1;
    for (int i = 0; i < n; i++) {
        const int p = (i % 2 == 0) ? i + dr : i - dr;
        if (p <= i || p >= n) continue;
        const int a = perm[i], b = perm[p];
        const SysScalars *sa = descs[a].sc, *sb = descs[b].sc;
        const double ua = energies ? energies[a] : (double)sa->utot_hi + (double)sa->utot_lo;
        const double ub = energies ? energies[b] : (double)sb->utot_hi + (double)sb->utot_lo;
        const double arg = (1.0 / temps[i] - 1.0 / temps[p]) * (ua - ub);
        const u4 q = philox4x32_10(u4{(uint32_t)rd, (uint32_t)(rd >> 32), (uint32_t)i, 0x50540001u}, seed, 0x50545054u);
        const double u = given ? given[1] : ((double)q.x + 0.5) * (1.0 / 4294967296.0);
        attempts[i]++;
        if (!(u > exp(arg))) {
            accepts[i]++;
            perm[i] = b;
            perm[p] = a;
            descs[a].kT = (float)temps[p];
            descs[b].kT = (float)temps[i];
        }
    }
    *round = rd + 1;
}

}  // namespace fg

struct fg_batch {
    std::vector<fg_system *> sys;
    cudaStream_t stream = nullptr;
    SysDesc *d_descs = nullptr;
    SysScalars *d_gather = nullptr;
    float2 *d_corr = nullptr;
    int64_t *d_counts = nullptr;
    int threads = 0;
    LaunchCfg cfg{};
    int maxN = 0, maxK = 0, maxSeg = 0, maxKcc = 0;
    bool rebuilds = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // parallel tempering
    int *d_perm = nullptr;
    double *d_temps = nullptr;
    int64_t *d_round = nullptr;
    long long *d_att = nullptr, *d_acc = nullptr;
    double *d_given = nullptr;        // fg_pt_swap: {u_direction, u_accept}, then per-system energies
    uint32_t pt_seed = 0;
    bool pt = false;
    cudaGraphExec_t graph = nullptr;
    int64_t graph_sweeps = -1;
    // fg_batch_run without external rebuilds: reset, sweep and gather of a
    // run captured once and replayed
    cudaGraphExec_t run_graph = nullptr;
    int run_graph_kernels = 0;
    bool in_kernel_rebuild = false;
    int rebuild_mode = 0;   // 0: in-kernel when the batch fills the GPU, 1: always, 2: never
    // Debye-Hueckel members without a cell list run the block kernel
    bool dh_block = false;
    DhGroups dh;
    int min_per_cta = 0;   // schedule: least particles per CTA (0: the tuned process default)
    bool counted = false;  // members' batch counts include this batch
};

namespace {

int batch_config(fg_batch *b) {
    fg_system *h0 = b->sys[0];
    b->cfg.fn = sweep_fn(h0);
    int T = b->threads;
    size_t sm = 0;
    b->maxN = b->maxK = b->maxSeg = b->maxKcc = 0;
    bool all_dh = true;   // DH+LJ block members run by CTA-count groups, whatever their one-CTA variant
    for (fg_system *h : b->sys) all_dh = all_dh && dh_block_ok(h);
    for (fg_system *h : b->sys) {
        if (!all_dh && sweep_fn(h) != b->cfg.fn)
            return fail(FG_ERR_INVALID, "batch members need the same kernel variant");
        if (b->threads == 0 || ewald_block_ok(h)) T = std::max(T, sweep_launch_threads(h));
        sm = std::max(sm, sweep_launch_smem(h));
        b->maxN = std::max(b->maxN, h->N);
        b->maxK = std::max(b->maxK, h->K);
        b->maxSeg = std::max(b->maxSeg, h->nseg);
        b->maxKcc = std::max(b->maxKcc, h->kc);
    }
    b->cfg.threads = T;
    b->cfg.smem = sm;
    if (b->run_graph) {
        cudaGraphExecDestroy(b->run_graph);
        b->run_graph = nullptr;
    }
    // the Ewald block kernel rebuilds Q(k) inside the sweep when the batch
    // fills the GPU (at least one system per SM); smaller batches leave the
    // rebuilds to the rebuild kernel, which spreads them over all SMs
    b->in_kernel_rebuild = ewald_block_ok(h0) && (b->rebuild_mode == 1 ||
                                                  (b->rebuild_mode == 0 && (int)b->sys.size() >= dh_sm_count()));
    b->rebuilds = b->maxK > 0 && !h0->desc.skip_rebuild && !b->in_kernel_rebuild;
    b->dh_block = true;
    std::vector<int> Ns;
    std::vector<double> w;
    for (fg_system *h : b->sys) {
        if (!dh_block_ok(h)) b->dh_block = false;
        Ns.push_back(h->N);
        w.push_back((double)h->N * h->N);   // a sweep of N trials over N partners
    }
    if (b->dh_block)   // the one-CTA kernel (cfg.fn) is not launched for these members
        return dh_groups_build(b->dh, Ns, w, b->min_per_cta > 0 ? b->min_per_cta : tuned_min_per_cta());
    return set_smem_attr((const void *)b->cfg.fn, sm);
}

// The sweep launch(es) of one pass over all members.
int batch_sweep(fg_batch *b, int64_t end) {
    if (b->dh_block) return dh_groups_launch(b->dh, b->d_descs, end, b->stream);
    b->cfg.fn<<<(int)b->sys.size(), b->cfg.threads, b->cfg.smem, b->stream>>>(b->d_descs, end, b->sys[0]->sc_tab);
    CK(cudaGetLastError());
    return FG_OK;
}

int batch_push_descs(fg_batch *b) {
    std::vector<SysDesc> v(b->sys.size());
    for (size_t s = 0; s < b->sys.size(); s++) {
        fg_system *h = b->sys[s];
        h->desc.trials = h->trials;
        // per-trial log of selected members (fg_batch_set_log), where the
        // buffers hold the member's whole stream
        const bool log = h->log_batch && !b->pt && h->log_cap >= h->n_trials;
        h->desc.log_trials = log ? 1 : 0;
        h->desc.rebuild_in_kernel = b->in_kernel_rebuild ? 1 : 0;
        h->desc.trial_du = h->log_du;
        h->desc.trial_acc = h->log_acc;
        v[s] = h->desc;
    }
    CK(cudaMemcpyAsync(b->d_descs, v.data(), v.size() * sizeof(SysDesc), cudaMemcpyHostToDevice, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return FG_OK;
}

// One run as a CUDA graph: reset the members' stream cursors, the sweep
// launch(es) over all members, gather the scalars. Captured on first use.
int batch_run_graph(fg_batch *b) {
    if (b->run_graph) return FG_OK;
    const int n = (int)b->sys.size();
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    fg::batch_reset_kernel<<<(n + 127) / 128, 128, 0, b->stream>>>(b->d_descs, n, b->d_counts);
    int rc = batch_sweep(b, INT64_MAX);
    fg::gather_scalars_kernel<<<(n + 127) / 128, 128, 0, b->stream>>>(b->d_descs, n, b->d_gather);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
        if (e == cudaSuccess) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    size_t nodes = 0;
    cudaGraphGetNodes(g, nullptr, &nodes);
    e = cudaGraphInstantiate(&b->run_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    b->run_graph_kernels = (int)(b->dh_block ? b->dh.C.size() + 2 : 3);
    (void)nodes;
    return FG_OK;
}

// Run every member's staged stream of counts[s] trials (also on the device).
int batch_run(fg_batch *b, const std::vector<int64_t> &counts, fg_sweep_stats *per, fg_sweep_stats *total) {
    const int n = (int)b->sys.size();
    std::vector<SysScalars> s0(n), s(n);
    fg::gather_scalars_kernel<<<(n + 127) / 128, 128, 0, b->stream>>>(b->d_descs, n, b->d_gather);
    CK(cudaMemcpyAsync(s0.data(), b->d_gather, n * sizeof(SysScalars), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    int launches = 0;
    int64_t kernels = 1;   // the first gather
    std::vector<cudaEvent_t> evs;
    bool graphed = false;
    if (!b->rebuilds) {
        // no external rebuilds: one launch runs every member's whole stream
        int rc = batch_run_graph(b);
        if (rc) return rc;
        CK(cudaEventRecord(b->ev0, b->stream));
        CK(cudaGraphLaunch(b->run_graph, b->stream));
        CK(cudaEventRecord(b->ev1, b->stream));
        CK(cudaMemcpyAsync(s.data(), b->d_gather, n * sizeof(SysScalars), cudaMemcpyDeviceToHost, b->stream));
        CK(cudaStreamSynchronize(b->stream));
        launches = 1;
        kernels += b->run_graph_kernels;
        graphed = true;
    } else {
        fg::batch_reset_kernel<<<(n + 127) / 128, 128, 0, b->stream>>>(b->d_descs, n, b->d_counts);
        CK(cudaEventRecord(b->ev0, b->stream));
        kernels++;
    }
    const int uf = std::max(b->sys[0]->P.ewald_update_frequency, 1);
    int64_t maxc = 0;
    for (auto c : counts) maxc = std::max(maxc, c);
    int64_t prev_done = -1;
    while (!graphed) {
        const int pairs = b->rebuilds ? (int)std::min<int64_t>(maxc / uf + 1, 64) : 1;
        for (int p = 0; p < pairs; p++) {
            cudaEvent_t e0, e1;
            CK(cudaEventCreate(&e0));
            CK(cudaEventCreate(&e1));
            evs.push_back(e0);
            evs.push_back(e1);
            CK(cudaEventRecord(e0, b->stream));
            {
                int rc = batch_sweep(b, INT64_MAX);
                if (rc) return rc;
            }
            CK(cudaEventRecord(e1, b->stream));
            launches++;
            kernels++;
            if (b->rebuilds) {
                int rc = launch_rebuild(b->d_descs, n, b->maxN, b->maxSeg, b->maxKcc, b->d_corr, b->stream);
                if (rc) return rc;
                kernels += 2;
            }
        }
        kernels++;
        fg::gather_scalars_kernel<<<(n + 127) / 128, 128, 0, b->stream>>>(b->d_descs, n, b->d_gather);
        CK(cudaMemcpyAsync(s.data(), b->d_gather, n * sizeof(SysScalars), cudaMemcpyDeviceToHost, b->stream));
        CK(cudaStreamSynchronize(b->stream));
        bool done = true, err = false;
        int64_t sum = 0;
        for (int i = 0; i < n; i++) {
            if (s[i].error) err = true;
            if (s[i].cursor < counts[i] || s[i].rebuild_pending) done = false;
            sum += s[i].cursor;
        }
        if (err || done) break;
        if (sum == prev_done) return fail(FG_ERR_DEVICE, "batch made no progress");
        prev_done = sum;
    }
    if (graphed) {
        for (int i = 0; i < n; i++)
            if (!s[i].error && s[i].cursor < counts[i])
                return fail(FG_ERR_DEVICE, "batch member %d stopped at trial %lld of %lld", i,
                            (long long)s[i].cursor, (long long)counts[i]);
    } else {
        CK(cudaEventRecord(b->ev1, b->stream));
    }
    CK(cudaEventSynchronize(b->ev1));
    float ms = 0.0f, sweep_ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    if (graphed) sweep_ms = ms;   // the graph's reset and gather take microseconds
    for (size_t e = 0; e + 1 < evs.size(); e += 2) {
        float t = 0.0f;
        CK(cudaEventElapsedTime(&t, evs[e], evs[e + 1]));
        sweep_ms += t;
        cudaEventDestroy(evs[e]);
        cudaEventDestroy(evs[e + 1]);
    }
    fg_sweep_stats tot{};
    int errs = 0;
    for (int i = 0; i < n; i++) {
        fg_sweep_stats st{};
        st.trials = s[i].cursor;
        st.accepted = s[i].n_accepted - s0[i].n_accepted;
        st.rebuilds = s[i].n_rebuilds - s0[i].n_rebuilds;
        st.energy_change = df_val(s[i].u_hi, s[i].u_lo);
        st.device_ms = ms;
        st.sweep_kernel_ms = sweep_ms;
        st.sweep_launches = launches;
        st.error_flags = s[i].error;
        st.kernel_launches = kernels;
        errs |= s[i].error;
        if (per) per[i] = st;
        tot.trials += st.trials;
        tot.accepted += st.accepted;
        tot.rebuilds += st.rebuilds;
        tot.energy_change += st.energy_change;
    }
    tot.device_ms = ms;
    tot.sweep_kernel_ms = sweep_ms;
    tot.sweep_launches = launches;
    tot.error_flags = errs;
    tot.kernel_launches = kernels;
    if (total) *total = tot;
    for (fg_system *h : b->sys) h->cnt_accepted_host = 0;
    if (errs) return fail(FG_ERR_DEVICE, "device error flags 0x%x in a batch member", errs);
    return FG_OK;
}

void batch_free(fg_batch *b) {
    void *ptrs[] = {b->d_descs, b->d_gather, b->d_corr, b->d_counts, b->d_perm, b->d_temps, b->d_round, b->d_att,
                    b->d_acc, b->d_given};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->run_graph) cudaGraphExecDestroy(b->run_graph);
    b->dh.release();
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
}

}  // namespace

extern "C" {

int fg_batch_create(fg_system *const *systems, int32_t n, fg_batch **out) {
    if (!systems || !out || n < 1) return fail(FG_ERR_INVALID, "bad argument");
    *out = nullptr;
    for (int i = 0; i < n; i++) {
        if (!systems[i]) return fail(FG_ERR_INVALID, "null system %d", i);
        if (!systems[i]->state_set) return fail(FG_ERR_STATE, "system %d has no state", i);
        if (systems[i]->trial_pending) return fail(FG_ERR_STATE, "system %d has a pending trial", i);
        CK(cudaStreamSynchronize(systems[i]->stream));
    }
    fg_batch *b = new fg_batch();
    b->sys.assign(systems, systems + n);
    auto bail = [&](int code) {
        batch_free(b);
        delete b;
        return code;
    };
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(FG_ERR_CUDA, "stream create failed"));
    cudaEventCreate(&b->ev0);
    cudaEventCreate(&b->ev1);
    if (cudaMalloc(&b->d_descs, n * sizeof(SysDesc)) != cudaSuccess ||
        cudaMalloc(&b->d_gather, n * sizeof(SysScalars)) != cudaSuccess ||
        cudaMalloc(&b->d_corr, n * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&b->d_counts, n * sizeof(int64_t)) != cudaSuccess)
        return bail(fail(FG_ERR_CUDA, "batch allocation failed"));
    int rc = batch_config(b);
    if (rc) return bail(rc);
    for (fg_system *h : b->sys) h->batches++;
    b->counted = true;
    *out = b;
    return FG_OK;
}

int fg_batch_destroy(fg_batch *b) {
    if (!b) return FG_OK;
    cudaStreamSynchronize(b->stream);
    if (b->counted)
        for (fg_system *h : b->sys) h->batches--;
    batch_free(b);
    delete b;
    return FG_OK;
}

int fg_batch_set_threads(fg_batch *b, int32_t threads) {
    if (!b || threads < 0 || threads > fg::kSweepThreads || threads % 32)
        return fail(FG_ERR_INVALID, "threads must be a multiple of 32 in [0, %d]", fg::kSweepThreads);
    b->threads = threads;
    return batch_config(b);
}

int fg_batch_stream_philox(fg_batch *b, const int64_t *counts, uint32_t seed, const uint32_t *stream_ids) {
    if (!b || !counts) return fail(FG_ERR_INVALID, "bad argument");
    const int n = (int)b->sys.size();
    int64_t maxc = 0;
    for (int s = 0; s < n; s++) {
        if (counts[s] < 0) return fail(FG_ERR_INVALID, "negative trial count");
        fg_system *h = b->sys[s];
        int rc = ensure_trials(h, counts[s], false);
        if (rc) return rc;
        h->n_trials = counts[s];
        h->desc.seed = seed;
        h->desc.stream_id = stream_ids ? stream_ids[s] : (uint32_t)s;
        h->desc.stream_first = 0;
        maxc = std::max(maxc, counts[s]);
    }
    int rc = batch_push_descs(b);
    if (rc) return rc;
    CK(cudaMemcpyAsync(b->d_counts, counts, n * sizeof(int64_t), cudaMemcpyHostToDevice, b->stream));
    if (maxc > 0) {
        dim3 g((unsigned)std::min<int64_t>((maxc + 255) / 256, 64), n);
        fg::batch_philox_kernel<<<g, 256, 0, b->stream>>>(b->d_descs, b->d_counts, nullptr);
        CK(cudaGetLastError());
    }
    CK(cudaStreamSynchronize(b->stream));
    return FG_OK;
}

int fg_batch_stream_upload(fg_batch *b, int32_t member, int64_t n, const int32_t *idx, const double *disp,
                           const double *u) {
    if (!b || member < 0 || member >= (int)b->sys.size()) return fail(FG_ERR_INVALID, "bad member");
    return fg_stream_upload(b->sys[member], n, idx, disp, u);
}

int fg_batch_run(fg_batch *b, fg_sweep_stats *per_system, fg_sweep_stats *total) {
    if (!b) return fail(FG_ERR_INVALID, "null batch");
    const int n = (int)b->sys.size();
    std::vector<int64_t> counts(n);
    for (int s = 0; s < n; s++) {
        fg_system *h = b->sys[s];
        counts[s] = h->n_trials;
        h->log_n = 0;
        if (h->log_batch && !b->pt) {
            int rc = ensure_trials(h, counts[s], true);
            if (rc) return rc;
        }
    }
    int rc = batch_push_descs(b);
    if (rc) return rc;
    CK(cudaMemcpyAsync(b->d_counts, counts.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice, b->stream));
    rc = batch_run(b, counts, per_system, total);
    for (int s = 0; s < n; s++)
        if (b->sys[s]->desc.log_trials) b->sys[s]->log_n = counts[s];
    return rc;
}

int fg_batch_set_rebuild_mode(fg_batch *b, int32_t mode) {
    if (!b || mode < 0 || mode > 2) return fail(FG_ERR_INVALID, "mode must be 0, 1 or 2");
    b->rebuild_mode = mode;
    return batch_config(b);
}

int fg_batch_set_log(fg_batch *b, int32_t member, int32_t on) {
    if (!b || member < 0 || member >= (int)b->sys.size()) return fail(FG_ERR_INVALID, "bad member");
    b->sys[member]->log_batch = on != 0;
    return FG_OK;
}

// ---------------------------------------------------------------- parallel tempering
int fg_pt_setup(fg_batch *b, const double *temperatures, uint32_t seed) {
    if (!b || !temperatures) return fail(FG_ERR_INVALID, "bad argument");
    const int n = (int)b->sys.size();
    for (int i = 0; i < n; i++)
        if (!(temperatures[i] > 0)) return fail(FG_ERR_INVALID, "temperatures must be positive");
    if (!b->d_perm) {
        CK(cudaMalloc(&b->d_perm, n * sizeof(int)));
        CK(cudaMalloc(&b->d_temps, n * sizeof(double)));
        CK(cudaMalloc(&b->d_round, sizeof(int64_t)));
        CK(cudaMalloc(&b->d_att, n * sizeof(long long)));
        CK(cudaMalloc(&b->d_acc, n * sizeof(long long)));
        CK(cudaMalloc(&b->d_given, (2 + n) * sizeof(double)));
    }
    std::vector<int> perm(n);
    for (int i = 0; i < n; i++) {
        perm[i] = i;
        b->sys[i]->desc.kT = (float)temperatures[i];
    }
    int64_t zero = 0;
    CK(cudaMemcpyAsync(b->d_perm, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemcpyAsync(b->d_temps, temperatures, n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemcpyAsync(b->d_round, &zero, sizeof(int64_t), cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemsetAsync(b->d_att, 0, n * sizeof(long long), b->stream));
    CK(cudaMemsetAsync(b->d_acc, 0, n * sizeof(long long), b->stream));
    b->pt_seed = seed;
    b->pt = true;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->graph_sweeps = -1;
    for (int s = 0; s < n; s++) {
        fg_system *h = b->sys[s];
        h->desc.seed = seed;
        h->desc.stream_id = (uint32_t)s;
        h->desc.stream_first = 0;
    }
    return FG_OK;
}

// `rounds` rounds of: sweeps_per_round sweeps on every replica (N_s trials
// per sweep, device-generated Philox streams), then one exchange attempt per
// neighbour pair. Captured once as a CUDA graph and replayed per round.
int fg_pt_run(fg_batch *b, int32_t rounds, int32_t sweeps_per_round, fg_sweep_stats *total) {
    if (!b || !b->pt) return fail(FG_ERR_STATE, "fg_pt_setup first");
    if (rounds < 0 || sweeps_per_round < 1) return fail(FG_ERR_INVALID, "bad rounds/sweeps");
    if (b->rebuilds) return fail(FG_ERR_INVALID, "parallel tempering supports systems without Q(k) rebuilds");
    const int n = (int)b->sys.size();
    std::vector<int64_t> counts(n);
    for (int s = 0; s < n; s++) {
        counts[s] = (int64_t)sweeps_per_round * b->sys[s]->N;
        int rc = ensure_trials(b->sys[s], counts[s], false);
        if (rc) return rc;
        b->sys[s]->n_trials = counts[s];
    }
    // kT lives in the device descriptors (the swap kernel edits it): push the
    // host copies only when (re)building the graph
    if (!b->graph || b->graph_sweeps != sweeps_per_round) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        std::vector<int> perm(n);
        CK(cudaMemcpyAsync(perm.data(), b->d_perm, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
        std::vector<double> temps(n);
        CK(cudaMemcpyAsync(temps.data(), b->d_temps, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
        CK(cudaStreamSynchronize(b->stream));
        for (int i = 0; i < n; i++) b->sys[perm[i]]->desc.kT = (float)temps[i];
        int rc = batch_push_descs(b);
        if (rc) return rc;
        CK(cudaMemcpyAsync(b->d_counts, counts.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice, b->stream));
        CK(cudaStreamSynchronize(b->stream));
        int64_t maxc = 0;
        for (auto c : counts) maxc = std::max(maxc, c);
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        dim3 pg((unsigned)std::min<int64_t>((maxc + 255) / 256, 64), n);
        fg::batch_philox_kernel<<<pg, 256, 0, b->stream>>>(b->d_descs, b->d_counts, b->d_round);
        fg::batch_reset_kernel<<<(n + 127) / 128, 128, 0, b->stream>>>(b->d_descs, n, b->d_counts);
        {
            const int rc_ = batch_sweep(b, INT64_MAX);
            if (rc_) {
                cudaGraph_t gg;
                cudaStreamEndCapture(b->stream, &gg);
                if (gg) cudaGraphDestroy(gg);
                return rc_;
            }
        }
        fg::pt_swap_kernel<<<1, 32, 0, b->stream>>>(b->d_descs, n, b->d_perm, b->d_temps, b->pt_seed, b->d_round,
                                                    b->d_att, b->d_acc, nullptr, nullptr);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess) return fail(FG_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(FG_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
        b->graph_sweeps = sweeps_per_round;
    }
    const int nth = n;
    std::vector<SysScalars> s0(nth), s(nth);
    fg::gather_scalars_kernel<<<(n + 127) / 128, 128, 0, b->stream>>>(b->d_descs, n, b->d_gather);
    CK(cudaMemcpyAsync(s0.data(), b->d_gather, n * sizeof(SysScalars), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaEventRecord(b->ev0, b->stream));
    for (int r = 0; r < rounds; r++) CK(cudaGraphLaunch(b->graph, b->stream));
    CK(cudaEventRecord(b->ev1, b->stream));
    CK(cudaEventSynchronize(b->ev1));
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    fg::gather_scalars_kernel<<<(n + 127) / 128, 128, 0, b->stream>>>(b->d_descs, n, b->d_gather);
    CK(cudaMemcpyAsync(s.data(), b->d_gather, n * sizeof(SysScalars), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    fg_sweep_stats tot{};
    int errs = 0;
    for (int i = 0; i < n; i++) {
        tot.trials += (int64_t)rounds * counts[i];
        tot.accepted += s[i].n_accepted - s0[i].n_accepted;
        errs |= s[i].error;
    }
    tot.device_ms = ms;
    tot.sweep_kernel_ms = ms;
    tot.sweep_launches = rounds;
    tot.error_flags = errs;
    tot.kernel_launches = 4 * (int64_t)rounds + 2;   // philox, reset, sweep, swap per round
    if (total) *total = tot;
    if (errs) return fail(FG_ERR_DEVICE, "device error flags 0x%x", errs);
    return FG_OK;
}

// One exchange attempt with caller-given randoms (and energies): the same
// kernel as the captured rounds, run once; the host copies of the systems'
// temperatures follow the new permutation, so that later fg_batch_run calls
// (which push the host descriptors) keep them.
int fg_pt_swap(fg_batch *b, double u_direction, double u_accept, const double *energies, int32_t *exchanged) {
    if (!b || !b->pt) return fail(FG_ERR_STATE, "fg_pt_setup first");
    if (!(u_direction >= 0.0 && u_direction <= 1.0) || !(u_accept >= 0.0 && u_accept <= 1.0))
        return fail(FG_ERR_INVALID, "uniforms must lie in [0, 1]");
    const int n = (int)b->sys.size();
    std::vector<double> g(2 + n, 0.0);
    g[0] = u_direction;
    g[1] = u_accept;
    if (energies)
        for (int i = 0; i < n; i++) {
            if (!std::isfinite(energies[i])) return fail(FG_ERR_INVALID, "non-finite energy of system %d", i);
            g[2 + i] = energies[i];
        }
    std::vector<int> before(n), after(n);
    CK(cudaMemcpyAsync(before.data(), b->d_perm, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaMemcpyAsync(b->d_given, g.data(), g.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    fg::pt_swap_kernel<<<1, 32, 0, b->stream>>>(b->d_descs, n, b->d_perm, b->d_temps, b->pt_seed, b->d_round,
                                                b->d_att, b->d_acc, b->d_given, energies ? b->d_given + 2 : nullptr);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(after.data(), b->d_perm, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    std::vector<double> temps(n);
    CK(cudaMemcpyAsync(temps.data(), b->d_temps, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    for (int i = 0; i < n; i++) {
        b->sys[after[i]]->desc.kT = (float)temps[i];
        if (exchanged) exchanged[i] = before[i] != after[i] ? 1 : 0;
    }
    return FG_OK;
}

// perm[rung] = system index; energies[system] = running total energy;
// attempts/accepts[rung] count exchanges between rung and rung+1 (or NULL).
int fg_pt_get(fg_batch *b, int32_t *perm, double *energies, int64_t *attempts, int64_t *accepts) {
    if (!b || !b->pt) return fail(FG_ERR_STATE, "fg_pt_setup first");
    const int n = (int)b->sys.size();
    if (perm) CK(cudaMemcpyAsync(perm, b->d_perm, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    if (attempts) CK(cudaMemcpyAsync(attempts, b->d_att, n * sizeof(long long), cudaMemcpyDeviceToHost, b->stream));
    if (accepts) CK(cudaMemcpyAsync(accepts, b->d_acc, n * sizeof(long long), cudaMemcpyDeviceToHost, b->stream));
    std::vector<SysScalars> s(n);
    fg::gather_scalars_kernel<<<(n + 127) / 128, 128, 0, b->stream>>>(b->d_descs, n, b->d_gather);
    CK(cudaMemcpyAsync(s.data(), b->d_gather, n * sizeof(SysScalars), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    if (energies)
        for (int i = 0; i < n; i++) energies[i] = df_val(s[i].utot_hi, s[i].utot_lo);
    return FG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- job server
struct fg_job {
    int64_t id;
    fg_params P;
    std::vector<double> xyz, q;
    std::vector<int32_t> ids;
    uint32_t seed;
    int64_t n_trials, done = 0, accepted = 0;
    int state = 0;   // 0 queued, 1 running, 2 done, 3 failed
    fg_system *sys = nullptr;
    std::vector<double> result;   // final coordinates, copied off the device
    std::vector<unsigned char> snapshot;   // resumed job: its system's state (fg_server_resume)
    size_t bytes = 0;
    double energy = 0;
};

struct fg_server {
    int64_t max_bytes;
    int threads;
    int64_t round_pairs;
    int64_t used = 0, next_id = 1;
    std::vector<fg_job *> jobs;   // all jobs not yet released
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;            // second kernel variant of a round
    cudaEvent_t fork = nullptr, join = nullptr;
    DhGroups dh;                               // block-kernel jobs of the current round
    SysDesc *d_descs = nullptr;
    SysScalars *d_gather = nullptr;
    int64_t *d_counts = nullptr;
    int cap = 0;
    std::string err;
};

namespace {

// Device bytes of one job as fg_create allocates them for a Debye-Hueckel
// system (coordinates, records, types, descriptor, scalars, tables) plus its
// per-round trial stream; Ewald systems add their k-space arrays.
size_t job_bytes(const fg_params &P, int N, int64_t round_trials) {
    size_t b = (size_t)N * (24 + 16 + 8 + 1) + sizeof(SysDesc) + sizeof(SysScalars) + 64 + 32 + 32 + 256 * 8 +
               FG_MAX_TYPES * 3 * 8 + 1024 * 8;
    double smax = 0;
    for (int i = 0; i < P.n_types; i++) smax = std::max(smax, P.type_sigma[i]);
    if (P.model == FG_MODEL_DH_LJ) b += 2 * 16 * (size_t)(std::ceil(smax / P.dh_debye_length * 128.0) + 4);
    if (P.model == FG_MODEL_EWALD_WCA) {
        const double kc = std::ceil(P.ewald_cutoff_k);
        b += (size_t)(4.2 * kc * kc * kc + 16) * (16 + 4 + 16 + 16) + 2 * 16 * (size_t)(P.ewald_alpha * smax * 128 + 4);
    }
    b += (size_t)std::max<int64_t>(round_trials, 1) * sizeof(Trial);
    return b;
}

// Trials of one round: about round_pairs pair evaluations for every job, so
// a round takes about as long for a small job as for a large one (at least 32
// trials, at most 2^20).
int64_t round_trials_for(const fg_server *s, int64_t N) {
    int64_t t = std::max<int64_t>(32, s->round_pairs / std::max<int64_t>(N, 1));
    return std::min<int64_t>(t, 1 << 20);
}
int64_t round_trials_of(const fg_server *s, const fg_job *j) {
    const int64_t N = j->sys ? j->sys->N : (int64_t)j->ids.size();
    return std::min<int64_t>(round_trials_for(s, N), j->n_trials - j->done);
}
// Block-kernel jobs on C CTAs do C times the work of a round.
int64_t round_trials_dh(const fg_server *s, int64_t N, int C, int64_t remaining) {
    int64_t t = std::max<int64_t>(32, (int64_t)C * s->round_pairs / std::max<int64_t>(N, 1));
    return std::min<int64_t>(std::min<int64_t>(t, 1 << 20), remaining);
}

int server_grow(fg_server *s, int n) {
    if (n <= s->cap) return FG_OK;
    int cap = std::max(n, 2 * s->cap);
    if (s->d_descs) cudaFree(s->d_descs);
    if (s->d_gather) cudaFree(s->d_gather);
    if (s->d_counts) cudaFree(s->d_counts);
    CK(cudaMalloc(&s->d_descs, cap * sizeof(SysDesc)));
    CK(cudaMalloc(&s->d_gather, cap * sizeof(SysScalars)));
    CK(cudaMalloc(&s->d_counts, cap * sizeof(int64_t)));
    s->cap = cap;
    return FG_OK;
}

int server_admit(fg_server *s, fg_job *j) {
    const int64_t Nj = (int64_t)j->ids.size();
    const bool blk = j->P.model == FG_MODEL_DH_LJ && !j->P.use_cell_list;
    const int64_t rt = blk ? round_trials_dh(s, Nj, dh_block_ctas_cap((int)Nj, tuned_min_per_cta()), j->n_trials)
                           : std::min<int64_t>(j->n_trials, round_trials_for(s, Nj));
    j->bytes = job_bytes(j->P, (int)j->ids.size(), rt);
    if (s->used + (int64_t)j->bytes > s->max_bytes) return 1;   // does not fit now
    fg_system *h = nullptr;
    int rc = fg_create(&j->P, (int)j->ids.size(), &h);
    if (rc) return rc;
    if (s->threads) fg_set_threads(h, s->threads);
    rc = j->snapshot.empty()
             ? fg_set_state(h, j->xyz.data(), j->q.empty() ? nullptr : j->q.data(), j->ids.data())
             : fg_restore(h, j->snapshot.data(), (int64_t)j->snapshot.size());
    if (rc) {
        fg_destroy(h);
        return rc;
    }
    j->snapshot.clear();
    j->snapshot.shrink_to_fit();
    // a job's stream depends on its seed only (Philox key (seed, 0)), so its
    // result does not depend on which other jobs share the GPU
    h->desc.seed = j->seed;
    h->desc.stream_id = 0;
    j->sys = h;
    j->state = 1;
    j->bytes = h->device_bytes + (size_t)std::min<int64_t>(rt, 1 << 20) * sizeof(Trial);
    s->used += (int64_t)j->bytes;
    return FG_OK;
}

}  // namespace

extern "C" {

int fg_server_create(int64_t max_device_bytes, int32_t threads, int64_t round_pairs, fg_server **out) {
    if (!out || max_device_bytes <= 0 || threads < 0 || threads > fg::kSweepThreads || threads % 32)
        return fail(FG_ERR_INVALID, "bad argument");
    fg_server *s = new fg_server();
    s->max_bytes = max_device_bytes;
    s->threads = threads;
    s->round_pairs = round_pairs > 0 ? round_pairs : ((int64_t)1 << 28);
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return fail(FG_ERR_CUDA, "stream create failed");
    }
    *out = s;
    return FG_OK;
}

int fg_server_destroy(fg_server *s) {
    if (!s) return FG_OK;
    cudaStreamSynchronize(s->stream);
    for (fg_job *j : s->jobs) {
        if (j->sys) fg_destroy(j->sys);
        delete j;
    }
    if (s->d_descs) cudaFree(s->d_descs);
    if (s->d_gather) cudaFree(s->d_gather);
    if (s->d_counts) cudaFree(s->d_counts);
    s->dh.release();
    if (s->stream2) {
        cudaStreamSynchronize(s->stream2);
        cudaStreamDestroy(s->stream2);
        cudaEventDestroy(s->fork);
        cudaEventDestroy(s->join);
    }
    cudaStreamDestroy(s->stream);
    delete s;
    return FG_OK;
}

// Queue a job: a system (params, coordinates, charges or NULL, types), its
// Philox seed and the number of trials to run.
int fg_server_submit(fg_server *s, const fg_params *params, int32_t n, const double *xyz, const double *charge,
                     const int32_t *type_ids, uint32_t seed, int64_t n_trials, int64_t *job_id) {
    if (!s || !params || !xyz || !type_ids || !job_id || n < 2 || n_trials < 0) return fail(FG_ERR_INVALID, "bad argument");
    if (params->model != FG_MODEL_DH_LJ && params->model != FG_MODEL_EWALD_WCA)
        return fail(FG_ERR_INVALID, "unsupported model");
    for (fg_job *o : s->jobs)
        if (o->P.model != params->model) return fail(FG_ERR_INVALID, "one model per server");
    const bool blk = params->model == FG_MODEL_DH_LJ && !params->use_cell_list;
    const int64_t rt = blk ? round_trials_dh(s, n, dh_block_ctas_cap(n, tuned_min_per_cta()), n_trials)
                           : std::min<int64_t>(n_trials, round_trials_for(s, n));
    if ((int64_t)job_bytes(*params, n, rt) > s->max_bytes) return fail(FG_ERR_CAPACITY, "job larger than the budget");
    fg_job *j = new fg_job();
    j->id = s->next_id++;
    j->P = *params;
    j->xyz.assign(xyz, xyz + 3 * (size_t)n);
    if (charge) j->q.assign(charge, charge + n);
    j->ids.assign(type_ids, type_ids + n);
    j->seed = seed;
    j->n_trials = n_trials;
    s->jobs.push_back(j);
    *job_id = j->id;
    return FG_OK;
}

// One round: admit queued jobs that fit the memory budget (in submission
// order), give every running job its next chunk of trials (about
// round_pairs / N trials) and run them all in one launch
// of the persistent sweep kernel, then retire finished jobs.
int fg_server_step(fg_server *s, int32_t *n_running, int32_t *n_finished, double *device_ms) {
    if (!s) return fail(FG_ERR_INVALID, "null server");
    for (fg_job *j : s->jobs)
        if (j->state == 0) {
            int rc = server_admit(s, j);
            if (rc == 1) break;   // keep submission order: wait for memory
            if (rc) {
                j->state = 3;
                continue;
            }
        }
    std::vector<fg_job *> run;
    for (fg_job *j : s->jobs)
        if (j->state == 1) run.push_back(j);
    if (n_running) *n_running = (int)run.size();
    if (n_finished) *n_finished = 0;
    if (device_ms) *device_ms = 0;
    if (run.empty()) return FG_OK;
    // jobs of one kernel variant run in one launch; variants run side by side
    // on their own streams (sizes that fit shared memory and those that do not)
    // classic-kernel jobs first (grouped by variant), then the block-kernel
    // (Debye-Hueckel, all-pairs) jobs as one contiguous range
    std::stable_sort(run.begin(), run.end(), [](const fg_job *a, const fg_job *b) {
        const bool ba = dh_block_ok(a->sys), bb = dh_block_ok(b->sys);
        if (ba != bb) return bb;
        return (const void *)sweep_fn(a->sys) < (const void *)sweep_fn(b->sys);
    });
    const int n = (int)run.size();
    int rc = server_grow(s, n);
    if (rc) return rc;
    std::vector<SysDesc> descs(n);
    std::vector<int64_t> counts(n);
    struct Group {
        SweepFn fn;
        int first, count, threads;
        size_t smem;
    };
    std::vector<Group> groups;
    int first_dh = -1;
    std::vector<int> dh_n, dh_c;
    std::vector<double> dh_w;
    // block-kernel jobs: CTAs in proportion to the work each has left, so the
    // largest jobs get the most SMs; a job on C CTAs runs C rounds of work
    for (int i = 0; i < n; i++)
        if (dh_block_ok(run[i]->sys)) {
            dh_n.push_back(run[i]->sys->N);
            dh_w.push_back((double)(run[i]->n_trials - run[i]->done) * run[i]->sys->N);
        }
    if (!dh_n.empty()) dh_c = dh_block_ctas_many(dh_n, dh_w, tuned_min_per_cta());
    int k_dh = 0;
    for (int i = 0; i < n; i++) {
        fg_job *j = run[i];
        fg_system *h = j->sys;
        counts[i] = dh_block_ok(h) ? round_trials_dh(s, h->N, std::min(dh_c[k_dh++], dh_block_ctas_cap(h->N, tuned_min_per_cta())),
                                                     j->n_trials - j->done)
                                   : round_trials_of(s, j);
        rc = ensure_trials(h, counts[i], false);
        if (rc) return rc;
        h->n_trials = counts[i];
        h->desc.trials = h->trials;
        h->desc.log_trials = 0;
        h->desc.skip_rebuild = 1;
        h->desc.rebuild_in_kernel = 0;
        h->desc.stream_first = j->done;
        descs[i] = h->desc;
        if (dh_block_ok(h)) {
            if (first_dh < 0) first_dh = i;
            continue;
        }
        const SweepFn fn = sweep_fn(h);
        if (groups.empty() || groups.back().fn != fn) groups.push_back(Group{fn, i, 0, s->threads, 0});
        Group &g = groups.back();
        g.count++;
        g.smem = std::max(g.smem, sweep_launch_smem(h));
        if (!s->threads || ewald_block_ok(h)) g.threads = std::max(g.threads, sweep_launch_threads(h));
    }
    for (Group &g : groups) {
        rc = set_smem_attr((const void *)g.fn, g.smem);
        if (rc) return rc;
    }
    if (groups.size() > 1 && !s->stream2) {
        if (cudaStreamCreateWithFlags(&s->stream2, cudaStreamNonBlocking) != cudaSuccess)
            return fail(FG_ERR_CUDA, "stream create failed");
        cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming);
    }
    CK(cudaMemcpyAsync(s->d_descs, descs.data(), n * sizeof(SysDesc), cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->d_counts, counts.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice, s->stream));
    int64_t maxc = 0;
    for (auto c : counts) maxc = std::max(maxc, c);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    CK(cudaEventRecord(e0, s->stream));
    dim3 pg((unsigned)std::min<int64_t>((maxc + 255) / 256, 64), n);
    fg::batch_philox_kernel<<<pg, 256, 0, s->stream>>>(s->d_descs, s->d_counts, nullptr);
    fg::batch_reset_kernel<<<(n + 127) / 128, 128, 0, s->stream>>>(s->d_descs, n, s->d_counts);
    for (size_t g = 0; g < groups.size(); g++) {
        const Group &G = groups[g];
        cudaStream_t st = s->stream;
        if (g > 0) {
            CK(cudaEventRecord(s->fork, s->stream));
            CK(cudaStreamWaitEvent(s->stream2, s->fork, 0));
            st = s->stream2;
        }
        G.fn<<<G.count, G.threads, G.smem, st>>>(s->d_descs + G.first, INT64_MAX, run[G.first]->sys->sc_tab);
        CK(cudaGetLastError());
    }
    if (groups.size() > 1) {
        CK(cudaEventRecord(s->join, s->stream2));
        CK(cudaStreamWaitEvent(s->stream, s->join, 0));
    }
    if (first_dh >= 0) {
        for (size_t k = 0; k < dh_c.size(); k++) dh_c[k] = std::min(dh_c[k], dh_block_ctas_cap(dh_n[k], tuned_min_per_cta()));
        rc = dh_groups_build_c(s->dh, dh_n, dh_c);
        if (rc) return rc;
        rc = dh_groups_launch(s->dh, s->d_descs + first_dh, INT64_MAX, s->stream);
        if (rc) return rc;
    }
    CK(cudaEventRecord(e1, s->stream));
    std::vector<SysScalars> sc(n);
    fg::gather_scalars_kernel<<<(n + 127) / 128, 128, 0, s->stream>>>(s->d_descs, n, s->d_gather);
    CK(cudaMemcpyAsync(sc.data(), s->d_gather, n * sizeof(SysScalars), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (device_ms) *device_ms = ms;
    int fin = 0;
    for (int i = 0; i < n; i++) {
        fg_job *j = run[i];
        if (sc[i].error) {
            j->state = 3;
            continue;
        }
        j->done += sc[i].cursor;
        j->accepted = sc[i].n_accepted;
        j->energy = df_val(sc[i].utot_hi, sc[i].utot_lo);
        if (j->done >= j->n_trials) {
            // results to host memory; the device memory goes back to the pool
            j->result.resize(3 * (size_t)j->sys->N);
            rc = fg_get_state(j->sys, j->result.data());
            if (rc) return rc;
            s->used -= (int64_t)j->bytes;
            fg_destroy(j->sys);
            j->sys = nullptr;
            j->state = 2;
            fin++;
        }
    }
    if (n_finished) *n_finished = fin;
    return FG_OK;
}

// state: 0 queued, 1 running, 2 done, 3 failed; trials done, accepted,
// running total energy; positions (3N, may be NULL) once done.
int fg_server_poll(fg_server *s, int64_t job_id, int32_t *state, int64_t *trials_done, int64_t *accepted,
                   double *energy, double *xyz) {
    if (!s) return fail(FG_ERR_INVALID, "null server");
    for (fg_job *j : s->jobs)
        if (j->id == job_id) {
            if (state) *state = j->state;
            if (trials_done) *trials_done = j->done;
            if (accepted) *accepted = j->accepted;
            if (energy) *energy = j->energy;
            if (xyz && j->state == 2) std::copy(j->result.begin(), j->result.end(), xyz);
            return FG_OK;
        }
    return fail(FG_ERR_INVALID, "unknown job %lld", (long long)job_id);
}

// Free a finished (or failed) job and its device memory.
int fg_server_release(fg_server *s, int64_t job_id) {
    if (!s) return fail(FG_ERR_INVALID, "null server");
    for (size_t k = 0; k < s->jobs.size(); k++) {
        fg_job *j = s->jobs[k];
        if (j->id != job_id) continue;
        if (j->state == 1) return fail(FG_ERR_STATE, "job %lld is running", (long long)job_id);
        delete j;
        s->jobs.erase(s->jobs.begin() + k);
        return FG_OK;
    }
    return fail(FG_ERR_INVALID, "unknown job %lld", (long long)job_id);
}

int fg_server_cancel(fg_server *s, int64_t job_id) {
    if (!s) return fail(FG_ERR_INVALID, "null server");
    for (size_t k = 0; k < s->jobs.size(); k++) {
        fg_job *j = s->jobs[k];
        if (j->id != job_id) continue;
        // rounds end synchronised (fg_server_step), so no kernel of this job
        // is in flight here; wait for both streams all the same
        CK(cudaStreamSynchronize(s->stream));
        if (s->stream2) CK(cudaStreamSynchronize(s->stream2));
        if (j->sys) {
            s->used -= (int64_t)j->bytes;
            fg_destroy(j->sys);
            j->sys = nullptr;
        }
        delete j;
        s->jobs.erase(s->jobs.begin() + k);
        return FG_OK;
    }
    return fail(FG_ERR_INVALID, "unknown job %lld", (long long)job_id);
}

int64_t fg_server_bytes_in_use(fg_server *s) { return s ? s->used : 0; }

}  // extern "C"
