// Launch-shape autotuner (included by fg_api.cu after the batch and molecule
// code). Each entry point times candidate launch shapes on the device, on a
// clone of the caller's system(s) so the caller's Markov chains do not
// advance, keeps the fastest, applies it, and records it process-wide:
//
//   fg_autotune        DH+LJ block sweeps: CTAs per system (cluster size);
//                      Ewald one-trial sweeps: threads per CTA. (The Ewald
//                      block kernel has one fixed shape: nothing to tune.)
//   fg_batch_autotune  the batch schedule: least particles per CTA when the
//                      SMs are shared out among members (also used by the
//                      job server and batches created afterwards), timed on
//                      equal sweeps of every member
//   fg_mol_autotune    rigid molecules: CTAs per system (cluster size)
//
// Timing: each candidate runs a warm-up stream, then a timed stream of
// n_trials device-generated (Philox) trials; the figure is device time per
// trial from the sweep's CUDA events. The shape changes only the order of
// the floating-point sums, never the trial sequence or the decisions beyond
// the stated tolerance.
namespace {

constexpr int kTuneMax = 8;

void report_add(fg_tune_report *r, int value, double us) {
    if (!r || r->n >= kTuneMax) return;
    r->value[r->n] = value;
    r->us_per_trial[r->n] = us;
    r->n++;
}

int report_pick(fg_tune_report *r, const std::vector<std::pair<int, double>> &t) {
    int best = -1;
    for (size_t i = 0; i < t.size(); i++)
        if (best < 0 || t[i].second < t[best].second) best = (int)i;
    if (r) r->chosen = best;
    return best;
}

// A new system with the same parameters and the current state of h.
int clone_system(fg_system *h, fg_system **out) {
    if (h->types.empty()) return fail(FG_ERR_STATE, "fg_set_state first");
    std::vector<double> xyz(3 * (size_t)h->N);
    int rc = fg_get_state(h, xyz.data());
    if (rc) return rc;
    fg_system *c = nullptr;
    rc = fg_create(&h->P, h->N, &c);
    if (rc) return rc;
    rc = fg_set_state(c, xyz.data(), h->charges.data(), h->types.data());
    if (!rc) rc = fg_set_rebuild_policy(c, h->desc.skip_rebuild);
    if (rc) {
        fg_destroy(c);
        return rc;
    }
    c->threads = h->threads;
    *out = c;
    return FG_OK;
}

// Device microseconds per trial of a warm-up plus a timed Philox stream.
int time_system(fg_system *c, int64_t n, uint32_t seed, double *us) {
    fg_sweep_stats st{};
    int rc = fg_stream_philox(c, std::max<int64_t>(32, n / 4), seed, 0);
    if (!rc) rc = fg_stream_run(c, &st);
    if (!rc) rc = fg_stream_philox(c, n, seed + 1, 0);
    if (!rc) rc = fg_stream_run(c, &st);
    if (rc) return rc;
    *us = st.trials > 0 ? st.device_ms * 1e3 / (double)st.trials : 0.0;
    return FG_OK;
}

}  // namespace

extern "C" {

int fg_autotune(fg_system *h, int64_t n_trials, fg_tune_report *report) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (n_trials < 32) return fail(FG_ERR_INVALID, "n_trials must be >= 32");
    if (report) *report = fg_tune_report{};
    const bool dh = dh_block_ok(h);
    const bool eb = !dh && h->model == FG_MODEL_EWALD_WCA && h->K > 0 && ewald_block_ok(h);
    std::vector<int> cand;
    if (dh) {
        for (int C = 1; C <= dh_block_max_cluster(); C *= 2)
            if (C == 1 || h->N / C >= 64) cand.push_back(C);
    } else if (eb) {
        for (int C = 1; C <= eb_cluster_max(h); C *= 2) cand.push_back(C);
    } else {
        for (int T = 128; T <= fg::kSweepThreads; T *= 2) cand.push_back(T);
    }
    fg_system *c = nullptr;
    int rc = clone_system(h, &c);
    if (rc) return rc;
    std::vector<std::pair<int, double>> t;
    for (int v : cand) {
        if (dh) c->ctas = v;
        else if (eb) c->eb_ctas = v;
        else c->threads = v;
        double us = 0;
        rc = time_system(c, n_trials, 0x7e57u + (uint32_t)v, &us);
        if (rc) break;
        t.emplace_back(v, us);
        report_add(report, v, us);
    }
    fg_destroy(c);
    if (rc) return rc;
    const int best = report_pick(report, t);
    if (best < 0) return FG_OK;
    if (dh) {
        h->ctas = t[best].first;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_dh_ctas[size_class(h->N)] = t[best].first;
    } else if (eb) {
        h->eb_ctas = t[best].first;
    } else {
        h->threads = t[best].first;
    }
    return FG_OK;
}

int fg_batch_autotune(fg_batch *b, int64_t n_trials, fg_tune_report *report) {
    if (!b) return fail(FG_ERR_INVALID, "null handle");
    if (n_trials < 32) return fail(FG_ERR_INVALID, "n_trials must be >= 32");
    if (report) *report = fg_tune_report{};
    if (!b->dh_block) return FG_OK;   // one CTA per member: no schedule to choose
    const int n = (int)b->sys.size();
    std::vector<fg_system *> cl(n, nullptr);
    int rc = FG_OK;
    for (int i = 0; i < n && !rc; i++) rc = clone_system(b->sys[i], &cl[i]);
    fg_batch *tb = nullptr;
    if (!rc) rc = fg_batch_create(cl.data(), n, &tb);
    std::vector<std::pair<int, double>> t;
    // equal sweeps for every member (trials in proportion to N, as in PT
    // rounds and served jobs): n_trials for the largest member
    int maxN = 1;
    for (fg_system *h : b->sys) maxN = std::max(maxN, h->N);
    std::vector<int64_t> counts(n), warm(n);
    for (int i = 0; i < n; i++) {
        counts[i] = std::max<int64_t>(32, n_trials * b->sys[i]->N / maxN);
        warm[i] = std::max<int64_t>(32, counts[i] / 4);
    }
    for (int m = 128; m <= 2048 && !rc; m *= 2) {
        tb->min_per_cta = m;
        rc = batch_config(tb);
        fg_sweep_stats tot{};
        if (!rc) rc = fg_batch_stream_philox(tb, warm.data(), 0x7e57u + (uint32_t)m, nullptr);
        if (!rc) rc = fg_batch_run(tb, nullptr, &tot);
        if (!rc) rc = fg_batch_stream_philox(tb, counts.data(), 0x7e58u + (uint32_t)m, nullptr);
        if (!rc) rc = fg_batch_run(tb, nullptr, &tot);
        if (rc) break;
        // device time per member trial (members run side by side)
        const double us = tot.trials > 0 ? tot.device_ms * 1e3 / (double)tot.trials : 0.0;
        t.emplace_back(m, us);
        report_add(report, m, us);
    }
    if (tb) fg_batch_destroy(tb);
    for (fg_system *c : cl)
        if (c) fg_destroy(c);
    if (rc) return rc;
    const int best = report_pick(report, t);
    if (best < 0) return FG_OK;
    b->min_per_cta = t[best].first;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_min_per_cta = t[best].first;
    }
    if (b->graph) {   // a captured round holds the old launch shapes
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
        b->graph_sweeps = -1;
    }
    return batch_config(b);
}

int fg_mol_autotune(fg_molsys *h, int64_t n_trials, fg_tune_report *report) {
    if (!h) return fail(FG_ERR_INVALID, "null handle");
    if (n_trials < 32) return fail(FG_ERR_INVALID, "n_trials must be >= 32");
    if (!h->state_set) return fail(FG_ERR_STATE, "fg_mol_set_state first");
    if (report) *report = fg_tune_report{};
    std::vector<double> xyz(3 * (size_t)h->N), mu(3 * (size_t)h->N), cm(3 * (size_t)h->M);
    int rc = fg_mol_get_state(h, xyz.data(), mu.data(), cm.data());
    if (rc) return rc;
    fg_molsys *c = nullptr;
    rc = fg_mol_create(&h->P, h->N, h->gs, &c);
    if (rc) return rc;
    rc = fg_mol_set_state(c, xyz.data(), mu.data(), h->mus_h.data(), h->types.data(), cm.data());
    // one host-drawn stream (TranslateRotate with dp = 1, dprot = 0.3) for every candidate
    const int64_t n = n_trials, nw = std::max<int64_t>(32, n_trials / 4);
    std::vector<int32_t> mol(n), center(n);
    std::vector<double> axis(3 * n), angle(n), trans(3 * n), u(n);
    if (!rc)
        rc = fg_mol_draw_stream(0x7e57u, h->M, n, 1.0, 0.3, 1, mol.data(), axis.data(), center.data(), angle.data(),
                                trans.data(), u.data());
    std::vector<std::pair<int, double>> t;
    for (int C = 1; C <= h->max_cluster && !rc; C *= 2) {
        if (fg_mol_set_cluster(c, C) != FG_OK) continue;   // slices do not fit at this size
        fg_sweep_stats st{};
        rc = fg_mol_stream_upload(c, nw, mol.data(), axis.data(), angle.data(), center.data(), trans.data(),
                                  u.data(), 1, 1);
        if (!rc) rc = fg_mol_run_many(&c, 1, nullptr, &st);
        if (!rc)
            rc = fg_mol_stream_upload(c, n, mol.data(), axis.data(), angle.data(), center.data(), trans.data(),
                                      u.data(), 1, 1);
        if (!rc) rc = fg_mol_run_many(&c, 1, nullptr, &st);
        if (rc) break;
        const double us = st.trials > 0 ? st.device_ms * 1e3 / (double)st.trials : 0.0;
        t.emplace_back(C, us);
        report_add(report, C, us);
    }
    fg_mol_destroy(c);
    if (rc) return rc;
    const int best = report_pick(report, t);
    if (best < 0) return FG_OK;
    return fg_mol_set_cluster(h, t[best].first);
}

int fg_tune_reset(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_dh_ctas.clear();
    g_tune_min_per_cta = 256;
    g_tune_dip_threads = 0;
    return FG_OK;
}

}  // extern "C"
