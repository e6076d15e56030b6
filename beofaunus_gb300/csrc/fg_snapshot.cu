// Snapshots: a device -> host copy of everything that determines how a system
// continues, and the way back, so that a run can stop and resume bit for bit
// (in another process, on another GPU of the same kind).
//
// Included by fg_api.cu after fg_batch.cu (one translation unit).
//
// The reference's counterparts: Space::save/load (space.h:376-377) write and
// read the particles as text, and the random state is written to
// move_out.json (slump.h:111-124, move.h:7900) but never read back. Here the
// state is binary and complete: the 64-bit fixed-point positions (not doubles:
// a decimal or FP64 round trip could move a particle by one unit of 2^-64 L),
// charges and types, the cell lists in their slot order (the order in which
// the real-space sum visits a cell), the exact integer Q(k), the running
// energies and surface dipole as df pairs, the accept counter of the next
// update_frequency rebuild, and the Philox key and counters of the system's
// device stream. Restoring checks Q(k) against a rebuild from the restored
// positions (they must agree bit for bit) before it adopts the snapshot.
//
// Layout: SnapHeader, the host sections (type ids, charges), then the device
// sections in the order of snap_sections, each padded to 8 bytes. Byte order
// and struct layout are the host's: a snapshot is read back by this library
// on a host of the same byte order.
namespace {

constexpr char kSnapMagic[8] = {'F', 'G', 'S', 'N', 'A', 'P', '0', '1'};
constexpr int32_t kSnapVersion = 1;

struct SnapHeader {
    char magic[8];
    int32_t version;
    int32_t N, K, model;
    int32_t use_cells, cap;
    int32_t nc[3];
    int32_t qk_shift;
    float qk_scale;
    int32_t cnt_accepted_host;
    uint32_t seed, stream_id;   // Philox key of the system's device stream
    int64_t stream_first;       // counter of the last staged stream's first trial
    int64_t next_counter;       // stream_first + the trials run from it
    double self_energy;
    fg_params P;
    uint64_t payload_bytes;
    uint64_t checksum;          // FNV-1a 64 of the payload
};

struct SnapSection {
    void *dev;
    size_t bytes;
};

uint64_t fnv1a64(const unsigned char *p, size_t n) {
    uint64_t h = 1469598103934665603ULL;
    for (size_t i = 0; i < n; i++) {
        h ^= p[i];
        h *= 1099511628211ULL;
    }
    return h;
}

size_t pad8(size_t b) { return (b + 7) & ~(size_t)7; }

// Device sections of a system, in file order.
std::vector<SnapSection> snap_sections(fg_system *h) {
    const size_t N = (size_t)h->N;
    std::vector<SnapSection> s = {{h->pos64, 24 * N}, {h->pos4, 16 * N}, {h->pos_ext, sizeof(short4) * N},
                                  {h->ptype, N}, {h->sc, sizeof(SysScalars)}};
    if (h->K > 0) s.push_back({h->qfix, sizeof(longlong2) * (size_t)h->K});
    if (h->use_cells) {
        const size_t ncell = (size_t)h->nc[0] * h->nc[1] * h->nc[2], slots = ncell * (size_t)h->cap;
        s.push_back({h->cell_count, 4 * ncell});
        s.push_back({h->cell_pid, 4 * slots});
        s.push_back({h->cell_pos, 16 * slots});
        s.push_back({h->cell_ext, sizeof(short4) * slots});
        s.push_back({h->p_cell, 4 * N});
        s.push_back({h->p_slot, 4 * N});
    }
    return s;
}

// Host sections: the uploaded type ids and charges (clones, energies).
size_t snap_host_bytes(int N) { return pad8(4 * (size_t)N) + 8 * (size_t)N; }

size_t snap_bytes(fg_system *h) {
    size_t b = sizeof(SnapHeader) + snap_host_bytes(h->N);
    for (const SnapSection &s : snap_sections(h)) b += pad8(s.bytes);
    return b;
}

fg_params params_key(const fg_params &P) {
    fg_params k = P;
    std::memset(k.reserved, 0, sizeof(k.reserved));
    return k;
}

// Q(k) of the restored positions from scratch, compared with the restored
// Q(k): the rebuild kernel's verifying mode (any difference sets
// kErrQkMismatch). Leaves Q(k) unchanged when they agree.
int snap_verify_qk(fg_system *h) {
    if (h->K == 0) return FG_OK;
    SysScalars s{};
    s.rebuild_pending = 1;
    s.verify_rebuild = 1;
    int rc = write_scalars(h, s);
    if (rc) return rc;
    rc = launch_rebuild(h->d_desc, 1, h->N, h->nseg, h->kc, h->corr, h->stream);
    if (rc) return rc;
    rc = read_scalars(h, s);
    if (rc) return rc;
    if (s.error & fg::kErrQkMismatch) return fail(FG_ERR_INVALID, "snapshot Q(k) does not match its positions");
    if (s.error) return fail(FG_ERR_DEVICE, "device error flags 0x%x while verifying Q(k)", s.error);
    return FG_OK;
}

}  // namespace

extern "C" {

int64_t fg_snapshot_bytes(fg_system *h) { return h ? (int64_t)snap_bytes(h) : 0; }

int fg_snapshot(fg_system *h, void *buf, int64_t size) {
    if (!h || !buf) return fail(FG_ERR_INVALID, "null argument");
    if (!h->state_set) return fail(FG_ERR_STATE, "fg_set_state first");
    if (h->trial_pending) return fail(FG_ERR_STATE, "commit the pending trial first");
    if (size < (int64_t)snap_bytes(h)) return fail(FG_ERR_CAPACITY, "snapshot needs %zu bytes", snap_bytes(h));
    unsigned char *out = (unsigned char *)buf;
    unsigned char *p = out + sizeof(SnapHeader);
    std::memset(p, 0, snap_bytes(h) - sizeof(SnapHeader));
    std::memcpy(p, h->types.data(), 4 * (size_t)h->N);
    p += pad8(4 * (size_t)h->N);
    std::memcpy(p, h->charges.data(), 8 * (size_t)h->N);
    p += 8 * (size_t)h->N;
    const unsigned char *scp = nullptr;
    for (const SnapSection &s : snap_sections(h)) {
        if (s.dev == h->sc) scp = p;
        CK(cudaMemcpyAsync(p, s.dev, s.bytes, cudaMemcpyDeviceToHost, h->stream));
        p += pad8(s.bytes);
    }
    CK(cudaStreamSynchronize(h->stream));
    SysScalars sc;
    std::memcpy(&sc, scp, sizeof(sc));
    SnapHeader hd{};
    std::memcpy(hd.magic, kSnapMagic, 8);
    hd.version = kSnapVersion;
    hd.N = h->N;
    hd.K = h->K;
    hd.model = h->model;
    hd.use_cells = h->use_cells ? 1 : 0;
    hd.cap = h->cap;
    for (int a = 0; a < 3; a++) hd.nc[a] = h->nc[a];
    hd.qk_shift = h->desc.qk_shift;
    hd.qk_scale = h->desc.qk_scale;
    hd.cnt_accepted_host = h->cnt_accepted_host;
    hd.seed = h->desc.seed;
    hd.stream_id = h->desc.stream_id;
    hd.stream_first = h->desc.stream_first;
    hd.next_counter = h->desc.stream_first + sc.cursor;
    hd.self_energy = h->self_energy;
    hd.P = params_key(h->P);
    hd.payload_bytes = snap_bytes(h) - sizeof(SnapHeader);
    hd.checksum = fnv1a64(out + sizeof(SnapHeader), hd.payload_bytes);
    std::memcpy(out, &hd, sizeof(hd));
    return FG_OK;
}

int fg_snapshot_info(const void *buf, int64_t size, fg_params *params, int32_t *n_particles, uint32_t *seed,
                     uint32_t *stream_id, int64_t *next_counter, int32_t *type_ids, double *charges) {
    if (!buf || size < (int64_t)sizeof(SnapHeader)) return fail(FG_ERR_INVALID, "not a snapshot");
    SnapHeader hd;
    std::memcpy(&hd, buf, sizeof(hd));
    if (std::memcmp(hd.magic, kSnapMagic, 8) != 0 || hd.version != kSnapVersion)
        return fail(FG_ERR_INVALID, "not a snapshot of this format");
    if (hd.N < 1 || hd.payload_bytes < snap_host_bytes(hd.N) || (uint64_t)size < sizeof(SnapHeader) + hd.payload_bytes)
        return fail(FG_ERR_INVALID, "snapshot truncated");
    if (params) *params = hd.P;
    if (n_particles) *n_particles = hd.N;
    if (seed) *seed = hd.seed;
    if (stream_id) *stream_id = hd.stream_id;
    if (next_counter) *next_counter = hd.next_counter;
    const unsigned char *p = (const unsigned char *)buf + sizeof(SnapHeader);
    if (type_ids) std::memcpy(type_ids, p, 4 * (size_t)hd.N);
    if (charges) std::memcpy(charges, p + pad8(4 * (size_t)hd.N), 8 * (size_t)hd.N);
    return FG_OK;
}

int fg_restore(fg_system *h, const void *buf, int64_t size) {
    if (!h || !buf) return fail(FG_ERR_INVALID, "null argument");
    if (h->trial_pending) return fail(FG_ERR_STATE, "commit the pending trial first");
    if (h->batches > 0) return fail(FG_ERR_STATE, "system is a member of a batch");
    int rc = fg_snapshot_info(buf, size, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (rc) return rc;
    SnapHeader hd;
    std::memcpy(&hd, buf, sizeof(hd));
    const fg_params key = params_key(h->P);
    if (hd.N != h->N || hd.K != h->K || hd.model != h->model || hd.use_cells != (h->use_cells ? 1 : 0) ||
        hd.cap != h->cap || hd.nc[0] != h->nc[0] || hd.nc[1] != h->nc[1] || hd.nc[2] != h->nc[2] ||
        std::memcmp(&hd.P, &key, sizeof(key)) != 0)
        return fail(FG_ERR_INVALID, "snapshot is of another system (particles, parameters or cell grid differ)");
    if (hd.payload_bytes != snap_bytes(h) - sizeof(SnapHeader)) return fail(FG_ERR_INVALID, "snapshot size mismatch");
    const unsigned char *in = (const unsigned char *)buf + sizeof(SnapHeader);
    if (fnv1a64(in, hd.payload_bytes) != hd.checksum) return fail(FG_ERR_INVALID, "snapshot checksum mismatch");
    const unsigned char *p = in;
    std::vector<int32_t> types(h->N);
    std::vector<double> charges(h->N);
    std::memcpy(types.data(), p, 4 * (size_t)h->N);
    p += pad8(4 * (size_t)h->N);
    std::memcpy(charges.data(), p, 8 * (size_t)h->N);
    p += 8 * (size_t)h->N;
    for (int32_t t : types)
        if (t < 0 || t >= h->P.n_types) return fail(FG_ERR_INVALID, "snapshot type id %d out of range", t);
    const unsigned char *scp = nullptr;
    for (const SnapSection &s : snap_sections(h)) {
        if (s.dev == h->sc) scp = p;
        else CK(cudaMemcpyAsync(s.dev, p, s.bytes, cudaMemcpyHostToDevice, h->stream));
        p += pad8(s.bytes);
    }
    CK(cudaStreamSynchronize(h->stream));
    h->types = types;
    h->charges = charges;
    h->self_energy = hd.self_energy;
    h->cnt_accepted_host = hd.cnt_accepted_host;
    h->desc.qk_shift = hd.qk_shift;
    h->desc.qk_scale = hd.qk_scale;
    h->desc.seed = hd.seed;
    h->desc.stream_id = hd.stream_id;
    h->desc.stream_first = hd.stream_first;
    rc = push_desc(h);
    if (rc) return rc;
    h->state_set = false;   // until Q(k) is verified
    rc = snap_verify_qk(h);
    if (rc) return rc;
    SysScalars sc;
    std::memcpy(&sc, scp, sizeof(sc));
    sc.rebuild_pending = 0;
    rc = write_scalars(h, sc);
    if (rc) return rc;
    h->state_set = true;
    return FG_OK;
}

// ---- server jobs
struct JobSnapHeader {
    char magic[8];
    int64_t n_trials, done, accepted;
    double energy;
    uint32_t seed;
    int32_t pad;
};
constexpr char kJobMagic[8] = {'F', 'G', 'J', 'O', 'B', '0', '0', '1'};
static_assert(sizeof(JobSnapHeader) == 48, "the Python wrapper skips 48 bytes of job fields");

int64_t fg_server_snapshot_bytes(fg_server *s, int64_t job_id) {
    if (!s) return 0;
    for (fg_job *j : s->jobs)
        if (j->id == job_id && j->sys) return (int64_t)(sizeof(JobSnapHeader) + snap_bytes(j->sys));
    return 0;
}

int fg_server_snapshot(fg_server *s, int64_t job_id, void *buf, int64_t size) {
    if (!s || !buf) return fail(FG_ERR_INVALID, "null argument");
    for (fg_job *j : s->jobs) {
        if (j->id != job_id) continue;
        if (j->state != 1 || !j->sys) return fail(FG_ERR_STATE, "job %lld is not running", (long long)job_id);
        // rounds end synchronised (fg_server_step): nothing of the job is in flight
        if (size < (int64_t)(sizeof(JobSnapHeader) + snap_bytes(j->sys)))
            return fail(FG_ERR_CAPACITY, "job snapshot needs %zu bytes", sizeof(JobSnapHeader) + snap_bytes(j->sys));
        JobSnapHeader jh{};
        std::memcpy(jh.magic, kJobMagic, 8);
        jh.n_trials = j->n_trials;
        jh.done = j->done;
        jh.accepted = j->accepted;
        jh.energy = j->energy;
        jh.seed = j->seed;
        std::memcpy(buf, &jh, sizeof(jh));
        return fg_snapshot(j->sys, (unsigned char *)buf + sizeof(jh), size - (int64_t)sizeof(jh));
    }
    return fail(FG_ERR_INVALID, "unknown job %lld", (long long)job_id);
}

int fg_server_resume(fg_server *s, const void *buf, int64_t size, int64_t *job_id) {
    if (!s || !buf || !job_id) return fail(FG_ERR_INVALID, "null argument");
    if (size < (int64_t)sizeof(JobSnapHeader)) return fail(FG_ERR_INVALID, "not a job snapshot");
    JobSnapHeader jh;
    std::memcpy(&jh, buf, sizeof(jh));
    if (std::memcmp(jh.magic, kJobMagic, 8) != 0) return fail(FG_ERR_INVALID, "not a job snapshot");
    const unsigned char *sys = (const unsigned char *)buf + sizeof(jh);
    const int64_t sys_size = size - (int64_t)sizeof(jh);
    fg_params P;
    int32_t n = 0;
    int rc = fg_snapshot_info(sys, sys_size, &P, &n, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (rc) return rc;
    if (jh.done < 0 || jh.done > jh.n_trials) return fail(FG_ERR_INVALID, "job snapshot counters out of range");
    if (P.model != FG_MODEL_DH_LJ && P.model != FG_MODEL_EWALD_WCA) return fail(FG_ERR_INVALID, "unsupported model");
    for (fg_job *o : s->jobs)
        if (o->P.model != P.model) return fail(FG_ERR_INVALID, "one model per server");
    const bool blk = P.model == FG_MODEL_DH_LJ && !P.use_cell_list;
    const int64_t left = jh.n_trials - jh.done;
    const int64_t rt = blk ? round_trials_dh(s, n, dh_block_ctas_cap(n, tuned_min_per_cta()), left)
                           : std::min<int64_t>(left, round_trials_for(s, n));
    if ((int64_t)job_bytes(P, n, rt) > s->max_bytes) return fail(FG_ERR_CAPACITY, "job larger than the budget");
    fg_job *j = new fg_job();
    j->id = s->next_id++;
    j->P = P;
    j->ids.assign(n, 0);   // the particle count (admission sizes the job by it)
    j->seed = jh.seed;
    j->n_trials = jh.n_trials;
    j->done = jh.done;
    j->accepted = jh.accepted;
    j->energy = jh.energy;
    j->snapshot.assign(sys, sys + sys_size);
    s->jobs.push_back(j);
    *job_id = j->id;
    return FG_OK;
}

}  // extern "C"
