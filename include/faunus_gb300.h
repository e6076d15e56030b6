/* C-ABI of the GB300 (sm_103a) Metropolis energy-change library.
 *
 * Plain pointers and sizes only. Every function returns 0 on success or a
 * negative FG_ERR_* code; fg_last_error() then describes the failure (per
 * host thread). A handle is not re-entrant: one host thread at a time per
 * handle (each handle owns one CUDA stream); separate handles may be used
 * concurrently. Units are the reference's: Angstrom and kT.
 *
 * Each entry point names the reference interface it replaces (paths within
 * the reference project, bjornstenqvist/beoFaunus).
 */
#ifndef FAUNUS_GB300_H
#define FAUNUS_GB300_H
#include <stdint.h>

#include "fg_params.h"

#ifdef __cplusplus
extern "C" {
#endif

#define FG_OK 0
#define FG_ERR_INVALID -1      /* bad argument or parameter combination */
#define FG_ERR_CUDA -2         /* CUDA runtime failure (no device, OOM, launch) */
#define FG_ERR_DEVICE -3       /* a kernel raised an error flag (see text) */
#define FG_ERR_STATE -4        /* call out of order (e.g. commit without trial) */
#define FG_ERR_CAPACITY -5     /* exceeds a compiled or admitted capacity */

typedef struct fg_system fg_system;
typedef struct fg_batch fg_batch;
typedef struct fg_server fg_server;

typedef struct fg_sweep_stats {
    int64_t trials;         /* trials run by this call */
    int64_t accepted;       /* of which accepted */
    int64_t rebuilds;       /* full Q(k) rebuilds performed */
    double energy_change;   /* sum of accepted dU + rebuild corrections, as
                               Movebase::move returns it (move.h:515-555) */
    double device_ms;       /* device time of the call (CUDA events) */
    double sweep_kernel_ms; /* of which in the sweep kernel */
    int32_t sweep_launches; /* sweep kernel launches */
    int32_t error_flags;    /* device error bits (0 = none) */
    int64_t kernel_launches; /* all kernels this call launched (sweep, Q(k)
                                rebuild, gather, reset, swap, stream draw) */
} fg_sweep_stats;

/* Library version (major*10000 + minor*100 + patch). */
int fg_version(void);

/* Last error message of the calling host thread ("" if none). */
const char *fg_last_error(void);

/* Create a system of n_particles on the current CUDA device.
 * Replaces: constructing Space + NonbondedEwald / Nonbonded (ewald.h:507-550,
 * energy.h:803-815) from the reference's JSON input. */
int fg_create(const fg_params *params, int32_t n_particles, fg_system **out);

/* Free all device memory of a system. */
int fg_destroy(fg_system *h);

/* Upload particles (xyz[3N], charge[N] or NULL for the type charge,
 * type_ids[N]) and rebuild Q(k) and cells from scratch.
 * Replaces: Energybase::setSpace -> NonbondedEwald::setSpace/setGeometry
 * (energy.h:88-92, ewald.h:731-756). */
int fg_set_state(fg_system *h, const double *xyz, const double *charge, const int32_t *type_ids);

/* Download current positions (xyz[3N], wrapped into [-L/2, L/2)). */
int fg_get_state(fg_system *h, double *xyz);

/* Energy change of moving particles idx[0..n_moved) to new_xyz[3*n_moved]
 * (already wrapped into the box). Only n_moved == 1 for atomic systems.
 * Replaces: Energybase::updateChange + Energy::energyChange
 * (ewald.h:651-705, energy.h:3577-3621) as called by Movebase::move
 * (move.h:534-536). */
int fg_trial_du(fg_system *h, int32_t n_moved, const int32_t *idx, const double *new_xyz, double *du);

/* Accept (1) or reject (0) the last trial; *correction receives the Ewald
 * rebuild correction (0 unless a rebuild ran).
 * Replaces: Movebase acceptMove/rejectMove + Energybase::update
 * (move.h:538-548, ewald.h:613-646). */
int fg_commit(fg_system *h, int32_t accepted, double *correction);

/* Total energy {pairs, reciprocal, self, surface, total} (kT).
 * Replaces: Energybase::systemEnergy (energy.h:169-180). */
int fg_total_energy(fg_system *h, double *components5);

/* Number of k-vectors (0 for non-Ewald systems). */
int fg_num_kvectors(fg_system *h);

/* Current Q(k) as interleaved (re, im) doubles, 2K values.
 * Mirrors: NonbondedEwald::Q_ion_tot (ewald.h:457). */
int fg_get_qk(fg_system *h, double *qk);

/* Recompute Q(k) from all positions; *correction as in fg_commit.
 * Replaces: NonbondedEwald::updateAllComplexNumbers (ewald.h:388-415). */
int fg_rebuild_qk(fg_system *h, double *correction);

/* Draw the reference's per-trial random stream for AtomicTranslation on one
 * atomic group of n particles, as the global `slump` (std::mt19937 seeded
 * with `seed`) is consumed by move.h:818-864, group.h:129-134 and
 * move.h:567-573: particle index, displacement dp*(u-0.5) per axis and the
 * Metropolis uniform. dp_per_type[] is indexed by the particle's type. */
int fg_draw_translation_stream(fg_system *h, uint32_t seed, int64_t n_trials, int32_t *idx, double *disp,
                               double *u_metropolis);

/* Run n trials on the device from a host trial stream (idx[n], disp[3n] in
 * Angstrom, u[n] Metropolis uniforms): the whole loop of Movebase::move
 * (move.h:515-555) for AtomicTranslation, with Q(k) rebuilds every
 * update_frequency accepted trials. Optional per-trial outputs accepted[n]
 * and du[n] (may be NULL). */
int fg_sweep(fg_system *h, int64_t n, const int32_t *idx, const double *disp, const double *u,
             uint8_t *accepted, double *du, fg_sweep_stats *stats);

/* Stage a host trial stream on the device without running it. */
int fg_stream_upload(fg_system *h, int64_t n, const int32_t *idx, const double *disp, const double *u);

/* Generate n trials on the device (Philox4x32-10, key = (seed, stream_id)). */
int fg_stream_philox(fg_system *h, int64_t n, uint32_t seed, uint32_t stream_id);

/* Copy trials [first, first+n) of the staged stream back to the host in
 * the fg_sweep input format (idx, disp in Angstrom, Metropolis uniform). */
int fg_stream_get(fg_system *h, int64_t first, int64_t n, int32_t *idx, double *disp, double *u);

/* Run the staged stream from its start on the device (no host copies). */
int fg_stream_run(fg_system *h, fg_sweep_stats *stats);

/* Block until all work of this handle is done. */
int fg_synchronize(fg_system *h);

/* Launch configuration of the sweep kernel: threads per system (0 = auto). */
int fg_set_threads(fg_system *h, int32_t threads);
int fg_get_threads(fg_system *h);

/* Ewald systems run alone (fg_stream_run, fg_sweep): CTAs of the
 * thread-block cluster that runs the block-of-trials sweep (1, 2, 4, 8 or 16;
 * 0 = the built-in choice: the most CTAs with at least 128 k-vectors each).
 * The k-vectors are split over the CTAs; the
 * size in effect is capped by what the device co-schedules and what fits in
 * shared memory. Batches run one CTA per system. Replaces nothing of the
 * reference (NonbondedEwald, ewald.h:269-715, runs on one host thread); a
 * launch-shape setting like fg_set_threads. */
int fg_set_cluster(fg_system *h, int32_t ctas);
/* The size in effect (ctas) and the largest that fits (max_ctas). */
int fg_get_cluster(fg_system *h, int32_t *ctas, int32_t *max_ctas);

/* One Philox4x32-10 block, host side (for tests of the generator). */
void fg_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Q(k) is kept as an exact integer sum of per-particle contributions, so a
 * rebuild reproduces it bit for bit. skip != 0: sweeps do not stop for the
 * update_frequency rebuilds (fg_rebuild_qk still verifies on demand);
 * skip == 0 (default): rebuild where NonbondedEwald::update would
 * (ewald.h:633) and flag any difference as a device error. */
int fg_set_rebuild_policy(fg_system *h, int32_t skip);

/* Running total energy: systemEnergy at upload plus every accepted dU and
 * rebuild correction since (what Propagator tracks for drift checks,
 * move.h:7730-7731, 7911-7913). */
int fg_running_energy(fg_system *h, double *energy);

/* Device bytes held by a system. */
int64_t fg_device_bytes(fg_system *h);

/* ---- batches: many independent systems per launch -------------------------
 * Replaces: running one Movebase::move loop per replica process. All members
 * must use the same model and kernel variant; each keeps its own stream of
 * trials and its own state. */
int fg_batch_create(fg_system *const *systems, int32_t n, fg_batch **out);
int fg_batch_destroy(fg_batch *b);
/* Threads per system CTA for the whole batch (0 = the largest member's). */
int fg_batch_set_threads(fg_batch *b, int32_t threads);
/* Device-generated streams: member s gets counts[s] trials from Philox with
 * key (seed, stream_ids[s]) (stream_ids may be NULL: s). */
int fg_batch_stream_philox(fg_batch *b, const int64_t *counts, uint32_t seed, const uint32_t *stream_ids);
/* Stage a host trial stream (fg_stream_upload format) for one member. */
int fg_batch_stream_upload(fg_batch *b, int32_t member, int64_t n, const int32_t *idx, const double *disp,
                           const double *u);
/* Run every member's staged stream; per-member and summed statistics. */
int fg_batch_run(fg_batch *b, fg_sweep_stats *per_system, fg_sweep_stats *total);
/* Where the Ewald block kernel's Q(k) rebuilds (every update_frequency
 * accepted trials, ewald.h:633-640) run: 0 (default) inside the sweep launch
 * when the batch has at least one member per SM, else in the separate
 * rebuild kernel spread over all SMs; 1 always inside; 2 never. Results are
 * identical either way (the rebuild reproduces the exact Q(k)). */
int fg_batch_set_rebuild_mode(fg_batch *b, int32_t mode);
/* Record per-trial dU and acceptance of one member in the following
 * fg_batch_run calls (on != 0), or stop (on == 0): the per-move record
 * Movebase::move keeps (move.h:515-555, its dusum and acceptance counters)
 * for one system of the batch, read back with fg_log_get. */
int fg_batch_set_log(fg_batch *b, int32_t member, int32_t on);
/* dU (kT, as the device computed it) and acceptance of trials
 * [first, first + n) of the system's last logged run (fg_sweep, or an
 * fg_batch_run with logging on for it); either output may be NULL. */
int fg_log_get(fg_system *h, int64_t first, int64_t n, double *du, uint8_t *accepted);

/* ---- parallel tempering over a batch ----------------------------------------
 * Replaces: Move::ParallelTempering (move.h:6542-6771) with MPI ranks as
 * temperature rungs. Member i starts at temperatures[i] (units of the
 * energy scale: the Boltzmann factor is exp(-dU/T)). */
int fg_pt_setup(fg_batch *b, const double *temperatures, uint32_t seed);
/* rounds x (sweeps_per_round sweeps of every member, then one exchange
 * attempt between each neighbouring pair picked as in findPartner,
 * move.h:6621-6633); one CUDA graph per round. */
int fg_pt_run(fg_batch *b, int32_t rounds, int32_t sweeps_per_round, fg_sweep_stats *total);
/* One exchange attempt with the caller's randoms: the pairing from
 * u_direction (> 0.5: rung 2i with 2i+1, else 2i with 2i-1, as findPartner
 * draws it, move.h:6621-6633) and, for every pair, the test not
 * u_accept > exp(-dU) of _energyChange (move.h:6700-6722), dU from
 * energies[system] (kT at unit temperature; NULL: the running totals).
 * Replaces the exchange step of Move::ParallelTempering::move when the host
 * replays the reference's own random streams; exchanged[rung] (or NULL) is 1
 * where the rung's system changed. */
int fg_pt_swap(fg_batch *b, double u_direction, double u_accept, const double *energies, int32_t *exchanged);
/* perm[rung] = member at that temperature; energies[member]; exchange
 * attempts/accepts per rung pair (rung, rung+1). Any pointer may be NULL. */
int fg_pt_get(fg_batch *b, int32_t *perm, double *energies, int64_t *attempts, int64_t *accepts);

/* ---- job server: continuous batching of independent Monte Carlo jobs --------
 * No counterpart in the reference (one job per process there). Jobs are
 * admitted in submission order while their device footprint fits
 * max_device_bytes; every fg_server_step advances all admitted jobs in one
 * launch (about round_pairs / N trials each, at least one sweep). */
int fg_server_create(int64_t max_device_bytes, int32_t threads, int64_t round_pairs, fg_server **out);
int fg_server_destroy(fg_server *s);
int fg_server_submit(fg_server *s, const fg_params *params, int32_t n, const double *xyz, const double *charge,
                     const int32_t *type_ids, uint32_t seed, int64_t n_trials, int64_t *job_id);
int fg_server_step(fg_server *s, int32_t *n_running, int32_t *n_finished, double *device_ms);
/* state: 0 queued, 1 running, 2 done, 3 failed. xyz (3N) filled once done
 * (finished jobs keep their results in host memory; their device memory is
 * returned to the budget at once). */
int fg_server_poll(fg_server *s, int64_t job_id, int32_t *state, int64_t *trials_done, int64_t *accepted,
                   double *energy, double *xyz);
int fg_server_release(fg_server *s, int64_t job_id);
/* Drop a job in any state (a client that went away): a running job stops
 * between rounds, its device memory returns to the budget at once and queued
 * jobs may be admitted in the next round. The other jobs' results are
 * unchanged (each keeps its own stream and state). */
int fg_server_cancel(fg_server *s, int64_t job_id);
int64_t fg_server_bytes_in_use(fg_server *s);

/* ---- snapshots: stop a run and resume it bit for bit ------------------------
 * Replaces: Space::save/load (space.h:376-377), which keep the particles as
 * text, and the random state the reference writes to move_out.json
 * (slump.h:111-124, move.h:7900) but never reads back. A snapshot holds
 * everything that decides how a system continues: the fixed-point positions,
 * charges and types, the cell lists in slot order, the exact integer Q(k),
 * the running energies and surface dipole, the accept count toward the next
 * update_frequency rebuild, and the key and counters of the system's Philox
 * stream. It is taken between runs (no trial pending) and holds no staged
 * trial stream. A system restored from it (fg_create with the same
 * parameters and particle count, then fg_restore) and given the same trial
 * streams runs exactly as the original does from that point: same positions,
 * Q(k), decisions, dU and running energy, to the bit. fg_restore refuses
 * another system's snapshot (particle count, parameters or cell grid) and a
 * damaged one (checksum) before it changes anything; it then rebuilds Q(k)
 * from the restored positions and refuses the snapshot unless the two agree
 * bit for bit, after which the system needs fg_set_state or a good snapshot
 * again. Binary, in the host's byte order. */
int64_t fg_snapshot_bytes(fg_system *h);
int fg_snapshot(fg_system *h, void *buf, int64_t size);
int fg_restore(fg_system *h, const void *buf, int64_t size);
/* Parameters, particle count, Philox key and next counter, type ids[N] and
 * charges[N] of a snapshot (any output may be NULL): what is needed to create
 * the system that fg_restore fills. */
int fg_snapshot_info(const void *buf, int64_t size, fg_params *params, int32_t *n_particles, uint32_t *seed,
                     uint32_t *stream_id, int64_t *next_counter, int32_t *type_ids, double *charges);
/* A running job's snapshot (between fg_server_step calls): its system plus
 * its seed, trial count, trials done, accepted count and energy. A job
 * resumed from it (fg_server_resume, on this server or another, after the
 * first was cancelled or its process ended) draws the remaining trials of
 * the same Philox stream and finishes with the result the uninterrupted job
 * would have had. */
int64_t fg_server_snapshot_bytes(fg_server *s, int64_t job_id);
int fg_server_snapshot(fg_server *s, int64_t job_id, void *buf, int64_t size);
int fg_server_resume(fg_server *s, const void *buf, int64_t size, int64_t *job_id);

/* ---- pair energy without device allocation ---------------------------------
 * No counterpart in the reference. For callers that cannot call cudaMalloc:
 * a plugin inside a host application that owns the whole GPU memory pool and
 * only hands out buffers it allocated itself, or a time-critical loop that
 * must not call the allocator (cudaMalloc/cudaFree may synchronize the
 * device). Computes the pair part of systemEnergy (energy.h:169-180; the
 * same value as component 0 of fg_total_energy) for n particles given in
 * caller-owned DEVICE buffers: d_xyz[3n], d_charge[n] (or NULL for the type
 * charges), d_types[n]; writes one double to d_energy, on `stream` (a
 * cudaStream_t, or NULL for the default stream). Asynchronous: synchronize
 * the stream before reading d_energy. Every d_types[i] must lie in
 * [0, params->n_types); the ids are in device memory, so they are checked
 * on the device: with any id outside that range d_energy receives NaN.
 * Every temporary lives in one fixed __device__ array of about 1.7 MB, held
 * by every GPU that loads this library until the process exits; the call
 * allocates nothing. n is limited to FG_NOALLOC_MAX_PARTICLES (larger n:
 * FG_ERR_CAPACITY). The first call on a device looks up that array's device
 * address, with the device current; make that first call before any stream
 * capture. All calls share the array: calls that overlap on the GPU race and
 * give wrong results, so serialize them. */
#define FG_NOALLOC_MAX_PARTICLES 65536
int fg_pair_energy_noalloc(const fg_params *params, int32_t n, const double *d_xyz, const double *d_charge,
                           const int32_t *d_types, double *d_energy, void *stream);

/* ------------------------------------------------------------------ rigid dipolar molecules
 * Space<Cuboid, DipoleParticle> with equal-size rigid molecules (contiguous
 * sites), energy NonbondedVector over CoulombGalore + LennardJonesLB +
 * IonDipole + DipoleDipoleGalore (reaction field, FG_MODEL_MULTIPOLE_RF), and
 * the TranslateRotate move. One system runs on a thread-block cluster of
 * CTAs (fg_mol_set_cluster). */
typedef struct fg_molsys fg_molsys;

/* Create a system of n_sites sites in molecules of sites_per_molecule (<= 31)
 * consecutive sites. Replaces: Space(json) with a molecular "moleculelist"
 * entry + NonbondedVector<Tspace, CombinedPairPotential<...>>(json)
 * (energy.h:1062-1090, multipole.h:600-640, 836-870, 983-990). */
int fg_mol_create(const fg_params *params, int32_t n_sites, int32_t sites_per_molecule, fg_molsys **out);
int fg_mol_destroy(fg_molsys *h);

/* Positions (3N), dipole unit vectors (3N, may be NULL: no dipoles), dipole
 * scalars in e*Angstrom (N, may be NULL), atom types (N), molecule mass
 * centres (3M, may be NULL: computed as Geometry::massCenter with equal
 * masses, geometry.h:714-738). Replaces: Energybase::setSpace
 * (energy.h:88-92) after Group::setMassCenter (group.h:174-179). */
int fg_mol_set_state(fg_molsys *h, const double *xyz, const double *mu_unit, const double *mu_scalar,
                     const int32_t *type_ids, const double *mass_centers);
int fg_mol_get_state(fg_molsys *h, double *xyz, double *mu_unit, double *mass_centers);

/* CTAs per system (power of two up to the device's cluster limit). */
int fg_mol_set_cluster(fg_molsys *h, int32_t ctas);
int fg_mol_get_cluster(fg_molsys *h, int32_t *ctas, int32_t *max_ctas);

/* dU of moving molecule `molecule` to new site positions (3*gs) and dipole
 * unit vectors (3*gs, may be NULL: unchanged), with its new mass centre (3,
 * may be NULL). Replaces: Energy::energyChange (energy.h:3577-3621) with a
 * whole-group Change (move.h:1685) -> g2All -> NonbondedVector::g2g. */
int fg_mol_trial_du(fg_molsys *h, int32_t molecule, const double *new_xyz, const double *new_mu_unit,
                    const double *new_mass_center, double *du);
/* Accept or reject the pending trial. Replaces: TranslateRotate::_acceptMove
 * / _rejectMove (move.h:1688-1705, Group::accept/undo group.h:370-385). */
int fg_mol_commit(fg_molsys *h, int32_t accepted);

/* The reference's global-slump draws of n TranslateRotate trials on one
 * molecule kind with "permol" (move.h:1624-1685, point.h:74-88, 567-573):
 * molecule, unit axis (3n), centre kind (0 mass centre, 1 first site, 2 last
 * site; only when center_rotation is 0), angle, translation (3n),
 * Metropolis uniform. Host only (no device). */
int fg_mol_draw_stream(uint32_t seed, int32_t n_molecules, int64_t n, double dp, double dprot,
                       int32_t center_rotation, int32_t *mol, double *axis, int32_t *center, double *angle,
                       double *trans, double *u);

/* n TranslateRotate trials on the device from those draws; rotate/translate
 * say whether dprot/dp exceed 1e-6 (move.h:1642, 1671). acc and du (may be
 * NULL) receive per-trial results. Replaces: Movebase::move with
 * TranslateRotate (move.h:515-555, 1620-1705). */
int fg_mol_sweep(fg_molsys *h, int64_t n, const int32_t *mol, const double *axis, const double *angle,
                 const int32_t *center, const double *trans, const double *u, int32_t rotate, int32_t translate,
                 uint8_t *acc, double *du, fg_sweep_stats *stats);

/* Stage a trial stream (fg_mol_sweep's arguments) without running it. */
int fg_mol_stream_upload(fg_molsys *h, int64_t n, const int32_t *mol, const double *axis, const double *angle,
                         const int32_t *center, const double *trans, const double *u, int32_t rotate,
                         int32_t translate);
/* Run the staged streams of independent systems (same cluster size) in one
 * launch: one cluster per system. per_system (may be NULL) gets n_systems
 * records. No counterpart in the reference (one system per process there). */
int fg_mol_run_many(fg_molsys *const *systems, int32_t n_systems, fg_sweep_stats *per_system, fg_sweep_stats *total);

/* comp = {intermolecular, intramolecular, total}, FP64. Replaces:
 * Energybase::systemEnergy (energy.h:169-180). */
int fg_mol_total_energy(fg_molsys *h, double *comp);
/* Total energy at fg_mol_set_state plus every accepted dU since. */
int fg_mol_running_energy(fg_molsys *h, double *u);
int64_t fg_mol_device_bytes(fg_molsys *h);

/* ---------------------------------------------------------------- volume move
 * Move::Isobaric (move.h:5529-5624) with Energy::ExternalPressure
 * (energy.h:1817-1890) on one atomic group: V' = exp(ln V + half * dp) with
 * half = slump.half() in [-0.5, 0.5), positions scaled by (V'/V)^(1/3) about
 * the origin, dU = E(V') - E(V) + pressure (V' - V) - (N + 1) ln(V'/V) with
 * pressure in particles per cubic Angstrom (the reference's mM input times
 * 1.0_mM, physconst.h:170-173), Metropolis with u (move.h:567-573). On
 * acceptance the system takes the new box (every box-dependent table is
 * rebuilt); a staged trial stream is dropped, and a system in a live batch
 * is refused (FG_ERR_STATE). reference_quirk (Ewald): take the trial's
 * reciprocal energy as the reference computes it, from the positions before
 * scaling in the new box (NonbondedEwald::setGeometry rebuilding Q(k) from
 * spc->p, ewald.h:731-756), so dU and decisions match the reference's. */
int fg_volume_move(fg_system *h, double half, double dp, double pressure, double u, int32_t reference_quirk,
                   double *du, int32_t *accepted);
/* systemEnergy (energy.h:169-180) in FP64 throughout: pairs and Q(k) on the
 * device in double, reciprocal/self/surface on the host; components as
 * fg_total_energy. The volume move's energies come from here. */
int fg_total_energy_fp64(fg_system *h, double *components5);
/* Current box lengths (Angstrom; changed by accepted volume moves). */
int fg_get_box(fg_system *h, double *box);
/* n draws of the reference's global slump() (slump.h:62-95) from seed: host only. */
int fg_slump_uniforms(uint32_t seed, int64_t n, double *u);

/* ---------------------------------------------------------------- analysis
 * AtomRDF::update (analysis.h:2116-2134): add the current configuration's
 * pair counts between atom types type1 and type2 (each unordered pair i < j
 * once) to hist[0 .. n_bins), bin = int(r / dr + 0.5) on the minimum-image
 * distance (Table2D::round, auxiliary.h:831; Cuboid::sqdist,
 * geometry.h:507-515). *n_pairs (may be NULL) grows by the pairs at any
 * distance (the normalisation sum of PairFunctionBase::normalize,
 * analysis.cpp:190-205). n_bins <= 8192. */
int fg_rdf_sample(fg_system *h, int32_t type1, int32_t type2, double dr, int32_t n_bins, int64_t *hist,
                  int64_t *n_pairs);

/* ---------------------------------------------------------------- state files
 * The reference's Space::save/load text format (space.h:736-764, 807-880):
 * box lengths, N particle records, G group records (front back molId molsize
 * and the mass centre, group.h:388-407), "randomstate" and an mt19937 state.
 * kind 0: PointParticle records (x y z charge radius mw id hydrophobic,
 * point.h:544-566); kind 1: DipoleParticle records (the same, then the dipole
 * unit vector, its scalar, the induced dipole and two 3x3 tensors,
 * point.h:649-666). Host only.
 *
 * fg_state_read fills what it is given (any output may be NULL; groups take
 * 4 int32 and group_cm 3 doubles per group) and fails with FG_ERR_CAPACITY
 * past n_max particles or g_max groups. fg_state_write writes the records
 * with 16 significant digits (NULL charge/radius/hydrophobic: 0, NULL mw: 1;
 * dipole records carry no induced dipole and zero tensors) and the state of
 * std::mt19937(rng_seed) for the reference to continue from. */
int fg_state_read(const char *path, int32_t kind, int32_t n_max, double *box, int32_t *n, double *xyz,
                  double *charge, double *radius, double *mw, int32_t *ids, int32_t *hydrophobic, double *mu_unit,
                  double *mu_scalar, int32_t g_max, int32_t *n_groups, int32_t *groups, double *group_cm);
int fg_state_write(const char *path, int32_t kind, const double *box, int32_t n, const double *xyz,
                   const double *charge, const double *radius, const double *mw, const int32_t *ids,
                   const int32_t *hydrophobic, const double *mu_unit, const double *mu_scalar, int32_t n_groups,
                   const int32_t *groups, const double *group_cm, uint32_t rng_seed);

/* ---------------------------------------------------------------- autotuner
 * Launch shapes chosen by timing candidates on the device, on a clone of the
 * caller's system(s): the caller's chains do not advance. Each call applies
 * the fastest candidate and records it for the process (later systems of the
 * same size class, later batches and the job server start from it). A shape
 * changes only the order of floating-point sums. No counterpart in the
 * reference (its loops have no launch shapes). */
typedef struct {
    int32_t n;                /* candidates timed (0: nothing to tune) */
    int32_t chosen;           /* index of the applied candidate */
    int32_t value[8];         /* the tuned quantity per candidate */
    double us_per_trial[8];   /* device time per trial (per member trial for batches) */
} fg_tune_report;

/* DH+LJ block sweeps: CTAs per system (cluster size, powers of two); Ewald
 * block sweeps: CTAs of the cluster a system alone runs on (fg_set_cluster);
 * Ewald one-trial sweeps: threads per CTA. n_trials >= 32 per candidate. */
int fg_autotune(fg_system *h, int64_t n_trials, fg_tune_report *report);
/* DH+LJ batches: least particles per CTA when the SMs are shared out among
 * members (128 .. 2048), timed on equal sweeps of the members (n_trials for
 * the largest, in proportion to N for the others). */
int fg_batch_autotune(fg_batch *b, int64_t n_trials, fg_tune_report *report);
/* Rigid molecules: CTAs per system (cluster size). */
int fg_mol_autotune(fg_molsys *h, int64_t n_trials, fg_tune_report *report);
/* Forget the recorded choices (back to the built-in heuristics). */
int fg_tune_reset(void);

/* ---------------------------------------------------------------- point dipoles under Ewald
 * Point charges and point dipoles (DipoleParticle, point.h:591-680) in one
 * atomic group, energy NonbondedEwald<Tspace, LennardJonesLB, useIonIon,
 * useIonDipole, useDipoleDipole> (ewald.h:228-757; params.ewald_terms holds
 * the three flags, params.ewald_dipole_quirk selects the sum as ewald.h
 * states it (0) or as its live code computes it (1)), moves AtomicRotation
 * (move.h:976-1072) and AtomicTranslation (move.h:818-901). FP64 throughout;
 * one CTA per system, many systems per launch (fg_dip_run_many). */
typedef struct fg_dipsys fg_dipsys;

/* Replaces: Space<Cuboid, DipoleParticle> + NonbondedEwald construction
 * (ewald.h:507-550). model must be FG_MODEL_EWALD_DIPOLE; cutoffK <= 31. */
int fg_dip_create(const fg_params *params, int32_t n_particles, fg_dipsys **out);
int fg_dip_destroy(fg_dipsys *h);
int fg_dip_num_kvectors(fg_dipsys *h);
/* Positions (Angstrom), dipole unit vectors, dipole scalars (e Angstrom),
 * charges (NULL: the type charges) and atom types. Q(k) is built from
 * scratch (setSpace, ewald.h:746-756). */
int fg_dip_set_state(fg_dipsys *h, const double *xyz, const double *mu_unit, const double *mu_scalar,
                     const double *charges, const int32_t *type_ids);
int fg_dip_get_state(fg_dipsys *h, double *xyz, double *mu_unit);
/* Threads per CTA (multiple of 32, 32..256; default 128). */
int fg_dip_set_threads(fg_dipsys *h, int32_t threads);
/* Energy change of moving particle i to new_xyz with dipole new_mu_unit
 * (NULL: unchanged); replaces Energy::energyChange after updateChange
 * (energy.h:3577-3621, ewald.h:651-705). One trial may be pending. */
int fg_dip_trial_du(fg_dipsys *h, int32_t i, const double *new_xyz, const double *new_mu_unit, double *du);
/* acceptMove / rejectMove + NonbondedEwald::update (ewald.h:613-646);
 * correction (may be NULL) = what update() returns: the reciprocal-energy
 * change of a Q(k) rebuild on this accept, else 0. */
int fg_dip_commit(fg_dipsys *h, int32_t accepted, double *correction);
/* n trials: kind[t] 1 = AtomicRotation of particle idx[t] by angle[t] about
 * axis[t] (3 per trial), 2 = AtomicTranslation by disp[t] (3 per trial);
 * Metropolis uniform u[t] (reject iff u > exp(-dU/kT)). acc/du may be NULL. */
int fg_dip_sweep(fg_dipsys *h, int64_t n, const int32_t *kind, const int32_t *idx, const double *axis,
                 const double *angle, const double *disp, const double *u, uint8_t *acc, double *du,
                 fg_sweep_stats *stats);
/* Stage a stream without running it; fg_dip_run_many runs the staged streams
 * of many systems in one launch sequence (one CTA per system). */
int fg_dip_stream_upload(fg_dipsys *h, int64_t n, const int32_t *kind, const int32_t *idx, const double *axis,
                         const double *angle, const double *disp, const double *u);
int fg_dip_run_many(fg_dipsys *const *systems, int32_t n_systems, fg_sweep_stats *per_system, fg_sweep_stats *total);
/* The reference's slump draws for n trials (see fg_dip.cu); with p_rotate < 0
 * kind[] is read (the caller's move order), else drawn. */
int fg_dip_draw_stream(uint32_t seed, int32_t n_particles, int64_t n, double p_rotate, double dp, double dprot,
                       int32_t *kind, int32_t *idx, double *axis, double *angle, double *disp, double *u);
/* comp = {EwaldReal pairs, LJ pairs, reciprocal, self, surface, total}, FP64. */
int fg_dip_total_energy(fg_dipsys *h, double *comp);
/* Total energy at fg_dip_set_state plus accepted dU and rebuild corrections since. */
int fg_dip_running_energy(fg_dipsys *h, double *u);
int64_t fg_dip_device_bytes(fg_dipsys *h);
/* Autotuner (see fg_autotune): threads per system, timed on clones of the
 * given systems run together (n_trials each per candidate); applied to them
 * and recorded for dipole systems created afterwards. */
int fg_dip_autotune(fg_dipsys *const *systems, int32_t n_systems, int64_t n_trials, fg_tune_report *report);

#ifdef __cplusplus
}
#endif
#endif
