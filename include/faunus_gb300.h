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

/* One Philox4x32-10 block, host side (for tests of the generator). */
void fg_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
