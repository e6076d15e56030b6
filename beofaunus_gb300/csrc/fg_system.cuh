// Device-resident layout of one Monte Carlo system and of the trial stream.
//
// HBM/L2 layout per system (struct-of-arrays, 16-byte records):
//   pos64  int64[3N]   master fixed-point coordinates (x,y,z per particle)
//   pos4   int4[N]     {X>>32, Y>>32, Z>>32, charge bits}: what pair loops read
//   pos_ext short4[N]  the next 16 bits of X, Y, Z: read only for pairs inside
//          the repulsive core, where 32-bit resolution is too coarse
//   ptype  uint8[N]    atom type
//   cells  (cell-list systems only) per cell `cap` slots of int4 positions and
//          int32 particle ids, plus counts; p_cell/p_slot locate each particle
//   Ewald  kvec float4[K] {kx, ky, kz, A_k * 2*pi*lB/V}, kpack uint32[K] (n
//          vector as signed bytes), qfix longlong2[K]: Q(k) as exact sums of
//          per-particle integer contributions (see qk_term_bits in fg_kernels.cu)
#pragma once
#include <cstdint>

#include "fg_device.cuh"

namespace fg {

constexpr int kMaxTypes = 16;
constexpr int kMaxThreads = 1024;
constexpr int kMaxKPerThread = 4;

enum : int32_t {
    kErrNone = 0,
    kErrCellOverflow = 1,   // a cell ran out of slots
    kErrStencil = 2,        // a particle moved more than one cell
    kErrKCapacity = 4,      // more k-vectors than threads * kMaxKPerThread
    kErrNonFinite = 8,      // dU was NaN
    kErrQkMismatch = 16,    // a rebuild did not reproduce the incremental Q(k)
    kErrLaunch = 64,        // a kernel ran with another cluster or block shape than it was written for
};

// One trial of the stream (40 bytes): particle index, fixed-point
// displacement, and the Metropolis threshold -ln(u) as a df number.
struct Trial {
    int32_t idx;
    int32_t pad;
    int64_t d[3];
    float thr_hi, thr_lo;
};

// Per-system scalars that persist across kernel launches.
struct SysScalars {
    int64_t cursor;        // next trial to run
    int64_t n_trials;      // trials in the stream
    int64_t n_accepted;
    int32_t cnt_accepted;  // accepted since the last Q(k) rebuild
    int32_t rebuild_pending;
    int32_t error;
    int32_t n_rebuilds;    // Q(k) rebuilds since upload
    float u_hi, u_lo;      // running sum of accepted dU + rebuild corrections
    float utot_hi, utot_lo; // running total energy (set at upload, then += dU)
    float m[3][2];         // surface dipole sum(q * eff * r) as df per axis
    int32_t verify_rebuild; // flag a rebuild that changes Q(k) as an error
    int32_t pad2;
};

// Everything a kernel needs to find one system (passed in global memory
// for batched launches, by value for single ones).
struct alignas(16) SysDesc {
    int32_t model;
    int32_t N;
    int32_t K;
    int32_t n_types;
    int32_t uniform_types;     // all type-pair tables equal
    int32_t use_cells;
    int32_t nc[3];             // cells per axis (use_cells)
    int32_t cap;               // slots per cell
    float L[3];                // box
    float s32[3];              // L / 2^32: Angstrom per unit of a high word
    float s32sq;               // s32[0]^2 (cubic boxes; difference-form pairs)
    float dl32[3];             // L / 2^64 in float for displacements
    float rc2;                 // real-space cutoff squared (Ewald), huge otherwise
    float alpha;               // Ewald alpha
    float lB;                  // Bjerrum length
    float kappa;               // Debye-Hueckel kappa
    float surf_c;              // 2*pi*lB/((2 eps_surf+1) V) * const_inf
    float kT;                  // temperature scale of the Boltzmann factor
    int32_t update_frequency;
    int32_t skip_rebuild;      // do not stop sweeps for Q(k) rebuilds
    int32_t rebuild_in_kernel; // the Ewald block kernel rebuilds Q(k) itself (else it exits for the rebuild kernel)
    int32_t log_trials;        // write per-trial dU/accept
    // per-type-pair tables (row-major nt*nt) and per-type effective charge
    float s2[kMaxTypes * kMaxTypes];
    float eps4[kMaxTypes * kMaxTypes];
    float wca2[kMaxTypes * kMaxTypes];   // s2 * 2^(1/3): WCA cut
    float qeqe[kMaxTypes * kMaxTypes];
    float eff[kMaxTypes];
    // df constants for the repulsive-core pair path (see pair_core_df)
    float2 pref_df[kMaxTypes * kMaxTypes];  // QeQe * lB (Ewald) or lB (DH) as df
    float2 s2_df[kMaxTypes * kMaxTypes];    // sigma_ij^2 as df
    float2 eps4_df[kMaxTypes * kMaxTypes];  // 4 eps_ij as df
    float2 coef_df;                         // alpha (Ewald) or kappa (DH) as df
    float2 s48_df[3];                       // L / 2^48 per axis as df
    int32_t core_tab_n;                     // entries of core_tab (spacing 1/128)
    const float4 *core_tab;                 // per entry: {f0 hi, f0 lo, f1 hi, f1 lo}
    const float4 *core_tab2;                // per entry: {f2, f3, f4, 0}
    // arrays
    int64_t *pos64;
    int4 *pos4;
    short4 *pos_ext;          // 16 more bits per axis below the high word
    uint8_t *ptype;
    int32_t *cell_count;
    int4 *cell_pos;
    short4 *cell_ext;
    int32_t *cell_pid;       // particle id | type << 24
    int32_t *p_cell;
    int32_t *p_slot;
    float4 *kvec;
    uint32_t *kpack;
    longlong2 *qfix;
    const Trial *trials;
    float2 *trial_du;        // per-trial dU (df), optional
    uint8_t *trial_acc;      // per-trial acceptance, optional
    SysScalars *sc;
    const float2 *sc_tab;    // cos/sin table at multiples of 2 pi / 256
    const int64_t *dp_fix;   // per type and axis: round(dp / L * 2^32)
    uint32_t stream_id;      // Philox key word of this system's trial stream
    uint32_t seed;           // Philox key word (seed)
    int64_t stream_first;    // counter of trial 0 in the current stream
    longlong2 *qnew;         // rebuild target (K)
    // Q(k) contributions: one particle adds 2^g c q eff e^{ik.r} with each
    // of its four real products rounded to an integer (each of magnitude
    // < 2^22, c = 4095/4096), shifted left by qk_shift = 28 - g; Q(k) is in
    // units of 2^-28 / c
    int32_t kcc;             // |n_a| <= kcc for every k-vector
    int32_t qk_shift;
    float qk_scale;          // 2^g c
    int32_t nseg;            // runs of k-vectors that share (nx, ny), for the rebuild
    const int2 *kseg;        // {k0 | len << 24, nx & 0xFF | (ny & 0xFF) << 8 | (nz0 & 0xFF) << 16}
    int32_t n_rb_items;      // in-kernel rebuild of the block kernel: k-vector pairs (+n, -n) per item
    const int4 *rb_items;    // {kp0 | len << 24, kn0 | n0 << 24, nx & 0xFF | (ny & 0xFF) << 8, 0}
    float reach2;            // no pair term acts beyond r^2 = reach2 (cutoff, WCA range, core)
    // Ewald block kernel on a thread-block cluster (a system alone): CTA rank r
    // holds the k-vectors [k0, k1) and owns rb_items [i0, i1), eb_ranges[r] =
    // {k0, k1, i0, i1}; eb_kmax = the most k-vectors one CTA holds. One CTA:
    // eb_ctas = 1, eb_ranges[0] = {0, K, 0, n_rb_items}, eb_kmax = K.
    int32_t eb_ctas;
    int32_t eb_kmax;
    const int4 *eb_ranges;
    // isotropic_pbc (ewald.h:347-360, 394-399): k-vectors in the positive
    // octant, Q(k) real (cosine products); one-trial kernels only
    int32_t iso;
};

}  // namespace fg
