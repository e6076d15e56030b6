// FP64 CPU oracle for the Metropolis energy-change path -- TEST INFRASTRUCTURE.
//
// A plain restatement, in double precision, of the reference's algorithm for
// the paths the GPU library implements. Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg may load it, and only as the checker or the
// timed CPU baseline; the product library never links or calls it.
//
// Pinned against: (1) the Ewald known answers of the reference's unit test
// (src/examples/unittests.cpp:131-170, values from doi:10.1063/1.481216) and
// (2) per-trial dU / acceptance logs of the reference itself, built from its
// own sources (oracle/ref) and committed as fixtures under tests/golden/.
//
// Each routine cites the reference file:line it restates (paths within the
// reference project).
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "../include/fg_params.h"
#include "or_common.h"

namespace {

using namespace orc;

struct Particle { V3 r; double q; int id; };

// ---------------------------------------------------------------- system
struct System {
    fg_params P;
    Cuboid geo;
    int N = 0;
    std::vector<Particle> p, trial;  // Space::p / Space::trial (space.h:255-272)
    // per-type pair tables (PairMatrix in the reference)
    int nt = 0;
    std::vector<double> s2, eps4, qeqe, eff;
    // Ewald state (NonbondedEwald members, ewald.h:451-461)
    double alpha = 0, alpha2 = 0, rc2 = 0, kappa = 0, lB = 0, V = 0, const_inf = 0;
    int K = 0;
    std::vector<V3> kv;
    std::vector<double> Ak;
    std::vector<std::complex<double>> Q, Qt;
    double surf = 0, surf_t = 0, recip = 0, recip_t = 0;
    int cnt_accepted = 0;
    double update_drift = 0;
    // DH
    double k_dh = 0;
    // pending trial
    std::vector<int> moved;

    // ---- pair potentials ------------------------------------------------
    // EwaldReal::operator() live branch, ewald.h:97-110
    double ewald_real(const Particle &a, const Particle &b, double r2) const {
        if (r2 > rc2) return 0.0;
        double r1 = std::sqrt(r2);
        return a.q * b.q *
               (std::erfc(alpha * r1 + kappa / 2.0 / alpha) * std::exp(kappa * r1) +
                std::erfc(alpha * r1 - kappa / 2.0 / alpha) * std::exp(-kappa * r1)) /
               (2.0 * r1) * qeqe[a.id * nt + b.id] * lB;
    }
    // WeeksChandlerAndersen::operator(), potentials.h:2186-2193
    double wca(const Particle &a, const Particle &b, double r2) const {
        double x = s2[a.id * nt + b.id];
        if (r2 > x * std::pow(2, 2 / 6.)) return 0;
        x = x / r2;
        x = x * x * x;
        return eps4[a.id * nt + b.id] * (x * x - x + 1 / 4.);
    }
    // DebyeHuckel::operator(), potentials.h:3314-3323
    double dh(const Particle &a, const Particle &b, double r2) const {
        double r = std::sqrt(r2);
        return lB * a.q * b.q / r * std::exp(-k_dh * r);
    }
    // LennardJonesMixed::operator(), potentials.h:2036-2040
    double lj(const Particle &a, const Particle &b, double r2) const {
        double x = s2[a.id * nt + b.id] / r2;
        x = x * x * x;
        return eps4[a.id * nt + b.id] * (x * x - x);
    }
    // i2i: NonbondedVector::i2i (energy.h:1119-1122) for Ewald, Nonbonded::i2i
    // (energy.h:842-845) for DH+LJ; CombinedPairPotential sums first+second
    // (potentials.h:3768-3771).
    double pair(const Particle &a, const Particle &b) const {
        if (P.model == FG_MODEL_EWALD_WCA) {
            V3 r = geo.vdist(a.r, b.r);
            double r2 = r.x * r.x + r.y * r.y + r.z * r.z;
            return ewald_real(a, b, r2) + wca(a, b, r2);
        }
        double r2 = geo.sqdist(a.r, b.r);
        return dh(a, b, r2) + lj(a, b, r2);
    }

    // ---- Ewald reciprocal space -----------------------------------------
    // kVectorChange (ewald.h:330-378); isotropic_pbc (ewald.h:347-360): n_y and
    // n_z from 0 and a factor 2 for each positive component
    void kvectors() {
        const bool iso = P.ewald_isotropic_pbc != 0;
        const int start = iso ? 0 : 1;
        double kc = P.ewald_cutoff_k, kc2 = kc * kc;
        int kcc = (int)std::ceil(kc);
        double maxL = std::max(P.box[0], std::max(P.box[1], P.box[2]));
        double check_k2_zero = 0.1 * (4 * PI * PI) / (maxL * maxL);  // ewald.h:162
        kv.clear(); Ak.clear();
        for (int kx = 0; kx <= kcc; kx++) {
            double dkx2 = double(kx * kx);
            for (int ky = -kcc * start; ky <= kcc; ky++) {
                double dky2 = double(ky * ky);
                for (int kz = -kcc * start; kz <= kcc; kz++) {
                    double factor = 1.0;
                    if (kx > 0) factor = 2.0;
                    if (ky > 0 && iso) factor = 2.0 * factor;
                    if (kz > 0 && iso) factor = 2.0 * factor;
                    double dkz2 = double(kz * kz);
                    V3 k = {2 * PI * (kx / P.box[0]), 2 * PI * (ky / P.box[1]), 2 * PI * (kz / P.box[2])};
                    double k2 = k.x * k.x + k.y * k.y + k.z * k.z;
                    if (k2 < check_k2_zero) continue;
                    if (P.ewald_spherical_sum)
                        if ((dkx2 / kc2) + (dky2 / kc2) + (dkz2 / kc2) > 1.0) continue;
                    kv.push_back(k);
                    Ak.push_back(factor * std::exp(-(k2 + kappa * kappa) / (4.0 * alpha2)) / (k2 + kappa * kappa));
                }
            }
        }
        K = (int)kv.size();
        Q.assign(K, 0.0);
        Qt.assign(K, 0.0);
    }
    // one particle's ion term of Q(k): q e^{ik.r} eff, or with isotropic_pbc
    // the real q cos(k_x x) cos(k_y y) cos(k_z z) eff (ewald.h:394-399, 669-675)
    std::complex<double> qk_term(const Particle &a, int k) const {
        if (P.ewald_isotropic_pbc)
            return a.q * std::cos(kv[k].x * a.r.x) * std::cos(kv[k].y * a.r.y) * std::cos(kv[k].z * a.r.z) * eff[a.id];
        double dot = kv[k].x * a.r.x + kv[k].y * a.r.y + kv[k].z * a.r.z;
        return a.q * std::complex<double>(std::cos(dot), std::sin(dot)) * eff[a.id];
    }
    // updateAllComplexNumbers (ewald.h:388-415), ion part
    void rebuild(const std::vector<Particle> &pv, std::vector<std::complex<double>> &q) const {
        for (int k = 0; k < K; k++) {
            std::complex<double> s(0.0, 0.0);
            for (int i = 0; i < N; i++) s += qk_term(pv[i], k);
            q[k] = s;
        }
    }
    // getReciprocalEnergy (ewald.h:298-311)
    double recip_energy(const std::vector<std::complex<double>> &q) const {
        double E = 0.0;
        for (int k = 0; k < K; k++) E += Ak[k] * std::norm(q[k]);
        return (2 * PI / V) * E * lB;
    }
    // getSurfaceEnergy (ewald.h:277-291), ion part
    double surface_energy(const std::vector<Particle> &pv) const {
        if (const_inf < 0.5) return 0.0;
        double qx = 0, qy = 0, qz = 0;
        for (int i = 0; i < N; i++) {
            double s = pv[i].q * eff[pv[i].id];
            qx = qx + s * pv[i].r.x; qy = qy + s * pv[i].r.y; qz = qz + s * pv[i].r.z;
        }
        return const_inf * (2 * PI / ((2 * P.ewald_eps_surf + 1) * V)) * (qx * qx + qy * qy + qz * qz) * lB;
    }
    // getSelfEnergy (ewald.h:259-270), ion part
    double self_energy(const std::vector<Particle> &pv) const {
        double Eq = 0;
        for (int i = 0; i < N; i++) Eq += pv[i].q * pv[i].q * eff[pv[i].id] * eff[pv[i].id];
        return (-alpha * (Eq) / std::sqrt(PI)) * lB;
    }
    // updateChange (ewald.h:651-705), fixed volume, ion branch
    void update_change() {
        for (int k = 0; k < K; k++) {
            std::complex<double> q2 = Q[k];
            for (int i : moved) {
                q2 += qk_term(trial[i], k);
                q2 -= qk_term(p[i], k);
            }
            Qt[k] = q2;
        }
    }
    // external (ewald.h:716-729)
    double external(bool is_trial) {
        if (P.model != FG_MODEL_EWALD_WCA) return 0.0;
        if (is_trial) {
            surf_t = surface_energy(trial);
            recip_t = recip_energy(Qt);
            return surf_t + recip_t;
        }
        surf = surface_energy(p);
        recip = recip_energy(Q);
        return surf + recip;
    }

    // energyChangeConfiguration for one atomic group (energy.h:3521-3572):
    // g2All (self g2g = 0) + external + g_external(group) + sum of i2i
    double configuration(bool is_trial) {
        const std::vector<Particle> &pv = is_trial ? trial : p;
        double du = 0;
        du += 0.0;  // g2All: the moved group against itself only
        du += external(is_trial);
        if (P.model == FG_MODEL_EWALD_WCA) du += self_energy(pv);  // g_external, ewald.h:712-714
        for (size_t a = 0; a < moved.size(); a++) {
            int j = moved[a];
            for (int k = 0; k < N; k++) {
                bool k_moved = false;
                for (int m : moved) if (m == k) k_moved = true;
                if (!k_moved || j > k) du += pair(pv[j], pv[k]);
            }
        }
        return du;
    }

    void init(const fg_params *prm) {
        P = *prm;
        geo.set(P.box);
        nt = P.n_types;
        lB = P.bjerrum;
        s2.assign(nt * nt, 0); eps4.assign(nt * nt, 0); qeqe.assign(nt * nt, 0); eff.assign(nt, 0);
        if (P.model == FG_MODEL_EWALD_WCA) {
            alpha = P.ewald_alpha; alpha2 = alpha * alpha;
            rc2 = P.ewald_cutoff * P.ewald_cutoff;
            kappa = 1.0 / P.ewald_debye_length;
            const_inf = (P.ewald_eps_surf < 1) ? 0.0 : 1.0;
        } else {
            k_dh = 1.0 / P.dh_debye_length;
        }
        // LorentzBerthelot mixing with eps stored x4 (potentials.h:2003-2023, 1816-1829)
        for (int i = 0; i < nt; i++)
            for (int j = 0; j < nt; j++) {
                double sig = 0.5 * (P.type_sigma[i] + P.type_sigma[j]);
                s2[i * nt + j] = sig * sig;
                eps4[i * nt + j] = 4 * std::sqrt(P.type_eps[i] * P.type_eps[j]);
            }
        // effective charges (ewald.h:532-549)
        for (int i = 0; i < nt; i++) {
            double ri = 0.5 * P.type_sigma[i];
            double qis = P.type_charge[i];
            if (std::fabs(kappa * ri) > 1e-9) qis *= std::sinh(ri * kappa) / ri / kappa;
            eff[i] = qis / P.type_charge[i];
            for (int j = 0; j < nt; j++) {
                double rj = 0.5 * P.type_sigma[j];
                double qjs = P.type_charge[j];
                if (std::fabs(kappa * rj) > 1e-9) qjs *= std::sinh(rj * kappa) / rj / kappa;
                qeqe[i * nt + j] = qis * qjs / P.type_charge[i] / P.type_charge[j];
            }
        }
        V = geo.volume();
        if (P.model == FG_MODEL_EWALD_WCA) kvectors();
    }

    void set_state(const double *xyz, const double *q, const int32_t *ids, int n) {
        N = n;
        p.resize(N);
        for (int i = 0; i < N; i++) {
            p[i].r = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
            p[i].id = ids[i];
            p[i].q = q ? q[i] : P.type_charge[ids[i]];
        }
        trial = p;
        if (P.model == FG_MODEL_EWALD_WCA) {
            // setSpace -> setGeometry -> updateAllComplexNumbers (ewald.h:731-756)
            rebuild(p, Q);
            Qt = Q;
            surf = surface_energy(p);
            recip = recip_energy(Q);
            surf_t = surf; recip_t = recip;
        }
        cnt_accepted = 0;
        update_drift = 0;
    }

    // Energy::energyChange (energy.h:3577-3621) after updateChange (move.h:534)
    double trial_du(int n, const int *idx, const double *xyz) {
        moved.assign(idx, idx + n);
        for (int a = 0; a < n; a++) trial[idx[a]].r = {xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]};
        if (P.model == FG_MODEL_EWALD_WCA) update_change();
        double duNew = configuration(true);
        double duOld = configuration(false);
        return duNew - duOld;
    }

    // acceptMove/rejectMove (move.h:866-889) + NonbondedEwald::update (ewald.h:613-646)
    double commit(bool accepted) {
        double ret = 0.0;
        if (!accepted) {
            for (int i : moved) trial[i] = p[i];
            if (P.model == FG_MODEL_EWALD_WCA) { Qt = Q; surf_t = surf; recip_t = recip; }
        } else {
            if (P.model == FG_MODEL_EWALD_WCA) {
                int uf = P.ewald_update_frequency;
                if (++cnt_accepted > uf - 1) {
                    double duB = recip_energy(Qt);
                    rebuild(trial, Qt);
                    double duA = recip_energy(Qt);
                    cnt_accepted = 0;
                    update_drift += std::fabs(duA - duB);
                    ret = duA - duB;
                }
                Q = Qt; surf = surf_t; recip = recip_t;
            }
            for (int i : moved) p[i] = trial[i];
        }
        moved.clear();
        return ret;
    }

    // Energybase::systemEnergy (energy.h:169-180) for one atomic group:
    // external + g_external + g_internal (all i<j pairs)
    void total_energy(double *comp) {
        double pairs = 0;
        for (int i = 0; i < N - 1; i++)
            for (int j = i + 1; j < N; j++) pairs += pair(p[i], p[j]);
        double rec = 0, sf = 0, sl = 0;
        if (P.model == FG_MODEL_EWALD_WCA) {
            rec = recip_energy(Q);
            sf = surface_energy(p);
            sl = self_energy(p);
        }
        comp[0] = pairs; comp[1] = rec; comp[2] = sl; comp[3] = sf;
        comp[4] = (sf + rec) + (sl + pairs);
    }
};

}  // namespace

// ==================================================================== C ABI
extern "C" {

void *or_create(const fg_params *p) {
    try {
        System *s = new System();
        s->init(p);
        return s;
    } catch (...) { return nullptr; }
}

void or_destroy(void *h) { delete (System *)h; }

int or_num_kvectors(void *h) { return ((System *)h)->K; }

int or_set_state(void *h, int n, const double *xyz, const double *q, const int32_t *ids) {
    ((System *)h)->set_state(xyz, q, ids, n);
    return 0;
}

int or_get_positions(void *h, double *xyz) {
    System *s = (System *)h;
    for (int i = 0; i < s->N; i++) {
        xyz[3 * i] = s->p[i].r.x; xyz[3 * i + 1] = s->p[i].r.y; xyz[3 * i + 2] = s->p[i].r.z;
    }
    return 0;
}

// Q(k) as interleaved (re, im); kvec as (kx,ky,kz); Ak.
int or_get_qk(void *h, double *qk, double *kvec, double *ak) {
    System *s = (System *)h;
    for (int k = 0; k < s->K; k++) {
        if (qk) { qk[2 * k] = s->Q[k].real(); qk[2 * k + 1] = s->Q[k].imag(); }
        if (kvec) { kvec[3 * k] = s->kv[k].x; kvec[3 * k + 1] = s->kv[k].y; kvec[3 * k + 2] = s->kv[k].z; }
        if (ak) ak[k] = s->Ak[k];
    }
    return 0;
}

double or_pair_energy(void *h, int i, int j) {
    System *s = (System *)h;
    return s->pair(s->p[i], s->p[j]);
}

// dU for moving particles idx[0..n) to xyz (already wrapped into the box).
double or_trial_du(void *h, int n, const int *idx, const double *xyz) {
    return ((System *)h)->trial_du(n, idx, xyz);
}

// Returns the Ewald rebuild correction (duA - duB) like NonbondedEwald::update.
double or_commit(void *h, int accepted) { return ((System *)h)->commit(accepted != 0); }

// comp = {pairs, reciprocal, self, surface, total}
int or_total_energy(void *h, double *comp) {
    ((System *)h)->total_energy(comp);
    return 0;
}

// Cuboid::boundary applied to a point in place.
void or_boundary(void *h, double *xyz) {
    System *s = (System *)h;
    V3 a = {xyz[0], xyz[1], xyz[2]};
    s->geo.boundary(a);
    xyz[0] = a.x; xyz[1] = a.y; xyz[2] = a.z;
}

// Draws the per-trial random stream of AtomicTranslation on one atomic group
// holding all particles, exactly as the reference consumes the global
// `slump` (move.h:818-864, group.h:129-134, move.h:567-573):
//   range(0, n_groups-1); range(0, N-1); 3 uniforms (x,y,z); 1 uniform (Metropolis).
// Outputs per trial: particle index, displacement (dp*(u-0.5) per axis), u_metropolis.
// The global slump() sequence (slump.h:62-95) for host-driven moves.
int or_uniforms(uint32_t seed, int64_t n, double *u) {
    Twister t(seed);
    for (int64_t i = 0; i < n; i++) u[i] = t();
    return 0;
}

int or_draw_translation_stream(uint32_t seed, int n_particles, const double *dp_per_particle,
                               int64_t n_trials, int32_t *idx, double *disp, double *umet) {
    Twister t(seed);
    for (int64_t n = 0; n < n_trials; n++) {
        t.range(0, 0);
        int i = t.range(0, n_particles - 1);
        double dp = dp_per_particle[i];
        double tx = dp, ty = dp, tz = dp;
        tx *= t() - 0.5;
        ty *= t() - 0.5;
        tz *= t() - 0.5;
        idx[n] = i;
        disp[3 * n] = tx; disp[3 * n + 1] = ty; disp[3 * n + 2] = tz;
        umet[n] = t();
    }
    return 0;
}

// The random streams of the reference's parallel tempering run as every
// rank sees them (all ranks seed the global slump alike, so they draw the
// same sequence; move.h:558-566 relies on it): per round, trials_per_round
// AtomicTranslation trials as or_draw_translation_stream draws them, then
// the one uniform ParallelTempering's Metropolis test takes from the global
// slump (move.h:567-573; drawn on every rank, with or without a partner),
// and the uniform findPartner takes from the MPI controller's own generator
// (default-seeded RandomTwister, move.h:6621-6633).
int or_pt_streams(uint32_t seed, int n_particles, const double *dp_per_particle, int64_t trials_per_round,
                  int rounds, int32_t *idx, double *disp, double *umet, double *u_accept, double *u_direction) {
    Twister t(seed), mpi(5489u);
    int64_t n = 0;
    for (int r = 0; r < rounds; r++) {
        for (int64_t k = 0; k < trials_per_round; k++, n++) {
            t.range(0, 0);
            int i = t.range(0, n_particles - 1);
            double dp = dp_per_particle[i];
            double tx = dp, ty = dp, tz = dp;
            tx *= t() - 0.5;
            ty *= t() - 0.5;
            tz *= t() - 0.5;
            idx[n] = i;
            disp[3 * n] = tx; disp[3 * n + 1] = ty; disp[3 * n + 2] = tz;
            umet[n] = t();
        }
        u_accept[r] = t();
        u_direction[r] = mpi();
    }
    return 0;
}

// Full Metropolis run (Movebase::move, move.h:515-555, with AtomicTranslation
// "peratom" on the single atomic group): n_trials trials from the global RNG
// seeded with `seed`. Optional per-trial logs (any may be NULL). Returns the
// sum of accepted dU plus Ewald rebuild corrections (Movebase's utot).
double or_mc_run(void *h, uint32_t seed, int64_t n_trials, int32_t *idx_out, double *trial_xyz_out,
                 double *du_out, uint8_t *acc_out) {
    System *s = (System *)h;
    Twister t(seed);
    double utot = 0;
    for (int64_t n = 0; n < n_trials; n++) {
        t.range(0, 0);                       // slump.element(gvec) (move.h:822)
        int i = t.range(0, s->N - 1);        // Group::random (group.h:129-134)
        double dp = s->P.type_dp[s->p[i].id];
        V3 tr = {dp, dp, dp};                // dir * dp, dir = (1,1,1)
        tr.x *= t() - 0.5;
        tr.y *= t() - 0.5;
        tr.z *= t() - 0.5;
        V3 r = s->p[i].r;                    // translate: += t, then boundary
        r.x += tr.x; r.y += tr.y; r.z += tr.z;
        s->geo.boundary(r);
        double xyz[3] = {r.x, r.y, r.z};
        double du = s->trial_du(1, &i, xyz);
        bool accept = !(t() > std::exp(-du));   // Movebase::metropolis
        if (accept) utot += du;
        utot += s->commit(accept);
        if (idx_out) idx_out[n] = i;
        if (trial_xyz_out) { trial_xyz_out[3 * n] = r.x; trial_xyz_out[3 * n + 1] = r.y; trial_xyz_out[3 * n + 2] = r.z; }
        if (du_out) du_out[n] = du;
        if (acc_out) acc_out[n] = accept ? 1 : 0;
    }
    return utot;
}

// Same loop as or_mc_run but from an explicit trial stream (particle index,
// displacement, Metropolis uniform per trial), e.g. one drawn on the device.
double or_mc_run_stream(void *h, int64_t n_trials, const int32_t *idx, const double *disp, const double *u,
                        double *du_out, uint8_t *acc_out) {
    System *s = (System *)h;
    double utot = 0;
    for (int64_t n = 0; n < n_trials; n++) {
        int i = idx[n];
        V3 r = s->p[i].r;
        r.x += disp[3 * n]; r.y += disp[3 * n + 1]; r.z += disp[3 * n + 2];
        s->geo.boundary(r);
        double xyz[3] = {r.x, r.y, r.z};
        double du = s->trial_du(1, &i, xyz);
        double kT = s->P.kT_scale > 0 ? s->P.kT_scale : 1.0;
        bool accept = !(u[n] > std::exp(-du / kT));
        if (accept) utot += du;
        utot += s->commit(accept);
        if (du_out) du_out[n] = du;
        if (acc_out) acc_out[n] = accept ? 1 : 0;
    }
    return utot;
}

// ---------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon et al., SC'11): the counter-based generator the GPU
// library uses for device-generated trial streams, restated here so those
// streams can be regenerated and checked on the host.
static void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1, n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

void or_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    philox(c, key[0], key[1]);
    for (int i = 0; i < 4; i++) out[i] = c[i];
}

// The device trial-stream definition: for trial g (counter), r = philox(g, 0),
// r2 = philox(g, 1) under key (seed, stream): particle floor(r0 N / 2^32),
// displacement_a = (r_a - 2^31) * round(dp_type / L_a * 2^32) in units of
// L_a / 2^64, u = (r2_0 + 0.5) / 2^32.
void or_philox_stream(uint32_t seed, uint32_t stream, int64_t first, int64_t n, int32_t n_particles,
                      const int32_t *types, const double *type_dp, const double *box, int32_t *idx, double *disp,
                      double *u) {
    for (int64_t t = 0; t < n; t++) {
        const int64_t g = first + t;
        uint32_t r[4] = {(uint32_t)g, (uint32_t)(g >> 32), 0u, 0u};
        uint32_t r2[4] = {(uint32_t)g, (uint32_t)(g >> 32), 1u, 0u};
        philox(r, seed, stream);
        philox(r2, seed, stream);
        const int i = (int)(((uint64_t)r[0] * (uint32_t)n_particles) >> 32);
        idx[t] = i;
        for (int a = 0; a < 3; a++) {
            const int64_t dpf = (int64_t)llrint(type_dp[types[i]] / box[a] * 4294967296.0);
            const int64_t dfix = (int64_t)(int32_t)(r[1 + a] - 0x80000000u) * dpf;
            disp[3 * t + a] = (double)dfix * (box[a] / 18446744073709551616.0);
        }
        u[t] = ((double)r2[0] + 0.5) * (1.0 / 4294967296.0);
    }
}

void or_set_kT(void *h, double kT) { ((System *)h)->P.kT_scale = kT; }

}  // extern "C"
