// FP64 oracle for point charges and point dipoles under Ewald summation --
// TEST INFRASTRUCTURE (see fg_oracle.cpp for who may load it).
//
// Restates NonbondedEwald<Tspace, LennardJonesLB, useIonIon, useIonDipole,
// useDipoleDipole> (ewald.h:228-757) on DipoleParticle (point.h:591-680) with
// the two single-particle moves that act on it, AtomicTranslation
// (move.h:838-975) and AtomicRotation (move.h:976-1072).
//
// Two readings of the Ewald sum (fg_params.ewald_dipole_quirk):
//   0  the sum as ewald.h:28-32 and 203-216 state it: real space with the
//      ion-dipole and dipole-dipole terms of EwaldReal (ewald.h:112-128, the
//      T1/T2 functions of ewald.h:45-47 evaluated exactly instead of from
//      splines), reciprocal |Q_ion + Q_dip|^2. Pinned by the Ewald known
//      answers of the reference's unit test (unittests.cpp:131-193, values of
//      doi:10.1063/1.481216), ion-ion and dipole-dipole.
//   1  what the reference's live code computes: EwaldReal::operator() returns
//      after its ion-ion term (ewald.h:109-110), and getReciprocalEnergy takes
//      2 Re(Q_ion Q_dip) for the cross term (ewald.h:304-305). Pinned by
//      per-move logs of the reference itself (tests/golden/dip_*.npz).
#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

#include "../include/fg_params.h"
#include "or_common.h"

namespace {

using namespace orc;
using cplx = std::complex<double>;

struct DParticle {
    V3 r;        // position
    V3 mu;       // dipole unit vector, DipoleParticle::mu()
    double mus;  // dipole scalar, DipoleParticle::muscalar()
    double q;    // charge
    int id;      // atom type
};

double dot(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

struct DipSystem {
    fg_params P;
    Cuboid geo;
    int N = 0, nt = 0, K = 0;
    bool ii = false, id = false, dd = false, quirk = false;
    std::vector<DParticle> p, trial;
    std::vector<double> s2, eps4, qeqe, eff;
    double alpha = 0, alpha2 = 0, rc2 = 0, kappa = 0, lB = 0, V = 0, const_inf = 0;
    std::vector<V3> kv;
    std::vector<double> Ak;
    std::vector<cplx> Qi, Qd, Qit, Qdt;   // Q_ion_tot, Q_dip_tot and their trial copies
    int cnt_accepted = 0;
    double update_drift = 0;
    int moved = -1;

    // ---- real space -------------------------------------------------------
    // EwaldReal (ewald.h:45-47 for T0..T2; 97-129 for the pair)
    double T1f(double r1) const {
        return r1 * 2.0 * alpha / std::sqrt(PI) * std::exp(-alpha2 * r1 * r1) + std::erfc(alpha * r1);
    }
    double T2f(double r1) const {
        return 3.0 * (T1f(r1) + 4.0 * alpha2 * alpha / 3.0 / std::sqrt(PI) * r1 * r1 * r1 * std::exp(-alpha2 * r1 * r1));
    }
    // r = vdist(a, b) = a - b (minimum image)
    double ewald_real(const DParticle &a, const DParticle &b, const V3 &r) const {
        if (!(ii || id || dd)) return 0.0;
        const double r2 = dot(r, r);
        if (r2 > rc2) return 0.0;
        const double r1 = std::sqrt(r2);
        double E = 0.0;
        if (quirk || ii)   // the live line (ewald.h:109) runs whatever the flags
            E += a.q * b.q *
                 (std::erfc(alpha * r1 + kappa / 2.0 / alpha) * std::exp(kappa * r1) +
                  std::erfc(alpha * r1 - kappa / 2.0 / alpha) * std::exp(-kappa * r1)) /
                 (2.0 * r1) * qeqe[a.id * nt + b.id] * lB;
        if (quirk) return E;
        double Ed = 0.0;
        const double T1 = T1f(r1) / r1 / r2;
        if (id) {
            Ed += a.q * dot(r, b.mu) * b.mus * T1;
            Ed -= b.q * dot(r, a.mu) * a.mus * T1;
        }
        if (dd) {
            const double t3 = -dot(b.mu, a.mu) * T1;
            const double t5 = dot(b.mu, r) * dot(a.mu, r) * T2f(r1) / r2 / r2 / r1;
            Ed += -(t5 + t3) * b.mus * a.mus;
        }
        return E + lB * Ed;
    }
    // LennardJonesMixed<LorentzBerthelot> (potentials.h:2036-2040), no cutoff
    double lj(const DParticle &a, const DParticle &b, double r2) const {
        double x = s2[a.id * nt + b.id] / r2;
        x = x * x * x;
        return eps4[a.id * nt + b.id] * (x * x - x);
    }
    // CombinedPairPotential<EwaldReal, LennardJonesLB> (potentials.h:3768-3771)
    double pair(const DParticle &a, const DParticle &b) const {
        const V3 r = geo.vdist(a.r, b.r);
        return ewald_real(a, b, r) + lj(a, b, dot(r, r));
    }

    // ---- reciprocal space ---------------------------------------------------
    // kVectorChange (ewald.h:330-378), non-isotropic branch
    void kvectors() {
        const double kc = P.ewald_cutoff_k, kc2 = kc * kc;
        const int kcc = (int)std::ceil(kc);
        const double maxL = std::max(P.box[0], std::max(P.box[1], P.box[2]));
        const double check_k2_zero = 0.1 * (4 * PI * PI) / (maxL * maxL);
        kv.clear();
        Ak.clear();
        for (int kx = 0; kx <= kcc; kx++)
            for (int ky = -kcc; ky <= kcc; ky++)
                for (int kz = -kcc; kz <= kcc; kz++) {
                    const double factor = kx > 0 ? 2.0 : 1.0;
                    const V3 k = {2 * PI * (kx / P.box[0]), 2 * PI * (ky / P.box[1]), 2 * PI * (kz / P.box[2])};
                    const double k2 = dot(k, k);
                    if (k2 < check_k2_zero) continue;
                    if (P.ewald_spherical_sum && (double(kx * kx) / kc2 + double(ky * ky) / kc2 + double(kz * kz) / kc2 > 1.0))
                        continue;
                    kv.push_back(k);
                    Ak.push_back(factor * std::exp(-(k2 + kappa * kappa) / (4.0 * alpha2)) / (k2 + kappa * kappa));
                }
        K = (int)kv.size();
    }
    // one particle's contributions to Q_ion and Q_dip (ewald.h:392-403, 665-680)
    void contrib(const DParticle &a, const V3 &k, cplx &ci, cplx &cd) const {
        const double d = dot(k, a.r);
        const cplx e(std::cos(d), std::sin(d));
        ci = a.q * e * eff[a.id];
        cd = dot(k, a.mu) * a.mus * cplx(-std::sin(d), std::cos(d));
    }
    bool ion_q() const { return ii || id; }
    // updateAllComplexNumbers (ewald.h:388-415): Q_dip is built there only
    // with useDipoleDipole; the physical reading keeps it for ion-dipole too
    bool dip_q_rebuild() const { return quirk ? dd : (dd || id); }
    void rebuild(const std::vector<DParticle> &pv, std::vector<cplx> &qi, std::vector<cplx> &qd) const {
        qi.assign(K, 0.0);
        qd.assign(K, 0.0);
        for (int k = 0; k < K; k++) {
            cplx si(0, 0), sd(0, 0);
            for (int i = 0; i < N; i++) {
                cplx ci, cd;
                contrib(pv[i], kv[k], ci, cd);
                if (ion_q()) si += ci;
                if (dip_q_rebuild()) sd += cd;
            }
            qi[k] = si;
            qd[k] = sd;
        }
    }
    // getReciprocalEnergy (ewald.h:298-311)
    double recip_energy(const std::vector<cplx> &qi, const std::vector<cplx> &qd) const {
        double E = 0.0;
        for (int k = 0; k < K; k++) {
            double Q2 = 0.0;
            if (ii) Q2 += std::norm(qi[k]);
            if (id) Q2 += 2.0 * std::real(quirk ? qi[k] * qd[k] : qi[k] * std::conj(qd[k]));
            if (dd) Q2 += std::norm(qd[k]);
            E += Ak[k] * Q2;
        }
        return (2 * PI / V) * E * lB;
    }
    // getSurfaceEnergy (ewald.h:277-291)
    double surface_energy(const std::vector<DParticle> &pv) const {
        if (const_inf < 0.5) return 0.0;
        V3 qrs = {0, 0, 0}, mus = {0, 0, 0};
        for (int i = 0; i < N; i++) {
            if (ion_q()) {
                const double s = pv[i].q * eff[pv[i].id];
                qrs = {qrs.x + s * pv[i].r.x, qrs.y + s * pv[i].r.y, qrs.z + s * pv[i].r.z};
            }
            if (id || dd) mus = {mus.x + pv[i].mu.x * pv[i].mus, mus.y + pv[i].mu.y * pv[i].mus, mus.z + pv[i].mu.z * pv[i].mus};
        }
        return const_inf * (2 * PI / ((2 * P.ewald_eps_surf + 1) * V)) * (dot(qrs, qrs) + 2 * dot(qrs, mus) + dot(mus, mus)) * lB;
    }
    // getSelfEnergy (ewald.h:259-270)
    double self_energy(const std::vector<DParticle> &pv) const {
        double Eq = 0, Emu = 0;
        for (int i = 0; i < N; i++) {
            if (ion_q()) Eq += pv[i].q * pv[i].q * eff[pv[i].id] * eff[pv[i].id];
            if (id || dd) Emu += pv[i].mus * pv[i].mus;
        }
        return (-alpha * (Eq + alpha2 * (2.0 / 3.0) * Emu) / std::sqrt(PI)) * lB;
    }
    // updateChange (ewald.h:651-705), fixed volume, non-isotropic branch
    void update_change() {
        Qit = Qi;
        Qdt = Qd;
        for (int k = 0; k < K; k++) {
            cplx ni, nd, oi, od;
            contrib(trial[moved], kv[k], ni, nd);
            contrib(p[moved], kv[k], oi, od);
            if (ion_q()) Qit[k] += ni - oi;
            if (dd || id) Qdt[k] += nd - od;
        }
    }
    // energyChangeConfiguration for one atomic group (energy.h:3521-3572)
    double configuration(bool is_trial) const {
        const std::vector<DParticle> &pv = is_trial ? trial : p;
        double du = surface_energy(pv) + recip_energy(is_trial ? Qit : Qi, is_trial ? Qdt : Qd);
        du += self_energy(pv);
        for (int k = 0; k < N; k++)
            if (k != moved) du += pair(pv[moved], pv[k]);
        return du;
    }

    void init(const fg_params *prm) {
        P = *prm;
        geo.set(P.box);
        nt = P.n_types;
        lB = P.bjerrum;
        ii = P.ewald_terms & FG_EWALD_ION_ION;
        id = P.ewald_terms & FG_EWALD_ION_DIPOLE;
        dd = P.ewald_terms & FG_EWALD_DIPOLE_DIPOLE;
        quirk = P.ewald_dipole_quirk != 0;
        alpha = P.ewald_alpha;
        alpha2 = alpha * alpha;
        rc2 = P.ewald_cutoff * P.ewald_cutoff;
        kappa = 1.0 / P.ewald_debye_length;
        const_inf = (P.ewald_eps_surf < 1) ? 0.0 : 1.0;
        s2.assign(nt * nt, 0);
        eps4.assign(nt * nt, 0);
        qeqe.assign(nt * nt, 0);
        eff.assign(nt, 0);
        for (int i = 0; i < nt; i++)
            for (int j = 0; j < nt; j++) {
                const double sig = 0.5 * (P.type_sigma[i] + P.type_sigma[j]);
                s2[i * nt + j] = sig * sig;
                eps4[i * nt + j] = 4 * std::sqrt(P.type_eps[i] * P.type_eps[j]);
            }
        // effective charges (ewald.h:532-549); a type without charge has none
        // (the reference divides 0 by 0 there and never uses the result when
        // no ion term is on)
        auto qs = [&](int t) {
            const double r = 0.5 * P.type_sigma[t];
            double q = P.type_charge[t];
            if (std::fabs(kappa * r) > 1e-9) q *= std::sinh(r * kappa) / r / kappa;
            return q;
        };
        for (int i = 0; i < nt; i++) {
            eff[i] = P.type_charge[i] != 0.0 ? qs(i) / P.type_charge[i] : 0.0;
            for (int j = 0; j < nt; j++)
                qeqe[i * nt + j] = (P.type_charge[i] != 0.0 && P.type_charge[j] != 0.0)
                                       ? qs(i) * qs(j) / P.type_charge[i] / P.type_charge[j] : 0.0;
        }
        V = geo.volume();
        kvectors();
    }

    void set_state(int n, const double *xyz, const double *mu, const double *mus, const double *q, const int32_t *ids) {
        N = n;
        p.resize(N);
        for (int i = 0; i < N; i++) {
            p[i].r = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
            p[i].mu = {mu[3 * i], mu[3 * i + 1], mu[3 * i + 2]};
            p[i].mus = mus[i];
            p[i].id = ids[i];
            p[i].q = q ? q[i] : P.type_charge[ids[i]];
        }
        trial = p;
        rebuild(p, Qi, Qd);   // setSpace -> setGeometry (ewald.h:731-756)
        Qit = Qi;
        Qdt = Qd;
        cnt_accepted = 0;
        update_drift = 0;
        moved = -1;
    }

    // Energy::energyChange (energy.h:3577-3621) for one moved particle
    double trial_du(int i, const double *xyz, const double *mu) {
        moved = i;
        trial[i].r = {xyz[0], xyz[1], xyz[2]};
        if (mu) trial[i].mu = {mu[0], mu[1], mu[2]};
        update_change();
        return configuration(true) - configuration(false);
    }

    // acceptMove/rejectMove + NonbondedEwald::update (ewald.h:613-646)
    double commit(bool accepted) {
        double ret = 0.0;
        if (moved < 0) return 0.0;
        if (!accepted) {
            trial[moved] = p[moved];
        } else {
            if (++cnt_accepted > P.ewald_update_frequency - 1) {
                const double duB = recip_energy(Qit, Qdt);
                rebuild(trial, Qit, Qdt);
                const double duA = recip_energy(Qit, Qdt);
                cnt_accepted = 0;
                update_drift += std::fabs(duA - duB);
                ret = duA - duB;
            }
            Qi = Qit;
            Qd = Qdt;
            p[moved] = trial[moved];
        }
        moved = -1;
        return ret;
    }

    // systemEnergy for one atomic group: {real pairs (EwaldReal), LJ,
    // reciprocal, self, surface, total}
    void total_energy(double *c) const {
        double er = 0, el = 0;
        for (int i = 0; i < N - 1; i++)
            for (int j = i + 1; j < N; j++) {
                const V3 r = geo.vdist(p[i].r, p[j].r);
                er += ewald_real(p[i], p[j], r);
                el += lj(p[i], p[j], dot(r, r));
            }
        c[0] = er;
        c[1] = el;
        c[2] = recip_energy(Qi, Qd);
        c[3] = self_energy(p);
        c[4] = surface_energy(p);
        c[5] = er + el + c[2] + c[3] + c[4];
    }
};

// Eigen's quaternion-vector product for AngleAxisd(angle, u) (the rotation
// of QuaternionRotate::setAxis, geometry.cpp:753-766, applied to mu by
// DipoleParticle::rotate, point.h:671-679)
V3 rotate(const V3 &axis, double angle, const V3 &p) {
    const double n = std::sqrt(dot(axis, axis));
    const double s = std::sin(0.5 * angle);
    const V3 v = {s * axis.x / n, s * axis.y / n, s * axis.z / n};
    const double w = std::cos(0.5 * angle);
    auto cross = [](const V3 &a, const V3 &b) {
        return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    };
    V3 uv = cross(v, p);
    uv = {uv.x + uv.x, uv.y + uv.y, uv.z + uv.z};
    const V3 c = cross(v, uv);
    return {p.x + w * uv.x + c.x, p.y + w * uv.y + c.y, p.z + w * uv.z + c.z};
}

}  // namespace

extern "C" {

void *or_dip_create(const fg_params *p) {
    try {
        DipSystem *s = new DipSystem();
        s->init(p);
        return s;
    } catch (...) { return nullptr; }
}

void or_dip_destroy(void *h) { delete (DipSystem *)h; }

int or_dip_num_kvectors(void *h) { return ((DipSystem *)h)->K; }

int or_dip_set_state(void *h, int n, const double *xyz, const double *mu, const double *mus, const double *q,
                     const int32_t *ids) {
    ((DipSystem *)h)->set_state(n, xyz, mu, mus, q, ids);
    return 0;
}

int or_dip_get_state(void *h, double *xyz, double *mu) {
    DipSystem *s = (DipSystem *)h;
    for (int i = 0; i < s->N; i++) {
        const DParticle &a = s->p[i];
        if (xyz) { xyz[3 * i] = a.r.x; xyz[3 * i + 1] = a.r.y; xyz[3 * i + 2] = a.r.z; }
        if (mu) { mu[3 * i] = a.mu.x; mu[3 * i + 1] = a.mu.y; mu[3 * i + 2] = a.mu.z; }
    }
    return 0;
}

// the pair energy EwaldReal + LJ of particles i and j; real_only drops LJ
double or_dip_pair(void *h, int i, int j, int real_only) {
    DipSystem *s = (DipSystem *)h;
    const V3 r = s->geo.vdist(s->p[i].r, s->p[j].r);
    return real_only ? s->ewald_real(s->p[i], s->p[j], r) : s->pair(s->p[i], s->p[j]);
}

double or_dip_trial_du(void *h, int i, const double *xyz, const double *mu) {
    return ((DipSystem *)h)->trial_du(i, xyz, mu);
}

double or_dip_commit(void *h, int accepted) { return ((DipSystem *)h)->commit(accepted != 0); }

int or_dip_total_energy(void *h, double *c) {
    ((DipSystem *)h)->total_energy(c);
    return 0;
}

// Metropolis over an explicit stream of single-particle moves: kind[t] 1 =
// AtomicRotation (axis[t], angle[t]), 2 = AtomicTranslation (disp[t]);
// reject iff u[t] > exp(-dU) (Movebase::metropolis, move.h:567-573).
// Returns the sum of accepted dU.
double or_dip_run_stream(void *h, int64_t n, const int32_t *kind, const int32_t *idx, const double *axis,
                         const double *angle, const double *disp, const double *u, double *du, uint8_t *acc) {
    DipSystem *s = (DipSystem *)h;
    double sum = 0.0;
    const double kT = s->P.kT_scale > 0 ? s->P.kT_scale : 1.0;
    for (int64_t t = 0; t < n; t++) {
        const int i = idx[t];
        DParticle a = s->p[i];
        if (kind[t] == 1) {
            a.mu = rotate({axis[3 * t], axis[3 * t + 1], axis[3 * t + 2]}, angle[t], a.mu);
        } else {
            a.r = {a.r.x + disp[3 * t], a.r.y + disp[3 * t + 1], a.r.z + disp[3 * t + 2]};
            s->geo.boundary(a.r);
        }
        const double xyz[3] = {a.r.x, a.r.y, a.r.z}, mu[3] = {a.mu.x, a.mu.y, a.mu.z};
        const double d = s->trial_du(i, xyz, mu);
        const bool ok = !(u[t] > std::exp(-d / kT));
        s->commit(ok);
        if (ok) sum += d;
        if (du) du[t] = d;
        if (acc) acc[t] = ok ? 1 : 0;
    }
    return sum;
}

// The draws of n single-particle moves on one atomic group of n_particles:
// per trial one uniform picks the move (rotation when below p_rotate), then
// the move's own draws as the reference takes them from slump:
// AtomicRotation (move.h:1008-1032): group, particle, ranunit axis (point.h:74-88),
// angle dprot * half(); AtomicTranslation (move.h:820-850): group, particle, three
// dp * half(); then the Metropolis uniform.
// With p_rotate < 0 the kinds are the caller's (kind[] is read, no uniform
// is drawn for them).
int or_dip_draw_stream(uint32_t seed, int32_t n_particles, int64_t n, double p_rotate, double dp, double dprot,
                       int32_t *kind, int32_t *idx, double *axis, double *angle, double *disp, double *u) {
    Twister rng(seed);
    for (int64_t t = 0; t < n; t++) {
        const bool rot = p_rotate < 0 ? kind[t] == 1 : rng() < p_rotate;
        kind[t] = rot ? 1 : 2;
        rng.range(0, 0);                        // randomMol / slump.element over the one group
        idx[t] = rng.range(0, n_particles - 1); // Group::random (group.h:129-134)
        double v[3] = {0, 0, 0}, an = 0, d[3] = {0, 0, 0};
        if (rot) {
            double r2;
            do {
                for (int a = 0; a < 3; a++) v[a] = 2 * rng() - 1;
                r2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
            } while (r2 > 1);
            const double s = std::sqrt(r2);
            for (int a = 0; a < 3; a++) v[a] /= s;
            an = dprot * (rng() - 0.5);
        } else {
            for (int a = 0; a < 3; a++) d[a] = dp * (rng() - 0.5);
        }
        u[t] = rng();
        for (int a = 0; a < 3; a++) {
            axis[3 * t + a] = v[a];
            disp[3 * t + a] = d[a];
        }
        angle[t] = an;
    }
    return 0;
}

}  // extern "C"
