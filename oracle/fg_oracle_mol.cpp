// FP64 CPU oracle, rigid dipolar molecules -- TEST INFRASTRUCTURE.
//
// A plain double-precision restatement of the reference's rigid-group path:
// Space<Cuboid, DipoleParticle> with molecular groups, the vector-distance
// energy NonbondedVector (energy.h:1062-1196) over the pair potential
//     CoulombGalore        (multipole.h:569-598, the live operator)
//   + LennardJonesLB       (potentials.h:2036-2040, 3891)
//   + IonDipole            (multipole.h:993-996 -> q2mu 269-277)
//   + DipoleDipoleGalore   (multipole.h:910-920 -> mu2mu 287-299, reaction
//                           field splitting 767-782)
// summed as CombinedPairPotential (potentials.h:3768-3771), and the
// TranslateRotate move (move.h:1620-1705) with Group::newrotate/translate
// (group.h:186-193, 259-277), QuaternionRotate (geometry.h:95-147,
// geometry.cpp:753-766) and Point::ranunit (point.h:74-88).
//
// Only tests/ and the benchmarks' CPU leg load it; the product never does.
// Pinned by per-trial logs of the reference itself (oracle/ref/
// ref_harness_mol.cpp, fixtures under tests/golden/).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/fg_params.h"
#include "or_common.h"

namespace {

using namespace orc;

struct Site {
    V3 r;       // position
    V3 mu;      // dipole unit vector (DipoleParticle::mu)
    double mus; // dipole scalar (DipoleParticle::muscalar), e*Angstrom
    double q;   // particle charge
    int id;     // atom type
};

double dot(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(const V3 &a, const V3 &b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

// Eigen::Quaterniond built from AngleAxisd (w = cos(a/2), v = sin(a/2) u)
// applied to a vector as Eigen's _transformVector does:
//   uv = v x p; uv += uv; p' = p + w uv + v x uv.
struct Quat {
    double w;
    V3 v;
    V3 apply(const V3 &p) const {
        V3 uv = cross(v, p);
        uv = {uv.x + uv.x, uv.y + uv.y, uv.z + uv.z};
        V3 c = cross(v, uv);
        return {p.x + w * uv.x + c.x, p.y + w * uv.y + c.y, p.z + w * uv.z + c.z};
    }
};

struct MolSystem {
    fg_params P;
    Cuboid geo;
    int N = 0, gs = 0, M = 0, nt = 0;
    std::vector<Site> p, trial;          // Space::p / Space::trial
    std::vector<V3> cm, cm_trial;        // Group::cm / Group::cm_trial
    std::vector<double> s2, eps4, lbqq;  // per type pair
    double lB = 0, rc = 0, rc2 = 0, a2 = 0, rfB = 0, kappa = 0;
    int moved = -1;

    // CoulombGalore::operator() (multipole.h:569-598): the splitting-function
    // table is not used; with kappa = 0 (every type but "yukawa") the
    // energy is lB q_i q_j Q5(r/rc) / r inside rc.
    double coulomb(const Site &a, const Site &b, double r2) const {
        if (r2 < rc2) {
            double r = std::sqrt(r2);
            double q = r / rc;
            double q2 = q * q;
            double Q = std::pow(q - 1.0, 3.0) * (5.0 / 22.0 * q2 * a2 + 9.0 / 22.0 * q * a2 - 0.6 * q2 - 1.2 * q - 1.0);
            return lbqq[a.id * nt + b.id] / r * std::exp(-r * kappa) * Q;
        }
        return 0;
    }
    // LennardJonesMixed<LorentzBerthelot>::operator() (potentials.h:2036-2040)
    double lj(const Site &a, const Site &b, double r2) const {
        double x = s2[a.id * nt + b.id] / r2;
        x = x * x * x;
        return eps4[a.id * nt + b.id] * (x * x - x);
    }
    // IonDipole::operator() -> q2mu (multipole.h:269-277, 993-996), r = a - b
    double ion_dipole(const Site &a, const Site &b, const V3 &r) const {
        double r2i = 1 / dot(r, r);
        double r1i = std::sqrt(r2i);
        double r3i = r1i * r2i;
        V3 mr = {-r.x, -r.y, -r.z};
        double W1 = (a.q * b.mus) * dot(b.mu, r) * r3i;
        double W2 = (b.q * a.mus) * dot(a.mu, mr) * r3i;
        return lB * (W1 + W2);
    }
    // DipoleDipoleGalore::operator() (multipole.h:910-920) with the reaction
    // field splitting A(q) = 1, B(q) = -(2(eps_rf-eps_r)/(2eps_rf+eps_r))/eps_r q^3
    // (767-782), and mu2mu (287-299).
    double dipole_dipole(const Site &a, const Site &b, const V3 &r) const {
        double r1 = std::sqrt(dot(r, r));
        if (r1 < rc) {
            double qq = r1 / rc;
            double af = 1.0, bf = rfB * qq * qq * qq;
            double r2i = 1 / dot(r, r);
            double r1i = std::sqrt(r2i);
            double d = dot(a.mu, b.mu);
            double T = (3 * dot(a.mu, r) * dot(b.mu, r) * r2i - d) * af + d * bf;
            return lB * (-(a.mus * b.mus) * T * r1i * r2i);
        }
        return 0.0;
    }
    // NonbondedVector::i2i (energy.h:1119-1122): pairpot(a, b, vdist(a, b))
    double pair(const Site &a, const Site &b) const {
        V3 r = geo.vdist(a.r, b.r);
        double r2 = dot(r, r);
        return (coulomb(a, b, r2) + lj(a, b, r2)) + (ion_dipole(a, b, r) + dipole_dipole(a, b, r));
    }

    // Energybase::g2All for one moved group (energy.h:182-215): g2g against
    // every other group (energy.h:1156-1196), moved<->itself = 0.
    double group_energy(const std::vector<Site> &pv, int g) const {
        double du = 0;
        for (int h = 0; h < M; h++) {
            if (h == g) continue;
            double u = 0;
            for (int i = g * gs; i < (g + 1) * gs; i++)
                for (int j = h * gs; j < (h + 1) * gs; j++) u += pair(pv[i], pv[j]);
            du += u;
        }
        return du;
    }

    void init(const fg_params *prm, int n, int group_size) {
        P = *prm;
        geo.set(P.box);
        nt = P.n_types;
        N = n;
        gs = group_size;
        M = N / gs;
        lB = P.bjerrum;
        rc = P.rf_cutoff;
        rc2 = rc * rc;
        kappa = 0.0;
        const double kappas = kappa * rc, kappas2 = kappas * kappas;
        a2 = -66.0 * (1027.0 * kappas2 + 8505.0 * kappas + 1494.0) / (5284.0 * kappas2 + 25515.0 * kappas + 56916.0);
        rfB = -(2 * (P.rf_eps_rf - P.rf_eps_r) / (2 * P.rf_eps_rf + P.rf_eps_r)) / P.rf_eps_r;
        s2.assign(nt * nt, 0);
        eps4.assign(nt * nt, 0);
        lbqq.assign(nt * nt, 0);
        for (int i = 0; i < nt; i++)
            for (int j = 0; j < nt; j++) {
                double sig = 0.5 * (P.type_sigma[i] + P.type_sigma[j]);
                s2[i * nt + j] = sig * sig;
                eps4[i * nt + j] = 4 * std::sqrt(P.type_eps[i] * P.type_eps[j]);
                lbqq[i * nt + j] = lB * P.type_charge[i] * P.type_charge[j];  // CoulombGalore lBxQeQe, kappa = 0
            }
    }

    // Geometry::anyCenter with mass weights (geometry.h:714-738): origin at
    // the middle particle, minimum-image offsets, equal masses here.
    V3 mass_center(const std::vector<Site> &pv, int g) const {
        const int front = g * gs, back = (g + 1) * gs - 1;
        V3 o = pv[(size_t)(front + (back - front) * 0.5)].r;
        V3 c = {0, 0, 0};
        double sum = 0;
        for (int i = front; i <= back; i++) {
            V3 t = {pv[i].r.x - o.x, pv[i].r.y - o.y, pv[i].r.z - o.z};
            geo.boundary(t);
            c = {c.x + t.x * 1.0, c.y + t.y * 1.0, c.z + t.z * 1.0};
            sum += 1.0;
        }
        c = {c.x / sum + o.x, c.y / sum + o.y, c.z / sum + o.z};
        geo.boundary(c);
        return c;
    }

    void set_state(const double *xyz, const double *mu, const double *mus, const int32_t *ids, const double *cms) {
        p.resize(N);
        for (int i = 0; i < N; i++) {
            p[i].r = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
            p[i].mu = mu ? V3{mu[3 * i], mu[3 * i + 1], mu[3 * i + 2]} : V3{0, 0, 0};
            p[i].mus = mus ? mus[i] : 0.0;
            p[i].id = ids[i];
            p[i].q = P.type_charge[ids[i]];
        }
        trial = p;
        cm.resize(M);
        for (int g = 0; g < M; g++) cm[g] = cms ? V3{cms[3 * g], cms[3 * g + 1], cms[3 * g + 2]} : mass_center(p, g);
        cm_trial = cm;
    }

    // QuaternionRotate::operator() (geometry.h:131-140)
    V3 rotate_point(const Quat &q, const V3 &origin, V3 a) const {
        a = {a.x - origin.x, a.y - origin.y, a.z - origin.z};
        geo.boundary(a);
        a = q.apply(a);
        a = {a.x + origin.x, a.y + origin.y, a.z + origin.z};
        geo.boundary(a);
        return a;
    }

    // TranslateRotate::_trialMove (move.h:1640-1685) given its draws:
    // unit vector u (ranunit), rotation centre kind (0 = mass centre,
    // 1 = first atom, 2 = last atom), angle, translation t.
    void make_trial(int g, const V3 &u, int center_kind, double angle, const V3 &t, bool rotate, bool translate) {
        moved = g;
        const int front = g * gs, back = (g + 1) * gs - 1;
        if (rotate) {
            V3 center = cm[g];
            if (center_kind == 1) center = trial[front].r;
            if (center_kind == 2) center = trial[back].r;
            V3 endp = {center.x + u.x, center.y + u.y, center.z + u.z};
            // QuaternionRotate::setAxis (geometry.cpp:753-766)
            V3 ax = {endp.x - center.x, endp.y - center.y, endp.z - center.z};
            geo.boundary(ax);
            double nrm = std::sqrt(dot(ax, ax));
            ax = {ax.x / nrm, ax.y / nrm, ax.z / nrm};
            const double ha = 0.5 * angle;
            Quat q{std::cos(ha), {std::sin(ha) * ax.x, std::sin(ha) * ax.y, std::sin(ha) * ax.z}};
            // Group::newrotate (group.h:259-277)
            cm_trial[g] = rotate_point(q, center, cm_trial[g]);
            const V3 zero = {0, 0, 0};
            for (int i = front; i <= back; i++) {
                trial[i].r = rotate_point(q, center, trial[i].r);
                trial[i].mu = rotate_point(q, zero, trial[i].mu);  // DipoleParticle::rotate (point.h:672-679)
            }
        }
        if (translate) {
            // Group::translate (group.h:186-193), Point::translate (point.h:96-100)
            V3 &c = cm_trial[g];
            c = {c.x + t.x, c.y + t.y, c.z + t.z};
            geo.boundary(c);
            for (int i = front; i <= back; i++) {
                V3 &r = trial[i].r;
                r = {r.x + t.x, r.y + t.y, r.z + t.z};
                geo.boundary(r);
            }
        }
    }

    // Energy::energyChange (energy.h:3577-3621) for one whole moved group
    double trial_du() const { return group_energy(trial, moved) - group_energy(p, moved); }

    // TranslateRotate::_acceptMove/_rejectMove (move.h:1688-1705) ->
    // Group::accept/undo (group.h:370-385)
    void commit(bool accepted) {
        const int g = moved;
        for (int i = g * gs; i < (g + 1) * gs; i++) {
            if (accepted) p[i] = trial[i];
            else trial[i] = p[i];
        }
        if (accepted) cm[g] = cm_trial[g];
        else cm_trial[g] = cm[g];
        moved = -1;
    }

    // Energybase::systemEnergy (energy.h:169-180): g_internal of every group
    // (NonbondedVector::g_internal, energy.h:1207-1216, all i<j site pairs of
    // the molecule) plus g2g over all group pairs.
    // comp = {intermolecular, intramolecular, total}
    void total_energy(double *comp) const {
        double ui = 0;
        for (int g = 0; g < M; g++) {
            double u = 0;
            for (int i = g * gs; i < (g + 1) * gs - 1; i++)
                for (int j = i + 1; j < (g + 1) * gs; j++) u += pair(p[i], p[j]);
            ui += u;
        }
        double up = 0;
        for (int a = 0; a < M; a++)
            for (int b = a + 1; b < M; b++) {
                double ug = 0;
                for (int i = a * gs; i < (a + 1) * gs; i++)
                    for (int j = b * gs; j < (b + 1) * gs; j++) ug += pair(p[i], p[j]);
                up += ug;
            }
        comp[0] = up;
        comp[1] = ui;
        comp[2] = ui + up;
    }
};

// The global-slump draws of one TranslateRotate trial plus its Metropolis
// uniform (move.h:1624-1685, 567-573): element(groups) -> range;
// ranunit -> 3 uniforms per attempt until |v|^2 <= 1 (point.h:74-88);
// if not rotating about the mass centre, one uniform picks the first (<0.5)
// or last atom; angle = dprot * half(); translation dp * half() per axis.
struct GroupDraw {
    int g;
    V3 u;
    int center;
    double angle;
    V3 t;
    double um;
};

GroupDraw draw_group(Twister &s, int M, double dp, double dprot, bool center_rotation) {
    GroupDraw d{};
    d.g = s.range(0, M - 1);
    if (dprot > 1e-6) {
        double r2;
        do {
            d.u.x = (2 * s() - 1) * 1.0;
            d.u.y = (2 * s() - 1) * 1.0;
            d.u.z = (2 * s() - 1) * 1.0;
            r2 = dot(d.u, d.u);
        } while (r2 > 1);
        double n = std::sqrt(r2);
        d.u = {d.u.x / n, d.u.y / n, d.u.z / n};
        d.center = 0;
        if (!center_rotation) d.center = (s() < 0.5) ? 1 : 2;
        d.angle = dprot * (s() - 0.5);
    }
    if (dp > 1e-6) {
        d.t.x = 1.0 * dp * (s() - 0.5);
        d.t.y = 1.0 * dp * (s() - 0.5);
        d.t.z = 1.0 * dp * (s() - 0.5);
    }
    d.um = s();
    return d;
}

}  // namespace

extern "C" {

void *or_mol_create(const fg_params *p, int n_sites, int group_size) {
    if (!p || group_size < 1 || n_sites < group_size || n_sites % group_size) return nullptr;
    MolSystem *s = new MolSystem();
    s->init(p, n_sites, group_size);
    return s;
}

void or_mol_destroy(void *h) { delete (MolSystem *)h; }

// mu: unit vectors (3N, may be NULL = no dipoles), mus: scalars (N), cms:
// group mass centres (3M) or NULL to compute them as the reference does.
int or_mol_set_state(void *h, const double *xyz, const double *mu, const double *mus, const int32_t *ids,
                     const double *cms) {
    ((MolSystem *)h)->set_state(xyz, mu, mus, ids, cms);
    return 0;
}

int or_mol_get_state(void *h, double *xyz, double *mu, double *cms) {
    MolSystem *s = (MolSystem *)h;
    for (int i = 0; i < s->N; i++) {
        if (xyz) { xyz[3 * i] = s->p[i].r.x; xyz[3 * i + 1] = s->p[i].r.y; xyz[3 * i + 2] = s->p[i].r.z; }
        if (mu) { mu[3 * i] = s->p[i].mu.x; mu[3 * i + 1] = s->p[i].mu.y; mu[3 * i + 2] = s->p[i].mu.z; }
    }
    if (cms)
        for (int g = 0; g < s->M; g++) { cms[3 * g] = s->cm[g].x; cms[3 * g + 1] = s->cm[g].y; cms[3 * g + 2] = s->cm[g].z; }
    return 0;
}

double or_mol_pair(void *h, int i, int j) {
    MolSystem *s = (MolSystem *)h;
    return s->pair(s->p[i], s->p[j]);
}

// dU for moving group g to explicit trial positions / dipoles (3*gs each).
double or_mol_trial_du_explicit(void *h, int g, const double *xyz, const double *mu) {
    MolSystem *s = (MolSystem *)h;
    s->moved = g;
    for (int a = 0; a < s->gs; a++) {
        Site &t = s->trial[g * s->gs + a];
        t.r = {xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]};
        if (mu) t.mu = {mu[3 * a], mu[3 * a + 1], mu[3 * a + 2]};
    }
    return s->trial_du();
}

void or_mol_commit(void *h, int accepted) { ((MolSystem *)h)->commit(accepted != 0); }

// comp = {intermolecular, intramolecular, total}
void or_mol_total_energy(void *h, double *comp) { ((MolSystem *)h)->total_energy(comp); }

// The reference's draws for n TranslateRotate trials (one molecule kind,
// "permol"): group, axis, centre kind, angle, translation, Metropolis u.
int or_mol_draw_stream(uint32_t seed, int n_groups, double dp, double dprot, int center_rotation, int64_t n,
                       int32_t *g, double *axis, int32_t *center, double *angle, double *trans, double *u) {
    Twister s(seed);
    for (int64_t k = 0; k < n; k++) {
        GroupDraw d = draw_group(s, n_groups, dp, dprot, center_rotation != 0);
        g[k] = d.g;
        axis[3 * k] = d.u.x; axis[3 * k + 1] = d.u.y; axis[3 * k + 2] = d.u.z;
        center[k] = d.center;
        angle[k] = d.angle;
        trans[3 * k] = d.t.x; trans[3 * k + 1] = d.t.y; trans[3 * k + 2] = d.t.z;
        u[k] = d.um;
    }
    return 0;
}

// Movebase::move loop (move.h:515-555) with TranslateRotate over an explicit
// stream; logs dU and acceptance per trial; returns the sum of accepted dU.
// rotate/translate: whether dprot/dp exceed 1e-6 (move.h:1642, 1671).
double or_mol_run_stream(void *h, int64_t n, const int32_t *g, const double *axis, const int32_t *center,
                         const double *angle, const double *trans, const double *u, int rotate, int translate,
                         double *du_out, uint8_t *acc_out) {
    MolSystem *s = (MolSystem *)h;
    double usum = 0;
    for (int64_t k = 0; k < n; k++) {
        s->make_trial(g[k], {axis[3 * k], axis[3 * k + 1], axis[3 * k + 2]}, center[k], angle[k],
                      {trans[3 * k], trans[3 * k + 1], trans[3 * k + 2]}, rotate != 0, translate != 0);
        double du = s->trial_du();
        bool acc = !(u[k] > std::exp(-du));  // Movebase::metropolis (move.h:567-573)
        s->commit(acc);
        if (acc) usum += du;
        if (du_out) du_out[k] = du;
        if (acc_out) acc_out[k] = acc ? 1 : 0;
    }
    return usum;
}

}  // extern "C"
