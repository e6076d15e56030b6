// Drop-in energy term for Faunus (bjornstenqvist/beoFaunus): the GB300
// library behind the reference's Energybase interface (energy.h:54-224).
//
// Header-only. Include it after the Faunus headers and link
// libfaunus_gb300.so. It replaces, in a reference program,
//
//     Energy::NonbondedEwald<Tspace, Potential::WeeksChandlerAndersen> pot(json);
//   or
//     Energy::Nonbonded<Tspace, CombinedPairPotential<DebyeHuckel,
//                       LennardJonesMixed<LorentzBerthelot>>> pot(json);
//
// with
//
//     Energy::NonbondedGPU<Tspace> pot(Energy::gpuParamsEwaldWCA(json));
//
// and leaves Movebase / AtomicTranslation / Propagator unchanged: Movebase::move
// (move.h:515-555) calls updateChange -> energyChange -> update, which land
// here as fg_trial_du (from external() on the trial vector) and fg_commit.
// i2i/g2All/g_external return 0 because the whole moved-particle sum is
// computed on the device; energyChangeConfiguration (energy.h:3521-3572)
// therefore sums to the device's dU.
//
// translateOnDevice runs whole sweeps on the device with the same random
// draws the reference makes from the global `slump` (move.h:818-864,
// group.h:129-134, move.h:567-573). For point dipoles (Space of
// DipoleParticle), NonbondedEwaldDipoleGPU replaces
//     Energy::NonbondedEwald<Tspace, Potential::LennardJonesLB, ii, id, dd>
// and dipoleMovesOnDevice runs AtomicRotation / AtomicTranslation sweeps.
#ifndef FAUNUS_GB300_ENERGY_HPP
#define FAUNUS_GB300_ENERGY_HPP

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "faunus_gb300.h"

namespace Faunus {
namespace Energy {

inline void fg_check(int rc) {
    if (rc != FG_OK) throw std::runtime_error(std::string("faunus_gb300: ") + fg_last_error());
}

// Atom types in the order of the global atom map (species.h), as fg_params
// wants them: charge, sigma, eps (kT), dp.
inline void gpuFillTypes(fg_params &p) {
    p.n_types = 0;
    for (auto &a : atom) {
        if (p.n_types >= FG_MAX_TYPES) throw std::runtime_error("faunus_gb300: too many atom types");
        const int t = p.n_types++;
        p.type_charge[t] = a.charge;
        p.type_sigma[t] = a.sigma;
        p.type_eps[t] = a.eps;
        p.type_dp[t] = a.dp;
    }
}

// fg_params for NonbondedEwald<Tspace, WeeksChandlerAndersen> from the
// reference's JSON keys (ewald.h:507-530; Coulomb epsr, src/potentials.cpp:357-363).
inline fg_params gpuParamsEwaldWCA(Tmjson &j) {
    fg_params p{};
    p.model = FG_MODEL_EWALD_WCA;
    auto e = j["energy"]["nonbonded"]["ewald"];
    double L = j["system"]["geometry"]["length"];
    p.box[0] = p.box[1] = p.box[2] = L;
    p.bjerrum = pc::lB(j["energy"]["nonbonded"].value("epsr", 80.0));
    p.ewald_alpha = e.at("alpha");
    p.ewald_cutoff = e.at("cutoff");
    p.ewald_cutoff_k = e.at("cutoffK");
    p.ewald_debye_length = e.at("debyelength");
    p.ewald_eps_surf = e.at("eps_surf");
    p.ewald_spherical_sum = e.value("spherical_sum", true) ? 1 : 0;
    p.ewald_isotropic_pbc = e.value("isotropic_pbc", false) ? 1 : 0;
    p.ewald_update_frequency = e.value("update_frequency", -1);
    p.kT_scale = 1.0;
    gpuFillTypes(p);
    return p;
}

// fg_params for Nonbonded<DebyeHuckel + LennardJonesMixed> (src/potentials.cpp:770-782).
inline fg_params gpuParamsDHLJ(Tmjson &j) {
    fg_params p{};
    p.model = FG_MODEL_DH_LJ;
    double L = j["system"]["geometry"]["length"];
    p.box[0] = p.box[1] = p.box[2] = L;
    p.bjerrum = pc::lB(j["energy"]["nonbonded"].value("epsr", 80.0));
    p.dh_debye_length = j["energy"]["nonbonded"].at("debyelength");
    p.kT_scale = 1.0;
    gpuFillTypes(p);
    return p;
}

template <class Tspace>
class NonbondedGPU : public Energybase<Tspace> {
    typedef Energybase<Tspace> Tbase;
    typedef typename Tbase::Tpvec Tpvec;
    fg_params P;
    fg_system *h = nullptr;
    std::vector<int> moved;
    std::string _info() override { return "GB300 device energy (faunus_gb300)\n"; }

  public:
    explicit NonbondedGPU(const fg_params &p) : P(p) { Tbase::name = "Nonbonded GB300"; }
    ~NonbondedGPU() override {
        if (h) fg_destroy(h);
    }
    fg_system *handle() { return h; }

    // Energybase::setSpace (energy.h:88-92): upload particles, build Q(k).
    void setSpace(Tspace &s) override {
        Tbase::setSpace(s);
        const int n = (int)s.p.size();
        if (!h || n != lastN) {
            if (h) fg_destroy(h);
            fg_check(fg_create(&P, n, &h));
            lastN = n;
        }
        std::vector<double> xyz(3 * n), q(n);
        std::vector<int32_t> ids(n);
        for (int i = 0; i < n; i++) {
            xyz[3 * i] = s.p[i].x();
            xyz[3 * i + 1] = s.p[i].y();
            xyz[3 * i + 2] = s.p[i].z();
            q[i] = s.p[i].charge;
            ids[i] = s.p[i].id;
        }
        fg_check(fg_set_state(h, xyz.data(), q.data(), ids.data()));
    }

    // NonbondedEwald::updateChange (ewald.h:651-705): remember the moved set.
    double updateChange(const typename Tspace::Change &c) override {
        moved.clear();
        for (auto &m : c.mvGroup)
            for (int i : m.second) moved.push_back(i);
        return 0;
    }

    // external(trial) carries the whole dU of the moved particle; external(p) 0.
    double external(const Tpvec &p) override {
        if (!Tbase::isTrial(p) || moved.empty()) return 0;
        if (moved.size() != 1) throw std::runtime_error("NonbondedGPU: one moved particle per trial");
        const int i = moved[0];
        const double xyz[3] = {p[i].x(), p[i].y(), p[i].z()};
        const int32_t idx = i;
        double du = 0;
        fg_check(fg_trial_du(h, 1, &idx, xyz, &du));
        return du;
    }

    // NonbondedEwald::update (ewald.h:613-646): commit, maybe rebuild Q(k).
    double update(bool accepted) override {
        if (moved.empty()) return 0;
        double corr = 0;
        fg_check(fg_commit(h, accepted ? 1 : 0, &corr));
        moved.clear();
        return corr;
    }

    // Energybase::systemEnergy (energy.h:169-180), every term in FP64 (the
    // reference's drift bookkeeping compares it with the running sum)
    double systemEnergy(const Tpvec &) override {
        double c[5];
        fg_check(fg_total_energy_fp64(h, c));
        return c[4];
    }

  private:
    int lastN = -1;
};

// AtomicTranslation on the device: the same draws from the global `slump`
// as AtomicTranslation::_trialMove and Movebase::metropolis, then one
// fg_sweep for the n trials; positions are copied back into Space.
template <class Tspace>
double translateOnDevice(Tspace &spc, NonbondedGPU<Tspace> &pot, int n) {
    const int N = (int)spc.p.size();
    std::vector<int32_t> idx(n);
    std::vector<double> disp(3 * (size_t)n), u(n);
    for (int t = 0; t < n; t++) {
        slump.range(0, 0);                               // slump.element(groups), one atomic group
        const int i = slump.range(0, N - 1);             // Group::random
        const double dp = atom[spc.p[i].id].dp;
        double tx = dp, ty = dp, tz = dp;
        tx *= slump() - 0.5;
        ty *= slump() - 0.5;
        tz *= slump() - 0.5;
        idx[t] = i;
        disp[3 * t] = tx;
        disp[3 * t + 1] = ty;
        disp[3 * t + 2] = tz;
        u[t] = slump();                                  // Movebase::metropolis
    }
    fg_sweep_stats st{};
    fg_check(fg_sweep(pot.handle(), n, idx.data(), disp.data(), u.data(), nullptr, nullptr, &st));
    std::vector<double> xyz(3 * (size_t)N);
    fg_check(fg_get_state(pot.handle(), xyz.data()));
    for (int i = 0; i < N; i++) {
        spc.p[i].x() = xyz[3 * i];
        spc.p[i].y() = xyz[3 * i + 1];
        spc.p[i].z() = xyz[3 * i + 2];
        spc.trial[i] = spc.p[i];
    }
    return st.energy_change;
}

// ---------------------------------------------------------------- point dipoles
// fg_params for NonbondedEwald<Tspace, LennardJonesLB, useIonIon,
// useIonDipole, useDipoleDipole> on DipoleParticle (ewald.h:228-550): terms is
// FG_EWALD_ION_ION | FG_EWALD_ION_DIPOLE | FG_EWALD_DIPOLE_DIPOLE as the
// template flags; quirk 1 computes the sum as the reference's live code does.
inline fg_params gpuParamsEwaldDipole(Tmjson &j, int terms, int quirk = 0) {
    fg_params p = gpuParamsEwaldWCA(j);
    p.model = FG_MODEL_EWALD_DIPOLE;
    p.ewald_terms = terms;
    p.ewald_dipole_quirk = quirk;
    return p;
}

// Replaces NonbondedEwald<Tspace, LennardJonesLB, ...> in a Space of
// DipoleParticle for AtomicTranslation and AtomicRotation: the moved
// particle's whole dU (position and dipole) comes from fg_dip_trial_du.
template <class Tspace>
class NonbondedEwaldDipoleGPU : public Energybase<Tspace> {
    typedef Energybase<Tspace> Tbase;
    typedef typename Tbase::Tpvec Tpvec;
    fg_params P;
    fg_dipsys *h = nullptr;
    std::vector<int> moved;
    int lastN = -1;
    std::string _info() override { return "GB300 dipolar Ewald (faunus_gb300)\n"; }

  public:
    explicit NonbondedEwaldDipoleGPU(const fg_params &p) : P(p) { Tbase::name = "NonbondedEwald dipoles GB300"; }
    ~NonbondedEwaldDipoleGPU() override {
        if (h) fg_dip_destroy(h);
    }
    fg_dipsys *handle() { return h; }

    void setSpace(Tspace &s) override {
        Tbase::setSpace(s);
        const int n = (int)s.p.size();
        if (!h || n != lastN) {
            if (h) fg_dip_destroy(h);
            fg_check(fg_dip_create(&P, n, &h));
            lastN = n;
        }
        std::vector<double> xyz(3 * n), mu(3 * n), mus(n), q(n);
        std::vector<int32_t> ids(n);
        for (int i = 0; i < n; i++) {
            for (int a = 0; a < 3; a++) {
                xyz[3 * i + a] = s.p[i][a];
                mu[3 * i + a] = s.p[i].mu()[a];
            }
            mus[i] = s.p[i].muscalar();
            q[i] = s.p[i].charge;
            ids[i] = s.p[i].id;
        }
        fg_check(fg_dip_set_state(h, xyz.data(), mu.data(), mus.data(), q.data(), ids.data()));
    }

    double updateChange(const typename Tspace::Change &c) override {
        moved.clear();
        for (auto &m : c.mvGroup)
            for (int i : m.second) moved.push_back(i);
        return 0;
    }

    double external(const Tpvec &p) override {
        if (!Tbase::isTrial(p) || moved.empty()) return 0;
        if (moved.size() != 1) throw std::runtime_error("NonbondedEwaldDipoleGPU: one moved particle per trial");
        const int i = moved[0];
        const double xyz[3] = {p[i].x(), p[i].y(), p[i].z()};
        const double mu[3] = {p[i].mu().x(), p[i].mu().y(), p[i].mu().z()};
        double du = 0;
        fg_check(fg_dip_trial_du(h, i, xyz, mu, &du));
        return du;
    }

    double update(bool accepted) override {
        if (moved.empty()) return 0;
        double corr = 0;
        fg_check(fg_dip_commit(h, accepted ? 1 : 0, &corr));
        moved.clear();
        return corr;
    }

    double systemEnergy(const Tpvec &) override {
        double c[6];
        fg_check(fg_dip_total_energy(h, c));
        return c[5];
    }
};

// AtomicRotation (rotate = true) or AtomicTranslation sweeps of n trials on
// the device, with the draws those moves take from the global `slump`
// (move.h:1008-1032, 818-864, 567-573); positions and dipoles are copied
// back into Space.
template <class Tspace>
double dipoleMovesOnDevice(Tspace &spc, NonbondedEwaldDipoleGPU<Tspace> &pot, int n, bool rotate) {
    const int N = (int)spc.p.size();
    std::vector<int32_t> kind(n, rotate ? 1 : 2), idx(n);
    std::vector<double> axis(3 * (size_t)n), angle(n), disp(3 * (size_t)n), u(n);
    for (int t = 0; t < n; t++) {
        slump.range(0, 0);                               // the one atomic group
        const int i = slump.range(0, N - 1);             // Group::random
        idx[t] = i;
        if (rotate) {
            Point v;
            v.ranunit(slump);                            // point.h:74-88
            double dprot = atom[spc.p[i].id].dprot;
            angle[t] = dprot * slump.half();
            for (int a = 0; a < 3; a++) axis[3 * t + a] = v[a];
        } else {
            const double dp = atom[spc.p[i].id].dp;
            for (int a = 0; a < 3; a++) disp[3 * t + a] = dp * (slump() - 0.5);
        }
        u[t] = slump();                                  // Movebase::metropolis
    }
    fg_sweep_stats st{};
    fg_check(fg_dip_sweep(pot.handle(), n, kind.data(), idx.data(), axis.data(), angle.data(), disp.data(), u.data(),
                          nullptr, nullptr, &st));
    std::vector<double> xyz(3 * (size_t)N), mu(3 * (size_t)N);
    fg_check(fg_dip_get_state(pot.handle(), xyz.data(), mu.data()));
    for (int i = 0; i < N; i++) {
        for (int a = 0; a < 3; a++) {
            spc.p[i][a] = xyz[3 * i + a];
            spc.p[i].mu()[a] = mu[3 * i + a];
        }
        spc.trial[i] = spc.p[i];
    }
    return st.energy_change;
}

}  // namespace Energy
}  // namespace Faunus

#endif
