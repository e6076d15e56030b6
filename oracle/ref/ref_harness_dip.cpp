// Reference harness for point dipoles: drives the UNMODIFIED Faunus classes
// (built from the reference's own sources by oracle/ref/Makefile) on
// Space<Cuboid, DipoleParticle> with NonbondedEwald<Tspace, LennardJonesLB,
// useIonIon, useIonDipole, useDipoleDipole> and writes what the reference
// computes to a JSON file. Test infrastructure only (golden vectors for the
// oracle's point-dipole system, oracle/fg_oracle_dip.cpp).
//
// Modes (input key "mode"):
//   "known" : the reference's Ewald unit test (unittests.cpp:131-193) run on
//             the reference's live code: the ion-ion and the dipole-dipole
//             configuration, with a charged atom type (the neutral id-0 type
//             of the unit test makes the effective-charge ratio 0/0,
//             ewald.h:539). Writes ureal, usurf_reci, uself and the system
//             energy of both.
//   "mc"    : a dipolar fluid driven by Move::AtomicRotation and
//             Move::AtomicTranslation ("peratom" on the one atomic group),
//             one sweep of each in turn (rotation first). Logs every trial:
//             move kind (1 rotation, 2 translation), particle, trial position
//             and dipole vector, dU and acceptance.
//   "bench" : like "mc" without logs; prints trials/s.
// With "state_file", "mc" also saves the final state (Space::save).
// "terms" selects the template flags: "ii_dd" (useIonIon, useDipoleDipole, as
// the unit test) or "ii_id_dd" (all three).
#include <faunus/faunus.h>
#include <faunus/ewald.h>
#include <chrono>
#include <cstdio>
#include <fstream>
#include <map>

using namespace Faunus;
typedef Space<Geometry::Cuboid, DipoleParticle> Tspace;

struct Out {
    std::map<std::string, std::vector<double>> v;
    void set(const std::string &k, double x) { v[k] = {x}; }
    template<class T> void set(const std::string &k, const std::vector<T> &x) { v[k].assign(x.begin(), x.end()); }
    void write(const char *path) const {
        FILE *f = fopen(path, "w");
        fprintf(f, "{");
        bool first = true;
        for (auto &kv : v) {
            fprintf(f, "%s\n\"%s\": [", first ? "" : ",", kv.first.c_str());
            for (size_t i = 0; i < kv.second.size(); i++) fprintf(f, "%s%.17g", i ? "," : "", kv.second[i]);
            fprintf(f, "]");
            first = false;
        }
        fprintf(f, "\n}\n");
        fclose(f);
    }
};

// Shared trial log of both moves.
struct Log {
    bool on = true;
    std::vector<int> kind, idx, acc;
    std::vector<double> xyz, mu, du;
    void trial(int k, const DipoleParticle &t, int i) {
        if (!on) return;
        kind.push_back(k);
        idx.push_back(i);
        xyz.push_back(t.x()); xyz.push_back(t.y()); xyz.push_back(t.z());
        mu.push_back(t.mu().x()); mu.push_back(t.mu().y()); mu.push_back(t.mu().z());
    }
};

// Each override calls the reference's own implementation and records it.
template<class Tsp>
class LoggedRotation : public Move::AtomicRotation<Tsp> {
    typedef Move::AtomicRotation<Tsp> base;
  public:
    Log *log;
    LoggedRotation(Energy::Energybase<Tsp> &e, Tsp &s, Tmjson &j, Log *l) : base(e, s, j), log(l) {}
  protected:
    void _trialMove() override {
        base::_trialMove();
        log->trial(1, this->spc->trial[this->iparticle], this->iparticle);
    }
    double _energyChange() override {
        double d = base::_energyChange();
        if (log->on) log->du.push_back(d);
        return d;
    }
    void _acceptMove() override { if (log->on) log->acc.push_back(1); base::_acceptMove(); }
    void _rejectMove() override { if (log->on) log->acc.push_back(0); base::_rejectMove(); }
};

template<class Tsp>
class LoggedTranslation : public Move::AtomicTranslation<Tsp> {
    typedef Move::AtomicTranslation<Tsp> base;
  public:
    Log *log;
    LoggedTranslation(Energy::Energybase<Tsp> &e, Tsp &s, Tmjson &j, Log *l) : base(e, s, j), log(l) {}
  protected:
    void _trialMove() override {
        base::_trialMove();
        log->trial(2, this->spc->trial[this->iparticle], this->iparticle);
    }
    double _energyChange() override {
        double d = base::_energyChange();
        if (log->on) log->du.push_back(d);
        return d;
    }
    void _acceptMove() override { if (log->on) log->acc.push_back(1); base::_acceptMove(); }
    void _rejectMove() override { if (log->on) log->acc.push_back(0); base::_rejectMove(); }
};

static Tmjson faunus_input(const Tmjson &in) {
    const int N = in["positions"].size();
    Tmjson j;
    j["system"]["temperature"] = in.value("temperature", 298.0);
    j["system"]["geometry"]["length"] = in["box"];
    int t = 0;
    for (auto &ty : in["types"]) {
        std::string name = "T" + std::to_string(t++);
        j["atomlist"][name] = {{"q", ty["q"]}, {"sigma", ty["sigma"]}, {"dp", ty["dp"]}};
    }
    j["atomlist"]["T0"]["Ninit"] = 0;
    j["moleculelist"]["sol"] = {{"atoms", "T0"}, {"Ninit", N}, {"atomic", true}};
    double lB_target = in["bjerrum"];
    pc::setT(j["system"]["temperature"].get<double>());
    j["energy"]["nonbonded"]["epsr"] = pc::lB(1.0) / lB_target;
    j["energy"]["nonbonded"]["ewald"] = {
        {"eps_surf", in["eps_surf"]}, {"alpha", in["alpha"]}, {"cutoff", in["cutoff"]},
        {"cutoffK", in["cutoffK"]}, {"debyelength", in.value("debyelength", 1e30)},
        {"spherical_sum", in.value("spherical_sum", true)},
        {"update_frequency", in.value("update_frequency", -1)}};
    j["moves"]["atomrotate"]["sol"] = {{"peratom", true}};
    j["moves"]["atomtranslate"]["sol"] = {{"peratom", true}};
    return j;
}

// Per-type parameters straight into the atom map (eps in kT, dprot in
// radians), then the particles with their dipoles.
static void place_particles(const Tmjson &in, Tspace &spc) {
    int t = 0;
    for (auto &ty : in["types"]) {
        auto &a = atom[atom["T" + std::to_string(t++)].id];
        a.eps = ty["eps"];
        a.sigma = ty["sigma"];
        a.radius = 0.5 * a.sigma;
        a.charge = ty["q"];
        a.dp = ty["dp"];
        a.dprot = ty["dprot"];
    }
    const int N = in["positions"].size();
    if ((int)spc.p.size() != N) throw std::runtime_error("particle count mismatch");
    for (int i = 0; i < N; i++) {
        int ty = in["type_ids"][i];
        spc.p[i] = atom[atom["T" + std::to_string(ty)].id];
        spc.p[i].x() = in["positions"][i][0];
        spc.p[i].y() = in["positions"][i][1];
        spc.p[i].z() = in["positions"][i][2];
        spc.p[i].charge = in["charges"][i];
        spc.p[i].mu() = Point(in["mu"][i][0], in["mu"][i][1], in["mu"][i][2]);
        spc.p[i].muscalar() = in["mus"][i];
    }
    spc.trial = spc.p;
    spc.initTracker();
}

template<class Tenergy>
static void run_mc(const Tmjson &in, Out &out, bool bench) {
    Tmjson j = faunus_input(in);
    Tspace spc(j);
    place_particles(in, spc);
    Tenergy pot(j);
    Log log;
    log.on = !bench;
    LoggedRotation<Tspace> rot(pot, spc, j["moves"]["atomrotate"], &log);
    LoggedTranslation<Tspace> tra(pot, spc, j["moves"]["atomtranslate"], &log);
    slump.seed(in.value("seed", 5489u));
    out.set("bjerrum", pot.pairpot.first.bjerrumLength());
    out.set("u0", Energy::systemEnergy(spc, pot, spc.p));
    const int sweeps = in.value("sweeps", 1);
    double usum = 0;
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < sweeps; s++) {
        usum += rot.move();
        usum += tra.move();
    }
    auto t1 = std::chrono::steady_clock::now();
    const double secs = std::chrono::duration<double>(t1 - t0).count();
    const double trials = 2.0 * sweeps * spc.p.size();
    out.set("seconds", secs);
    out.set("trials", trials);
    out.set("trials_per_s", trials / secs);
    out.set("u_move_sum", usum);
    out.set("u1", Energy::systemEnergy(spc, pot, spc.p));
    if (in.count("state_file")) {
        // Space::save (space.h:736-764) of the final state, DipoleParticle records
        spc.initTracker();
        spc.save(in["state_file"].get<std::string>());
    }
    if (!bench) {
        std::vector<double> fx, fm;
        for (auto &a : spc.p)
            for (int k = 0; k < 3; k++) {
                fx.push_back(a[k]);
                fm.push_back(a.mu()[k]);
            }
        out.set("final_positions", fx);
        out.set("final_mu", fm);
        out.set("kind", log.kind);
        out.set("idx", log.idx);
        out.set("trial_xyz", log.xyz);
        out.set("trial_mu", log.mu);
        out.set("du", log.du);
        out.set("acc", log.acc);
    }
}

// unittests.cpp:131-193 on the live code, with type T0 charged
template<class Tenergy>
static void run_known(const Tmjson &in, Out &out) {
    Tmjson j = faunus_input(in);
    Tspace spc(j);
    place_particles(in, spc);
    Tenergy pot(j);
    Group g(0, 3);
    for (int i = 0; i < 4; i++) { spc.p[i].charge = 0.0; spc.p[i].muscalar() = 0.0; }
    spc.p[0].charge = 1.0;
    spc.p[1].charge = -1.0;
    spc.trial = spc.p;
    pot.setSpace(spc);
    out.set("bjerrum", pot.pairpot.first.bjerrumLength());
    out.set("ii_real", pot.pairpot(spc.p[0], spc.p[1], spc.p[1] - spc.p[0]));
    out.set("ii_recip_surf", pot.external(spc.p));
    out.set("ii_self", pot.g_external(spc.p, g));
    out.set("ii_total", Energy::systemEnergy(spc, pot, spc.p));
    spc.p[0].charge = 0.0;
    spc.p[1].charge = 0.0;
    spc.p[2].muscalar() = 1.0;
    spc.p[3].muscalar() = 1.0;
    spc.p[2].mu() = Point(1, 0, 0);
    spc.p[3].mu() = Point(1, 0, 0);
    spc.trial = spc.p;
    pot.setSpace(spc);
    out.set("dd_real", pot.pairpot(spc.p[2], spc.p[3], spc.p[2] - spc.p[3]));
    out.set("dd_recip_surf", pot.external(spc.p));
    out.set("dd_self", pot.g_external(spc.p, g));
    out.set("dd_total", Energy::systemEnergy(spc, pot, spc.p));
}

int main(int argc, char **argv) {
    if (argc != 3) { std::cerr << "usage: ref_harness_dip in.json out.json\n"; return 2; }
    std::ifstream f(argv[1]);
    Tmjson in;
    f >> in;
    Out out;
    const std::string mode = in.value("mode", std::string("mc"));
    const std::string terms = in.value("terms", std::string("ii_dd"));
    typedef Energy::NonbondedEwald<Tspace, Potential::LennardJonesLB, true, false, true> Tiidd;
    typedef Energy::NonbondedEwald<Tspace, Potential::LennardJonesLB, true, true, true> Tall;
    if (mode == "known" && terms == "ii_dd") run_known<Tiidd>(in, out);
    else if (mode == "known") run_known<Tall>(in, out);
    else if (terms == "ii_dd") run_mc<Tiidd>(in, out, mode == "bench");
    else run_mc<Tall>(in, out, mode == "bench");
    out.write(argv[2]);
    return 0;
}
