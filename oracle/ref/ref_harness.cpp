// Reference harness: drives the UNMODIFIED Faunus classes (built from the
// reference's own sources by oracle/ref/Makefile) on a system described in a
// JSON file, and writes what the reference computes to a JSON file.
//
// Test infrastructure only: it produces the golden vectors that pin the FP64
// oracle (oracle/fg_oracle.cpp) and can serve as the timed CPU reference. It
// never ships in the product library.
//
// Modes (input key "mode"):
//   "mc"     : Space<Cuboid,PointParticle> + NonbondedEwald<WCA> ("ewald_wca")
//              or Nonbonded<DebyeHuckel+LennardJonesMixed> ("dh_lj"),
//              driven by Move::AtomicTranslation ("peratom" on the one atomic
//              group), exactly as the reference's example programs do
//              (bulk.cpp: Space(json) -> energy -> moves -> move()).
//              Logs every trial: particle index, trial position, dU, accept.
//   "ewald_known" : the ion-ion part of the reference's Ewald unit test
//              (src/examples/unittests.cpp:131-170) with charged atom types.
//   "bench"  : like "mc" but logs nothing; prints trials/s. With a "seconds"
//              entry the move runs one trial per call ("peratom" off: the same
//              draws per trial) and the run is `warmup` + `steps` samples of
//              at least that many seconds each; "rates" lists the timed
//              samples' trials/s (the CPU reference of the benchmark).
//   "isobaric" : the same Space and pair energy plus Energy::ExternalPressure
//              (energy.h:1817-1890), driven by Move::Isobaric (move.h:5424-5640)
//              as bulk.cpp wires them; logs every volume move: dU, acceptance
//              and the volume after it.
// With an "rdf" entry {t1, t2, dr}, "mc" also samples the reference's
// Analysis::AtomRDF (analysis.h:2116-2134) after every sweep and writes its
// raw histogram (bin keys and counts, before normalisation) and <V>.
#include <faunus/faunus.h>
#include <faunus/ewald.h>
#include <chrono>
#include <cstdio>
#include <fstream>
#include <map>
#include <memory>

using namespace Faunus;
typedef Space<Geometry::Cuboid, PointParticle> Tspace;

// Output record: every value is written with 17 significant digits so the
// golden vectors keep full FP64 precision.
struct Out {
    std::map<std::string, std::vector<double>> v;
    std::vector<double> &operator[](const std::string &k) { return v[k]; }
    void set(const std::string &k, double x) { v[k] = {x}; }
    template<class T> void set(const std::string &k, const std::vector<T> &x) {
        v[k].assign(x.begin(), x.end());
    }
    void write(const char *path) const {
        FILE *f = fopen(path, "w");
        fprintf(f, "{");
        bool first = true;
        for (auto &kv : v) {
            fprintf(f, "%s\n\"%s\": [", first ? "" : ",", kv.first.c_str());
            for (size_t i = 0; i < kv.second.size(); i++)
                fprintf(f, "%s%.17g", i ? "," : "", kv.second[i]);
            fprintf(f, "]");
            first = false;
        }
        fprintf(f, "\n}\n");
        fclose(f);
    }
};

// Exposes AtomRDF's raw histogram (the reference normalises it only when
// saving to disk) without changing how it samples.
class RdfProbe : public Analysis::AtomRDF<Tspace> {
  public:
    RdfProbe(Tmjson j, Tspace &s) : Analysis::AtomRDF<Tspace>(j, s) {}
    std::map<double, double> raw() { return this->datavec[0].hist.getMap(); }
    double volume() { return this->V.avg(); }
};

// Logs what Isobaric does without changing it (move.h:5529-5624).
template<class Tsp>
class LoggedIsobaric : public Move::Isobaric<Tsp> {
    typedef Move::Isobaric<Tsp> base;
  public:
    std::vector<double> du;
    std::vector<int> acc;
    template<class Tenergy> LoggedIsobaric(Tenergy &e, Tsp &s, Tmjson &j) : base(e, s, j) {}
  protected:
    double _energyChange() override {
        const double d = base::_energyChange();
        du.push_back(d);
        return d;
    }
    void _acceptMove() override {
        base::_acceptMove();
        acc.push_back(1);
    }
    void _rejectMove() override {
        base::_rejectMove();
        acc.push_back(0);
    }
};

// Logs what AtomicTranslation does without changing it: every override
// calls the reference's own implementation (move.h:818-901).
template<class Tsp>
class LoggedTranslation : public Move::AtomicTranslation<Tsp> {
    typedef Move::AtomicTranslation<Tsp> base;
  public:
    bool log = true;
    std::vector<int> idx;
    std::vector<double> trial_xyz, du;
    std::vector<int> acc;
    LoggedTranslation(Energy::Energybase<Tsp> &e, Tsp &s, Tmjson &j) : base(e, s, j) {}
  protected:
    void _trialMove() override {
        base::_trialMove();
        if (log) {
            idx.push_back(this->iparticle);
            auto &t = this->spc->trial[this->iparticle];
            trial_xyz.push_back(t.x()); trial_xyz.push_back(t.y()); trial_xyz.push_back(t.z());
        }
    }
    double _energyChange() override {
        double d = base::_energyChange();
        if (log) du.push_back(d);
        return d;
    }
    void _acceptMove() override { if (log) acc.push_back(1); base::_acceptMove(); }
    void _rejectMove() override { if (log) acc.push_back(0); base::_rejectMove(); }
};

static Tmjson faunus_input(const Tmjson &in) {
    // Builds the reference's own JSON input from the harness description.
    const int N = in["positions"].size();
    Tmjson j;
    j["system"]["temperature"] = in.value("temperature", 298.0);
    j["system"]["geometry"]["length"] = in["box"];
    std::string atoms;
    int t = 0;
    for (auto &ty : in["types"]) {
        std::string name = "T" + std::to_string(t++);
        // the time-bounded bench builds the Space with point atoms: the
        // reference then inserts the N particles without overlap tests (every
        // position and atom parameter is set right after construction, and
        // the global random stream is seeded after that)
        const double sig = in.count("seconds") ? 0.0 : ty["sigma"].get<double>();
        j["atomlist"][name] = {{"q", ty["q"]}, {"sigma", sig}, {"dp", ty["dp"]}};
        atoms += (atoms.empty() ? "" : " ") + name;
    }
    // one atomic group holding all N particles (Space::insert merges atomic groups)
    j["atomlist"]["T0"]["Ninit"] = 0;
    // the time-bounded bench inserts one particle here and the other N - 1
    // in one call after construction (run_mc): the reference's atom tracker
    // re-registers the whole group on every insert, which is cubic in N when
    // the N particles arrive one at a time
    j["moleculelist"]["salt"] = {{"atoms", "T0"}, {"Ninit", in.count("seconds") ? 1 : N}, {"atomic", true}};
    double lB_target = in["bjerrum"];
    pc::setT(j["system"]["temperature"].get<double>());
    j["energy"]["nonbonded"]["epsr"] = pc::lB(1.0) / lB_target;
    if (in["model"] == "ewald_wca") {
        j["energy"]["nonbonded"]["ewald"] = {
            {"eps_surf", in["eps_surf"]}, {"alpha", in["alpha"]}, {"cutoff", in["cutoff"]},
            {"cutoffK", in["cutoffK"]}, {"debyelength", in.value("debyelength", 1e30)},
            {"spherical_sum", in.value("spherical_sum", true)},
            {"isotropic_pbc", in.value("isotropic_pbc", false)},
            {"update_frequency", in.value("update_frequency", -1)}};
    } else {
        j["energy"]["nonbonded"]["debyelength"] = in["debyelength"];
    }
    j["moves"]["atomtranslate"]["salt"] = {{"peratom", true}};
    return j;
}

// Per-type parameters straight into the atom map (eps in kT, no kJ/mol
// round trip), then every particle's type and position.
static void fill_space(const Tmjson &in, Tspace &spc) {
    int t = 0;
    for (auto &ty : in["types"]) {
        auto &a = atom[atom["T" + std::to_string(t++)].id];
        a.eps = ty["eps"];
        a.sigma = ty["sigma"];
        a.radius = 0.5 * a.sigma;
        a.charge = ty["q"];
        a.dp = ty["dp"];
    }
    const int N = in["positions"].size();
    if ((int)spc.p.size() != N) throw std::runtime_error("particle count mismatch");
    for (int i = 0; i < N; i++) {
        int ty = in["type_ids"][i];
        spc.p[i] = atom[atom["T" + std::to_string(ty)].id];
        spc.p[i].x() = in["positions"][i][0];
        spc.p[i].y() = in["positions"][i][1];
        spc.p[i].z() = in["positions"][i][2];
    }
    spc.trial = spc.p;
}

template<class Tenergy>
static void run_mc(const Tmjson &in, Out &out, bool bench) {
    Tmjson j = faunus_input(in);
    const bool timed = bench && in.count("seconds");
    if (timed) j["moves"]["atomtranslate"]["salt"]["peratom"] = false;
    Tspace spc(j);
    if (timed) {   // the rest of the atomic group in one Space::insert (space.h:950-1000)
        const int N = in["positions"].size();
        Tspace::ParticleVector more(N - 1);
        for (auto &x : more) x = atom[atom["T0"].id];
        spc.insert(spc.molList()["salt"].id, more);
    }
    fill_space(in, spc);
    const int N = spc.p.size();
    Tenergy pot(j);
    LoggedTranslation<Tspace> mv(pot, spc, j["moves"]["atomtranslate"]); // calls pot.setSpace(spc)
    mv.log = !bench;
    slump.seed(in.value("seed", 5489u));
    out.set("bjerrum", pot.pairpot.first.bjerrumLength());
    if (timed) {
        const double secs = in["seconds"];
        const int steps = in.value("steps", 1), warm = in.value("warmup", 0);
        std::vector<double> rates;
        for (int s = 0; s < warm + steps; s++) {
            long n = 0;
            double el = 0;
            auto t0 = std::chrono::steady_clock::now();
            do {
                for (int k = 0; k < 8; k++) mv.move();
                n += 8;
                el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            } while (el < secs);
            if (s >= warm) rates.push_back(n / el);
        }
        out.set("rates", rates);
        return;
    }
    out.set("u0", Energy::systemEnergy(spc, pot, spc.p));
    const int sweeps = in.value("sweeps", 1);
    std::unique_ptr<RdfProbe> rdf;
    if (in.count("rdf")) {
        const auto &r = in["rdf"];
        Tmjson rj = {{"nstep", 1},
                     {"pairs", {{{"name1", "T" + std::to_string(r["t1"].get<int>())},
                                 {"name2", "T" + std::to_string(r["t2"].get<int>())},
                                 {"dim", 3}, {"dr", r["dr"]}, {"file", "rdf.dat"}}}}};
        rdf.reset(new RdfProbe(rj, spc));
    }
    double usum = 0;
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < sweeps; s++) {
        usum += mv.move();
        if (rdf) rdf->sample();
    }
    auto t1 = std::chrono::steady_clock::now();
    double secs = std::chrono::duration<double>(t1 - t0).count();
    out.set("seconds", secs);
    out.set("trials", (double)sweeps * N);
    out.set("trials_per_s", sweeps * (double)N / secs);
    out.set("u_move_sum", usum);
    out.set("u1", Energy::systemEnergy(spc, pot, spc.p));
    if (!bench) {
        out.set("idx", mv.idx);
        out.set("trial_xyz", mv.trial_xyz);
        out.set("du", mv.du);
        out.set("acc", mv.acc);
        std::vector<double> fin;
        for (auto &p : spc.p) { fin.push_back(p.x()); fin.push_back(p.y()); fin.push_back(p.z()); }
        out.set("final_positions", fin);
    }
    if (in.count("state_file")) {
        // the particles were typed in place above: refresh the atom trackers
        // Space::save checks (space.h:388-405), then save (space.h:736-764)
        spc.initTracker();
        spc.save(in["state_file"].get<std::string>());
    }
    if (rdf) {
        std::vector<double> key, cnt;
        for (auto &kv : rdf->raw()) {
            key.push_back(kv.first);
            cnt.push_back(kv.second);
        }
        out.set("rdf_key", key);
        out.set("rdf_count", cnt);
        out.set("rdf_volume", rdf->volume());
    }
}

static void run_ewald_known(const Tmjson &in, Out &out) {
    // unittests.cpp:131-170 with atom types carrying charge (the id-0 type is
    // neutral there, which makes the effective-charge ratio 0/0, ewald.h:539).
    Tmjson j;
    j["system"]["temperature"] = 298.0;
    j["system"]["geometry"]["length"] = 10.0;
    j["atomlist"]["P"] = {{"q", 1.0}, {"r", 0.0}};
    j["atomlist"]["M"] = {{"q", -1.0}, {"r", 0.0}};
    j["moleculelist"]["salt"] = {{"atoms", "P M"}, {"atomic", true}};
    j["energy"]["nonbonded"]["epsr"] = 1.0;
    j["energy"]["nonbonded"]["ewald"] = {{"epsr", 1.0}, {"eps_surf", 1.0}, {"cutoff", 5},
        {"alpha", 0.894427190999916}, {"cutoffK", 11}, {"spherical_sum", true},
        {"update_frequency", 10}, {"debyelength", 1e30}};
    Space<Geometry::Cuboid, PointParticle> spc(j);
    auto pot = Energy::NonbondedEwald<Tspace, Potential::HardSphere>(j);
    spc.p.resize(4);
    for (auto &p : spc.p) p = atom[atom["P"].id];
    spc.p[1] = atom[atom["M"].id];
    Group g(0, 3);
    spc.groupList().push_back(&g);
    spc.p[0] = Point(0, 0, 0);
    spc.p[1] = Point(1, 0, 0);
    spc.p[2] = Point(0, 0, 1);
    spc.p[3] = Point(1, 0, 1);
    spc.p[2].charge = 0; spc.p[3].charge = 0;
    spc.trial = spc.p;
    pot.setSpace(spc);
    // same incremental round trip as the unit test: move particle 0 away and back
    spc.p[0] = Point(0.5, 0, 0);
    spc.trial = spc.p;
    pot.setSpace(spc);
    spc.trial[0] = Point(0, 0, 0);
    Tspace::Change c;
    c.mvGroup[0].push_back(0);
    pot.updateChange(c);
    pot.update(true);
    spc.p = spc.trial;
    out.set("bjerrum", pc::lB(1.0));
    out.set("real", pot.pairpot.first(spc.p[0], spc.p[1], spc.p[1] - spc.p[0]));
    out.set("recip_surf", pot.external(spc.p));
    out.set("self", pot.g_external(spc.p, g));
    out.set("total", Energy::systemEnergy(spc, pot, spc.p));
}

// Places the described particles into spc (types T0, T1, ... as faunus_input
// named them) with the per-type parameters set directly.
static void place_particles(const Tmjson &in, Tspace &spc) {
    int t = 0;
    for (auto &ty : in["types"]) {
        auto &a = atom[atom["T" + std::to_string(t++)].id];
        a.eps = ty["eps"];
        a.sigma = ty["sigma"];
        a.radius = 0.5 * a.sigma;
        a.charge = ty["q"];
        a.dp = ty["dp"];
    }
    const int N = in["positions"].size();
    if ((int)spc.p.size() != N) throw std::runtime_error("particle count mismatch");
    for (int i = 0; i < N; i++) {
        int ty = in["type_ids"][i];
        spc.p[i] = atom[atom["T" + std::to_string(ty)].id];
        spc.p[i].x() = in["positions"][i][0];
        spc.p[i].y() = in["positions"][i][1];
        spc.p[i].z() = in["positions"][i][2];
    }
    spc.trial = spc.p;
    spc.initTracker();
}

template<class Tenergy>
static void run_isobaric(const Tmjson &in, Out &out) {
    Tmjson j = faunus_input(in);
    j["moves"]["isobaric"] = {{"dp", in["volume_dp"]}, {"pressure", in["pressure_mM"]}};
    Tspace spc(j);
    place_particles(in, spc);
    auto pot = Tenergy(j) + Energy::ExternalPressure<Tspace>(j);
    LoggedIsobaric<Tspace> mv(pot, spc, j["moves"]["isobaric"]);
    slump.seed(in.value("seed", 5489u));
    out.set("bjerrum", pot.first.pairpot.first.bjerrumLength());
    out.set("v0", spc.geo.getVolume());
    const int moves = in["moves"];
    std::vector<double> vol;
    double usum = 0;
    for (int m = 0; m < moves; m++) {
        usum += mv.move();
        vol.push_back(spc.geo.getVolume());
    }
    out.set("du", mv.du);
    out.set("acc", mv.acc);
    out.set("volume", vol);
    out.set("u_move_sum", usum);
    std::vector<double> fin;
    for (auto &p : spc.p) { fin.push_back(p.x()); fin.push_back(p.y()); fin.push_back(p.z()); }
    out.set("final_positions", fin);
}

#ifndef FG_HARNESS_NO_MAIN
int main(int argc, char **argv) {
    if (argc != 3) { std::cerr << "usage: ref_harness in.json out.json\n"; return 2; }
    std::ifstream f(argv[1]);
    Tmjson in;
    f >> in;
    Out out;
    std::string mode = in.value("mode", std::string("mc"));
    bool bench = (mode == "bench");
    typedef Energy::NonbondedEwald<Tspace, Potential::WeeksChandlerAndersen> Tewald;
    typedef Energy::Nonbonded<Tspace, Potential::CombinedPairPotential<Potential::DebyeHuckel,
            Potential::LennardJonesMixed<Potential::LorentzBerthelot>>> Tdhlj;
    if (mode == "ewald_known")
        run_ewald_known(in, out);
    else if (mode == "isobaric" && in["model"] == "ewald_wca")
        run_isobaric<Tewald>(in, out);
    else if (mode == "isobaric" && in["model"] == "dh_lj")
        run_isobaric<Tdhlj>(in, out);
    else if (in["model"] == "ewald_wca")
        run_mc<Tewald>(in, out, bench);
    else if (in["model"] == "dh_lj")
        run_mc<Tdhlj>(in, out, bench);
    else { std::cerr << "unknown model\n"; return 2; }
    out.write(argv[2]);
    return 0;
}
#endif
