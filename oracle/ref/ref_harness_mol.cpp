// Reference harness, rigid dipolar molecules: drives the UNMODIFIED Faunus
// classes (built from the reference's own sources by oracle/ref/Makefile) and
// writes what they compute to a JSON file. Test infrastructure only: its
// output pins the FP64 oracle (oracle/fg_oracle_mol.cpp).
//
// Space<Cuboid, DipoleParticle> with one molecule kind (a structure file the
// harness writes), energy NonbondedVector over
//   CombinedPairPotential<CombinedPairPotential<CoulombGalore, LennardJonesLB>,
//                         CombinedPairPotential<IonDipole, DipoleDipoleGalore>>
// with "coulombtype": "reactionfield", and the TranslateRotate move
// ("moltransrot", "permol") as the reference's example programs use them
// (stockmayer.cpp, water2.cpp: Space(json) -> energy -> moves -> move()).
// Particle types, positions and dipoles are overwritten after construction
// with the harness input, then every group's mass centre is recomputed.
//
// Modes: "mol_mc" logs every trial (group, trial position of its first
// site, dU, accepted); "mol_pairs" evaluates the pair potential on listed
// site pairs; "mol_bench" times the trials.
#include <faunus/faunus.h>
#include <chrono>
#include <cstdio>
#include <fstream>
#include <map>

using namespace Faunus;
typedef Space<Geometry::Cuboid, DipoleParticle> Tspace;
typedef Potential::CombinedPairPotential<
    Potential::CombinedPairPotential<Potential::CoulombGalore, Potential::LennardJonesLB>,
    Potential::CombinedPairPotential<Potential::IonDipole, Potential::DipoleDipoleGalore>>
    Tpair;
typedef Energy::NonbondedVector<Tspace, Tpair> Tenergy;

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

// Logs what TranslateRotate does; every override calls the reference's own
// implementation (move.h:1620-1705).
template<class Tsp>
class LoggedTranslateRotate : public Move::TranslateRotate<Tsp> {
    typedef Move::TranslateRotate<Tsp> base;
  public:
    bool log = true;
    std::vector<int> grp;
    std::vector<double> first_xyz, first_mu, du;
    std::vector<int> acc;
    LoggedTranslateRotate(Energy::Energybase<Tsp> &e, Tsp &s, Tmjson &j) : base(e, s, j) {}
  protected:
    void _trialMove() override {
        base::_trialMove();
        if (log) {
            int g = this->spc->findIndex(this->igroup);
            grp.push_back(g);
            auto &t = this->spc->trial[this->igroup->front()];
            first_xyz.push_back(t.x()); first_xyz.push_back(t.y()); first_xyz.push_back(t.z());
            first_mu.push_back(t.mu().x()); first_mu.push_back(t.mu().y()); first_mu.push_back(t.mu().z());
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

static Tmjson faunus_input(const Tmjson &in, const std::string &aam) {
    Tmjson j;
    const double T = in.value("temperature", 298.0);
    j["system"]["temperature"] = T;
    j["system"]["geometry"]["length"] = in["box"];
    int t = 0;
    for (auto &ty : in["types"]) {
        std::string name = "T" + std::to_string(t++);
        j["atomlist"][name] = {{"q", ty["q"]}, {"sigma", ty["sigma"]}};
    }
    j["moleculelist"]["mol"] = {{"structure", aam}, {"Ninit", in["n_mol"]}};
    pc::setT(T);
    const double epsr = pc::lB(1.0) / in["bjerrum"].get<double>();
    j["energy"]["nonbonded"] = {{"coulombtype", "reactionfield"}, {"cutoff", in["cutoff"]}, {"epsr", epsr},
                                {"eps_rf", in["eps_rf"]}};
    j["moves"]["moltransrot"]["mol"] = {{"dp", in["dp"]}, {"dprot", in["dprot"]}, {"permol", true}};
    j["moves"]["moltransrot"]["center_rotation"] = in.value("center_rotation", true);
    return j;
}

// Structure file of one molecule (FormatAAM, io.h): name num x y z q mw radius
static void write_aam(const std::string &path, int gs) {
    FILE *f = fopen(path.c_str(), "w");
    fprintf(f, "%d\n", gs);
    for (int s = 0; s < gs; s++) fprintf(f, "T0 %d %.1f 0.0 0.0 0.0 1.0 1.0\n", s + 1, 4.0 * s);
    fclose(f);
}

static void setup(Tspace &spc, const Tmjson &in) {
    int t = 0;
    for (auto &ty : in["types"]) {
        auto &a = atom[atom["T" + std::to_string(t++)].id];
        a.eps = ty["eps"];        // kT, straight into the atom map before the potential reads it
        a.sigma = ty["sigma"];
        a.radius = 0.5 * a.sigma;
        a.charge = ty["q"];
        a.mw = 1.0;
    }
    const int N = in["positions"].size();
    if ((int)spc.p.size() != N) throw std::runtime_error("site count mismatch");
    for (int i = 0; i < N; i++) {
        int ty = in["type_ids"][i];
        spc.p[i] = atom[atom["T" + std::to_string(ty)].id];
        spc.p[i].x() = in["positions"][i][0];
        spc.p[i].y() = in["positions"][i][1];
        spc.p[i].z() = in["positions"][i][2];
        spc.p[i].mu() = Point(in["mu"][i][0], in["mu"][i][1], in["mu"][i][2]);
        spc.p[i].muscalar() = in["muscalar"][i];
        spc.p[i].mup() = spc.p[i].mu() * spc.p[i].muscalar();
    }
    spc.trial = spc.p;
    for (auto g : spc.groupList()) g->setMassCenter(spc);
}

int main(int argc, char **argv) {
    if (argc != 3) { std::cerr << "usage: ref_harness_mol in.json out.json\n"; return 2; }
    std::ifstream f(argv[1]);
    Tmjson in;
    f >> in;
    Out out;
    const std::string mode = in.value("mode", std::string("mol_mc"));
    const std::string aam = std::string(argv[2]) + ".mol.aam";
    write_aam(aam, in["molsize"]);
    Tmjson j = faunus_input(in, aam);
    Tspace spc(j);
    setup(spc, in);
    Tenergy pot(j);
    if (mode == "mol_pairs") {
        pot.setSpace(spc);
        std::vector<double> u;
        for (auto &pr : in["pairs"]) {
            int a = pr[0], b = pr[1];
            u.push_back(pot.i2i(spc.p, a, b));
        }
        out.set("u", u);
        out.set("total", Energy::systemEnergy(spc, pot, spc.p));
        out.set("bjerrum", pc::lB(j["energy"]["nonbonded"]["epsr"].get<double>()));
        out.write(argv[2]);
        return 0;
    }
    LoggedTranslateRotate<Tspace> mv(pot, spc, j["moves"]["moltransrot"]);  // calls pot.setSpace(spc)
    mv.log = (mode != "mol_bench");
    slump.seed(in.value("seed", 5489u));
    std::vector<double> cm0;
    for (auto g : spc.groupList()) { cm0.push_back(g->cm.x()); cm0.push_back(g->cm.y()); cm0.push_back(g->cm.z()); }
    out.set("cm0", cm0);
    out.set("u0", Energy::systemEnergy(spc, pot, spc.p));
    const int sweeps = in.value("sweeps", 1);
    double usum = 0;
    auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < sweeps; s++) usum += mv.move();
    auto t1 = std::chrono::steady_clock::now();
    const double secs = std::chrono::duration<double>(t1 - t0).count();
    const double trials = (double)sweeps * spc.groupList().size();
    out.set("seconds", secs);
    out.set("trials", trials);
    out.set("trials_per_s", trials / secs);
    out.set("u_move_sum", usum);
    out.set("u1", Energy::systemEnergy(spc, pot, spc.p));
    if (mv.log) {
        out.set("group", mv.grp);
        out.set("first_xyz", mv.first_xyz);
        out.set("first_mu", mv.first_mu);
        out.set("du", mv.du);
        out.set("acc", mv.acc);
        std::vector<double> fin, fmu, cm1;
        for (auto &p : spc.p) {
            fin.push_back(p.x()); fin.push_back(p.y()); fin.push_back(p.z());
            fmu.push_back(p.mu().x()); fmu.push_back(p.mu().y()); fmu.push_back(p.mu().z());
        }
        for (auto g : spc.groupList()) { cm1.push_back(g->cm.x()); cm1.push_back(g->cm.y()); cm1.push_back(g->cm.z()); }
        out.set("final_positions", fin);
        out.set("final_mu", fmu);
        out.set("final_cm", cm1);
    }
    out.write(argv[2]);
    return 0;
}
