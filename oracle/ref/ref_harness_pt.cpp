// Reference harness for parallel tempering: one process per temperature
// rung running the UNMODIFIED Move::ParallelTempering (move.h:6520-6771)
// between sweeps of Move::AtomicTranslation on Space<Cuboid, PointParticle>
// with Nonbonded<DebyeHuckel + LennardJonesMixed>, built with ENABLE_MPI
// against the stand-in MPI of oracle/ref/fakempi (the ranks are processes,
// messages are files). Test infrastructure only: it produces the golden
// vectors that pin the swap rule of the GPU's parallel tempering.
//
// Input (JSON, the same file for every rank): box, bjerrum, debyelength,
// types [{q, sigma, eps, dp}], type_ids, seed, rounds, sweeps_per_round and
// ranks [{temperature, positions}]. Rung r runs at reduced temperature T_r:
// its Bjerrum length and LJ epsilons are those of the input divided by T_r,
// so its energies are E/T_r in units of kT_r.
//
// Output (JSON per rank): per round the uniform findPartner draws from the
// MPI controller's generator (read from a copy, the generator itself
// untouched), the Metropolis uniform the move then draws from the global
// generator (likewise), uold and unew as the move computed them (this rank's
// energy of its own and of the partner's configuration), whether the
// configuration was exchanged, plus the accepted translations per round and
// the final positions.
#include <faunus/faunus.h>
#include <cmath>
#include <cstdio>
#include <limits>
#include <fstream>
#include <map>

using namespace Faunus;
typedef Space<Geometry::Cuboid, PointParticle> Tspace;
typedef Energy::Nonbonded<Tspace, Potential::CombinedPairPotential<Potential::DebyeHuckel,
        Potential::LennardJonesMixed<Potential::LorentzBerthelot>>> Tdhlj;

struct Out {
    std::map<std::string, std::vector<double>> v;
    void set(const std::string &k, const std::vector<double> &x) { v[k] = x; }
    void write(const char *path) const {
        FILE *f = fopen(path, "w");
        fprintf(f, "{");
        bool first = true;
        for (auto &kv : v) {
            fprintf(f, "%s\n\"%s\": [", first ? "" : ",", kv.first.c_str());
            for (size_t i = 0; i < kv.second.size(); i++) {
                if (std::isnan(kv.second[i])) fprintf(f, "%sNaN", i ? "," : "");   // as Python's json reads it
                else fprintf(f, "%s%.17g", i ? "," : "", kv.second[i]);
            }
            fprintf(f, "]");
            first = false;
        }
        fprintf(f, "\n}\n");
        fclose(f);
    }
};

// What the reference's ParallelTempering computes is read through its public
// hook: setEnergyFunction replaces the energy it calls (usys, by default
// Energy::systemEnergy) with a wrapper that calls systemEnergy and records
// the result. _energyChange calls it for uold (own configuration) and unew
// (the partner's), and tests (unew - uold) + the partner's own difference.
struct EnergyLog {
    std::vector<double> calls;
};
class CountedTranslation : public Move::AtomicTranslation<Tspace> {
    typedef Move::AtomicTranslation<Tspace> base;
  public:
    long accepted = 0;
    CountedTranslation(Energy::Energybase<Tspace> &e, Tspace &s, Tmjson &j) : base(e, s, j) {}
  protected:
    void _acceptMove() override {
        accepted++;
        base::_acceptMove();
    }
};

int main(int argc, char **argv) {
    if (argc != 3) {
        std::cerr << "usage: ref_harness_pt in.json out_prefix (the rank is appended)\n";
        return 2;
    }
    MPI::MPIController mpi;   // MPI_Init: the rank comes from the launcher
    std::ifstream f(argv[1]);
    Tmjson in;
    f >> in;
    const int rank = mpi.rank();
    const Tmjson &me = in["ranks"][rank];
    const double T = me["temperature"];
    const int N = me["positions"].size();

    Tmjson j;
    j["system"]["temperature"] = 298.0;
    j["system"]["geometry"]["length"] = in["box"];
    std::string atoms;
    int t = 0;
    for (auto &ty : in["types"]) {
        std::string name = "T" + std::to_string(t++);
        j["atomlist"][name] = {{"q", ty["q"]}, {"sigma", ty["sigma"]}, {"dp", ty["dp"]}};
    }
    j["atomlist"]["T0"]["Ninit"] = 0;
    j["moleculelist"]["salt"] = {{"atoms", "T0"}, {"Ninit", N}, {"atomic", true}};
    pc::setT(298.0);
    const double lB = in["bjerrum"].get<double>() / T;
    j["energy"]["nonbonded"]["epsr"] = pc::lB(1.0) / lB;
    j["energy"]["nonbonded"]["debyelength"] = in["debyelength"];
    j["moves"]["atomtranslate"]["salt"] = {{"peratom", true}};
    j["moves"]["temper"] = {{"prob", 1.0}, {"format", "XYZQI"}};
    Tspace spc(j);
    t = 0;
    for (auto &ty : in["types"]) {
        auto &a = atom[atom["T" + std::to_string(t++)].id];
        a.eps = ty["eps"].get<double>() / T;
        a.sigma = ty["sigma"];
        a.radius = 0.5 * a.sigma;
        a.charge = ty["q"];
        a.dp = ty["dp"];
    }
    if ((int)spc.p.size() != N) throw std::runtime_error("particle count mismatch");
    for (int i = 0; i < N; i++) {
        const int ty = in["type_ids"][i];
        spc.p[i] = atom[atom["T" + std::to_string(ty)].id];
        for (int a = 0; a < 3; a++) spc.p[i][a] = me["positions"][i][a];
    }
    spc.trial = spc.p;
    Tdhlj pot(j);
    CountedTranslation mv(pot, spc, j["moves"]["atomtranslate"]);
    Move::ParallelTempering<Tspace> temper(pot, spc, j["moves"]["temper"], mpi);
    EnergyLog elog;
    temper.setEnergyFunction([&elog](Tspace &s, Energy::Energybase<Tspace> &e, const Tspace::ParticleVector &p) {
        const double u = Energy::systemEnergy(s, e, p);
        elog.calls.push_back(u);
        return u;
    });
    slump.seed(in["seed"].get<unsigned>());   // the same stream on every rank, as the reference runs it

    Out out;
    std::vector<double> u_dir, u_acc, uold, unew, acc, tr_acc;
    const int rounds = in["rounds"], sweeps = in["sweeps_per_round"];
    out.set("u0", {Energy::systemEnergy(spc, pot, spc.p)});
    out.set("bjerrum", {pot.pairpot.first.bjerrumLength()});
    for (int r = 0; r < rounds; r++) {
        const long a0 = mv.accepted;
        for (int s = 0; s < sweeps; s++) mv.move();
        tr_acc.push_back((double)(mv.accepted - a0));
        RandomTwister<> peek_dir(static_cast<const RandomTwister<> &>(mpi.random));
        RandomTwister<> peek_acc(static_cast<const RandomTwister<> &>(slump));
        u_dir.push_back(peek_dir());
        u_acc.push_back(peek_acc());
        const Tspace::ParticleVector before = spc.p;
        elog.calls.clear();
        temper.move();
        // with a partner the move calls the energy twice (uold, unew); a rank
        // at the end of the ladder without one calls it never (dU = infinity)
        uold.push_back(elog.calls.size() == 2 ? elog.calls[0] : Energy::systemEnergy(spc, pot, before));
        unew.push_back(elog.calls.size() == 2 ? elog.calls[1] : std::numeric_limits<double>::quiet_NaN());
        bool changed = false;
        for (int i = 0; i < N && !changed; i++)
            for (int a = 0; a < 3; a++) changed = changed || spc.p[i][a] != before[i][a];
        acc.push_back(changed ? 1.0 : 0.0);
    }
    out.set("u_direction", u_dir);
    out.set("u_accept", u_acc);
    out.set("uold", uold);
    out.set("unew", unew);
    out.set("acc", acc);
    out.set("translations_accepted", tr_acc);
    out.set("temperature", {T});
    out.set("u1", {Energy::systemEnergy(spc, pot, spc.p)});
    std::vector<double> fin;
    for (auto &p : spc.p) {
        fin.push_back(p.x());
        fin.push_back(p.y());
        fin.push_back(p.z());
    }
    out.set("final_positions", fin);
    out.write((std::string(argv[2]) + std::to_string(rank) + ".json").c_str());
    return 0;
}
