// Runs the drop-in adapter (include/faunus_gb300_energy.hpp) inside the
// reference's own, unmodified move classes: the same Space and JSON input as
// the reference harness's "mc" mode (ref_harness.cpp), with the reference's
// energy term replaced by Energy::NonbondedGPU (the GB300 library behind the
// Energybase interface, energy.h:54-224). Built by `make -C oracle/ref
// adapter` against the reference's sources and libfaunus_gb300.so; needs a
// GPU. Test infrastructure only.
//
// Modes (input key "mode"):
//   "movebase" : Move::AtomicTranslation (move.h:818-901) driven by
//                Movebase::move (move.h:515-555) calls updateChange ->
//                energyChange -> update on the adapter for every trial (the
//                plain per-trial path, fg_trial_du / fg_commit). Logs every
//                trial like the harness: index, trial position, dU, accept.
//   "device"   : translateOnDevice: the same draws from the global `slump`,
//                then whole sweeps on the device (fg_sweep).
// Output: the same keys as the harness's "mc" mode (u0, u1, final_positions,
// and for "movebase" idx, trial_xyz, du, acc).
#define FG_HARNESS_NO_MAIN
#include "ref_harness.cpp"

#include "faunus_gb300_energy.hpp"

template <class Tpot>
static void run_adapter(const Tmjson &in, Out &out, const fg_params &P, Tspace &spc, Tmjson &j) {
    Tpot pot(P);
    const int N = spc.p.size();
    const int sweeps = in.value("sweeps", 1);
    const std::string mode = in.value("mode", std::string("movebase"));
    if (mode == "movebase") {
        LoggedTranslation<Tspace> mv(pot, spc, j["moves"]["atomtranslate"]);   // calls pot.setSpace(spc)
        slump.seed(in.value("seed", 5489u));
        out.set("u0", Energy::systemEnergy(spc, pot, spc.p));
        double usum = 0;
        for (int s = 0; s < sweeps; s++) usum += mv.move();
        out.set("u_move_sum", usum);
        out.set("idx", mv.idx);
        out.set("trial_xyz", mv.trial_xyz);
        out.set("du", mv.du);
        out.set("acc", mv.acc);
    } else {
        pot.setSpace(spc);
        slump.seed(in.value("seed", 5489u));
        out.set("u0", Energy::systemEnergy(spc, pot, spc.p));
        out.set("u_move_sum", Energy::translateOnDevice(spc, pot, sweeps * N));
    }
    out.set("u1", Energy::systemEnergy(spc, pot, spc.p));
    std::vector<double> fin;
    for (auto &p : spc.p) {
        fin.push_back(p.x());
        fin.push_back(p.y());
        fin.push_back(p.z());
    }
    out.set("final_positions", fin);
}

int main(int argc, char **argv) {
    if (argc != 3) {
        std::cerr << "usage: adapter_run in.json out.json\n";
        return 2;
    }
    std::ifstream f(argv[1]);
    Tmjson in;
    f >> in;
    Out out;
    Tmjson j = faunus_input(in);
    Tspace spc(j);
    fill_space(in, spc);
    try {
        if (in["model"] == "ewald_wca")
            run_adapter<Energy::NonbondedGPU<Tspace>>(in, out, Energy::gpuParamsEwaldWCA(j), spc, j);
        else if (in["model"] == "dh_lj")
            run_adapter<Energy::NonbondedGPU<Tspace>>(in, out, Energy::gpuParamsDHLJ(j), spc, j);
        else {
            std::cerr << "unknown model\n";
            return 2;
        }
    } catch (std::exception &e) {
        std::cerr << e.what() << "\n";
        return 1;
    }
    out.write(argv[2]);
    return 0;
}
