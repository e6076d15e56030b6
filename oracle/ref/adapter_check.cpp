// Compile-only check that the drop-in adapter (include/faunus_gb300_energy.hpp)
// builds against the reference's own headers, instantiated for the Space type
// of the reference's examples. Used by tests/test_adapter_compile.py.
#include <faunus/faunus.h>
#include <faunus/ewald.h>

#include "faunus_gb300_energy.hpp"

using namespace Faunus;
typedef Space<Geometry::Cuboid, PointParticle> Tspace;
template class Faunus::Energy::NonbondedGPU<Tspace>;
template double Faunus::Energy::translateOnDevice<Tspace>(Tspace &, Faunus::Energy::NonbondedGPU<Tspace> &, int);
typedef Space<Geometry::Cuboid, DipoleParticle> Tdspace;
template class Faunus::Energy::NonbondedEwaldDipoleGPU<Tdspace>;
template double Faunus::Energy::dipoleMovesOnDevice<Tdspace>(Tdspace &, Faunus::Energy::NonbondedEwaldDipoleGPU<Tdspace> &,
                                                            int, bool);

int main(int argc, char **argv) {
    if (argc < 2) return 0;
    Tmjson j = openjson(argv[1]);
    Tspace spc(j);
    Energy::NonbondedGPU<Tspace> pot(Energy::gpuParamsEwaldWCA(j));
    Move::AtomicTranslation<Tspace> mv(pot, spc, j["moves"]["atomtranslate"]);
    return mv.move() == mv.move() ? 0 : 1;
}
