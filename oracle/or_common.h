// Shared pieces of the FP64 oracle -- TEST INFRASTRUCTURE (see fg_oracle.cpp).
#ifndef FG_ORACLE_COMMON_H
#define FG_ORACLE_COMMON_H
#include <cmath>
#include <cstdint>
#include <random>

namespace orc {

const double PI = std::acos(-1.0);  // pc::pi, physconst.h:52

struct V3 { double x, y, z; };

// ---------------------------------------------------------------- geometry
// Geometry::Cuboid (geometry.h:468-547)
struct Cuboid {
    double L[3], Lh[3], Linv[3];
    void set(const double *len) {
        for (int d = 0; d < 3; d++) { L[d] = len[d]; Lh[d] = 0.5 * len[d]; Linv[d] = 1.0 / len[d]; }
    }
    static int anint(double x) { return int(x > 0. ? x + .5 : x - .5); }  // geometry.h:56-59
    // vdist, geometry.h:519-537
    V3 vdist(const V3 &a, const V3 &b) const {
        double r[3] = {a.x - b.x, a.y - b.y, a.z - b.z};
        for (int d = 0; d < 3; d++) {
            if (r[d] > Lh[d]) r[d] -= L[d];
            else if (r[d] < -Lh[d]) r[d] += L[d];
        }
        return {r[0], r[1], r[2]};
    }
    // sqdist, geometry.h:507-517
    double sqdist(const V3 &a, const V3 &b) const {
        double d[3] = {std::fabs(a.x - b.x), std::fabs(a.y - b.y), std::fabs(a.z - b.z)};
        for (int k = 0; k < 3; k++)
            if (d[k] > Lh[k]) d[k] -= 2 * Lh[k];
        return d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    }
    // boundary, geometry.h:539-547
    void boundary(V3 &a) const {
        if (std::fabs(a.x) > Lh[0]) a.x -= L[0] * anint(a.x * Linv[0]);
        if (std::fabs(a.y) > Lh[1]) a.y -= L[1] * anint(a.y * Linv[1]);
        if (std::fabs(a.z) > Lh[2]) a.z -= L[2] * anint(a.z * Linv[2]);
    }
    double volume() const { return L[0] * L[1] * L[2]; }
};

// ---------------------------------------------------------------- RNG
// RandomTwister (slump.h:24-126): std::mt19937 with per-call
// uniform_int_distribution<int>(min,max) and uniform_real_distribution<double>(0,1).
struct Twister {
    std::mt19937 eng;
    std::uniform_real_distribution<double> dist{0, 1};
    explicit Twister(uint32_t s) { eng.seed(s); }
    int range(int a, int b) { std::uniform_int_distribution<int> d(a, b); return d(eng); }
    double operator()() { return dist(eng); }
};


}  // namespace orc

#endif
