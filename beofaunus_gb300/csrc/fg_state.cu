// State files in the reference's text format (included by fg_api.cu; host
// code only). Space::save/load (space.h:736-764, 807-880):
//
//   Lx Ly Lz
//   N
//   N particle records
//   G
//   G group records: front back molId molsize cm_x cm_y cm_z  (group.h:388-407)
//   randomstate
//   <std::mt19937 state, as operator<< writes it>
//
// PointParticle record (point.h:544-566): x y z charge radius mw id hydrophobic.
// DipoleParticle record (point.h:649-666): the PointParticle record, then the
// dipole unit vector (3), its scalar, the induced dipole (3) and the
// polarisability and its companion tensor, six upper-triangle numbers each.
// Records are whitespace-separated tokens, so line layout does not matter to
// a reader. Numbers are written with 16 significant digits, the precision
// Space::save sets (digits10 + 1).
#include <fstream>
#include <sstream>

namespace {

constexpr int kStatePoint = 0, kStateDipole = 1;

bool read_tokens(std::istream &in, double *v, int n) {
    for (int i = 0; i < n; i++)
        if (!(in >> v[i])) return false;
    return true;
}

}  // namespace

extern "C" {

int fg_state_read(const char *path, int32_t kind, int32_t n_max, double *box, int32_t *n, double *xyz,
                  double *charge, double *radius, double *mw, int32_t *ids, int32_t *hydrophobic, double *mu_unit,
                  double *mu_scalar, int32_t g_max, int32_t *n_groups, int32_t *groups, double *group_cm) {
    if (!path || !n) return fail(FG_ERR_INVALID, "null argument");
    if (kind != kStatePoint && kind != kStateDipole) return fail(FG_ERR_INVALID, "kind must be 0 or 1");
    std::ifstream f(path);
    if (!f) return fail(FG_ERR_INVALID, "cannot open %s", path);
    double L[3];
    long long np = 0;
    if (!read_tokens(f, L, 3) || !(f >> np) || np < 0) return fail(FG_ERR_INVALID, "%s: bad header", path);
    if (np > n_max) return fail(FG_ERR_CAPACITY, "%s holds %lld particles, room for %d", path, np, n_max);
    if (box)
        for (int a = 0; a < 3; a++) box[a] = L[a];
    const int rec = kind == kStateDipole ? 27 : 8;
    std::vector<double> r(rec);
    for (long long i = 0; i < np; i++) {
        if (!read_tokens(f, r.data(), rec)) return fail(FG_ERR_INVALID, "%s: particle %lld incomplete", path, i);
        if (xyz)
            for (int a = 0; a < 3; a++) xyz[3 * i + a] = r[a];
        if (charge) charge[i] = r[3];
        if (radius) radius[i] = r[4];
        if (mw) mw[i] = r[5];
        if (ids) ids[i] = (int32_t)r[6];
        if (hydrophobic) hydrophobic[i] = (int32_t)r[7];
        if (kind == kStateDipole) {
            if (mu_unit)
                for (int a = 0; a < 3; a++) mu_unit[3 * i + a] = r[8 + a];
            if (mu_scalar) mu_scalar[i] = r[11];
        }
    }
    *n = (int32_t)np;
    long long ng = 0;
    if (!(f >> ng) || ng < 0) return fail(FG_ERR_INVALID, "%s: no group count", path);
    if (ng > g_max && (groups || group_cm)) return fail(FG_ERR_CAPACITY, "%s holds %lld groups, room for %d", path, ng, g_max);
    for (long long g = 0; g < ng; g++) {
        double v[7];
        if (!read_tokens(f, v, 7)) return fail(FG_ERR_INVALID, "%s: group %lld incomplete", path, g);
        if (groups)
            for (int k = 0; k < 4; k++) groups[4 * g + k] = (int32_t)v[k];
        if (group_cm)
            for (int a = 0; a < 3; a++) group_cm[3 * g + a] = v[4 + a];
    }
    if (n_groups) *n_groups = (int32_t)ng;
    return FG_OK;   // the random state that may follow belongs to the reference's engine
}

int fg_state_write(const char *path, int32_t kind, const double *box, int32_t n, const double *xyz,
                   const double *charge, const double *radius, const double *mw, const int32_t *ids,
                   const int32_t *hydrophobic, const double *mu_unit, const double *mu_scalar, int32_t n_groups,
                   const int32_t *groups, const double *group_cm, uint32_t rng_seed) {
    if (!path || !box || !xyz || !ids || n < 0 || n_groups < 0 || (n_groups > 0 && !groups))
        return fail(FG_ERR_INVALID, "null or negative argument");
    if (kind != kStatePoint && kind != kStateDipole) return fail(FG_ERR_INVALID, "kind must be 0 or 1");
    std::ostringstream o;
    o.precision(16);
    o << box[0] << " " << box[1] << " " << box[2] << "\n" << n << "\n";
    for (int i = 0; i < n; i++) {
        o << xyz[3 * i] << " " << xyz[3 * i + 1] << " " << xyz[3 * i + 2] << " " << (charge ? charge[i] : 0.0)
          << " " << (radius ? radius[i] : 0.0) << " " << (mw ? mw[i] : 1.0) << " " << ids[i] << " "
          << (hydrophobic ? hydrophobic[i] : 0);
        if (kind == kStateDipole) {
            const double m0 = mu_unit ? mu_unit[3 * i] : 0.0, m1 = mu_unit ? mu_unit[3 * i + 1] : 0.0,
                         m2 = mu_unit ? mu_unit[3 * i + 2] : 0.0;
            o << " " << m0 << " " << m1 << " " << m2 << " " << (mu_scalar ? mu_scalar[i] : 0.0)
              << " 0 0 0 0 0 0 0 0 0 0 0 0 0 0 0";   // no induced dipole, zero tensors
        }
        o << "\n";
    }
    o << n_groups << "\n";
    for (int g = 0; g < n_groups; g++) {
        o << groups[4 * g] << " " << groups[4 * g + 1] << " " << groups[4 * g + 2] << " " << groups[4 * g + 3];
        for (int a = 0; a < 3; a++) o << " " << (group_cm ? group_cm[3 * g + a] : 0.0);
        o << "\n";
    }
    // a fresh engine for whoever continues from this state (the device
    // streams here are counter-based and have no mt19937 state)
    std::mt19937 eng(rng_seed);
    o << "randomstate\n" << eng << "\n";
    std::ofstream f(path);
    if (!f || !(f << o.str())) return fail(FG_ERR_INVALID, "cannot write %s", path);
    return FG_OK;
}

}  // extern "C"
