// The reference's text state format, for interchange with open-Qmin runs:
// multirankSimulation::saveState / loadState for a single rank
// (multirankSimulation.cpp:566-665).  Built on the public C ABI only.
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/qmin_gb300.h"

namespace qmin {
extern thread_local std::string g_last_error;
}

namespace {

std::string state_file(const char *prefix) { return std::string(prefix) + "_x0y0z0.txt"; }

int set_error(int code, const std::string &msg)
{
    qmin::g_last_error = msg;
    return code;
}

}  // namespace

extern "C" int qmin_save_state(qmin_handle h, const char *prefix, int lattice_skip, int defect_kind)
{
    if (!h || !prefix) return set_error(QMIN_EINVAL, "qmin_save_state: null argument");
    int Lx = 0, Ly = 0, Lz = 0;
    int r = qmin_get_sides(h, &Lx, &Ly, &Lz);
    if (r) return r;
    const size_t N = (size_t)Lx * Ly * Lz;
    std::vector<double> Q(5 * N), defects(N);
    std::vector<int32_t> types(N);
    if ((r = qmin_get_state(h, Q.data(), nullptr, nullptr, QMIN_LAYOUT_AOS)) ||
        (r = qmin_get_types(h, types.data())) || (r = qmin_defect_measures(h, defect_kind, defects.data())))
        return r;
    const int stride = lattice_skip < 1 ? 1 : lattice_skip;
    const std::string fn = state_file(prefix);
    FILE *f = std::fopen(fn.c_str(), "w");
    if (!f) return set_error(QMIN_EINVAL, "qmin_save_state: cannot open " + fn);
    bool ok = true;
    for (size_t i = 0; i < N && ok; ++i) {
        const int x = (int)(i % Lx), y = (int)((i / Lx) % Ly), z = (int)(i / ((size_t)Lx * Ly));
        if (x % stride || y % stride || z % stride) continue;
        const double *q = &Q[5 * i];
        // C++ stream insertion of int and double (default precision 6) prints as %d and %g
        ok = std::fprintf(f, "%d\t%d\t%d\t%g\t%g\t%g\t%g\t%g\t%d\t%g\n", x, y, z, q[0], q[1], q[2], q[3], q[4],
                          types[i], defects[i]) > 0;
    }
    ok = std::fclose(f) == 0 && ok;
    return ok ? QMIN_OK : set_error(QMIN_EINVAL, "qmin_save_state: write failed for " + fn);
}

extern "C" int qmin_load_state(qmin_handle h, const char *prefix)
{
    if (!h || !prefix) return set_error(QMIN_EINVAL, "qmin_load_state: null argument");
    int Lx = 0, Ly = 0, Lz = 0;
    int r = qmin_get_sides(h, &Lx, &Ly, &Lz);
    if (r) return r;
    const size_t N = (size_t)Lx * Ly * Lz;
    std::vector<double> Q(5 * N);
    if ((r = qmin_get_state(h, Q.data(), nullptr, nullptr, QMIN_LAYOUT_AOS))) return r;
    const std::string fn = state_file(prefix);
    FILE *f = std::fopen(fn.c_str(), "r");
    if (!f) return set_error(QMIN_EINVAL, "qmin_load_state: cannot open " + fn);
    int x, y, z, t;
    double q[5], defect;
    // the reference's `while (file >> px >> py >> pz >> qxx ... >> type >> defect)` loop
    while (std::fscanf(f, "%d %d %d %lf %lf %lf %lf %lf %d %lf", &x, &y, &z, &q[0], &q[1], &q[2], &q[3], &q[4], &t,
                       &defect) == 10) {
        if (x < 0 || y < 0 || z < 0 || x >= Lx || y >= Ly || z >= Lz) {
            std::fclose(f);
            return set_error(QMIN_EINVAL, "qmin_load_state: a site in " + fn + " lies outside the lattice");
        }
        const size_t i = (size_t)x + (size_t)Lx * ((size_t)y + (size_t)Ly * z);
        for (int k = 0; k < 5; ++k) Q[5 * i + k] = q[k];
    }
    std::fclose(f);
    return qmin_set_positions(h, Q.data(), QMIN_LAYOUT_AOS);
}

extern "C" int qmin_load_field_map(qmin_handle h, const char *prefix, double chi, double mu0, double dchi)
{
    if (!h || !prefix) return set_error(QMIN_EINVAL, "qmin_load_field_map: null argument");
    int Lx = 0, Ly = 0, Lz = 0;
    int r = qmin_get_sides(h, &Lx, &Ly, &Lz);
    if (r) return r;
    const size_t N = (size_t)Lx * Ly * Lz;
    std::vector<double> H(3 * N, 0.0);  // sites not listed keep a zero field
    const std::string fn = state_file(prefix);
    FILE *f = std::fopen(fn.c_str(), "r");
    if (!f) return set_error(QMIN_EINVAL, "qmin_load_field_map: cannot open " + fn);
    double fx, fy, fz, hx, hy, hz;
    // landauDeGennesLC::setSpatiallyVaryingField: `while (file >> fx >> fy >> fz >> Hx >> Hy >> Hz)`,
    // positions read as reals and truncated to int
    while (std::fscanf(f, "%lf %lf %lf %lf %lf %lf", &fx, &fy, &fz, &hx, &hy, &hz) == 6) {
        const int x = (int)fx, y = (int)fy, z = (int)fz;
        if (x < 0 || y < 0 || z < 0 || x >= Lx || y >= Ly || z >= Lz) {
            std::fclose(f);
            return set_error(QMIN_EINVAL, "qmin_load_field_map: a site in " + fn + " lies outside the lattice");
        }
        const size_t i = (size_t)x + (size_t)Lx * ((size_t)y + (size_t)Ly * z);
        H[3 * i] = hx;
        H[3 * i + 1] = hy;
        H[3 * i + 2] = hz;
    }
    std::fclose(f);
    return qmin_set_field_map(h, H.data(), chi, mu0, dchi);
}
