// Host-side initial conditions and object builders.  The reference runs all
// of these on the host even in GPU runs (openQmin.cpp:261-268); they are
// one-time set-up, not part of the minimisation hot path.
#include <cmath>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/qmin_gb300.h"

namespace {

const double kPi = 3.14159265358979323846;  // inc/std_include.h:37

// qTensorFromDirector (inc/qTensorFunctions.h:34-51)
void q_from_director(double nx, double ny, double nz, double S0, double *q)
{
    double scale = std::sqrt(nx * nx + ny * ny + nz * nz);
    if (scale == 0) {
        q[0] = -0.5 * S0;
        q[3] = -0.5 * S0;
    } else if (scale != 1) {
        nx /= scale;
        ny /= scale;
        nz /= scale;
    }
    q[0] = 1.5 * S0 * (nx * nx - 1.0 / 3.0);
    q[1] = 1.5 * S0 * nx * ny;
    q[2] = 1.5 * S0 * nx * nz;
    q[3] = 1.5 * S0 * (ny * ny - 1.0 / 3.0);
    q[4] = 1.5 * S0 * ny * nz;
}

int wrap(int x, int m)  // inc/functions.h:299-307
{
    int a = x;
    if (x >= m) a = x % m;
    while (a < 0) a += m;
    return a;
}

// cubicLattice::createBoundaryObject (cubicLattice.cpp:267-294) after the
// periodic wrap of multirankSimulation::createMultirankBoundaryObject
// (multirankSimulationBoundaries.cpp:512-543)
int add_object(int Lx, int Ly, int Lz, const std::vector<int> &xyz, const std::vector<double> &qs, int kind,
               double W, double S0, double *Q, int32_t *types, qmin_object *objs, int *nobj)
{
    if (*nobj >= 127) return QMIN_EINVAL;
    const int j = *nobj + 1;
    const size_t n = xyz.size() / 3;
    std::vector<size_t> idx(n);
    for (size_t s = 0; s < n; ++s) {
        int x = wrap(xyz[3 * s], Lx), y = wrap(xyz[3 * s + 1], Ly), z = wrap(xyz[3 * s + 2], Lz);
        idx[s] = (size_t)x + (size_t)Lx * ((size_t)y + (size_t)Ly * z);
        for (int k = 0; k < 5; ++k) Q[5 * idx[s] + k] = qs[5 * s + k];
    }
    for (size_t s = 0; s < n; ++s) types[idx[s]] = j;
    for (size_t s = 0; s < n; ++s) {
        const size_t i = idx[s];
        const int x = (int)(i % Lx), y = (int)((i / Lx) % Ly), z = (int)(i / ((size_t)Lx * Ly));
        const int nb[6][3] = {{x - 1, y, z}, {x + 1, y, z}, {x, y - 1, z}, {x, y + 1, z}, {x, y, z - 1}, {x, y, z + 1}};
        for (int k = 0; k < 6; ++k) {
            size_t m = (size_t)wrap(nb[k][0], Lx) + (size_t)Lx * ((size_t)wrap(nb[k][1], Ly) + (size_t)Ly * wrap(nb[k][2], Lz));
            if (types[m] < 1) types[m] = -1;
        }
    }
    objs[*nobj].kind = kind;
    objs[*nobj].W = W;
    objs[*nobj].S0 = S0;
    *nobj = j;
    return QMIN_OK;
}

}  // namespace

extern "C" {

// noiseSource (noiseSource.cpp:16-25, 38-46) drawing as
// qTensorLatticeModel::setNematicQTensorRandomly (qTensorLatticeModel.cpp:134-162)
int qmin_host_random_nematic(int Lx, int Ly, int Lz, int seed, double S0, double *Q)
{
    if (!Q || Lx < 1 || Ly < 1 || Lz < 1) return QMIN_EINVAL;
    std::mt19937 gen(seed);
    auto uniform = [&gen]() {
        std::uniform_real_distribution<double> u(0.0, 1.0);
        return u(gen);
    };
    (void)uniform();  // global theta
    (void)uniform();  // global phi
    const size_t N = (size_t)Lx * Ly * Lz;
    for (size_t i = 0; i < N; ++i) {
        double theta = std::acos(2.0 * uniform() - 1);
        double phi = 2.0 * kPi * uniform();
        q_from_director(std::cos(phi) * std::sin(theta), std::sin(phi) * std::sin(theta), std::cos(theta), S0,
                        Q + 5 * i);
    }
    return QMIN_OK;
}

int qmin_host_add_wall(int Lx, int Ly, int Lz, int xyz, int plane, int kind, double W, double S0, double *Q,
                       int32_t *types, qmin_object *objs, int *nobj)
{
    if (!Q || !types || !objs || !nobj || xyz < 0 || xyz > 2) return QMIN_EINVAL;
    if (kind != QMIN_HOMEOTROPIC && kind != QMIN_DEGENERATE_PLANAR) return QMIN_EINVAL;
    double q[5] = {0, 0, 0, 0, 0};
    if (kind == QMIN_HOMEOTROPIC) {
        if (xyz == 0) { q[0] = S0; q[3] = -0.5 * S0; }
        else if (xyz == 1) { q[0] = -0.5 * S0; q[3] = S0; }
        else { q[0] = -0.5 * S0; q[3] = -0.5 * S0; }
    } else {
        q[xyz] = 1.0;
    }
    const int s1 = xyz == 0 ? Ly : Lx, s2 = xyz == 2 ? Ly : Lz;
    std::vector<int> pos;
    std::vector<double> qs;
    pos.reserve((size_t)3 * s1 * s2);
    qs.reserve((size_t)5 * s1 * s2);
    for (int a = 0; a < s1; ++a)
        for (int b = 0; b < s2; ++b) {
            if (xyz == 0) pos.insert(pos.end(), {plane, a, b});
            else if (xyz == 1) pos.insert(pos.end(), {a, plane, b});
            else pos.insert(pos.end(), {a, b, plane});
            qs.insert(qs.end(), q, q + 5);
        }
    return add_object(Lx, Ly, Lz, pos, qs, kind, W, S0, Q, types, objs, nobj);
}

int qmin_host_add_sphere(int Lx, int Ly, int Lz, const double center[3], double radius, int kind, double W,
                         double S0, double *Q, int32_t *types, qmin_object *objs, int *nobj)
{
    if (!Q || !types || !objs || !nobj || !center || !(radius > 0)) return QMIN_EINVAL;
    if (kind != QMIN_HOMEOTROPIC && kind != QMIN_DEGENERATE_PLANAR) return QMIN_EINVAL;
    std::vector<int> pos;
    std::vector<double> qs;
    double q[5] = {0, 0, 0, 0, 0};
    for (int x = (int)std::ceil(center[0] - radius); x < std::floor(center[0] + radius); ++x)
        for (int y = (int)std::ceil(center[1] - radius); y < std::floor(center[1] + radius); ++y)
            for (int z = (int)std::ceil(center[2] - radius); z < std::floor(center[2] + radius); ++z) {
                const double dx = x - center[0], dy = y - center[1], dz = z - center[2];
                if (dx * dx + dy * dy + dz * dz < radius * radius) {
                    pos.insert(pos.end(), {x, y, z});
                    if (kind == QMIN_HOMEOTROPIC) {
                        q_from_director(dx, dy, dz, S0, q);
                    } else {
                        const double nrm = std::sqrt(dx * dx + dy * dy + dz * dz);
                        q[0] = dx / nrm;
                        q[1] = dy / nrm;
                        q[2] = dz / nrm;
                    }
                    qs.insert(qs.end(), q, q + 5);
                }
            }
    return add_object(Lx, Ly, Lz, pos, qs, kind, W, S0, Q, types, objs, nobj);
}

}  // extern "C"

// multirankSimulation::createBoundaryFromFile (multirankSimulationBoundaries.cpp:43-96)
// for one rank: every object's sites go through add_object (periodic wrap, Q
// set from the file, neighbours marked -1).
extern "C" int qmin_host_boundary_file(int Lx, int Ly, int Lz, const char *path, double *Q, int32_t *types,
                                       qmin_object *objs, int max_objs, int *nobj)
{
    if (!path || !Q || !types || !objs || !nobj || Lx < 1 || Ly < 1 || Lz < 1) return QMIN_EINVAL;
    std::ifstream in(path);
    if (!in) return QMIN_EINVAL;
    std::string line;
    int count = 0;
    if (!std::getline(in, line) || !(std::istringstream(line) >> count) || count < 0) return QMIN_EINVAL;
    for (int o = 0; o < count; ++o) {
        int kind = 0, n = 0;
        double W = 0.0, S0 = 0.0;
        if (!std::getline(in, line)) return QMIN_EINVAL;
        std::istringstream hs(line);
        if (!(hs >> kind >> W >> S0 >> n) || n < 0) return QMIN_EINVAL;
        std::vector<int> xyz;
        std::vector<double> qs;
        xyz.reserve(3 * (size_t)n);
        qs.reserve(5 * (size_t)n);
        for (int e = 0; e < n && std::getline(in, line); ++e) {
            std::istringstream ls(line);
            int x, y, z;
            double c[5];
            if (!(ls >> x >> y >> z >> c[0] >> c[1] >> c[2] >> c[3] >> c[4])) return QMIN_EINVAL;
            xyz.insert(xyz.end(), {x, y, z});
            qs.insert(qs.end(), c, c + 5);
        }
        if (*nobj >= max_objs) return QMIN_EINVAL;
        const int r = add_object(Lx, Ly, Lz, xyz, qs, kind == 0 ? QMIN_HOMEOTROPIC : QMIN_DEGENERATE_PLANAR, W, S0, Q,
                                 types, objs, nobj);
        if (r) return r;
    }
    return QMIN_OK;
}
