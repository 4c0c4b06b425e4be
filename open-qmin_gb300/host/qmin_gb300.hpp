// C++ host layer over the qmin_gb300 C ABI, shaped like open-Qmin's own
// classes so that C++ code written against the reference reads the same:
//   qTensorLatticeModel (src/model/qTensorLatticeModel.h), landauDeGennesLC
//   (src/forces/landauDeGennesLC.h:34-93), energyMinimizerFIRE
//   (src/updaters/energyMinimizerFIRE.h:20-112), energyMinimizerAdam,
//   energyMinimizerNesterovAG, energyMinimizerLoLBFGS and a single-domain
//   multirankSimulation (src/simulation/multirankSimulation.h:15-158).
// Set-up runs on the host as in the reference; finalizeObjects() moves the
// state to the GPU, where it stays.  Errors throw qmin_gb300::error.
#pragma once
#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "qmin_gb300.h"

namespace qmin_gb300 {

struct error : std::runtime_error {
    int code;
    error(int c, const std::string &m) : std::runtime_error("qmin error " + std::to_string(c) + ": " + m), code(c) {}
};

inline void check(int rc)
{
    if (rc != QMIN_OK) throw error(rc, qmin_last_error_string());
}

enum class boundaryType { homeotropic = QMIN_HOMEOTROPIC, degeneratePlanar = QMIN_DEGENERATE_PLANAR };

struct boundaryObject {
    boundaryType boundary;
    double P1, P2;
    boundaryObject(boundaryType b, double p1, double p2) : boundary(b), P1(p1), P2(p2) {}
};

// openQmin.cpp:173-175 phase-constant rescaling and the S0 of openQmin.cpp:266
struct cliPhase {
    double a, b, c, S0;
    explicit cliPhase(double A = -0.172, double B = -2.12, double C = 1.73)
        : a(-1.0), b(-B / A), c(-C / A), S0((-b + std::sqrt(b * b - 24 * a * c)) / (6 * c)) {}
};

class qTensorLatticeModel {
  public:
    qTensorLatticeModel(int lx, int ly, int lz, int precision = QMIN_FP64, int metric = QMIN_METRIC_CPU)
        : L{lx, ly, lz}, prec(precision), metric_mode(metric), N((size_t)lx * ly * lz), Q(5 * N, 0.0), types(N, 0)
    {
    }
    ~qTensorLatticeModel()
    {
        if (h) qmin_destroy(h);
    }
    int getNumberOfParticles() const { return (int)N; }
    void setNematicQTensorRandomly(int seed, double S0)
    {
        check(qmin_host_random_nematic(L[0], L[1], L[2], seed, S0, Q.data()));
    }
    std::vector<double> returnPositions()
    {
        if (!h) return Q;
        std::vector<double> out(5 * N);
        check(qmin_get_state(h, out.data(), nullptr, nullptr, QMIN_LAYOUT_AOS));
        return out;
    }
    const std::vector<int32_t> &returnTypes() const { return types; }

    int L[3];
    int prec, metric_mode;
    size_t N;
    std::vector<double> Q;
    std::vector<int32_t> types;
    std::vector<qmin_object> objects = std::vector<qmin_object>(127);
    int nobj = 0;
    qmin_handle h = nullptr;
};

class landauDeGennesLC {
  public:
    void setPhaseConstants(double a = -1, double b = -12.325581395, double c = 10.058139535)
    {
        p.A = a;
        p.B = b;
        p.C = c;
    }
    void setElasticConstants(double l1 = 2.32, double l2 = 0, double l3 = 0, double l4 = 0, double l6 = 0)
    {
        if (l6 != 0) throw error(QMIN_EINVAL, "the L6 distortion term is not supported");
        p.L1 = l1;
        p.L2 = l2;
        p.L3 = l3;
        p.L4 = l4;
        p.multi_constant = (l2 != 0 || l3 != 0 || l4 != 0);
    }
    void setEField(const double f[3], double eps, double eps0, double deltaEps)
    {
        p.efield = 1;
        for (int k = 0; k < 3; ++k) p.E[k] = f[k];
        p.eps = eps;
        p.eps0 = eps0;
        p.deps = deltaEps;
    }
    void setHField(const double f[3], double chi, double mu0, double deltaChi)
    {
        p.hfield = 1;
        for (int k = 0; k < 3; ++k) p.H[k] = f[k];
        p.chi = chi;
        p.mu0 = mu0;
        p.dchi = deltaChi;
    }
    qmin_ldg_params p{-1.0, -12.325581395, 10.058139535, 2.32, 0, 0, 0, 0, 0, {0, 0, 0}, 0, 0, 0, 0, {0, 0, 0}, 0, 0, 0};
    double energyComponents[5] = {0, 0, 0, 0, 0};
};

class updater {
  public:
    virtual ~updater() = default;
    void setMaximumIterations(int n) { maxIterations = n; }
    double getMaxForce() const { return forceMax; }
    int getCurrentIterations() const { return iterations; }
    virtual void minimize() = 0;
    void performUpdate() { minimize(); }
    qTensorLatticeModel *model = nullptr;
    int maxIterations = 1000, iterations = 0;
    double forceMax = 100.0;
};

class energyMinimizerFIRE : public updater {
  public:
    explicit energyMinimizerFIRE(qTensorLatticeModel *m = nullptr) { model = m; }
    // energyMinimizerFIRE::setFIREParameters (energyMinimizerFIRE.h:33)
    void setFIREParameters(double deltaT, double alphaStart, double deltaTMax, double deltaTInc, double deltaTDec,
                           double alphaDec, int nMin, double forceCutoff, double alphaMin = 0.75)
    {
        fp = {deltaT, alphaStart, deltaTMax, deltaTInc, deltaTDec, alphaDec, alphaMin, forceCutoff, nMin};
        ready = false;
    }
    void minimize() override
    {
        if (!ready) {
            check(qmin_fire_init(model->h, &fp));
            ready = true;
        }
        qmin_fire_result r;
        check(qmin_fire_run(model->h, maxIterations, &r));
        iterations = r.iterations;
        forceMax = r.force_max;
        alpha = r.alpha;
        deltaT = r.dt;
        Power = r.power;
    }
    double alpha = 0.99, deltaT = 0.01, Power = 0.0;

  private:
    qmin_fire_params fp{0.01, 0.99, 0.1, 1.05, 0.95, 0.9, 0.0, 1e-7, 5};
    bool ready = false;
};

class energyMinimizerAdam : public updater {
  public:
    explicit energyMinimizerAdam(qTensorLatticeModel *m = nullptr) { model = m; }
    void setAdamParameters(double b1 = 0.9, double b2 = 0.99, double eps = 1e-8, double dt = 1e-4, double fc = 1e-12)
    {
        beta1 = b1; beta2 = b2; epsilon = eps; deltaT = dt; cutoff = fc; fresh = true;
    }
    void minimize() override
    {
        check(qmin_adam_run(model->h, beta1, beta2, epsilon, deltaT, cutoff, maxIterations, fresh, &iterations,
                            &forceMax));
        fresh = false;
    }

  private:
    double beta1 = 0.9, beta2 = 0.99, epsilon = 1e-8, deltaT = 1e-4, cutoff = 1e-12;
    bool fresh = true;
};

class energyMinimizerNesterovAG : public updater {
  public:
    explicit energyMinimizerNesterovAG(qTensorLatticeModel *m = nullptr) { model = m; }
    void setNesterovAGParameters(double dt = 1e-4, double mu_ = 0.01, double fc = 1e-12)
    {
        deltaT = dt; mu = mu_; cutoff = fc; fresh = true;
    }
    void minimize() override
    {
        check(qmin_nesterov_run(model->h, deltaT, mu, cutoff, maxIterations, fresh, &iterations, &forceMax));
        fresh = false;
    }

  private:
    double deltaT = 1e-4, mu = 0.01, cutoff = 1e-12;
    bool fresh = true;
};

class energyMinimizerLoLBFGS : public updater {
  public:
    explicit energyMinimizerLoLBFGS(qTensorLatticeModel *m = nullptr) { model = m; }
    void setLoLBFGSParameters(int m_ = 5, double dt = 1e-4, double c = 1.0, double fc = 1e-12, double tau = 10)
    {
        (void)c;
        (void)tau;
        m = m_; eta = dt; cutoff = fc; fresh = true;
    }
    void minimize() override
    {
        check(qmin_lbfgs_run(model->h, m, eta, cutoff, maxIterations, fresh, &iterations, &forceMax));
        fresh = false;
    }

  private:
    int m = 5;
    double eta = 1e-4, cutoff = 1e-12;
    bool fresh = true;
};

// single-domain multirankSimulation: set-up calls on the host, then the GPU
class multirankSimulation {
  public:
    multirankSimulation(int = 0, int xDiv = 1, int yDiv = 1, int zDiv = 1, bool = false, bool = false)
    {
        if (xDiv != 1 || yDiv != 1 || zDiv != 1)
            throw error(QMIN_EINVAL, "qmin_gb300 runs a single domain on one GPU");
    }
    void setConfiguration(qTensorLatticeModel *m) { model = m; }
    void addForce(landauDeGennesLC *f) { force = f; }
    void addUpdater(updater *u) { updaters.push_back(u); }
    void createWall(int xyz, int plane, const boundaryObject &b)
    {
        check(qmin_host_add_wall(model->L[0], model->L[1], model->L[2], xyz, plane, (int)b.boundary, b.P1, b.P2,
                                 model->Q.data(), model->types.data(), model->objects.data(), &model->nobj));
    }
    void createSphericalColloid(const double center[3], double radius, const boundaryObject &b)
    {
        check(qmin_host_add_sphere(model->L[0], model->L[1], model->L[2], center, radius, (int)b.boundary, b.P1,
                                   b.P2, model->Q.data(), model->types.data(), model->objects.data(), &model->nobj));
    }
    void finalizeObjects()
    {
        if (!model->h) {
            qmin_lattice_desc d{model->L[0], model->L[1], model->L[2], model->prec, model->metric_mode};
            check(qmin_create(&d, &model->h));
        }
        check(qmin_set_params(model->h, &force->p));
        check(qmin_set_objects(model->h, model->objects.data(), model->nobj));
        check(qmin_set_state(model->h, model->Q.data(), model->types.data(), QMIN_LAYOUT_AOS));
        check(qmin_n_active(model->h, &NActive));
    }
    void computeForces(double *F_out = nullptr) { check(qmin_force(model->h, F_out)); }
    double computePotentialEnergy()
    {
        double e = 0;
        check(qmin_energy(model->h, &e, force->energyComponents));
        return e;
    }
    void performTimestep()
    {
        for (auto *u : updaters) u->performUpdate();
    }
    long long NActive = 0;

  private:
    qTensorLatticeModel *model = nullptr;
    landauDeGennesLC *force = nullptr;
    std::vector<updater *> updaters;
};

}  // namespace qmin_gb300
