// landauDeGennesLC_gb300: open-Qmin's Landau-de Gennes force computer with its
// force and energy evaluated by qmin_gb300 on a GB300.  A drop-in subclass of
// the reference's landauDeGennesLC (src/forces/landauDeGennesLC.h:12), itself
// a baseLatticeForce (src/forces/baseLatticeForce.h:9): the reference's
// constructors, parameter setters (setPhaseConstants, setElasticConstants,
// setNumberOfConstants, setEField, setHField, setSpatiallyVaryingField) and
// setModel are inherited unchanged, so a caller replaces
//     auto lc = make_shared<landauDeGennesLC>(...);
// by
//     auto lc = make_shared<landauDeGennesLC_gb300>(...);
// and multirankSimulation::addForce / computeForces / computePotentialEnergy
// call into the GPU through the two virtual overrides below.
//
// State transfer: every computeForces / computeEnergy call uploads the
// model's host positions and site types (GPUArray host copies, AoS dVec =
// the C ABI's double[N][5]); parameters, objects and the spatially varying
// field are uploaded when they change.  A minimiser that keeps the state on
// the device for a whole minimisation is energyMinimizerFIRE_gb300.
//
// Metric correction: multirankSimulation::computeForces calls each force
// computer twice on its CPU branch (type 0, then type 1 with zeroOutForce =
// false; multirankSimulation.cpp:462-466), which leaves bulk sites with the
// metric applied twice and boundary sites once; on its GPU branch it calls
// once (metric once everywhere).  The handle computes the whole force of the
// branch in use in one call (QMIN_METRIC_CPU when useGPU is false,
// QMIN_METRIC_SINGLE when true), so the type-1 call of the CPU branch adds
// nothing.  That is exact when this is the simulation's only force computer,
// as in the reference's CLI and examples.
//
// Errors: the reference reports failures by throwing (HANDLE_ERROR,
// inc/std_include.h:170-184); this class throws std::runtime_error with
// qmin_last_error_string().
#ifndef LANDAUDEGENNESLC_GB300_H
#define LANDAUDEGENNESLC_GB300_H

#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "landauDeGennesLC.h"
#include "qmin_gb300.h"

class landauDeGennesLC_gb300 : public landauDeGennesLC
    {
    public:
        using landauDeGennesLC::landauDeGennesLC;

        ~landauDeGennesLC_gb300() { release(); }  // force has no virtual destructor: make_shared keeps this one

        string reportSelfName() override { return "landauDeGennesLC_gb300"; }

        //! precision of the state resident on the GPU: QMIN_FP64 (default, the
        //! reference's arithmetic) or QMIN_FP32 (FP32 stencils, FP64 reductions)
        void setPrecision(int precision)
            {
            if (precision != precision_)
                {
                release();
                precision_ = precision;
                }
            }

        //! landauDeGennesLC::computeForces (landauDeGennesLC.cpp:125-135)
        void computeForces(GPUArray<dVec> &forces, bool zeroOutForce = true, int type = 0) override
            {
            if (!useGPU && type != 0)
                return;
            qmin_handle h = upload();
            const int N = lattice->getNumberOfParticles();
            buffer_.resize((size_t)5 * N);
            check(qmin_force(h, buffer_.data()), "qmin_force");
            ArrayHandle<dVec> f(forces, access_location::host,
                                zeroOutForce ? access_mode::overwrite : access_mode::readwrite);
            for (int i = 0; i < N; ++i)
                for (int k = 0; k < 5; ++k)
                    f.data[i][k] = zeroOutForce ? buffer_[(size_t)5 * i + k] : f.data[i][k] + buffer_[(size_t)5 * i + k];
            }

        //! landauDeGennesLC::computeEnergyCPU (landauDeGennesLC.cpp:204-353):
        //! the total (multirankSimulation::computePotentialEnergy divides by
        //! NActive) and energyComponents = phase, distortion, anchoring, E, H
        scalar computeEnergy(bool verbose = false) override
            {
            qmin_handle h = upload();
            double perSite = 0.0, comps[5];
            check(qmin_energy(h, &perSite, comps), "qmin_energy");
            energyComponents.assign(comps, comps + 5);
            energy = comps[0] + comps[1] + comps[2] + comps[3] + comps[4];
            if (verbose)
                printf("%f %f %f %f %f\n", comps[0], comps[1], comps[2], comps[3], comps[4]);
            return energy;
            }

        //! the handle, holding the model's current positions and types and this
        //! object's parameters, objects and field
        qmin_handle upload()
            {
            if (!lattice)
                throw std::runtime_error("landauDeGennesLC_gb300: setModel has not been called");
            const int metric = useGPU ? QMIN_METRIC_SINGLE : QMIN_METRIC_CPU;
            if (h_ && metric != metric_)
                release();
            if (!h_)
                {
                qmin_lattice_desc d{lattice->latticeSites.x, lattice->latticeSites.y, lattice->latticeSites.z,
                                    precision_, metric};
                check(qmin_create(&d, &h_), "qmin_create");
                metric_ = metric;
                }
            uploadParameters();
            uploadObjects();
            const int N = lattice->getNumberOfParticles();
            ArrayHandle<dVec> q(lattice->returnPositions(), access_location::host, access_mode::read);
            ArrayHandle<int> t(lattice->returnTypes(), access_location::host, access_mode::read);
            check(qmin_set_state(h_, &q.data[0][0], t.data, QMIN_LAYOUT_AOS), "qmin_set_state");
            if (spatiallyVaryingFieldContribution)
                {
                ArrayHandle<scalar3> hf(spatiallyVaryingField, access_location::host, access_mode::read);
                const double *H = &hf.data[0].x;
                const bool same = field_.size() == (size_t)3 * N && fieldConsts_[0] == Chi && fieldConsts_[1] == mu0 &&
                                  fieldConsts_[2] == deltaChi &&
                                  std::memcmp(field_.data(), H, sizeof(double) * 3 * N) == 0;
                if (!same)
                    {
                    check(qmin_set_field_map(h_, H, Chi, mu0, deltaChi), "qmin_set_field_map");
                    field_.assign(H, H + (size_t)3 * N);
                    fieldConsts_[0] = Chi;
                    fieldConsts_[1] = mu0;
                    fieldConsts_[2] = deltaChi;
                    }
                }
            return h_;
            }

        //! the handle as it is (no upload): for a minimiser that continues from
        //! the state already resident on the GPU
        qmin_handle handle() const { return h_; }

    protected:
        static void check(int rc, const char *what)
            {
            if (rc != QMIN_OK)
                throw std::runtime_error(std::string("landauDeGennesLC_gb300: ") + what + ": " +
                                         qmin_last_error_string());
            }

        void release()
            {
            if (h_)
                qmin_destroy(h_);
            h_ = nullptr;
            field_.clear();
            haveParams_ = false;
            objects_.clear();
            haveObjects_ = false;
            }

        //! the force parameters as this object holds them (landauDeGennesLC.h:34-36, 76-91)
        void uploadParameters()
            {
            qmin_ldg_params p;
            std::memset(&p, 0, sizeof p);
            p.A = A;
            p.B = B;
            p.C = C;
            p.L1 = L1;
            p.L2 = L2;
            p.L3 = L3;
            p.L4 = L4;
            p.L6 = L6;
            p.multi_constant = numberOfConstants == distortionEnergyType::multiConstant ? 1 : 0;
            p.efield = computeEfieldContribution ? 1 : 0;
            if (computeEfieldContribution)
                {
                p.E[0] = Efield.x;
                p.E[1] = Efield.y;
                p.E[2] = Efield.z;
                p.eps = epsilon;
                p.eps0 = epsilon0;
                p.deps = deltaEpsilon;
                }
            p.hfield = computeHfieldContribution ? 1 : 0;
            if (computeHfieldContribution)
                {
                p.H[0] = Hfield.x;
                p.H[1] = Hfield.y;
                p.H[2] = Hfield.z;
                p.chi = Chi;
                p.mu0 = mu0;
                p.dchi = deltaChi;
                }
            if (haveParams_ && std::memcmp(&p, &params_, sizeof p) == 0)
                return;
            check(qmin_set_params(h_, &p), "qmin_set_params");
            std::memcpy(&params_, &p, sizeof p);  // padding bytes included: compared with memcmp above
            haveParams_ = true;
            }

        //! cubicLattice::boundaries (cubicLattice.h:78) as {kind, W = P1, S0 = P2}
        void uploadObjects()
            {
            const int n = lattice->boundaries.getNumElements();
            std::vector<qmin_object> o;
            if (n > 0)
                {
                ArrayHandle<boundaryObject> b(lattice->boundaries, access_location::host, access_mode::read);
                for (int k = 0; k < n; ++k)
                    o.push_back({b.data[k].boundary == boundaryType::degeneratePlanar ? QMIN_DEGENERATE_PLANAR
                                                                                      : QMIN_HOMEOTROPIC,
                                 b.data[k].P1, b.data[k].P2});
                }
            bool same = haveObjects_ && o.size() == objects_.size();
            for (size_t k = 0; same && k < o.size(); ++k)
                same = o[k].kind == objects_[k].kind && o[k].W == objects_[k].W && o[k].S0 == objects_[k].S0;
            if (same)
                return;
            check(qmin_set_objects(h_, o.data(), (int)o.size()), "qmin_set_objects");
            objects_ = o;
            haveObjects_ = true;
            }

        qmin_handle h_ = nullptr;
        int precision_ = QMIN_FP64;
        int metric_ = QMIN_METRIC_CPU;
        std::vector<double> buffer_;
        std::vector<double> field_;
        double fieldConsts_[3] = {0, 0, 0};
        qmin_ldg_params params_;
        bool haveParams_ = false;
        std::vector<qmin_object> objects_;
        bool haveObjects_ = false;
    };

#endif
