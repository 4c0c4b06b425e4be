// energyMinimizerFIRE_gb300: open-Qmin's FIRE minimiser with the whole
// minimisation (velocity Verlet, Landau-de Gennes force, FIRE velocity mix and
// schedule) run by qmin_gb300 on a GB300.  A drop-in subclass of the
// reference's energyMinimizerFIRE (src/updaters/energyMinimizerFIRE.h:20):
// its constructor, setFIREParameters / set* setters, setMaximumIterations and
// getMaxForce are inherited unchanged, and the virtual hook the simulation
// calls -- updater::Update -> performUpdate (energyMinimizerFIRE.h:64) -- runs
// one GPU minimisation instead of minimize().
//
//     auto lc = make_shared<landauDeGennesLC_gb300>(true);   // instead of landauDeGennesLC
//     ...
//     auto fire = make_shared<energyMinimizerFIRE_gb300>(Conf, lc);  // instead of energyMinimizerFIRE(Conf)
//     fire->setFIREParameters(dt, .99, 100 * dt, 1.1, 0.95, 0.9, 4, fc, 0.0);
//     sim->addUpdater(fire, Conf);
//     sim->performTimestep();
//
// One performUpdate() does what energyMinimizerFIRE::minimize()
// (energyMinimizerFIRE.cpp:151-170) does: forces at the current state, then
// iterations until forceMax <= forceCutoff or maxIterations, at least one.
// The model's positions, velocities and site types and this object's FIRE
// state (iterations, forceMax, alpha, deltaT, deltaTMin, Power,
// NSinceNegativePower) go to the GPU at entry; positions, velocities, forces
// and the FIRE state come back at exit.  So consecutive calls continue
// exactly as the reference's do, and the model can be read or changed on the
// host between them.  Nothing crosses between host and device inside a call.
#ifndef ENERGYMINIMIZERFIRE_GB300_H
#define ENERGYMINIMIZERFIRE_GB300_H

#include <stdexcept>
#include <string>

#include "energyMinimizerFIRE.h"
#include "landauDeGennesLC_gb300.h"
#include "qmin_gb300.h"

class energyMinimizerFIRE_gb300 : public energyMinimizerFIRE
    {
    public:
        //! the model to minimise and the force computer whose parameters it uses
        energyMinimizerFIRE_gb300(shared_ptr<simpleModel> system, shared_ptr<landauDeGennesLC_gb300> lc)
            : energyMinimizerFIRE(system), force_(lc)
            {
            }

        //! energyMinimizerFIRE::performUpdate -> minimize (energyMinimizerFIRE.cpp:151-170) on the GPU
        void performUpdate() override
            {
            if (Ndof != model->getNumberOfParticles())
                initializeFromModel();
            qmin_handle h = force_->upload();  // positions, types, parameters, objects
            qmin_fire_params fp{deltaT, alphaStart, deltaTMax, deltaTInc, deltaTDec, alphaDec, alphaMin,
                                forceCutoff, NMin};
            check(qmin_fire_init(h, &fp), "qmin_fire_init");
            qmin_fire_state st{iterations, forceMax, alpha, deltaT, deltaTMin, Power, NSinceNegativePower};
            check(qmin_fire_set_state(h, &st), "qmin_fire_set_state");
                {
                // after qmin_fire_init, which starts FIRE from rest (zero velocities)
                ArrayHandle<dVec> v(model->returnVelocities(), access_location::host, access_mode::read);
                check(qmin_set_velocities(h, &v.data[0][0], QMIN_LAYOUT_AOS), "qmin_set_velocities");
                }
            qmin_fire_result r;
            const int rc = qmin_fire_run(h, maxIterations, &r);
            if (rc != QMIN_OK && rc != QMIN_ENONFINITE)
                check(rc, "qmin_fire_run");
                {
                ArrayHandle<dVec> q(model->returnPositions(), access_location::host, access_mode::readwrite);
                ArrayHandle<dVec> v(model->returnVelocities(), access_location::host, access_mode::overwrite);
                ArrayHandle<dVec> f(model->returnForces(), access_location::host, access_mode::overwrite);
                check(qmin_get_state(h, &q.data[0][0], &v.data[0][0], &f.data[0][0], QMIN_LAYOUT_AOS),
                      "qmin_get_state");
                }
            iterations = r.iterations;
            forceMax = r.force_max;
            alpha = r.alpha;
            deltaT = r.dt;
            Power = r.power;
            NSinceNegativePower = r.n_since;
            if (rc == QMIN_ENONFINITE)
                check(rc, "qmin_fire_run");  // state and counters above are those of the failing iteration
            }

    protected:
        static void check(int rc, const char *what)
            {
            if (rc != QMIN_OK)
                throw std::runtime_error(std::string("energyMinimizerFIRE_gb300: ") + what + ": " +
                                         qmin_last_error_string());
            }

        shared_ptr<landauDeGennesLC_gb300> force_;
    };

#endif
