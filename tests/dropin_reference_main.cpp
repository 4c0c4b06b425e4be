// Drives the drop-in classes landauDeGennesLC_gb300 and
// energyMinimizerFIRE_gb300 through the reference's own multirankSimulation,
// multirankQTensorLatticeModel, geometry builders and updater machinery,
// compiled from the reference's sources (its single-rank CPU objects).  The
// set-up follows the reference CLI (openQmin.cpp:171-299): a 12 x 11 x 10
// lattice, L1-L3 = 2.32/1.0/0.5, homeotropic z-walls and a sphere, the CLI's
// FIRE parameters.
//
// Usage: dropin_reference_main MODE ITERS
//   MODE ref    the reference's own landauDeGennesLC + energyMinimizerFIRE
//   MODE gb300  the drop-in classes (needs a CUDA device)
// Prints one line "iterations forceMax E/NActive" (%.17g); a failure inside
// the drop-in prints "DROPIN_ERROR <message>" and exits with status 3.
#include "std_include.h"
#include "multirankQTensorLatticeModel.h"
#include "multirankSimulation.h"
#include "landauDeGennesLC.h"
#include "energyMinimizerFIRE.h"
#include "noiseSource.h"

#include "landauDeGennesLC_gb300.h"
#include "energyMinimizerFIRE_gb300.h"

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: dropin_reference_main ref|gb300 ITERS\n");
        return 2;
    }
    const string mode = argv[1];
    const int iters = atoi(argv[2]);
    const int Lx = 12, Ly = 11, Lz = 10;
    // openQmin.cpp:173-180: a = -1, b = -B/A, c = -C/A from A, B, C = -0.172, -2.12, 1.73
    const double A = -0.172, B = -2.12, C = 1.73;
    const double a = -1, b = -B / A, c = -C / A;
    noiseSource noise(true);
    noise.setReproducibleSeed(7);

    auto Conf = make_shared<multirankQTensorLatticeModel>(Lx, Ly, Lz, false, false, false, false, true);
    auto sim = make_shared<multirankSimulation>(0, 1, 1, 1, false, false);
    shared_ptr<landauDeGennesLC> lc;
    shared_ptr<landauDeGennesLC_gb300> lc_gb300;
    if (mode == "gb300") {
        lc_gb300 = make_shared<landauDeGennesLC_gb300>(true);
        lc = lc_gb300;
    } else {
        lc = make_shared<landauDeGennesLC>(true);
    }
    sim->setConfiguration(Conf);
    lc->setPhaseConstants(a, b, c);
    lc->setElasticConstants(2.32, 1.0, 0.5, 0.0, 0.0);
    lc->setNumberOfConstants(distortionEnergyType::multiConstant);
    lc->setModel(Conf);
    sim->addForce(lc);
    sim->setCPUOperation(true);
    const double S0 = (-b + sqrt(b * b - 24 * a * c)) / (6 * c);
    Conf->setNematicQTensorRandomly(noise, S0);
    boundaryObject hom(boundaryType::homeotropic, 5.3, S0);
    sim->createWall(2, 0, hom);
    sim->createWall(2, Lz - 1, hom);
    sim->createSphericalColloid(make_scalar3(6.0, 5.5, 5.0), 2.7, hom);

    shared_ptr<energyMinimizerFIRE> fire;
    if (mode == "gb300")
        fire = make_shared<energyMinimizerFIRE_gb300>(Conf, lc_gb300);
    else
        fire = make_shared<energyMinimizerFIRE>(Conf);
    fire->setMaximumIterations(iters);
    // openQmin.cpp:256-258
    fire->setFIREParameters(5e-4, .99, 100 * 5e-4, 1.1, 0.95, 0.9, 4, 1e-12, 0.0);
    sim->addUpdater(fire, Conf);
    sim->finalizeObjects();
    try {
        // two minimize() calls with a growing cap: the second continues from the first
        fire->setMaximumIterations(iters / 2);
        sim->performTimestep();
        fire->setMaximumIterations(iters);
        sim->performTimestep();
        const double e = sim->computePotentialEnergy();
        printf("%d %.17g %.17g\n", fire->getCurrentIterations(), fire->getMaxForce(), e);
    } catch (const std::exception &ex) {
        printf("DROPIN_ERROR %s\n", ex.what());
        return 3;
    }
    return 0;
}
