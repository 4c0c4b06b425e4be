// The reference CLI's default run, `openQmin -i 100 -l 50 --L1 2.32`
// (openQmin.cpp:171-336), written against the C++ host layer: random-director
// 50^3 lattice, seed 13371, one-constant L1 = 2.32, 100 FIRE iterations.
// Optional arguments: lattice side, iterations, L2, L3 (multi-constant).
// Prints "minimized to <forceMax> E=<E/site>" like the CLI.
#include <cstdio>
#include <cstdlib>

#include "qmin_gb300.hpp"

using namespace qmin_gb300;

int main(int argc, char **argv)
{
    const int L = argc > 1 ? std::atoi(argv[1]) : 50;
    const int iters = argc > 2 ? std::atoi(argv[2]) : 100;
    const double L2 = argc > 3 ? std::atof(argv[3]) : 0.0, L3 = argc > 4 ? std::atof(argv[4]) : 0.0;
    try {
        cliPhase ph;
        qTensorLatticeModel model(L, L, L);
        multirankSimulation sim(0, 1, 1, 1, false, false);
        landauDeGennesLC lc;
        sim.setConfiguration(&model);
        lc.setPhaseConstants(ph.a, ph.b, ph.c);
        lc.setElasticConstants(2.32, L2, L3);
        sim.addForce(&lc);
        energyMinimizerFIRE fire(&model);
        fire.setMaximumIterations(iters);
        const double dt = 0.0005;
        fire.setFIREParameters(dt, .99, 100 * dt, 1.1, 0.95, 0.9, 4, 1e-12, 0.0);
        sim.addUpdater(&fire);
        model.setNematicQTensorRandomly(13371, ph.S0);
        sim.finalizeObjects();
        sim.performTimestep();
        const double E = sim.computePotentialEnergy();
        std::printf("minimized to %.17g E=%.17g iterations %d\n", fire.getMaxForce(), E, fire.getCurrentIterations());
    } catch (const error &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return e.code == QMIN_ENODEVICE ? 3 : 1;
    }
    return 0;
}
