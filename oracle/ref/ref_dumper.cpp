// Golden-vector dumper: drives the reference's own CPU objects (compiled from
// the reference tree by oracle/ref/Makefile) through the same set-up sequence
// as the reference CLI (openQmin.cpp:171-299) and writes binary dumps that the
// test-suite compares against.  Written for this project; runs only where the
// reference tree is mounted.
//
// Usage: ref_dumper OUTDIR key=value ...
//   L=Lx,Ly,Lz  seed=S  ABC=A,B,C (CLI phase constants, rescaled as
//   openQmin.cpp:173-175)  Ls=L1,L2,L3,L4,L6  wall=xyz,plane,kind,W
//   sphere=cx,cy,cz,r,kind,W  (kind h = homeotropic, p = degenerate planar;
//   S0 of every object is the bulk S0)  E=Ex,Ey,Ez,eps,eps0,deps
//   H=Hx,Hy,Hz,chi,mu0,dchi  minimizer=fire|adam|nesterov|lbfgs|gd|none  iters=N
//   bfile=PATH (boundary file)  loadstate=PREFIX  savestate=PREFIX,SKIP,DEFECTTYPE  defects=1
//   hfile=PREFIX,chi,mu0,dchi (spatially varying H field)  objforce=1
//   dt=DT  fc=cutoff  trace=1 (per-iteration trace, one minimize() call per
//   iteration)  qin=file (load Q0 from a raw float64 AoS file instead of the
//   random initialisation)
//
// Files written (raw little-endian): q0.f64 (N*5, AoS), types.i32 (N),
// force0.f64 (one sim->computeForces() at Q0, CPU semantics),
// raw0.f64 (computeForceCPU type 0 + type 1 without the metric correction),
// energy0.txt (E/NActive and the 5 components at Q0), trace.txt
// (iteration forceMax alpha dt power nsince), qfinal.f64, vfinal.f64,
// ffinal.f64, final.txt (iterations forceMax E/NActive components).
#include "std_include.h"
#include "multirankQTensorLatticeModel.h"
#include "multirankSimulation.h"
#include "landauDeGennesLC.h"
#include "energyMinimizerFIRE.h"
#include "energyMinimizerAdam.h"
#include "energyMinimizerNesterovAG.h"
#include "energyMinimizerGradientDescent.h"
#include "energyMinimizerLoLBFGS.h"
#include "noiseSource.h"
#include <map>

struct FireProbe : public energyMinimizerFIRE {
    FireProbe(shared_ptr<simpleModel> s) : energyMinimizerFIRE(s) {}
    double getAlpha() { return alpha; }
    double getDt() { return deltaT; }
    double getPower() { return Power; }
    int getNSince() { return NSinceNegativePower; }
};

static vector<double> parse_list(const string &s)
{
    vector<double> out;
    stringstream ss(s);
    string item;
    while (getline(ss, item, ',')) out.push_back(atof(item.c_str()));
    return out;
}
static vector<string> parse_strs(const string &s)
{
    vector<string> out;
    stringstream ss(s);
    string item;
    while (getline(ss, item, ',')) out.push_back(item);
    return out;
}

template <class T>
static void dump(const string &path, const T *p, size_t n)
{
    FILE *f = fopen(path.c_str(), "wb");
    fwrite(p, sizeof(T), n, f);
    fclose(f);
}
static void dump_dvec(const string &path, GPUArray<dVec> &arr, int N)
{
    ArrayHandle<dVec> h(arr, access_location::host, access_mode::read);
    vector<double> buf((size_t)N * 5);
    for (int i = 0; i < N; ++i)
        for (int c = 0; c < 5; ++c) buf[(size_t)i * 5 + c] = h.data[i][c];
    dump(path, buf.data(), buf.size());
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: ref_dumper OUTDIR key=value...\n");
        return 2;
    }
    string out = argv[1];
    multimap<string, string> kv;
    for (int i = 2; i < argc; ++i) {
        string a = argv[i];
        size_t eq = a.find('=');
        kv.insert({a.substr(0, eq), a.substr(eq + 1)});
    }
    auto get = [&](const string &k, const string &def) {
        auto it = kv.find(k);
        return it == kv.end() ? def : it->second;
    };
    vector<double> Ls = parse_list(get("L", "8,8,8"));
    int Lx = (int)Ls[0], Ly = (int)Ls[1], Lz = (int)Ls[2];
    int seed = atoi(get("seed", "13371").c_str());
    vector<double> ABC = parse_list(get("ABC", "-0.172,-2.12,1.73"));
    vector<double> Lc = parse_list(get("Ls", "2.32,0,0,0,0"));
    while (Lc.size() < 5) Lc.push_back(0.0);
    string minimizer = get("minimizer", "none");
    int iters = atoi(get("iters", "0").c_str());
    double dt = atof(get("dt", "0.0005").c_str());
    double fc = atof(get("fc", "1e-12").c_str());
    bool trace = atoi(get("trace", "0").c_str()) != 0;
    string qin = get("qin", "");
    string bfile = get("bfile", "");        // multirankSimulation::createBoundaryFromFile
    string loadstate = get("loadstate", "");  // multirankSimulation::loadState prefix (before minimising)
    string savestate = get("savestate", "");  // multirankSimulation::saveState prefix,skip,defectType (after)
    bool defects = atoi(get("defects", "0").c_str()) != 0;  // dump computeDefectMeasures 0, 1, 2 (after)
    bool objforce = atoi(get("objforce", "0").c_str()) != 0;  // dump computeObjectForces of every object (after)

    // openQmin.cpp:173-180
    double a = -1, b = -ABC[1] / ABC[0], c = -ABC[2] / ABC[0];
    noiseSource noise(true);
    noise.setReproducibleSeed(seed);
    bool oneConstant = !(Lc[1] != 0 || Lc[2] != 0 || Lc[3] != 0 || Lc[4] != 0);

    // openQmin.cpp:194-197 (single rank, CPU only)
    auto Conf = make_shared<multirankQTensorLatticeModel>(Lx, Ly, Lz, false, false, false, false, true);
    auto sim = make_shared<multirankSimulation>(0, 1, 1, 1, false, false);
    auto lc = make_shared<landauDeGennesLC>(true);
    sim->setConfiguration(Conf);
    lc->setPhaseConstants(a, b, c);
    if (oneConstant) {
        lc->setElasticConstants(Lc[0]);
        lc->setNumberOfConstants(distortionEnergyType::oneConstant);
    } else {
        lc->setElasticConstants(Lc[0], Lc[1], Lc[2], Lc[3], Lc[4]);
        lc->setNumberOfConstants(distortionEnergyType::multiConstant);
    }
    if (kv.count("E")) {
        vector<double> e = parse_list(get("E", ""));
        lc->setEField(make_scalar3(e[0], e[1], e[2]), e[3], e[4], e[5]);
    }
    if (kv.count("H")) {
        vector<double> h = parse_list(get("H", ""));
        lc->setHField(make_scalar3(h[0], h[1], h[2]), h[3], h[4], h[5]);
    }
    lc->setModel(Conf);
    if (kv.count("hfile")) {
        // landauDeGennesLC::setSpatiallyVaryingField(prefix, chi, mu0, dchi, rank parity 0)
        vector<string> hf = parse_strs(get("hfile", ""));
        int3 parity;
        parity.x = parity.y = parity.z = 0;
        lc->setSpatiallyVaryingField(hf[0], atof(hf[1].c_str()), atof(hf[2].c_str()), atof(hf[3].c_str()), parity);
    }
    sim->addForce(lc);

    // openQmin.cpp:261-268 and setInitialConditions.h:37-41
    sim->setCPUOperation(true);
    double S0 = (-b + sqrt(b * b - 24 * a * c)) / (6 * c);
    int N = Conf->getNumberOfParticles();
    if (qin.empty()) {
        Conf->setNematicQTensorRandomly(noise, S0);
    } else {
        vector<double> buf((size_t)N * 5);
        FILE *f = fopen(qin.c_str(), "rb");
        if (!f || fread(buf.data(), sizeof(double), buf.size(), f) != buf.size()) {
            fprintf(stderr, "cannot read %s\n", qin.c_str());
            return 3;
        }
        fclose(f);
        ArrayHandle<dVec> h(Conf->returnPositions());
        for (int i = 0; i < N; ++i)
            for (int cc = 0; cc < 5; ++cc) h.data[i][cc] = buf[(size_t)i * 5 + cc];
    }

    // objects, in command-line order (addObjectsToOpenQmin.h pattern)
    for (auto it = kv.lower_bound("wall"); it != kv.upper_bound("wall"); ++it) {
        vector<string> w = parse_strs(it->second);
        boundaryType bt = w[2] == "p" ? boundaryType::degeneratePlanar : boundaryType::homeotropic;
        boundaryObject bo(bt, atof(w[3].c_str()), S0);
        sim->createWall(atoi(w[0].c_str()), atoi(w[1].c_str()), bo);
    }
    for (auto it = kv.lower_bound("sphere"); it != kv.upper_bound("sphere"); ++it) {
        vector<string> s = parse_strs(it->second);
        boundaryType bt = s[4] == "p" ? boundaryType::degeneratePlanar : boundaryType::homeotropic;
        boundaryObject bo(bt, atof(s[5].c_str()), S0);
        sim->createSphericalColloid(make_scalar3(atof(s[0].c_str()), atof(s[1].c_str()), atof(s[2].c_str())),
                                    atof(s[3].c_str()), bo);
    }
    if (!bfile.empty()) sim->createBoundaryFromFile(bfile, false);
    if (!loadstate.empty()) sim->loadState(loadstate);
    // minimisers are created after the initial state is in place, so that
    // state-copying constructors (Nesterov's alternate sequence) see Q0
    shared_ptr<FireProbe> fire;
    shared_ptr<energyMinimizerAdam> adam;
    shared_ptr<energyMinimizerNesterovAG> nest;
    shared_ptr<energyMinimizerLoLBFGS> lbfgs;
    shared_ptr<energyMinimizerGradientDescent> gd;
    if (minimizer == "fire") {
        fire = make_shared<FireProbe>(Conf);
        fire->setMaximumIterations(iters);
        // openQmin.cpp:256-258
        fire->setFIREParameters(dt, .99, 100 * dt, 1.1, 0.95, 0.9, 4, fc, 0.0);
        sim->addUpdater(fire, Conf);
    } else if (minimizer == "adam") {
        adam = make_shared<energyMinimizerAdam>();
        adam->setModel(Conf);
        adam->setAdamParameters(0.9, 0.99, 1e-8, dt, fc);
        adam->setMaximumIterations(iters);
        sim->addUpdater(adam, Conf);
    } else if (minimizer == "nesterov") {
        nest = make_shared<energyMinimizerNesterovAG>(Conf);
        nest->setNesterovAGParameters(dt, atof(get("mu", "0.01").c_str()), fc);
        nest->setMaximumIterations(iters);
        sim->addUpdater(nest, Conf);
    } else if (minimizer == "gd") {
        gd = make_shared<energyMinimizerGradientDescent>(Conf);
        gd->setGradientDescentParameters(dt, fc);
        gd->setMaximumIterations(iters);
        sim->addUpdater(gd, Conf);
    } else if (minimizer == "lbfgs") {
        lbfgs = make_shared<energyMinimizerLoLBFGS>(Conf);
        lbfgs->setLoLBFGSParameters(5, dt, 1.0, fc, 10);
        lbfgs->setMaximumIterations(iters);
        sim->addUpdater(lbfgs, Conf);
    }

    sim->finalizeObjects();

    dump_dvec(out + "/q0.f64", Conf->returnPositions(), N);
    {
        ArrayHandle<int> t(Conf->returnTypes(), access_location::host, access_mode::read);
        dump(out + "/types.i32", t.data, (size_t)N);
    }
    // raw force: both CPU passes without the metric correction
    {
        GPUArray<dVec> raw;
        raw.resize(N);
        lc->computeForceCPU(raw, true, 0);
        lc->computeForceCPU(raw, false, 1);
        dump_dvec(out + "/raw0.f64", raw, N);
    }
    sim->computeForces();
    dump_dvec(out + "/force0.f64", Conf->returnForces(), N);
    {
        double e = sim->computePotentialEnergy(false);
        FILE *f = fopen((out + "/energy0.txt").c_str(), "w");
        fprintf(f, "%.17g", e);
        for (int k = 0; k < 5; ++k) fprintf(f, " %.17g", lc->energyComponents[k]);
        fprintf(f, "\n");
        fclose(f);
    }

    double fmax = 0.0;
    int done = 0;
    if (minimizer != "none" && iters > 0) {
        if (fire && trace) {
            FILE *f = fopen((out + "/trace.txt").c_str(), "w");
            for (int k = 1; k <= iters; ++k) {
                fire->setMaximumIterations(k);
                sim->performTimestep();
                fprintf(f, "%d %.17g %.17g %.17g %.17g %d\n", fire->getCurrentIterations(), fire->getMaxForce(),
                        fire->getAlpha(), fire->getDt(), fire->getPower(), fire->getNSince());
                if (fire->getCurrentIterations() < k) break;
            }
            fclose(f);
        } else {
            sim->performTimestep();
        }
        if (fire) { fmax = fire->getMaxForce(); done = fire->getCurrentIterations(); }
        if (adam) { fmax = adam->getMaxForce(); done = adam->getCurrentIterations(); }
        if (nest) { fmax = nest->getMaxForce(); done = nest->getCurrentIterations(); }
        if (lbfgs) { fmax = lbfgs->getMaxForce(); done = lbfgs->getCurrentIterations(); }
        if (gd) { fmax = gd->getMaxForce(); done = gd->getCurrentIterations(); }
    }
    if (defects) {
        for (int dt2 = 0; dt2 < 3; ++dt2) {
            Conf->computeDefectMeasures(dt2);
            ArrayHandle<scalar> dm(Conf->returnDefectMeasures(), access_location::host, access_mode::read);
            dump(out + "/defects" + to_string(dt2) + ".f64", dm.data, (size_t)N);
        }
    }
    if (objforce) {
        FILE *f = fopen((out + "/objforce.txt").c_str(), "w");
        for (int j = 0; j < (int)Conf->boundaryForce.size(); ++j) {
            lc->computeObjectForces(j);
            fprintf(f, "%.17g %.17g %.17g\n", Conf->boundaryForce[j].x, Conf->boundaryForce[j].y,
                    Conf->boundaryForce[j].z);
        }
        fclose(f);
    }
    if (!savestate.empty()) {
        vector<string> sv = parse_strs(savestate);
        sim->saveState(sv[0], atoi(sv[1].c_str()), atoi(sv[2].c_str()));
    }
    dump_dvec(out + "/qfinal.f64", Conf->returnPositions(), N);
    dump_dvec(out + "/vfinal.f64", Conf->returnVelocities(), N);
    dump_dvec(out + "/ffinal.f64", Conf->returnForces(), N);
    {
        double e = sim->computePotentialEnergy(false);
        FILE *f = fopen((out + "/final.txt").c_str(), "w");
        fprintf(f, "%d %.17g %.17g", done, fmax, e);
        for (int k = 0; k < 5; ++k) fprintf(f, " %.17g", lc->energyComponents[k]);
        fprintf(f, "\n");
        fclose(f);
    }
    return 0;
}
