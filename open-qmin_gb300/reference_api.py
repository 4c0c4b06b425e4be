"""Reference-shaped host classes over the qmin_gb300 C ABI.

Mirrors the open-Qmin classes a minimisation script touches, with the same
method names and argument meaning:

* ``qTensorLatticeModel``  (src/model/qTensorLatticeModel.h, cubicLattice.h)
* ``landauDeGennesLC``     (src/forces/landauDeGennesLC.h:34-36, 76-93)
* ``energyMinimizerFIRE``  (src/updaters/energyMinimizerFIRE.h:20-112)
* ``energyMinimizerAdam``, ``energyMinimizerNesterovAG``, ``energyMinimizerLoLBFGS``
* ``multirankSimulation``  (src/simulation/multirankSimulation.h:15-158), single domain

Set-up (initial Q, walls, colloids) happens on the host as in the reference;
``finalizeObjects`` uploads the state and from then on Q, velocities and
forces stay resident on the GPU.  Errors raise ``QminError``.
"""
import numpy as np

from . import (DEGENERATE_PLANAR, FP64, HOMEOTROPIC, METRIC_CPU, Geometry, Lattice, host_random_nematic)


class boundaryType:
    homeotropic = HOMEOTROPIC
    degeneratePlanar = DEGENERATE_PLANAR


class boundaryObject:
    """boundaryObject(boundaryType, P1 = W, P2 = S0) (latticeBoundaries.h:20-39)."""

    def __init__(self, boundary, P1, P2):
        self.boundary, self.P1, self.P2 = boundary, float(P1), float(P2)


class qTensorLatticeModel:
    """Cubic lattice of 5-component Q tensors with site types and objects."""

    def __init__(self, Lx, Ly=None, Lz=None, precision=FP64, metric_mode=METRIC_CPU):
        Ly = Lx if Ly is None else Ly
        Lz = Lx if Lz is None else Lz
        self.L = (int(Lx), int(Ly), int(Lz))
        self.N = self.L[0] * self.L[1] * self.L[2]
        self.precision, self.metric_mode = precision, metric_mode
        self.geometry = Geometry(self.L, np.zeros((self.N, 5)))
        self.lattice = None  # the GPU handle, created by multirankSimulation.finalizeObjects

    def getNumberOfParticles(self):
        return self.N

    def setNematicQTensorRandomly(self, seed, S0):
        """qTensorLatticeModel::setNematicQTensorRandomly with noiseSource seed `seed`."""
        self.geometry.Q[:] = host_random_nematic(self.L, seed, S0)

    def setPositions(self, Q):
        self.geometry.Q[:] = np.asarray(Q, dtype=np.float64).reshape(self.N, 5)
        if self.lattice is not None:
            self.lattice.set_state(self.geometry.Q, self.geometry.types)

    def returnPositions(self):
        if self.lattice is None:
            return self.geometry.Q.copy()
        return self.lattice.get_state(Q=True)[0]

    def returnVelocities(self):
        return self.lattice.get_state(Q=False, V=True)[1]

    def returnForces(self):
        return self.lattice.get_state(Q=False, F=True)[2]

    def returnTypes(self):
        return self.geometry.types.copy()

    def computeDefectMeasures(self, defectType=0):
        """qTensorLatticeModel::computeDefectMeasures; returns the per-site values."""
        self.defectMeasures = self.lattice.defect_measures(defectType)
        return self.defectMeasures


class landauDeGennesLC:
    """Landau-de Gennes force: bulk A, B, C; L1-L4 distortion; anchoring; E/H fields."""

    def __init__(self, A=-1.0, B=-12.325581395, C=10.058139535, L1=2.32, L2=0.0, L3=0.0, L4=0.0):
        self.A, self.B, self.C = A, B, C
        self.L1, self.L2, self.L3, self.L4 = L1, L2, L3, L4
        self.multi = None
        self.E = None
        self.H = None
        self.sim = None
        self.energyComponents = np.zeros(5)

    def setPhaseConstants(self, a=-1, b=-12.325581395, c=10.058139535):
        self.A, self.B, self.C = a, b, c

    def setElasticConstants(self, l1=2.32, l2=0.0, l3=0.0, l4=0.0, l6=0.0):
        if l6 != 0:
            raise NotImplementedError("the L6 (cubic) distortion term is not supported")
        self.L1, self.L2, self.L3, self.L4 = l1, l2, l3, l4

    def setNumberOfConstants(self, multi):
        """False/0: one-constant approximation; True/1: multi-constant forms."""
        self.multi = bool(multi)

    def setEField(self, field, eps, eps0, deltaEps):
        self.E = (float(field[0]), float(field[1]), float(field[2]), eps, eps0, deltaEps)

    def setHField(self, field, chi, mu0, deltaChi):
        self.H = (float(field[0]), float(field[1]), float(field[2]), chi, mu0, deltaChi)

    def setSpatiallyVaryingField(self, fname, chi, mu0, deltaChi, rankParity=(0, 0, 0)):
        """Per-site H field read from fname_x0y0z0.txt (single rank)."""
        self.field_map = (fname, chi, mu0, deltaChi)

    def apply(self, lattice):
        multi = self.multi if self.multi is not None else any(x != 0 for x in (self.L2, self.L3, self.L4))
        lattice.set_params(self.A, self.B, self.C, self.L1, self.L2, self.L3, self.L4, multi_constant=multi,
                           E=self.E, H=self.H)
        if getattr(self, "field_map", None):
            lattice.load_field_map(*self.field_map)

    def computeForces(self):
        return self.sim.computeForces()

    def computeEnergy(self):
        e, comps = self.sim.model.lattice.energy()
        self.energyComponents = comps
        return float(np.sum(comps))


class _Updater:
    def __init__(self, model=None):
        self.model = model
        self.sim = None
        self.maxIterations = 1000
        self.iterations = 0
        self.forceMax = 100.0

    def setMaximumIterations(self, n):
        self.maxIterations = int(n)

    def getMaxForce(self):
        return self.forceMax

    def getCurrentIterations(self):
        return self.iterations

    def Update(self, timestep=0):
        self.performUpdate()

    def performUpdate(self):
        self.minimize()


class energyMinimizerFIRE(_Updater):
    """FIRE with velocity-Verlet; defaults of energyMinimizerFIRE::initializeParameters."""

    def __init__(self, model=None):
        super().__init__(model)
        self.params = dict(dt=0.01, alpha_start=0.99, dt_max=0.1, dt_inc=1.05, dt_dec=0.95, alpha_dec=0.9, n_min=5,
                           force_cutoff=1e-7, alpha_min=0.0)
        self._initialised = False
        self.alpha = self.params["alpha_start"]
        self.deltaT = self.params["dt"]

    def setFIREParameters(self, deltaT, alphaStart, deltaTMax, deltaTInc, deltaTDec, alphaDec, nMin, forceCutoff,
                          alphaMin=0.75):
        self.params = dict(dt=deltaT, alpha_start=alphaStart, dt_max=deltaTMax, dt_inc=deltaTInc, dt_dec=deltaTDec,
                           alpha_dec=alphaDec, n_min=nMin, force_cutoff=forceCutoff, alpha_min=alphaMin)
        self._initialised = False

    def minimize(self):
        lat = self.sim.model.lattice
        if not self._initialised:
            lat.fire_init(**self.params)
            self._initialised = True
        r = lat.fire_run(self.maxIterations)
        self.iterations, self.forceMax = r["iterations"], r["forceMax"]
        self.alpha, self.deltaT, self.Power = r["alpha"], r["dt"], r["power"]
        return r


class energyMinimizerAdam(_Updater):
    def __init__(self, model=None):
        super().__init__(model)
        self.setAdamParameters()
        self._fresh = True

    def setAdamParameters(self, b1=0.9, b2=0.99, eps=1e-8, _dt=1e-4, fc=1e-12):
        self.beta1, self.beta2, self.epsilon, self.deltaT, self.forceCutoff = b1, b2, eps, _dt, fc
        self._fresh = True

    def minimize(self):
        r = self.sim.model.lattice.adam_run(self.maxIterations, dt=self.deltaT, beta1=self.beta1, beta2=self.beta2,
                                            eps=self.epsilon, force_cutoff=self.forceCutoff, reset=self._fresh)
        self._fresh = False
        self.iterations, self.forceMax = r["iterations"], r["forceMax"]
        return r


class energyMinimizerNesterovAG(_Updater):
    def __init__(self, model=None):
        super().__init__(model)
        self.setNesterovAGParameters()

    def setNesterovAGParameters(self, _dt=1e-4, _mu=0.01, fc=1e-12):
        self.deltaT, self.mu, self.forceCutoff = _dt, _mu, fc
        self._fresh = True

    def minimize(self):
        r = self.sim.model.lattice.nesterov_run(self.maxIterations, dt=self.deltaT, mu=self.mu,
                                                force_cutoff=self.forceCutoff, reset=self._fresh)
        self._fresh = False
        self.iterations, self.forceMax = r["iterations"], r["forceMax"]
        return r


class energyMinimizerGradientDescent(_Updater):
    def __init__(self, model=None):
        super().__init__(model)
        self.setGradientDescentParameters(0.01, 1e-7)
        self.maxIterations = 1000  # energyMinimizerGradientDescent::initializeParameters

    def setGradientDescentParameters(self, deltaT, forceCutoff):
        self.deltaT, self.forceCutoff = deltaT, forceCutoff
        self._fresh = True

    def minimize(self):
        r = self.sim.model.lattice.gd_run(self.maxIterations, dt=self.deltaT, force_cutoff=self.forceCutoff,
                                          reset=self._fresh)
        self._fresh = False
        self.iterations, self.forceMax = r["iterations"], r["forceMax"]
        return r


class energyMinimizerLoLBFGS(_Updater):
    def __init__(self, model=None):
        super().__init__(model)
        self.setLoLBFGSParameters()

    def setLoLBFGSParameters(self, _m=5, _dt=1e-4, _c=1.0, fc=1e-12, _tau=10):
        self.m, self.deltaT, self.c, self.forceCutoff, self.tau = _m, _dt, _c, fc, _tau
        self._fresh = True

    def minimize(self):
        r = self.sim.model.lattice.lbfgs_run(self.maxIterations, eta=self.deltaT, m=self.m,
                                             force_cutoff=self.forceCutoff, reset=self._fresh)
        self._fresh = False
        self.iterations, self.forceMax = r["iterations"], r["forceMax"]
        return r


class multirankSimulation:
    """Single-domain simulation driver (the multirank halo path is not used)."""

    def __init__(self, myRank=0, xDiv=1, yDiv=1, zDiv=1, edges=False, corners=False):
        if (xDiv, yDiv, zDiv) != (1, 1, 1):
            raise NotImplementedError("qmin_gb300 runs a single domain on one GPU")
        self.model = None
        self.forces = []
        self.updaters = []
        self.NActive = 0

    def setConfiguration(self, model):
        self.model = model

    def addForce(self, force, model=None):
        force.sim = self
        self.forces.append(force)

    def addUpdater(self, upd, model=None):
        upd.sim = self
        self.updaters.append(upd)

    def createWall(self, xyz, plane, bObj):
        self.model.geometry.add_wall(xyz, plane, bObj.boundary, bObj.P1, bObj.P2)

    def createSphericalColloid(self, center, radius, bObj):
        self.model.geometry.add_sphere(center, radius, bObj.boundary, bObj.P1, bObj.P2)

    def createBoundaryFromFile(self, fname, verbose=False):
        self.model.geometry.add_boundary_file(fname)

    def saveState(self, fname, latticeSkip=1, defectType=0):
        self.model.lattice.save_state(fname, latticeSkip, defectType)

    def loadState(self, fname):
        self.model.lattice.load_state(fname)

    def finalizeObjects(self):
        m = self.model
        if m.lattice is None:
            m.lattice = Lattice(m.L, m.precision, m.metric_mode)
        for f in self.forces:
            f.apply(m.lattice)
        m.lattice.set_objects(m.geometry.objects())
        m.lattice.set_state(m.geometry.Q, m.geometry.types)
        self.NActive = m.lattice.n_active()

    def computeForces(self):
        return self.model.lattice.force()

    def computePotentialEnergy(self, verbose=False):
        e, comps = self.model.lattice.energy()
        for f in self.forces:
            f.energyComponents = comps
        return e

    def performTimestep(self):
        for u in self.updaters:
            u.Update()
