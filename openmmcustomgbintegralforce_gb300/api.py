"""Host-side mirror of the reference's plugin interface for the GB hot path.

The classes keep the reference's names, argument meanings and error
behaviour so that code (and tests) written against the OpenMM plugin read
the same here:

* ``CharmmGBSWForce``  -- openmmapi/include/openmm/CharmmGBSWForce.h:58-203
* ``CharmmGBMVForce``  -- openmmapi/include/openmm/CharmmGBMVForce.h:63-526
  (per-particle/global parameters, computed values, energy terms and
  ``addGBIntegral`` / ``setGBIntegralType``).  The device path evaluates the
  canonical CHARMM expressions; other expressions raise ``GBXError``
  (unsupported) instead of silently computing something else.
* ``CalcCharmmGBSWForceKernel`` / ``CalcCharmmGBMVForceKernel`` -- the
  kernel interface (openmmapi/include/openmm/charmmKernels.h:49-129) with
  ``initialize``, ``execute`` and ``copyParametersToContext``, implemented on
  the gbx C ABI.

There is no CPU path: every evaluation runs the CUDA library.
"""
from __future__ import annotations

import re

import numpy as np

from ._lib import Context, CustomContext, GBXError
from .spec import TABLE_PERIODIC, GBModel

# CharmmGBMVForce.h:87-104
SingleParticle, ParticlePair, ParticlePairNoExclusions = 0, 1, 2
GBSWIntegral, GBMVIntegralTypeI, GBMVIntegralTypeII, CustomIntegral = 0, 1, 2, 3
NoCutoff, CutoffNonPeriodic, CutoffPeriodic = 0, 1, 2

ONE_4PI_EPS0 = 138.935456


class OpenMMException(GBXError):
    """Raised where the reference throws OpenMMException."""

    def __init__(self, message: str):
        super().__init__(1, message)


def _assert_index(index, seq):
    if index < 0 or index >= len(seq):
        raise OpenMMException("Index out of range")


class CharmmGBSWForce:
    """Fixed-function GBSW force (CharmmGBSWForce.h:58-203; defaults from
    CharmmGBSWForce.cpp:40)."""

    NoCutoff, CutoffNonPeriodic, CutoffPeriodic = NoCutoff, CutoffNonPeriodic, CutoffPeriodic

    def __init__(self):
        self._particles = []
        self._method = NoCutoff
        self._cutoff = 1.0
        self._solvent = 78.3
        self._solute = 1.0
        self._sa = 2.25936
        self._contexts = []

    def getNumParticles(self):
        return len(self._particles)

    def addParticle(self, charge, radius, scalingFactor):
        self._particles.append([float(charge), float(radius), float(scalingFactor)])
        return len(self._particles) - 1

    def getParticleParameters(self, index):
        _assert_index(index, self._particles)
        return tuple(self._particles[index])

    def setParticleParameters(self, index, charge, radius, scalingFactor):
        _assert_index(index, self._particles)
        self._particles[index] = [float(charge), float(radius), float(scalingFactor)]

    def getSolventDielectric(self):
        return self._solvent

    def setSolventDielectric(self, d):
        self._solvent = float(d)

    def getSoluteDielectric(self):
        return self._solute

    def setSoluteDielectric(self, d):
        self._solute = float(d)

    def getSurfaceAreaEnergy(self):
        return self._sa

    def setSurfaceAreaEnergy(self, e):
        self._sa = float(e)

    def getNonbondedMethod(self):
        return self._method

    def setNonbondedMethod(self, method):
        if method < 0 or method > 2:
            raise OpenMMException("CharmmGBSWForce: Illegal value for nonbonded method")
        self._method = int(method)

    def getCutoffDistance(self):
        return self._cutoff

    def setCutoffDistance(self, d):
        self._cutoff = float(d)

    def usesPeriodicBoundaryConditions(self):
        return self._method == CutoffPeriodic

    def updateParametersInContext(self, kernel):
        kernel.copyParametersToContext(self)

    # arrays for the kernel
    def _arrays(self):
        p = np.array(self._particles, dtype=np.float64).reshape(-1, 3)
        return p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()


class Continuous1DFunction:
    """OpenMM's tabulated function of one variable: a natural cubic spline
    through ``values`` at evenly spaced points from ``min`` to ``max``, zero
    outside that range (the only TabulatedFunction type the compiled
    expressions take)."""

    def __init__(self, values, min, max):
        self.setFunctionParameters(values, min, max)

    def getFunctionParameters(self):
        return list(self._values), self._min, self._max

    def setFunctionParameters(self, values, min, max):
        if len(values) < 2:
            raise OpenMMException("Continuous1DFunction: must have at least two points")
        if max <= min:
            raise OpenMMException("Continuous1DFunction: max <= min for a tabulated function.")
        self._values, self._min, self._max = [float(v) for v in values], float(min), float(max)


class CharmmGBMVForce:
    """CustomGBForce-style GB force with GB integrals (CharmmGBMVForce.h:63-526)."""

    NoCutoff, CutoffNonPeriodic, CutoffPeriodic = NoCutoff, CutoffNonPeriodic, CutoffPeriodic
    SingleParticle, ParticlePair, ParticlePairNoExclusions = SingleParticle, ParticlePair, ParticlePairNoExclusions
    GBSWIntegral, GBMVIntegralTypeI, GBMVIntegralTypeII, CustomIntegral = (GBSWIntegral, GBMVIntegralTypeI,
                                                                          GBMVIntegralTypeII, CustomIntegral)

    def __init__(self):
        self._method = NoCutoff
        self._cutoff = 1.0
        self._type = GBSWIntegral
        self._perparticle = []
        self._globals = []
        self._particles = []
        self._exclusions = []
        self._values = []
        self._integrals = []
        self._terms = []
        self._param_derivs = []
        self._functions = []

    # --- counts (CharmmGBMVForce.h:113-171)
    def getNumParticles(self):
        return len(self._particles)

    def getNumExclusions(self):
        return len(self._exclusions)

    def getNumPerParticleParameters(self):
        return len(self._perparticle)

    def getNumGlobalParameters(self):
        return len(self._globals)

    def getNumEnergyParameterDerivatives(self):
        return len(self._param_derivs)

    def getNumComputedValues(self):
        return len(self._values)

    def getNumGBIntegrals(self):
        return len(self._integrals)

    def getNumEnergyTerms(self):
        return len(self._terms)

    def getNumTabulatedFunctions(self):
        return len(self._functions)

    # --- nonbonded method
    def getNonbondedMethod(self):
        return self._method

    def setNonbondedMethod(self, m):
        if m < 0 or m > 2:
            raise OpenMMException("CharmmGBMVForce: Illegal value for nonbonded method")
        self._method = int(m)

    def getCutoffDistance(self):
        return self._cutoff

    def setCutoffDistance(self, d):
        self._cutoff = float(d)

    def usesPeriodicBoundaryConditions(self):
        return self._method == CutoffPeriodic

    # --- parameters
    def addPerParticleParameter(self, name):
        self._perparticle.append(name)
        return len(self._perparticle) - 1

    def getPerParticleParameterName(self, index):
        _assert_index(index, self._perparticle)
        return self._perparticle[index]

    def setPerParticleParameterName(self, index, name):
        _assert_index(index, self._perparticle)
        self._perparticle[index] = name

    def addGlobalParameter(self, name, defaultValue):
        self._globals.append([name, float(defaultValue)])
        return len(self._globals) - 1

    def getGlobalParameterName(self, index):
        _assert_index(index, self._globals)
        return self._globals[index][0]

    def setGlobalParameterName(self, index, name):
        _assert_index(index, self._globals)
        self._globals[index][0] = name

    def getGlobalParameterDefaultValue(self, index):
        _assert_index(index, self._globals)
        return self._globals[index][1]

    def setGlobalParameterDefaultValue(self, index, value):
        _assert_index(index, self._globals)
        self._globals[index][1] = float(value)

    def addEnergyParameterDerivative(self, name):
        for k, (n, _) in enumerate(self._globals):
            if n == name:
                self._param_derivs.append(k)
                return
        raise OpenMMException("addEnergyParameterDerivative: Unknown global parameter '" + name + "'")

    def getEnergyParameterDerivativeName(self, index):
        _assert_index(index, self._param_derivs)
        return self._globals[self._param_derivs[index]][0]

    def addParticle(self, parameters=()):
        self._particles.append([float(v) for v in parameters])
        return len(self._particles) - 1

    def getParticleParameters(self, index):
        _assert_index(index, self._particles)
        return list(self._particles[index])

    def setParticleParameters(self, index, parameters):
        _assert_index(index, self._particles)
        self._particles[index] = [float(v) for v in parameters]

    # --- computed values, integrals, energy terms
    def addComputedValue(self, name, expression, type):
        self._values.append([name, expression, int(type)])
        return len(self._values) - 1

    def getComputedValueParameters(self, index):
        _assert_index(index, self._values)
        return tuple(self._values[index])

    def setComputedValueParameters(self, index, name, expression, type):
        _assert_index(index, self._values)
        self._values[index] = [name, expression, int(type)]

    def addGBIntegral(self, name, parametersInt=(), parametersReal=()):
        self._integrals.append([name, [int(v) for v in parametersInt], [float(v) for v in parametersReal]])
        return len(self._integrals) - 1

    def getGBIntegralParameters(self, index):
        _assert_index(index, self._integrals)
        name, pi, pr = self._integrals[index]
        return name, list(pi), list(pr)

    def setGBIntegralParameters(self, index, name, parametersInt, parametersReal):
        _assert_index(index, self._integrals)
        self._integrals[index] = [name, [int(v) for v in parametersInt], [float(v) for v in parametersReal]]

    def setGBIntegralType(self, type):
        self._type = int(type)

    def getGBIntegralType(self):
        return self._type

    def addEnergyTerm(self, expression, type):
        self._terms.append([expression, int(type)])
        return len(self._terms) - 1

    # --- tabulated functions (CharmmGBMVForce.h:434-463)
    def addTabulatedFunction(self, name, function):
        self._functions.append([name, function])
        return len(self._functions) - 1

    def getTabulatedFunction(self, index):
        _assert_index(index, self._functions)
        return self._functions[index][1]

    def getTabulatedFunctionName(self, index):
        _assert_index(index, self._functions)
        return self._functions[index][0]

    def getEnergyTermParameters(self, index):
        _assert_index(index, self._terms)
        return tuple(self._terms[index])

    def setEnergyTermParameters(self, index, expression, type):
        _assert_index(index, self._terms)
        self._terms[index] = [expression, int(type)]

    def addExclusion(self, particle1, particle2):
        self._exclusions.append((int(particle1), int(particle2)))
        return len(self._exclusions) - 1

    def getExclusionParticles(self, index):
        _assert_index(index, self._exclusions)
        return self._exclusions[index]

    def updateParametersInContext(self, kernel):
        kernel.copyParametersToContext(self)


# ---------------------------------------------------------------------------
# The canonical CHARMM GB expression set the device path implements.
# ---------------------------------------------------------------------------
CANONICAL_BORN = "1/(alpha0*(1/0.05-I4)+alpha1*(1/(4*0.05^4)-I7)^(1/4))"
CANONICAL_SELF = "-0.5*{k}*(1-1/80)*q^2/B"
CANONICAL_PAIR = "-{k}*(1-1/80)*q1*q2/sqrt(r^2+B1*B2*exp(-r^2/(4*B1*B2)))"


def canonical_gbmv_force(integral_type: int = GBSWIntegral, alpha0: float = -0.180, alpha1: float = 1.817):
    """A CharmmGBMVForce set up with the canonical CHARMM expressions
    (params q, radius; integrals I4 {4}, I7 {7}; value B; self + pair terms)."""
    f = CharmmGBMVForce()
    f.addPerParticleParameter("q")
    f.addPerParticleParameter("radius")
    f.addGlobalParameter("alpha0", alpha0)
    f.addGlobalParameter("alpha1", alpha1)
    f.addGBIntegral("I4", [4], [])
    f.addGBIntegral("I7", [7], [])
    f.addComputedValue("B", CANONICAL_BORN, SingleParticle)
    f.addEnergyTerm(CANONICAL_SELF.format(k=ONE_4PI_EPS0), SingleParticle)
    f.addEnergyTerm(CANONICAL_PAIR.format(k=ONE_4PI_EPS0), ParticlePairNoExclusions)
    f.addEnergyParameterDerivative("alpha0")
    f.addEnergyParameterDerivative("alpha1")
    f.setGBIntegralType(integral_type)
    return f


def _norm(expr: str) -> str:
    return re.sub(r"\s+", "", expr)


def _check_canonical(force: CharmmGBMVForce):
    if force.getGBIntegralType() == CustomIntegral:
        raise GBXError(4, "CustomIntegral has no implementation")
    names = [force.getPerParticleParameterName(i) for i in range(force.getNumPerParticleParameters())]
    if "radius" not in names:
        raise OpenMMException("GBSWIntegral: the per perticle parameter 'radius' must be defined")
    for k in range(force.getNumGBIntegrals()):
        _, pi, _ = force.getGBIntegralParameters(k)
        if len(pi) == 0:
            raise OpenMMException("GBSWIntegral: the order of integral must be given")
        if pi[0] < 2:
            raise OpenMMException("GBSWIntegral: the order of integral must be greater or equal to 2")
    want_int = [("I4", [4]), ("I7", [7])]
    got_int = [(force.getGBIntegralParameters(k)[0], force.getGBIntegralParameters(k)[1][:1])
               for k in range(force.getNumGBIntegrals())]
    # energy parameter derivatives come from the compiled path only
    ok = got_int == want_int and "q" in names and force.getNumEnergyParameterDerivatives() == 0
    ok = ok and [(_norm(n), _norm(e), t) for n, e, t in (force.getComputedValueParameters(k)
                                                          for k in range(force.getNumComputedValues()))] == \
        [("B", _norm(CANONICAL_BORN), SingleParticle)]
    terms = [(_norm(e), t) for e, t in (force.getEnergyTermParameters(k) for k in range(force.getNumEnergyTerms()))]
    ok = ok and terms == [(_norm(CANONICAL_SELF.format(k=ONE_4PI_EPS0)), SingleParticle),
                          (_norm(CANONICAL_PAIR.format(k=ONE_4PI_EPS0)), ParticlePairNoExclusions)]
    if not ok:
        raise GBXError(4, "the device path evaluates the canonical CHARMM GB expressions only "
                          "(see canonical_gbmv_force)")
    return names.index("q"), names.index("radius")


def custom_spec(force: CharmmGBMVForce) -> dict:
    """The force's expressions as a gbx_create_custom description: computed
    values SingleParticle; energy terms SingleParticle, ParticlePair (skips
    the force's exclusions) or ParticlePairNoExclusions; the globals named
    by addEnergyParameterDerivative; its tabulated functions
    (Continuous1DFunction)."""
    functions = {}
    for k in range(force.getNumTabulatedFunctions()):
        fn = force.getTabulatedFunction(k)
        if not isinstance(fn, Continuous1DFunction):
            raise GBXError(4, "only Continuous1DFunction tabulated functions are supported by the compiled expressions")
        values, lo, hi = fn.getFunctionParameters()
        functions[force.getTabulatedFunctionName(k)] = (values, lo, hi)
    if force.getGBIntegralType() == CustomIntegral:
        raise GBXError(4, "CustomIntegral has no implementation")
    names = [force.getPerParticleParameterName(i) for i in range(force.getNumPerParticleParameters())]
    if "radius" not in names:
        raise OpenMMException("GBSWIntegral: the per perticle parameter 'radius' must be defined")
    integrals = []
    for k in range(force.getNumGBIntegrals()):
        name, pi, _ = force.getGBIntegralParameters(k)
        if len(pi) == 0:
            raise OpenMMException("GBSWIntegral: the order of integral must be given")
        if pi[0] < 2:
            raise OpenMMException("GBSWIntegral: the order of integral must be greater or equal to 2")
        integrals.append((name, pi[0]))
    values = []
    for k in range(force.getNumComputedValues()):
        name, expr, t = force.getComputedValueParameters(k)
        if t != SingleParticle:
            raise GBXError(4, "computed values must be SingleParticle")
        values.append((name, expr))
    terms = []
    for k in range(force.getNumEnergyTerms()):
        expr, t = force.getEnergyTermParameters(k)
        terms.append((expr, {SingleParticle: 0, ParticlePair: 1, ParticlePairNoExclusions: 2}[t]))
    globals_ = {force.getGlobalParameterName(k): force.getGlobalParameterDefaultValue(k)
                for k in range(force.getNumGlobalParameters())}
    return {"params": names, "globals": globals_, "integrals": integrals, "values": values, "terms": terms,
            "exclusions": [force.getExclusionParticles(k) for k in range(force.getNumExclusions())],
            "param_derivs": [force.getEnergyParameterDerivativeName(k)
                             for k in range(force.getNumEnergyParameterDerivatives())],
            "functions": functions}


class CalcCharmmGBSWForceKernel:
    """Kernel for CharmmGBSWForce (charmmKernels.h:94-129) on the gbx C ABI.

    ``model`` overrides the quadrature / table settings (default: the
    reference's 24 x 38 CharmmGBSWForce settings)."""

    Name = "CalcCharmmGBSWForce"

    def __init__(self, model: GBModel | None = None, box=None):
        """``box``: the rectangular periodic box edges (nm) a CutoffPeriodic
        force needs (the Context's box vectors in OpenMM)."""
        self.model = model or GBModel.charmm_gbsw()
        self.box = box
        self.ctx = None

    def initialize(self, numParticles: int, force: CharmmGBSWForce):
        if force.getNumParticles() != numParticles:
            raise OpenMMException("CharmmGBSWForce must have exactly as many particles as the System it belongs to.")
        m = self.model
        if force.getNonbondedMethod() == CutoffPeriodic:
            # CharmmReferenceKernels.cpp:414-430: minimum-image distances in the box
            if self.box is None:
                raise OpenMMException("CutoffPeriodic needs the periodic box: pass box= or call setPeriodicBox first")
            m = m.replace(cutoff=force.getCutoffDistance(), periodic=True, box=tuple(float(b) for b in self.box))
        if force.getNonbondedMethod() == CutoffNonPeriodic:
            m = m.replace(cutoff=force.getCutoffDistance())
        self.model = m
        self.ctx = Context(m, numParticles)
        self.copyParametersToContext(force)

    def copyParametersToContext(self, force: CharmmGBSWForce):
        if self.ctx is None:
            raise OpenMMException("kernel not initialized")
        if force.getNumParticles() != self.ctx.n:
            raise OpenMMException("updateParametersInContext: The number of particles has changed")
        q, R, _ = force._arrays()
        self.ctx.set_particle_parameters(q, R)

    def setPeriodicBox(self, box):
        """The box edges (nm) for the next calls (a barostat step, say)."""
        self.box = box
        if self.ctx is not None:
            self.ctx.set_box(box)

    def execute(self, positions, includeForces: bool = True, includeEnergy: bool = True):
        """Returns (energy, forces[n,3]) for positions in nm."""
        return self.ctx.execute_host(positions, forces=includeForces, energy=includeEnergy)


class CalcCharmmGBMVForceKernel:
    """Kernel for CharmmGBMVForce (charmmKernels.h:49-89) on the gbx C ABI."""

    Name = "CalcCharmmGBMVForce"

    def __init__(self, model: GBModel | None = None, box=None):
        self.model = model
        self.box = box
        self.ctx = None

    def initialize(self, numParticles: int, force: CharmmGBMVForce):
        if force.getNumParticles() != numParticles:
            raise OpenMMException("CharmmGBMVForce must have exactly as many particles as the System it belongs to.")
        for i in range(force.getNumParticles()):
            if len(force.getParticleParameters(i)) != force.getNumPerParticleParameters():
                raise OpenMMException(f"CharmmGBMVForce: Wrong number of parameters for particle {i}")
        try:
            self._iq, self._ir = _check_canonical(force)
            self.custom = None
        except GBXError as e:
            if e.status != 4:
                raise
            # outside the canonical set: the expressions are compiled for the device
            self.custom = custom_spec(force)
        t = force.getGBIntegralType()
        box = tuple(self.box) if self.box is not None else (10.0, 10.0, 10.0)
        base = {GBSWIntegral: GBModel.gbsw_integral(), GBMVIntegralTypeI: GBModel.gbmv1(box=box),
                GBMVIntegralTypeII: GBModel.gbmv2(box=box)}[t]
        m = self.model or base
        if force.getNonbondedMethod() == CutoffPeriodic:
            # the integral classes measure distances by minimum image, GBSWIntegral on the
            # box-sampled table (GBSWIntegral.cpp:63-68,109), and the pair terms too
            # (CharmmReferenceGBMV.cpp:294-297)
            if self.box is None:
                raise OpenMMException("CutoffPeriodic needs the periodic box: pass box= to the kernel")
            m = m.replace(cutoff=force.getCutoffDistance(), periodic=True, box=tuple(float(b) for b in self.box),
                          table_mode=TABLE_PERIODIC)
        if force.getNonbondedMethod() == CutoffNonPeriodic:
            m = m.replace(cutoff=force.getCutoffDistance())
        globals_ = {force.getGlobalParameterName(k): force.getGlobalParameterDefaultValue(k)
                    for k in range(force.getNumGlobalParameters())}
        m = m.replace(alpha0=globals_.get("alpha0", m.alpha0), alpha1=globals_.get("alpha1", m.alpha1),
                      pref=-ONE_4PI_EPS0 * (1 - 1 / 80))
        if self.custom is not None:
            m = m.replace(orders=tuple(o for _, o in self.custom["integrals"]))
        self.model = m
        self.ctx = Context(m, numParticles) if self.custom is None else CustomContext(m, numParticles, self.custom)
        self.copyParametersToContext(force)

    def copyParametersToContext(self, force: CharmmGBMVForce):
        if force.getNumParticles() != self.ctx.n:
            raise OpenMMException("updateParametersInContext: The number of particles has changed")
        p = np.array([force.getParticleParameters(i) for i in range(force.getNumParticles())], dtype=np.float64)
        if self.custom is not None:
            self.ctx.set_custom_parameters(p)
        else:
            self.ctx.set_particle_parameters(p[:, self._iq], p[:, self._ir])

    def setGlobalParameters(self, alpha0, alpha1):
        self.ctx.set_global_parameters(alpha0, alpha1)

    def setGlobalParameter(self, name, value):
        """A global parameter of a force outside the canonical set (Context.setParameter)."""
        if self.custom is None:
            raise GBXError(4, "the canonical set takes alpha0, alpha1 through setGlobalParameters")
        self.ctx.set_custom_global(name, value)

    def setPeriodicBox(self, box):
        self.ctx.set_box(box)

    def execute(self, positions, includeForces: bool = True, includeEnergy: bool = True):
        return self.ctx.execute_host(positions, forces=includeForces, energy=includeEnergy)

    def getEnergyParameterDerivatives(self) -> dict:
        """dE/dg of the last execute for each global the force named with
        addEnergyParameterDerivative (State.getEnergyParameterDerivatives)."""
        if self.custom is None or not self.custom["param_derivs"]:
            return {}
        return dict(zip(self.custom["param_derivs"], (float(v) for v in self.ctx.param_derivs())))
