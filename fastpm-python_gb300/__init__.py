"""fastpm_gb300 — GB300-native FastPM particle-mesh engine.

Drop-in for the reference's ``fastpm.core`` path: Solver(pm, cosmology, B)
with .whitenoise / .linear / .lpt / .nbody, leapfrog / autostages, StateVector
(X, V, S, P, F, RHO), running every mesh and particle operation in hand-written
sm_103a CUDA kernels behind the C ABI of include/fastpm_gb300.h.
"""
from .core import Solver, StateVector, FastPMStep, leapfrog, leapfrog_with_lpt, autostages
from .background import MatterDominated, PerturbationGrowth
from .cosmology import Cosmology, Planck15, EHPower, LinearPower
from .pm import ParticleMesh, RealField, ComplexField
from .power import power
from . import _lib

__version__ = '0.1.0'
