"""qusim_gb300 -- GB300 (sm_103a) split-operator time evolution, a drop-in
GPU_GB300 device for QuSim's SplittingMethod1D/2D (O2, O4).

The engine is libqsg.so (C ABI, include/qsg.h); this package holds its
sources (csrc/), its build (build.py) and a Python mirror of the reference's
Evolver/Options API (evolver.py) and of its Born-series scattering solvers
QuPerturbation1D/2D (born.py).
"""
from ._lib import Plan1D, Plan2D, QsgError, Spec, load  # noqa: F401
from .evolver import (Batch, BoundaryCondition, Calculator, Context, Evolver1D, Evolver2D,  # noqa: F401
                      Functor2DWrapper, FunctorWrapper, Instance, Options, Server, SolverMethod,
                      candidate_plans_1d, default_context)
from .born import QuPerturbation1D, QuPerturbation2D  # noqa: F401
