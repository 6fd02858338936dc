"""mpimc -- host side of the GB300 Implicit Monte Carlo engine.

Mirrors the module layout of MixedPrecisionIMC.jl (Input, Constants, Mesh, Output,
Update, Sourcing, Transport, Clean, Tally, EnergyCheck, Utilities and the
main module's SimVars / timestep / main) over the C ABI of libimc.so
(include/imc.h).  Every particle and mesh computation runs in the library's
sm_103a kernels.
"""
from . import Constants, Input, Mesh, Output, Utilities  # noqa: F401
from . import Clean, EnergyCheck, Sourcing, Tally, Transport, Update  # noqa: F401
from .driver import ParticleList, RunResult, SimVars, main, make_simvars, timestep  # noqa: F401
from .engine import Engine, build_deck, device_info, run_batch  # noqa: F401
from ._lib import ImcError  # noqa: F401
