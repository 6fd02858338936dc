"""``Tally.tally`` (src/imc_tally.jl:11-149): material energy, temperature and
census radiation energy density, FP64 on the GPU (imc_tally)."""
from .driver import _pull_tally


def tally(inputs, mesh, simvars, particles):
    eng = mesh.engine
    eng.tally()
    _pull_tally(mesh, eng)
