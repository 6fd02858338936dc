"""``Update.update`` (src/imc_update.jl:12-56): opacities, beta and Fleck factor
per cell, computed in FP64 by the ``k_update`` kernel (imc_update)."""
from .driver import _pull_update, ensure_engine


def update(inputs, mesh, simvars):
    eng = ensure_engine(inputs, mesh, simvars)
    eng.update()
    _pull_update(mesh, eng)
