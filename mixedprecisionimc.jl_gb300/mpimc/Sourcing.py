"""``Sourcing.sourcing`` (src/imc_sourcing.jl:12-370): emission energies,
particle budget and births, appended to the GPU-resident particle list
(imc_sourcing)."""
from .driver import _grid_k, particles_for


def sourcing(mesh, simvars, particles):
    eng = mesh.engine
    if eng is None:
        raise RuntimeError("Update.update must run first: it creates the device state")
    particles_for(mesh, particles)
    eng.set_time(float(simvars.t), float(simvars.dt))
    eng.sourcing()
    mesh.emittedenergy = _grid_k(mesh, eng.field("emittedenergy"), eng.nscales)
