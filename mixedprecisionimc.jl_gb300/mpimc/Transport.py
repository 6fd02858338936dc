"""``Transport.MC`` / ``Transport.MC2D`` (src/imc_transport.jl:13-210, :483-732):
every history to census, escape or cut-off on the GPU (imc_transport).
``MC_RW`` (src/imc_transport.jl:212-479), the 1D random-walk acceleration, is
not provided: thick cells are the job of the learned transport surrogate."""
from .driver import _grid_k, particles_for


def MC(mesh, simvars, particles):
    eng = mesh.engine
    if eng is None:
        raise RuntimeError("Update.update must run first: it creates the device state")
    particles_for(mesh, particles)
    eng.transport()
    mesh.energydep = _grid_k(mesh, eng.field("energydep"), eng.nscales)


MC2D = MC
