"""``Transport.MC`` / ``Transport.MC2D`` (src/imc_transport.jl:13-210, :483-732):
every history to census, escape or cut-off on the GPU (imc_transport).
``MC_RW`` (src/imc_transport.jl:212-479), the 1D random-walk acceleration, is
taken by the learned thick-cell surrogate (mpimc.surrogate): the same GPU
transport with the surrogate turned on, for FP32 / FP16 particle state."""
from .driver import _grid_k, particles_for


def MC(mesh, simvars, particles):
    eng = mesh.engine
    if eng is None:
        raise RuntimeError("Update.update must run first: it creates the device state")
    particles_for(mesh, particles)
    eng.transport()
    mesh.energydep = _grid_k(mesh, eng.field("energydep"), eng.nscales)


MC2D = MC


def MC_RW(mesh, simvars, rwvars, particles):
    """RANDOMWALK = TRUE: transport with the learned surrogate in thick cells
    (``rwvars``, the reference's random-walk table, is not needed and may be
    None)."""
    from . import surrogate
    eng = mesh.engine
    if eng is None:
        raise RuntimeError("Update.update must run first: it creates the device state")
    surrogate.enable(eng)
    MC(mesh, simvars, particles)
