"""``EnergyCheck.energychecker`` (src/imc_energycheck.jl:10-56): the relative
energy-balance error of the step, FP64 on the GPU (imc_energycheck)."""


def energychecker(inputs, mesh, simvars, particles):
    eng = mesh.engine
    err = eng.energycheck()
    st = eng.stats()
    mesh.totalenergy = st["total_energy"]
    mesh.totalenergydep = st["energy_dep"]
    mesh.radenergyold = st["rad_energy"]
    mesh.lostenergy = 0.0
    return err
