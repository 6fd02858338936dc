"""``Clean.clean`` (src/imc_clean.jl:6-19): stable removal of killed particles
(slot 8 == -1.0), run by the GPU compaction kernels (imc_clean).

``clean`` accepts the GPU-resident ``ParticleList`` or, as the reference's own
test does, a plain list of records; a plain list is staged through a scratch
one-cell FP64 engine whose compaction decides which records survive."""
import numpy as np

from .driver import ParticleList


def _scratch_engine():
    from . import Mesh
    from .engine import Engine
    inputs = {
        "PRECISION": np.float64, "GEOMETRY": "1D", "MESHTYPE": "UNIFORM", "XSIZE": "1.0", "DX": "1.0",
        "T_INIT": "1.0", "T_SURFACE_VALS": ["0.0", "0.0"], "SIGMA_A_REGS": [""], "SIGMA_A_VALS": ["1.0"],
        "SIGMA_A_POWERS": ["0.0"], "SIGMA_S_REGS": [""], "SIGMA_S_VALS": ["0.0"], "SIGMA_S_POWERS": ["0.0"],
        "BEE_REGS": [""], "BEE_VALS": ["1.0"], "RADSOURCE_REGS": [""], "RADSOURCE_VALS": ["0.0"],
        "ENERGYSCALES": ["1.0"], "DISTANCESCALE": "1.0", "PHYS_C": "1.0", "PHYS_A": "1.0", "ALPHA": "1.0",
        "LEFTBC": "REFLECT", "RIGHTBC": "REFLECT", "TIMESTEPPING": "CONSTANT", "DT": "1.0", "ENDTIME": "1.0",
        "NINPUT": "0", "NMAX": "0", "CELLMIN": "0", "SEED": "0",
    }
    return Engine(inputs, Mesh.mesh_generation(inputs))


def clean(particles):
    if isinstance(particles, ParticleList):
        particles.mesh.engine.clean()
        return
    n = len(particles)
    if n == 0:
        return
    with _scratch_engine() as eng:
        # slot 8 carries the kill flag; the record index rides in t (exact in FP64)
        eng.set_particles({"t": np.arange(n, dtype=np.float64), "x": np.zeros(n), "mu": np.ones(n),
                           "E": np.ones(n), "E0": np.array([float(r[7]) for r in particles]),
                           "cell": np.zeros(n, dtype=np.int32)})
        eng.clean()
        keep = eng.particles()["t"].astype(np.int64)
    survivors = [particles[i] for i in keep]
    particles[:] = survivors
