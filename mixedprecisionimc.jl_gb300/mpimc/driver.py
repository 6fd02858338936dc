"""Driver of the reference's main module (src/MixedPrecisionIMC.jl): ``SimVars``,
``timestep``, ``main(args)``, plus the glue the per-stage mirrors share.

The stage functions keep the reference's signatures -- ``update(inputs, mesh,
simvars)``, ``sourcing(mesh, simvars, particles)``, ``MC(mesh, simvars,
particles)``, ``clean(particles)``, ``tally(inputs, mesh, simvars, particles)``,
``energychecker(inputs, mesh, simvars, particles)`` -- and each runs one C-ABI
stage on the GPU.  The device state lives in ``mesh.engine``; after each stage
the mirrors copy back the mesh fields that stage changes, so code written
against the reference's in-place mutation sees the same fields change.
``main`` drives whole steps (imc_step / imc_run) without those copies.
"""
import sys
import time
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from . import Constants, Input, Mesh
from .engine import Engine


@dataclass
class SimVars:
    """src/MixedPrecisionIMC.jl:35-51, the 15 positional fields in order."""
    t: Any
    dt: Any
    dt0: Any
    k: Any
    dtmax: Any
    t_end: Any
    timesteps: Any
    iterations: int
    n_input: int
    n_max: int
    cellmin: Any
    pairwise: Any
    BC: Any
    precision: Any
    geometry: Any


def _shape(mesh):
    return (mesh.Ncells,) if np.ndim(mesh.Ncells) == 0 else tuple(mesh.Ncells)


def _grid(mesh, flat):
    """engine cell order (x fastest) -> the mesh's (Nx[, Ny]) array"""
    return np.asarray(flat).reshape(_shape(mesh), order="F")


def _grid_k(mesh, flat, K):
    a = np.asarray(flat).reshape((K,) + (int(np.prod(_shape(mesh))),))
    return np.stack([_grid(mesh, a[k]) for k in range(K)], axis=-1)


def ensure_engine(inputs, mesh, simvars=None):
    """The device state behind ``mesh`` (created on first use), clock = simvars."""
    if mesh.engine is None:
        mesh.engine = Engine(inputs, mesh)
    eng = mesh.engine
    if simvars is not None:
        eng.set_time(float(simvars.t), float(simvars.dt))
    return eng


class ParticleList:
    """The particle list, resident on the GPU.  ``len`` is the list length;
    ``records()`` copies it to the host in the reference's record layout
    (1D: [origin, t, cell, x, mu, freq, E, E0, escale], 1-based cell;
    2D: [t, ix, iy, x, y, angle, freq, E, E0, escale])."""

    def __init__(self, mesh=None):
        self.mesh = mesh

    def __len__(self):
        if self.mesh is None or self.mesh.engine is None:
            return 0
        return self.mesh.engine.num_particles()

    def records(self):
        eng = self.mesh.engine
        p = eng.particles()
        scales = np.asarray(self.mesh.energyscales)
        out = []
        for i in range(len(p["E"])):
            s = float(scales[p["scale"][i]])
            if eng.geometry == 1:
                c = int(p["cell"][i]) + 1
                out.append([c, p["t"][i], c, p["x"][i], p["mu"][i], 1.0, p["E"][i], p["E0"][i], s])
            else:
                ix, iy = int(p["cell"][i]) % eng.nx + 1, int(p["cell"][i]) // eng.nx + 1
                ang = float(np.arctan2(p["uy"][i], p["ux"][i]))
                out.append([p["t"][i], ix, iy, p["x"][i], p["y"][i], ang, 1.0, p["E"][i], p["E0"][i], s])
        return out


def particles_for(mesh, particles):
    if isinstance(particles, ParticleList):
        particles.mesh = mesh
    return particles


def timestep(timestepping, simvars):
    """src/MixedPrecisionIMC.jl:181-222 (host clock; the engine keeps its own
    identical FP64 copy)."""
    if simvars.t == simvars.t_end:
        simvars.t = simvars.t_end + simvars.dt
        return
    if timestepping == "CONSTANT":
        if simvars.t + simvars.dt > simvars.t_end:
            simvars.dt = simvars.t_end - simvars.t
            simvars.t = simvars.t_end
        else:
            simvars.t = simvars.t + simvars.dt
    elif timestepping == "RAMP":
        if simvars.dt < simvars.dtmax:
            simvars.dt = simvars.dt * simvars.k
            if simvars.dt > simvars.dtmax:
                simvars.dt = simvars.dtmax
        if simvars.t + simvars.dt > simvars.t_end:
            simvars.dt = simvars.t_end - simvars.t
            simvars.t = simvars.t_end
        else:
            simvars.t = simvars.t + simvars.dt
    simvars.timesteps.append(simvars.t)


def make_simvars(inputs, mesh):
    """src/MixedPrecisionIMC.jl:88-125 (clock values kept in FP64)."""
    precision = inputs.get("PRECISION", np.float64)
    p = lambda k: float(precision(float(inputs[k])))
    f64 = lambda k: float(inputs[k])  # the clock is FP64 for every PRECISION
    ts = str(inputs["TIMESTEPPING"]).upper()
    if ts == "CONSTANT":
        dt, t_end, dt0, k, dtmax = f64("DT"), f64("ENDTIME"), 0.0, 0.0, 0.0
    elif ts == "RAMP":
        dt0, k, dtmax, t_end = f64("DT0"), f64("K"), f64("DTMAX"), f64("ENDTIME")
        dt = dt0
    else:
        raise ValueError("TIMESTEPPING must be CONSTANT or RAMP")
    geometry = str(inputs["GEOMETRY"])
    if geometry == "1D":
        BC = (str(inputs["LEFTBC"]).upper(), str(inputs["RIGHTBC"]).upper())
    else:
        BC = tuple(str(inputs[k]).upper() for k in ("LEFTBC", "RIGHTBC", "TOPBC", "BOTTOMBC"))
    return SimVars(0.0, dt, dt0, k, dtmax, t_end, [], 0, int(float(inputs["NINPUT"])),
                   int(float(inputs["NMAX"])), p("CELLMIN"), inputs.get("PAIRWISE", "FALSE"), BC, precision,
                   geometry)


@dataclass
class RunResult:
    """What main() leaves behind: the mesh fields of the final step and the
    per-step scalars the reference prints (src/imc_energycheck.jl:31-38)."""
    inputs: dict
    mesh: Any
    simvars: SimVars
    steps: list = field(default_factory=list)
    wall_seconds: float = 0.0
    device_ms: float = 0.0


def main(args, verbose=True, saved=False):
    """src/MixedPrecisionIMC.jl:59-179: read the deck, build the mesh and run
    every timestep on the GPU.  With ``saved`` the per-step temperature,
    radiation and material energy densities are kept as the reference keeps
    them (mesh.temp_saved, radenergy_saved, matenergy_saved)."""
    if not args:
        print("No input file provided, exiting... ")
        return None
    t0 = time.perf_counter()
    input_file = args[0]
    if verbose:
        print("Input file: ", input_file)
    inputs = Input.readInputs(input_file)
    Constants.set_constants(inputs)
    mesh = Mesh.mesh_generation(inputs)
    simvars = make_simvars(inputs, mesh)
    eng = ensure_engine(inputs, mesh)
    if str(inputs.get("RANDOMWALK", "FALSE")).upper() == "TRUE":
        # src/MixedPrecisionIMC.jl:127,140: Transport.MC_RW -> the learned surrogate
        from . import surrogate
        on = surrogate.enable(eng)
        if verbose:
            print("Random walk: learned thick-cell surrogate", "on" if on else "off (needs 1D, FP32/FP16 state)")
    res = RunResult(inputs=inputs, mesh=mesh, simvars=simvars)
    ts = str(inputs["TIMESTEPPING"]).upper()
    if saved:
        done = False
        while not done:
            st, done = eng.step()
            res.steps.append(st)
            _pull_tally(mesh, eng)
            simvars.iterations += int(st["segments"])
            if verbose:
                _print_step(st)
            timestep(ts, simvars)
    else:
        steps, ms = eng.run()
        res.steps = steps
        res.device_ms = ms
        for st in steps:
            simvars.iterations += int(st["segments"])
            timestep(ts, simvars)
            if verbose:
                _print_step(st)
        _pull_tally(mesh, eng, save=False)
    res.wall_seconds = time.perf_counter() - t0
    if verbose:
        print("The simulation took ", res.wall_seconds, " seconds to run ")
    return res


def _print_step(st):
    print("Time: ", st["t"])
    print("Total energy: ", st["total_energy"], " Total energy deposition: ", st["energy_dep"],
          " Radiation energy change: ", st["rad_energy"] - st["rad_energy_old"], " Lost energy: ", st["lost_energy"])
    print("The energy conservation error is: ", st["energy_error"], " ")


def _pull_update(mesh, eng):
    mesh.beta = _grid(mesh, eng.field("beta"))
    mesh.fleck = _grid(mesh, eng.field("fleck"))
    mesh.bee = _grid(mesh, eng.field("bee"))
    mesh.sigma_a = mesh.sigma_a.copy()
    mesh.sigma_s = mesh.sigma_s.copy()
    mesh.sigma_a[..., 0] = _grid(mesh, eng.field("sigma_a"))
    mesh.sigma_s[..., 0] = _grid(mesh, eng.field("sigma_s"))


def _pull_tally(mesh, eng, save=True):
    mesh.temp = _grid(mesh, eng.field("temp"))
    mesh.matenergydens = _grid(mesh, eng.field("matenergydens"))
    mesh.radenergydens = _grid(mesh, eng.field("radenergydens"))
    if save:
        mesh.temp_saved.append(mesh.temp.copy())
        mesh.matenergy_saved.append(mesh.matenergydens.copy())
        mesh.radenergy_saved.append(mesh.radenergydens.copy())


if __name__ == "__main__":
    main(sys.argv[1:])
