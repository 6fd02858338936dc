"""``Output`` (src/imc_output.jl): the saved run, and checkpoints.

``save`` writes what ``Output.plotting`` saves with ``jldsave`` (src/imc_output.jl:54-56):
the step times, cell centres and the per-step temperature, radiation and
material energy densities kept by ``main(args, saved=True)``, as NPZ (no JLD2
here), under ``<directory>/<NAME>_<PRECISION>.npz``.  The plots themselves
(Plots.jl) are not reproduced.

``checkpoint`` / ``restore`` write and read the engine's whole state
(imc_save_state / imc_load_state): a restored run continues exactly as the
saved one would have.
"""
import os

import numpy as np


def _precision_name(inputs):
    p = inputs.get("PRECISION", np.float64)
    return {np.float64: "Float64", np.float32: "Float32", np.float16: "Float16"}.get(p, str(p))


def save(inputs, mesh, simvars, directory="outputs"):
    """Writes the saved per-step fields of a run; returns the file path."""
    os.makedirs(directory, exist_ok=True)
    path = os.path.join(directory, "%s_%s.npz" % (inputs["NAME"], _precision_name(inputs)))
    centers = mesh.centers
    if isinstance(centers, tuple):
        extra = {"centers_x": np.asarray(centers[0], dtype=np.float64),
                 "centers_y": np.asarray(centers[1], dtype=np.float64)}
    else:
        extra = {"centers": np.asarray(centers, dtype=np.float64)}
    np.savez_compressed(path, timesteps=np.asarray(simvars.timesteps, dtype=np.float64),
                        temp_saved=np.asarray(mesh.temp_saved, dtype=np.float64),
                        radenergy_saved=np.asarray(mesh.radenergy_saved, dtype=np.float64),
                        matenergy_saved=np.asarray(mesh.matenergy_saved, dtype=np.float64), **extra)
    return path


def checkpoint(engine, path):
    """Writes the engine's state (clock, scalars, cell fields, particles)."""
    blob = engine.save_state()
    with open(path, "wb") as f:
        f.write(blob)
    return len(blob)


def restore(engine, path):
    """Loads a state written by ``checkpoint`` from an engine of the same deck."""
    with open(path, "rb") as f:
        engine.load_state(f.read())
