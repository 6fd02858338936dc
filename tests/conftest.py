"""Shared test set-up: import paths for the host package and the oracle, the
``gpu`` marker, and deck helpers."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "mixedprecisionimc.jl_gb300")
for p in (PKG, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

DECKS = os.path.join(REPO, "tests", "golden", "decks")
# Root of a reference checkout, for the tests that read its files directly
# (its decks and its own test deck); they skip when IMC_REFERENCE is unset.
REFERENCE = os.environ.get("IMC_REFERENCE", "")


def reference_file(rel):
    """Path of a file of the reference checkout, or None if it is absent."""
    if not REFERENCE:
        return None
    p = os.path.join(REFERENCE, rel)
    return p if os.path.exists(p) else None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103)")


def deck_path(name):
    return os.path.join(DECKS, name + ".txt")


def load_deck(name, **overrides):
    """(inputs, mesh) of a test deck; overrides replace deck keywords."""
    import mpimc
    inputs = mpimc.Input.readInputs(deck_path(name))
    for k, v in overrides.items():
        inputs[k] = v
    mesh = mpimc.Mesh.mesh_generation(inputs)
    return inputs, mesh


@pytest.fixture(scope="session")
def gpu_lib():
    """libimc.so, built if needed; the GPU tests fail (not skip) without it."""
    import mpimc._build
    mpimc._build.build()
    import mpimc._lib
    return mpimc._lib.load()


@pytest.fixture(scope="session")
def surrogate_params(gpu_lib):
    """The learned surrogate, trained once per session on the GPU with the
    default configuration (mpimc.surrogate.DEFAULT_TRAIN), and its loss curve."""
    from mpimc import surrogate
    return surrogate.train(return_loss=True)
