"""The C-ABI library (CPU): libimc.so builds for sm_103a, loads, and exports
every function include/imc.h declares.  No compute calls: none of these
needs a GPU."""
import ctypes as C
import os
import re

import pytest

from conftest import REPO


def _declared():
    src = open(os.path.join(REPO, "include", "imc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*int\s+(imc_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_the_stage_entry_points():
    names = _declared()
    for stage in ("imc_update", "imc_sourcing", "imc_transport", "imc_clean", "imc_tally", "imc_energycheck",
                  "imc_timestep", "imc_step", "imc_run", "imc_create", "imc_destroy"):
        assert stage in names


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = C.CDLL(gpu_lib._name)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(gpu_lib):
    from mpimc._lib import SIGNATURES
    assert sorted(SIGNATURES) == _declared()


def test_abi_version_and_null_arguments(gpu_lib):
    assert gpu_lib.imc_abi_version() == 1
    h = C.c_void_p()
    rc = gpu_lib.imc_create(None, C.byref(h))
    assert rc == 1 and not h.value  # IMC_ERR_INVALID_ARG, before any CUDA call
    buf = C.create_string_buffer(128)
    assert gpu_lib.imc_last_error(None, buf, 128) == 1 and b"NULL" in buf.value


def test_invalid_deck_rejected_before_device_use(gpu_lib):
    import numpy as np
    import mpimc
    from conftest import load_deck
    inputs, mesh = load_deck("tiny_1d")
    d, keep = mpimc.build_deck(inputs, mesh)
    d.n_scales = 0
    h = C.c_void_p()
    assert gpu_lib.imc_create(C.byref(d), C.byref(h)) == 1
    d.n_scales = 2
    d.abi_version = 99
    assert gpu_lib.imc_create(C.byref(d), C.byref(h)) == 1


def test_batch_entry_points_reject_bad_lists_before_device_use(gpu_lib):
    """Both batch entry points check the handle list before touching any
    handle: NULL list, empty list, a NULL handle, a handle given twice, and
    (fused) more decks than its constant-memory table holds."""
    fake = [C.c_void_p(0x1000 + 0x100 * i) for i in range(257)]

    def arr(ptrs):
        return (C.c_void_p * len(ptrs))(*[p.value if p is not None else None for p in ptrs])

    steps = (C.c_int64 * 257)()
    wall, bad = C.c_double(), C.c_int32()
    fused = gpu_lib.imc_run_batch_fused
    assert fused(None, 1, 10, steps, C.byref(wall), C.byref(bad)) == 1
    assert fused(arr(fake[:1]), 0, 10, steps, C.byref(wall), C.byref(bad)) == 1
    assert fused(arr(fake), 257, 10, steps, C.byref(wall), C.byref(bad)) == 1
    assert fused(arr([fake[0], None]), 2, 10, steps, C.byref(wall), C.byref(bad)) == 1
    assert fused(arr([fake[0], fake[0]]), 2, 10, steps, C.byref(wall), C.byref(bad)) == 1
    side = gpu_lib.imc_run_batch
    assert side(None, 1, 10, 4, steps, C.byref(wall), C.byref(bad)) == 1
    assert side(arr([fake[0], None]), 2, 10, 4, steps, C.byref(wall), C.byref(bad)) == 1
    assert side(arr([fake[0], fake[0]]), 2, 10, 4, steps, C.byref(wall), C.byref(bad)) == 1
    assert side(arr(fake[:1]), 1, 10, 0, steps, C.byref(wall), C.byref(bad)) == 1
