"""Output: the saved per-step fields (Output.plotting's jldsave,
src/imc_output.jl:54-56) as NPZ, and checkpoint / resume."""
import os
from types import SimpleNamespace

import numpy as np
import pytest

from conftest import load_deck


def test_save_writes_the_reference_fields(tmp_path):
    import mpimc
    inputs = {"NAME": "Slab", "PRECISION": np.float32}
    mesh = SimpleNamespace(centers=np.linspace(0.05, 0.95, 10), temp_saved=[np.ones(10)] * 4,
                           radenergy_saved=[np.zeros(10)] * 3, matenergy_saved=[np.zeros(10)] * 3)
    simvars = SimpleNamespace(timesteps=[0.0, 0.1, 0.2])
    path = mpimc.Output.save(inputs, mesh, simvars, directory=str(tmp_path))
    assert os.path.basename(path) == "Slab_Float32.npz"
    z = np.load(path)
    assert z["timesteps"].shape == (3,) and z["temp_saved"].shape == (4, 10)
    assert z["radenergy_saved"].shape == (3, 10) and z["centers"].shape == (10,)


@pytest.mark.gpu
@pytest.mark.parametrize("deck,ov", [("c1_slab", {}), ("tiny_2d", {}), ("c1_slab", {"precision": 2, "scale_select_precision": 2})])
def test_checkpoint_resume_is_exact(deck, ov, tmp_path, gpu_lib):
    """A run restored from a mid-run checkpoint ends with the same fields,
    bit for bit, as the run that wrote it."""
    import mpimc
    inputs, mesh = load_deck(deck)
    a = mpimc.Engine(inputs, mesh, ov)
    a.run(max_steps=5)
    path = os.path.join(str(tmp_path), "state.bin")
    nbytes = mpimc.Output.checkpoint(a, path)
    assert nbytes > 0
    sa, _ = a.run()
    b = mpimc.Engine(inputs, mesh, ov)
    mpimc.Output.restore(b, path)
    assert b.time()[2] == 5
    sb, _ = b.run()
    assert len(sa) == len(sb)
    for f in ("temp", "radenergydens", "matenergydens", "energydep"):
        assert np.array_equal(a.field(f), b.field(f)), f
    assert [s["segments"] for s in sa] == [s["segments"] for s in sb]
    a.close()
    b.close()


@pytest.mark.gpu
def test_restore_rejects_another_deck(tmp_path, gpu_lib):
    import mpimc
    a = mpimc.Engine(*load_deck("c1_slab"))
    a.run(max_steps=2)
    blob = a.save_state()
    b = mpimc.Engine(*load_deck("tiny_1d"))
    with pytest.raises(mpimc.ImcError):
        b.load_state(blob)
    with pytest.raises(mpimc.ImcError):
        b.load_state(blob[:100])
    a.close()
    b.close()


@pytest.mark.gpu
def test_main_saved_run_writes_output(tmp_path, gpu_lib):
    import mpimc
    from conftest import deck_path
    res = mpimc.main([deck_path("tiny_1d")], verbose=False, saved=True)
    path = mpimc.Output.save(res.inputs, res.mesh, res.simvars, directory=str(tmp_path))
    z = np.load(path)
    assert len(z["temp_saved"]) == len(res.steps) + 1  # the initial field and one per step
    assert z["radenergy_saved"].shape[0] == len(res.steps)
