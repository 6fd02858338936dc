"""Host-side utilities of the reference's ``Utilities`` module
(src/imc_utilities.jl:6-21).  ``sorter`` (src/imc_utilities.jl:23-54) runs on
the GPU inside the update, sourcing and tally kernels; it has no host copy."""
import numpy as np


def tointeger(x):
    """src/imc_utilities.jl:6-21: Float16 -> UInt16, Float32 -> Int32, else Int64;
    raises like Julia's InexactError when x is not integral."""
    v = float(x)
    if v != v or v in (float("inf"), float("-inf")) or v != int(v):
        raise ValueError("InexactError: %r is not an integer" % (x,))
    if isinstance(x, np.float16):
        return np.uint16(v)
    if isinstance(x, np.float32):
        return np.int32(v)
    return int(v)
