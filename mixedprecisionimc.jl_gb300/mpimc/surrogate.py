"""Learned thick-cell transport surrogate: training and test calls.

Inside one cell a history of Transport.MC (src/imc_transport.jl:72-193) is a
random walk whose outcome depends only on its state in mean free paths
(distance to the nearer face d_n, to the farther face d_f, direction cosine
mu' away from the nearer face, and the path lmax after which census or the
1 % energy cut-off ends it).  A 4-64-64-64-64 ReLU network trained on GPU-
generated analog walks gives the outcome's probabilities and the quantiles of
its exit path / exit angle, or final displacement / direction; the transport
kernel samples them instead of walking (Engine.set_surrogate).

All calls run on the GPU through libimc.so (include/imc.h); arrays are numpy.
"""
import ctypes as C

import numpy as np

from . import _lib

N_PARAMS = 12800
NEAR, FAR, TRUNC = 0, 1, 2
LMAX_MIN, LMAX_MAX, CELL_MIN, MIN_GAIN = 32.0, 1.0e4, 8.0, 100.0

# default training run: 2^23 walks, 30000 Adam steps of 8192 walks
DEFAULT_TRAIN = dict(seed=20240607, n_samples=1 << 23, batch=8192, iterations=30000, lr=2e-3, lr_min=1e-5)


def _ok(rc, what):
    if rc != _lib.IMC_OK:
        raise _lib.ImcError(rc, "%s failed: %s" % (what, _lib.ERROR_NAMES.get(rc, str(rc))))


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None and a.shape != shape:
        raise ValueError("expected shape %s, got %s" % (shape, a.shape))
    return a


def train(seed=None, n_samples=None, batch=None, iterations=None, lr=None, lr_min=None, return_loss=False):
    """Generates analog walks and trains the network on the GPU; returns the
    FP32 parameters (and the per-step mean batch loss)."""
    cfg = dict(DEFAULT_TRAIN)
    for k, v in dict(seed=seed, n_samples=n_samples, batch=batch, iterations=iterations, lr=lr,
                     lr_min=lr_min).items():
        if v is not None:
            cfg[k] = v
    c = _lib.ImcSurrogateTrainConfig(cfg["seed"], cfg["n_samples"], cfg["batch"], cfg["iterations"], cfg["lr"],
                                     cfg["lr_min"])
    P = np.zeros(N_PARAMS, np.float32)
    loss = np.zeros(cfg["iterations"], np.float32)
    _ok(_lib.load().imc_surrogate_train(C.byref(c), _ptr(P), _ptr(loss)), "imc_surrogate_train")
    return (P, loss) if return_loss else P


_CACHE = {}


def trained_params():
    """The default network, trained once per process (about 2.5 s on a GB300)."""
    if "P" not in _CACHE:
        _CACHE["P"] = train()
    return _CACHE["P"]


def enable(engine):
    """Turns the surrogate on for an Engine if its deck allows it (1D, FP32 or
    FP16 particle state); returns whether it is on."""
    if engine.surrogate_active():
        return True
    if engine.geometry != _lib.IMC_GEOM_1D or engine.deck.precision == _lib.IMC_FP64:
        return False
    engine.set_surrogate(trained_params())
    return True


def walk(seed, state=None, n=None):
    """Analog in-cell walks: (x n x 4, cls n, tgt n x 2).  state: n x 4 rows of
    (d_n, d_f, mu', lmax), or None to draw n training states."""
    if state is not None:
        state = _f32(state)
        n = len(state)
    x = np.zeros((n, 4), np.float32)
    cls = np.zeros(n, np.int32)
    tgt = np.zeros((n, 2), np.float32)
    _ok(_lib.load().imc_surrogate_walk(seed, _ptr(state) if state is not None else None, n, _ptr(x), _ptr(cls),
                                       _ptr(tgt)), "imc_surrogate_walk")
    return x, cls, tgt


def grad(params, x, cls, tgt):
    """(mean loss, gradient) of the training loss on the GPU in FP32."""
    P = _f32(params, (N_PARAMS,))
    x = _f32(x)
    cls = np.ascontiguousarray(cls, dtype=np.int32)
    tgt = _f32(tgt)
    g = np.zeros(N_PARAMS, np.float32)
    loss = C.c_double(0.0)
    _ok(_lib.load().imc_surrogate_grad(_ptr(P), _ptr(x), _ptr(cls), _ptr(tgt), len(x), _ptr(g), C.byref(loss)),
        "imc_surrogate_grad")
    return loss.value, g


def forward(params, x):
    """Network outputs (n x 64) by the transport kernel's BF16 tensor-core pass."""
    P = _f32(params, (N_PARAMS,))
    x = _f32(x)
    out = np.zeros((len(x), 64), np.float32)
    _ok(_lib.load().imc_surrogate_forward(_ptr(P), _ptr(x), len(x), _ptr(out)), "imc_surrogate_forward")
    return out


def sample(params, seed, state):
    """Outcomes sampled from the network at the given walk states, as the
    transport kernel samples them: (cls, y0, y1)."""
    P = _f32(params, (N_PARAMS,))
    state = _f32(state)
    n = len(state)
    cls = np.zeros(n, np.int32)
    y0 = np.zeros(n, np.float32)
    y1 = np.zeros(n, np.float32)
    _ok(_lib.load().imc_surrogate_sample(_ptr(P), seed, _ptr(state), n, _ptr(cls), _ptr(y0), _ptr(y1)),
        "imc_surrogate_sample")
    return cls, y0, y1
