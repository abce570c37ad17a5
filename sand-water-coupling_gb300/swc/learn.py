"""Learned CG warm start: training-data collection and device-side training.

The network (8 -> 64 -> 64 -> 1, SiLU) predicts, per active virtual particle, a
correction of the pressure extrapolated in time from the node's previous
pressures, in units of sD / alpha_hat_I (see include/swc.h for the feature
definitions).  Training data are logged by the plain solver started from that
extrapolated pressure (CG to the configured tolerance); training runs on the GPU
through swc_trainer_* (one fused tensor-core pass for the gradient, Adam).  A trained
model is a pair (params[N_PARAMS], norm[N_NORM]) stored in an .npz file.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .liquid import DualParticleSphLiquid

N_IN = _lib.MLP_IN
N_PARAMS = _lib.MLP_PARAMS
N_NORM = _lib.MLP_NORM


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation (small output layer)."""
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, np.sqrt(2.0 / N_IN), size=(64, N_IN))
    W2 = rng.normal(0, np.sqrt(2.0 / 64), size=(64, 64))
    w3 = rng.normal(0, np.sqrt(1.0 / 64), size=64) * 0.1
    p = np.concatenate([W1.ravel(), np.zeros(64), W2.ravel(), np.zeros(64), w3, [0.0]])
    return p.astype(np.float32)


def normalisation(features: np.ndarray, targets: np.ndarray) -> np.ndarray:
    """Feature means / standard deviations and target mean / std of a dataset."""
    f = np.asarray(features, dtype=np.float64)
    t = np.asarray(targets, dtype=np.float64)
    fm, fs = f.mean(0), f.std(0)
    fs[fs < 1e-6] = 1.0
    ts = t.std() if t.std() > 1e-12 else 1.0
    return np.concatenate([fm, fs, [t.mean(), ts]]).astype(np.float32)


# rows kept for training: a pressure history of at least two steps (history scale
# s above ten times its floor, feature f5 = ln s) and a target within +-TARGET_CLIP
MIN_LOG_SCALE = float(np.log(10 * _lib.MLP_SCALE_EPS))
TARGET_CLIP = 50.0


def collect(scene, steps: int, every: int = 1, keep_fraction: float = 1.0, seed: int = 0, tolerance=None):
    """Run the plain solver on `scene` and log (features, targets) of the projections.

    The solver starts CG from the pressure extrapolated in time (the base of the
    learned correction).  Rows without history (where the network's correction
    vanishes with the scale s) and outlying targets are dropped;
    `keep_fraction` subsamples the remaining nodes per step."""
    rng = np.random.default_rng(seed)
    liq = DualParticleSphLiquid(scene, warm_start="extrapolate", keep_features=True, tolerance=tolerance)
    liq.initialize()
    fs, ts = [], []
    for k in range(steps):
        liq.advance(scene.dt)
        if k % every:
            continue
        f, t = liq.features()
        m = (f[:, 5] > MIN_LOG_SCALE) & (np.abs(t) < TARGET_CLIP)
        f, t = f[m], t[m]
        if keep_fraction < 1.0 and f.shape[0] > 0:
            m = rng.random(f.shape[0]) < keep_fraction
            f, t = f[m], t[m]
        fs.append(f)
        ts.append(t)
    liq.close()
    return np.concatenate(fs), np.concatenate(ts)


class Trainer:
    """Device-side trainer (swc_trainer_*)."""

    def __init__(self, capacity: int, batch: int = 4096):
        self.L = _lib.load()
        h = C.c_void_p()
        rc = self.L.swc_trainer_create(int(capacity), int(batch), C.byref(h))
        if rc:
            raise _lib.SwcError(rc, "swc_trainer_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.swc_trainer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, features, targets):
        f = np.ascontiguousarray(features, dtype=np.float32)
        t = np.ascontiguousarray(targets, dtype=np.float32)
        rc = self.L.swc_trainer_add(self.h, _fp(f), _fp(t), f.shape[0])
        if rc:
            raise _lib.SwcError(rc, "swc_trainer_add")

    def set_params(self, params, norm):
        p = np.ascontiguousarray(params, dtype=np.float32)
        q = np.ascontiguousarray(norm, dtype=np.float32)
        rc = self.L.swc_trainer_set_params(self.h, _fp(p), _fp(q))
        if rc:
            raise _lib.SwcError(rc, "swc_trainer_set_params")

    def params(self):
        p = np.empty(N_PARAMS, dtype=np.float32)
        q = np.empty(N_NORM, dtype=np.float32)
        rc = self.L.swc_trainer_get_params(self.h, _fp(p), _fp(q))
        if rc:
            raise _lib.SwcError(rc, "swc_trainer_get_params")
        return p, q

    def fit(self, epochs: int = 20, lr: float = 1e-3, seed: int = 0):
        loss = np.zeros(max(epochs, 1), dtype=np.float32)
        rc = self.L.swc_trainer_fit(self.h, int(epochs), float(lr), int(seed), _fp(loss))
        if rc:
            raise _lib.SwcError(rc, "swc_trainer_fit")
        return loss[:epochs]


def train(features, targets, epochs: int = 20, lr: float = 1e-3, batch: int = 4096, seed: int = 0):
    """Adam (lr 1e-3) over the logged data on the GPU; returns (params, norm, loss per epoch)."""
    norm = normalisation(features, targets)
    tr = Trainer(features.shape[0], batch)
    tr.add(features, targets)
    tr.set_params(init_params(seed), norm)
    loss = tr.fit(epochs, lr, seed)
    p, q = tr.params()
    tr.close()
    return p, q, loss


def forward(params, norm, features) -> np.ndarray:
    L = _lib.load()
    p = np.ascontiguousarray(params, dtype=np.float32)
    q = np.ascontiguousarray(norm, dtype=np.float32)
    f = np.ascontiguousarray(features, dtype=np.float32)
    out = np.empty(f.shape[0], dtype=np.float32)
    rc = L.swc_mlp_forward(_fp(p), _fp(q), _fp(f), f.shape[0], _fp(out))
    if rc:
        raise _lib.SwcError(rc, "swc_mlp_forward")
    return out


def gradient(params, norm, features, targets):
    L = _lib.load()
    p = np.ascontiguousarray(params, dtype=np.float32)
    q = np.ascontiguousarray(norm, dtype=np.float32)
    f = np.ascontiguousarray(features, dtype=np.float32)
    t = np.ascontiguousarray(targets, dtype=np.float32)
    g = np.empty(N_PARAMS, dtype=np.float32)
    loss = C.c_float()
    rc = L.swc_mlp_gradient(_fp(p), _fp(q), _fp(f), _fp(t), f.shape[0], _fp(g), C.byref(loss))
    if rc:
        raise _lib.SwcError(rc, "swc_mlp_gradient")
    return g, loss.value


def save(path, params, norm, **meta):
    np.savez(path, params=np.asarray(params, dtype=np.float32), norm=np.asarray(norm, dtype=np.float32), **meta)


def load_model(path):
    d = np.load(path)
    p, q = d["params"], d["norm"]
    if p.size != N_PARAMS or q.size != N_NORM:
        raise ValueError(f"{path}: network of {p.size} parameters / {q.size} normalisation values; "
                         f"expected {N_PARAMS} / {N_NORM}")
    return p, q
