"""Python handle on the learned warm-start network of the C ABI (b3g_mlp_*).

The network predicts per-contact-point impulses (contact row, second and first friction rows)
from 12 local features; see include/b3g_capi.h for the feature list and the parameter layout.
Everything runs on the GPU through the library; this module only moves host arrays.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import capi
from .capi import call, fptr

N_FEATURES, N_OUTPUTS = 12, 3
N_PARAMS, N_NORM = 35075, 30
DEFAULT_WEIGHTS = Path(__file__).resolve().parent / "data" / "warmstart_mlp.npz"


class WarmStartMLP:
    def __init__(self, device: int = 0, seed: int = 0):
        capi.load()
        self.handle = C.c_void_p()
        call("b3g_mlp_create", C.c_int(device), C.c_ulonglong(seed), C.byref(self.handle))

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and capi._LIB is not None:
            capi._LIB.b3g_mlp_destroy(h)
            self.handle = None

    # ---- parameters
    @property
    def params(self) -> np.ndarray:
        p = np.zeros(N_PARAMS, np.float32)
        call("b3g_mlp_get_params", self.handle, fptr(p), C.c_int(N_PARAMS))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        call("b3g_mlp_set_params", self.handle, fptr(p), C.c_int(len(p)))

    @property
    def normalization(self) -> np.ndarray:
        n = np.zeros(N_NORM, np.float32)
        call("b3g_mlp_get_normalization", self.handle, fptr(n), C.c_int(N_NORM))
        return n

    @normalization.setter
    def normalization(self, n):
        n = np.ascontiguousarray(n, np.float32)
        call("b3g_mlp_set_normalization", self.handle, fptr(n), C.c_int(len(n)))

    def fit_normalization(self, x, t):
        """Feature and target mean / inverse std of a training set (std floored at 1e-6)."""
        x = np.asarray(x, np.float64)
        t = np.asarray(t, np.float64)
        n = np.concatenate([x.mean(0), 1.0 / np.maximum(x.std(0), 1e-6), t.mean(0), 1.0 / np.maximum(t.std(0), 1e-6)])
        self.normalization = n.astype(np.float32)

    # ---- inference / training
    def predict(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32).reshape(-1, N_FEATURES)
        y = np.zeros((len(x), N_OUTPUTS), np.float32)
        call("b3g_mlp_predict", self.handle, fptr(x), C.c_int(len(x)), fptr(y))
        return y

    def set_training_data(self, x, t):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, N_FEATURES)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, N_OUTPUTS)
        call("b3g_mlp_set_training_data", self.handle, fptr(x), fptr(t), C.c_int(len(x)))

    def train(self, steps: int, batch: int, lr: float, first_batch: int = 0) -> float:
        loss = C.c_double()
        call("b3g_mlp_train", self.handle, C.c_int(steps), C.c_int(batch), C.c_float(lr), C.c_int(first_batch),
             C.byref(loss))
        return loss.value

    def gradients(self, x, t):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, N_FEATURES)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, N_OUTPUTS)
        g = np.zeros(N_PARAMS, np.float32)
        loss = C.c_double()
        call("b3g_mlp_gradients", self.handle, fptr(x), fptr(t), C.c_int(len(x)), fptr(g), C.byref(loss))
        return g, loss.value

    # ---- files
    def save(self, path=DEFAULT_WEIGHTS, **meta):
        Path(path).parent.mkdir(parents=True, exist_ok=True)
        np.savez_compressed(path, params=self.params, normalization=self.normalization,
                            **{k: np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS, device: int = 0) -> "WarmStartMLP":
        d = np.load(path)
        m = cls(device)
        m.params = d["params"]
        m.normalization = d["normalization"]
        return m


def _time_kernels(argv=None) -> int:
    """Times the network's device work on random features, for profiling runs:

        python -m bullet3_gb300.warmstart [--rows N] [--batch B] [--train-steps S] [--repeat R]

    `predict` over N rows (the fused forward kernel; the call also copies the features in and the
    predictions out) and S training steps of batch B (forward and backward GEMMs, Adam); prints the
    wall times per call."""
    import argparse
    import json
    import time
    p = argparse.ArgumentParser()
    p.add_argument("--rows", type=int, default=1 << 20)
    p.add_argument("--batch", type=int, default=65536)
    p.add_argument("--train-steps", type=int, default=1)
    p.add_argument("--repeat", type=int, default=3)
    a = p.parse_args(argv)
    rng = np.random.Generator(np.random.PCG64(0))
    m = WarmStartMLP.load()
    x = rng.standard_normal((a.rows, N_FEATURES)).astype(np.float32)
    t = rng.standard_normal((a.rows, N_OUTPUTS)).astype(np.float32)
    m.predict(x[:1024])
    t0 = time.perf_counter()
    for _ in range(a.repeat):
        m.predict(x)
    predict_s = (time.perf_counter() - t0) / a.repeat
    m.set_training_data(x, t)
    m.train(1, a.batch, 1e-4)
    t0 = time.perf_counter()
    loss = m.train(a.train_steps, a.batch, 1e-4)
    train_s = (time.perf_counter() - t0) / max(a.train_steps, 1)
    print(json.dumps({"rows": a.rows, "predict_ms": 1000 * predict_s, "batch": a.batch,
                      "train_step_ms": 1000 * train_s, "loss": loss}))
    return 0


if __name__ == "__main__":
    raise SystemExit(_time_kernels())
