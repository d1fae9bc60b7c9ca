"""The learned tuner's cost model: an MLP run and trained by the library's
CUDA kernels (dedispersion_gb300/csrc/dd_mlp.cu) through the C ABI.

The network maps features of (shape, input bits, subbands, tile
configuration) to log(run time); the tuner (``dedispersion_gb300.tuning``)
times only the configurations it ranks best.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._abi import check, lib

_F32P = C.POINTER(C.c_float)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class MLP:
    """in -> hidden x layers -> 1, ReLU, bf16 weights, fp32 accumulation."""

    def __init__(self, in_features: int, hidden: int = 128, layers: int = 3, seed: int = 0,
                 device: int = 0):
        self.in_features, self.hidden, self.layers = in_features, hidden, layers
        self._h = C.c_void_p()
        check(lib().dd_mlp_create(C.byref(self._h), in_features, hidden, layers, seed, device))
        n = C.c_uint64(0)
        check(lib().dd_mlp_param_count(self._h, C.byref(n)))
        self.nparams = n.value

    def dims(self) -> list[tuple[int, int]]:
        """(in, out) of every layer, in order."""
        d, prev = [], self.in_features
        for _ in range(self.layers):
            d.append((prev, self.hidden))
            prev = self.hidden
        d.append((prev, 1))
        return d

    def params(self) -> np.ndarray:
        p = np.zeros(self.nparams, np.float32)
        check(lib().dd_mlp_get_params(self._h, p.ctypes.data_as(_F32P), self.nparams))
        return p

    def set_params(self, p) -> None:
        p = _f32(p)
        check(lib().dd_mlp_set_params(self._h, p.ctypes.data_as(_F32P), p.size))

    def forward(self, x) -> np.ndarray:
        x = _f32(x)
        y = np.zeros(x.shape[0], np.float32)
        check(lib().dd_mlp_forward(self._h, x.ctypes.data_as(_F32P), x.shape[0],
                                   y.ctypes.data_as(_F32P)))
        return y

    def gradients(self, x, t):
        x, t = _f32(x), _f32(t)
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_float(0)
        check(lib().dd_mlp_gradients(self._h, x.ctypes.data_as(_F32P), t.ctypes.data_as(_F32P),
                                     x.shape[0], g.ctypes.data_as(_F32P), C.byref(loss)))
        return g, loss.value

    def train(self, x, t, steps: int, lr: float) -> float:
        x, t = _f32(x), _f32(t)
        loss = C.c_float(0)
        check(lib().dd_mlp_train(self._h, x.ctypes.data_as(_F32P), t.ctypes.data_as(_F32P),
                                 x.shape[0], steps, lr, C.byref(loss)))
        return loss.value

    def close(self) -> None:
        if self._h:
            lib().dd_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
