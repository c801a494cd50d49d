"""The doma_unet C ABI as a Python object (device tensors are torch tensors)."""
from __future__ import annotations

import ctypes

import numpy as np

from .. import abi

IN_CHANNELS = 16


class UNet:
    """A U-Net resident on the current CUDA device."""

    def __init__(self, seed: int = 0):
        self.lib = abi.load_library()
        h = ctypes.c_void_p()
        abi.check(self.lib.doma_unet_create(seed, ctypes.byref(h)), "doma_unet_create", self.lib)
        self._h = h
        self.num_params = int(self.lib.doma_unet_num_params(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.doma_unet_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int | None) -> None:
        abi.check(self.lib.doma_unet_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)),
                  "doma_unet_set_stream", self.lib)

    def params(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        abi.check(self.lib.doma_unet_get_params(self._h, out.ctypes.data_as(abi._fp), out.size),
                  "doma_unet_get_params", self.lib)
        return out

    def set_params(self, flat: np.ndarray) -> None:
        flat = np.ascontiguousarray(flat, dtype=np.float32)
        abi.check(self.lib.doma_unet_set_params(self._h, flat.ctypes.data_as(abi._fp), flat.size),
                  "doma_unet_set_params", self.lib)

    def grads(self) -> np.ndarray:
        out = np.empty(self.num_params, dtype=np.float32)
        abi.check(self.lib.doma_unet_get_grads(self._h, out.ctypes.data_as(abi._fp), out.size),
                  "doma_unet_get_grads", self.lib)
        return out

    @staticmethod
    def _shape(x):
        b, z, y, w, c = x.shape
        if c != IN_CHANNELS:
            raise ValueError(f"input needs {IN_CHANNELS} channels")
        return b, z, y, w

    def forward(self, x, out) -> None:
        """x: [B,Z,Y,X,16] bfloat16 cuda tensor; out: [B,Z,Y,X] float32 cuda tensor."""
        b, z, y, w = self._shape(x)
        abi.check(self.lib.doma_unet_forward(self._h, ctypes.c_void_p(x.data_ptr()),
                                             ctypes.c_void_p(out.data_ptr()), b, z, y, w),
                  "doma_unet_forward", self.lib)

    def backward(self, x, target, weight=None) -> None:
        """Forward, mean-square loss and gradients; weight: optional [B] float32
        cuda tensor scaling each sample's squared error."""
        b, z, y, w = self._shape(x)
        if weight is None:
            abi.check(self.lib.doma_unet_backward(self._h, ctypes.c_void_p(x.data_ptr()),
                                                  ctypes.c_void_p(target.data_ptr()), b, z, y, w),
                      "doma_unet_backward", self.lib)
            return
        weight = weight.contiguous()
        abi.check(self.lib.doma_unet_backward_weighted(
            self._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(target.data_ptr()),
            ctypes.c_void_p(weight.data_ptr()), b, z, y, w), "doma_unet_backward_weighted", self.lib)

    def loss(self) -> float:
        v = ctypes.c_double()
        abi.check(self.lib.doma_unet_last_loss(self._h, ctypes.byref(v)), "doma_unet_last_loss",
                  self.lib)
        return v.value

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        abi.check(self.lib.doma_unet_adam(self._h, lr, beta1, beta2, eps), "doma_unet_adam", self.lib)

    # -- weights file: bf16 weights (exactly what inference uses), fp32 rest --
    def save(self, path) -> None:
        p = self.params()
        np.savez_compressed(path, bf16_bits=_to_bf16_bits(p), count=np.int64(p.size))

    def load(self, path) -> None:
        d = np.load(path)
        if int(d["count"]) != self.num_params:
            raise ValueError("weights file does not match this network")
        self.set_params(_from_bf16_bits(d["bf16_bits"]))


def _to_bf16_bits(p: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(p, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def _from_bf16_bits(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32)
