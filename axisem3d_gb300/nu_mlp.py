"""The Nu network through the C-ABI (ax3d_mlp_* in include/ax3d.h).

Host-side plumbing only: device buffers are torch CUDA tensors whose pointers go to the
library's kernels; every forward, gradient and Adam step runs in libax3d.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .capi import AX3D_OK, Ax3dError, load_library

NIN, NHID, NPARAM = 16, 128, 35329
# offsets of the parameter vector: W1 [128][16], b1, W2 [128][128], b2, W3, b3, w4, b4
OFFSETS = {}
_o = 0
for _name, _size in (("W1", NHID * NIN), ("b1", NHID), ("W2", NHID * NHID), ("b2", NHID),
                     ("W3", NHID * NHID), ("b3", NHID), ("w4", NHID), ("b4", 1)):
    OFFSETS[_name] = (_o, _size)
    _o += _size
assert _o == NPARAM


def init_params(seed: int = 0) -> np.ndarray:
    """U(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights and biases, seeded."""
    rng = np.random.default_rng(seed)
    out = np.zeros(NPARAM, np.float32)
    fan = {"W1": NIN, "b1": NIN, "W2": NHID, "b2": NHID, "W3": NHID, "b3": NHID, "w4": NHID, "b4": NHID}
    for name, (o, n) in OFFSETS.items():
        a = 1.0 / np.sqrt(fan[name])
        out[o:o + n] = rng.uniform(-a, a, n)
    return out


def _bind(lib):
    if getattr(lib, "_mlp_bound", False):
        return
    vp, i32, i64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_float
    lib.ax3d_mlp_create.argtypes = [i32, i32, C.POINTER(vp)]
    lib.ax3d_mlp_set_params.argtypes = [vp, C.POINTER(C.c_float), i64]
    lib.ax3d_mlp_get_params.argtypes = [vp, C.POINTER(C.c_float), i64]
    lib.ax3d_mlp_forward.argtypes = [vp, vp, i32, vp, vp]
    lib.ax3d_mlp_gradient.argtypes = [vp, vp, vp, i32, vp, vp, vp]
    lib.ax3d_mlp_train_step.argtypes = [vp, vp, vp, i32, f32, vp, vp]
    lib.ax3d_mlp_destroy.argtypes = [vp]
    lib._mlp_bound = True


class NuMLP:
    """One network on one device.  x: float32 CUDA tensor [n, 16]; targets [n]."""

    def __init__(self, max_batch: int, device: int = 0, params: np.ndarray | None = None, seed: int = 0):
        import torch
        self.torch = torch
        self.lib = load_library()
        _bind(self.lib)
        self.device = device
        self.max_batch = int(max_batch)
        h = C.c_void_p()
        self._ck(self.lib.ax3d_mlp_create(self.max_batch, device, C.byref(h)))
        self.h = h
        self.set_params(init_params(seed) if params is None else params)
        self._loss = torch.zeros(1, dtype=torch.float32, device=f"cuda:{device}")

    def _ck(self, rc):
        if rc != AX3D_OK:
            buf = C.create_string_buffer(1024)
            self.lib.ax3d_last_error(buf, 1024)
            raise Ax3dError(rc, buf.value.decode(errors="replace"))

    def _stream(self):
        return C.c_void_p(self.torch.cuda.current_stream(self.device).cuda_stream)

    def _dev(self, a):
        t = self.torch
        if not isinstance(a, t.Tensor):
            a = t.as_tensor(np.asarray(a, np.float32))
        return a.to(device=f"cuda:{self.device}", dtype=t.float32).contiguous()

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        self._ck(self.lib.ax3d_mlp_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)), NPARAM))

    def get_params(self) -> np.ndarray:
        out = np.zeros(NPARAM, np.float32)
        self._ck(self.lib.ax3d_mlp_get_params(self.h, out.ctypes.data_as(C.POINTER(C.c_float)), NPARAM))
        return out

    def forward(self, x):
        x = self._dev(x)
        y = self.torch.empty(x.shape[0], dtype=self.torch.float32, device=x.device)
        self._ck(self.lib.ax3d_mlp_forward(self.h, C.c_void_p(x.data_ptr()), x.shape[0],
                                           C.c_void_p(y.data_ptr()), self._stream()))
        return y

    def gradient(self, x, t):
        x, t = self._dev(x), self._dev(t)
        g = self.torch.empty(NPARAM, dtype=self.torch.float32, device=x.device)
        self._ck(self.lib.ax3d_mlp_gradient(self.h, C.c_void_p(x.data_ptr()), C.c_void_p(t.data_ptr()),
                                            x.shape[0], C.c_void_p(g.data_ptr()),
                                            C.c_void_p(self._loss.data_ptr()), self._stream()))
        return g, self._loss.clone()

    def train_step(self, x, t, lr: float, loss_out=None):
        """One Adam step; loss_out (a CUDA float32 tensor [1]) receives the batch loss."""
        lp = C.c_void_p(loss_out.data_ptr()) if loss_out is not None else None
        self._ck(self.lib.ax3d_mlp_train_step(self.h, C.c_void_p(x.data_ptr()), C.c_void_p(t.data_ptr()),
                                              x.shape[0], C.c_float(lr), lp, self._stream()))

    def fit(self, x, t, epochs: int, batch: int, lr: float, seed: int = 0, lr_final: float | None = None):
        """Mini-batch Adam over (x, t) for `epochs` passes, reshuffled per epoch on the device
        (seeded); cosine decay from lr to lr_final.  Returns the mean loss per epoch."""
        torch = self.torch
        x, t = self._dev(x), self._dev(t)
        n = x.shape[0]
        batch = min(batch, self.max_batch, n)
        gen = torch.Generator(device=x.device)
        gen.manual_seed(seed)
        nb = n // batch
        losses = torch.zeros(epochs * nb, dtype=torch.float32, device=x.device)
        lr_final = lr if lr_final is None else lr_final
        k = 0
        for ep in range(epochs):
            perm = torch.randperm(n, generator=gen, device=x.device)
            xs, ts = x[perm].contiguous(), t[perm].contiguous()
            for i in range(nb):
                f = k / max(1, epochs * nb - 1)
                lr_k = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * f))
                self.train_step(xs[i * batch:(i + 1) * batch], ts[i * batch:(i + 1) * batch], lr_k,
                                losses[k:k + 1])
                k += 1
        return losses.view(epochs, nb).mean(1).cpu().numpy()

    def close(self):
        if getattr(self, "h", None):
            self.lib.ax3d_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
