"""Host-side handle of the GPU network (gb_mlp in include/gb_newton.h)."""
import ctypes

import numpy as np

from . import _lib


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class GpuMLP:
    """n_in -> width x hidden_layers (tanh) -> n_out, FP32 on the GPU."""

    def __init__(self, n_in, width, hidden_layers, n_out, seed=0):
        self._L = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self._L.gb_mlp_create(n_in, width, hidden_layers, n_out, seed,
                                         ctypes.byref(h)))
        self.h = h
        self.widths = [n_in] + [width] * hidden_layers + [n_out]
        self.nparam = self._L.gb_mlp_num_params(self.h)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self._L.gb_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        p = np.empty(self.nparam, np.float32)
        _lib.check(self._L.gb_mlp_get_params(self.h, _fp(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        _lib.check(self._L.gb_mlp_set_params(self.h, _fp(p)))

    def grads(self):
        g = np.empty(self.nparam, np.float32)
        _lib.check(self._L.gb_mlp_get_grads(self.h, _fp(g)))
        return g

    # device tensors (torch) in, device tensors out.  The library's network
    # entry points run on the network's own stream, which does not wait for
    # torch's: the current stream is synchronised first so that the inputs
    # are complete on the device.
    @staticmethod
    def _inputs_ready(t):
        import torch
        torch.cuda.current_stream(t.device).synchronize()

    def forward(self, x):
        import torch
        x = x.contiguous().float()
        y = torch.empty((x.shape[0], self.widths[-1]), dtype=torch.float32, device=x.device)
        self._inputs_ready(x)
        _lib.check(self._L.gb_mlp_forward_device(self.h, x.data_ptr(), x.shape[0], y.data_ptr()))
        return y

    def forward_noalloc(self, x, y, stream=None):
        """Forward pass into the caller's y without any device allocation
        (gb_mlp_forward_noalloc): x [B, n_in] and y [B, n_out] are FP32 device
        tensors the caller owns; B x hidden width <= MLP_NOALLOC_MAX_ACT.  The
        pass is queued on `stream` (a torch.cuda.Stream; default: torch's
        current stream) in order with the work already queued there."""
        import torch
        s = stream if stream is not None else torch.cuda.current_stream(x.device)
        _lib.check(self._L.gb_mlp_forward_noalloc(self.h, x.data_ptr(), x.shape[0], y.data_ptr(),
                                                  ctypes.c_void_p(s.cuda_stream)))
        return y

    def loss_grad(self, x, t, mask):
        self._inputs_ready(x)
        loss = ctypes.c_float()
        _lib.check(self._L.gb_mlp_loss_grad_device(self.h, x.data_ptr(), t.data_ptr(),
                                                   mask.data_ptr(), x.shape[0],
                                                   ctypes.byref(loss)))
        return loss.value

    def adam_step(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        _lib.check(self._L.gb_mlp_adam_step(self.h, lr, b1, b2, eps))

    def train(self, x, t, mask, steps, batch=4096, lr=1e-3, seed=0):
        self._inputs_ready(x)
        loss = ctypes.c_float()
        _lib.check(self._L.gb_mlp_train_device(self.h, x.data_ptr(), t.data_ptr(), mask.data_ptr(),
                                               x.shape[0], steps, batch, lr, seed,
                                               ctypes.byref(loss)))
        return loss.value
