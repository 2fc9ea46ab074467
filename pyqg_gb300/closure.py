"""Learned subgrid closure: a convolutional net on the tcgen05 tensor cores.

No counterpart in the reference.  :class:`ConvNet` wraps the ``pqg_cnn_*``
C ABI (5x5 periodic convolutions, ReLU between layers, BF16 weights and
activations, FP32 accumulation, Adam); :class:`CNNParameterization` plugs a
trained net into any model through the ``q_parameterization`` hook
(``pyqg/model.py:203-212``), returning its PV forcing as a device array so the
step never leaves the GPU.

The default architecture is 2 -> 128 -> 64 -> 32 -> 32 -> 32 -> 32 -> 32 -> 2
channels (8 layers, 366,400 multiply-adds per pixel).
"""
import ctypes

import numpy as np

from . import _lib
from .parameterizations import QParameterization

DEFAULT_CHANNELS = (2, 128, 64, 32, 32, 32, 32, 32, 2)


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("pyqg_gb300 needs a CUDA device; none is visible")
    return torch


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class ConvNet:
    """Fully convolutional net with 5x5 periodic kernels.

    ``channels`` lists the channel counts from input to output; images are
    ``(batch, channels, ny, 64)``.  Weights and biases are initialised
    uniform in +-1/sqrt(fan_in) from ``seed`` (the usual default for
    convolutions, which Adam at lr 1e-3 expects).
    """

    def __init__(self, channels=DEFAULT_CHANNELS, ny=64, nx=64, max_batch=64, seed=0):
        torch = _torch()
        self._L = _lib.lib()
        self.channels = tuple(int(c) for c in channels)
        self.ny, self.nx, self.max_batch = int(ny), int(nx), int(max_batch)
        ch = (ctypes.c_int * len(self.channels))(*self.channels)
        h = ctypes.c_void_p()
        self._check(self._L.pqg_cnn_create(ctypes.byref(h), len(self.channels) - 1, ch,
                                           self.ny, self.nx, self.max_batch))
        self._h = h
        n = ctypes.c_longlong()
        self._check(self._L.pqg_cnn_nparams(h, ctypes.byref(n)))
        self.nparams = n.value
        self._stream = torch.cuda.current_stream()
        self.params = self.initial_params(seed)

    # -- layout of the parameter vector ------------------------------------
    def layer_slices(self):
        """[(weight slice, weight shape (co, 5, 5, ci), bias slice)] per layer."""
        out, off = [], 0
        for ci, co in zip(self.channels[:-1], self.channels[1:]):
            nw = co * 25 * ci
            out.append((slice(off, off + nw), (co, 5, 5, ci), slice(off + nw, off + nw + co)))
            off += nw + co
        return out

    def initial_params(self, seed=0):
        rng = np.random.default_rng(seed)
        p = np.zeros(self.nparams, dtype=np.float32)
        for ws, shape, bs in self.layer_slices():
            fan_in = shape[1] * shape[2] * shape[3]
            bound = 1.0 / np.sqrt(fan_in)
            p[ws] = rng.uniform(-bound, bound, size=ws.stop - ws.start).astype(np.float32)
            p[bs] = rng.uniform(-bound, bound, size=bs.stop - bs.start).astype(np.float32)
        return p

    def _check(self, rc):
        if rc != _lib.PQG_OK:
            msg = self._L.pqg_cnn_last_error().decode(errors="replace")
            if rc == _lib.PQG_ERR_INVALID:
                raise ValueError(msg)
            if rc == _lib.PQG_ERR_UNSUPPORTED:
                raise NotImplementedError(msg)
            raise _lib.PQGError(rc, msg)

    def _sp(self):
        return ctypes.c_void_p(self._stream.cuda_stream)

    @property
    def params(self):
        out = np.empty(self.nparams, dtype=np.float32)
        self._check(self._L.pqg_cnn_get_params(self._h, out.ctypes.data, self._sp()))
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.shape != (self.nparams,):
            raise ValueError("expected %d parameters" % self.nparams)
        self._check(self._L.pqg_cnn_set_params(self._h, p.ctypes.data, self._sp()))

    @property
    def grads(self):
        out = np.empty(self.nparams, dtype=np.float32)
        self._check(self._L.pqg_cnn_get_grads(self._h, out.ctypes.data, self._sp()))
        return out

    def set_norm(self, in_mean, in_std, out_mean, out_std):
        """Per-channel standardisation applied by :meth:`forward`."""
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (in_mean, in_std, out_mean, out_std)]
        self._keep = arrs
        self._check(self._L.pqg_cnn_set_norm(self._h, *[a.ctypes.data for a in arrs]))

    def _batch(self, x):
        torch = _torch()
        if not (isinstance(x, torch.Tensor) and x.is_cuda and x.is_contiguous()):
            raise ValueError("expected a contiguous CUDA tensor")
        if x.dim() == 3:
            return 1
        return x.shape[0]

    def forward(self, x, out=None):
        """net(x) with the standardisation of :meth:`set_norm`; x is a CUDA
        tensor (batch, cin, ny, nx) or (cin, ny, nx), FP32 or FP64."""
        torch = _torch()
        b = self._batch(x)
        if out is None:
            shape = (self.channels[-1],) + tuple(x.shape[-2:])
            if x.dim() == 4:
                shape = (b,) + shape
            out = torch.empty(shape, dtype=x.dtype, device=x.device)
        self._check(self._L.pqg_cnn_forward(self._h, _ptr(x), int(x.dtype == torch.float64), _ptr(out),
                                            int(out.dtype == torch.float64), b, self._sp()))
        return out

    def backward(self, x, t):
        """Gradient of the MSE of net(x) against t (standardised FP32 CUDA
        tensors); returns the loss."""
        b = self._batch(x)
        loss = ctypes.c_float()
        self._check(self._L.pqg_cnn_backward(self._h, _ptr(x), _ptr(t), b, ctypes.byref(loss), self._sp()))
        return loss.value

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self._check(self._L.pqg_cnn_adam(self._h, lr, beta1, beta2, eps, self._sp()))

    def train_step(self, x, t, lr=1e-3):
        b = self._batch(x)
        loss = ctypes.c_float()
        self._check(self._L.pqg_cnn_train_step(self._h, _ptr(x), _ptr(t), b, lr, ctypes.byref(loss),
                                               self._sp()))
        return loss.value

    def save(self, path, **extra):
        np.savez(path, channels=np.array(self.channels), params=self.params, **extra)

    def __del__(self):
        h = self.__dict__.get("_h")
        if h is not None and h.value:
            try:
                _torch().cuda.synchronize()
                self._L.pqg_cnn_destroy(h)
            except Exception:
                pass
            self._h = None


class CNNParameterization(QParameterization):
    """PV forcing predicted by a :class:`ConvNet` from the model's q.

    The net maps standardised q to the standardised subgrid forcing
    S = filtered(J(psi, q)) - J(filtered psi, filtered q); the tendency added
    to dq/dt is -S.  ``stats`` = (q_mean, q_std, S_mean, S_std) per layer.
    """

    def __init__(self, net, stats):
        self.net = net
        q_mean, q_std, s_mean, s_std = [np.asarray(a, dtype=np.float64) for a in stats]
        self.stats = (q_mean, q_std, s_mean, s_std)
        net.set_norm(q_mean, q_std, -s_mean, -s_std)

    def __call__(self, m):
        return self.net.forward(m.device_field("q"))

    def __repr__(self):
        return "CNNParameterization(channels=%s)" % (self.net.channels,)
