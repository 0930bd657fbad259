"""Helpers for the GPU parity tests: device context and raw C-ABI calls."""
import ctypes

import numpy as np
import torch

from mfem_gb300 import _lib
from mfem_gb300.pa import Device

_dev = None


def dev():
    global _dev
    if _dev is None:
        _dev = Device("cuda")
    return _dev


def T(a, dtype=None):
    a = np.ascontiguousarray(a)
    t = torch.from_numpy(a)
    if dtype is not None:
        t = t.to(dtype)
    return t.to(dev().torch_device).contiguous()


def H(t):
    return t.detach().cpu().numpy()


_keep = []


def p(t):
    """Device pointer of t; t is kept alive until the next call() returns, so
    a temporary's memory cannot be handed to another argument of the same
    call by the caching allocator."""
    if t is None:
        return None
    _keep.append(t)
    return ctypes.c_void_p(t.data_ptr())


def call(name, *args):
    d = dev()
    st = getattr(d.lib, name)(d.ctx, *args)
    _keep.clear()
    _lib.check(st, name)
    return st


def zeros(n, dtype=torch.float64):
    return torch.zeros(n, dtype=dtype, device=dev().torch_device)


def relerr(a, b):
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)
