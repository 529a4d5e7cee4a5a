"""Host runtime over the C ABI: context, device pattern, SpMV.

torch is used only for device memory and streams.  Every compute call goes
through libsimit_gb300.so.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import F32, F64, P, call

_TORCH_DT = {F32: torch.float32, F64: torch.float64}


def dtype_code(t):
    if t.dtype == torch.float64:
        return F64
    if t.dtype == torch.float32:
        return F32
    raise TypeError("unsupported dtype %s" % t.dtype)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class Context:
    """One sg_ctx: a device and its stream.  `torch_stream` lets torch ops be
    ordered on the same stream (use `with ctx.stream():`)."""

    def __init__(self, device=0):
        _lib.load()
        torch.cuda.init()
        h = P()
        call("sg_ctx_create", device, ctypes.byref(h))
        self.h = h
        self.device = torch.device("cuda", device)
        self.torch_stream = torch.cuda.ExternalStream(_lib.load().sg_ctx_stream(h),
                                                      device=self.device)

    def stream(self):
        return torch.cuda.stream(self.torch_stream)

    def sync(self):
        call("sg_ctx_sync", self.h)

    def close(self):
        if self.h:
            _lib.load().sg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pattern:
    """Blocked-CSR pattern of `map f to E` plus incidence and slot map, built
    on the device (sg_incidence_build / sg_pattern_count / sg_pattern_fill /
    sg_slots_build)."""

    def __init__(self, ctx, n, endpoints, card, with_slots=True):
        dev = ctx.device
        ep = torch.as_tensor(np.ascontiguousarray(endpoints, np.int32)) \
            if not isinstance(endpoints, torch.Tensor) else endpoints
        ep = ep.to(device=dev, dtype=torch.int32).contiguous()
        nE = ep.numel() // card
        self.n, self.card, self.nE, self.endpoints = n, card, nE, ep
        with ctx.stream():
            self.ve_ptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
            self.ve_idx = torch.empty(max(1, nE * card), dtype=torch.int32, device=dev)
            self.rowptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
        call("sg_incidence_build", ctx.h, n, ptr(ep), nE, card, ptr(self.ve_ptr),
             ptr(self.ve_idx))
        nnzb = ctypes.c_int64()
        call("sg_pattern_count", ctx.h, n, ptr(ep), nE, card, ptr(self.ve_ptr),
             ptr(self.ve_idx), ptr(self.rowptr), ctypes.byref(nnzb))
        self.nnzb = nnzb.value
        with ctx.stream():
            self.colidx = torch.empty(max(1, self.nnzb), dtype=torch.int32, device=dev)
        call("sg_pattern_fill", ctx.h, n, ptr(ep), nE, card, ptr(self.ve_ptr),
             ptr(self.ve_idx), ptr(self.rowptr), ptr(self.colidx))
        self.slots = None
        if with_slots:
            with ctx.stream():
                self.slots = torch.empty(max(1, nE * card * card), dtype=torch.int32, device=dev)
            call("sg_slots_build", ctx.h, n, ptr(ep), nE, card, ptr(self.rowptr),
                 ptr(self.colidx), ptr(self.slots))

    def host(self):
        """(rowptr, colidx) as uint32 numpy arrays."""
        rp = self.rowptr.cpu().numpy().view(np.uint32)
        ci = self.colidx[:self.nnzb].cpu().numpy().view(np.uint32)
        return rp, ci


def bspmv(ctx, n, bs, rowptr, colidx, vals, x, y=None, g=0):
    if y is None:
        with ctx.stream():
            y = torch.empty_like(x)
    call("sg_bspmv", ctx.h, n, bs, ptr(rowptr), ptr(colidx), dtype_code(vals), ptr(vals),
         dtype_code(x), ptr(x), ptr(y), g)
    return y


def dot(ctx, a, b):
    out = ctypes.c_double()
    call("sg_dot", ctx.h, a.numel(), dtype_code(a), ptr(a), ptr(b), ctypes.byref(out))
    return out.value
