"""Thin Python handle over the C ABI, with device memory held in torch tensors.

torch is only the allocator and stream provider here; every transform and
field operation runs in libcsimgpu.so. Fields are planar fp32 tensors of
shape [F, 2, rows, cols] (real plane, imaginary plane).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import CSG_PREC_BF16X6, CSG_PREC_HIGH, CsgError, call  # noqa: F401


def ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("device tensor expected")
    if not t.is_contiguous():
        raise ValueError("contiguous tensor expected")
    return t.data_ptr()


def to_planar(e: np.ndarray, device="cuda") -> torch.Tensor:
    """complex numpy [..., R, C] -> planar fp32 tensor [F, 2, R, C] (host-side
    staging used by tests and examples; the ABI's upload call is the
    reference-facing path)."""
    e = np.asarray(e)
    e = e.reshape((-1,) + e.shape[-2:])
    out = np.ascontiguousarray(np.stack([e.real, e.imag], axis=1), dtype=np.float32)
    return torch.from_numpy(out).to(device)


def from_planar(t: torch.Tensor) -> np.ndarray:
    a = t.detach().cpu().numpy().astype(np.float64)
    return a[:, 0] + 1j * a[:, 1]


def dvec(x, dtype=torch.float64, device="cuda") -> torch.Tensor:
    return torch.as_tensor(np.asarray(x), dtype=dtype).to(device).contiguous()


class Context:
    """One csg_ctx bound to torch's current stream on `device`."""

    def __init__(self, device: int = 0):
        self.device = device
        torch.cuda.set_device(device)
        h = C.c_void_p()
        call("csg_create", C.byref(h), device)
        self.h = h
        self.bind_stream(torch.cuda.current_stream(device))

    def bind_stream(self, stream: torch.cuda.Stream):
        call("csg_set_stream", self.h, C.c_void_p(stream.cuda_stream))

    def sync(self):
        call("csg_sync", self.h)

    def close(self):
        if self.h:
            call("csg_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ elements
    def point_source(self, field, dx, dy, amp, tip, tilt):
        F, _, R, Cc = field.shape
        call("csg_point_source", self.h, ptr(field), F, R, Cc, dx, dy, ptr(amp), ptr(tip),
             ptr(tilt))

    def mask_real(self, field, mask, ref_quirk=True):
        F, _, R, Cc = field.shape
        call("csg_mask_real", self.h, ptr(field), F, R, Cc, ptr(mask), int(ref_quirk))

    def phase_screen(self, field, sag, lam, sign=1.0):
        F, _, R, Cc = field.shape
        call("csg_phase_screen", self.h, ptr(field), F, R, Cc, ptr(sag), ptr(lam), float(sign))

    def complex_mask(self, field, amp, ph):
        F, _, R, Cc = field.shape
        call("csg_complex_mask", self.h, ptr(field), F, R, Cc, ptr(amp), ptr(ph), amp.shape[0],
             amp.shape[1])

    def fft2d(self, field, direction=-1, precision=None):
        F, _, R, Cc = field.shape
        if R != Cc:
            raise ValueError("square fields only")
        if precision is None:
            call("csg_fft2d", self.h, ptr(field), F, R, direction)
        else:
            call("csg_fft2d_prec", self.h, ptr(field), F, R, direction, int(precision))

    def fresnel(self, field, lam, ap_rad, z, precision=None):
        F, _, R, Cc = field.shape
        if precision is None:
            call("csg_fresnel", self.h, ptr(field), F, R, ptr(lam), float(ap_rad), float(z))
        else:
            call("csg_fresnel_prec", self.h, ptr(field), F, R, ptr(lam), float(ap_rad), float(z),
                 int(precision))

    def hex_mask(self, hex_id, count, n_sub, sags, cand, lam, phase_sign=1.0, flip=True,
                 subtract=1.0, use_only_hex=-1, out=None):
        S = hex_id.shape[-1]
        n_cand, n_hex = sags.shape
        n_out = cand.shape[0]
        if out is None:
            out = torch.empty((n_out, 2, S, S), dtype=torch.float32, device=sags.device)
        call("csg_hex_mask", self.h, ptr(hex_id), ptr(count), S, n_sub, ptr(sags), n_hex, n_out,
             ptr(cand), ptr(lam), float(phase_sign), int(flip), float(subtract),
             int(use_only_hex), ptr(out))
        return out

    def region_reduce(self, field, per_group, pix_idx, mode=0, scale=1.0, out=None):
        F, _, R, Cc = field.shape
        groups = F // per_group
        if out is None:
            out = torch.empty(groups, dtype=torch.float64, device=field.device)
        call("csg_region_reduce", self.h, ptr(field), R, Cc, groups, per_group, ptr(pix_idx),
             pix_idx.numel(), mode, float(scale), ptr(out))
        return out

    def intensity(self, field):
        F, _, R, Cc = field.shape
        out = torch.empty((R, Cc), dtype=torch.float64, device=field.device)
        mx = torch.empty(1, dtype=torch.float64, device=field.device)
        call("csg_intensity", self.h, ptr(field), R, Cc, F, ptr(out), ptr(mx))
        return out, mx


class Mft:
    """Plan of csg_mft_create: out = pref * A_y . in . B_x^T (see csimgpu.h)."""

    def __init__(self, ctx: Context, yin, xin, yout, xout, lf, pref=None, sgn=-1.0,
                 precision=CSG_PREC_BF16X6):
        self.ctx = ctx
        yin, xin, yout, xout = (np.ascontiguousarray(v, dtype=np.float64) for v in (yin, xin, yout, xout))
        lf = np.ascontiguousarray(np.atleast_1d(lf), dtype=np.float64)
        self.shape_in = (yin.size, xin.size)
        self.shape_out = (yout.size, xout.size)
        pr = None
        if pref is not None:
            pc = np.atleast_1d(np.asarray(pref, dtype=np.complex128))
            pr = np.ascontiguousarray(np.stack([pc.real, pc.imag], -1).ravel())
        h = C.c_void_p()
        dp = lambda a: a.ctypes.data_as(C.c_void_p) if a is not None else None  # noqa: E731
        call("csg_mft_create", ctx.h, C.byref(h), yin.size, xin.size, yout.size, xout.size,
             dp(yin), dp(xin), dp(yout), dp(xout), lf.size, dp(lf), dp(pr), float(sgn),
             int(precision))
        self.h = h

    def set_tile(self, bn: int):
        """Fix the tensor-core tile width (64, 128 or 256; 0: default / autotuned)."""
        call("csg_mft_set_tile", self.h, int(bn))

    def __call__(self, field_in, slot, out=None, accumulate=False, in_mul=None, mul_idx=None):
        F = field_in.shape[0]
        if out is None:
            out = torch.empty((F, 2) + self.shape_out, dtype=torch.float32, device=field_in.device)
        call("csg_mft_execute", self.ctx.h, self.h, ptr(field_in), ptr(out), F, ptr(slot),
             int(accumulate), ptr(in_mul), ptr(mul_idx))
        return out

    def execute_lo(self, field_in, slot):
        """CSG_PREC_HIGH plans: (out, out_lo), the two-float transform."""
        F = field_in.shape[0]
        out = torch.empty((F, 2) + self.shape_out, dtype=torch.float32, device=field_in.device)
        lo = torch.empty_like(out)
        call("csg_mft_execute_lo", self.ctx.h, self.h, ptr(field_in), ptr(out), ptr(lo), F,
             ptr(slot))
        return out, lo

    def close(self):
        if self.h:
            call("csg_mft_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
