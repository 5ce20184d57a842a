"""CPU restatement of the reference's tools around the propagation (test
infrastructure only: nothing in the shipped library imports it).

contrast_curve follows contrastCurve.cpp:122-151; fd_jacobian follows
linearOptimizer.cpp:420-495 on fields from the FP64 chain.
"""
from __future__ import annotations

import numpy as np


def linspace(start: float, end: float, n: int) -> np.ndarray:
    """arma::linspace (start + i delta, the last value exactly end)."""
    d = (end - start) / (n - 1)
    out = start + np.arange(n) * d
    out[-1] = end
    return out


def contrast_curve(full_norm: np.ndarray, pixel_x_lod: np.ndarray, pixel_y_lod: np.ndarray,
                   pixel_sampling: int = 1):
    """(ccPos, ccAvg) of contrastCurve.cpp:127-140: sample points
    linspace(0, max(pixelX / loD), (nX - 2) / pixelSampling); bin i averages
    the normalised intensity where s[i-1] < RR < s[i+1]."""
    nx = pixel_x_lod.size
    s = linspace(0.0, float(np.max(pixel_x_lod)), int((nx - 2) / pixel_sampling))
    xx = np.broadcast_to(pixel_x_lod[None, :], full_norm.shape)
    yy = np.broadcast_to(pixel_y_lod[:, None], full_norm.shape)
    rr = np.sqrt(xx ** 2 + yy ** 2)
    avg = np.zeros(s.size - 2)
    pos = np.zeros(s.size - 2)
    for i in range(1, s.size - 1):
        sel = (rr > s[i - 1]) & (rr < s[i + 1])
        avg[i - 1] = full_norm[sel].mean() if sel.any() else np.nan
        pos[i - 1] = s[i]
    return pos, avg


def fd_jacobian(field_fn, x0: np.ndarray, dx: float, var_idx, pix_idx: np.ndarray,
                n_base: int) -> np.ndarray:
    """Columns var_idx of the finite-difference Jacobian: field_fn(x, b) is
    base field b's image for optimisation vector x; rows [Re; Im] over the
    region pixels per base field."""
    base = [field_fn(x0, b).ravel()[pix_idx] for b in range(n_base)]
    cols = []
    for i in var_idx:
        x = np.array(x0, dtype=np.float64)
        x[i] += dx
        col = []
        for b in range(n_base):
            d = (field_fn(x, b).ravel()[pix_idx] - base[b]) / dx
            col += [d.real, d.imag]
        cols.append(np.concatenate(col))
    return np.stack(cols, axis=1)
