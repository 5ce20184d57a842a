"""Seeded synthetic inputs with the shapes of the benchmark configurations.

The reference's own example data (pupils, PIAA sags, hex tables, response
matrices) are not available, so every workload here is generated from a
seed: apertures, Zernike aberrations, PIAA even-polynomial sags, standard hex
layouts and uniform hex sags. Hex interpolation tables are built on the GPU
by csg_hex_tables.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import coronagraph as cg
from .synth import (BroadbandSpec, PiaacmcSpec, PlainLyotSpec, broadband_arrays,  # noqa: F401
                    circle_mask, hex_layout_standard, piaa_sag, piaacmc_arrays,
                    plain_lyot_arrays, segmented_hex_aperture)
from ._lib import call
from .runtime import Context, dvec, ptr


def hex_tables(ctx: Context, hex_x, hex_y, n_rings, design_size, fpm_scale_factor, hex_gap,
               pitch, S, n_sub, pixel_scale, fpm_radius, reference_single_thread=False):
    """Interpolation tables [3][S][S] (int16 ids, uint16 counts) built on the
    GPU; returned as host numpy arrays. reference_single_thread: the
    reference's tables as its loop builds them on one OpenMP thread."""
    hx, hy = dvec(hex_x), dvec(hex_y)
    ids = torch.empty((3, S, S), dtype=torch.int16, device="cuda")
    cnt = torch.empty((3, S, S), dtype=torch.int16, device="cuda")
    over = C.c_int()
    call("csg_hex_tables", ctx.h, ptr(hx), ptr(hy), hx.numel(), n_rings, design_size,
         fpm_scale_factor, hex_gap, pitch, S, n_sub, pixel_scale, fpm_radius, ptr(ids), ptr(cnt),
         C.byref(over), int(bool(reference_single_thread)))
    return ids.cpu().numpy(), cnt.cpu().numpy().view(np.uint16), over.value


def build_piaacmc(ctx: Context, spec: PiaacmcSpec, sources=None, precision: int = 6,
                  support_crop: bool = True):
    """Returns (coronagraph, inputs dict with every array the oracle needs);
    the hex tables are built on the GPU."""
    a = piaacmc_arrays(spec, sources)
    ids, cnt, over = hex_tables(ctx, a["hex_x"], a["hex_y"], spec.n_rings, spec.design_size,
                                spec.fpm_scale_factor, spec.hex_gap, 1.0, spec.S, spec.n_sub,
                                a["dm"], a["fpm_radius"])
    a.update(hex_id=ids, count=cnt, overflow=over)
    elems = [
        cg.Mask(a["pupil"]),
        cg.Mirror(a["sag1"], 1.0),
        cg.FresnelPropagator(spec.z),
        cg.Mirror(a["sag2"], -1.0),
        cg.FpmPupToLyotHex(ids, cnt, spec.n_sub, len(a["hex_x"]), a["dm"], spec.fpm_focal_ratio),
        cg.Mask(a["lyot"]),
        cg.FraunhoferFocal(a["lam_ref"], spec.spl, spec.n_out_fov),
    ]
    cor = cg.Coronagraph(ctx, a["tel"], a["ef"], elems, precision, support_crop)
    return cor, a


def build_plain_lyot(ctx: Context, spec: PlainLyotSpec, sources=None, precision: int = 6,
                     fft_fpm_babinet: bool = True):
    """Plain Lyot coronagraph chain: pupil -> aberration -> padded-FFT
    occulter -> Lyot stop -> final MFT. Returns (coronagraph, inputs).
    fft_fpm_babinet = False keeps the occulter as a padded FFT."""
    a = plain_lyot_arrays(spec, sources)
    elems = [
        cg.Mask(a["pupil"]),
        cg.Mirror(a["sag"], 1.0),
        cg.PaddedFftFpm(spec.pad, a["occulter"]),
        cg.Mask(a["lyot"]),
        cg.FraunhoferFocal(a["lam_ref"], spec.spl, spec.n_out_fov),
    ]
    cor = cg.Coronagraph(ctx, a["tel"], a["ef"], elems, precision,
                         fft_fpm_babinet=fft_fpm_babinet)
    return cor, a


def build_broadband(ctx: Context, spec: BroadbandSpec, precision: int = 6):
    """Broadband chain: segmented aperture -> DM -> per-wavelength ragged
    final MFT; the batch is every (wavelength, source) pair (33 fields)."""
    a = broadband_arrays(spec)
    elems = [
        cg.Mask(a["pupil"]),
        cg.DeformableMirror(a["act"], spec.dm_sigma, 1.0),
        cg.FraunhoferFocalRagged(a["lam_ref"], spec.spl, a["n_out"]),
    ]
    cor = cg.Coronagraph(ctx, a["tel"], a["ef"], elems, precision)
    a["dm_surface"] = cor.dm_surface
    return cor, a


def random_sags(rng: np.random.Generator, n_cand: int, n_hex: int, half_range: float):
    return rng.uniform(-half_range, half_range, (n_cand, n_hex))
