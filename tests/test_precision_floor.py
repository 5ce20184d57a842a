"""Where fp32 fields put the error floor of the 1024^2 PIAACMC chain (CPU).

The GPU path keeps fields and element tables in fp32 and is specified
against a peak-normalised field error of 1e-7 from the FP64 oracle. This
test measures, with the FP64 plain path (`baseline/fp64_gpu.py`) on the CPU:
  * the storage floor: FP64 arithmetic with every table and every stored
    intermediate field rounded to complex64 -- 0.7e-7 of the calibration
    peak, so no fp32-field implementation can do much better;
  * the same with the Fresnel FFTs in single precision (pocketfft) and FP64
    matrix transforms -- 1.1e-7: single-precision FFTs alone already pass
    the 1e-7 mark;
  * the plain complex64 evaluation (complex64 FFTs and matmuls) -- above
    1e-6, the level a straightforward single-precision port lands at.
The GPU path measures 3.7e-7 (calibration) and 5.0e-7 (final field) on the
same configuration (tests/test_gpu_chain.py, full size).
"""
import numpy as np
import torch

from baseline.fp64_gpu import Fp64Piaacmc
from csim_gb300.synth import PiaacmcSpec
from oracle.chain import host_inputs

C64, C128 = torch.complex64, torch.complex128


def _rnd(t):
    return t.to(C64).to(C128)


def _walk(m, p, mask, fpm, table, field, fft):
    """The chain of Fp64Piaacmc.field with a rounding rule for tables and
    stored fields and a choice of FFT precision."""
    e = field(table(p["pre"]) * 1.0)
    e = field(fft(e, torch.fft.fft2))
    e = field(fft(field(e * table(p["H"])), torch.fft.ifft2))
    e = field(e * table(p["m2"]))
    if fpm:
        f = field(p["A1"] @ e @ p["A1"].T)
        g = p["c"] * (p["A2"] @ field(table(mask) * f) @ p["A2"].T)
        e = field(e + g)
    e = field(e * table(m.lyot))
    return field(p["pref3"] * (p["A3"] @ e @ p["A3"].T))


def test_fp32_storage_floor_of_the_full_size_chain():
    torch.set_num_threads(min(8, torch.get_num_threads()))
    spec = PiaacmcSpec()
    inp = host_inputs(spec)
    m = Fp64Piaacmc(inp, spec, device="cpu")
    sags = torch.as_tensor(np.random.default_rng(21).uniform(-spec.sag_range, spec.sag_range,
                                                              spec.n_hex))
    p = m.per_lam[0]
    mask = m.mask(sags, p["lam"])
    ident = lambda t: t  # noqa: E731
    fft64 = lambda e, f: f(e)  # noqa: E731
    fft32 = lambda e, f: f(e.to(C64)).to(C128)  # noqa: E731
    ref_cal = _walk(m, p, mask, False, ident, ident, fft64)
    ref = _walk(m, p, mask, True, ident, ident, fft64)
    peak = ref_cal.abs().max().item()

    def err(fpm, table, field, fft):
        got = _walk(m, p, mask, fpm, table, field, fft)
        return ((got - (ref if fpm else ref_cal)).abs().max() / peak).item()

    floor = max(err(False, _rnd, _rnd, fft64), err(True, _rnd, _rnd, fft64))
    with_fft32 = max(err(False, _rnd, _rnd, fft32), err(True, _rnd, _rnd, fft32))
    plain = Fp64Piaacmc(inp, spec, device="cpu", dtype=C64)
    e_plain = max(((plain.field(0, 1.0, sags, calibrating=cal).to(C128) - r).abs().max()
                   / peak).item() for cal, r in ((True, ref_cal), (False, ref)))
    print(f"\nstorage floor {floor:.3e}, with single-precision FFTs {with_fft32:.3e}, "
          f"plain complex64 {e_plain:.3e} (of the calibration peak)")
    assert 3e-8 < floor < 2e-7
    assert with_fft32 < 2 * floor
    assert e_plain > 5e-7
