"""Minimal FITS primary-HDU reader/writer for the oracle and the fixtures.

TEST INFRASTRUCTURE ONLY: this module belongs to the CPU oracle. Nothing in the
shipped library imports it.

Conventions follow the reference's cfitsio wrappers (src/lib/csim_fits.cpp):
  * a FITS array with NAXIS1 = n_cols, NAXIS2 = n_rows, NAXIS3 = n_slices is an
    Armadillo cube (row, col, slice); read in C order it is a numpy array
    [slice][row][col], which is the layout used everywhere in this project
    (csim_fits.cpp:195-233 load_mat, :235-261 save_cube, :311-368 load_cube);
  * complex cubes are stored as a pair of real files "<root>_re.fits" and
    "<root>_im.fits" (csim_fits.cpp:263-286 save_cube(cx_cube), :370-402).
Only BITPIX -64/-32/8/16/32/64 primary arrays are supported (all the fixtures
are -64).
"""
from __future__ import annotations

import numpy as np

_BLOCK = 2880
_DT = {-64: ">f8", -32: ">f4", 8: "u1", 16: ">i2", 32: ">i4", 64: ">i8"}


def read(path: str) -> np.ndarray:
    """Read the primary array of a FITS file; returns shape (NAXISn, ..., NAXIS1)."""
    with open(path, "rb") as fh:
        raw = fh.read()
    hdr: dict[str, str] = {}
    pos = 0
    while True:
        card = raw[pos:pos + 80].decode("ascii", "replace")
        pos += 80
        key = card[:8].strip()
        if key == "END":
            break
        if card[8:10] == "= ":
            hdr[key] = card[10:].split("/")[0].strip()
    start = ((pos + _BLOCK - 1) // _BLOCK) * _BLOCK
    bitpix = int(hdr["BITPIX"])
    naxis = int(hdr["NAXIS"])
    shape = tuple(int(hdr[f"NAXIS{i}"]) for i in range(naxis, 0, -1))
    count = int(np.prod(shape)) if shape else 0
    data = np.frombuffer(raw, dtype=_DT[bitpix], count=count, offset=start)
    return data.reshape(shape).astype(np.float64 if bitpix < 0 else np.int64)


def write(path: str, arr: np.ndarray) -> None:
    """Write a float64 primary array (C order, last axis = NAXIS1)."""
    arr = np.ascontiguousarray(arr, dtype=">f8")
    cards = ["SIMPLE  =                    T", "BITPIX  =                  -64",
             f"NAXIS   = {arr.ndim:20d}"]
    for i, n in enumerate(arr.shape[::-1], start=1):
        cards.append(f"NAXIS{i:<3d}= {n:20d}")
    cards.append("EXTEND  =                    T")
    cards.append("END")
    head = "".join(c.ljust(80) for c in cards).encode("ascii")
    head += b" " * ((-len(head)) % _BLOCK)
    body = arr.tobytes()
    body += b"\0" * ((-len(body)) % _BLOCK)
    with open(path, "wb") as fh:
        fh.write(head + body)


def read_complex(root: str) -> np.ndarray:
    """Read a complex cube saved as <root>_re.fits / <root>_im.fits."""
    return read(root + "_re.fits") + 1j * read(root + "_im.fits")
