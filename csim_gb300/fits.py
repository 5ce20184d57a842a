"""FITS primary-array reader and writer with the reference's conventions.

The reference reads and writes its fixtures through cfitsio
(src/lib/csim_fits.cpp): a FITS array with NAXIS1 = n_cols, NAXIS2 = n_rows
(and NAXIS3 = n_slices) is the Armadillo matrix (row, col) (cube
(row, col, slice)), i.e. a numpy array [row][col] ([slice][row][col]) read in
C order (load_mat csim_fits.cpp:195-233, save_cube :235-261, load_cube
:311-368); complex cubes are a pair of real files <root>_re.fits and
<root>_im.fits (:263-286, :370-402); vectors are one-axis arrays. Scripts
name mask, sag and table files in this form.
"""
from __future__ import annotations

import os

import numpy as np

_BLOCK = 2880
_DTYPES = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}


def _header(raw: bytes) -> tuple[dict, int]:
    hdr: dict[str, str] = {}
    pos = 0
    while pos + 80 <= len(raw):
        card = raw[pos:pos + 80].decode("ascii", "replace")
        pos += 80
        key = card[:8].strip()
        if key == "END":
            return hdr, ((pos + _BLOCK - 1) // _BLOCK) * _BLOCK
        if card[8:10] == "= ":
            hdr[key] = card[10:].split("/")[0].strip()
    raise ValueError("FITS header has no END card")


def read(path: str) -> np.ndarray:
    """The primary array as float64 (integer data scaled by BSCALE/BZERO),
    shape (NAXISn, ..., NAXIS1)."""
    with open(path, "rb") as fh:
        raw = fh.read()
    hdr, start = _header(raw)
    bitpix = int(hdr["BITPIX"])
    if bitpix not in _DTYPES:
        raise ValueError(f"{path}: unsupported BITPIX {bitpix}")
    naxis = int(hdr.get("NAXIS", "0"))
    shape = tuple(int(hdr[f"NAXIS{i}"]) for i in range(naxis, 0, -1))
    count = int(np.prod(shape)) if shape else 0
    if start + count * abs(bitpix) // 8 > len(raw):
        raise ValueError(f"{path}: data shorter than the header says")
    data = np.frombuffer(raw, dtype=_DTYPES[bitpix], count=count, offset=start).astype(np.float64)
    scale, zero = float(hdr.get("BSCALE", "1")), float(hdr.get("BZERO", "0"))
    if scale != 1.0 or zero != 0.0:
        data = data * scale + zero
    return data.reshape(shape)


def write(path: str, arr: np.ndarray) -> None:
    """A float64 primary array (C order, last axis = NAXIS1)."""
    arr = np.ascontiguousarray(np.asarray(arr, dtype=np.float64)).astype(">f8")
    cards = ["SIMPLE  =                    T", "BITPIX  =                  -64",
             f"NAXIS   = {arr.ndim:20d}"]
    for i, n in enumerate(arr.shape[::-1], start=1):
        cards.append(f"NAXIS{i:<3d}= {n:20d}")
    cards.append("END")
    head = "".join(c.ljust(80) for c in cards).encode("ascii")
    head += b" " * ((-len(head)) % _BLOCK)
    body = arr.tobytes()
    body += b"\0" * ((-len(body)) % _BLOCK)
    with open(path, "wb") as fh:
        fh.write(head + body)


def read_complex(root: str) -> np.ndarray:
    """A complex array stored as <root>_re.fits and <root>_im.fits."""
    return read(root + "_re.fits") + 1j * read(root + "_im.fits")


def write_complex(root: str, arr: np.ndarray) -> None:
    write(root + "_re.fits", np.real(arr))
    write(root + "_im.fits", np.imag(arr))


def read_vector(path: str) -> np.ndarray:
    """A vector file (one axis, or a 1 x n / n x 1 matrix), flattened."""
    return read(path).reshape(-1)


def exists(path: str) -> bool:
    return os.path.isfile(path)
