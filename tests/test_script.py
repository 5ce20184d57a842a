"""Reference-format scripts and FITS files (no GPU): the parser's block
semantics (csim_parser.cpp), the efield wavelength setters (efield.cpp),
the reference hex layout against the oracle, FITS round trips with the
reference's conventions (csim_fits.cpp), and the errors unsupported input
raises."""
import os

import numpy as np
import pytest

from csim_gb300 import fits
from csim_gb300 import script as S
from oracle import elements as oe
from oracle import fits as ofits

SCRIPT = """#
# comment lines and blank lines are skipped
start
\ttelescope
\tprimaryDiameter:2.4
\tprimaryFRatio:15.1
end
start
    efield
    setSize:256, 256, 1
    pointSource:1.0, 0.0, 0.0
    pointSource:0.25, 0.5, -0.5
    wavelengthBandwidth: 6.5e-07, 0.1, 5
    beamRadiusPhysical:0.022
    pixelScale:1.100e-04
end
start
\tcoronagraph
\tstart
\t\tmask
\t\tfilename:pupil.fits
\t\tposition:0
\t\tname:entrance pupil
\tend
\tstart
\t\tfpmPupToLyot
\t\tfocalRatio: 80
\t\tdisableForCalibration:on
\t\tstart
\t\t\tfpmIntHexCMCForPupToLyot
\t\t\tzoomFactor: 16
\t\t\tstart
\t\t\t\tcomplexHexMaskFPM
\t\t\t\tmaskNRings: 3
\t\t\tend
\t\tend
\tend
end
"""


def test_parser_blocks_and_keys():
    blocks = S.parse(SCRIPT)
    assert [b.kind for b in blocks] == ["telescope", "efield", "coronagraph"]
    ef = blocks[1]
    assert ef.all("pointSource") == ["1.0, 0.0, 0.0", "0.25, 0.5, -0.5"]
    cor = blocks[2]
    assert [b.kind for b in cor.blocks] == ["mask", "fpmPupToLyot"]
    assert cor.blocks[0].get("name") == "entrance pupil"
    fpm = cor.blocks[1]
    assert fpm.get("focalRatio") == " 80"  # the value is everything after the first colon
    assert fpm.blocks[0].kind == "fpmIntHexCMCForPupToLyot"
    assert fpm.blocks[0].blocks[0].kind == "complexHexMaskFPM"
    assert fpm.blocks[0].blocks[0].get("maskNRings") == " 3"
    with pytest.raises(S.ScriptError):
        S.parse("start\n mask\n")
    with pytest.raises(S.ScriptError):
        S.parse("end\n")
    # commands outside blocks form a leading unnamed block
    loose = S.parse("execute\nstart\n telescope\nend\n")
    assert loose[0].kind == "" and loose[0].params == [("execute", "")]


def test_efield_wavelength_setters():
    blk = S.Block("efield", [("wavelengthBandwidth", "6.5e-07, 0.1, 5")])
    c, f, n = 6.5e-7, 0.1, 5  # efield.cpp:368-389
    a, b = c - c * f / 2, c + c * f / 2
    assert np.allclose(S.wavelengths(blk), a + (b - a) / (n - 1.0) * np.arange(n), rtol=0,
                       atol=1e-22)
    blk = S.Block("efield", [("wavelengthRange", "5e-7, 6e-7, 2.5e-8")])
    assert S.wavelengths(blk).size == 5  # round((end - start) / step) + 1
    blk = S.Block("efield", [("wavelength", "5.5e-7"), ("wavelengthList", "5e-7 6e-7")])
    assert np.array_equal(S.wavelengths(blk), [5e-7, 6e-7])  # the last setter wins


def test_reference_hex_layout_matches_oracle():
    for n_rings in (3, 8, 20, 32):
        hx, hy = S.hex_centers_reference(n_rings)
        _, ox, oy, _ = oe.hex_centers(n_rings)
        assert np.array_equal(hx, ox) and np.array_equal(hy, oy)


def test_fits_round_trip_and_reference_conventions(tmp_path):
    rng = np.random.default_rng(0)
    cube = rng.standard_normal((3, 5, 7))  # [slice][row][col]
    p = str(tmp_path / "c.fits")
    fits.write(p, cube)
    assert np.array_equal(fits.read(p), cube)
    assert np.array_equal(ofits.read(p), cube)  # same file layout as the oracle's reader
    z = cube + 1j * rng.standard_normal(cube.shape)
    fits.write_complex(str(tmp_path / "z"), z)
    assert np.array_equal(fits.read_complex(str(tmp_path / "z")), z)
    assert os.path.isfile(str(tmp_path / "z_re.fits"))
    # float32 data with NAXIS1 = columns reads as [row][col]
    m = rng.standard_normal((4, 6)).astype(">f4")
    cards = ["SIMPLE  =                    T", "BITPIX  =                  -32",
             "NAXIS   =                    2", "NAXIS1  =                    6",
             "NAXIS2  =                    4", "END"]
    head = "".join(c.ljust(80) for c in cards).encode()
    head += b" " * ((-len(head)) % 2880)
    body = m.tobytes()
    body += b"\0" * ((-len(body)) % 2880)
    (tmp_path / "f.fits").write_bytes(head + body)
    assert np.array_equal(fits.read(str(tmp_path / "f.fits")), m.astype(np.float64))


def test_unsupported_input_raises(tmp_path):
    b = S._Builder(None, str(tmp_path), 6)
    with pytest.raises(S.ScriptError, match="not supported"):
        b.element(S.Block("zoomDftPropagator"), None, None)
    with pytest.raises(S.ScriptError, match="key"):
        b.element(S.Block("fresnelPropagator", [("bogus", "1")]), None, None)
    # padFactor is supported: the element carries it
    assert b.element(S.Block("fresnelPropagator", [("padFactor", "2")]), None, None) == \
        ("fresnel", 1.0, 2.0)
    with pytest.raises(S.ScriptError, match="on or off"):
        b.element(S.Block("mask", [("disableForCalibration", "yes")]), None, None)
