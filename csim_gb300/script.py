"""Reference input scripts driving the GPU chain.

The reference is configured by text scripts (src/lib/csim_parser.cpp:60-190):
lines with leading blanks removed, '#' comments and empty lines skipped,
`key:value` split at the first colon, and `start` / `end` delimiting nested
blocks whose first line names the block (telescope, efield, coronagraph, an
element type, a mask adapter). `load` parses such a script and builds the
same objects the reference's `coronagraph::init` (coronagraph.cpp:67-155)
and the elements' `set` methods would, reading the FITS files the script
names (relative to the script's directory unless `base_dir` is given), and
returns a batched `Coronagraph` on the GPU.

Supported blocks and keys (the rest raise ScriptError, never ignored
silently):
  telescope           primaryDiameter, primaryFRatio | primaryfRatio, magnification
  efield              setSize (square), pointSource (repeatable), wavelength,
                      wavelengthRange, wavelengthBandwidth, wavelengthList,
                      referenceWavelength, beamRadiusPhysical, pixelScale, name,
                      outputDirectory
  every element       position, name, disableForCalibration (on/off), draw (display
                      only: ignored)
  mask                filename
  mirror              filename, sign
  fresnelPropagator   propagationSign, padFactor (1)
  complexMask         filename (amplitude, phase), maskIndex (0)
  deformableMirror    actuatorFilename, sign, sigma, nActuatorRows, nActuatorCols
  fpmPupToLyot        focalRatio, fRatioSign, zoomFftSign, with a
                      fpmIntHexCMCForPupToLyot block (zoomFactor) holding a
                      complexHexMaskFPM block: maskNRings, fpmArraySize, nSubPix,
                      hexStep (1), fpmScaleFactor, hexGap, lambdaRef, phaseSign,
                      fpmFRatio, fpmRadius, fpmMaskSize, fpmMaskPhysicalSize,
                      pixelScale, sagFilename, setSag, maskFilenameRoot
  fraunhoferFocal     referenceLambda, samplesPerflD, FOVflD
Top-level tool blocks, run by `run_tools`:
  regionContrast      referenceLambda, radii, anglesInDegrees, xlimit, filename, draw
  makeContrastCurve   filename, draw, drawTo (draw / drawTo: display only)
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import coronagraph as cg
from . import fits
from .synth import EField, PointSource, Telescope


class ScriptError(ValueError):
    """A script the GPU chain cannot run (unknown element or key, bad value)."""


@dataclass
class Block:
    """One start/end block: its type (first line), key:value lines in order,
    nested blocks in order."""
    kind: str
    params: list = field(default_factory=list)
    blocks: list = field(default_factory=list)

    def get(self, key: str, default=None):
        for k, v in reversed(self.params):  # a later line overrides an earlier one
            if k == key:
                return v
        return default

    def all(self, key: str) -> list:
        return [v for k, v in self.params if k == key]


def _lines(text: str):
    for line in text.splitlines():
        line = line.lstrip(" \t").rstrip("\r\n")
        if not line or line[0] == "#":
            continue
        if ":" in line:
            k, v = line.split(":", 1)
            yield k.strip(), v
        else:
            yield line.strip(), ""


def parse(text: str) -> list:
    """Top-level blocks of a script, in order; commands outside any block
    form a leading block of kind "" (csim_parser.cpp:131-190)."""
    root = Block("")
    stack = [root]
    pending = False  # the next command names the block just started
    for k, v in _lines(text):
        if k == "start":
            blk = Block("")
            stack[-1].blocks.append(blk)
            stack.append(blk)
            pending = True
        elif k == "end":
            if len(stack) == 1:
                raise ScriptError("'end' without 'start'")
            stack.pop()
            pending = False
        elif pending:
            stack[-1].kind = k
            pending = False
            if v.strip():
                stack[-1].params.append((k, v))
        else:
            stack[-1].params.append((k, v))
    if len(stack) != 1:
        raise ScriptError("unterminated 'start' block")
    out = list(root.blocks)
    if root.params:
        out.insert(0, Block("", root.params))
    return out


def _floats(v: str, n: int | None = None) -> list:
    try:
        vals = [float(x) for x in v.replace(",", " ").split()]
    except ValueError as e:
        raise ScriptError(f"bad number list {v!r}") from e
    if n is not None and len(vals) != n:
        raise ScriptError(f"expected {n} numbers, got {v!r}")
    return vals


def _float(v: str) -> float:
    return _floats(v, 1)[0]


def _onoff(v: str) -> bool:
    s = v.strip()
    if s not in ("on", "off"):
        raise ScriptError(f"disableForCalibration must be on or off, got {v!r}")
    return s == "on"


def _check_keys(blk: Block, allowed: set):
    for k, _ in blk.params:
        if k != blk.kind and k not in allowed:
            raise ScriptError(f"{blk.kind}: key {k!r} is not supported")


_COMMON = {"position", "name", "disableForCalibration", "draw"}


def wavelengths(blk: Block) -> np.ndarray:
    """The efield block's wavelength list (efield.cpp:309-417): wavelength,
    wavelengthRange (start, end, step; round((end - start) / step) + 1
    values), wavelengthBandwidth (centre, fraction, n: n values across
    centre (1 +- fraction / 2)), wavelengthList; the last one given wins."""
    lam = None
    for k, v in blk.params:
        if k == "wavelength":
            lam = np.array([_float(v)])
        elif k == "wavelengthRange":
            a, b, d = _floats(v, 3)
            n = int(round((b - a) / d)) + 1
            lam = a + d * np.arange(n)
        elif k == "wavelengthBandwidth":
            c, f, n = _floats(v, 3)
            n = int(n)
            a, b = c - c * f / 2, c + c * f / 2
            d = (b - a) / (n - 1.0)
            lam = a + d * np.arange(n)
        elif k == "wavelengthList":
            lam = np.array(_floats(v))
    if lam is None:
        raise ScriptError("efield: no wavelength given")
    return lam


def hex_centers_reference(n_rings: int, hex_step: float = 1.0):
    """The reference's own hex layout (complexHexMaskFPM.cpp:236-315): a
    lattice of pairs ((3 i, sqrt3 j) and that + (1.5, sqrt3 / 2)) in hex-step
    units, kept where (int)|c| < nRings, numbered ring by ring in lattice
    order. Returns (hex_x, hex_y) sorted by hex number."""
    i_max = int(n_rings / 3 + 2)
    j_max = int(n_rings / math.sqrt(3) + 2)
    cells = []  # (ring, lattice order, x, y)
    order = 0
    for i in range(-i_max, i_max):
        for j in range(-j_max, j_max):
            x, y = hex_step * i * 3.0, hex_step * j * math.sqrt(3.0)
            for _ in range(2):
                ring = int(math.sqrt(x * x + y * y))
                if ring < n_rings:
                    cells.append((ring, order, x, y))
                order += 1
                x += hex_step * 1.5
                y += hex_step * math.sqrt(3.0) / 2.0
    cells.sort(key=lambda c: (c[0], c[1]))
    return np.array([c[2] for c in cells]), np.array([c[3] for c in cells])


@dataclass
class ScriptChain:
    """What a script describes, as built on the GPU."""
    coronagraph: "cg.Coronagraph"
    telescope: Telescope
    efield: EField
    elements: list          # the chain's element objects, in order
    names: list             # the script's element names (or types)
    positions: list
    sags: np.ndarray | None  # hex FPM sags from the script (candidate 0)
    tools: list = field(default_factory=list)  # regionContrast / makeContrastCurve blocks


class _Builder:
    def __init__(self, ctx, base_dir: str, precision: int):
        self.ctx, self.base, self.precision = ctx, base_dir, precision
        self.sags = None  # the hex FPM's sags, once its block is read

    def path(self, v: str) -> str:
        p = v.strip()
        return p if os.path.isabs(p) else os.path.join(self.base, p)

    def read2d(self, v: str, n: int, what: str) -> np.ndarray:
        a = fits.read(self.path(v))
        if a.ndim == 3 and a.shape[0] == 1:
            a = a[0]
        if a.shape != (n, n):
            raise ScriptError(f"{what} {v.strip()!r}: shape {a.shape}, the efield is {n} x {n}")
        return a

    def telescope(self, blk: Block) -> Telescope:
        _check_keys(blk, {"primaryDiameter", "primaryFRatio", "primaryfRatio", "magnification"})
        d = blk.get("primaryDiameter")
        f = blk.get("primaryFRatio", blk.get("primaryfRatio"))
        if d is None or f is None:
            raise ScriptError("telescope: primaryDiameter and primaryFRatio are required")
        return Telescope(_float(d), _float(f), _float(blk.get("magnification", "1")))

    def efield(self, blk: Block, tel: Telescope) -> EField:
        _check_keys(blk, {"setSize", "pointSource", "wavelength", "wavelengthRange",
                          "wavelengthBandwidth", "wavelengthList", "referenceWavelength",
                          "beamRadiusPhysical", "pixelScale", "name", "outputDirectory"})
        size = blk.get("setSize")
        if size is None:
            raise ScriptError("efield: setSize is required")
        rows, cols, _ = (int(x) for x in _floats(size, 3))
        if rows != cols:
            raise ScriptError("efield: only square arrays are supported")
        srcs = []
        for v in blk.all("pointSource"):
            flux, tip, tilt = _floats(v, 3)
            srcs.append(PointSource(flux, tip, tilt))
        for k in ("beamRadiusPhysical", "pixelScale"):
            if blk.get(k) is None:
                raise ScriptError(f"efield: {k} is required")
        return EField(rows, _float(blk.get("beamRadiusPhysical")), _float(blk.get("pixelScale")),
                      wavelengths(blk), srcs or [PointSource()])

    def element(self, blk: Block, ef: EField, tel: Telescope):
        k = blk.kind
        dis = _onoff(blk.get("disableForCalibration", "off"))
        if blk.get("save") is not None or blk.get("break") is not None:
            raise ScriptError(f"{k}: save / break are not supported")
        if k == "mask":
            _check_keys(blk, _COMMON | {"filename"})
            return cg.Mask(self.read2d(blk.get("filename", ""), ef.n, "mask"), True, dis)
        if k == "mirror":
            _check_keys(blk, _COMMON | {"filename", "sign"})
            sag = self.read2d(blk.get("filename", ""), ef.n, "mirror")
            return cg.Mirror(sag.astype(np.float32), _float(blk.get("sign", "1")))
        if k == "fresnelPropagator":
            _check_keys(blk, _COMMON | {"propagationSign", "padFactor"})
            return ("fresnel", _float(blk.get("propagationSign", "1")),
                    _float(blk.get("padFactor", "1")))
        if k == "complexMask":
            _check_keys(blk, _COMMON | {"filename", "maskIndex"})
            if int(_float(blk.get("maskIndex", "0"))) != 0:
                raise ScriptError("complexMask: only maskIndex 0 is supported")
            parts = blk.get("filename", "").split(",")
            if len(parts) != 2:
                raise ScriptError("complexMask: filename needs amplitude and phase files")
            amp, ph = (fits.read(self.path(p)) for p in parts)
            return cg.ComplexMask(amp.astype(np.float32), ph.astype(np.float32), dis)
        if k == "deformableMirror":
            _check_keys(blk, _COMMON | {"actuatorFilename", "sign", "sigma", "nActuatorRows",
                                        "nActuatorCols"})
            act = fits.read(self.path(blk.get("actuatorFilename", "")))
            if act.ndim != 2 or act.shape[0] != act.shape[1]:
                raise ScriptError("deformableMirror: a square actuator array is required")
            return cg.DeformableMirror(act, _float(blk.get("sigma", "1")),
                                       _float(blk.get("sign", "1")))
        if k == "fraunhoferFocal":
            _check_keys(blk, _COMMON | {"referenceLambda", "samplesPerflD", "FOVflD"})
            return cg.FraunhoferFocal(_float(blk.get("referenceLambda")),
                                      _float(blk.get("samplesPerflD")), _float(blk.get("FOVflD")))
        if k == "fpmPupToLyot":
            return self.fpm(blk, ef, dis)
        raise ScriptError(f"element {k!r} is not supported")

    def fpm(self, blk: Block, ef: EField, dis: bool):
        from .workloads import hex_tables
        _check_keys(blk, _COMMON | {"focalRatio", "fRatioSign", "zoomFftSign"})
        if self.sags is not None:
            raise ScriptError("fpmPupToLyot: one hex FPM per chain (its sags are the "
                              "optimisation vector)")
        if len(blk.blocks) != 1 or blk.blocks[0].kind != "fpmIntHexCMCForPupToLyot":
            raise ScriptError("fpmPupToLyot: only an fpmIntHexCMCForPupToLyot mask is supported")
        ad = blk.blocks[0]
        _check_keys(ad, {"zoomFactor"})
        zoom = _float(ad.get("zoomFactor", "-1"))
        if len(ad.blocks) != 1 or ad.blocks[0].kind != "complexHexMaskFPM":
            raise ScriptError("fpmIntHexCMCForPupToLyot: a complexHexMaskFPM block is required")
        hm = ad.blocks[0]
        _check_keys(hm, {"name", "maskNRings", "fpmArraySize", "nSubPix", "hexStep",
                         "fpmScaleFactor", "hexGap", "lambdaRef", "phaseSign", "fpmFRatio",
                         "fpmRadius", "fpmMaskSize", "fpmMaskPhysicalSize", "pixelScale",
                         "sagFilename", "setSag", "maskFilenameRoot"})
        g = lambda key, d="-1": _float(hm.get(key, d))  # noqa: E731
        S, n_sub, n_rings = int(g("fpmMaskSize")), int(g("nSubPix")), int(g("maskNRings"))
        if S <= 0 or n_sub <= 0 or n_rings <= 0:
            raise ScriptError("complexHexMaskFPM: fpmMaskSize, nSubPix, maskNRings required")
        if g("hexStep", "1") != 1:
            raise ScriptError("complexHexMaskFPM: only hexStep 1 is supported")
        # mask pixel scale (complexHexMaskFPM.cpp init_mask)
        pix = g("pixelScale")
        if pix == -1:
            if g("fpmMaskPhysicalSize") > -1:
                pix = g("fpmMaskPhysicalSize") / S
            elif zoom > -1 and g("lambdaRef") > -1 and g("fpmFRatio") > -1:
                pix = (2 * (ef.beamRadiusPhysical / (ef.pixelScale * S * zoom)) * g("lambdaRef")
                       * g("fpmFRatio"))
            else:
                raise ScriptError("complexHexMaskFPM: the mask pixel scale is undetermined")
        hx, hy = hex_centers_reference(n_rings)
        n_hex = len(hx)
        root = hm.get("maskFilenameRoot")
        f_cnt = f_ids = None
        if root is not None:
            stem = self.path(root) + f"_{S}"
            f_cnt, f_ids = stem + "_nSubPix.fits", stem + "_hexNum.fits"
        if f_cnt and fits.exists(f_cnt) and fits.exists(f_ids):
            # precomputed interpolation tables (as init_mask loads them)
            cnt = fits.read(f_cnt).astype(np.uint16)
            ids = fits.read(f_ids).astype(np.int16)
            if cnt.shape != (3, S, S) or ids.shape != (3, S, S):
                raise ScriptError("complexHexMaskFPM: interpolation tables must be 3 x S x S")
        else:
            ids, cnt, over = hex_tables(self.ctx, hx, hy, n_rings, int(g("fpmArraySize")),
                                        g("fpmScaleFactor"), g("hexGap"), math.sqrt(3.0), S,
                                        n_sub, pix, g("fpmRadius"))
            if over:
                raise ScriptError(f"complexHexMaskFPM: {over} mask pixels see more than "
                                  "three hexes (the reference asserts)")
        sags = np.zeros(n_hex)
        if hm.get("sagFilename") is not None:
            s = fits.read_vector(self.path(hm.get("sagFilename")))
            sags[:min(n_hex, s.size)] = s[:n_hex]
        for v in hm.all("setSag"):
            i, val = _floats(v, 2)
            sags[int(i)] = val
        self.sags = sags
        return cg.FpmPupToLyotHex(ids, cnt, n_sub, n_hex, pix, _float(blk.get("focalRatio")),
                                  _float(blk.get("fRatioSign", "1")),
                                  _float(blk.get("zoomFftSign", "1")),
                                  _float(hm.get("phaseSign", "1")), dis)


def load(path: str, ctx, base_dir: str | None = None, precision: int = 6) -> ScriptChain:
    """Parse the script at `path` and build its coronagraph on the GPU."""
    with open(path) as fh:
        blocks = parse(fh.read())
    b = _Builder(ctx, base_dir or os.path.dirname(os.path.abspath(path)), precision)
    by_kind, tools = {}, []
    for blk in blocks:
        if blk.kind in ("regionContrast", "makeContrastCurve"):
            tools.append(blk)
            continue
        if blk.kind in by_kind:
            raise ScriptError(f"more than one {blk.kind!r} block")
        by_kind[blk.kind] = blk
    extra = set(by_kind) - {"telescope", "efield", "coronagraph"}
    if extra:
        raise ScriptError(f"unsupported top-level blocks: {sorted(extra)}")
    for t in tools:
        _check_keys(t, {"referenceLambda", "radii", "anglesInDegrees", "xlimit", "filename",
                        "draw", "drawTo"})
    for k in ("telescope", "efield", "coronagraph"):
        if k not in by_kind:
            raise ScriptError(f"the script has no {k} block")
    tel = b.telescope(by_kind["telescope"])
    ef = b.efield(by_kind["efield"], tel)
    cor_blk = by_kind["coronagraph"]
    if cor_blk.params and any(k != "coronagraph" for k, _ in cor_blk.params):
        raise ScriptError("coronagraph: keys outside element blocks are not supported")
    built, names, pos = [], [], []
    for blk in cor_blk.blocks:
        built.append(b.element(blk, ef, tel))
        names.append((blk.get("name") or blk.kind).strip())
        pos.append(_float(blk.get("position", "0")))
    # fresnelPropagator: z = sign |next.position - prev.position| (fresnelPropagator.cpp:32)
    elems = []
    for i, e in enumerate(built):
        if isinstance(e, tuple) and e[0] == "fresnel":
            if i == 0 or i == len(built) - 1:
                raise ScriptError("fresnelPropagator needs an element before and after it")
            elems.append(cg.FresnelPropagator(e[1] * abs(pos[i + 1] - pos[i - 1]), e[2]))
        else:
            elems.append(e)
    cor = cg.Coronagraph(ctx, tel, ef, elems, precision)
    if b.sags is not None:  # the script's sags are candidate 0
        import torch
        cor.sags(1)[0].copy_(torch.as_tensor(b.sags, dtype=torch.float64))
    return ScriptChain(cor, tel, ef, elems, names, pos, b.sags, tools)


def _pair32(v: str) -> tuple:
    """Two values read as the reference does (sscanf "%f, %f": float32)."""
    a, b = _floats(v, 2)
    return float(np.float32(a)), float(np.float32(b))


def run_tools(sc: ScriptChain, out_dir: str | None = None) -> dict:
    """Run the script's regionContrast and makeContrastCurve blocks
    (regionContrast.cpp:145-205, contrastCurve.cpp:68-158): one calibration
    walk and one full walk of the sources x wavelengths batch, the region
    contrast and the contrast curve of the normalised intensity, and each
    block's output file in the reference's format (written under out_dir
    when given). Returns {"regionContrast": [..], "contrastCurve": [(pos,
    mean), ..]}."""
    cor, ctx = sc.coronagraph, sc.coronagraph.ctx
    F = cor.batch_all(1)
    cal = cor.execute(calibrating=True).clone()
    full = cor.execute(calibrating=False).clone()
    n_out = full.shape[-1]
    out = {"regionContrast": [], "contrastCurve": []}
    for t in sc.tools:
        if t.kind == "regionContrast":
            lam = _float(t.get("referenceLambda", "-1"))
            if lam <= 0:
                raise ScriptError("regionContrast: referenceLambda is required")
            r1, r2 = _pair32(t.get("radii", "0, 0"))
            a1, a2 = _pair32(t.get("anglesInDegrees", "-180, 180"))
            x1, x2 = _pair32(t.get("xlimit", "-1e16, 1e16")) if t.get("xlimit") else (-1e16,
                                                                                       1e16)
            reg = cg.RegionContrast(ctx, n_out, cor.out_pixel, sc.telescope.compute_loD(lam),
                                    r1, r2, a1, a2, x1, x2)
            cmax = reg.calibration_max(cal)
            c = float(reg.contrast(full, F, cmax).cpu().numpy()[0])
            out["regionContrast"].append(c)
            if out_dir and t.get("filename"):
                with open(os.path.join(out_dir, t.get("filename").strip()), "w") as fh:
                    fh.write(f"{a1:f}, {a2:f}\n{r1:f}, {r2:f}\n{x1:f}, {x2:f}\n{c:e}\n")
        else:  # makeContrastCurve: loD at wavelength n_lambda / 2 (integer division)
            lam = sc.efield.wavelengths[len(sc.efield.wavelengths) // 2]
            cc = cg.ContrastCurve(ctx, n_out, cor.out_pixel, sc.telescope.compute_loD(lam))
            _, mx = ctx.intensity(cal)
            ctx.sync()
            pos, mean = cc.compute(full, F, float(mx.item()))
            out["contrastCurve"].append((pos, mean))
            if out_dir and t.get("filename"):
                with open(os.path.join(out_dir, t.get("filename").strip()), "w") as fh:
                    fh.write(cg.ContrastCurve.lines(pos, mean))
    return out
