"""Generate the committed golden fixtures from the reference's own data files.

Usage: python tests/golden/make_golden.py REFERENCE_TREE (or with the tree's
path in the CSIM_REFERENCE environment variable); writes tests/golden/*.npz.
The GPU machine never needs the reference: the tests read the .npz files only.

Fixtures:
  mono_response.npz  donutPiaaFullCircleExample/mono_2_6/responseData: the
                     response matrix M (complex128 [1][636][500], FITS
                     transposed back to Armadillo (row, col) order as the
                     reference's load_cube does), wavelengths, calibration
                     intensity; plus every recorded bestOptVector.fits of the
                     mono runs and the last recorded best value of each run.
  hex_counts.npz     wfirst_sags.fits length (1237 = reference hex layout
                     with 32 rings).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import fits  # noqa: E402



def last_best(path):
    lines = [l.split() for l in open(path) if l.strip()]
    return int(lines[-1][0]), float(lines[-1][1])


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CSIM_REFERENCE")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_golden.py REFERENCE_TREE (or set CSIM_REFERENCE)")
    ex = os.path.join(ref, "donutPiaaFullCircleExample")
    mono = os.path.join(ex, "mono_2_6")
    m = fits.read_complex(os.path.join(mono, "responseData", "responseData_s0_p0"))
    params = open(os.path.join(mono, "responseData", "problemParams.txt")).read().split("\n")
    calib = float(params[0].split(":")[1])
    lam = [float(v) for v in params[1].split(":")[1].split()]
    xs, bests, its, runs = [], [], [], []
    for run in ("optTest", "optTest1"):
        d = os.path.join(mono, run)
        xs.append(fits.read(os.path.join(d, "bestOptVector.fits")))
        it, b = last_best(os.path.join(d, "optBestVal.txt"))
        its.append(it)
        bests.append(b)
        runs.append(run)
    np.savez(os.path.join(HERE, "mono_response.npz"), M=m, wavelengths=np.array(lam),
             calib=np.array(calib), best_x=np.array(xs), best_val=np.array(bests),
             best_iter=np.array(its), runs=np.array(runs))
    w = fits.read(os.path.join(ref, "wfirst_sags.fits"))
    np.savez(os.path.join(HERE, "hex_counts.npz"), wfirst_sags_len=np.array(w.size))
    print("wrote fixtures; M", m.shape, "calib", calib, "lambda", lam, "best", bests)


if __name__ == "__main__":
    main()
