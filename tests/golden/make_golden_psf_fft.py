"""Golden vectors of the PSF-FFT model from the reference's own pure-Python
version of psf_fft.c (psf_fft/psf_fft_py.py, loaded from the reference
tree by path: the package's __init__ needs matplotlib, which is not
installed here).  Run in a container that has the reference tree:

    SA_REFERENCE=/path/to/storm-analysis python tests/golden/make_golden_psf_fft.py

Writes tests/golden/g_psf_fft.npz: for the test PSF of oracle/psf_fft.py
and a set of (dx, dy, dz) translations, the middle-plane PSF and its x, y
and z derivatives."""
import importlib.util
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import psf_fft as opf  # noqa: E402

REF = os.environ.get("SA_REFERENCE", "/root/reference")
spec = importlib.util.spec_from_file_location(
    "psf_fft_py", os.path.join(REF, "storm_analysis", "psf_fft", "psf_fft_py.py"))
ref = importlib.util.module_from_spec(spec)
spec.loader.exec_module(ref)

TRANSLATIONS = [(0.0, 0.0, 0.0), (0.5, 0.25, 0.2), (-0.3, 0.7, -1.4), (0.2, 0.0, 0.0), (0.0, -0.45, 2.1)]


def main():
    out = {}
    # odd z sizes, as the reference's own test (17 planes): with an even z size
    # the C and Python versions differ at the z Nyquist plane
    for name, (z, size) in (("a", (17, 20)), ("b", (21, 16))):
        psf = opf.test_psf(z, size, seed=3)
        out[name + "_psf"] = psf
        rows = []
        for (dx, dy, dz) in TRANSLATIONS:
            p = ref.PSFFFT(psf)
            p.translate(dx, dy, dz)
            rows.append(numpy.stack([p.getPSF(), p.getPSFdx(), p.getPSFdy(), p.getPSFdz()]))
        out[name + "_out"] = numpy.stack(rows)
    out["translations"] = numpy.array(TRANSLATIONS)
    numpy.savez_compressed(os.path.join(HERE, "g_psf_fft.npz"), **out)


if __name__ == "__main__":
    main()
