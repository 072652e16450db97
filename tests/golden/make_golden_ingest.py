"""
Generate tests/golden/g_ingest.npz with the REFERENCE's own Python frame
readers (sa_library/datareader.py DaxReader, sa_library/analysis_io.py
FrameReaderStd / FrameReaderSCMOS, sa_library/fitting.py padArray),
imported from the reference tree with import-only stand-ins for modules
that need absent packages or unbuilt C libraries (matplotlib, tifffile,
h5py, sa_h5py, writeinsight3 -- none is on the frame-reading path).

Inputs are small synthetic .dax movies (big- and little-endian) and a v2
sCMOS calibration written to a temporary directory.  Run here:

    python tests/golden/make_golden_ingest.py
"""
import os
import sys
import tempfile
import types

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree (a Python package importable from here); SA_REFERENCE overrides
REFERENCE = os.environ.get("SA_REFERENCE", "/root/reference")


def import_reference():
    for name in ["matplotlib", "matplotlib.pyplot", "tifffile", "h5py", "storm_analysis.sa_library.sa_h5py",
                 "storm_analysis.sa_library.writeinsight3"]:
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["matplotlib"].use = lambda *a, **k: None
    sys.modules["tifffile"].TiffWriter = object
    sys.modules["tifffile"].TiffFile = object
    sys.path.insert(0, REFERENCE)
    import storm_analysis.sa_library.analysis_io as aio
    return aio


def reference_pad_array():
    """padArray from the reference's sa_library/fitting.py, compiled from
    its source alone (the module imports C libraries that are not built)."""
    import ast
    path = os.path.join(REFERENCE, "storm_analysis", "sa_library", "fitting.py")
    tree = ast.parse(open(path).read())
    fn = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "padArray"][0]
    ns = {"numpy": numpy}
    exec(compile(ast.Module(body=[fn], type_ignores=[]), path, "exec"), ns)
    return ns["padArray"]


def write_dax(path, frames, bigendian):
    n, h, w = frames.shape
    data = frames.astype(">u2" if bigendian else "<u2")
    data.tofile(path)
    with open(os.path.splitext(path)[0] + ".inf", "w") as f:
        f.write("binning = 1 x 1\n")
        f.write("data type = 16 bit integers (binary, %s endian)\n" % ("big" if bigendian else "little"))
        f.write("frame dimensions = %d x %d\n" % (w, h))
        f.write("number of frames = %d\n" % n)


def main():
    aio = import_reference()
    pad_array = reference_pad_array()
    rng = numpy.random.default_rng(11)
    out = {}
    tmp = tempfile.mkdtemp()
    h, w, n = 40, 56, 3
    frames = rng.integers(90, 400, size=(n, h, w)).astype(numpy.uint16)
    frames[0, :3, :5] = 0                       # below the offset: clipped to 1
    frames[1, 10, 10] = 65535
    out["frames"] = frames
    for tag, big in (("big", 1), ("little", 0)):
        path = os.path.join(tmp, "movie_%s.dax" % tag)
        write_dax(path, frames, big)
        out["raw_%s" % tag] = numpy.fromfile(path, dtype=numpy.uint16).reshape(n, h, w)
        rd = aio.FrameReaderStd(movie_file=path, camera_gain=2.5, camera_offset=100.0)
        std = numpy.stack([rd.loadAFrame(i) for i in range(n)])
        out["std_%s" % tag] = std
        out["std_%s_pad7" % tag] = numpy.stack([pad_array(f, 7) for f in std])
        rd.close()
    offset = rng.normal(100.0, 2.0, (h, w))
    variance = rng.gamma(2.0, 2.0, (h, w))
    gain = rng.normal(2.0, 0.05, (h, w))
    rqe = rng.normal(1.0, 0.02, (h, w))
    cal = os.path.join(tmp, "calib.npy")
    numpy.save(cal, numpy.array([offset, variance, gain, rqe, 2], dtype=object), allow_pickle=True)
    out.update(offset=offset, variance=variance, gain=gain, rqe=rqe)
    rd = aio.FrameReaderSCMOS(movie_file=os.path.join(tmp, "movie_big.dax"), calibration_file=cal)
    sc = numpy.stack([rd.loadAFrame(i) for i in range(n)])
    out["scmos_big"] = sc
    out["scmos_big_pad11"] = numpy.stack([pad_array(f, 11) for f in sc])
    rd.close()
    numpy.savez_compressed(os.path.join(HERE, "g_ingest.npz"), **out)
    print("wrote g_ingest.npz:", sorted(out))


if __name__ == "__main__":
    main()
