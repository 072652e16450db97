"""
Build libsa_cuda.so (the engine) from storm-analysis_gb300/csrc for sm_103a.

The five translation units (the fitter for float and double pixels, the
fitter's host API, the peak finder and the batched solver check) are compiled in parallel with nvcc
and linked into sa_gb300/libsa_cuda.so; only the CUDA runtime is linked (no
torch).  libsa_matched_filter.so and libsa_ia_utilities.so, the
reference-named matched-filter and image-analysis entry points, are linked
against it.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
REPO = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
LIB = os.path.join(HERE, "libsa_cuda.so")
MF_LIB = os.path.join(HERE, "libsa_matched_filter.so")
IA_LIB = os.path.join(HERE, "libsa_ia_utilities.so")
# reference-named forwarding libraries linked against libsa_cuda.so
SHIMS = [(MF_LIB, "sa_matched_filter.cpp"), (IA_LIB, "sa_ia_utilities.cpp")]
BUILD_DIR = os.path.join(PKG_ROOT, "_build")

SOURCES = ["sa_launch_f32.cu", "sa_launch_f64.cu", "sa_api.cu", "sa_finder.cu", "sa_solve.cu", "sa_psf_fft.cu", "sa_mp.cu",
           "sa_pupil_fn.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _compile(src, verbose):
    obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + FLAGS + ["-I", INCLUDE, "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def _stale():
    outs = [LIB] + [lib for lib, _ in SHIMS]
    if not all(os.path.exists(p) for p in outs):
        return True
    t = min(os.path.getmtime(p) for p in outs)
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    return False


def build(force=False, verbose=False):
    """Compile the engine library if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    for lib, src in SHIMS:
        tmp = lib + ".tmp"
        cmd = [nvcc(), "-shared", "-Xcompiler", "-fPIC,-O2", "-I", INCLUDE, "-o", tmp,
               os.path.join(CSRC, src), "-L", HERE, "-lsa_cuda", "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link of %s failed:\n%s\n%s" % (os.path.basename(lib), r.stdout, r.stderr))
        os.replace(tmp, lib)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
