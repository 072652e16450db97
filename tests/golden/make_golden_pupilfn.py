"""Golden vectors of the pupil-function PSF model from the reference's own
Python pupil math (simulator/pupil_math.py: Geometry, changeFocus,
translatePf, dx, toRealSpace), which pupilfn/pupil_function.c is written
to match ("This library matches the conventions established by
simulator/pupil_math.py, verified by test/test_pupilfn.py").  The module is
loaded from the reference tree by path, with stand-ins for the imports it
does not use here (tifffile and three compiled helper libraries, none of
which Geometry's construction or these transforms call).  Run in a
container that has the reference tree:

    SA_REFERENCE=/path/to/storm-analysis python tests/golden/make_golden_pupilfn.py

Writes tests/golden/g_pupilfn.npz: for two geometries (20 px as the
reference's tests, 30 px as its pupil-function diagnostics), the
geometry's kx, ky, kz, an astigmatic / comatic pupil function restricted
to the NA, and for a set of (dx, dy, dz) translations the complex PSF and
its x, y and z derivatives as pupil_function.c defines them:

    psf = toRealSpace(translatePf(changeFocus(pf, dz), dx, dy))
    dx  = toRealSpace(-2 pi i kx * T)      (T the translated pupil function)
    dy  = toRealSpace(-2 pi i ky * T)
    dz  = toRealSpace(+2 pi i kz * T)

(pfnGetPSFdx / dy multiply by -i k, pfnGetPSFdz negates the product with
-i kz: pupil_function.c:135-203.)"""
import importlib.util
import math
import os
import sys
import types

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("SA_REFERENCE", "/root/reference")


def load_pupil_math():
    class SAException(Exception):
        pass

    stubs = {
        "tifffile": types.ModuleType("tifffile"),
        "storm_analysis": types.ModuleType("storm_analysis"),
        "storm_analysis.pupilfn": types.ModuleType("storm_analysis.pupilfn"),
        "storm_analysis.pupilfn.otf_scaling_c": types.ModuleType("storm_analysis.pupilfn.otf_scaling_c"),
        "storm_analysis.pupilfn.pupil_function_c": types.ModuleType("storm_analysis.pupilfn.pupil_function_c"),
        "storm_analysis.simulator": types.ModuleType("storm_analysis.simulator"),
        "storm_analysis.simulator.pf_math_c": types.ModuleType("storm_analysis.simulator.pf_math_c"),
    }
    stubs["storm_analysis"].SAException = SAException
    stubs["storm_analysis"].pupilfn = stubs["storm_analysis.pupilfn"]
    stubs["storm_analysis"].simulator = stubs["storm_analysis.simulator"]
    stubs["storm_analysis.pupilfn"].otf_scaling_c = stubs["storm_analysis.pupilfn.otf_scaling_c"]
    stubs["storm_analysis.pupilfn"].pupil_function_c = stubs["storm_analysis.pupilfn.pupil_function_c"]
    stubs["storm_analysis.simulator"].pf_math_c = stubs["storm_analysis.simulator.pf_math_c"]
    saved = {k: sys.modules.get(k) for k in stubs}
    sys.modules.update(stubs)
    try:
        spec = importlib.util.spec_from_file_location(
            "pupil_math_ref", os.path.join(REF, "storm_analysis", "simulator", "pupil_math.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return mod


TRANSLATIONS = [(0.0, 0.0, 0.0), (0.5, 0.25, 0.2), (-0.3, 0.7, -0.4), (0.2, 0.0, 0.0), (0.0, -0.45, 0.6)]


def test_pf(geo, seed):
    """A plane wave restricted to the NA times an astigmatic (r^2 cos 2t)
    and comatic (r^3 sin t) phase, with a weak random amplitude ripple so
    that no symmetry hides a transposed axis."""
    rng = numpy.random.default_rng(seed)
    pf = geo.createPlaneWave(1.0)
    x = geo.kx * geo.size
    y = geo.ky * geo.size
    t = numpy.arctan2(y, x)
    r = geo.r
    phase = 1.3 * r * r * numpy.cos(2.0 * t) + 0.6 * r * r * r * numpy.sin(t)
    amp = 1.0 + 0.05 * rng.standard_normal(pf.shape)
    return geo.applyNARestriction(pf * amp * numpy.exp(1j * phase))


def main():
    pm = load_pupil_math()
    out = {}
    for name, (size, pixel, sim) in (("a", (20, 0.1, False)), ("b", (30, 0.1, True))):
        cls = pm.GeometrySim if sim else pm.Geometry
        geo = cls(size, pixel, 0.6, 1.5, 1.4)
        pf = test_pf(geo, seed=11 + size)
        out[name + "_kx"] = numpy.ascontiguousarray(geo.kx, dtype=numpy.float64)
        out[name + "_ky"] = numpy.ascontiguousarray(geo.ky, dtype=numpy.float64)
        out[name + "_kz"] = numpy.ascontiguousarray(numpy.real(geo.kz), dtype=numpy.float64)
        out[name + "_pf"] = pf
        rows = []
        for (dx, dy, dz) in TRANSLATIONS:
            tr = geo.translatePf(geo.changeFocus(pf, dz), dx, dy)
            rows.append(numpy.stack([
                pm.toRealSpace(tr),
                pm.toRealSpace(geo.dx(tr)),
                pm.toRealSpace(-1j * 2.0 * math.pi * geo.ky * tr),
                pm.toRealSpace(1j * 2.0 * math.pi * geo.kz * tr),
            ]))
        out[name + "_out"] = numpy.stack(rows)
    out["translations"] = numpy.array(TRANSLATIONS)
    numpy.savez_compressed(os.path.join(HERE, "g_pupilfn.npz"), **out)


if __name__ == "__main__":
    main()
