"""
Parity metrics between two fits of the same peaks (e.g. the GPU engine and
the FP64 CPU oracle): status agreement and parameter errors of the peaks
that converged in both.

Tolerances: status agreement >= 99.9 %, and for peaks CONVERGED in both
|dx|, |dy| <= 1e-4 px, |dz| <= 1e-3 (um for the Z model, spline units for
splines), relative height / background <= 1e-4.
"""
import numpy

TOL = {"status": 0.999, "xy": 1.0e-4, "z": 1.0e-3, "rel": 1.0e-4}


def compare(a, b, z_scale=1.0):
    """a, b: dicts of per-peak arrays (x, y, z, height, background, status).
    Returns a dict of agreement / error statistics."""
    n = int(numpy.asarray(b["status"]).size)
    st_a = numpy.asarray(a["status"])
    st_b = numpy.asarray(b["status"])
    agree = st_a == st_b
    conv = agree & (st_b == 1)
    out = {"n": n, "status_agree": float(agree.mean()) if n else 1.0,
           "n_status_diff": int((~agree).sum()), "n_conv_both": int(conv.sum())}

    def mx(v):
        return float(v.max()) if v.size else 0.0

    if conv.any():
        out["max_dx"] = mx(numpy.abs(a["x"][conv] - b["x"][conv]))
        out["max_dy"] = mx(numpy.abs(a["y"][conv] - b["y"][conv]))
        out["max_dz"] = mx(numpy.abs(a["z"][conv] - b["z"][conv]) * z_scale)
        out["max_rel_h"] = mx(numpy.abs(a["height"][conv] - b["height"][conv]) /
                              numpy.abs(b["height"][conv]))
        out["max_rel_bg"] = mx(numpy.abs(a["background"][conv] - b["background"][conv]) /
                               numpy.maximum(numpy.abs(b["background"][conv]), 1e-12))
        for k, t in (("max_dx", "xy"), ("max_dy", "xy"), ("max_dz", "z"), ("max_rel_h", "rel"),
                     ("max_rel_bg", "rel")):
            key = k.replace("max_", "frac_ok_")
            diff = {"max_dx": numpy.abs(a["x"][conv] - b["x"][conv]),
                    "max_dy": numpy.abs(a["y"][conv] - b["y"][conv]),
                    "max_dz": numpy.abs(a["z"][conv] - b["z"][conv]) * z_scale,
                    "max_rel_h": numpy.abs(a["height"][conv] - b["height"][conv]) / numpy.abs(b["height"][conv]),
                    "max_rel_bg": numpy.abs(a["background"][conv] - b["background"][conv]) /
                    numpy.maximum(numpy.abs(b["background"][conv]), 1e-12)}[k]
            out[key] = float((diff <= TOL[t]).mean())
    return out


def within_tolerance(stats, min_fraction=0.999):
    """True when the spec bar holds: status agreement and, for the
    peaks converged in both, every parameter within tolerance for at least
    min_fraction of them."""
    if stats["status_agree"] < TOL["status"]:
        return False
    for k in ("frac_ok_dx", "frac_ok_dy", "frac_ok_dz", "frac_ok_rel_h", "frac_ok_rel_bg"):
        if k in stats and stats[k] < min_fraction:
            return False
    return True
