"""
Seeded synthetic localisation workloads for the LM fitter.

No public dataset is involved: every workload is drawn from numpy's
``default_rng(seed)``.  Shapes, densities and value ranges follow the five
benchmark configurations of the fitting step:

  cfg 0  '2d'  1 x 256^2, 200 emitters (>= 4 px apart), sigma 1.3 px,
         height U(500, 3000), background 20, Poisson, roi 10
  cfg 1  '3d'  64 x 512^2, Poisson(0.5 /um^2) emitters (~3355 / frame),
         sigma_x, sigma_y U(1, 2) px, height log-U(200, 5000),
         background U(5, 50) per frame, Poisson, roi 18
  cfg 2  'Z'   128 x 256^2, 1000 emitters, w0 1.6 px, c +-0.15 um, d 0.4 um,
         z U(-0.4, 0.4) um, height U(1000, 4000), sCMOS camera noise
         (offset N(100, 2), variance Gamma(2, 2) ADU^2, gain N(2, 0.05)), roi 12
  cfg 3  spline 256 x 256^2, 800 emitters, 21^3-knot tricubic spline of the
         cfg-2 astigmatic PSF with a 0.05-amplitude smooth random aberration,
         z U(-0.5, 0.5) um, Poisson
  cfg 4  serving mix of the above models and sizes (see ``serving_requests``)

The camera model and pre-processing follow the reference:
sCMOS noise per simulator/camera.py:121-137 and ADU -> e- conversion with
the clip to >= 1 per sa_library/analysis_io.py:243-260.

Initial guesses for every configuration: x/y = truth + N(0, 0.3 px),
height and sigma x U(0.8, 1.2), background = truth, Z: z = truth + N(0, 0.05 um).
They are passed in the reference's pre-specified ("hdf5") peak format so
both the oracle and the GPU engine start from identical parameters.
"""
import math

import numpy

PIXEL_UM = 0.160

# Z model defocus curves: [w0 (px), c (um), d (um), A, B] (sa_library/parameters.py:557-574 units).
WX_PARAMS = numpy.array([1.6, 0.15, 0.4, 0.0, 0.0])
WY_PARAMS = numpy.array([1.6, -0.15, 0.4, 0.0, 0.0])
Z_RANGE = (-0.5, 0.5)

SPLINE_ZMIN_NM = -600.0
SPLINE_ZMAX_NM = 600.0
SPLINE_KNOTS = 21


def _widths_from_z(z, wp):
    """sigma_x or sigma_y (px) of the Z model at z (um) (dao_fit.c:1009-1035)."""
    z0 = (z - wp[1]) / wp[2]
    t = 1.0 + z0 * z0 + wp[3] * z0 ** 3 + wp[4] * z0 ** 4
    # width = 2/(w0^2 t) = 1/(2 sigma^2)  ->  sigma = w0 sqrt(t) / 2
    return 0.5 * wp[0] * numpy.sqrt(t)


def _place_uniform(rng, n, nx, ny, margin, min_sep=0.0):
    """Uniform positions inside [margin, size - margin - 1], optional min separation."""
    lo = float(margin)
    hix = float(nx - margin - 1)
    hiy = float(ny - margin - 1)
    if min_sep <= 0.0:
        return rng.uniform(lo, hix, n), rng.uniform(lo, hiy, n)
    # rejection sampling; accepted points are binned in min_sep cells so that
    # a candidate is checked against the 3 x 3 neighbouring cells only
    xs, ys = [], []
    grid = {}
    s2 = min_sep * min_sep
    tries = 0
    while len(xs) < n and tries < 200 * n:
        tries += 1
        x = rng.uniform(lo, hix)
        y = rng.uniform(lo, hiy)
        cx, cy = int(x // min_sep), int(y // min_sep)
        ok = True
        for gx in (cx - 1, cx, cx + 1):
            for gy in (cy - 1, cy, cy + 1):
                for (a, b) in grid.get((gx, gy), ()):
                    if (a - x) ** 2 + (b - y) ** 2 < s2:
                        ok = False
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            xs.append(x)
            ys.append(y)
            grid.setdefault((cx, cy), []).append((x, y))
    return numpy.array(xs), numpy.array(ys)


def _render_gauss(nx, ny, x, y, h, sx, sy, out):
    """Add h * exp(-(c-x)^2/(2 sx^2) - (r-y)^2/(2 sy^2)) at pixel centres (c, r)."""
    rad = 8
    for i in range(x.size):
        cx, cy = int(round(x[i])), int(round(y[i]))
        rad_x = int(min(max(rad, 5.0 * sx[i]), 40))
        rad_y = int(min(max(rad, 5.0 * sy[i]), 40))
        c0, c1 = max(0, cx - rad_x), min(nx, cx + rad_x + 1)
        r0, r1 = max(0, cy - rad_y), min(ny, cy + rad_y + 1)
        cc = numpy.arange(c0, c1) - x[i]
        rr = numpy.arange(r0, r1) - y[i]
        gx = numpy.exp(-cc * cc / (2.0 * sx[i] * sx[i]))
        gy = numpy.exp(-rr * rr / (2.0 * sy[i] * sy[i]))
        out[r0:r1, c0:c1] += h[i] * numpy.outer(gy, gx)


def _camera_poisson(rng, expected, offset=100.0, gain=1.0):
    """Poisson camera, then the reference's pre-processing (ADU -> e-, clip >= 1)."""
    adu = rng.poisson(expected).astype(numpy.float64) * gain + offset
    img = (adu - offset) / gain
    img[img < 1.0] = 1.0
    return img


def _camera_scmos(rng, expected, rqe, offset, variance, gain):
    """sCMOS camera (simulator/camera.py:121-137) + pre-processing (analysis_io.py:243-260)."""
    e = rng.poisson(expected * rqe).astype(numpy.float64)
    adu = e * gain + rng.normal(0.0, 1.0, size=e.shape) * numpy.sqrt(variance) + offset
    img = (adu - offset) / gain / rqe
    img[img < 1.0] = 1.0
    return img


# ----------------------------------------------------------------------------
# spline PSF
# ----------------------------------------------------------------------------

_CR = numpy.array([[0.0, 1.0, 0.0, 0.0],
                   [-0.5, 0.0, 0.5, 0.0],
                   [1.0, -2.5, 2.0, -0.5],
                   [-0.5, 1.5, -1.5, 0.5]])


def tricubic_coefficients(samples):
    """Per-cell monomial coefficients of a C1 tricubic (Catmull-Rom) interpolant.

    samples: (n, n, n) knot values indexed [x, y, z].  Returns (n-1, n-1, n-1, 64)
    with coefficient i*16+j*4+k multiplying dx^i dy^j dz^k, the layout the
    fitter reads (spliner/cubic_spline.c:509-522, spliner/spline3D.py:72-102).
    """
    s = numpy.asarray(samples, dtype=numpy.float64)
    n = s.shape[0]
    p = numpy.pad(s, ((1, 2), (1, 2), (1, 2)), mode="edge")
    w = numpy.lib.stride_tricks.sliding_window_view(p, (4, 4, 4))[:n - 1, :n - 1, :n - 1]
    c = numpy.einsum("im,jn,ko,abcmno->abcijk", _CR, _CR, _CR, w, optimize=True)
    return numpy.ascontiguousarray(c.reshape(n - 1, n - 1, n - 1, 64))


def bicubic_coefficients(samples):
    """2D analogue: (n, n) knots [x, y] -> (n-1, n-1, 16), index 4*i+j <-> dx^i dy^j."""
    s = numpy.asarray(samples, dtype=numpy.float64)
    n = s.shape[0]
    p = numpy.pad(s, ((1, 2), (1, 2)), mode="edge")
    w = numpy.lib.stride_tricks.sliding_window_view(p, (4, 4))[:n - 1, :n - 1]
    c = numpy.einsum("im,jn,abmn->abij", _CR, _CR, w, optimize=True)
    return numpy.ascontiguousarray(c.reshape(n - 1, n - 1, 16))


def _aberrated_psf(dx, dy, z_um, coef):
    sx = _widths_from_z(z_um, WX_PARAMS)
    sy = _widths_from_z(z_um, WY_PARAMS)
    g = numpy.exp(-dx * dx / (2.0 * sx * sx) - dy * dy / (2.0 * sy * sy))
    u, v = dx / 10.0, dy / 10.0
    poly = (coef[0] * u + coef[1] * v + coef[2] * (u * u - v * v) + coef[3] * u * v +
            coef[4] * z_um * u + coef[5] * z_um * v)
    return g * (1.0 + 0.05 * numpy.tanh(poly))


def make_spline(seed=3, knots=SPLINE_KNOTS):
    """Spline PSF for cfg 3: knots^3 samples, spline z in [0, knots-1] <-> [zmin, zmax] nm."""
    rng = numpy.random.default_rng(1000 + seed)
    coef = rng.normal(0.0, 1.0, 6)
    half = (knots - 1) / 2.0
    a = numpy.arange(knots) - half
    zs = SPLINE_ZMIN_NM + numpy.arange(knots) * (SPLINE_ZMAX_NM - SPLINE_ZMIN_NM) / (knots - 1)
    X, Y, Z = numpy.meshgrid(a, a, zs * 1.0e-3, indexing="ij")
    samples = _aberrated_psf(X, Y, Z, coef)
    return {"coeff": tricubic_coefficients(samples), "coef_ab": coef,
            "zmin": SPLINE_ZMIN_NM, "zmax": SPLINE_ZMAX_NM, "size": knots - 1}


def spline_scaled_z(z_um, size):
    """spliner/spline_to_psf.py:202-203 getScaledZ (z given in nm there)."""
    return float(size) * (z_um * 1000.0 - SPLINE_ZMIN_NM) / (SPLINE_ZMAX_NM - SPLINE_ZMIN_NM)


# ----------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------

CONFIGS = {
    0: dict(model="2d", frames=1, nx=256, ny=256, roi=10),
    1: dict(model="3d", frames=64, nx=512, ny=512, roi=18),
    2: dict(model="Z", frames=128, nx=256, ny=256, roi=12),
    3: dict(model="spline3D", frames=256, nx=256, ny=256, roi=19),
}


def fitter_kwargs(cfg, spline=None):
    """Constructor arguments of the MultiFitter sub-class for a configuration."""
    c = CONFIGS[cfg]
    if c["model"] == "2d":
        return dict(model="2d", roi_size=10, sigma_range=[0.5, 3.0])
    if c["model"] == "3d":
        return dict(model="3d", roi_size=18, sigma_range=[0.5, 4.0])
    if c["model"] == "Z":
        return dict(model="Z", roi_size=12, wx_params=WX_PARAMS.copy(),
                    wy_params=WY_PARAMS.copy(), min_z=Z_RANGE[0], max_z=Z_RANGE[1])
    return dict(model="spline3D", spline=spline)


_SPLINES = {}


def cached_spline(seed):
    if seed not in _SPLINES:
        _SPLINES[seed] = make_spline(seed)
    return _SPLINES[seed]


def make_workload(cfg, frames=None, nx=None, ny=None, seed=None, n_emitters=None, camera_seed=None,
                  min_sep=4.0):
    """Return a dict with per-frame images, backgrounds, truth and initial guesses.

    images[f] and backgrounds[f] are float64 (ny, nx) arrays in photo-electrons;
    guesses[f] is the dict of columns for newPeaks(..., "hdf5").  camera_seed
    fixes the camera (sCMOS calibration, spline PSF) independently of the
    frame content, as for frames of one camera in a request stream.
    min_sep is the minimum emitter separation (px) of configuration 0.
    """
    c = dict(CONFIGS[cfg])
    if frames is not None:
        c["frames"] = frames
    if nx is not None:
        c["nx"] = nx
    if ny is not None:
        c["ny"] = ny
    seed = cfg if seed is None else seed
    rng = numpy.random.default_rng(seed)
    nx, ny, roi = c["nx"], c["ny"], c["roi"]
    margin = roi // 2 + 2
    out = dict(cfg=cfg, model=c["model"], nx=nx, ny=ny, roi=roi, images=[], backgrounds=[],
               truth=[], guesses=[], rqe=numpy.ones((ny, nx)), scmos_cal=numpy.zeros((ny, nx)))
    spline = None
    cam = rng if camera_seed is None else numpy.random.default_rng(camera_seed)
    if cfg == 3:
        spline = make_spline(seed) if camera_seed is None else cached_spline(camera_seed)
        out["spline"] = spline
    if cfg == 2:
        offset = cam.normal(100.0, 2.0, size=(ny, nx))
        variance = cam.gamma(2.0, 2.0, size=(ny, nx))
        gain = cam.normal(2.0, 0.05, size=(ny, nx))
        out["scmos_cal"] = variance / (gain * gain)
    area_um2 = (nx * PIXEL_UM) * (ny * PIXEL_UM)
    for f in range(c["frames"]):
        if cfg == 0:
            n = 200 if n_emitters is None else n_emitters
            x, y = _place_uniform(rng, n, nx, ny, margin, min_sep=min_sep)
            n = x.size
            sx = numpy.full(n, 1.3)
            sy = sx.copy()
            h = rng.uniform(500.0, 3000.0, n)
            bg = 20.0
            z = numpy.zeros(n)
        elif cfg == 1:
            n = rng.poisson(0.5 * area_um2) if n_emitters is None else n_emitters
            x, y = _place_uniform(rng, n, nx, ny, margin)
            sx = rng.uniform(1.0, 2.0, n)
            sy = rng.uniform(1.0, 2.0, n)
            h = numpy.exp(rng.uniform(math.log(200.0), math.log(5000.0), n))
            bg = rng.uniform(5.0, 50.0)
            z = numpy.zeros(n)
        elif cfg == 2:
            n = 1000 if n_emitters is None else n_emitters
            x, y = _place_uniform(rng, n, nx, ny, margin)
            z = rng.uniform(-0.4, 0.4, n)
            sx = _widths_from_z(z, WX_PARAMS)
            sy = _widths_from_z(z, WY_PARAMS)
            h = rng.uniform(1000.0, 4000.0, n)
            bg = 20.0
        else:
            n = 800 if n_emitters is None else n_emitters
            x, y = _place_uniform(rng, n, nx, ny, margin)
            z = rng.uniform(-0.5, 0.5, n)
            h = rng.uniform(1000.0, 4000.0, n)
            bg = 20.0
            sx = sy = None
        expected = numpy.full((ny, nx), float(bg))
        if cfg == 3:
            half = 10
            coef = spline["coef_ab"]
            for i in range(n):
                cx, cy = int(round(x[i])), int(round(y[i]))
                c0, c1 = max(0, cx - half), min(nx, cx + half + 1)
                r0, r1 = max(0, cy - half), min(ny, cy + half + 1)
                dxg, dyg = numpy.meshgrid(numpy.arange(c0, c1) - x[i], numpy.arange(r0, r1) - y[i])
                expected[r0:r1, c0:c1] += h[i] * _aberrated_psf(dxg, dyg, z[i], coef)
        else:
            _render_gauss(nx, ny, x, y, h, sx, sy, expected)
        if cfg == 2:
            img = _camera_scmos(rng, expected, out["rqe"], offset, variance, gain)
        else:
            img = _camera_poisson(rng, expected)
        # Initial guesses (identical for the oracle and the engine).
        gx = x + rng.normal(0.0, 0.3, n)
        gy = y + rng.normal(0.0, 0.3, n)
        gh = h * rng.uniform(0.8, 1.2, n)
        g = {"x": gx, "y": gy, "background": numpy.full(n, float(bg)), "height": gh}
        if cfg == 3:
            g["z"] = numpy.array([spline_scaled_z(zz, spline["size"]) for zz in
                                  (z + rng.normal(0.0, 0.05, n))])
        else:
            fs = rng.uniform(0.8, 1.2, n)
            if c["model"] == "2d":
                g["xsigma"] = sx * fs
                g["ysigma"] = sx * fs
            else:
                g["xsigma"] = sx * fs
                g["ysigma"] = sy * rng.uniform(0.8, 1.2, n)
            g["z"] = (z + rng.normal(0.0, 0.05, n)) if cfg == 2 else numpy.zeros(n)
        out["images"].append(img)
        out["backgrounds"].append(numpy.full((ny, nx), float(bg)))
        out["truth"].append({"x": x, "y": y, "z": z, "height": h})
        out["guesses"].append(g)
    out["fitter"] = fitter_kwargs(cfg, spline)
    return out


def serving_requests(n_requests=10000, rate_hz=2000.0, seed=4, sizes=(128, 256, 512, 2048),
                     models=("2d", "3d", "Z", "spline3D")):
    """Request stream of cfg 4: arrival times, frame size, density and model per request."""
    rng = numpy.random.default_rng(seed)
    t = numpy.cumsum(rng.exponential(1.0 / rate_hz, n_requests))
    sizes = rng.choice(list(sizes), n_requests)
    dens = numpy.exp(rng.uniform(math.log(0.05), math.log(2.0), n_requests))
    models = rng.choice(list(models), n_requests)
    return dict(t=t, size=sizes, density=dens, model=models)


MODEL_CFG = {"2d": 0, "3d": 1, "Z": 2, "spline3D": 3}


def serving_frame(model, size, density, seed):
    """One request of the serving stream: a single frame of `size` x `size`
    pixels at `density` emitters / um^2 (uniform positions, no minimum
    separation) with the model's configuration parameters; the camera
    (calibration, spline) is fixed per model and size.  Returns the
    make_workload dict of one frame."""
    cfg = MODEL_CFG[model]
    n = max(1, int(round(density * (size * PIXEL_UM) ** 2)))
    return make_workload(cfg, frames=1, nx=size, ny=size, seed=seed, n_emitters=n,
                         camera_seed=10000 + 97 * cfg + size, min_sep=0.0)


# ---------------------------------------------------------------------------
# FFT PSF model workload (psf_fft / fft_fit)
# ---------------------------------------------------------------------------

def fft_psf_stack(z_size=17, size=20, seed=3):
    """A measured-PSF stand-in for the FFT PSF model: an astigmatic stack
    of z_size planes on a size x size grid (x fastest), widths 1.6 px at the
    middle plane changing +-35 % across the stack, a 2 % per-plane ripple,
    the middle plane summing to 1."""
    rng = numpy.random.default_rng(seed)
    zz = numpy.linspace(-1.0, 1.0, z_size)[:, None, None]
    yy = (numpy.arange(size) - size / 2.0)[None, :, None]
    xx = (numpy.arange(size) - size / 2.0)[None, None, :]
    sx = 1.6 * (1.0 + 0.35 * zz + 0.2 * zz * zz)
    sy = 1.6 * (1.0 - 0.35 * zz + 0.2 * zz * zz)
    psf = numpy.exp(-xx * xx / (2 * sx * sx) - yy * yy / (2 * sy * sy))
    psf = psf * (1.0 + 0.02 * rng.standard_normal((z_size, 1, 1)))
    return psf / psf[z_size // 2].sum()


def fft_workload(frames=4, nx=256, ny=256, n_emitters=300, seed=21, background=10.0):
    """Frames of emitters drawn with the FFT PSF model itself (the PSF
    translated by its spectrum, psf_fft_c.PSFFFT; Poisson noise) and
    "hdf5" starting peaks: the truth perturbed by 0.3 px in x / y, half its
    z, 80 % of its height.  z in z pixels of the stack, within +-3."""
    from . import psf_fft_c
    psf = fft_psf_stack()
    pf = psf_fft_c.PSFFFT(psf)
    size = psf.shape[1]
    xoff, yoff = 0.5 * size - 1.0, 0.5 * psf.shape[1] - 1.0
    rng = numpy.random.default_rng(seed)
    out = dict(model="fft", nx=nx, ny=ny, images=[], backgrounds=[], truth=[], guesses=[],
               rqe=numpy.ones((ny, nx)), scmos_cal=numpy.zeros((ny, nx)), fitter={"model": "fft", "psf": psf})
    for _ in range(frames):
        img = numpy.full((ny, nx), background)
        x = rng.uniform(size, nx - size, n_emitters)
        y = rng.uniform(size, ny - size, n_emitters)
        z = rng.uniform(-3.0, 3.0, n_emitters)
        h = rng.uniform(3000.0, 20000.0, n_emitters)
        for i in range(n_emitters):
            px, py = x[i] - xoff, y[i] - yoff
            xi, yi = int(math.floor(px)), int(math.floor(py))
            pf.translate(px - xi, py - yi, z[i])
            img[yi:yi + size, xi:xi + size] += h[i] * pf.getPSF()
        out["images"].append(rng.poisson(img).astype(numpy.float64))
        out["backgrounds"].append(numpy.full((ny, nx), background))
        out["truth"].append(dict(x=x, y=y, z=z, height=h))
        out["guesses"].append(dict(x=x + rng.normal(0.0, 0.3, n_emitters), y=y + rng.normal(0.0, 0.3, n_emitters),
                                   z=0.5 * z, background=numpy.full(n_emitters, background), height=0.8 * h))
    pf.cleanup()
    return out


def pupil_function_data(size=30, pixel_size=0.1, seed=5, astigmatism=1.3, coma=0.4, sim=True):
    """A pupil-function file's contents (the dict a reference .pfn pickle
    holds) for a size x size pupil at the given camera pixel size (um),
    emission 0.6 um, oil immersion (1.5), NA 1.4, with astigmatic
    (r^2 cos 2t) and comatic (r^3 sin t) phase and a 5 % amplitude ripple,
    normalised to a peak PSF intensity of 1 at focus."""
    from . import pupil_math
    rng = numpy.random.default_rng(seed)
    cls = pupil_math.GeometrySim if sim else pupil_math.Geometry
    geo = cls(size, pixel_size, 0.6, 1.5, 1.4)
    t = numpy.arctan2(geo.ky, geo.kx)
    r = geo.r
    phase = astigmatism * r * r * numpy.cos(2.0 * t) + coma * r * r * r * numpy.sin(t)
    pf = geo.createFromPhase(1.0, phase) * (1.0 + 0.05 * rng.standard_normal((size, size)))
    pf = geo.applyNARestriction(pf)
    pf = pf / math.sqrt(numpy.max(pupil_math.intensity(pupil_math.toRealSpace(pf))))
    return {"pf": pf.astype(numpy.complex128), "pixel_size": pixel_size, "geo_sim_pf": sim, "wavelength": 0.6,
            "immersion_index": 1.5, "numerical_aperture": 1.4}


def pupil_workload(frames=4, nx=256, ny=256, n_emitters=300, seed=23, background=10.0, size=30):
    """Frames of emitters drawn with the pupil-function model itself (the
    pupil function translated and transformed, pupil_function_c; Poisson
    noise) and "hdf5" starting peaks: the truth perturbed by 0.3 px in
    x / y, half its z, 80 % of its height.  z in microns within +-0.4."""
    from . import pupil_fn
    pf_data = pupil_function_data(size=size)
    pfn = pupil_fn.PupilFunction(pf_data=pf_data, zmin=-500.0, zmax=500.0)
    c = pfn.pupil_fn_c
    off = 0.5 * size
    rng = numpy.random.default_rng(seed)
    out = dict(model="pupil", nx=nx, ny=ny, images=[], backgrounds=[], truth=[], guesses=[],
               rqe=numpy.ones((ny, nx)), scmos_cal=numpy.zeros((ny, nx)),
               fitter={"model": "pupil", "pf_data": pf_data, "zmin": -500.0, "zmax": 500.0})
    for _ in range(frames):
        img = numpy.full((ny, nx), background)
        x = rng.uniform(size, nx - size, n_emitters)
        y = rng.uniform(size, ny - size, n_emitters)
        z = rng.uniform(-0.4, 0.4, n_emitters)
        h = rng.uniform(3000.0, 20000.0, n_emitters)
        for i in range(n_emitters):
            px, py = x[i] - off, y[i] - off
            xi, yi = int(math.floor(px)), int(math.floor(py))
            c.translate(px - xi, py - yi, z[i])
            p = c.getPSF()
            # the pupil's first index is the image's x
            img[yi:yi + size, xi:xi + size] += h[i] * (p.real * p.real + p.imag * p.imag).T
        out["images"].append(rng.poisson(img).astype(numpy.float64))
        out["backgrounds"].append(numpy.full((ny, nx), background))
        out["truth"].append(dict(x=x, y=y, z=z, height=h))
        out["guesses"].append(dict(x=x + rng.normal(0.0, 0.3, n_emitters), y=y + rng.normal(0.0, 0.3, n_emitters),
                                   z=0.5 * z, background=numpy.full(n_emitters, background), height=0.8 * h))
    pfn.cleanup()
    return out


def multiplane_workload(n_channels=2, nx=256, ny=256, n_emitters=200, seed=31, background=20.0):
    """One multi-plane frame of 2D Gaussian emitters: plane 0 as drawn, the
    other planes through small affine maps (rotation, scale, shift) and
    wider (defocused) with less signal, Poisson noise; "finder" starting
    peaks (x, y within 0.4 px of the truth, z 0, sigma 1.5) in plane 0's
    coordinates.  maps = (xt_0toN, yt_0toN, xt_Nto0, yt_Nto0), 3
    coefficients per plane."""
    rng = numpy.random.default_rng(seed)
    x0N, y0N, xN0, yN0 = [], [], [], []
    for c in range(n_channels):
        if c == 0:
            a, t = numpy.eye(2), numpy.zeros(2)
        else:
            th = rng.uniform(-0.01, 0.01)
            s = 1.0 + rng.uniform(-0.004, 0.004)
            a = s * numpy.array([[math.cos(th), -math.sin(th)], [math.sin(th), math.cos(th)]])
            t = rng.uniform(-2.0, 2.0, 2)
        ai = numpy.linalg.inv(a)
        ti = -ai @ t
        x0N += [t[0], a[0, 0], a[0, 1]]
        y0N += [t[1], a[1, 0], a[1, 1]]
        xN0 += [ti[0], ai[0, 0], ai[0, 1]]
        yN0 += [ti[1], ai[1, 0], ai[1, 1]]
    maps = tuple(numpy.array(v) for v in (x0N, y0N, xN0, yN0))
    x = rng.uniform(14.0, nx - 14.0, n_emitters)
    y = rng.uniform(14.0, ny - 14.0, n_emitters)
    h = rng.uniform(400.0, 1500.0, n_emitters)
    yy, xx = numpy.mgrid[0:ny, 0:nx]
    images = []
    for c in range(n_channels):
        cx = maps[0][3 * c] + maps[0][3 * c + 1] * x + maps[0][3 * c + 2] * y
        cy = maps[1][3 * c] + maps[1][3 * c + 1] * x + maps[1][3 * c + 2] * y
        sig = 1.3 + 0.35 * c
        img = numpy.full((ny, nx), background)
        for i in range(n_emitters):
            x0, x1 = max(0, int(cx[i]) - 8), min(nx, int(cx[i]) + 9)
            y0, y1 = max(0, int(cy[i]) - 8), min(ny, int(cy[i]) + 9)
            img[y0:y1, x0:x1] += (h[i] / (1.0 + 0.5 * c)) * numpy.exp(
                -((xx[y0:y1, x0:x1] - cx[i]) ** 2 + (yy[y0:y1, x0:x1] - cy[i]) ** 2) / (2 * sig * sig))
        images.append(rng.poisson(img).astype(numpy.float64))
    peaks = {"x": numpy.round(x) + rng.uniform(-0.4, 0.4, n_emitters),
             "y": numpy.round(y) + rng.uniform(-0.4, 0.4, n_emitters),
             "z": numpy.zeros(n_emitters), "sigma": numpy.full(n_emitters, 1.5)}
    return {"images": images, "backgrounds": [numpy.full((ny, nx), background) for _ in range(n_channels)],
            "maps": maps, "peaks": peaks, "nx": nx, "ny": ny, "n_channels": n_channels}
