/*
 * sa_oracle.c -- CPU FP64 oracle for the multi-emitter LM fitter.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline).
 * It restates the reference's algorithm; every function names the
 * reference lines it follows.  It keeps the reference's per-pixel error
 * cache (stale / err_i / t_fi, multi_fit.c:111-195) so that it reproduces
 * the reference's results on identical inputs, including the cases in
 * which the cache is read while stale.
 *
 * Structure (our own): one fitter object holds the frame arrays, a peak
 * array and a working peak; the peak model is a switch on an enum rather
 * than a table of callbacks.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sa_oracle.h"

/* pi as the reference's M_PI (not defined under -std=c99) */
#define ORA_PI 3.14159265358979323846

/* Parameter slots (multi_fit.h:20-26). */
enum { PH = 0, PX = 1, PXW = 2, PY = 3, PYW = 4, PBG = 5, PZ = 6 };

/* Status values (multi_fit.h:33-35). */
enum { RUNNING = 0, CONVERGED = 1, ERROR = 2 };

/* LM lambda schedule (multi_fit.h:42-46). */
#define LAMBDA_START 1.0
#define LAMBDA_DOWN  0.75
#define LAMBDA_MAX   1.0e+20
#define LAMBDA_MIN   1.0e-3
#define LAMBDA_UP    4.0
#define PEAK_BLOCK   500      /* storage growth unit, multi_fit.h:49 */

/* Counter slots, in the reference's fitData order (multi_fit.h:87-94). */
enum { C_DPOSV = 0, C_ITER, C_LOST, C_MARGIN, C_NEGFI, C_NEGH, C_NONCONV, C_NONDECR };

typedef struct {
  double p[7];
  double error;
  double lambda;
  double wxt, wyt;        /* Z model: squared defocus polynomial (dao_fit.c:1021-1032) */
  int xi, yi, zi;
  int status, iterations, added;
  int xs, ys;             /* spline start offsets (cubic_fit.c:459-469) */
  double xd, yd, zd;      /* spline cell deltas */
  double *psf;            /* roi_n values */
} OPeak;

struct oraFit {
  int model, jac, nx, ny, roi, nroi;
  int *rx, *ry;
  double xoff, yoff, zoff, tol, min_height;
  double wmin, wmax, zmin, zmax, wx[5], wy[5];
  int sx, sy, sz;
  double *aij;            /* spline coefficients; ORA_FFT: the PSF spectrum (re, im);
                             ORA_PUPIL: 2 pi kx, 2 pi ky, 2 pi kz, then the pupil
                             function as pfnSetPF stores it (re, im), see pupil_eval */
  double *fft_tw;         /* ORA_FFT: twiddle tables, see fft_eval */
  double *rqe, *scmos, *x, *f, *bg, *bgest, *err, *tfi;
  int *cnt, *stale;
  OPeak *pk;
  int nfit, maxfit;
  OPeak w;
  int64_t ctr[8];
};

/* ------------------------------------------------------------------ */
/* small helpers                                                        */
/* ------------------------------------------------------------------ */

/* A peak's psf buffer holds its roi*roi shape values and, after them, the
 * Gaussian models' four ROI tables xt, ext, yt, eyt (roi values each), kept
 * with the peak as the reference's daoPeak keeps them (dao_fit.c:968-998
 * fills them, the daoCalcJH* functions read them). */
static double *shape_tabs(const oraFit *fit, const OPeak *pk)
{
  return pk->psf + (size_t)fit->roi * fit->roi;
}

static void peak_copy(const oraFit *fit, OPeak *dst, const OPeak *src)
{
  double *keep = dst->psf;
  *dst = *src;
  dst->psf = keep;
  memcpy(dst->psf, src->psf, sizeof(double) * fit->nroi);
  memcpy(shape_tabs(fit, dst), shape_tabs(fit, src), sizeof(double) * 4 * fit->roi);
}

static int is_fft(const oraFit *fit) { return fit->model == ORA_FFT; }
static int is_pupil(const oraFit *fit) { return fit->model == ORA_PUPIL; }

static int is_spline(const oraFit *fit)
{
  return (fit->model == ORA_SPLINE2D) || (fit->model == ORA_SPLINE3D);
}

/* rangeCheckD / rangeCheckI, cubic_spline.c:798-855 (silent clamps). */
static double clampd(double v, double lo, double hi)
{
  if (v < lo) v = lo;
  if (v > hi) v = hi;
  return v;
}
static int clampi(int v, int lo, int hi_excl)
{
  if (v < lo) v = lo;
  if (v >= hi_excl) v = hi_excl - 1;
  return v;
}

/* ------------------------------------------------------------------ */
/* spline evaluation (cubic_spline.c:66-138, 205-522)                   */
/* ------------------------------------------------------------------ */

/* Monomial tables for value and d/dx, d/dy, d/dz (computeDelta3D,
 * cubic_spline.c:105-138): index i*16+j*4+k <-> x^i y^j z^k. */
static void deltas3d(double zd, double yd, double xd,
                     double *df, double *ddx, double *ddy, double *ddz)
{
  int i, j, k;
  double cx, cy, cz;
  xd = clampd(xd, 0.0, 1.0);
  yd = clampd(yd, 0.0, 1.0);
  zd = clampd(zd, 0.0, 1.0);
  memset(ddx, 0, sizeof(double) * 64);
  memset(ddy, 0, sizeof(double) * 64);
  memset(ddz, 0, sizeof(double) * 64);
  cx = 1.0;
  for (i = 0; i < 4; i++) {
    cy = 1.0;
    for (j = 0; j < 4; j++) {
      cz = 1.0;
      for (k = 0; k < 4; k++) {
        df[i * 16 + j * 4 + k] = cx * cy * cz;
        if (i < 3) ddx[(i + 1) * 16 + j * 4 + k] = ((double)i + 1) * cx * cy * cz;
        if (j < 3) ddy[i * 16 + (j + 1) * 4 + k] = ((double)j + 1) * cx * cy * cz;
        if (k < 3) ddz[i * 16 + j * 4 + k + 1] = ((double)k + 1) * cx * cy * cz;
        cz = cz * zd;
      }
      cy = cy * yd;
    }
    cx = cx * xd;
  }
}

/* computeDelta2D, cubic_spline.c:66-91: index 4*i+j <-> x^i y^j. */
static void deltas2d(double yd, double xd, double *df, double *ddx, double *ddy)
{
  int i, j;
  double cx, cy;
  xd = clampd(xd, 0.0, 1.0);
  yd = clampd(yd, 0.0, 1.0);
  memset(ddx, 0, sizeof(double) * 16);
  memset(ddy, 0, sizeof(double) * 16);
  cx = 1.0;
  for (i = 0; i < 4; i++) {
    cy = 1.0;
    for (j = 0; j < 4; j++) {
      df[4 * i + j] = cx * cy;
      if (i < 3) ddx[4 * (i + 1) + j] = ((double)i + 1) * cx * cy;
      if (j < 3) ddy[4 * i + j + 1] = ((double)j + 1) * cx * cy;
      cy = cy * yd;
    }
    cx = cx * xd;
  }
}

static double dotn(const double *a, const double *b, int n)
{
  int i;
  double s = 0.0;
  for (i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/* Cell base pointer with the index clamps of fAt3D/dxfAt3D (cubic_spline.c:509-522). */
static const double *cell3d(const oraFit *fit, int zc, int yc, int xc)
{
  xc = clampi(xc, 0, fit->sx);
  yc = clampi(yc, 0, fit->sy);
  zc = clampi(zc, 0, fit->sz);
  return fit->aij + ((size_t)xc * (fit->sy * fit->sz) + (size_t)yc * fit->sz + zc) * 64;
}

static const double *cell2d(const oraFit *fit, int yc, int xc)
{
  xc = clampi(xc, 0, fit->sx);
  yc = clampi(yc, 0, fit->sy);
  return fit->aij + ((size_t)xc * fit->sy + yc) * 16;
}

double oraSplineEval3D(const double *aij, int sx, int sy, int sz,
                       double z, double y, double x, int which)
{
  double df[64], ddx[64], ddy[64], ddz[64];
  const double *c;
  int xc, yc, zc;
  x = clampd(x, 0.0, (double)sx);
  y = clampd(y, 0.0, (double)sy);
  z = clampd(z, 0.0, (double)sz);
  xc = (int)x; yc = (int)y; zc = (int)z;
  deltas3d(z - zc, y - yc, x - xc, df, ddx, ddy, ddz);
  xc = clampi(xc, 0, sx); yc = clampi(yc, 0, sy); zc = clampi(zc, 0, sz);
  c = aij + ((size_t)xc * (sy * sz) + (size_t)yc * sz + zc) * 64;
  switch (which) {
  case 1: return dotn(c, ddx, 64);
  case 2: return dotn(c, ddy, 64);
  case 3: return dotn(c, ddz, 64);
  default: return dotn(c, df, 64);
  }
}

/* ------------------------------------------------------------------ */
/* ROI geometry                                                         */
/* ------------------------------------------------------------------ */

/* Circular ROI, mFitInitializeROIIndexing multi_fit.c:1031-1060. */
static void roi_index(oraFit *fit, int roi)
{
  int i, j, n = 0;
  double c = 0.5 * (double)roi, rr = c * c, dx, dy;
  fit->roi = roi;
  fit->rx = (int *)malloc(sizeof(int) * roi * roi);
  fit->ry = (int *)malloc(sizeof(int) * roi * roi);
  for (i = 0; i < roi; i++) {
    dy = (double)i - c + 0.5;
    for (j = 0; j < roi; j++) {
      dx = (double)j - c + 0.5;
      if ((dx * dx + dy * dy) <= rr) {
        fit->rx[n] = j;
        fit->ry[n] = i;
        n++;
      }
    }
  }
  fit->nroi = n;
}

/* ------------------------------------------------------------------ */
/* model pieces                                                         */
/* ------------------------------------------------------------------ */

/* daoCalcWidthsFromZ, dao_fit.c:1009-1035 (w0 is stored squared). */
static void widths_from_z(const oraFit *fit, OPeak *pk)
{
  double z0, z1, z2, z3, t;
  z0 = (pk->p[PZ] - fit->wx[1]) / fit->wx[2];
  z1 = z0 * z0; z2 = z1 * z0; z3 = z2 * z0;
  t = 1.0 + z1 + fit->wx[3] * z2 + fit->wx[4] * z3;
  pk->wxt = t * t;
  pk->p[PXW] = 2.0 / (fit->wx[0] * t);
  z0 = (pk->p[PZ] - fit->wy[1]) / fit->wy[2];
  z1 = z0 * z0; z2 = z1 * z0; z3 = z2 * z0;
  t = 1.0 + z1 + fit->wy[3] * z2 + fit->wy[4] * z3;
  pk->wyt = t * t;
  pk->p[PYW] = 2.0 / (fit->wy[0] * t);
}

/* ORA_FFT: the translated PSF and its x, y, z derivatives on the PSF's
 * x-y grid, the middle z plane of the c2r inverse of the translated
 * spectrum (pFTTranslate psf_fft.c:372-420, pFTGetPSF :116-137,
 * pFTGetPSFdx/dy/dz :147-272).  Evaluated separably: for each (ky, kx) the
 * z sum, then for each (y, kx) the y sum, then for each (y, x) the x sum
 * with the c2r weights (1 for the DC and Nyquist bins of x, whose
 * imaginary parts the c2r drops, 2 otherwise).  Shift vectors as
 * pFTCalcShiftVector :43-60 (the z shift with -dz), derivative factors as
 * pFTCalcShiftVectorDerivative :70-84 (the spectrum times -i d). */
static void shift_vec(double dx, int size, double *re, double *im)
{
  int i;
  double t1 = -ORA_PI * 2.0 * dx / ((double)size);
  re[0] = 1.0;
  im[0] = 0.0;
  for (i = 1; i < (size / 2 + 1); i++) {
    double t2 = t1 * (double)i;
    double tr = cos(t2), tc = sin(t2);
    re[size - i] = tr;
    re[i] = tr;
    im[size - i] = -tc;
    im[i] = tc;
  }
}

static void shift_deriv(int size, double *d)
{
  int i;
  double t1 = -ORA_PI * 2.0 / ((double)size);
  d[0] = 0.0;
  for (i = 1; i < (size / 2 + 1); i++) {
    double t2 = t1 * (double)i;
    d[size - i] = t2;
    d[i] = -t2;
  }
}

/* e^{2 pi i k n / N} with k n reduced mod N first */
static void twiddle(long k, long n, long N, double *re, double *im)
{
  double a = 2.0 * ORA_PI * (double)((k * n) % N) / (double)N;
  *re = cos(a);
  *im = sin(a);
}

static void fft_eval(const oraFit *fit, double dx, double dy, double dz,
                     double *psf, double *gx, double *gy, double *gz)
{
  int nx = fit->sx, ny = fit->sy, nz = fit->sz, nk = nx / 2 + 1, zm = nz / 2;
  int kz, ky, kx, y, x;
  double *sxr = malloc(sizeof(double) * 6 * 64), *sxi = sxr + 64, *syr = sxr + 128, *syi = sxr + 192,
         *szr = sxr + 256, *szi = sxr + 320;
  double dkx[64], dky[64], dkz[64];
  double *Cr = calloc((size_t)ny * nk * 10, sizeof(double));
  double *Ci = Cr + ny * nk, *Czr = Ci + ny * nk, *Czi = Czr + ny * nk;
  double *Dr = Czi + ny * nk, *Di = Dr + ny * nk, *Dyr = Di + ny * nk, *Dyi = Dyr + ny * nk;
  double *Dzr = Dyi + ny * nk, *Dzi = Dzr + ny * nk;
  shift_vec(dx, nx, sxr, sxi);
  shift_vec(dy, ny, syr, syi);
  shift_vec(-dz, nz, szr, szi);
  shift_deriv(nx, dkx);
  shift_deriv(ny, dky);
  shift_deriv(nz, dkz);
  for (ky = 0; ky < ny; ky++) {
    for (kx = 0; kx < nk; kx++) {
      double cr = 0.0, ci = 0.0, czr = 0.0, czi = 0.0;
      for (kz = 0; kz < nz; kz++) {
        const double *w = fit->aij + 2 * (((size_t)kz * ny + ky) * nk + kx);
        double r1 = w[0], c1 = w[1], r2, c2, er, ei, pr, pi;
        /* z, y, x shifts in the reference's order */
        r2 = r1 * szr[kz] - c1 * szi[kz];
        c2 = r1 * szi[kz] + c1 * szr[kz];
        r1 = r2 * syr[ky] - c2 * syi[ky];
        c1 = r2 * syi[ky] + c2 * syr[ky];
        r2 = r1 * sxr[kx] - c1 * sxi[kx];
        c2 = r1 * sxi[kx] + c1 * sxr[kx];
        twiddle(kz, zm, nz, &er, &ei);
        pr = r2 * er - c2 * ei;
        pi = r2 * ei + c2 * er;
        cr += pr;
        ci += pi;
        /* times -i dkz: (pr, pi) -> (pi dkz, -pr dkz) */
        czr += pi * dkz[kz];
        czi -= pr * dkz[kz];
      }
      Cr[ky * nk + kx] = cr; Ci[ky * nk + kx] = ci;
      Czr[ky * nk + kx] = czr; Czi[ky * nk + kx] = czi;
    }
  }
  for (y = 0; y < ny; y++) {
    for (kx = 0; kx < nk; kx++) {
      double dr = 0.0, di = 0.0, dyr = 0.0, dyi = 0.0, dzr = 0.0, dzi = 0.0;
      for (ky = 0; ky < ny; ky++) {
        double er, ei, ar = Cr[ky * nk + kx], ai = Ci[ky * nk + kx], pr, pi;
        twiddle(ky, y, ny, &er, &ei);
        pr = ar * er - ai * ei;
        pi = ar * ei + ai * er;
        dr += pr;
        di += pi;
        dyr += pi * dky[ky];
        dyi -= pr * dky[ky];
        ar = Czr[ky * nk + kx]; ai = Czi[ky * nk + kx];
        dzr += ar * er - ai * ei;
        dzi += ar * ei + ai * er;
      }
      Dr[y * nk + kx] = dr; Di[y * nk + kx] = di;
      Dyr[y * nk + kx] = dyr; Dyi[y * nk + kx] = dyi;
      Dzr[y * nk + kx] = dzr; Dzi[y * nk + kx] = dzi;
    }
  }
  for (y = 0; y < ny; y++) {
    for (x = 0; x < nx; x++) {
      double vp = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
      for (kx = 0; kx < nk; kx++) {
        double er, ei, c = ((kx == 0) || (2 * kx == nx)) ? 1.0 : 2.0;
        double pr, pi;
        twiddle(kx, x, nx, &er, &ei);
        pr = Dr[y * nk + kx] * er - Di[y * nk + kx] * ei;
        pi = Dr[y * nk + kx] * ei + Di[y * nk + kx] * er;
        vp += c * pr;
        vx += c * pi * dkx[kx];   /* Re((pr + i pi)(-i dkx)) */
        vy += c * (Dyr[y * nk + kx] * er - Dyi[y * nk + kx] * ei);
        vz += c * (Dzr[y * nk + kx] * er - Dzi[y * nk + kx] * ei);
      }
      if (psf) psf[y * nx + x] = vp;
      if (gx) gx[y * nx + x] = vx;
      if (gy) gy[y * nx + x] = vy;
      if (gz) gz[y * nx + x] = -vz;
    }
  }
  free(Cr);
  free(sxr);
}

/* Exported for the tests of the evaluation itself. */
void oraFFTEval(const oraFit *fit, double dx, double dy, double dz, double *psf, double *gx, double *gy, double *gz)
{
  fft_eval(fit, dx, dy, dz, psf, gx, gy, gz);
}

/* ORA_PUPIL: the complex PSF of the translated pupil function and its x, y,
 * z derivatives on the pupil grid, index u * N + v with u along the pupil's
 * first index (pfnTranslate pupil_function.c:448-506, pfnGetPSF :80-98,
 * pfnGetPSFdx / dy / dz :135-203: FFTW's unnormalised backward 2D DFT of
 * the translated pupil function, times -i kx, -i ky, -i kz for the
 * derivatives, dz negated).  The DFT is evaluated directly: sums over the
 * second index, then over the first.  Any output may be NULL. */
static void pupil_eval(const oraFit *fit, double dx, double dy, double dz, double *pr, double *pc,
                       double *xr, double *xc, double *yr, double *yc, double *zr, double *zc)
{
  int n = fit->sx, m = n / 2, m1 = m + 1, i, j, k, u, v, f;
  size_t nn = (size_t)n * n;
  const double *kx = fit->aij, *ky = kx + nn, *kz = ky + nn, *pf = kz + nn;
  double *sx = malloc(sizeof(double) * 4 * n), *szt = malloc(sizeof(double) * 2 * m1 * m1);
  double *ws = malloc(sizeof(double) * 2 * nn), *in = malloc(sizeof(double) * 2 * nn);
  double *mid = malloc(sizeof(double) * 2 * nn), *tw = malloc(sizeof(double) * 2 * nn);
  double *sy = sx + 2 * n;
  double *outs[4][2];
  outs[0][0] = pr; outs[0][1] = pc;
  outs[1][0] = xr; outs[1][1] = xc;
  outs[2][0] = yr; outs[2][1] = yc;
  outs[3][0] = zr; outs[3][1] = zc;
  /* pfnTranslate: x and y multipliers from kx's first column, z over the
   * pie slice with -dz */
  for (i = 0; i < n; i++) {
    double dd = kx[(size_t)i * n] * dx;
    sx[2 * i] = cos(dd);
    sx[2 * i + 1] = -sin(dd);
    dd = kx[(size_t)i * n] * dy;
    sy[2 * i] = cos(dd);
    sy[2 * i + 1] = -sin(dd);
  }
  for (i = 0; i <= m; i++) {
    for (j = i; j <= m; j++) {
      double dd = -kz[(size_t)(m - i) * n + (m - j)] * dz;
      szt[2 * (i * m1 + j)] = cos(dd);
      szt[2 * (i * m1 + j) + 1] = -sin(dd);
      szt[2 * (j * m1 + i)] = szt[2 * (i * m1 + j)];
      szt[2 * (j * m1 + i) + 1] = szt[2 * (i * m1 + j) + 1];
    }
  }
  for (i = 0; i < n; i++) {
    for (j = 0; j < n; j++) {
      size_t l = (size_t)i * n + j;
      int o = abs(i - m) * m1 + abs(j - m);
      double r2 = sx[2 * i] * sy[2 * j] - sx[2 * i + 1] * sy[2 * j + 1];
      double c2 = sx[2 * i] * sy[2 * j + 1] + sx[2 * i + 1] * sy[2 * j];
      double r1 = r2 * szt[2 * o] - c2 * szt[2 * o + 1];
      double c1 = r2 * szt[2 * o + 1] + c2 * szt[2 * o];
      ws[2 * l] = r1 * pf[2 * l] - c1 * pf[2 * l + 1];
      ws[2 * l + 1] = r1 * pf[2 * l + 1] + c1 * pf[2 * l];
    }
  }
  for (u = 0; u < n; u++) {
    for (v = 0; v < n; v++) {
      double a = 2.0 * ORA_PI * (double)(((long)u * v) % n) / (double)n;
      tw[2 * ((size_t)u * n + v)] = cos(a);
      tw[2 * ((size_t)u * n + v) + 1] = sin(a);
    }
  }
  for (f = 0; f < 4; f++) {
    const double *km = (f == 1) ? kx : ((f == 2) ? ky : kz);
    if (!outs[f][0] && !outs[f][1]) continue;
    for (i = 0; i < (int)nn; i++) {
      if (f == 0) {
        in[2 * i] = ws[2 * i];
        in[2 * i + 1] = ws[2 * i + 1];
      } else {
        in[2 * i] = ws[2 * i + 1] * km[i];
        in[2 * i + 1] = -ws[2 * i] * km[i];
      }
    }
    for (i = 0; i < n; i++) {
      for (v = 0; v < n; v++) {
        double sr = 0.0, si = 0.0;
        for (k = 0; k < n; k++) {
          const double *a = in + 2 * ((size_t)i * n + k), *t = tw + 2 * ((size_t)k * n + v);
          sr += a[0] * t[0] - a[1] * t[1];
          si += a[0] * t[1] + a[1] * t[0];
        }
        mid[2 * ((size_t)i * n + v)] = sr;
        mid[2 * ((size_t)i * n + v) + 1] = si;
      }
    }
    for (u = 0; u < n; u++) {
      for (v = 0; v < n; v++) {
        double sr = 0.0, si = 0.0, sg = (f == 3) ? -1.0 : 1.0;
        for (i = 0; i < n; i++) {
          const double *a = mid + 2 * ((size_t)i * n + v), *t = tw + 2 * ((size_t)i * n + u);
          sr += a[0] * t[0] - a[1] * t[1];
          si += a[0] * t[1] + a[1] * t[0];
        }
        if (outs[f][0]) outs[f][0][(size_t)u * n + v] = sg * sr;
        if (outs[f][1]) outs[f][1][(size_t)u * n + v] = sg * si;
      }
    }
  }
  free(sx); free(szt); free(ws); free(in); free(mid); free(tw);
}

/* Exported for the tests of the evaluation itself. */
void oraPupilEval(const oraFit *fit, double dx, double dy, double dz, double *pr, double *pc, double *xr,
                  double *xc, double *yr, double *yc, double *zr, double *zc)
{
  pupil_eval(fit, dx, dy, dz, pr, pc, xr, xc, yr, yc, zr, zc);
}

/* Peak shape into pk->psf: daoCalcPeakShape dao_fit.c:968-998 (note the
 * y offset also uses xoff, :979), cfCalcPeakShape cubic_fit.c:435-502. */
static void peak_shape(const oraFit *fit, OPeak *pk)
{
  int i;
  if (is_pupil(fit)) {
    /* pfitCalcPeakShape pupil_fit.c:133-170: |psf|^2 at psf[roi_x * N + roi_y] */
    size_t ng = (size_t)fit->sx * fit->sx;
    double *gr = malloc(sizeof(double) * 2 * ng), *gc = gr + ng;
    pupil_eval(fit, pk->p[PX] - (double)pk->xi, pk->p[PY] - (double)pk->yi, pk->p[PZ], gr, gc, NULL, NULL, NULL,
               NULL, NULL, NULL);
    for (i = 0; i < fit->nroi; i++) {
      size_t g = (size_t)fit->rx[i] * fit->sx + fit->ry[i];
      pk->psf[i] = gr[g] * gr[g] + gc[g] * gc[g];
    }
    free(gr);
    return;
  }
  if (is_fft(fit)) {
    /* ftFitCalcPeakShape fft_fit.c:127-155 */
    double *grid = malloc(sizeof(double) * fit->sx * fit->sy);
    fft_eval(fit, pk->p[PX] - (double)pk->xi, pk->p[PY] - (double)pk->yi, pk->p[PZ], grid, NULL, NULL, NULL);
    for (i = 0; i < fit->nroi; i++) pk->psf[i] = grid[fit->ry[i] * fit->sx + fit->rx[i]];
    free(grid);
    return;
  }
  if (!is_spline(fit)) {
    double *xt = shape_tabs(fit, pk), *ext = xt + fit->roi, *yt = xt + 2 * fit->roi, *eyt = xt + 3 * fit->roi;
    double xo, yo;
    xo = -(pk->p[PX] - (double)pk->xi) - fit->xoff;
    yo = -(pk->p[PY] - (double)pk->yi) - fit->xoff;
    for (i = 0; i < fit->roi; i++) {
      xt[i] = (double)i + xo;
      ext[i] = exp(-xt[i] * xt[i] * pk->p[PXW]);
      yt[i] = (double)i + yo;
      eyt[i] = exp(-yt[i] * yt[i] * pk->p[PYW]);
    }
    for (i = 0; i < fit->nroi; i++) pk->psf[i] = eyt[fit->ry[i]] * ext[fit->rx[i]];
  } else {
    double xd = 1.5 - (pk->p[PX] - pk->xi);
    double yd = 1.5 - (pk->p[PY] - pk->yi);
    double zd = pk->p[PZ] - pk->zi;
    pk->xs = 0;
    if (xd >= 1.0) { xd -= 1.0; pk->xs = 1; }
    pk->ys = 0;
    if (yd >= 1.0) { yd -= 1.0; pk->ys = 1; }
    pk->xd = xd; pk->yd = yd; pk->zd = zd;
    if (fit->model == ORA_SPLINE3D) {
      double df[64], a[64], b[64], c[64];
      deltas3d(zd, yd, xd, df, a, b, c);
      for (i = 0; i < fit->nroi; i++)
        pk->psf[i] = dotn(cell3d(fit, pk->zi, fit->ry[i] + pk->ys, fit->rx[i] + pk->xs), df, 64);
    } else {
      double df[16], a[16], b[16];
      deltas2d(yd, xd, df, a, b);
      for (i = 0; i < fit->nroi; i++)
        pk->psf[i] = dotn(cell2d(fit, fit->ry[i] + pk->ys, fit->rx[i] + pk->xs), df, 16);
    }
  }
}

/* Image offset of the peak's ROI origin. */
static size_t roi_base(const oraFit *fit, const OPeak *pk)
{
  return (size_t)pk->yi * fit->nx + pk->xi;
}

/* mFitAddPeak multi_fit.c:28-57 / mFitSubtractPeak :1894-1922. */
static void add_peak(oraFit *fit, OPeak *pk, int sign)
{
  int j;
  size_t b = roi_base(fit, pk), k;
  double h = pk->p[PH], bgv = pk->p[PBG], r;
  pk->added += sign;
  for (j = 0; j < fit->nroi; j++) {
    k = (size_t)fit->ry[j] * fit->nx + fit->rx[j] + b;
    r = fit->rqe[k];
    if (sign > 0) {
      fit->f[k] += h * pk->psf[j] * r;
      fit->cnt[k] += 1;
      fit->bg[k] += bgv * r + fit->scmos[k];
    } else {
      fit->f[k] -= h * pk->psf[j] * r;
      fit->cnt[k] -= 1;
      fit->bg[k] -= (bgv * r + fit->scmos[k]);
    }
    fit->stale[k] = 1;
  }
}

/* MLE error with the stale-pixel cache, mFitCalcErr multi_fit.c:111-195.
 * Returns 1 (and leaves pk->error unchanged) if fi <= 0 is met. */
static int calc_err(oraFit *fit, OPeak *pk)
{
  int j;
  size_t b, k;
  double e = 0.0, fi, xi;
  if (pk->status != RUNNING) return 0;
  b = roi_base(fit, pk);
  for (j = 0; j < fit->nroi; j++) {
    k = (size_t)fit->ry[j] * fit->nx + fit->rx[j] + b;
    if (fit->stale[k] != 0) {
      fi = fit->f[k] + fit->bg[k] / ((double)fit->cnt[k]);
      if (fi <= 0.0) {
        fit->ctr[C_NEGFI]++;
        return 1;
      }
      fit->tfi[k] = fi;
      xi = fit->x[k];
      fit->err[k] = 2.0 * ((fi - xi) - xi * log(fi / xi));
      fit->stale[k] = 0;
    }
    e += fit->err[k];
  }
  pk->error = e;
  return 0;
}

/* Jacobian (b) and upper-triangle Hessian (A) for the MLE model:
 * daoCalcJH2DFixed dao_fit.c:48-105, daoCalcJH2D :409-467,
 * daoCalcJH3D :811-871, daoCalcJHZ :883-958, cfCalcJH2D cubic_fit.c:48-108,
 * cfCalcJH3D :120-182.  Per pixel: t1 = 2(1 - x/f), t2 = 2x/f^2,
 * b += t1*jt, A(l,m>=l) += t2*jt_l*jt_m. */
static void calc_jh(const oraFit *fit, const OPeak *pk, double *jac, double *hes)
{
  int n = fit->jac, j, l, m;
  size_t b = roi_base(fit, pk), k;
  double jt[7], fi, xi, rq, t1, t2, h = pk->p[PH];
  const double *xt = shape_tabs(fit, pk), *ext = xt + fit->roi, *yt = xt + 2 * fit->roi, *eyt = xt + 3 * fit->roi;
  double gx = 0.0, gy = 0.0;
  double df3[64], dx3[64], dy3[64], dz3[64];
  double df2[16], dx2[16], dy2[16];

  double *fg = NULL;   /* ORA_FFT: x, y, z derivative grids */

  for (l = 0; l < n; l++) jac[l] = 0.0;
  for (l = 0; l < n * n; l++) hes[l] = 0.0;

  if (is_pupil(fit)) {
    /* pfitCalcJH3D pupil_fit.c:45-123: translate, then the derivatives */
    size_t ng = (size_t)fit->sx * fit->sx;
    fg = malloc(sizeof(double) * 8 * ng);
    pupil_eval(fit, pk->p[PX] - (double)pk->xi, pk->p[PY] - (double)pk->yi, pk->p[PZ], fg, fg + ng, fg + 2 * ng,
               fg + 3 * ng, fg + 4 * ng, fg + 5 * ng, fg + 6 * ng, fg + 7 * ng);
  } else if (is_fft(fit)) {
    /* ftFitCalcJH3D fft_fit.c:43-117: translate, then the derivatives */
    size_t ng = (size_t)fit->sx * fit->sy;
    fg = malloc(sizeof(double) * 3 * ng);
    fft_eval(fit, pk->p[PX] - (double)pk->xi, pk->p[PY] - (double)pk->yi, pk->p[PZ], NULL, fg, fg + ng,
             fg + 2 * ng);
  } else if (!is_spline(fit)) {
    /* the shape tables of the peak's current state (peak_shape) */
    if (fit->model == ORA_Z) {
      /* d width / d z terms, dao_fit.c:904-916. */
      double z0, z1, z2, zt;
      z0 = (pk->p[PZ] - fit->wx[1]) / fit->wx[2];
      z1 = z0 * z0; z2 = z1 * z0;
      zt = 2.0 * z0 + 3.0 * fit->wx[3] * z1 + 4.0 * fit->wx[4] * z2;
      gx = -2.0 * zt / (fit->wx[0] * pk->wxt);
      z0 = (pk->p[PZ] - fit->wy[1]) / fit->wy[2];
      z1 = z0 * z0; z2 = z1 * z0;
      zt = 2.0 * z0 + 3.0 * fit->wy[3] * z1 + 4.0 * fit->wy[4] * z2;
      gy = -2.0 * zt / (fit->wy[0] * pk->wyt);
    }
  } else if (fit->model == ORA_SPLINE3D) {
    deltas3d(pk->zd, pk->yd, pk->xd, df3, dx3, dy3, dz3);
  } else {
    deltas2d(pk->yd, pk->xd, df2, dx2, dy2);
  }

  for (j = 0; j < fit->nroi; j++) {
    int ry = fit->ry[j], rx = fit->rx[j];
    k = (size_t)ry * fit->nx + rx + b;
    fi = fit->tfi[k];
    rq = fit->rqe[k];
    xi = fit->x[k];
    switch (fit->model) {
    case ORA_2DFIXED: {
      double e_t = ext[rx] * eyt[ry], w = pk->p[PXW];
      jt[0] = rq * e_t;
      jt[1] = rq * 2.0 * h * w * xt[rx] * e_t;
      jt[2] = rq * 2.0 * h * w * yt[ry] * e_t;
      jt[3] = rq;
      break;
    }
    case ORA_2D: {
      double e_t = ext[rx] * eyt[ry], w = pk->p[PXW];
      jt[0] = rq * e_t;
      jt[1] = rq * 2.0 * h * w * xt[rx] * e_t;
      jt[2] = rq * 2.0 * h * w * yt[ry] * e_t;
      jt[3] = rq * (-h * xt[rx] * xt[rx] * e_t - h * yt[ry] * yt[ry] * e_t);
      jt[4] = rq;
      break;
    }
    case ORA_3D: {
      double e_t = ext[rx] * eyt[ry];
      jt[0] = rq * e_t;
      jt[1] = rq * 2.0 * h * pk->p[PXW] * xt[rx] * e_t;
      jt[2] = rq * (-h * xt[rx] * xt[rx] * e_t);
      jt[3] = rq * 2.0 * h * pk->p[PYW] * yt[ry] * e_t;
      jt[4] = rq * (-h * yt[ry] * yt[ry] * e_t);
      jt[5] = rq;
      break;
    }
    case ORA_Z: {
      double e_t = ext[rx] * eyt[ry];
      jt[0] = rq * e_t;
      jt[1] = rq * 2.0 * h * pk->p[PXW] * xt[rx] * e_t;
      jt[2] = rq * 2.0 * h * pk->p[PYW] * yt[ry] * e_t;
      jt[3] = rq * (-h * xt[rx] * xt[rx] * gx * e_t - h * yt[ry] * yt[ry] * gy * e_t);
      jt[4] = rq;
      break;
    }
    case ORA_FFT: {
      size_t ng = (size_t)fit->sx * fit->sy, g = (size_t)ry * fit->sx + rx;
      jt[0] = rq * pk->psf[j];
      jt[1] = rq * h * fg[g];
      jt[2] = rq * h * fg[ng + g];
      jt[3] = rq * h * fg[2 * ng + g];
      jt[4] = rq;
      break;
    }
    case ORA_PUPIL: {
      /* pupil_fit.c:103-107 */
      size_t ng = (size_t)fit->sx * fit->sx, g = (size_t)rx * fit->sx + ry;
      double ar = fg[g], ac = fg[ng + g];
      jt[0] = rq * (ar * ar + ac * ac);
      jt[1] = rq * 2.0 * h * (ar * fg[2 * ng + g] + ac * fg[3 * ng + g]);
      jt[2] = rq * 2.0 * h * (ar * fg[4 * ng + g] + ac * fg[5 * ng + g]);
      jt[3] = rq * 2.0 * h * (ar * fg[6 * ng + g] + ac * fg[7 * ng + g]);
      jt[4] = rq;
      break;
    }
    case ORA_SPLINE3D: {
      const double *c = cell3d(fit, pk->zi, ry + pk->ys, rx + pk->xs);
      jt[0] = rq * pk->psf[j];
      jt[1] = -rq * h * dotn(c, dx3, 64);
      jt[2] = -rq * h * dotn(c, dy3, 64);
      jt[3] = rq * h * dotn(c, dz3, 64);
      jt[4] = rq;
      break;
    }
    default: { /* ORA_SPLINE2D */
      const double *c = cell2d(fit, ry + pk->ys, rx + pk->xs);
      jt[0] = rq * pk->psf[j];
      jt[1] = -rq * h * dotn(c, dx2, 16);
      jt[2] = -rq * h * dotn(c, dy2, 16);
      jt[3] = rq;
      break;
    }
    }
    t1 = 2.0 * (1.0 - xi / fi);
    for (l = 0; l < n; l++) jac[l] += t1 * jt[l];
    t2 = 2.0 * xi / (fi * fi);
    for (l = 0; l < n; l++)
      for (m = l; m < n; m++) hes[l * n + m] += t2 * jt[l] * jt[m];
  }
  free(fg);
}

/* Parameter update from the solved step, in each model's delta order:
 * daoUpdate2DFixed dao_fit.c:1777-1792, daoUpdate2D :1801-1816,
 * daoUpdate3D :1826-1842, daoUpdateZ :1851-1880, cfUpdate2D
 * cubic_fit.c:939-952, cfUpdate3D :962-978 with cfZRangeCheck :987-1005;
 * the ROI re-anchor is mFitUpdate multi_fit.c:1933-1946. */
static void anchor_update(OPeak *pk)
{
  double dx = pk->p[PX] - pk->xi, dy;
  if ((dx < -0.5) || (dx > 1.5)) pk->xi = (int)floor(pk->p[PX]);
  dy = pk->p[PY] - pk->yi;
  if ((dy < -0.5) || (dy > 1.5)) pk->yi = (int)floor(pk->p[PY]);
}

static void apply_update(const oraFit *fit, OPeak *pk, const double *d)
{
  switch (fit->model) {
  case ORA_2DFIXED:
  case ORA_SPLINE2D:
    pk->p[PH] -= d[0]; pk->p[PX] -= d[1]; pk->p[PY] -= d[2]; pk->p[PBG] -= d[3];
    anchor_update(pk);
    break;
  case ORA_2D:
    pk->p[PH] -= d[0]; pk->p[PX] -= d[1]; pk->p[PY] -= d[2]; pk->p[PXW] -= d[3]; pk->p[PBG] -= d[4];
    pk->p[PYW] = pk->p[PXW];
    anchor_update(pk);
    break;
  case ORA_3D:
    pk->p[PH] -= d[0]; pk->p[PX] -= d[1]; pk->p[PXW] -= d[2]; pk->p[PY] -= d[3]; pk->p[PYW] -= d[4];
    pk->p[PBG] -= d[5];
    anchor_update(pk);
    break;
  case ORA_Z:
    pk->p[PH] -= d[0]; pk->p[PX] -= d[1]; pk->p[PY] -= d[2]; pk->p[PZ] -= d[3]; pk->p[PBG] -= d[4];
    if (pk->p[PZ] < fit->zmin) pk->p[PZ] = fit->zmin;
    if (pk->p[PZ] > fit->zmax) pk->p[PZ] = fit->zmax;
    anchor_update(pk);
    widths_from_z(fit, pk);
    break;
  case ORA_FFT: {
    /* ftFitUpdate3D fft_fit.c:481-497, ftFitZRangeCheck :506-524 */
    double max_z = ((double)fit->sz) * 0.5 - 1.0e-12;
    pk->p[PH] -= d[0]; pk->p[PX] -= d[1]; pk->p[PY] -= d[2]; pk->p[PZ] -= d[3]; pk->p[PBG] -= d[4];
    anchor_update(pk);
    if (pk->p[PZ] < -max_z) pk->p[PZ] = -max_z;
    if (pk->p[PZ] > max_z) pk->p[PZ] = max_z;
    break;
  }
  case ORA_PUPIL:
    /* pfitUpdate3D pupil_fit.c:529-546, pfitZRangeCheck :555-570 */
    pk->p[PH] -= d[0]; pk->p[PX] -= d[1]; pk->p[PY] -= d[2]; pk->p[PZ] -= d[3]; pk->p[PBG] -= d[4];
    anchor_update(pk);
    if (pk->p[PZ] < fit->zmin) pk->p[PZ] = fit->zmin;
    if (pk->p[PZ] > fit->zmax) pk->p[PZ] = fit->zmax;
    break;
  default: { /* ORA_SPLINE3D */
    double zmax;
    pk->p[PH] -= d[0]; pk->p[PX] -= d[1]; pk->p[PY] -= d[2]; pk->p[PZ] -= d[3]; pk->p[PBG] -= d[4];
    anchor_update(pk);
    if (pk->p[PZ] < 1.0e-12) pk->p[PZ] = 1.0e-12;
    zmax = ((double)fit->sz) - 1.0e-12;
    if (pk->p[PZ] > zmax) pk->p[PZ] = zmax;
    pk->zi = (int)(pk->p[PZ]);
    break;
  }
  }
}

/* mFitCheck multi_fit.c:470-502 (margin and negative height). */
static int base_check(oraFit *fit, OPeak *pk)
{
  if ((pk->xi < 0) || (pk->xi >= (fit->nx - fit->roi)) ||
      (pk->yi < 0) || (pk->yi >= (fit->ny - fit->roi))) {
    fit->ctr[C_MARGIN]++;
    return 1;
  }
  if (pk->p[PH] < 0.0) {
    fit->ctr[C_NEGH]++;
    return 1;
  }
  return 0;
}

/* Model check: daoCheck2D dao_fit.c:1061-1088 (clamps XWIDTH only),
 * daoCheck3D :1100-1119 (and YWIDTH); the rest use mFitCheck. */
static int model_check(oraFit *fit, OPeak *pk)
{
  if (base_check(fit, pk)) return 1;
  if ((fit->model == ORA_2D) || (fit->model == ORA_3D)) {
    if (pk->p[PXW] < fit->wmin) pk->p[PXW] = fit->wmin;
    else if (pk->p[PXW] > fit->wmax) pk->p[PXW] = fit->wmax;
  }
  if (fit->model == ORA_3D) {
    if (pk->p[PYW] < fit->wmin) pk->p[PYW] = fit->wmin;
    else if (pk->p[PYW] > fit->wmax) pk->p[PYW] = fit->wmax;
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* Cholesky solve (stands in for LAPACK dposv, multi_fit.c:1839-1883)   */
/* ------------------------------------------------------------------ */

int oraSolve(double *a, double *b, int n)
{
  /* a: row-major upper triangle a[i*n+j], j >= i (read as the lower
   * triangle of the column-major matrix, as dposv("Lower") does). */
  double L[49];
  int i, j, k;
  for (j = 0; j < n; j++) {
    double d = a[j * n + j];
    for (k = 0; k < j; k++) d -= L[j * 7 + k] * L[j * 7 + k];
    if (!(d > 0.0)) return j + 1;   /* not positive definite (or NaN) */
    d = sqrt(d);
    L[j * 7 + j] = d;
    for (i = j + 1; i < n; i++) {
      double s = a[j * n + i];
      for (k = 0; k < j; k++) s -= L[i * 7 + k] * L[j * 7 + k];
      L[i * 7 + j] = s / d;
    }
  }
  for (i = 0; i < n; i++) {
    double s = b[i];
    for (k = 0; k < i; k++) s -= L[i * 7 + k] * b[k];
    b[i] = s / L[i * 7 + i];
  }
  for (i = n - 1; i >= 0; i--) {
    double s = b[i];
    for (k = i + 1; k < n; k++) s -= L[k * 7 + i] * b[k];
    b[i] = s / L[i * 7 + i];
  }
  for (i = 0; i < n; i++)
    if (isnan(b[i])) return 1;
  return 0;
}

/* ------------------------------------------------------------------ */
/* public API                                                           */
/* ------------------------------------------------------------------ */

oraFit *oraCreate(int model, const double *rqe, const double *scmos, double tol,
                  int nx, int ny, int roi_size,
                  double wmin, double wmax,
                  const double *wx, const double *wy, double zmin, double zmax,
                  const double *aij, int sx, int sy, int sz)
{
  oraFit *fit = (oraFit *)calloc(1, sizeof(oraFit));
  size_t np = (size_t)nx * ny, i;
  fit->model = model;
  fit->nx = nx;
  fit->ny = ny;
  fit->tol = tol;
  fit->min_height = -1.0;          /* multi_fit.c:965 */
  fit->rqe = (double *)malloc(sizeof(double) * np);
  fit->scmos = (double *)malloc(sizeof(double) * np);
  fit->x = (double *)calloc(np, sizeof(double));
  fit->f = (double *)calloc(np, sizeof(double));
  fit->bg = (double *)calloc(np, sizeof(double));
  fit->bgest = (double *)calloc(np, sizeof(double));
  fit->err = (double *)calloc(np, sizeof(double));
  fit->tfi = (double *)calloc(np, sizeof(double));
  fit->cnt = (int *)calloc(np, sizeof(int));
  fit->stale = (int *)calloc(np, sizeof(int));
  for (i = 0; i < np; i++) {
    fit->rqe[i] = rqe[i];
    fit->scmos[i] = scmos[i];
  }
  switch (model) {
  case ORA_2DFIXED: fit->jac = 4; break;
  case ORA_2D: fit->jac = 5; break;
  case ORA_3D: fit->jac = 6; break;
  case ORA_Z: fit->jac = 5; break;
  case ORA_SPLINE2D: fit->jac = 4; break;
  default: fit->jac = 5; break;
  }
  if (is_pupil(fit)) {
    /* pfitInitialize pupil_fit.c:288-332 with pfnInitialize / pfnSetPF
     * pupil_function.c:321-410: aij holds kx, ky, kz and the pupil
     * function's real and imaginary parts (sx x sx each); ROI = sx,
     * xoff = yoff = sx / 2 */
    size_t nn = (size_t)sx * sx, l;
    int a, b;
    fit->sx = sx; fit->sy = sx; fit->sz = 0;
    fit->aij = (double *)malloc(sizeof(double) * 5 * nn);
    for (l = 0; l < 3 * nn; l++) fit->aij[l] = 2.0 * ORA_PI * aij[l];
    for (a = 0; a < sx; a++) {
      for (b = 0; b < sx; b++) {
        double sg = (((a + b) % 2) == 0) ? 1.0 : -1.0, nrm = 1.0 / ((double)sx);
        l = (size_t)a * sx + b;
        fit->aij[3 * nn + 2 * l] = sg * aij[3 * nn + l] * nrm;
        fit->aij[3 * nn + 2 * l + 1] = sg * aij[4 * nn + l] * nrm;
      }
    }
    fit->xoff = 0.5 * ((double)sx);
    fit->yoff = 0.5 * ((double)sx);
    fit->zmin = zmin;
    fit->zmax = zmax;
    roi_index(fit, sx);
  } else if (is_fft(fit)) {
    /* ftFitInitialize fft_fit.c:254-310: ROI = PSF x size */
    size_t nc = (size_t)sz * sy * (sx / 2 + 1) * 2;
    fit->sx = sx; fit->sy = sy; fit->sz = sz;
    fit->aij = (double *)malloc(sizeof(double) * nc);
    memcpy(fit->aij, aij, sizeof(double) * nc);
    fit->xoff = 0.5 * ((double)sx) - 1.0;
    fit->yoff = 0.5 * ((double)sy) - 1.0;
    roi_index(fit, sx);
  } else if (!is_spline(fit)) {
    /* daoInitialize dao_fit.c:1251-1309 */
    roi_index(fit, roi_size);
    fit->xoff = 0.5 * ((double)roi_size) - 1.0;
    fit->yoff = fit->xoff;
    fit->wmin = wmin;
    fit->wmax = wmax;
    if (model == ORA_Z) {
      /* daoInitializeZ dao_fit.c:1545-1571: w0 squared. */
      for (i = 0; i < 5; i++) { fit->wx[i] = wx[i]; fit->wy[i] = wy[i]; }
      fit->wx[0] = fit->wx[0] * fit->wx[0];
      fit->wy[0] = fit->wy[0] * fit->wy[0];
      fit->zmin = zmin;
      fit->zmax = zmax;
    }
  } else {
    /* cfInitialize cubic_fit.c:602-664: ROI = spline size - 1. */
    size_t nc = (model == ORA_SPLINE3D) ? (size_t)sx * sy * sz * 64 : (size_t)sx * sy * 16;
    int s = sx - 1;
    fit->sx = sx; fit->sy = sy; fit->sz = (model == ORA_SPLINE3D) ? sz : 0;
    fit->aij = (double *)malloc(sizeof(double) * nc);
    memcpy(fit->aij, aij, sizeof(double) * nc);
    if ((s % 2) == 1) {
      fit->xoff = (double)(s / 2) - 0.5;
      fit->yoff = (double)((sy - 1) / 2) - 0.5;
    } else {
      fit->xoff = (double)(s / 2) - 1.0;
      fit->yoff = (double)((sy - 1) / 2) - 1.0;
    }
    roi_index(fit, s);
  }
  fit->w.psf = (double *)malloc(sizeof(double) * (fit->roi * fit->roi + 4 * fit->roi));
  return fit;
}

void oraDestroy(oraFit *fit)
{
  int i;
  if (fit == NULL) return;
  for (i = 0; i < fit->maxfit; i++) free(fit->pk[i].psf);
  free(fit->pk);
  free(fit->w.psf);
  free(fit->rx); free(fit->ry);
  free(fit->aij);
  free(fit->rqe); free(fit->scmos); free(fit->x); free(fit->f); free(fit->bg);
  free(fit->bgest); free(fit->err); free(fit->tfi); free(fit->cnt); free(fit->stale);
  free(fit);
}

/* mFitNewImage multi_fit.c:1382-1408. */
void oraNewImage(oraFit *fit, const double *image)
{
  size_t i, np = (size_t)fit->nx * fit->ny;
  for (i = 0; i < np; i++) fit->x[i] = image[i] * fit->rqe[i] + fit->scmos[i];
  for (i = 0; i < np; i++) {
    fit->cnt[i] = 0;
    fit->bg[i] = 0.0;
    fit->err[i] = 0.0;
    fit->f[i] = 0.0;
    fit->stale[i] = 1;
  }
  fit->nfit = 0;
}

/* mFitNewBackground multi_fit.c:1360-1370. */
void oraNewBackground(oraFit *fit, const double *background)
{
  size_t i, np = (size_t)fit->nx * fit->ny;
  for (i = 0; i < np; i++) {
    fit->bgest[i] = background[i] * fit->rqe[i];
    fit->stale[i] = 1;
  }
}

/* mFitEstimatePeakBackground multi_fit.c:638-662. */
static void estimate_bg(oraFit *fit, OPeak *pk)
{
  int j;
  size_t b = roi_base(fit, pk), k;
  double t = 0.0;
  for (j = 0; j < fit->nroi; j++) {
    k = (size_t)fit->ry[j] * fit->nx + fit->rx[j] + b;
    t += fit->bgest[k] / fit->rqe[k];
  }
  pk->p[PBG] = t / ((double)fit->nroi);
}

/* mFitEstimatePeakHeight multi_fit.c:678-700. */
static void estimate_height(oraFit *fit, OPeak *pk)
{
  int j;
  size_t b = roi_base(fit, pk), k;
  double sp = 0.0, sxv = 0.0, t;
  for (j = 0; j < fit->nroi; j++) {
    k = (size_t)fit->ry[j] * fit->nx + fit->rx[j] + b;
    t = pk->psf[j] * fit->rqe[k];
    sp += t * t * t;
    sxv += t * t * (fit->x[k] - fit->f[k] - fit->bgest[k]);
  }
  pk->p[PH] = sxv / sp;
}

/* Storage growth with ERROR compaction, mFitNewPeaks multi_fit.c:1419-1499. */
static void grow_peaks(oraFit *fit, int n_new)
{
  int i, j, n_alloc;
  OPeak *np;
  if ((fit->nfit + n_new) <= fit->maxfit) return;
  n_alloc = PEAK_BLOCK * ((fit->nfit + n_new) / PEAK_BLOCK + 1);
  np = (OPeak *)calloc(n_alloc, sizeof(OPeak));
  for (j = 0; j < n_alloc; j++) np[j].psf = (double *)calloc(fit->roi * fit->roi + 4 * fit->roi, sizeof(double));
  i = 0;
  for (j = 0; j < fit->nfit; j++) {
    if (fit->pk[j].status != ERROR) {
      peak_copy(fit, &np[i], &fit->pk[j]);
      i++;
    }
  }
  for (j = 0; j < fit->maxfit; j++) free(fit->pk[j].psf);
  free(fit->pk);
  fit->pk = np;
  fit->maxfit = n_alloc;
  fit->nfit = i;
}

/* daoNewPeaks dao_fit.c:1582-1766 and cfNewPeaks cubic_fit.c:758-928. */
void oraNewPeaks(oraFit *fit, const double *peaks, int ptype, int n_peaks)
{
  /* arbitrary-PSF input formats (x, y, z [, background, height]) for the
   * splines and the FFT PSF (cubic_fit.c:776-914, fft_fit.c:318-470) */
  int i, start, stop, spline = is_spline(fit) || is_fft(fit) || is_pupil(fit);
  int ncol;
  grow_peaks(fit, n_peaks);
  start = fit->nfit;
  stop = fit->nfit + n_peaks;
  for (i = start; i < stop; i++) {
    OPeak *pk = &fit->pk[i];
    pk->added = 0;
    pk->iterations = 0;
    pk->status = RUNNING;
    pk->error = 0.0;
    pk->lambda = LAMBDA_START;
  }
  if (ptype == ORA_PEAKS_TEXT) ncol = spline ? 5 : 7;
  else ncol = spline ? 3 : 4;

  for (i = start; i < stop; i++) {
    const double *q = peaks + (size_t)ncol * (i - start);
    OPeak *pk = &fit->pk[i];
    pk->p[PX] = q[0] - fit->xoff;
    pk->p[PY] = q[1] - fit->yoff;
    pk->p[PZ] = q[2] - fit->zoff;
    if (ptype == ORA_PEAKS_TEXT) {
      pk->p[PBG] = q[3];
      pk->p[PH] = q[4];
      if (!spline) {
        pk->p[PXW] = 1.0 / (2.0 * q[5] * q[5]);
        pk->p[PYW] = 1.0 / (2.0 * q[6] * q[6]);
        if (fit->model == ORA_Z) widths_from_z(fit, pk);
      }
    } else {
      if (!spline) {
        if (fit->model == ORA_Z) {
          widths_from_z(fit, pk);
        } else {
          double w = 1.0 / (2.0 * q[3] * q[3]);
          pk->p[PXW] = w;
          pk->p[PYW] = w;
        }
      }
    }
    pk->xi = (int)floor(pk->p[PX]);
    pk->yi = (int)floor(pk->p[PY]);
    if (is_spline(fit)) pk->zi = (int)pk->p[PZ];
    if (ptype != ORA_PEAKS_TEXT) {
      pk->p[PBG] = 1.0;
      pk->p[PH] = 1.0;
    }
    peak_copy(fit, &fit->w, pk);
    /* Spline models use mFitCheck as fn_check (cubic_fit.c:660). */
    if (spline ? base_check(fit, &fit->w) : model_check(fit, &fit->w)) {
      fit->w.status = ERROR;
      peak_copy(fit, pk, &fit->w);
      continue;
    }
    peak_shape(fit, &fit->w);
    if (ptype != ORA_PEAKS_TEXT) {
      estimate_bg(fit, &fit->w);
      if (ptype == ORA_PEAKS_FINDER) {
        estimate_height(fit, &fit->w);
        if (fit->w.p[PH] < fit->min_height) fit->w.p[PH] = fit->min_height;
        if (fit->w.p[PH] <= 0.0) {
          fit->w.status = ERROR;
          peak_copy(fit, pk, &fit->w);
          continue;
        }
      }
    }
    add_peak(fit, &fit->w, +1);
    peak_copy(fit, pk, &fit->w);
  }
  /* Initial error of the new peaks (dao_fit.c:1757-1763). */
  for (i = start; i < stop; i++) {
    peak_copy(fit, &fit->w, &fit->pk[i]);
    calc_err(fit, &fit->w);
    peak_copy(fit, &fit->pk[i], &fit->w);
  }
  fit->nfit = stop;
}

/* Restore the working peak from the stored one, keeping 'added' and
 * raising lambda; mFitResetPeak multi_fit.c:1788-1798. */
static void reset_working(oraFit *fit, int i)
{
  int added = fit->w.added;
  double lam = fit->w.lambda;
  peak_copy(fit, &fit->w, &fit->pk[i]);
  fit->w.added = added;
  fit->w.lambda = lam * LAMBDA_UP;
}

/* mFitRecenterPeaks multi_fit.c:1644-1690. */
static void recenter(oraFit *fit)
{
  int i;
  for (i = 0; i < fit->nfit; i++) {
    OPeak *pk = &fit->pk[i];
    double dx, dy;
    if (pk->status != RUNNING) continue;
    dx = pk->p[PX] - pk->xi;
    dy = pk->p[PY] - pk->yi;
    if ((dx < -0.25) || (dx > 1.25) || (dy < -0.25) || (dy > 1.25)) {
      peak_copy(fit, &fit->w, pk);
      add_peak(fit, &fit->w, -1);
      fit->w.xi = (int)floor(pk->p[PX]);
      fit->w.yi = (int)floor(pk->p[PY]);
      if (base_check(fit, &fit->w)) {
        fit->ctr[C_LOST]++;
        fit->w.status = ERROR;
      } else {
        peak_shape(fit, &fit->w);
        add_peak(fit, &fit->w, +1);
      }
      peak_copy(fit, pk, &fit->w);
    }
  }
}

/* One Gauss-Seidel LM sweep, mFitIterateLM multi_fit.c:1072-1349. */
void oraIterate(oraFit *fit)
{
  int i, k, l, n = fit->jac;
  double jac[7], wjac[7], hes[49], whes[49], e0;
  OPeak *w = &fit->w;

  for (i = 0; i < fit->nfit; i++) {
    if (fit->pk[i].status != RUNNING) continue;
    peak_copy(fit, w, &fit->pk[i]);
    calc_err(fit, w);                 /* return value ignored, :1122 */
    e0 = w->error;
    calc_jh(fit, w, jac, hes);
    add_peak(fit, w, -1);
    for (;;) {
      if (w->lambda > LAMBDA_MAX) {
        fit->ctr[C_LOST]++;
        w->status = ERROR;
        break;
      }
      w->iterations++;
      fit->ctr[C_ITER]++;
      w->status = RUNNING;
      for (k = 0; k < n; k++) {
        wjac[k] = jac[k];
        for (l = 0; l < n; l++)
          whes[k * n + l] = (k == l) ? (1.0 + w->lambda) * hes[k * n + l] : hes[k * n + l];
      }
      if (oraSolve(whes, wjac, n) != 0) {
        fit->ctr[C_DPOSV]++;
        w->status = ERROR;
        w->lambda = w->lambda * LAMBDA_UP;
        continue;
      }
      apply_update(fit, w, wjac);
      if ((is_spline(fit) || is_fft(fit) || is_pupil(fit)) ? base_check(fit, w) : model_check(fit, w)) {
        reset_working(fit, i);
        w->status = ERROR;
        continue;
      }
      peak_shape(fit, w);
      add_peak(fit, w, +1);
      if (calc_err(fit, w)) {
        add_peak(fit, w, -1);
        reset_working(fit, i);
        w->status = ERROR;
        continue;
      }
      if (w->error > e0) {
        if (((w->error - e0) / e0) < fit->tol) {
          w->status = CONVERGED;
          break;
        }
        fit->ctr[C_NONDECR]++;
        add_peak(fit, w, -1);
        reset_working(fit, i);
      } else {
        if (((e0 - w->error) / e0) < fit->tol) {
          w->status = CONVERGED;
          break;
        }
        if (w->lambda > LAMBDA_MIN) w->lambda = LAMBDA_DOWN * w->lambda;
        break;
      }
    }
    peak_copy(fit, &fit->pk[i], w);
  }
  recenter(fit);
}

/* MultiFitter.doFit, dao_fit_c.py:332-356: one sweep, then sweeps while
 * any peak is RUNNING and fewer than max_iterations were made.
 * Returns the number of sweeps. */
int oraDoFit(oraFit *fit, int max_iterations)
{
  int i = 0;
  oraIterate(fit);
  while (oraGetUnconverged(fit) && (i < max_iterations)) {
    oraIterate(fit);
    i++;
  }
  return i + 1;
}

int oraGetUnconverged(oraFit *fit)
{
  int i, c = 0;
  for (i = 0; i < fit->nfit; i++) c += (fit->pk[i].status == RUNNING);
  return c;
}

int oraGetNError(oraFit *fit)
{
  int i, c = 0;
  for (i = 0; i < fit->nfit; i++) c += (fit->pk[i].status == ERROR);
  return c;
}

int oraGetNFit(oraFit *fit) { return fit->nfit; }
int oraGetNFitMax(oraFit *fit) { return fit->maxfit; }
int oraGetJacSize(oraFit *fit) { return fit->jac; }
int oraGetRoiN(oraFit *fit) { return fit->nroi; }

void oraGetRoiIndex(oraFit *fit, int32_t *rx, int32_t *ry)
{
  int i;
  for (i = 0; i < fit->nroi; i++) { rx[i] = fit->rx[i]; ry[i] = fit->ry[i]; }
}

double oraGetOffset(oraFit *fit, int axis)
{
  return (axis == 0) ? fit->xoff : ((axis == 1) ? fit->yoff : fit->zoff);
}

void oraGetCounters(oraFit *fit, int64_t *out8)
{
  int i;
  for (i = 0; i < 8; i++) out8[i] = fit->ctr[i];
}

/* mFitPeakBgSum multi_fit.c:1518-1565. */
static double bg_sum(oraFit *fit, OPeak *pk)
{
  int j;
  size_t b = roi_base(fit, pk), k;
  double s = 0.0, ps = 0.0, psf, fg, bgv;
  for (j = 0; j < fit->nroi; j++) {
    k = (size_t)fit->ry[j] * fit->nx + fit->rx[j] + b;
    psf = pk->psf[j];
    ps += psf;
    fg = pk->p[PH] * psf;
    bgv = (fit->x[k] - fit->scmos[k]) / fit->rqe[k] - fg;
    s += bgv * psf * psf;
  }
  if ((s > 0.0) && (ps > 0.0)) return s / (ps * ps);
  return 1.0;
}

/* mFitPeakFgSum multi_fit.c:1578-1610. */
static double fg_sum(oraFit *fit, OPeak *pk)
{
  int j;
  double s = 0.0, ps = 0.0;
  for (j = 0; j < fit->nroi; j++) {
    ps += pk->psf[j];
    s += pk->psf[j] * pk->psf[j];
  }
  s = pk->p[PH] * s;
  return (ps > 0.0) ? s / ps : 1.0;
}

/* mFitGetPeakPropertyDouble multi_fit.c:754-839. */
void oraGetPeakPropertyDouble(oraFit *fit, double *v, int prop)
{
  int i, j;
  for (i = 0; i < fit->nfit; i++) {
    OPeak *pk = &fit->pk[i];
    switch (prop) {
    case ORA_PROP_BACKGROUND: v[i] = pk->p[PBG]; break;
    case ORA_PROP_BG_SUM: v[i] = bg_sum(fit, pk); break;
    case ORA_PROP_ERROR: v[i] = pk->error; break;
    case ORA_PROP_FG_SUM: v[i] = fg_sum(fit, pk); break;
    case ORA_PROP_HEIGHT: v[i] = pk->p[PH]; break;
    case ORA_PROP_SUM: {
      double s = 0.0;
      for (j = 0; j < fit->nroi; j++) s += pk->psf[j];
      v[i] = s * pk->p[PH];
      break;
    }
    case ORA_PROP_X: v[i] = pk->p[PX] + fit->xoff; break;
    case ORA_PROP_XSIGMA: v[i] = sqrt(1.0 / (2.0 * pk->p[PXW])); break;
    case ORA_PROP_Y: v[i] = pk->p[PY] + fit->yoff; break;
    case ORA_PROP_YSIGMA: v[i] = sqrt(1.0 / (2.0 * pk->p[PYW])); break;
    case ORA_PROP_Z: v[i] = pk->p[PZ] + fit->zoff; break;
    case ORA_PROP_JACOBIAN: {
      double jac[7], hes[49];
      calc_jh(fit, pk, jac, hes);
      for (j = 0; j < fit->jac; j++) v[i * fit->jac + j] = jac[j];
      break;
    }
    default: break;
    }
  }
}

void oraGetPeakPropertyInt(oraFit *fit, int32_t *v, int prop)
{
  int i;
  for (i = 0; i < fit->nfit; i++)
    v[i] = (prop == ORA_PROP_ITERATIONS) ? fit->pk[i].iterations : fit->pk[i].status;
}

/* mFitGetFitImage multi_fit.c:708-720. */
void oraGetFitImage(oraFit *fit, double *out)
{
  size_t i, np = (size_t)fit->nx * fit->ny;
  for (i = 0; i < np; i++) out[i] = fit->f[i] / fit->rqe[i];
}

/* mFitGetResidual multi_fit.c:880-888. */
void oraGetResidual(oraFit *fit, double *out)
{
  size_t i, np = (size_t)fit->nx * fit->ny;
  for (i = 0; i < np; i++) out[i] = fit->x[i] - fit->f[i];
}

/* mFitSetPeakStatus multi_fit.c:1809-1831. */
void oraSetPeakStatus(oraFit *fit, const int32_t *status)
{
  int i;
  for (i = 0; i < fit->nfit; i++) {
    if ((status[i] == ERROR) && (fit->pk[i].added > 0)) {
      peak_copy(fit, &fit->w, &fit->pk[i]);
      add_peak(fit, &fit->w, -1);
      peak_copy(fit, &fit->pk[i], &fit->w);
    }
    fit->pk[i].status = status[i];
  }
}

/* mFitRemoveErrorPeaks multi_fit.c:1704-1735. */
void oraRemoveErrorPeaks(oraFit *fit)
{
  int i = 0, j;
  for (j = 0; j < fit->nfit; j++) {
    if (fit->pk[j].status != ERROR) {
      if (j != i) peak_copy(fit, &fit->pk[i], &fit->pk[j]);
      i++;
    }
  }
  fit->nfit = i;
}

/* mFitRemoveRunningPeaks multi_fit.c:1750-1779. */
void oraRemoveRunningPeaks(oraFit *fit)
{
  int i = 0, j;
  for (j = 0; j < fit->nfit; j++) {
    if (fit->pk[j].status != RUNNING) {
      if (j != i) peak_copy(fit, &fit->pk[i], &fit->pk[j]);
      i++;
    } else {
      fit->ctr[C_NONCONV]++;
    }
  }
  fit->nfit = i;
}

/* mFitEstimatePeakHeight's lower bound (multi_fit.c:965 sets -1; the
 * multi-plane channel initialisers set 1, mp_fit_arb.c / mp_fit_dao.c). */
void oraSetMinHeight(oraFit *fit, double h) { fit->min_height = h; }

/* ------------------------------------------------------------------ */
/* multi-plane fitting: multi_plane/mp_fit.c (the coupled LM sweep),    */
/* mp_fit_arb.c (arbitrary PSFs: spline, pupil, FFT) and mp_fit_dao.c   */
/* (2D Gaussians).  A group is one peak per channel at the same index;  */
/* its channels share status and lambda, their x / y are tied through   */
/* the affine maps and their z (and, unless independent, height)        */
/* through weighted averages of the per-channel LM steps.               */
/* ------------------------------------------------------------------ */

#define ORA_MP_MAXCH 8

struct oraMP {
  int nc, indep, kind;          /* kind: ORA_MP_ARB or ORA_MP_DAO */
  double tol, w_z_offset, w_z_scale;
  int n_weights;
  double xt0N[3 * ORA_MP_MAXCH], yt0N[3 * ORA_MP_MAXCH], xtN0[3 * ORA_MP_MAXCH], ytN0[3 * ORA_MP_MAXCH];
  double *w_bg, *w_h, *w_x, *w_y, *w_z;
  double heights[ORA_MP_MAXCH];
  double dl[ORA_MP_MAXCH][7];   /* the per-channel LM steps (w_jacobian after the solve) */
  oraFit *ch[ORA_MP_MAXCH];
};

/* mpInitialize mp_fit.c:146-175 (channels are attached with oraMPSetChannel). */
oraMP *oraMPCreate(int n_channels, int independent_heights, int kind, double tol)
{
  oraMP *mp;
  if (n_channels < 1 || n_channels > ORA_MP_MAXCH) return NULL;
  mp = (oraMP *)calloc(1, sizeof(oraMP));
  mp->nc = n_channels;
  mp->indep = independent_heights;
  mp->kind = kind;
  mp->tol = tol;
  return mp;
}

void oraMPDestroy(oraMP *mp)
{
  if (!mp) return;
  free(mp->w_bg); free(mp->w_h); free(mp->w_x); free(mp->w_y); free(mp->w_z);
  free(mp);
}

/* The channel fitter (created with oraCreate; mpArbInitialize*Channel /
 * mpDaoInitialize2DChannel set its minimum height to 1). */
void oraMPSetChannel(oraMP *mp, int channel, oraFit *fit)
{
  mp->ch[channel] = fit;
  fit->min_height = 1.0;
}

/* mpSetTransforms mp_fit.c:535-548. */
void oraMPSetTransforms(oraMP *mp, const double *xt_0toN, const double *yt_0toN, const double *xt_Nto0,
                        const double *yt_Nto0)
{
  int i;
  for (i = 0; i < 3 * mp->nc; i++) {
    mp->xt0N[i] = xt_0toN[i];
    mp->yt0N[i] = yt_0toN[i];
    mp->xtN0[i] = xt_Nto0[i];
    mp->ytN0[i] = yt_Nto0[i];
  }
}

/* mpSetWeights mp_fit.c:561-592 (z the slow index, channel the fast one;
 * relative heights start at 1). */
void oraMPSetWeights(oraMP *mp, const double *w_bg, const double *w_h, const double *w_x, const double *w_y,
                     const double *w_z, int z_size)
{
  int i, n = mp->nc * z_size;
  double **dst[5] = {&mp->w_bg, &mp->w_h, &mp->w_x, &mp->w_y, &mp->w_z};
  const double *src[5] = {w_bg, w_h, w_x, w_y, w_z};
  mp->n_weights = z_size;
  for (i = 0; i < 5; i++) {
    free(*dst[i]);
    *dst[i] = (double *)malloc(sizeof(double) * n);
    memcpy(*dst[i], src[i], sizeof(double) * n);
  }
  for (i = 0; i < mp->nc; i++) mp->heights[i] = 1.0;
}

/* mpSetWeightsIndexing mp_fit.c:600-604. */
void oraMPSetWeightsIndexing(oraMP *mp, double z_offset, double z_scale)
{
  mp->w_z_offset = z_offset;
  mp->w_z_scale = z_scale;
}

/* mpWeightIndex mp_fit.c:703-725 (from channel 0's working z). */
static void mp_weight_index(const oraMP *mp, double *dz, int *zi)
{
  double t = mp->w_z_scale * (mp->ch[0]->w.p[PZ] - mp->w_z_offset);
  *zi = (int)t;
  *dz = t - (double)*zi;
  if (*zi < 0) *zi = 0;
  if (*zi > (mp->n_weights - 2)) *zi = mp->n_weights - 2;
}

/* mpWeightInterpolate mp_fit.c:732-741. */
static double mp_weight(const double *w, double dz, int zi, int nc, int c)
{
  double w1 = w[nc * zi + c], w2 = w[nc * (zi + 1) + c];
  return w1 + (w2 - w1) * dz;
}

/* The z range checks the multi-plane update calls (fn_zrange):
 * ftFitZRangeCheck fft_fit.c:506-524, pfitZRangeCheck pupil_fit.c:555-570,
 * cfZRangeCheck cubic_fit.c:987-1005 (which also sets zi). */
static void mp_z_range(const oraFit *fit, OPeak *pk)
{
  if (fit->model == ORA_FFT) {
    double max_z = ((double)fit->sz) * 0.5 - 1.0e-12;
    if (pk->p[PZ] < -max_z) pk->p[PZ] = -max_z;
    if (pk->p[PZ] > max_z) pk->p[PZ] = max_z;
  } else if (fit->model == ORA_PUPIL) {
    if (pk->p[PZ] < fit->zmin) pk->p[PZ] = fit->zmin;
    if (pk->p[PZ] > fit->zmax) pk->p[PZ] = fit->zmax;
  } else if (fit->model == ORA_SPLINE3D) {
    double zmax = ((double)fit->sz) - 1.0e-12;
    if (pk->p[PZ] < 1.0e-12) pk->p[PZ] = 1.0e-12;
    if (pk->p[PZ] > zmax) pk->p[PZ] = zmax;
    pk->zi = (int)(pk->p[PZ]);
  }
}

/* mpUpdate mp_fit.c:626-696: x and y from the channels' steps mapped back
 * to channel 0 and averaged with the weights times the relative heights,
 * mapped out to the other channels; anchors; backgrounds per channel. */
static void mp_update_xy(oraMP *mp)
{
  int i, zi, nc = mp->nc;
  double dz, p_ave, p_total, w, delta, t;
  OPeak *w0 = &mp->ch[0]->w;
  double xoff = mp->ch[0]->xoff, yoff = mp->ch[0]->yoff;
  mp_weight_index(mp, &dz, &zi);
  p_ave = 0.0;
  p_total = 0.0;
  for (i = 0; i < nc; i++) {
    w = mp_weight(mp->w_x, dz, zi, nc, i);
    delta = mp->xtN0[i * 3 + 1] * mp->dl[i][1];
    delta += mp->xtN0[i * 3 + 2] * mp->dl[i][2];
    p_ave += delta * w * mp->heights[i];
    p_total += w * mp->heights[i];
  }
  w0->p[PX] -= p_ave / p_total;
  p_ave = 0.0;
  p_total = 0.0;
  for (i = 0; i < nc; i++) {
    w = mp_weight(mp->w_y, dz, zi, nc, i);
    delta = mp->ytN0[i * 3 + 1] * mp->dl[i][1];
    delta += mp->ytN0[i * 3 + 2] * mp->dl[i][2];
    p_ave += delta * w * mp->heights[i];
    p_total += w * mp->heights[i];
  }
  w0->p[PY] -= p_ave / p_total;
  for (i = 1; i < nc; i++) {
    OPeak *pk = &mp->ch[i]->w;
    t = mp->xt0N[i * 3];
    t += mp->xt0N[i * 3 + 1] * (w0->p[PX] + xoff);
    t += mp->xt0N[i * 3 + 2] * (w0->p[PY] + yoff);
    pk->p[PX] = t - xoff;
    t = mp->yt0N[i * 3];
    t += mp->yt0N[i * 3 + 1] * (w0->p[PX] + xoff);
    t += mp->yt0N[i * 3 + 2] * (w0->p[PY] + yoff);
    pk->p[PY] = t - yoff;
  }
  for (i = 0; i < nc; i++) anchor_update(&mp->ch[i]->w);
  for (i = 0; i < nc; i++) mp->ch[i]->w.p[PBG] -= mp->dl[i][4];
}

/* mpArbUpdateZ mp_fit_arb.c:351-384. */
static void mp_arb_update_z(oraMP *mp)
{
  int i, zi, nc = mp->nc;
  double dz, p_ave = 0.0, p_total = 0.0, w, delta;
  mp_weight_index(mp, &dz, &zi);
  for (i = 0; i < nc; i++) {
    w = mp_weight(mp->w_z, dz, zi, nc, i);
    p_ave += mp->dl[i][3] * w * mp->heights[i];
    p_total += w * mp->heights[i];
  }
  delta = p_ave / p_total;
  for (i = 0; i < nc; i++) {
    mp->ch[i]->w.p[PZ] -= delta;
    mp_z_range(mp->ch[i], &mp->ch[i]->w);
  }
}

/* fn_update: mpArbUpdateFixed mp_fit_arb.c:400-432, mpArbUpdateIndependent
 * :449-470, mpDaoUpdate mp_fit_dao.c:164-209 (the 2D Gaussian's x width
 * only -- its y width keeps its value -- and daoCheck2D's clamp, whose
 * result is not used). */
static void mp_update(oraMP *mp)
{
  int i, zi, nc = mp->nc;
  double dz, p_ave, p_total, w;
  if (mp->kind == ORA_MP_DAO) {
    for (i = 0; i < nc; i++) {
      OPeak *pk = &mp->ch[i]->w;
      pk->p[PH] -= mp->dl[i][0];
      if (pk->p[PH] < 0.01) pk->p[PH] = 0.01;
      mp->heights[i] = pk->p[PH];
    }
    for (i = 0; i < nc; i++) {
      mp->ch[i]->w.p[PXW] -= mp->dl[i][3];
      model_check(mp->ch[i], &mp->ch[i]->w);
    }
    mp_update_xy(mp);
    return;
  }
  if (mp->indep) {
    for (i = 0; i < nc; i++) {
      OPeak *pk = &mp->ch[i]->w;
      pk->p[PH] -= mp->dl[i][0];
      if (pk->p[PH] < 0.01) pk->p[PH] = 0.01;
      mp->heights[i] = pk->p[PH];
    }
  } else {
    mp_weight_index(mp, &dz, &zi);
    p_ave = 0.0;
    p_total = 0.0;
    for (i = 0; i < nc; i++) {
      w = mp_weight(mp->w_h, dz, zi, nc, i);
      p_ave += mp->dl[i][0] * w;
      p_total += w;
    }
    mp->ch[0]->w.p[PH] -= p_ave / p_total;
    for (i = 1; i < nc; i++) mp->ch[i]->w.p[PH] = mp->ch[0]->w.p[PH];
  }
  mp_update_xy(mp);
  mp_arb_update_z(mp);
}

static int mp_check(oraMP *mp, oraFit *fit, OPeak *pk)
{
  (void)mp;
  return (fit->model == ORA_2D) ? model_check(fit, pk) : base_check(fit, pk);
}

/* mpResetWorkingPeaks mp_fit.c:500-521. */
static void mp_reset(oraMP *mp, int i)
{
  int c;
  for (c = 0; c < mp->nc; c++) {
    reset_working(mp->ch[c], i);
    mp->ch[c]->w.status = ERROR;
  }
}

/* mpCheckError mp_fit.c:43-68. */
static void mp_check_error(oraMP *mp, int i)
{
  int c, bad = 0;
  for (c = 0; c < mp->nc; c++) {
    if (mp->ch[c]->pk[i].status == ERROR) {
      bad = 1;
      break;
    }
  }
  if (!bad) return;
  for (c = 0; c < mp->nc; c++) {
    oraFit *fit = mp->ch[c];
    if (fit->pk[i].status != ERROR) {
      peak_copy(fit, &fit->w, &fit->pk[i]);
      add_peak(fit, &fit->w, -1);
      peak_copy(fit, &fit->pk[i], &fit->w);
    }
    fit->pk[i].status = ERROR;
  }
}

/* mpIterateLM mp_fit.c:183-478. */
void oraMPIterate(oraMP *mp)
{
  int i, c, k, l, nc = mp->nc, nfit = mp->ch[0]->nfit;
  double jac[ORA_MP_MAXCH][7], hes[ORA_MP_MAXCH][49], whes[49], e0, e1;
  for (i = 0; i < nfit; i++) {
    int bad;
    if (mp->ch[0]->pk[i].status != RUNNING) continue;
    e0 = 0.0;
    for (c = 0; c < nc; c++) {
      oraFit *fit = mp->ch[c];
      peak_copy(fit, &fit->w, &fit->pk[i]);
      calc_err(fit, &fit->w);          /* return value ignored, mp_fit.c:220 */
      e0 += fit->w.error;
      calc_jh(fit, &fit->w, jac[c], hes[c]);
      add_peak(fit, &fit->w, -1);
    }
    for (;;) {
      bad = 0;
      if (mp->ch[0]->w.lambda > LAMBDA_MAX) {
        for (c = 0; c < nc; c++) {
          mp->ch[c]->ctr[C_LOST]++;
          mp->ch[c]->w.status = ERROR;
        }
        break;
      }
      for (c = 0; c < nc; c++) mp->ch[c]->w.status = RUNNING;
      for (c = 0; c < nc; c++) {
        oraFit *fit = mp->ch[c];
        int n = fit->jac;
        fit->w.iterations++;
        fit->ctr[C_ITER]++;
        for (k = 0; k < n; k++) {
          mp->dl[c][k] = jac[c][k];
          for (l = 0; l < n; l++)
            whes[k * n + l] = (k == l) ? (1.0 + fit->w.lambda) * hes[c][k * n + l] : hes[c][k * n + l];
        }
        if (oraSolve(whes, mp->dl[c], n) != 0) {
          bad = 1;
          fit->ctr[C_DPOSV]++;
          break;
        }
      }
      if (bad) {
        for (c = 0; c < nc; c++) {
          mp->ch[c]->w.status = ERROR;
          mp->ch[c]->w.lambda = mp->ch[c]->w.lambda * LAMBDA_UP;
        }
        continue;
      }
      mp_update(mp);
      for (c = 0; c < nc; c++)
        if (mp_check(mp, mp->ch[c], &mp->ch[c]->w)) bad = 1;
      if (bad) {
        mp_reset(mp, i);
        continue;
      }
      for (c = 0; c < nc; c++) {
        peak_shape(mp->ch[c], &mp->ch[c]->w);
        add_peak(mp->ch[c], &mp->ch[c]->w, +1);
      }
      e1 = 0.0;
      for (c = 0; c < nc; c++) {
        if (calc_err(mp->ch[c], &mp->ch[c]->w)) bad = 1;
        else e1 += mp->ch[c]->w.error;
      }
      if (bad) {
        for (c = 0; c < nc; c++) add_peak(mp->ch[c], &mp->ch[c]->w, -1);
        mp_reset(mp, i);
        continue;
      }
      if (e1 > e0) {
        if (((e1 - e0) / e0) < mp->tol) {
          for (c = 0; c < nc; c++) mp->ch[c]->w.status = CONVERGED;
          break;
        }
        for (c = 0; c < nc; c++) {
          mp->ch[c]->ctr[C_NONDECR]++;
          add_peak(mp->ch[c], &mp->ch[c]->w, -1);
        }
        mp_reset(mp, i);
        continue;
      }
      if (((e0 - e1) / e0) < mp->tol) {
        for (c = 0; c < nc; c++) mp->ch[c]->w.status = CONVERGED;
      } else if (mp->ch[0]->w.lambda > LAMBDA_MIN) {
        for (c = 0; c < nc; c++) mp->ch[c]->w.lambda = mp->ch[c]->w.lambda * LAMBDA_DOWN;
      }
      break;
    }
    /* mpCopyFromWorking mp_fit.c:124-134 (channel 0's status for all) */
    for (c = 0; c < nc; c++) {
      mp->ch[c]->w.status = mp->ch[0]->w.status;
      peak_copy(mp->ch[c], &mp->ch[c]->pk[i], &mp->ch[c]->w);
    }
  }
  for (c = 0; c < nc; c++) recenter(mp->ch[c]);
  for (i = 0; i < nfit; i++) mp_check_error(mp, i);
}

/* mpArbNewPeaks mp_fit_arb.c:180-340 and mpDaoNewPeaks mp_fit_dao.c:82-152:
 * channel 0 takes the peaks as given, the others their positions mapped
 * through xt_0toN / yt_0toN; with fixed heights the "finder" / "testing"
 * peaks of a group then take the channels' mean height; groups with an
 * ERROR peak in any channel are made ERROR in all. */
void oraMPNewPeaks(oraMP *mp, const double *peaks, int ptype, int n_peaks)
{
  int i, j, c, nc = mp->nc, start = mp->ch[0]->nfit, stop = start + n_peaks;
  int arb = (mp->kind == ORA_MP_ARB);
  int ncol = (ptype == ORA_PEAKS_TEXT) ? (arb ? 5 : 7) : (arb ? 3 : 4);
  double *mapped = (double *)malloc(sizeof(double) * ncol * (n_peaks > 0 ? n_peaks : 1));
  for (c = 0; c < nc; c++) {
    if (c == 0) {
      oraNewPeaks(mp->ch[0], peaks, ptype, n_peaks);
      continue;
    }
    for (j = 0; j < n_peaks; j++) {
      const double *q = peaks + (size_t)ncol * j;
      double *o = mapped + (size_t)ncol * j, tx = q[0], ty = q[1];
      memcpy(o, q, sizeof(double) * ncol);
      o[0] = mp->xt0N[c * 3] + tx * mp->xt0N[c * 3 + 1] + ty * mp->xt0N[c * 3 + 2];
      o[1] = mp->yt0N[c * 3] + tx * mp->yt0N[c * 3 + 1] + ty * mp->yt0N[c * 3 + 2];
    }
    oraNewPeaks(mp->ch[c], mapped, ptype, n_peaks);
  }
  free(mapped);
  if (arb && !mp->indep && (ptype != ORA_PEAKS_TEXT)) {
    for (i = start; i < stop; i++) {
      double height = 0.0;
      for (c = 0; c < nc; c++) {
        oraFit *fit = mp->ch[c];
        peak_copy(fit, &fit->w, &fit->pk[i]);
        height += fit->w.p[PH];
      }
      height = height / ((double)nc);
      for (c = 0; c < nc; c++)
        if (mp->ch[c]->w.status != ERROR) add_peak(mp->ch[c], &mp->ch[c]->w, -1);
      for (c = 0; c < nc; c++) {
        oraFit *fit = mp->ch[c];
        fit->w.p[PH] = height;
        if (fit->w.status != ERROR) {
          add_peak(fit, &fit->w, +1);
          calc_err(fit, &fit->w);
        }
        peak_copy(fit, &fit->pk[i], &fit->w);
      }
    }
  }
  for (i = start; i < stop; i++) mp_check_error(mp, i);
}

int oraMPGetUnconverged(oraMP *mp) { return oraGetUnconverged(mp->ch[0]); }
