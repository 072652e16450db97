/*
 * sa_oracle.h -- CPU FP64 oracle for the multi-emitter Levenberg-Marquardt
 * fitting step of storm-analysis (3D-DAOSTORM Gaussian models and Spliner).
 *
 * TEST INFRASTRUCTURE ONLY.  This is a restatement of the reference's
 * algorithm (sa_library/multi_fit.c, sa_library/dao_fit.c,
 * spliner/cubic_fit.c, spliner/cubic_spline.c) used as the checker for the
 * GPU engine and as the timed CPU baseline.  No product code path links,
 * loads or calls it.
 *
 * Error model: MLE (Poisson deviance), the reference default
 * (sa_library/parameters.py fit_error_model "MLE").
 */
#ifndef SA_ORACLE_H
#define SA_ORACLE_H

#include <stdint.h>

/* Peak models (the reference's fitter sub-classes). */
#define ORA_2DFIXED   0   /* dao_fit.c daoInitialize2DFixed */
#define ORA_2D        1   /* dao_fit.c daoInitialize2D      */
#define ORA_3D        2   /* dao_fit.c daoInitialize3D      */
#define ORA_Z         3   /* dao_fit.c daoInitializeZ       */
#define ORA_SPLINE2D  4   /* cubic_fit.c cfInitialize2D     */
#define ORA_SPLINE3D  5   /* cubic_fit.c cfInitialize3D     */
#define ORA_FFT       6   /* psf_fft/fft_fit.c ftFitInitialize: FFT-translated 3D PSF */
#define ORA_PUPIL     7   /* pupilfn/pupil_fit.c pfitInitialize: pupil-function PSF */

/* Peak input formats (dao_fit.c:1603-1753, cubic_fit.c:776-914). */
#define ORA_PEAKS_FINDER   0
#define ORA_PEAKS_TESTING  1
#define ORA_PEAKS_TEXT     2   /* "text" and "hdf5" */

/* Double properties (multi_fit.c:754-839). */
#define ORA_PROP_BACKGROUND 0
#define ORA_PROP_BG_SUM     1
#define ORA_PROP_ERROR      2
#define ORA_PROP_FG_SUM     3
#define ORA_PROP_HEIGHT     4
#define ORA_PROP_SUM        5
#define ORA_PROP_X          6
#define ORA_PROP_XSIGMA     7
#define ORA_PROP_Y          8
#define ORA_PROP_YSIGMA     9
#define ORA_PROP_Z         10
#define ORA_PROP_JACOBIAN  11

/* Integer properties (multi_fit.c:851-868). */
#define ORA_PROP_ITERATIONS 0
#define ORA_PROP_STATUS     1

typedef struct oraFit oraFit;

/*
 * Create a fitter.  Arrays are copied.  Unused model arguments may be NULL/0.
 *   roi_size      Gaussian ROI size (ignored for splines: ROI = spline size - 1).
 *   wmin, wmax    width clamp for 2D/3D (width = 1/(2 sigma^2)).
 *   wx, wy        5 defocus-curve parameters [w0, c, d, A, B] for Z.
 *   aij, sx..sz   spline coefficients (sx*sy*sz*64 for 3D, sx*sy*16 for 2D);
 *                 for ORA_FFT the PSF's r2c spectrum (pFTInitialize
 *                 psf_fft.c:253-318: the transform of psf / (sz*sy*sx)) as
 *                 (re, im) pairs, sz x sy x (sx/2 + 1), and the PSF's x, y,
 *                 z sizes in sx, sy, sz; for ORA_PUPIL the geometry's kx,
 *                 ky, kz and the pupil function's real and imaginary parts
 *                 (sx x sx doubles each, as pfnInitialize / pfnSetPF take
 *                 them), the pupil size in sx and the z clamp in zmin, zmax.
 */
oraFit *oraCreate(int model, const double *rqe, const double *scmos, double tol,
                  int nx, int ny, int roi_size,
                  double wmin, double wmax,
                  const double *wx, const double *wy, double zmin, double zmax,
                  const double *aij, int sx, int sy, int sz);
void oraDestroy(oraFit *fit);

void oraNewImage(oraFit *fit, const double *image);
void oraNewBackground(oraFit *fit, const double *background);
void oraNewPeaks(oraFit *fit, const double *peaks, int peak_type, int n_peaks);
void oraIterate(oraFit *fit);
int  oraDoFit(oraFit *fit, int max_iterations);

int  oraGetUnconverged(oraFit *fit);
int  oraGetNError(oraFit *fit);
int  oraGetNFit(oraFit *fit);
int  oraGetNFitMax(oraFit *fit);
int  oraGetJacSize(oraFit *fit);
int  oraGetRoiN(oraFit *fit);
void oraGetRoiIndex(oraFit *fit, int32_t *rx, int32_t *ry);
double oraGetOffset(oraFit *fit, int axis);
void oraGetCounters(oraFit *fit, int64_t *out8);

void oraGetPeakPropertyDouble(oraFit *fit, double *values, int prop);
void oraGetPeakPropertyInt(oraFit *fit, int32_t *values, int prop);
void oraGetFitImage(oraFit *fit, double *out);
void oraGetResidual(oraFit *fit, double *out);

void oraSetPeakStatus(oraFit *fit, const int32_t *status);
void oraRemoveErrorPeaks(oraFit *fit);
void oraRemoveRunningPeaks(oraFit *fit);

/* Spline evaluation at a point (cubic_spline.c fSpline3D/dxfSpline3D/...).
 * which: 0 f, 1 dx, 2 dy, 3 dz. */
double oraSplineEval3D(const double *aij, int sx, int sy, int sz,
                       double z, double y, double x, int which);

/* ORA_PUPIL: the complex PSF of the pupil function translated by (dx, dy,
 * dz) and its x, y, z derivatives on the sx x sx pupil grid (index
 * u * sx + v); any output may be NULL. */
void oraPupilEval(const oraFit *fit, double dx, double dy, double dz, double *pr, double *pc, double *xr,
                  double *xc, double *yr, double *yc, double *zr, double *zc);

/* Multi-plane fitting (multi_plane/mp_fit.c, mp_fit_arb.c, mp_fit_dao.c):
 * channel fitters made with oraCreate (one per image plane, same size),
 * coupled by oraMPIterate.  kind: arbitrary PSFs (spline, pupil, FFT) or
 * 2D Gaussians. */
#define ORA_MP_ARB 0
#define ORA_MP_DAO 1
typedef struct oraMP oraMP;
oraMP *oraMPCreate(int n_channels, int independent_heights, int kind, double tol);
void oraMPDestroy(oraMP *mp);
void oraMPSetChannel(oraMP *mp, int channel, oraFit *fit);
void oraMPSetTransforms(oraMP *mp, const double *xt_0toN, const double *yt_0toN, const double *xt_Nto0,
                        const double *yt_Nto0);
void oraMPSetWeights(oraMP *mp, const double *w_bg, const double *w_h, const double *w_x, const double *w_y,
                     const double *w_z, int z_size);
void oraMPSetWeightsIndexing(oraMP *mp, double z_offset, double z_scale);
void oraMPNewPeaks(oraMP *mp, const double *peaks, int peak_type, int n_peaks);
void oraMPIterate(oraMP *mp);
int oraMPGetUnconverged(oraMP *mp);
void oraSetMinHeight(oraFit *fit, double h);

/* FP64 Cholesky solve of a k x k system given as a row-major upper triangle
 * (the layout dposv("Lower") reads, multi_fit.c:1851).  Returns 0 on success. */
int oraSolve(double *hessian, double *rhs, int k);

#endif
