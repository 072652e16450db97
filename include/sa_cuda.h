/*
 * sa_cuda.h -- C ABI of libsa_cuda.so, the GB300 multi-emitter
 * Levenberg-Marquardt fitting engine behind storm-analysis's MultiFitter
 * classes.
 *
 * The first group of entry points keeps the names, argument meaning and
 * call order of the reference's fitting libraries (libdao_fit.so and
 * libcubic_fit.so), as bound by sa_library/dao_fit_c.py:147-238 and
 * spliner/cubic_fit_c.py:21-98, so either Python binding can load this
 * library instead.  Each declaration cites the reference function it
 * replaces.  Pointers are host pointers to C-contiguous arrays, as in the
 * reference; the library copies what it needs to the GPU.
 *
 * The second group (sa*) is new: error reporting, precision selection,
 * device-driven doFit and the batched multi-frame engine.
 *
 * Error behaviour: the reference's entry points return nothing and print on
 * bad input; here they print the same message, record it (saGetLastError)
 * and leave the handle unchanged.  The sa* entry points return 0 on success
 * and a negative value on failure.
 */
#ifndef SA_CUDA_H
#define SA_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Handle.  Its leading fields have the layout of the reference's fitData
 * (sa_library/multi_fit.h:80-143) because Python reads nfit, max_nfit,
 * jac_size, roi_n_index, roi_x_index/roi_y_index and the counters through a
 * ctypes mirror of that struct (sa_library/dao_fit_c.py:22-77) and writes
 * n_iterations.  Pointer fields other than roi_x_index/roi_y_index are NULL:
 * the per-pixel arrays live on the GPU.
 */
typedef struct saFitData {
  int n_dposv;
  int n_iterations;
  int n_lost;
  int n_margin;
  int n_neg_fi;
  int n_neg_height;
  int n_non_converged;
  int n_non_decr;

  int fit_size_x;
  int fit_size_y;
  int image_size_x;
  int image_size_y;
  int jac_size;
  int max_nfit;
  int nfit;
  int roi_n_index;

  double minimum_height;
  double xoff;
  double yoff;
  double zoff;
  double tolerance;

  int *bg_counts;
  int *roi_x_index;
  int *roi_y_index;
  int *stale;

  double *as_xi;
  double *bg_data;
  double *bg_estimate;
  double *err_i;
  double *f_data;
  double *rqe;
  double *scmos_term;
  double *t_fi;
  double *x_data;

  void *working_peak;
  void *fit;
  void *fit_model;

  void *fn_reserved[9];

  void *engine;             /* private */
} saFitData;

/* ---- Gaussian fitters (sa_library/dao_fit.c) ---------------------------- */

/* dao_fit.c:1251 daoInitialize */
saFitData *daoInitialize(double *rqe, double *scmos_calibration, double tol, int im_size_x,
                         int im_size_y, int roi_size);
/* dao_fit.c:1319 daoInitialize2DFixed */
void daoInitialize2DFixed(saFitData *fit);
/* dao_fit.c:1395 daoInitialize2D */
void daoInitialize2D(saFitData *fit, double width_min, double width_max);
/* dao_fit.c:1518 daoInitialize3D */
void daoInitialize3D(saFitData *fit, double width_min, double width_max);
/* dao_fit.c:1545 daoInitializeZ */
void daoInitializeZ(saFitData *fit, double *wx_vs_z, double *wy_vs_z, double z_min, double z_max);
/* dao_fit.c:1582 daoNewPeaks */
void daoNewPeaks(saFitData *fit, double *peak_params, char *p_type, int n_peaks);
/* dao_fit.c:1181 daoCleanup */
void daoCleanup(saFitData *fit);

/* Error-model variants of dao_fit.c:1337-1503 (ALS, LS, DWLS, FWLS).  Exported
 * so the reference bindings load; this engine implements the MLE model only
 * and these report an error. */
void daoInitialize2DFixedALS(saFitData *fit);
void daoInitialize2DFixedLS(saFitData *fit);
void daoInitialize2DFixedDWLS(saFitData *fit);
void daoInitialize2DFixedFWLS(saFitData *fit);
void daoInitialize2DALS(saFitData *fit, double width_min, double width_max);
void daoInitialize2DLS(saFitData *fit, double width_min, double width_max);
void daoInitialize2DDWLS(saFitData *fit, double width_min, double width_max);
void daoInitialize2DFWLS(saFitData *fit, double width_min, double width_max);

/* ---- spline fitter (spliner/cubic_fit.c, spliner/cubic_spline.c) -------- */

/* cubic_spline.c:698 initSpline2D */
void *initSpline2D(double *aij, int xsize, int ysize);
/* cubic_spline.c:749 initSpline3D */
void *initSpline3D(double *aij, int xsize, int ysize, int zsize);
/* cubic_spline.c:862 splineCleanup */
void splineCleanup(void *spline_data);
/* cubic_spline.c:660-687 getXSize / getYSize / getZSize */
int getXSize(void *spline_data);
int getYSize(void *spline_data);
int getZSize(void *spline_data);
/* cubic_fit.c:602 cfInitialize */
saFitData *cfInitialize(void *spline_data, double *rqe, double *scmos_calibration, double tol,
                        int im_size_x, int im_size_y);
/* cubic_fit.c:674 cfInitialize2D */
void cfInitialize2D(saFitData *fit);
/* cubic_fit.c:690 cfInitialize3D */
void cfInitialize3D(saFitData *fit);
/* cubic_fit.c:707-748 error-model variants (report an error, see above) */
void cfInitialize3DALS(saFitData *fit);
void cfInitialize3DLS(saFitData *fit);
void cfInitialize3DFWLS(saFitData *fit);
/* cubic_fit.c:758 cfNewPeaks */
void cfNewPeaks(saFitData *fit, double *peak_params, char *p_type, int n_peaks);
/* cubic_fit.c:511 cfCleanup (also frees the spline) */
void cfCleanup(saFitData *fit);

/* The FFT PSF model.  psf_fft/psf_fft.c (bound by psf_fft/psf_fft_c.py):
 * a 3D PSF (z_size x y_size x x_size doubles, x fastest), its spectrum and
 * the middle z plane of the translated PSF, host-side. */
/* psf_fft.c:310 pFTInitialize */
void *pFTInitialize(double *psf, int z_size, int y_size, int x_size);
/* psf_fft.c:89 pFTCleanup */
void pFTCleanup(void *pfft);
/* psf_fft.c:372 pFTTranslate */
void pFTTranslate(void *pfft, double dx, double dy, double dz);
/* psf_fft.c:116 pFTGetPSF, :147 pFTGetPSFdx, :191 pFTGetPSFdy, :235 pFTGetPSFdz
 * (y_size x x_size doubles each) */
void pFTGetPSF(void *pfft, double *psf);
void pFTGetPSFdx(void *pfft, double *dx);
void pFTGetPSFdy(void *pfft, double *dy);
void pFTGetPSFdz(void *pfft, double *dz);
/* psf_fft.c:274 pFTGetXSize, :282 pFTGetYSize, :290 pFTGetZSize */
int pFTGetXSize(void *pfft);
int pFTGetYSize(void *pfft);
int pFTGetZSize(void *pfft);

/* psf_fft/fft_fit.c (bound by psf_fft/fft_fit_c.py).  The FFT PSF model runs
 * in the FP64 engine whatever saSetPrecision asked for. */
/* fft_fit.c:254 ftFitInitialize (psf_fft from pFTInitialize) */
saFitData *ftFitInitialize(void *psf_fft, double *rqe, double *scmos_calibration, double tol, int im_size_x,
                           int im_size_y);
/* fft_fit.c:318 ftFitNewPeaks */
void ftFitNewPeaks(saFitData *fit, double *peak_params, char *p_type, int n_peaks);
/* fft_fit.c:165 ftFitCleanup (the PSF object stays the caller's) */
void ftFitCleanup(saFitData *fit);

/* The pupil-function PSF model.  pupilfn/pupil_function.c (bound by
 * pupilfn/pupil_function_c.py): a complex pupil function of size x size
 * samples (size even) with the geometry's kx, ky, kz (size x size doubles
 * each), translated, and its PSF and derivatives as complex size x size
 * arrays (real and imaginary parts), host-side. */
/* pupil_function.c:321 pfnInitialize */
void *pfnInitialize(double *kx, double *ky, double *kz, int size);
/* pupil_function.c:42 pfnCleanup */
void pfnCleanup(void *pupil_data);
/* pupil_function.c:370 pfnSetPF */
void pfnSetPF(void *pupil_data, double *r_pf, double *c_pf);
/* pupil_function.c:419 pfnSetPNEN (dipole patterns of a vectorial PSF) */
void pfnSetPNEN(void *pupil_data, double *px_ex, double *px_ey, double *py_ex, double *py_ey, double *pz_ex,
                double *pz_ey);
/* pupil_function.c:448 pfnTranslate (x, y in pixels, z in microns), :515 pfnTranslateZ */
void pfnTranslate(void *pupil_data, double dx, double dy, double dz);
void pfnTranslateZ(void *pupil_data, double dz);
/* pupil_function.c:80 pfnGetPSF, :135 pfnGetPSFdx, :160 pfnGetPSFdy, :185 pfnGetPSFdz */
void pfnGetPSF(void *pupil_data, double *psf_r, double *psf_c);
void pfnGetPSFdx(void *pupil_data, double *psf_dx_r, double *psf_dx_c);
void pfnGetPSFdy(void *pupil_data, double *psf_dy_r, double *psf_dy_c);
void pfnGetPSFdz(void *pupil_data, double *psf_dz_r, double *psf_dz_c);
/* pupil_function.c:108 pfnGetPSFIntensity */
void pfnGetPSFIntensity(void *pupil_data, double *psf_r);
/* pupil_function.c:239-302 pfnGetPXEX .. pfnGetPZEY (after pfnSetPNEN) */
void pfnGetPXEX(void *pupil_data, double *psf_r, double *psf_c);
void pfnGetPXEY(void *pupil_data, double *psf_r, double *psf_c);
void pfnGetPYEX(void *pupil_data, double *psf_r, double *psf_c);
void pfnGetPYEY(void *pupil_data, double *psf_r, double *psf_c);
void pfnGetPZEX(void *pupil_data, double *psf_r, double *psf_c);
void pfnGetPZEY(void *pupil_data, double *psf_r, double *psf_c);
/* pupil_function.c:309 pfnGetSize */
int pfnGetSize(void *pupil_data);

/* pupilfn/pupil_fit.c (bound by pupilfn/pupil_fit_c.py).  The pupil model
 * runs in the FP64 engine whatever saSetPrecision asked for; the handle
 * keeps the pupil function's tables as they are at pfitInitialize.  kx
 * must be constant along the pupil function's rows (pfnTranslate takes the
 * x shift from its first column); pfitInitialize returns NULL otherwise. */
/* pupil_fit.c:288 pfitInitialize (pupil_data from pfnInitialize) */
saFitData *pfitInitialize(void *pupil_data, double *rqe, double *scmos_calibration, double tol, int im_size_x,
                          int im_size_y);
/* pupil_fit.c:342 pfitNewPeaks */
void pfitNewPeaks(saFitData *fit, double *peak_params, char *p_type, int n_peaks);
/* pupil_fit.c:511 pfitSetZRange (the z clamp; open until called) */
void pfitSetZRange(saFitData *fit, double min_z, double max_z);
/* pupil_fit.c:180 pfitCleanup (the pupil data stays the caller's) */
void pfitCleanup(saFitData *fit);

/* ---- multi-plane fitting (multi_plane/mp_fit.c, mp_fit_arb.c, mp_fit_dao.c;
 * bound by multi_plane/mp_fit_c.py, mp_fit_arb_c.py, mp_fit_dao_c.py) -------
 * The leading fields are the reference's mpFit (mp_fit.h:12-44): its Python
 * reads n_channels and passes fit_data[i] -- one handle of this library per
 * image plane -- to the mFit* calls.  The channels run in the FP64 engine;
 * the coupled sweep runs on the device.  At most 8 channels. */
typedef struct saMPFit {
  int im_size_x;
  int im_size_y;
  int independent_heights;
  int n_channels;
  int n_weights;
  double tolerance;
  double w_z_offset;
  double w_z_scale;
  double zmin;
  double zmax;
  double *xt_0toN;
  double *yt_0toN;
  double *xt_Nto0;
  double *yt_Nto0;
  double *w_bg;
  double *w_h;
  double *w_x;
  double *w_y;
  double *w_z;
  double *heights;
  void *jacobian;
  void *w_jacobian;
  void *hessian;
  void *w_hessian;
  saFitData **fit_data;
  void *fn_cleanup;
  void *fn_newpeaks;
  void *fn_peak_xi_yi;
  void *fn_update;
  void *fn_zrange;
  void *engine;  /* private */
} saMPFit;

/* mp_fit.c:146 mpInitialize */
saMPFit *mpInitialize(double tolerance, int n_channels, int independent_heights, int im_size_x, int im_size_y);
/* mp_fit.c:76 mpCleanup (also the channels' fitters) */
void mpCleanup(saMPFit *mp_fit);
/* mp_fit.c:183 mpIterateLM */
void mpIterateLM(saMPFit *mp_fit);
/* mp_fit.c:535 mpSetTransforms (3 coefficients per channel: offset, x, y) */
void mpSetTransforms(saMPFit *mp_fit, double *xt_0toN, double *yt_0toN, double *xt_Nto0, double *yt_Nto0);
/* mp_fit.c:561 mpSetWeights ([z_size][n_channels] each) */
void mpSetWeights(saMPFit *mp_fit, double *w_bg, double *w_h, double *w_x, double *w_y, double *w_z, int z_size);
/* mp_fit.c:600 mpSetWeightsIndexing */
void mpSetWeightsIndexing(saMPFit *mp_fit, double z_offset, double z_scale);
/* No reference counterpart: how many non-overlapping groups of a frame step
 * at once in a sweep (1..8), or 0 (the default) to choose it from the
 * number of frames (8 for a lone frame, down to 2 as the frames fill the
 * GPU).
 * The results do not depend on it.  Returns 0, or -1 on error. */
int mpSetTeams(saMPFit *mp_fit, int teams);
/* mp_fit_arb.c:36 mpArbInitializePSFFFTChannel, :85 mpArbInitializePupilFnChannel,
 * :135 mpArbInitializeSplineChannel (a 3D spline) */
void mpArbInitializePSFFFTChannel(saMPFit *mp_fit, void *psf_fft, double *rqe, double *variance, int channel);
void mpArbInitializePupilFnChannel(saMPFit *mp_fit, void *pupil_data, double *rqe, double *variance, double zmin,
                                   double zmax, int channel);
void mpArbInitializeSplineChannel(saMPFit *mp_fit, void *spline, double *rqe, double *variance, int channel);
/* mp_fit_arb.c:180 mpArbNewPeaks (n_peaks per channel, channel 0's coordinates) */
void mpArbNewPeaks(saMPFit *mp_fit, double *peak_params, char *p_type, int n_peaks);
/* mp_fit_dao.c:28 mpDaoInitialize2DChannel */
void mpDaoInitialize2DChannel(saMPFit *mp_fit, double *rqe, double *variance, double width_min, double width_max,
                              int roi_size, int channel);
/* mp_fit_dao.c:82 mpDaoNewPeaks */
void mpDaoNewPeaks(saMPFit *mp_fit, double *peak_params, char *p_type, int n_peaks);

/* Batched multi-plane fitting (no reference counterpart): n_frames frames
 * on every channel (saSetFrames), images with saNewImages /
 * saNewBackgrounds on each fit_data[i], new peaks of every frame in
 * channel 0's coordinates (counts[f] rows each, frames one after another;
 * the frames' images just loaded), then doFit's sweeps for every frame at
 * once (one warp per frame); results per channel with saGetResultsBatch.
 * Return 0 (mpDoFitBatch: the number of sweeps) or -1 (saGetLastError). */
int mpSetFrames(saMPFit *mp_fit, int n_frames, int peaks_capacity);
int mpNewPeaksBatch(saMPFit *mp_fit, const double *peak_params, const int32_t *counts, const char *p_type);
int mpDoFitBatch(saMPFit *mp_fit, int max_iterations);

/* ---- shared LM core (sa_library/multi_fit.c) ----------------------------- */

/* multi_fit.c:90 mFitAnscombeTransformImage (ALS only; reports an error) */
void mFitAnscombeTransformImage(saFitData *fit);
/* multi_fit.c:708 mFitGetFitImage */
void mFitGetFitImage(saFitData *fit, double *fit_image);
/* multi_fit.c:730 mFitGetNError */
int mFitGetNError(saFitData *fit);
/* multi_fit.c:754 mFitGetPeakPropertyDouble */
void mFitGetPeakPropertyDouble(saFitData *fit, double *values, char *what);
/* multi_fit.c:851 mFitGetPeakPropertyInt */
void mFitGetPeakPropertyInt(saFitData *fit, int32_t *values, char *what);
/* multi_fit.c:880 mFitGetResidual */
void mFitGetResidual(saFitData *fit, double *residual);
/* multi_fit.c:898 mFitGetUnconverged */
int mFitGetUnconverged(saFitData *fit);
/* multi_fit.c:1072 mFitIterateLM: one Gauss-Seidel LM sweep */
void mFitIterateLM(saFitData *fit);
/* multi_fit.c:1360 mFitNewBackground */
void mFitNewBackground(saFitData *fit, double *background);
/* multi_fit.c:1382 mFitNewImage */
void mFitNewImage(saFitData *fit, double *new_image);
/* multi_fit.c:1704 mFitRemoveErrorPeaks */
void mFitRemoveErrorPeaks(saFitData *fit);
/* multi_fit.c:1750 mFitRemoveRunningPeaks */
void mFitRemoveRunningPeaks(saFitData *fit);
/* multi_fit.c:1809 mFitSetPeakStatus */
void mFitSetPeakStatus(saFitData *fit, int32_t *status);

/* ---- engine extensions (no reference counterpart) ------------------------ */

/* Copy the last error message into buf; returns its length (0: none). */
int saGetLastError(char *buf, int len);
/* Forget the last error message. */
void saClearLastError(void);
/* Number of CUDA devices visible (0 when none); never fails loudly. */
int saDeviceCount(void);
/* Pixel arithmetic precision, 32 (FP32 model/Jacobian, FP64 solve and
 * decisions) or 64 (FP64 throughout).  Call before the first image. */
int saSetPrecision(saFitData *fit, int bits);
/* Footprint dilation (pixels) used by the dependency scheduler in the first
 * 10 sweeps of a fit (default 3); later sweeps use 0. */
int saSetDilation(saFitData *fit, int pixels);
/* At most `ctas` CTAs (4 warps each) for the handle's sweep kernel; 0 (the
 * default) uses the full persistent grid.  A small cap lets the sweeps of
 * several handles run side by side on the device (serving lanes). */
int saSetSweepCTAs(saFitData *fit, int ctas);
/* Use this CUDA stream (cudaStream_t) for all work of the handle. */
int saSetStream(saFitData *fit, void *stream);
/* The whole doFit loop of dao_fit_c.py:332-356 on the device: one sweep,
 * then sweeps while any peak is RUNNING, at most max_iterations more.
 * Returns the number of sweeps made, or < 0 on error. */
int saDoFit(saFitData *fit, int max_iterations);
/* Counters (multi_fit.h:87-94 order, then the starting-error failures). */
int saGetCounters(saFitData *fit, int64_t *out9);
/* Scheduler statistics: [sweep attempts beyond the first, escapes]. */
int saGetSchedStats(saFitData *fit, int64_t *out2);

/* Batched frame sets: n_frames frames of the handle's image size share the
 * model, rqe and sCMOS calibration.  Frame f's peaks are rows
 * [sum(counts[:f]), sum(counts[:f+1])) of the concatenated input. */
int saSetFrames(saFitData *fit, int n_frames, int peaks_per_frame_capacity);
int saNewImages(saFitData *fit, const void *images, int n_frames, int dtype_bits, int on_device);
int saNewBackgrounds(saFitData *fit, const void *backgrounds, int n_frames, int dtype_bits,
                     int on_device);
int saNewPeaksBatch(saFitData *fit, const double *peaks, const int32_t *counts, int n_frames,
                    const char *p_type);
/* As saNewPeaksBatch, with the peak rows already in device memory. */
int saNewPeaksBatchDevice(saFitData *fit, const double *d_peaks, const int32_t *counts, int n_frames,
                          const char *p_type);
int saDoFitBatch(saFitData *fit, int max_iterations);
/* As saDoFitBatch for the frames with active[f] != 0 only; the others are
 * left untouched (a frame the find / fit loop gave no new peaks). */
int saDoFitBatchFrames(saFitData *fit, int max_iterations, const int32_t *active);
/* mFitSetPeakStatus for every frame: status holds all frames' peaks, frames
 * in order (multi_fit.c:1809-1831). */
int saSetPeakStatusBatch(saFitData *fit, const int32_t *status);
/* mFitRemoveErrorPeaks (status 2) / mFitRemoveRunningPeaks (status 0) for
 * every frame (multi_fit.c:1704-1779). */
int saRemovePeaksBatch(saFitData *fit, int status);
/* Grow every frame's peak storage to at least capacity_per_frame, keeping
 * the peaks (saSetFrames drops them). */
int saReservePeaksBatch(saFitData *fit, int capacity_per_frame);
/* mFitGetFitImage (residual 0) / mFitGetResidual (1) of every frame into
 * device memory d_out (n_frames x image_size_y x image_size_x doubles). */
int saGetFitImagesDevice(saFitData *fit, double *d_out, int residual);
int saGetNFitBatch(saFitData *fit, int32_t *counts);
int saGetPeakPropertyBatch(saFitData *fit, double *values, const char *what);
int saGetPeakPropertyIntBatch(saFitData *fit, int32_t *values, const char *what);
/* All frames' results with one device-to-host copy: per peak 8 doubles
 * (x, y, z, height, background, xsigma, ysigma, error) and 2 ints (status,
 * iterations), frames in order.  Returns the number of peaks. */
int saGetResultsBatch(saFitData *fit, double *values, int32_t *ints);
/* Make device `device` current for this thread (cudaSetDevice). */
int saSetDevice(int device);
/* Device time of the sweep kernels since the last reset, for profiling:
 * enable with saSetTiming(fit, 1); returns total ms and launch count. */
int saSetTiming(saFitData *fit, int on);
int saGetTiming(saFitData *fit, double *total_ms, int64_t *launches, int64_t *ticks);
/* Per-launch sweep kernel times (ms) recorded since saSetTiming(fit, 1);
 * returns how many were written (at most max_n). */
int saGetSweepTimes(saFitData *fit, float *out, int max_n);
/* Number of kernels this handle has launched. */
int64_t saGetKernelLaunches(saFitData *fit);

/* Serving slots (no reference counterpart).  The frames of a frame set
 * (saSetFrames) are slots that fit independently: a slot can be loaded with
 * a new frame while the others are mid-fit, and the device state machine
 * runs every loaded slot's sweeps as in saDoFit.
 *   saSlotLoad    frame + background (host, bits 32/64) + peak rows into one
 *                 slot and start its fit (max_iterations as doFit); the
 *                 handle's stream is synchronised (call it between bursts)
 *   saSlotLaunch  enqueue n_ticks sweep ticks for all slots and an
 *                 asynchronous read-back of the slots' states
 *   saSlotPoll    wait for that read-back; phases (PH_* : 0 idle, 4 done) and
 *                 sweeps per slot; returns the number of slots still fitting
 *   saSlotResults one slot's results as saGetResultsBatch; returns its peak
 *                 count */
int saSlotLoad(saFitData *fit, int slot, const void *image, const void *background, int bits,
               const double *peaks, int n_peaks, const char *p_type, int max_iterations);
int saSlotLaunch(saFitData *fit, int n_ticks);
int saSlotPoll(saFitData *fit, int32_t *phases, int32_t *sweeps);
/* 1 when the read-back of the last saSlotLaunch has completed (saSlotPoll
 * will not block), 0 while it is in flight, < 0 on error. */
int saSlotReady(saFitData *fit);
int saSlotResults(saFitData *fit, int slot, double *values, int32_t *ints);

/* No reference counterpart: scheduler parameters.  A peak's step waits for
 * the lower-index RUNNING peaks whose footprints, dilated by `dil` pixels
 * (saSetDilation, before the first image), overlap its own; from sweep
 * dil_switch of a fit on the dilation is dil_late (<= dil), except in a
 * frame whose previous sweep re-ran more than once.  The results do
 * not depend on these (the order of every pixel's updates is the
 * reference's whatever they are), only the time does.  Any time between
 * fits.  Returns 0, or -1 on error. */
int saSetSchedule(saFitData *fit, int dil_late, int dil_switch);
/* No reference counterpart: when every frame still fitting has at most
 * `peaks` RUNNING peaks left, their remaining sweeps run in one launch, the
 * steps of a frame one after another in index order, instead of three
 * launches and a host poll per sweep (default 8; 0 never).  The results do
 * not change.  Returns 0, or -1 on error. */
int saSetTailPeaks(saFitData *fit, int peaks);
/* No reference counterpart: the CTA count of the persistent sweep grid at
 * full occupancy (SMs x resident CTAs), once the handle has its first
 * image; -1 before.  saSetSweepCTAs caps it. */
int saGetSweepGrid(saFitData *fit);

/* No reference counterpart: the engine's damped solves in checkable form.
 * mFitSolve (multi_fit.c:1839-1883) solves (H + lam diag H) x = b with
 * LAPACK dposv("Lower") and reports failure (not positive definite, or a
 * NaN in x); the engine replaces that call by device solvers, which this
 * runs on n_sys systems: a holds n_sys row-major k x k matrices H (only
 * the upper triangle is read), b and x n_sys x k, info n_sys statuses (0 =
 * solved, nonzero = the failure mFitSolve reports).  engine 0: the FP64
 * Cholesky (FP64 engine; fallback of both FP32 solvers); 1: the FP32
 * Gaussian step's solver, given H rounded to FP32 as that step keeps it
 * (k 4 to 6); 2: the FP32 spline step's solver.  Host arrays; allocates
 * temporary device memory.  Returns 0, or -1 on error (saGetLastError). */
int saSolveDamped(const double *a, const double *b, int n_sys, int k, double lam, int engine, double *x,
                  int32_t *info);

/* No reference counterpart.  Fit image (residual = 0, as mFitGetFitImage) or
 * residual (residual = 1, as mFitGetResidual) of frame `frame` of the frame
 * set, written to the host array out (image_size_x * image_size_y doubles),
 * without allocating device memory: the kernel writes into a fixed 8 MiB
 * device scratch array compiled into the library, so frames of at most
 * 1,048,576 pixels are accepted (larger ones return -1).  For callers that
 * must not allocate: cudaMalloc / cudaFree (which the other output paths
 * may call to grow their staging buffer) can synchronise the whole device,
 * and a serving loop with work in flight on other streams, or one that has
 * reserved its device memory up front, cannot afford that.  The scratch's
 * address is looked up (cudaGetSymbolAddress, which loads the library's
 * device module on first use) once per device when a handle is created
 * (daoInitialize / cfInitialize) with that device current, so this call
 * itself only launches one kernel and copies.  Calls that overlap in time
 * (other threads or streams, any handle) share the one scratch array and
 * race.
 * Returns 0 on success, -1 on error (saGetLastError). */
int saGetFitImageNoAlloc(saFitData *fit, int frame, double *out, int residual);

#ifdef __cplusplus
}
#endif

#endif
