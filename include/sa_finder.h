/*
 * sa_finder.h -- C ABI of the peak finder in libsa_cuda.so: matched filters,
 * the local-maxima finder and the fused Gaussian peak-finding pass, on the
 * GPU and batched over frames of one size.
 *
 * The reference implements these on the host: sa_library/matched_filter.c
 * (FFT convolution through FFTW, bound by sa_library/matched_filter_c.py),
 * sa_library/ia_utilities.c (calcMaxPeaks / findLocalMaxima, bound by
 * sa_library/ia_utilities_c.py) and the numpy pipeline of
 * PeakFinderGaussian.peakFinder (sa_library/fitting.py:444-501).  Each
 * declaration cites what it replaces.  The matched-filter entry points also
 * exist under the reference's own names in libsa_matched_filter.so
 * (include/sa_matched_filter.h), which can stand in for libmatched_filter.so.
 *
 * Arrays are row-major doubles, rows = shape[0] (the reference's x_size /
 * ysize), cols = shape[1] (y_size / xsize).  "Device" entry points take and
 * return device pointers; the others take host pointers.  Every entry point
 * returns 0 (or a count / a handle) on success and a negative value (or
 * NULL) on failure, with the message kept for saGetLastError.
 */
#ifndef SA_FINDER_H
#define SA_FINDER_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Matched filter ------------------------------------------------------ */

/* matched_filter.c:163 initialize.  psf: the PSF already recentred for
 * circular convolution (matched_filter_c.py:58-71 recentres it), x_size x
 * y_size.  max_diff > 0 enables convolveMemo.  estimate (an FFTW planning
 * flag) is accepted and ignored.  The convolution is computed directly: as
 * two 1D passes when the PSF is separable (rank 1 to 1e-12 of its maximum,
 * true of every Gaussian the finder draws), else as a 2D sum over the PSF's
 * support (at most about 60 x 60 pixels).  Returns NULL on failure. */
void *saFilterCreate(const double *psf, double max_diff, int x_size, int y_size, int estimate);
/* No reference counterpart; host only, no device needed: how saFilterCreate
 * will convolve with this recentred PSF.  out5 = [separable, taps along
 * rows (na), taps along cols (nb), first row offset (a0), first col offset
 * (b0)]; when separable, u (na) and v (nb), if not NULL, receive the 1D taps
 * with psf[(a0 + i) mod x_size][(b0 + j) mod y_size] = u[i] * v[j].  na and
 * nb are only known after the call, so size u for x_size and v for y_size
 * entries (na <= x_size, nb <= y_size always hold). */
int saFilterAnalyze(const double *psf, int x_size, int y_size, int32_t *out5, double *u, double *v);
/* matched_filter.c:93 convolve: result = image (*) psf, circular. */
int saFilterConvolve(void *flt, const double *image, double *result);
/* matched_filter.c:118 convolveMemo: as convolve when some pixel differs
 * from the image of the last convolution by more than max_diff, else the
 * previous result (the recentred PSF before any convolution). */
int saFilterConvolveMemo(void *flt, const double *image, double *result);
/* matched_filter.c:66 cleanup. */
void saFilterCleanup(void *flt);
/* No reference counterpart: n_frames images (device, frame-major), each
 * with its own memo state when memo = 1.  Results stay in the handle
 * (saFilterResultDevice) and are copied to d_result when it is not NULL. */
int saFilterConvolveDevice(void *flt, const double *d_images, int n_frames, int memo, double *d_result);
const double *saFilterResultDevice(void *flt);
/* [separable (2: separable passes in double-float on the FP32 pipe, the
 * default; 1: FP64 passes, with SA_FINDER_FP64=1 set when the filter is
 * created; 0: the FP64 2D path), taps along rows, taps along cols, first row
 * offset, first col offset, frames allocated] */
int saFilterInfo(void *flt, int32_t *out6);
int saFilterSetStream(void *flt, void *stream);

/* ---- Local maxima -------------------------------------------------------- */

/* The reference's flmData (sa_library/ia_utilities.c:20-36), field for
 * field, as ia_utilities_c.py fills it: margin already includes the +1 the
 * Python adds; taken and images are arrays of zsize host pointers. */
typedef struct saFlmData {
  int margin;
  int n_peaks;
  int z_range;
  int xsize;
  int ysize;
  int zsize;
  double radius;
  double threshold;
  double *z_values;
  int32_t **taken;
  double **images;
} saFlmData;

/* ia_utilities.c:58 calcMaxPeaks: pixels inside the margin above threshold
 * and not yet taken, over all planes. */
int saCalcMaxPeaks(saFlmData *flm);
/* ia_utilities.c:105 findLocalMaxima: at most flm->n_peaks maxima, in plane,
 * row, column order; flm->n_peaks is set to the number found; taken is
 * incremented at each.  Runs on the GPU (images and taken are copied there
 * and taken back). */
void saFindLocalMaxima(saFlmData *flm, double *z, double *y, double *x, double *h);

/* No reference counterpart: a maxima finder whose taken counts live on the
 * GPU, for n_frames stacks of n_planes images at a time.  margin, z_range,
 * radius, threshold mean what they mean in saFlmData; taken starts at
 * 1 - n_duplicates (ia_utilities_c.py:185-191). */
void *saMaximaCreate(int margin, int z_range, double radius, double threshold,
                     const double *z_values, int n_planes, int n_duplicates);
/* Find the maxima of images (n_frames x n_planes x rows x cols; device
 * memory when on_device, else host), advance taken, and keep the peaks as
 * rows of 4 doubles, frames in order: (x, y, z, height), or (x, y, z,
 * sigma) -- daoNewPeaks' "finder" rows -- when sigma > 0.  counts (host,
 * n_frames) gets each frame's count; returns the total. */
int saMaximaFind(void *mh, const double *images, int on_device, int rows, int cols, int n_frames,
                 int32_t *counts, double sigma);
const double *saMaximaPeaksDevice(void *mh);
int saMaximaGetPeaks(void *mh, double *rows);
int saMaximaResetTaken(void *mh);
int saMaximaGetTaken(void *mh, int32_t *taken);
int saMaximaSetStream(void *mh, void *stream);
void saMaximaCleanup(void *mh);

/* ---- Post-fit culling ---------------------------------------------------- */

/* The neighbour queries of the find / fit loop (sa_library/fitting.py:
 * 716-782), on host arrays as the reference binds them.  The reference
 * searches a kd-tree (dbscan/kdtree.c) per call; here a uniform grid of
 * cells at least the radius wide is built on the GPU.  A point is a
 * neighbour when dx*dx + dy*dy <= r*r.  Statuses: 0 RUNNING, 1 CONVERGED,
 * 2 ERROR. */
/* ia_utilities.c:221 markDimmerPeaks: non-ERROR peaks with a brighter peak
 * within r_removal become ERROR, and CONVERGED peaks within r_neighbors of
 * one become RUNNING; returns the number marked. */
int saMarkDimmerPeaks(double *x, double *y, double *h, int32_t *status, double r_removal, double r_neighbors,
                      int np);
/* ia_utilities.c:292 markLowSignificancePeaks: non-ERROR peaks whose
 * significance is not above min_sig become ERROR, with the same neighbour
 * rule; returns the number marked. */
int saMarkLowSignificancePeaks(double *x, double *y, double *sig, int32_t *status, double min_sig,
                               double r_neighbors, int np);
/* ia_utilities.c:401 runningIfHasNeighbors: current peaks that are neither
 * RUNNING nor ERROR become RUNNING when a new peak is within radius. */
void saRunningIfHasNeighbors(double *c_x, double *c_y, double *n_x, double *n_y, int32_t *status, double radius,
                             int nc, int nn);
/* ia_utilities.c:82 createKDTree / :166 freeKDTree / :347 nearestKDTree:
 * distance to and index of the nearest point within radius (-1 / -1 when
 * none); points at equal distance go to the lower index (the reference
 * takes the first its tree returns). */
void *saCreateKDTree(double *x, double *y, int n);
void saFreeKDTree(void *kd);
void saNearestKDTree(void *kd, double *x, double *y, double *dist, int32_t *index, double radius, int n);

/* ---- Frame ingest -------------------------------------------------------- */

/* FrameReader.loadAFrame (sa_library/analysis_io.py:243-260) fused with
 * padArray (sa_library/fitting.py:112-132): each raw rows x cols frame
 * becomes (frame - offset) * scale (offset and scale per pixel, host arrays,
 * or NULL for the scalars offset0 / scale0; scale is the reference's
 * gain * rqe product), values below 1 set to 1 when clip, mirror-padded by
 * pad pixels (pad <= rows, cols) into doubles.  Raw pixels: dtype_bits 16
 * (uint16; big_endian swaps the bytes as DaxReader.loadAFrame does,
 * sa_library/datareader.py:232-243), 32 (float) or 64 (double), host or
 * device.  The padded frames go to d_out (device) or, when it is NULL, to a
 * buffer of the handle (saIngestResultDevice). */
void *saIngestCreate(int rows, int cols, int pad, const double *offset, const double *scale, double offset0,
                     double scale0, int clip);
int saIngestFrames(void *ih, const void *frames, int n_frames, int dtype_bits, int big_endian, int on_device,
                   double *d_out);
const double *saIngestResultDevice(void *ih);
int saIngestGetFrames(void *ih, double *out);
int saIngestSetStream(void *ih, void *stream);
int64_t saIngestKernelLaunches(void *ih);
void saIngestCleanup(void *ih);

/* ---- Gaussian peak finder ------------------------------------------------ */

/* PeakFinderGaussian (sa_library/fitting.py:361-501) on n_frames padded
 * frames of rows x cols.  bg_filter is the background matched filter,
 * fg_filter / fv_filter the optional foreground filter and the filter of
 * the PSF squared (both NULL when foreground_sigma is not set); the caller
 * keeps ownership of the three.  margin is the finder's margin (the maxima
 * finder uses margin + 1), radius find_max_radius, threshold the
 * significance threshold, z_value the z of every found peak, sigma the
 * sigma of the "finder" rows. */
void *saFinderCreate(int rows, int cols, void *bg_filter, void *fg_filter, void *fv_filter,
                     int margin, double radius, double threshold, double z_value, double sigma);
/* PeakFinderArbitraryPSF (sa_library/fitting.py:504-672): the finder of
 * Spliner / pupil-function / PSF-FFT analysis.  Per plane z (n_planes z
 * values): the foreground filter fg_filters[z] (the PSF at that z) and the
 * PSF-squared filter fv_filters[z], the variance taking |fit| (:618); the
 * maxima are searched over all planes (z_range = n_planes) and each peak's
 * z is z_values of its plane.  Peak rows are (x, y, z, height). */
void *saFinderCreateArbitrary(int rows, int cols, void *bg_filter, int n_planes, void **fg_filters,
                              void **fv_filters, const double *z_values, int margin, double radius,
                              double threshold);
/* setVariance (fitting.py:353-359): the padded camera variance, host. */
int saFinderSetVariance(void *fh, const double *camera_variance);
/* The peak mask (fitting.py:134-176), host; NULL for none. */
int saFinderSetMask(void *fh, const double *peak_mask);
/* newImage (fitting.py:304-339, 424-442): n_frames padded images (doubles,
 * host or device); resets the taken counts. */
int saFinderNewImages(void *fh, const double *images, int n_frames, int on_device);
/* estimateBackground (fitting.py:250-272): background = bg_filter applied
 * (memoised) to image - fit; fit NULL means a zero fit image.  With
 * bg_estimate != NULL the given background is used instead. */
int saFinderEstimateBackground(void *fh, const double *fit, const double *bg_estimate, int on_device);
/* peakFinder (fitting.py:444-501): the maxima of the foreground over the
 * noise; the peaks are kept as "finder" rows (x, y, z, sigma), frames in
 * order.  counts (host, n_frames) gets each frame's count; returns the
 * total. */
int saFinderFindPeaks(void *fh, const double *fit, int on_device, int32_t *counts);
const double *saFinderBackgroundDevice(void *fh);
const double *saFinderPeaksDevice(void *fh);
int saFinderGetPeaks(void *fh, double *rows);
/* Host copy of a per-frame array (all frames): 0 background, 1 the masked
 * foreground / noise ratio of the last saFinderFindPeaks (all planes of a
 * frame together). */
int saFinderGetArray(void *fh, int which, double *out);
int saFinderSetStream(void *fh, void *stream);
/* Kernels the finder has launched (its filters' and maxima finder's
 * included). */
int64_t saFinderKernelLaunches(void *fh);
void saFinderCleanup(void *fh);

#ifdef __cplusplus
}
#endif

#endif
