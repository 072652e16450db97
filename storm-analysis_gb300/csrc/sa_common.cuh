// sa_common.cuh -- shared definitions of the GB300 multi-emitter LM engine.
//
// Layout in HBM (one "frame set" = F frames of identical size and model):
//   x      [F][ny*nx]  T      image * rqe + sCMOS term (mFitNewImage, multi_fit.c:1394-1396)
//   f      [F][ny*nx]  int64  fit image, fixed point 2^-36 (f_data, multi_fit.c:52)
//   bg     [F][ny*nx]  int64  summed peak backgrounds, fixed point (bg_data, multi_fit.c:54)
//   cnt    [F][ny*nx]  int32  peaks covering each pixel (bg_counts, multi_fit.c:53)
//   bgest  [F][ny*nx]  double background estimate * rqe (multi_fit.c:1367)
//   rqe, scmos [ny*nx] T      shared by all frames (multi_fit.c:972-981)
//   pk     [peaks]     PeakRec, 128-byte records, frame f at pk_off[f]
//
// The fit image and background sums are kept as 64-bit fixed point so that
// adding and then subtracting a peak restores the pixel bit-exactly and so
// that contributions of different peaks commute.  That makes recentering,
// rollback and new-peak insertion order-independent, hence deterministic
// with plain integer atomics.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sa {

// Parameter slots (multi_fit.h:20-26).
enum { PH = 0, PX = 1, PXW = 2, PY = 3, PYW = 4, PBG = 5, PZ = 6 };
// Peak status (multi_fit.h:33-35).
enum { RUNNING = 0, CONVERGED = 1, ERROR = 2 };
// Models.
enum { M_2DFIXED = 0, M_2D = 1, M_3D = 2, M_Z = 3, M_SPLINE2D = 4, M_SPLINE3D = 5, M_FFT = 6, M_PUPIL = 7 };
// Counter slots in the reference's fitData order (multi_fit.h:87-94), plus
// one diagnostic slot of our own: starting-error evaluations that met fi <= 0.
enum { C_DPOSV = 0, C_ITER, C_LOST, C_MARGIN, C_NEGFI, C_NEGH, C_NONCONV, C_NONDECR, C_STARTFAIL,
       NCOUNTERS };

// LM schedule (multi_fit.h:42-46).
constexpr double LAMBDA_START = 1.0;
constexpr double LAMBDA_DOWN = 0.75;
constexpr double LAMBDA_MAX = 1.0e+20;
constexpr double LAMBDA_MIN = 1.0e-3;
constexpr double LAMBDA_UP = 4.0;

// Fixed point of the fit image / background accumulators.
constexpr double FX_SCALE = 68719476736.0;        // 2^36
constexpr double FX_INV = 1.0 / 68719476736.0;

// Peak input formats (dao_fit.c:1603-1753).
enum { PT_FINDER = 0, PT_TESTING = 1, PT_TEXT = 2 };

// Frame phases of the device-side doFit state machine.
enum { PH_IDLE = 0, PH_SWEEP_PENDING = 1, PH_IN_SWEEP = 2, PH_RERUN_PENDING = 3, PH_DONE = 4 };

constexpr int MAX_BARRIERS = 256;     // per frame; beyond this the frame runs in index order
constexpr int MAX_ESCAPES = 128;      // per sweep attempt; beyond this likewise
constexpr int MAX_ROI = 64;           // ROI edge limit (ext/eyt tables)
constexpr int MAX_JAC = 7;

struct __align__(16) PeakRec {
  double p[7];          // height, x, x-width, y, y-width, background, z
  double error;
  double lambda;
  double wxt, wyt;      // Z model squared width polynomials (dao_fit.c:1021-1032)
  int xi, yi, zi;
  int status, iterations, added;
  int pad[4];
};
static_assert(sizeof(PeakRec) == 128, "PeakRec must be one 128-byte line");

// Constant model description (one per fitter).
struct ModelCfg {
  int model;
  int jac;
  int nx, ny;
  int roi, nroi;
  int sx, sy, sz;        // spline cells (x, y, z); M_FFT: the PSF's x, y, z sizes; M_PUPIL: sx = sy = pupil size
  int dil;               // footprint dilation (pixels)
  int cell;              // scheduling grid cell (pixels)
  int gx, gy;            // grid cells per frame
  double xoff, yoff, zoff;
  double tol;
  double wmin, wmax;
  double wx[5], wy[5];   // w0 stored squared (dao_fit.c:1566-1567)
  double zmin, zmax;     // M_Z, M_PUPIL: the z clamp
  double min_height;
  int force_serial;      // 1: every frame runs its peaks strictly in index order
  int rqe_one;           // 1: rqe is 1 at every pixel (no per-pixel loads)
  int scmos_zero;        // 1: the sCMOS term is 0 at every pixel
  int dil_late;          // dilation from sweep dil_switch on (<= dil)
  int dil_switch;
  const double* fft;     // M_FFT: the PSF's spectrum and twiddle tables on the device (fft_layout);
                         // M_PUPIL: the pupil function's tables (pupil_layout)
};

// Per-frame control block of the device state machine.
struct FrameCtl {
  int phase;
  int sweeps;            // completed sweeps
  int max_sweeps;        // 1 + max_iterations (dao_fit_c.py:340-346)
  int start;             // first run rank of the current attempt
  int grab;              // next run rank to hand out
  int escaped_min;       // lowest escaped run rank of this attempt (INT_MAX: none)
  int n_escaped;
  int n_barrier;
  int frontier;          // every run rank in [start, frontier) is done (kept when n_barrier > 0)
  int serial;            // 1: every peak waits for its predecessor (index order)
  int unconverged;
  int nrun;
  int attempts;
  int reruns_total;      // sweep attempts beyond the first, all sweeps
  int barriers_total;    // escaped peaks made barriers, all sweeps
  int dil;               // footprint dilation of the current sweep
  long long ctr[NCOUNTERS];
  // device-only lists (the host's polls copy the fields above them)
  int escaped[MAX_ESCAPES];
  int barrier[MAX_BARRIERS];   // ascending
};

// Device pointers of a frame set.  T is the pixel arithmetic type.
template <typename T>
struct FrameSet {
  int F;
  long long npix;
  const T* x;
  const long long* xq;    // FP32 engine: the data in fixed point (2^-36), exact
  const float2* xff;      // FP32 engine: the same value as a float-float pair
  const T* rqe;
  const T* scmos;
  long long* f;
  long long* bg;
  int* cnt;
  const double* bgest;
  const T* aij;
  PeakRec* pk;
  PeakRec* snap;
  const int* pk_off;
  int* nfit;
  int* run;              // run list: local peak index per run rank
  unsigned* anchor0;     // packed (xi | yi << 16) per run rank at sweep start
  int* done;             // epoch per run rank
  int* epoch;            // epoch of the current tick (one int; k_post advances it)
  int* cell_start;       // [F][gx*gy+1]
  int2* cell_items;      // run ranks grouped by cell, each with its packed anchor
  int* stepctr;          // [peaks][NCOUNTERS] counters of the latest step of each peak
  FrameCtl* ctl;
  unsigned* err_flag;    // bit 0: wait timeout, bit 1: ROI too large
  const unsigned short* roi_xy;  // packed (rx | ry << 8)
};

// Fit-image / background accumulators.  FP32 pixel arithmetic keeps one
// int64 word per pixel in units of 2^-36; FP64 keeps two words (units 2^-18
// and 2^-50) whose sum resolves 8.9e-16 absolute, finer than a double at
// the pixel magnitudes of a fit, so that FP64 runs follow the reference's
// double arithmetic to rounding while add/subtract stay exact and
// order-free.
template <typename T>
struct AccW {
  static constexpr int W = sizeof(T) == 8 ? 2 : 1;
};

struct Q2 {
  long long h, l;
};

template <int W>
__host__ __device__ inline Q2 acc_quant(double v) {
  Q2 q;
  if (W == 1) {
#ifdef __CUDA_ARCH__
    q.h = __double2ll_rn(v * FX_SCALE);
#else
    q.h = (long long)llrint(v * FX_SCALE);
#endif
    q.l = 0;
  } else {
    const double s = v * 262144.0;   // 2^18, exact
#ifdef __CUDA_ARCH__
    q.h = __double2ll_rd(s);
#else
    q.h = (long long)floor(s);
#endif
    const double r = v - (double)q.h * (1.0 / 262144.0);   // exact, in [0, 2^-18)
#ifdef __CUDA_ARCH__
    q.l = __double2ll_rn(r * 1125899906842624.0);         // 2^50
#else
    q.l = (long long)llrint(r * 1125899906842624.0);
#endif
  }
  return q;
}

template <int W>
__host__ __device__ inline double acc_value(Q2 q) {
  if (W == 1) return (double)q.h * FX_INV;
  return (double)q.h * (1.0 / 262144.0) + (double)q.l * (1.0 / 1125899906842624.0);
}

__host__ __device__ inline long long fx_q(double v) { return acc_quant<1>(v).h; }

}  // namespace sa
