// sa_finder.cu -- the peak finder of libsa_cuda.so (include/sa_finder.h):
// matched filters (circular convolution with a PSF, the job of
// sa_library/matched_filter.c), the local-maxima finder
// (sa_library/ia_utilities.c:58-210) and the fused Gaussian peak-finding pass
// of PeakFinderGaussian.peakFinder (sa_library/fitting.py:444-501), batched
// over frames of one size.
//
// The reference convolves through FFTW.  Here the PSFs the finder uses are
// small-support Gaussians, so the convolution is computed directly: two 1D
// passes for a separable PSF (81 + 81 taps for the background filter of
// sigma 8) in double-float arithmetic on the FP32 pipe (FP64 passes with
// SA_FINDER_FP64=1), a 2D FP64 sum over the support otherwise.  Each pass
// stages its rows (with the circular halo) in shared memory.  The local-maxima finder marks candidates one warp per image row
// (ballot bit masks), scans the row counts in one block and emits the peaks
// in the reference's plane, row, column order, so the lists are identical.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "sa_finder.h"
#include "sa_launch.h"

namespace {

void ferr(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  sa::record_error(buf);
}

#define FCK(call)                                                             \
  do {                                                                        \
    cudaError_t e__ = (call);                                                 \
    if (e__ != cudaSuccess) {                                                 \
      ferr("%s failed: %s", #call, cudaGetErrorString(e__));                  \
      return -1;                                                              \
    }                                                                         \
  } while (0)

constexpr int kThreads = 256;
constexpr int kSlowTR = 64;   // output rows per block of the slow-axis pass
constexpr int kTC = 32;       // columns per block of the slow-axis and 2D passes
constexpr int k2dTR = 16;     // output rows per block of the 2D pass
constexpr size_t kSmemMax = 200 * 1024;

template <typename P>
void dfree(P*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------

// flag[f] = 1 when some pixel of frame f differs from the image of its last
// convolution by more than max_diff (matched_filter.c:118-133).
__global__ void k_memo_diff(const double* __restrict__ in, const double* __restrict__ old,
                            int npix, double max_diff, int* __restrict__ flag) {
  const int f = blockIdx.y;
  const size_t base = (size_t)f * npix;
  int hit = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
    if (fabs(in[base + i] - old[base + i]) > max_diff) {
      hit = 1;
      break;
    }
  }
  if (__syncthreads_or(hit) && threadIdx.x == 0) flag[f] = 1;
}

// old = in for the frames that will be convolved (matched_filter.c:135-139).
__global__ void k_memo_copy(const double* __restrict__ in, double* __restrict__ old, int npix,
                            const int* __restrict__ flag) {
  const int f = blockIdx.y;
  if (!flag[f]) return;
  const size_t base = (size_t)f * npix;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x)
    old[base + i] = in[base + i];
}

// Pass along the fast axis: out[r][c] = sum_j w[j] in[r][(c - b0 - j) mod C].
// One block per (row, frame); the row and its circular halo are staged as
// ext[t] = in[r][(t - b0 - nb + 1) mod C], so that the tap j of output c is
// ext[c + nb - 1 - j].
__global__ void __launch_bounds__(kThreads)
k_conv_fast(const double* __restrict__ in, double* __restrict__ out, int R, int C,
            const double* __restrict__ w, int b0, int nb, const int* __restrict__ flag) {
  extern __shared__ double sm[];
  const int r = blockIdx.x, f = blockIdx.y;
  if (!flag[f]) return;
  double* ws = sm;
  double* ext = sm + nb;
  const size_t row = ((size_t)f * R + r) * C;
  for (int j = threadIdx.x; j < nb; j += blockDim.x) ws[j] = w[j];
  int base = (-b0 - nb + 1) % C;
  if (base < 0) base += C;
  const int next = C + nb - 1;
  for (int t = threadIdx.x; t < next; t += blockDim.x) ext[t] = in[row + (t + base) % C];
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    const double* e = ext + c + nb - 1;
    double s = 0.0;
    for (int j = 0; j < nb; ++j) s = fma(ws[j], e[-j], s);
    out[row + c] = s;
  }
}

// Pass along the slow axis: out[r][c] = sum_i w[i] in[(r - a0 - i) mod R][c].
// Block (32, 8) covers 32 columns x kSlowTR output rows; ext row t holds input
// row (r0 - a0 - na + 1 + t) mod R.
__global__ void __launch_bounds__(kThreads)
k_conv_slow(const double* __restrict__ in, double* __restrict__ out, int R, int C,
            const double* __restrict__ w, int a0, int na, const int* __restrict__ flag) {
  extern __shared__ double sm[];
  const int f = blockIdx.z;
  if (!flag[f]) return;
  const int c0 = blockIdx.x * kTC, r0 = blockIdx.y * kSlowTR;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTC + tx;
  double* ws = sm;
  double* ext = sm + na;
  const size_t fb = (size_t)f * R * C;
  for (int j = tid; j < na; j += kThreads) ws[j] = w[j];
  int base = (r0 - a0 - na + 1) % R;
  if (base < 0) base += R;
  const int nrows = kSlowTR + na - 1;
  const int c = c0 + tx;
  for (int t = ty; t < nrows; t += kThreads / kTC)
    ext[t * kTC + tx] = (c < C) ? in[fb + (size_t)((base + t) % R) * C + c] : 0.0;
  __syncthreads();
  if (c >= C) return;
  for (int q = ty; q < kSlowTR; q += kThreads / kTC) {
    const int r = r0 + q;
    if (r >= R) break;
    const double* e = ext + (q + na - 1) * kTC + tx;
    double s = 0.0;
    for (int i = 0; i < na; ++i) s = fma(ws[i], e[-i * kTC], s);
    out[fb + (size_t)r * C + c] = s;
  }
}

// The same two passes on the FP32 pipe in double-float arithmetic: GB300
// issues FP32 FMAs at many times its FP64 rate, so each tap is computed as a
// float pair.  A double input x is split as x = xh + xl (floats, exact to
// 2^-48 |x|); a tap adds w * x with the exact product wh*xh (p + e by FMA)
// plus the cross terms wh*xl + wl*xh, and the running sum is kept as a
// normalised float pair (Knuth two-sum, then fast two-sum).  Per tap about
// 2^-48 of the running sum is lost: the result agrees with the FP64 sum to
// ~1e-14 of its magnitude.  The explicit-rounding intrinsics keep the
// compiler from fusing the two-sum steps.
__device__ __forceinline__ float2 ff_split(double v) {
  const float h = __double2float_rn(v);
  return make_float2(h, __double2float_rn(v - (double)h));
}

__device__ __forceinline__ void ff_tap(float2 w, float2 x, float& sh, float& sl) {
  const float p = __fmul_rn(w.x, x.x);
  float e = fmaf(w.x, x.x, -p);
  e = fmaf(w.x, x.y, e);
  e = fmaf(w.y, x.x, e);
  const float s = __fadd_rn(sh, p);
  const float v = __fsub_rn(s, sh);
  float t = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, v)), __fsub_rn(p, v));
  t = __fadd_rn(__fadd_rn(t, sl), e);
  sh = __fadd_rn(s, t);
  sl = __fsub_rn(t, __fsub_rn(sh, s));
}

__global__ void __launch_bounds__(kThreads)
k_conv_fast_ff(const double* __restrict__ in, double* __restrict__ out, int R, int C,
               const float2* __restrict__ w, int b0, int nb, const int* __restrict__ flag) {
  extern __shared__ float2 smf[];
  const int r = blockIdx.x, f = blockIdx.y;
  if (!flag[f]) return;
  float2* ws = smf;
  float2* ext = smf + nb;
  const size_t row = ((size_t)f * R + r) * C;
  for (int j = threadIdx.x; j < nb; j += blockDim.x) ws[j] = w[j];
  int base = (-b0 - nb + 1) % C;
  if (base < 0) base += C;
  const int next = C + nb - 1;
  for (int t = threadIdx.x; t < next; t += blockDim.x) ext[t] = ff_split(in[row + (t + base) % C]);
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    const float2* e = ext + c + nb - 1;
    float sh = 0.0f, sl = 0.0f;
    for (int j = 0; j < nb; ++j) ff_tap(ws[j], e[-j], sh, sl);
    out[row + c] = (double)sh + (double)sl;
  }
}

__global__ void __launch_bounds__(kThreads)
k_conv_slow_ff(const double* __restrict__ in, double* __restrict__ out, int R, int C,
               const float2* __restrict__ w, int a0, int na, const int* __restrict__ flag) {
  extern __shared__ float2 smf[];
  const int f = blockIdx.z;
  if (!flag[f]) return;
  const int c0 = blockIdx.x * kTC, r0 = blockIdx.y * kSlowTR;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTC + tx;
  float2* ws = smf;
  float2* ext = smf + na;
  const size_t fb = (size_t)f * R * C;
  for (int j = tid; j < na; j += kThreads) ws[j] = w[j];
  int base = (r0 - a0 - na + 1) % R;
  if (base < 0) base += R;
  const int nrows = kSlowTR + na - 1;
  const int c = c0 + tx;
  for (int t = ty; t < nrows; t += kThreads / kTC)
    ext[t * kTC + tx] = (c < C) ? ff_split(in[fb + (size_t)((base + t) % R) * C + c]) : make_float2(0.0f, 0.0f);
  __syncthreads();
  if (c >= C) return;
  for (int q = ty; q < kSlowTR; q += kThreads / kTC) {
    const int r = r0 + q;
    if (r >= R) break;
    const float2* e = ext + (q + na - 1) * kTC + tx;
    float sh = 0.0f, sl = 0.0f;
    for (int i = 0; i < na; ++i) ff_tap(ws[i], e[-i * kTC], sh, sl);
    out[fb + (size_t)r * C + c] = (double)sh + (double)sl;
  }
}

// Direct 2D circular convolution over the PSF's support (na x nb taps,
// w[i * nb + j] = psf[(a0 + i) mod R][(b0 + j) mod C]).  Block (32, 8) covers
// 32 columns x k2dTR rows; ext holds the input tile with its halo.
__global__ void __launch_bounds__(kThreads)
k_conv_2d(const double* __restrict__ in, double* __restrict__ out, int R, int C,
          const double* __restrict__ w, int a0, int na, int b0, int nb,
          const int* __restrict__ flag) {
  extern __shared__ double sm[];
  const int f = blockIdx.z;
  if (!flag[f]) return;
  const int c0 = blockIdx.x * kTC, r0 = blockIdx.y * k2dTR;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kTC + tx;
  const int er = k2dTR + na - 1, ec = kTC + nb - 1;
  double* ws = sm;
  double* ext = sm + na * nb;
  const size_t fb = (size_t)f * R * C;
  for (int k = tid; k < na * nb; k += kThreads) ws[k] = w[k];
  int rb = (r0 - a0 - na + 1) % R;
  if (rb < 0) rb += R;
  int cb = (c0 - b0 - nb + 1) % C;
  if (cb < 0) cb += C;
  for (int k = tid; k < er * ec; k += kThreads) {
    const int t = k / ec, u = k - t * ec;
    ext[k] = in[fb + (size_t)((rb + t) % R) * C + (cb + u) % C];
  }
  __syncthreads();
  const int c = c0 + tx;
  if (c >= C) return;
  for (int q = ty; q < k2dTR; q += kThreads / kTC) {
    const int r = r0 + q;
    if (r >= R) break;
    double s = 0.0;
    for (int i = 0; i < na; ++i) {
      const double* e = ext + (q + na - 1 - i) * ec + tx + nb - 1;
      const double* wr = ws + i * nb;
      for (int j = 0; j < nb; ++j) s = fma(wr[j], e[-j], s);
    }
    out[fb + (size_t)r * C + c] = s;
  }
}

// Local maxima (ia_utilities.c:105-210).
struct LMax {
  const double* img;   // F x Z x R x C
  int32_t* taken;      // F x Z x R x C
  uint32_t* bits;      // F x Z x R x W candidate masks
  int32_t* rowcnt;     // F x Z x R
  int R, C, Z, W, nrows;
  int margin, z_range, rr, cr;
  double radius, threshold;
};

// isLocalMaxima (ia_utilities.c:177-210): the search box uses the C
// conversions of the reference (y: truncation of yi -/+ radius; x: ceil
// radius; radius**2 truncated to int).  Ties go to the pixel with the larger
// row and column.
__device__ bool is_local_max(const LMax& a, const double* fimg, int zi, int yi, int xi, double cur) {
  const int sz = max(zi - a.z_range, 0), ez = min(zi + a.z_range, a.Z - 1);
  const int sy = max((int)(yi - a.radius), 0), ey = min((int)(yi + a.radius), a.R - 1);
  const int sx = max(xi - a.cr, 0), ex = min(xi + a.cr, a.C - 1);
  // A necessary condition first: the 3 x 3 neighbourhood in the candidate's
  // own plane (part of the search below).  Most candidates sit on the slope
  // of a peak and fail here after a few reads; the outcome is the same
  // since the test is a conjunction over the search region.
  {
    const double* p = fimg + (size_t)zi * a.R * a.C;
    for (int y = max(yi - 1, sy); y <= min(yi + 1, ey); ++y)
      for (int x = max(xi - 1, sx); x <= min(xi + 1, ex); ++x) {
        if ((x - xi) * (x - xi) + (y - yi) * (y - yi) > a.rr) continue;
        const double v = p[(size_t)y * a.C + x];
        if (y <= yi && x <= xi) {
          if (v > cur) return false;
        } else if (v >= cur) {
          return false;
        }
      }
  }
  for (int z = sz; z <= ez; ++z) {
    const double* p = fimg + (size_t)z * a.R * a.C;
    for (int y = sy; y <= ey; ++y) {
      const int dy = (y - yi) * (y - yi);
      const double* row = p + (size_t)y * a.C;
      for (int x = sx; x <= ex; ++x) {
        const int dx = (x - xi) * (x - xi);
        if (dx + dy > a.rr) continue;
        const double v = row[x];
        if (y <= yi && x <= xi) {
          if (v > cur) return false;
        } else if (v >= cur) {
          return false;
        }
      }
    }
  }
  return true;
}

// One warp per (frame, plane, row): candidate bits by ballot, row count.
__global__ void k_lmax_mark(LMax a) {
  const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (warp >= a.nrows) return;
  const int y = warp % a.R, fz = warp / a.R, zi = fz % a.Z, f = fz / a.Z;
  const double* fimg = a.img + (size_t)f * a.Z * a.R * a.C;
  const double* row = fimg + ((size_t)zi * a.R + y) * a.C;
  const int32_t* tk = a.taken + (size_t)warp * a.C;
  uint32_t* bits = a.bits + (size_t)warp * a.W;
  const bool row_in = y >= a.margin && y < a.R - a.margin;
  int cnt = 0;
  for (int w = 0; w < a.W; ++w) {
    const int x = w * 32 + lane;
    bool flag = false;
    if (row_in && x >= a.margin && x < a.C - a.margin) {
      const double cur = row[x];
      if (cur > a.threshold && tk[x] < 1) flag = is_local_max(a, fimg, zi, y, x, cur);
    }
    const uint32_t b = __ballot_sync(0xffffffffu, flag);
    if (lane == 0) bits[w] = b;
    cnt += __popc(b);
  }
  if (lane == 0) a.rowcnt[warp] = cnt;
}

// Exclusive scan of the row counts in one block of 1024 threads; fcount[f]
// is frame f's total and fcount[F] the grand total.
__global__ void __launch_bounds__(1024)
k_lmax_scan(const int32_t* __restrict__ rowcnt, int32_t* __restrict__ rowoff, int nrows,
            int rows_per_frame, int F, int32_t* __restrict__ fcount) {
  __shared__ int32_t wsum[32];
  __shared__ int32_t carry_s;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (int base = 0; base < nrows; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < nrows ? rowcnt[i] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int s = wsum[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      wsum[lane] = s;
    }
    __syncthreads();
    const int incl = x + (wid ? wsum[wid - 1] : 0);
    const int carry = carry_s;
    if (i < nrows) rowoff[i] = carry + incl - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry_s = carry + incl;
    __syncthreads();
  }
  for (int f = threadIdx.x; f < F; f += 1024) {
    const int s = rowoff[f * rows_per_frame];
    const int e = (f + 1 < F) ? rowoff[(f + 1) * rows_per_frame] : carry_s;
    fcount[f] = e - s;
  }
  if (threadIdx.x == 0) fcount[F] = carry_s;
}

// One warp per row with candidates: write the peaks at their scanned
// positions (plane, row, column order) and advance taken.  Peaks at or past
// cap are dropped, as findLocalMaxima stops at n_peaks.
__global__ void k_lmax_emit(LMax a, const int32_t* __restrict__ rowoff,
                            const double* __restrict__ zvalues, double* __restrict__ out, int cap,
                            double sigma) {
  const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (warp >= a.nrows) return;
  if (a.rowcnt[warp] == 0) return;
  const int y = warp % a.R, fz = warp / a.R, zi = fz % a.Z;
  const double* row = a.img + (size_t)warp * a.C;
  int32_t* tk = a.taken + (size_t)warp * a.C;
  const uint32_t* bits = a.bits + (size_t)warp * a.W;
  int pos = rowoff[warp];
  for (int w = 0; w < a.W; ++w) {
    const uint32_t b = bits[w];
    if (b == 0) continue;
    if ((b >> lane) & 1u) {
      const int p = pos + __popc(b & ((1u << lane) - 1u));
      if (p < cap) {
        const int x = w * 32 + lane;
        double* o = out + (size_t)p * 4;
        o[0] = (double)x;
        o[1] = (double)y;
        o[2] = zvalues[zi];
        o[3] = sigma > 0.0 ? sigma : row[x];
        tk[x] += 1;
      }
    }
    pos += __popc(b);
  }
}

// calcMaxPeaks (ia_utilities.c:58-75): candidates inside the margin.
__global__ void k_lmax_count(LMax a, int32_t* __restrict__ count) {
  int n = 0;
  const size_t total = (size_t)a.nrows * a.C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % a.C);
    const int y = (int)((i / a.C) % a.R);
    if (y >= a.margin && y < a.R - a.margin && x >= a.margin && x < a.C - a.margin &&
        a.img[i] > a.threshold && a.taken[i] < 1)
      ++n;
  }
  for (int o = 16; o > 0; o >>= 1) n += __shfl_down_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(count, n);
}

__global__ void k_fill_i32(int32_t* __restrict__ p, size_t n, int32_t v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    p[i] = v;
}

// Finder arithmetic of fitting.py:453-457 and :479, in the reference's order:
// bgv = (background + fit) + camera_variance; fgr = (image - background) - fit.
// The arbitrary-PSF finder takes |fit| in the variance (fitting.py:618).
__global__ void k_find_prep(const double* __restrict__ image, const double* __restrict__ bg,
                            const double* __restrict__ fit, const double* __restrict__ camvar,
                            double* __restrict__ bgv, double* __restrict__ fgr, int npix,
                            size_t total, int abs_fit) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const double b = bg[i];
    const double ft = fit ? fit[i] : 0.0;
    double v = b + (abs_fit ? fabs(ft) : ft);
    if (camvar) v += camvar[i % npix];
    bgv[i] = v;
    fgr[i] = (image[i] - b) - ft;
  }
}

// image - fit, the input of the background filter (fitting.py:265).
__global__ void k_sub(const double* __restrict__ a, const double* __restrict__ b,
                      double* __restrict__ out, size_t total) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = b ? a[i] - b[i] : a[i];
}

// masked = (fg / sqrt(bgv <= 0.1 ? 0.1 : bgv)) * mask (fitting.py:470-497).
// out holds n_planes planes per frame; this call writes plane z.
__global__ void k_find_ratio(const double* __restrict__ fg, const double* __restrict__ bgv,
                             const double* __restrict__ mask, double* __restrict__ out, int npix,
                             size_t total, int z, int n_planes) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    double v = bgv[i];
    if (v <= 0.1) v = 0.1;
    double r = fg[i] / sqrt(v);
    if (mask) r = r * mask[i % npix];
    const size_t o = n_planes == 1 ? i : ((i / npix) * n_planes + z) * npix + i % npix;
    out[o] = r;
  }
}

// Frame ingest: FrameReader.loadAFrame (sa_library/analysis_io.py:243-260:
// (frame - offset) * (gain * rqe), values below 1 set to 1) and padArray
// (sa_library/fitting.py:112-132: mirror padding that repeats the edge
// pixel).  Raw pixels are uint16 (byte swapped for big-endian .dax data),
// float32 or float64.  One thread per padded output pixel: coalesced
// writes, reads from the mirrored source.
__device__ __forceinline__ int mirror_index(int i, int n) {
  return i < 0 ? -1 - i : (i >= n ? 2 * n - 1 - i : i);
}

// GB300 issues few FP64 instructions per clock, so the exact parts of the
// conversion run on the integer pipe: a uint16 becomes a double by building
// its bits (exponent from the leading one, the rest as mantissa), and
// "v < 1.0" is decided on the bit pattern.
__device__ __forceinline__ double u16_to_double(unsigned int u) {
  if (u == 0) return 0.0;
  const int e = 31 - __clz(u);
  const unsigned long long m = ((unsigned long long)u << (52 - e)) & 0xFFFFFFFFFFFFFull;
  return __longlong_as_double((long long)(((unsigned long long)(1023 + e) << 52) | m));
}

__device__ __forceinline__ bool less_than_one(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  if ((b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull) return false;   // NaN
  return (b >> 63) ? true : b < 0x3FF0000000000000ull;
}

__global__ void __launch_bounds__(kThreads)
k_ingest(const void* __restrict__ raw, int bits, int swap, int rows, int cols, int pad,
         const double* __restrict__ offset, const double* __restrict__ scale, double off0, double sc0,
         int clip, double* __restrict__ out) {
  // one thread per padded output pixel of frame blockIdx.y
  const int prow = rows + 2 * pad, pcol = cols + 2 * pad;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= prow * pcol) return;
  const int f = blockIdx.y;
  const int y = i / pcol, x = i - y * pcol;
  const int sy = mirror_index(y - pad, rows), sx = mirror_index(x - pad, cols);
  const int p = sy * cols + sx;
  const size_t src = (size_t)f * rows * cols + p;
  double v;
  if (bits == 16) {
    unsigned int u = static_cast<const uint16_t*>(raw)[src];
    if (swap) u = ((u >> 8) | (u << 8)) & 0xffffu;
    v = u16_to_double(u);
  } else if (bits == 32) {
    v = (double)static_cast<const float*>(raw)[src];
  } else {
    v = static_cast<const double*>(raw)[src];
  }
  v = (v - (offset ? offset[p] : off0)) * (scale ? scale[p] : sc0);
  if (clip && less_than_one(v)) v = 1.0;
  out[(size_t)f * prow * pcol + i] = v;
}

// ---------------------------------------------------------------------------
// Neighbour queries of the post-fit culling (sa_library/ia_utilities.c:221-430)
// ---------------------------------------------------------------------------
// The reference builds a kd-tree per call; here points are hashed into a
// uniform grid of cells at least the query radius wide, so every point
// within the radius lies in the 3 x 3 cells around the query.  Cells hash
// into a power-of-two table (a bucket may hold several cells; the distance
// test decides).  Membership follows kd_nearest_range (dbscan/kdtree.c:
// 262-293): dx*dx + dy*dy <= r*r, in that order.

struct PointGrid {
  const double* x;
  const double* y;
  const int32_t* start;   // T bucket starts (exclusive scan of the counts)
  const int32_t* total;   // total points (end of the last bucket)
  const int32_t* items;   // point indices by bucket
  int T;
  double cs;
};

__device__ __forceinline__ long long cell_of(double v, double cs) { return (long long)floor(v / cs); }

__device__ __forceinline__ int bucket_of(long long cx, long long cy, int T) {
  const unsigned long long h = (unsigned long long)cx * 0x9E3779B97F4A7C15ull ^
                               ((unsigned long long)cy * 0xC2B2AE3D27D4EB4Full + 0x165667B19E3779F9ull);
  return (int)((h ^ (h >> 29)) & (unsigned long long)(T - 1));
}

__global__ void k_grid_count(const double* __restrict__ x, const double* __restrict__ y, int n, double cs, int T,
                             int32_t* __restrict__ counts) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    atomicAdd(&counts[bucket_of(cell_of(x[i], cs), cell_of(y[i], cs), T)], 1);
}

__global__ void k_grid_fill(const double* __restrict__ x, const double* __restrict__ y, int n, double cs, int T,
                            const int32_t* __restrict__ start, int32_t* __restrict__ cursor,
                            int32_t* __restrict__ items) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int b = bucket_of(cell_of(x[i], cs), cell_of(y[i], cs), T);
    items[start[b] + atomicAdd(&cursor[b], 1)] = i;
  }
}

// Visit every grid point within r of (qx, qy); fn(k, dd) returns true to stop.
template <typename Fn>
__device__ void grid_visit(const PointGrid& g, double qx, double qy, double r, Fn fn) {
  const long long cx = cell_of(qx, g.cs), cy = cell_of(qy, g.cs);
  const double rr = __dmul_rn(r, r);
  for (int dy = -1; dy <= 1; ++dy)
    for (int dx = -1; dx <= 1; ++dx) {
      const int b = bucket_of(cx + dx, cy + dy, g.T);
      const int s = g.start[b], e = (b + 1 < g.T) ? g.start[b + 1] : *g.total;
      for (int j = s; j < e; ++j) {
        const int k = g.items[j];
        const double ex = g.x[k] - qx, ey = g.y[k] - qy;
        // unfused, as the reference's host build evaluates it
        const double dd = __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey));
        if (dd <= rr && fn(k, dd)) return;
      }
    }
}

constexpr int32_t kRunning = 0, kConverged = 1, kError = 2;

// markDimmerPeaks, first half: a non-ERROR peak with a brighter peak within
// r_removal is marked (ia_utilities.c:236-268).
__global__ void k_mark_dimmer(PointGrid g, const double* __restrict__ h, const int32_t* __restrict__ status,
                              int n, double r, int32_t* __restrict__ marked, int32_t* __restrict__ n_marked) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int m = 0;
    if (status[i] != kError) {
      const double hi = h[i];
      grid_visit(g, g.x[i], g.y[i], r, [&](int k, double) {
        if (h[k] > hi) m = 1;
        return m != 0;
      });
    }
    marked[i] = m;
    if (m) atomicAdd(n_marked, 1);
  }
}

// markLowSignificancePeaks, first half: a non-ERROR peak whose significance
// is not above the minimum is marked (ia_utilities.c:305-315).
__global__ void k_mark_low_sig(const double* __restrict__ sig, const int32_t* __restrict__ status, int n,
                               double min_sig, int32_t* __restrict__ marked, int32_t* __restrict__ n_marked) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int m = (status[i] != kError && !(sig[i] > min_sig)) ? 1 : 0;
    marked[i] = m;
    if (m) atomicAdd(n_marked, 1);
  }
}

// Second half of both: marked peaks become ERROR; a CONVERGED peak within
// r_neighbors of a marked peak becomes RUNNING.  In the reference's loop a
// peak is marked from its own brightness / significance alone, so the
// result does not depend on the order the peaks are visited in.
__global__ void k_mark_apply(PointGrid g, const int32_t* __restrict__ marked, const int32_t* __restrict__ in,
                             int32_t* __restrict__ out, int n, double r) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int32_t st = in[i];
    if (marked[i]) {
      st = kError;
    } else if (st == kConverged) {
      bool near = false;
      grid_visit(g, g.x[i], g.y[i], r, [&](int k, double) {
        near = marked[k] != 0;
        return near;
      });
      if (near) st = kRunning;
    }
    out[i] = st;
  }
}

// runningIfHasNeighbors (ia_utilities.c:401-430): a peak that is neither
// RUNNING nor ERROR becomes RUNNING when a new peak is within radius.
__global__ void k_running_if_neighbors(PointGrid g, const double* __restrict__ cx, const double* __restrict__ cy,
                                       int32_t* __restrict__ status, int nc, double r) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
    if (status[i] == kRunning || status[i] == kError) continue;
    bool near = false;
    grid_visit(g, cx[i], cy[i], r, [&](int, double) {
      near = true;
      return true;
    });
    if (near) status[i] = kRunning;
  }
}

// nearestKDTree (ia_utilities.c:347-391): the nearest point within radius
// (distance and index), -1 / -1 when there is none.  Equal distances go to
// the lower index.
__global__ void k_nearest(PointGrid g, const double* __restrict__ qx, const double* __restrict__ qy, int n,
                          double r, double* __restrict__ dist, int32_t* __restrict__ index) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double best = __dadd_rn(__dmul_rn(r, r), 0.1);
    int bi = -1;
    grid_visit(g, qx[i], qy[i], r, [&](int k, double dd) {
      if (dd < best || (dd == best && k < bi)) {
        best = dd;
        bi = k;
      }
      return false;
    });
    dist[i] = bi >= 0 ? sqrt(best) : -1.0;
    index[i] = bi;
  }
}

int grid_for(size_t n) {
  size_t g = (n + kThreads - 1) / kThreads;
  return (int)std::min<size_t>(std::max<size_t>(g, 1), 152 * 16);
}

// ---------------------------------------------------------------------------
// Matched filter
// ---------------------------------------------------------------------------

// The smallest circular arc [start, start + len) of 0..n-1 holding every
// index with nz set; start in (-n, n).  No nonzero index: len 0.
void circular_support(const std::vector<char>& nz, int n, int* start, int* len) {
  int count = 0;
  for (char v : nz) count += v ? 1 : 0;
  if (count == 0) {
    *start = 0;
    *len = 0;
    return;
  }
  if (count == n) {
    *start = -(n / 2);
    *len = n;
    return;
  }
  // the longest circular run of zeros; the support is its complement
  int best = -1, best_at = 0;
  for (int i = 0; i < n; ++i) {
    if (nz[i] || !nz[(i + n - 1) % n]) continue;   // runs start after a nonzero
    int k = 0;
    while (k < n && !nz[(i + k) % n]) ++k;
    if (k > best) {
      best = k;
      best_at = i;
    }
  }
  int s = (best_at + best) % n;
  *len = n - best;
  if (s > n / 2) s -= n;
  *start = s;
}

struct MFilter {
  int R = 0, C = 0;
  int separable = 1;
  int a0 = 0, na = 1, b0 = 0, nb = 1;
  double* d_wa = nullptr;   // separable: taps along rows (slow axis)
  double* d_wb = nullptr;   // separable: taps along columns (fast axis)
  float2* d_wa_ff = nullptr;   // the same taps as float pairs
  float2* d_wb_ff = nullptr;
  int ff = 1;                  // separable passes in double-float (FP32 pipe)
  double* d_w2 = nullptr;   // 2D: na x nb
  double max_diff = 0.0;
  std::vector<double> h_rc;   // the recentred PSF, first content of every frame's result
  int F = 0;
  double* d_last = nullptr;   // F x R x C: each frame's last result
  double* d_old = nullptr;    // F x R x C: each frame's last convolved image (memo)
  double* d_tmp = nullptr;    // F x R x C: fast-axis pass output
  int* d_flag = nullptr;      // F
  double* d_io = nullptr;     // R x C staging of the host entry points
  double* d_io2 = nullptr;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  size_t smem_fast = 0, smem_slow = 0, smem_2d = 0;
};

void filter_free(MFilter* m) {
  dfree(m->d_wa);
  dfree(m->d_wb);
  dfree(m->d_wa_ff);
  dfree(m->d_wb_ff);
  dfree(m->d_w2);
  dfree(m->d_last);
  dfree(m->d_old);
  dfree(m->d_tmp);
  dfree(m->d_flag);
  dfree(m->d_io);
  dfree(m->d_io2);
}

int filter_frames(MFilter* m, int F, cudaStream_t s) {
  if (F <= m->F) return 0;
  const size_t npix = (size_t)m->R * m->C;
  double *last = nullptr, *old = nullptr, *tmp = nullptr;
  int* flag = nullptr;
  FCK(cudaMalloc(&last, sizeof(double) * npix * F));
  FCK(cudaMalloc(&old, sizeof(double) * npix * F));
  FCK(cudaMalloc(&tmp, sizeof(double) * npix * F));
  FCK(cudaMalloc(&flag, sizeof(int) * F));
  FCK(cudaStreamSynchronize(s));
  if (m->F > 0) {
    FCK(cudaMemcpy(last, m->d_last, sizeof(double) * npix * m->F, cudaMemcpyDeviceToDevice));
    FCK(cudaMemcpy(old, m->d_old, sizeof(double) * npix * m->F, cudaMemcpyDeviceToDevice));
  }
  for (int f = m->F; f < F; ++f)
    FCK(cudaMemcpy(last + npix * f, m->h_rc.data(), sizeof(double) * npix, cudaMemcpyHostToDevice));
  FCK(cudaMemset(old + npix * m->F, 0, sizeof(double) * npix * (F - m->F)));
  dfree(m->d_last);
  dfree(m->d_old);
  dfree(m->d_tmp);
  dfree(m->d_flag);
  m->d_last = last;
  m->d_old = old;
  m->d_tmp = tmp;
  m->d_flag = flag;
  m->F = F;
  return 0;
}

// Convolve n frames of d_in (device) into the handle's results; memo as
// convolveMemo, else every frame.
int filter_run(MFilter* m, const double* d_in, int n, int memo, cudaStream_t s) {
  if (n < 1) return 0;
  if (filter_frames(m, n, s)) return -1;
  const int npix = m->R * m->C;
  if (memo) {
    if (m->max_diff <= 0.0) {
      ferr("convolveMemo: the filter was created without memoisation (max_diff 0)");
      return -1;
    }
    FCK(cudaMemsetAsync(m->d_flag, 0, sizeof(int) * n, s));
    const dim3 g(std::min(64, (npix + kThreads - 1) / kThreads), n);
    k_memo_diff<<<g, kThreads, 0, s>>>(d_in, m->d_old, npix, m->max_diff, m->d_flag);
    k_memo_copy<<<g, kThreads, 0, s>>>(d_in, m->d_old, npix, m->d_flag);
    m->launches += 2;
  } else {
    FCK(cudaMemsetAsync(m->d_flag, 0x01, sizeof(int) * n, s));
  }
  if (m->separable) {
    const dim3 g((m->C + kTC - 1) / kTC, (m->R + kSlowTR - 1) / kSlowTR, n);
    if (m->ff) {
      k_conv_fast_ff<<<dim3(m->R, n), kThreads, m->smem_fast, s>>>(d_in, m->d_tmp, m->R, m->C, m->d_wb_ff,
                                                                  m->b0, m->nb, m->d_flag);
      k_conv_slow_ff<<<g, dim3(kTC, kThreads / kTC), m->smem_slow, s>>>(m->d_tmp, m->d_last, m->R, m->C,
                                                                         m->d_wa_ff, m->a0, m->na, m->d_flag);
    } else {
      k_conv_fast<<<dim3(m->R, n), kThreads, m->smem_fast, s>>>(d_in, m->d_tmp, m->R, m->C, m->d_wb,
                                                               m->b0, m->nb, m->d_flag);
      k_conv_slow<<<g, dim3(kTC, kThreads / kTC), m->smem_slow, s>>>(m->d_tmp, m->d_last, m->R, m->C,
                                                                      m->d_wa, m->a0, m->na, m->d_flag);
    }
    m->launches += 2;
  } else {
    const dim3 g((m->C + kTC - 1) / kTC, (m->R + k2dTR - 1) / k2dTR, n);
    k_conv_2d<<<g, dim3(kTC, kThreads / kTC), m->smem_2d, s>>>(d_in, m->d_last, m->R, m->C, m->d_w2,
                                                                m->a0, m->na, m->b0, m->nb, m->d_flag);
    m->launches += 1;
  }
  FCK(cudaGetLastError());
  return 0;
}

// Host analysis of a recentred PSF (R x C): the smallest circular support
// along each axis (offsets a0 .. a0 + na - 1 along rows, b0 .. b0 + nb - 1
// along columns) and whether the PSF is rank 1 to 1e-12 of its maximum
// (then psf[a][b] = u[a - a0] * v[b - b0], from its pivot row and column).
struct PsfTaps {
  int a0 = 0, na = 1, b0 = 0, nb = 1, separable = 1;
  std::vector<double> u, v;
};

PsfTaps analyze_psf(const std::vector<double>& p, int R, int C) {
  PsfTaps t;
  std::vector<char> rnz(R, 0), cnz(C, 0);
  double pmax = 0.0;
  int pr = 0, pc = 0;
  for (int r = 0; r < R; ++r)
    for (int c = 0; c < C; ++c) {
      const double v = p[(size_t)r * C + c];
      if (v != 0.0) {
        rnz[r] = 1;
        cnz[c] = 1;
      }
      if (std::fabs(v) > pmax) {
        pmax = std::fabs(v);
        pr = r;
        pc = c;
      }
    }
  int a0, na, b0, nb;
  circular_support(rnz, R, &a0, &na);
  circular_support(cnz, C, &b0, &nb);
  if (na == 0) {   // an all-zero PSF: one zero tap
    a0 = b0 = 0;
    na = nb = 1;
  }
  auto at = [&](int a, int b) { return p[(size_t)(((a % R) + R) % R) * C + ((b % C) + C) % C]; };
  // rank-1 test against the pivot row and column
  t.u.assign(na, 0.0);
  t.v.assign(nb, 0.0);
  const double piv = at(pr, pc);
  for (int i = 0; i < na; ++i) t.u[i] = at(a0 + i, pc);
  for (int j = 0; j < nb; ++j) t.v[j] = piv != 0.0 ? at(pr, b0 + j) / piv : 0.0;
  double resid = 0.0;
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < nb; ++j) resid = std::max(resid, std::fabs(at(a0 + i, b0 + j) - t.u[i] * t.v[j]));
  t.separable = resid <= 1e-12 * pmax;
  t.a0 = a0;
  t.na = na;
  t.b0 = b0;
  t.nb = nb;
  return t;
}

MFilter* filter_create(const double* psf, double max_diff, int R, int C) {
  if (!psf || R < 1 || C < 1) {
    ferr("saFilterCreate: bad arguments (psf %p, %d x %d)", (const void*)psf, R, C);
    return nullptr;
  }
  MFilter* m = new MFilter();
  m->R = R;
  m->C = C;
  m->max_diff = max_diff > 0.0 ? max_diff : 0.0;
  m->h_rc.assign(psf, psf + (size_t)R * C);
  const std::vector<double>& p = m->h_rc;
  const PsfTaps taps = analyze_psf(p, R, C);
  const std::vector<double>& u = taps.u;
  const std::vector<double>& v = taps.v;
  const int a0 = taps.a0, na = taps.na, b0 = taps.b0, nb = taps.nb;
  auto at = [&](int a, int b) { return p[(size_t)(((a % R) + R) % R) * C + ((b % C) + C) % C]; };
  m->separable = taps.separable;
  m->a0 = a0;
  m->na = na;
  m->b0 = b0;
  m->nb = nb;
  bool ok = true, reported = false;
  if (m->separable) {
    m->smem_fast = sizeof(double) * (size_t)(2 * nb + C - 1);
    m->smem_slow = sizeof(double) * (size_t)(na + (kSlowTR + na - 1) * kTC);
    if (m->smem_fast > kSmemMax || m->smem_slow > kSmemMax) {
      ferr("saFilterCreate: a %d x %d image with a %d x %d tap PSF exceeds the shared-memory tile", R, C,
           na, nb);
      ok = false;
      reported = true;
    }
    // float-pair copies of the taps (hi = nearest float, lo = nearest float
    // of the remainder)
    auto split = [](const std::vector<double>& a) {
      std::vector<float2> o(a.size());
      for (size_t k = 0; k < a.size(); ++k) {
        const float h = (float)a[k];
        o[k] = make_float2(h, (float)(a[k] - (double)h));
      }
      return o;
    };
    const std::vector<float2> uf = split(u), vf = split(v);
    const char* env = getenv("SA_FINDER_FP64");
    m->ff = !(env && env[0] == '1');
    ok = ok && cudaMalloc(&m->d_wa, sizeof(double) * na) == cudaSuccess &&
         cudaMalloc(&m->d_wb, sizeof(double) * nb) == cudaSuccess &&
         cudaMalloc(&m->d_wa_ff, sizeof(float2) * na) == cudaSuccess &&
         cudaMalloc(&m->d_wb_ff, sizeof(float2) * nb) == cudaSuccess &&
         cudaMemcpy(m->d_wa, u.data(), sizeof(double) * na, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(m->d_wb, v.data(), sizeof(double) * nb, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(m->d_wa_ff, uf.data(), sizeof(float2) * na, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(m->d_wb_ff, vf.data(), sizeof(float2) * nb, cudaMemcpyHostToDevice) == cudaSuccess;
  } else {
    m->smem_2d = sizeof(double) * (size_t)(na * nb + (k2dTR + na - 1) * (kTC + nb - 1));
    if (m->smem_2d > kSmemMax) {
      ferr("saFilterCreate: the PSF is not separable and its support (%d x %d) is too large for "
           "direct convolution", na, nb);
      ok = false;
      reported = true;
    }
    std::vector<double> w((size_t)na * nb);
    for (int i = 0; i < na; ++i)
      for (int j = 0; j < nb; ++j) w[(size_t)i * nb + j] = at(a0 + i, b0 + j);
    ok = ok && cudaMalloc(&m->d_w2, sizeof(double) * w.size()) == cudaSuccess &&
         cudaMemcpy(m->d_w2, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  }
  ok = ok && cudaFuncSetAttribute(k_conv_fast, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax) == cudaSuccess &&
       cudaFuncSetAttribute(k_conv_fast_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax) == cudaSuccess &&
       cudaFuncSetAttribute(k_conv_slow_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax) == cudaSuccess &&
       cudaFuncSetAttribute(k_conv_slow, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax) == cudaSuccess &&
       cudaFuncSetAttribute(k_conv_2d, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemMax) == cudaSuccess &&
       cudaMalloc(&m->d_io, sizeof(double) * (size_t)R * C) == cudaSuccess &&
       cudaMalloc(&m->d_io2, sizeof(double) * (size_t)R * C) == cudaSuccess;
  if (!ok) {
    if (!reported) ferr("saFilterCreate: device set-up failed: %s", cudaGetErrorString(cudaGetLastError()));
    filter_free(m);
    delete m;
    return nullptr;
  }
  return m;
}

int filter_host(MFilter* m, const double* image, double* result, int memo) {
  if (!m || !image || !result) {
    ferr("convolve: NULL argument");
    return -1;
  }
  const size_t bytes = sizeof(double) * (size_t)m->R * m->C;
  FCK(cudaMemcpyAsync(m->d_io, image, bytes, cudaMemcpyHostToDevice, m->stream));
  if (filter_run(m, m->d_io, 1, memo, m->stream)) return -1;
  FCK(cudaMemcpyAsync(result, m->d_last, bytes, cudaMemcpyDeviceToHost, m->stream));
  FCK(cudaStreamSynchronize(m->stream));
  return 0;
}

// ---------------------------------------------------------------------------
// Local maxima
// ---------------------------------------------------------------------------

struct Maxima {
  int margin = 0, z_range = 0, Z = 1, n_dup = 1;
  double radius = 0.0, threshold = 0.0;
  double* d_zvalues = nullptr;
  int R = 0, C = 0, W = 0, F = 0;
  int32_t* d_taken = nullptr;
  uint32_t* d_bits = nullptr;
  int32_t* d_rowcnt = nullptr;
  int32_t* d_rowoff = nullptr;
  int32_t* d_fcount = nullptr;
  int32_t* h_fcount = nullptr;   // pinned, F + 1
  double* d_out = nullptr;
  int out_cap = 0, n_out = 0;
  double* d_stage = nullptr;   // host images staged for saMaximaFind
  size_t stage_bytes = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
};

void maxima_free(Maxima* h) {
  dfree(h->d_stage);
  dfree(h->d_zvalues);
  dfree(h->d_taken);
  dfree(h->d_bits);
  dfree(h->d_rowcnt);
  dfree(h->d_rowoff);
  dfree(h->d_fcount);
  dfree(h->d_out);
  if (h->h_fcount) cudaFreeHost(h->h_fcount);
  h->h_fcount = nullptr;
}

LMax lmax_args(const Maxima* h, const double* d_img, int n) {
  LMax a;
  a.img = d_img;
  a.taken = h->d_taken;
  a.bits = h->d_bits;
  a.rowcnt = h->d_rowcnt;
  a.R = h->R;
  a.C = h->C;
  a.Z = h->Z;
  a.W = h->W;
  a.nrows = n * h->Z * h->R;
  a.margin = h->margin;
  a.z_range = h->z_range;
  a.rr = (int)(h->radius * h->radius);
  a.cr = (int)std::ceil(h->radius);
  a.radius = h->radius;
  a.threshold = h->threshold;
  return a;
}

int maxima_reset(Maxima* h, cudaStream_t s) {
  if (h->F < 1) return 0;
  const size_t n = (size_t)h->F * h->Z * h->R * h->C;
  k_fill_i32<<<grid_for(n), kThreads, 0, s>>>(h->d_taken, n, 1 - h->n_dup);
  h->launches += 1;
  FCK(cudaGetLastError());
  return 0;
}

// Size the per-frame state for n frames of R x C (taken starts at
// 1 - n_duplicates; frames keep their counts when the set grows).
int maxima_frames(Maxima* h, int R, int C, int n, cudaStream_t s) {
  if (h->F > 0 && (R != h->R || C != h->C)) {
    ferr("maxima finder: image size changed from %d x %d to %d x %d", h->R, h->C, R, C);
    return -1;
  }
  if (n <= h->F) return 0;
  const int W = (C + 31) / 32;
  const size_t per = (size_t)h->Z * R;
  int32_t *taken = nullptr, *rowcnt = nullptr, *rowoff = nullptr, *fcount = nullptr, *hf = nullptr;
  uint32_t* bits = nullptr;
  FCK(cudaMalloc(&taken, sizeof(int32_t) * per * C * n));
  FCK(cudaMalloc(&bits, sizeof(uint32_t) * per * W * n));
  FCK(cudaMalloc(&rowcnt, sizeof(int32_t) * per * n));
  FCK(cudaMalloc(&rowoff, sizeof(int32_t) * per * n));
  FCK(cudaMalloc(&fcount, sizeof(int32_t) * (n + 1)));
  FCK(cudaMallocHost(&hf, sizeof(int32_t) * (n + 1)));
  FCK(cudaStreamSynchronize(s));
  const size_t old = (size_t)h->F * per * C;
  if (h->F > 0) FCK(cudaMemcpy(taken, h->d_taken, sizeof(int32_t) * old, cudaMemcpyDeviceToDevice));
  const size_t fresh = per * C * n - old;
  k_fill_i32<<<grid_for(fresh), kThreads, 0, s>>>(taken + old, fresh, 1 - h->n_dup);
  h->launches += 1;
  FCK(cudaGetLastError());
  dfree(h->d_taken);
  dfree(h->d_bits);
  dfree(h->d_rowcnt);
  dfree(h->d_rowoff);
  dfree(h->d_fcount);
  if (h->h_fcount) cudaFreeHost(h->h_fcount);
  h->d_taken = taken;
  h->d_bits = bits;
  h->d_rowcnt = rowcnt;
  h->d_rowoff = rowoff;
  h->d_fcount = fcount;
  h->h_fcount = hf;
  h->R = R;
  h->C = C;
  h->W = W;
  h->F = n;
  return 0;
}

// Mark, scan and read back the counts of n frames; returns the total.
int maxima_mark(Maxima* h, const double* d_img, int n, cudaStream_t s) {
  const LMax a = lmax_args(h, d_img, n);
  const int warps_per_block = kThreads / 32;
  const int blocks = (a.nrows + warps_per_block - 1) / warps_per_block;
  k_lmax_mark<<<blocks, kThreads, 0, s>>>(a);
  k_lmax_scan<<<1, 1024, 0, s>>>(h->d_rowcnt, h->d_rowoff, a.nrows, h->Z * h->R, n, h->d_fcount);
  h->launches += 2;
  FCK(cudaGetLastError());
  FCK(cudaMemcpyAsync(h->h_fcount, h->d_fcount, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost, s));
  FCK(cudaStreamSynchronize(s));
  return h->h_fcount[n];
}

int maxima_emit(Maxima* h, const double* d_img, int n, int cap, double sigma, cudaStream_t s) {
  if (cap > h->out_cap) {
    dfree(h->d_out);
    const int want = std::max(cap, 1024);
    FCK(cudaMalloc(&h->d_out, sizeof(double) * 4 * (size_t)want));
    h->out_cap = want;
  }
  const LMax a = lmax_args(h, d_img, n);
  const int warps_per_block = kThreads / 32;
  const int blocks = (a.nrows + warps_per_block - 1) / warps_per_block;
  k_lmax_emit<<<blocks, kThreads, 0, s>>>(a, h->d_rowoff, h->d_zvalues, h->d_out, cap, sigma);
  h->launches += 1;
  FCK(cudaGetLastError());
  h->n_out = cap;
  return 0;
}

// Find: mark + scan + emit every found peak; counts per frame to host.
int maxima_find(Maxima* h, const double* d_img, int R, int C, int n, int32_t* counts, double sigma,
                cudaStream_t s) {
  if (maxima_frames(h, R, C, n, s)) return -1;
  const int total = maxima_mark(h, d_img, n, s);
  if (total < 0) return -1;
  if (counts)
    for (int f = 0; f < n; ++f) counts[f] = h->h_fcount[f];
  if (maxima_emit(h, d_img, n, total, sigma, s)) return -1;
  // the peak rows are complete when this returns: callers hand them to work
  // on other streams (the fitter's)
  FCK(cudaStreamSynchronize(s));
  return total;
}

Maxima* maxima_create(int margin, int z_range, double radius, double threshold, const double* z_values,
                      int n_planes, int n_dup) {
  if (n_planes < 1 || !z_values) {
    ferr("saMaximaCreate: need at least one plane and its z value");
    return nullptr;
  }
  Maxima* h = new Maxima();
  h->margin = margin;
  h->z_range = z_range;
  h->radius = radius;
  h->threshold = threshold;
  h->Z = n_planes;
  h->n_dup = n_dup;
  if (cudaMalloc(&h->d_zvalues, sizeof(double) * n_planes) != cudaSuccess ||
      cudaMemcpy(h->d_zvalues, z_values, sizeof(double) * n_planes, cudaMemcpyHostToDevice) != cudaSuccess) {
    ferr("saMaximaCreate: device allocation failed");
    maxima_free(h);
    delete h;
    return nullptr;
  }
  return h;
}

// ---------------------------------------------------------------------------
// Fused Gaussian finder
// ---------------------------------------------------------------------------

struct Finder {
  int R = 0, C = 0, F = 0;
  MFilter* bg = nullptr;
  std::vector<MFilter*> fms, fvs;   // per plane: foreground filter and PSF-squared filter (may be empty)
  int Z = 1;                        // planes (z values) of the maxima search
  int abs_fit = 0;                  // |fit| in the variance (arbitrary-PSF finder)
  Maxima* mx = nullptr;
  double sigma = 1.0;
  double* d_image = nullptr;    // F x R x C
  double* d_bgest = nullptr;    // F x R x C: a given background (bg_estimate)
  const double* d_background = nullptr;   // the current background (bg->d_last or d_bgest)
  double* d_a = nullptr;        // F x R x C scratch (bg_var / image - fit)
  double* d_b = nullptr;        // F x R x C scratch (foreground)
  double* d_ratio = nullptr;    // F x Z x R x C: masked foreground / noise per plane
  double* d_fit = nullptr;      // F x R x C staging of a host fit image
  double* d_camvar = nullptr;   // R x C
  double* d_mask = nullptr;     // R x C
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  int n_peaks = 0;
};

void finder_free_frames(Finder* h) {
  dfree(h->d_image);
  dfree(h->d_bgest);
  dfree(h->d_a);
  dfree(h->d_b);
  dfree(h->d_ratio);
  dfree(h->d_fit);
}

int finder_frames(Finder* h, int n) {
  if (n <= h->F) return 0;
  FCK(cudaStreamSynchronize(h->stream));
  finder_free_frames(h);
  const size_t bytes = sizeof(double) * (size_t)h->R * h->C * n;
  FCK(cudaMalloc(&h->d_image, bytes));
  FCK(cudaMalloc(&h->d_a, bytes));
  FCK(cudaMalloc(&h->d_b, bytes));
  FCK(cudaMalloc(&h->d_ratio, bytes * h->Z));
  h->d_background = nullptr;
  h->F = n;
  return 0;
}

// A per-frame array argument: device pointers are used as they are, host
// arrays are staged into dst.
const double* finder_input(Finder* h, const double* p, int on_device, double** dst, int n) {
  if (!p || on_device) return p;
  const size_t bytes = sizeof(double) * (size_t)h->R * h->C * n;
  if (!*dst && cudaMalloc(dst, sizeof(double) * (size_t)h->R * h->C * h->F) != cudaSuccess) {
    ferr("peak finder: device allocation failed");
    return nullptr;
  }
  if (cudaMemcpyAsync(*dst, p, bytes, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) {
    ferr("peak finder: host-to-device copy failed");
    return nullptr;
  }
  return *dst;
}

// Device arrays of the culling entry points (host arrays in and out),
// kept per thread and grown on demand so that a call allocates nothing in
// the steady state.
struct CullBuf {
  double* d = nullptr;    // x, y, value (3 n) + query x, y (2 nq)
  int32_t* i = nullptr;   // status in/out (2 n), marked (n), items (n), counts/starts/cursor (3 T), misc (8)
  double* dq = nullptr;   // nearest distances (nq)
  size_t cap_d = 0, cap_i = 0, cap_q = 0;
  int n = 0, nq = 0, T = 0;
};

CullBuf& cull_buf() {
  static thread_local CullBuf b;
  return b;
}

template <typename P>
int grow(P*& p, size_t* cap, size_t want) {
  if (want <= *cap) return 0;
  dfree(p);
  FCK(cudaMalloc(&p, sizeof(P) * want));
  *cap = want;
  return 0;
}

int table_size(int n) {
  int T = 1024;
  while (T < 2 * n && T < (1 << 26)) T <<= 1;
  return T;
}

// Build the bucket grid of points (x, y) (device) with cells of width >= r.
int build_grid(const double* x, const double* y, int n, double r, int T, int32_t* counts, int32_t* starts,
               int32_t* cursor, int32_t* items, int32_t* total2, PointGrid* g) {
  const double cs = std::max(r * (1.0 + 1e-9), 1e-6);
  FCK(cudaMemsetAsync(counts, 0, sizeof(int32_t) * T, 0));
  FCK(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * T, 0));
  if (n > 0) k_grid_count<<<grid_for(n), kThreads>>>(x, y, n, cs, T, counts);
  k_lmax_scan<<<1, 1024>>>(counts, starts, T, T, 1, total2);
  if (n > 0) k_grid_fill<<<grid_for(n), kThreads>>>(x, y, n, cs, T, starts, cursor, items);
  FCK(cudaGetLastError());
  g->x = x;
  g->y = y;
  g->start = starts;
  g->total = total2 + 1;
  g->items = items;
  g->T = T;
  g->cs = cs;
  return 0;
}

// Points + values + statuses to the device, grid built, for the host-array
// culling entry points.
int cull_setup(CullBuf& b, int n, int nq, const double* x, const double* y, const double* v, const int32_t* status,
               const double* qx, const double* qy, double r, PointGrid* g) {
  b.n = n;
  b.nq = nq;
  b.T = table_size(n);
  const size_t nd = 3 * (size_t)n + 2 * (size_t)nq + 2, ni = 4 * (size_t)std::max(n, nq) + 3 * (size_t)b.T + 8;
  if (grow(b.d, &b.cap_d, nd) || grow(b.i, &b.cap_i, ni) || grow(b.dq, &b.cap_q, (size_t)nq + 1)) return -1;
  double *dx = b.d, *dy = b.d + n, *dv = b.d + 2 * n, *qxd = b.d + 3 * n, *qyd = qxd + nq;
  if (n > 0) {
    FCK(cudaMemcpy(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice));
    FCK(cudaMemcpy(dy, y, sizeof(double) * n, cudaMemcpyHostToDevice));
    if (v) FCK(cudaMemcpy(dv, v, sizeof(double) * n, cudaMemcpyHostToDevice));
  }
  if (nq > 0) {
    FCK(cudaMemcpy(qxd, qx, sizeof(double) * nq, cudaMemcpyHostToDevice));
    FCK(cudaMemcpy(qyd, qy, sizeof(double) * nq, cudaMemcpyHostToDevice));
  }
  const int m = std::max(n, nq);
  int32_t* st_in = b.i;
  if (status && m > 0) FCK(cudaMemcpy(st_in, status, sizeof(int32_t) * m, cudaMemcpyHostToDevice));
  int32_t* items = b.i + 3 * (size_t)m;
  int32_t* counts = b.i + 4 * (size_t)m;
  int32_t* starts = counts + b.T;
  int32_t* cursor = starts + b.T;
  int32_t* misc = cursor + b.T;
  FCK(cudaMemset(misc, 0, sizeof(int32_t) * 8));
  return build_grid(dx, dy, n, r, b.T, counts, starts, cursor, items, misc, g);
}

struct Ingest {
  int rows = 0, cols = 0, pad = 0, clip = 1;
  double off0 = 0.0, sc0 = 1.0;
  double* d_offset = nullptr;   // rows x cols, or none
  double* d_scale = nullptr;    // rows x cols, or none
  void* d_raw = nullptr;        // staging of host frames
  size_t raw_bytes = 0;
  double* d_out = nullptr;      // frames x (rows + 2 pad) x (cols + 2 pad)
  size_t out_bytes = 0;
  int n_frames = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
};

void ingest_free(Ingest* h) {
  dfree(h->d_offset);
  dfree(h->d_scale);
  dfree(h->d_raw);
  dfree(h->d_out);
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

int saFilterAnalyze(const double* psf, int x_size, int y_size, int32_t* out5, double* u, double* v) {
  if (!psf || !out5 || x_size < 1 || y_size < 1) {
    ferr("saFilterAnalyze: bad arguments");
    return -1;
  }
  const std::vector<double> p(psf, psf + (size_t)x_size * y_size);
  const PsfTaps t = analyze_psf(p, x_size, y_size);
  out5[0] = t.separable;
  out5[1] = t.na;
  out5[2] = t.nb;
  out5[3] = t.a0;
  out5[4] = t.b0;
  if (u) std::copy(t.u.begin(), t.u.end(), u);
  if (v) std::copy(t.v.begin(), t.v.end(), v);
  return 0;
}

void* saFilterCreate(const double* psf, double max_diff, int x_size, int y_size, int estimate) {
  (void)estimate;
  return filter_create(psf, max_diff, x_size, y_size);
}

int saFilterConvolve(void* flt, const double* image, double* result) {
  return filter_host(static_cast<MFilter*>(flt), image, result, 0);
}

int saFilterConvolveMemo(void* flt, const double* image, double* result) {
  return filter_host(static_cast<MFilter*>(flt), image, result, 1);
}

void saFilterCleanup(void* flt) {
  MFilter* m = static_cast<MFilter*>(flt);
  if (!m) return;
  cudaStreamSynchronize(m->stream);
  filter_free(m);
  delete m;
}

int saFilterConvolveDevice(void* flt, const double* d_images, int n_frames, int memo, double* d_result) {
  MFilter* m = static_cast<MFilter*>(flt);
  if (!m || !d_images || n_frames < 1) {
    ferr("saFilterConvolveDevice: bad arguments");
    return -1;
  }
  if (filter_run(m, d_images, n_frames, memo, m->stream)) return -1;
  if (d_result)
    FCK(cudaMemcpyAsync(d_result, m->d_last, sizeof(double) * (size_t)m->R * m->C * n_frames,
                        cudaMemcpyDeviceToDevice, m->stream));
  return 0;
}

const double* saFilterResultDevice(void* flt) {
  MFilter* m = static_cast<MFilter*>(flt);
  return m ? m->d_last : nullptr;
}

int saFilterInfo(void* flt, int32_t* out6) {
  MFilter* m = static_cast<MFilter*>(flt);
  if (!m || !out6) return -1;
  out6[0] = m->separable ? (m->ff ? 2 : 1) : 0;
  out6[1] = m->na;
  out6[2] = m->nb;
  out6[3] = m->a0;
  out6[4] = m->b0;
  out6[5] = m->F;
  return 0;
}

int saFilterSetStream(void* flt, void* stream) {
  MFilter* m = static_cast<MFilter*>(flt);
  if (!m) return -1;
  m->stream = static_cast<cudaStream_t>(stream);
  return 0;
}

int saCalcMaxPeaks(saFlmData* flm) {
  if (!flm || !flm->images || !flm->taken || flm->zsize < 1) {
    ferr("calcMaxPeaks: bad flmData");
    return -1;
  }
  const int Z = flm->zsize, R = flm->ysize, C = flm->xsize;
  const size_t plane = (size_t)R * C;
  double* d_img = nullptr;
  int32_t *d_taken = nullptr, *d_count = nullptr;
  int n = -1;
  if (cudaMalloc(&d_img, sizeof(double) * plane * Z) == cudaSuccess &&
      cudaMalloc(&d_taken, sizeof(int32_t) * plane * Z) == cudaSuccess &&
      cudaMalloc(&d_count, sizeof(int32_t)) == cudaSuccess) {
    bool ok = cudaMemset(d_count, 0, sizeof(int32_t)) == cudaSuccess;
    for (int z = 0; ok && z < Z; ++z)
      ok = cudaMemcpy(d_img + plane * z, flm->images[z], sizeof(double) * plane, cudaMemcpyHostToDevice) ==
               cudaSuccess &&
           cudaMemcpy(d_taken + plane * z, flm->taken[z], sizeof(int32_t) * plane,
                      cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok) {
      LMax a{};
      a.img = d_img;
      a.taken = d_taken;
      a.R = R;
      a.C = C;
      a.Z = Z;
      a.nrows = Z * R;
      a.margin = flm->margin;
      a.threshold = flm->threshold;
      k_lmax_count<<<grid_for(plane * Z), kThreads>>>(a, d_count);
      int32_t hc = 0;
      if (cudaGetLastError() == cudaSuccess &&
          cudaMemcpy(&hc, d_count, sizeof(int32_t), cudaMemcpyDeviceToHost) == cudaSuccess)
        n = hc;
    }
  }
  if (n < 0) ferr("calcMaxPeaks: device step failed: %s", cudaGetErrorString(cudaGetLastError()));
  dfree(d_img);
  dfree(d_taken);
  dfree(d_count);
  return n;
}

void saFindLocalMaxima(saFlmData* flm, double* z, double* y, double* x, double* h) {
  if (!flm || !flm->images || !flm->taken || !flm->z_values || flm->zsize < 1 || !z || !y || !x || !h) {
    ferr("findLocalMaxima: bad flmData");
    return;
  }
  const int Z = flm->zsize, R = flm->ysize, C = flm->xsize;
  const size_t plane = (size_t)R * C;
  Maxima* mh = maxima_create(flm->margin, flm->z_range, flm->radius, flm->threshold, flm->z_values, Z, 1);
  if (!mh) return;
  double* d_img = nullptr;
  bool ok = cudaMalloc(&d_img, sizeof(double) * plane * Z) == cudaSuccess && maxima_frames(mh, R, C, 1, 0) == 0;
  for (int k = 0; ok && k < Z; ++k)
    ok = cudaMemcpy(d_img + plane * k, flm->images[k], sizeof(double) * plane, cudaMemcpyHostToDevice) ==
             cudaSuccess &&
         cudaMemcpy(mh->d_taken + plane * k, flm->taken[k], sizeof(int32_t) * plane,
                    cudaMemcpyHostToDevice) == cudaSuccess;
  int total = ok ? maxima_mark(mh, d_img, 1, 0) : -1;
  ok = total >= 0;
  const int cap = ok ? std::min(total, std::max(flm->n_peaks, 0)) : 0;
  if (ok && flm->n_peaks > 0 && total >= flm->n_peaks) printf("Warning! Found maximum number of peaks!\n");
  ok = ok && maxima_emit(mh, d_img, 1, cap, 0.0, 0) == 0;
  std::vector<double> rows((size_t)cap * 4);
  if (ok && cap > 0)
    ok = cudaMemcpy(rows.data(), mh->d_out, sizeof(double) * rows.size(), cudaMemcpyDeviceToHost) == cudaSuccess;
  for (int k = 0; ok && k < Z; ++k)
    ok = cudaMemcpy(flm->taken[k], mh->d_taken + plane * k, sizeof(int32_t) * plane,
                    cudaMemcpyDeviceToHost) == cudaSuccess;
  if (ok) {
    for (int i = 0; i < cap; ++i) {
      x[i] = rows[4 * i];
      y[i] = rows[4 * i + 1];
      z[i] = rows[4 * i + 2];
      h[i] = rows[4 * i + 3];
    }
    flm->n_peaks = cap;
  } else {
    ferr("findLocalMaxima: device step failed: %s", cudaGetErrorString(cudaGetLastError()));
  }
  dfree(d_img);
  maxima_free(mh);
  delete mh;
}

void* saMaximaCreate(int margin, int z_range, double radius, double threshold, const double* z_values,
                     int n_planes, int n_duplicates) {
  return maxima_create(margin, z_range, radius, threshold, z_values, n_planes, n_duplicates);
}

int saMaximaFind(void* mh, const double* images, int on_device, int rows, int cols, int n_frames,
                 int32_t* counts, double sigma) {
  Maxima* h = static_cast<Maxima*>(mh);
  if (!h || !images || rows < 1 || cols < 1 || n_frames < 1) {
    ferr("saMaximaFind: bad arguments");
    return -1;
  }
  const double* d_img = images;
  if (!on_device) {
    const size_t bytes = sizeof(double) * (size_t)n_frames * h->Z * rows * cols;
    if (bytes > h->stage_bytes) {
      dfree(h->d_stage);
      FCK(cudaMalloc(&h->d_stage, bytes));
      h->stage_bytes = bytes;
    }
    FCK(cudaMemcpyAsync(h->d_stage, images, bytes, cudaMemcpyHostToDevice, h->stream));
    d_img = h->d_stage;
  }
  return maxima_find(h, d_img, rows, cols, n_frames, counts, sigma, h->stream);
}

const double* saMaximaPeaksDevice(void* mh) {
  Maxima* h = static_cast<Maxima*>(mh);
  return h ? h->d_out : nullptr;
}

int saMaximaGetPeaks(void* mh, double* rows) {
  Maxima* h = static_cast<Maxima*>(mh);
  if (!h || !rows) return -1;
  if (h->n_out > 0) {
    FCK(cudaMemcpyAsync(rows, h->d_out, sizeof(double) * 4 * (size_t)h->n_out, cudaMemcpyDeviceToHost,
                        h->stream));
    FCK(cudaStreamSynchronize(h->stream));
  }
  return h->n_out;
}

int saMaximaResetTaken(void* mh) {
  Maxima* h = static_cast<Maxima*>(mh);
  if (!h) return -1;
  return maxima_reset(h, h->stream);
}

int saMaximaGetTaken(void* mh, int32_t* taken) {
  Maxima* h = static_cast<Maxima*>(mh);
  if (!h || !taken) return -1;
  if (h->F > 0) {
    FCK(cudaMemcpyAsync(taken, h->d_taken, sizeof(int32_t) * (size_t)h->F * h->Z * h->R * h->C,
                        cudaMemcpyDeviceToHost, h->stream));
    FCK(cudaStreamSynchronize(h->stream));
  }
  return h->F;
}

int saMaximaSetStream(void* mh, void* stream) {
  Maxima* h = static_cast<Maxima*>(mh);
  if (!h) return -1;
  h->stream = static_cast<cudaStream_t>(stream);
  return 0;
}

void saMaximaCleanup(void* mh) {
  Maxima* h = static_cast<Maxima*>(mh);
  if (!h) return;
  cudaStreamSynchronize(h->stream);
  maxima_free(h);
  delete h;
}

int saMarkDimmerPeaks(double* x, double* y, double* h, int32_t* status, double r_removal, double r_neighbors,
                      int np) {
  if (np <= 0) return 0;
  if (!x || !y || !h || !status) {
    ferr("markDimmerPeaks: NULL argument");
    return -1;
  }
  CullBuf& b = cull_buf();
  PointGrid g;
  if (cull_setup(b, np, 0, x, y, h, status, nullptr, nullptr, std::max(r_removal, r_neighbors), &g)) return -1;
  int32_t* st_in = b.i;
  int32_t* st_out = b.i + np;
  int32_t* marked = b.i + 2 * (size_t)np;
  int32_t* misc = b.i + 4 * (size_t)np + 3 * (size_t)b.T;
  k_mark_dimmer<<<grid_for(np), kThreads>>>(g, b.d + 2 * np, st_in, np, r_removal, marked, misc + 4);
  k_mark_apply<<<grid_for(np), kThreads>>>(g, marked, st_in, st_out, np, r_neighbors);
  FCK(cudaGetLastError());
  int32_t removed = 0;
  FCK(cudaMemcpy(status, st_out, sizeof(int32_t) * np, cudaMemcpyDeviceToHost));
  FCK(cudaMemcpy(&removed, misc + 4, sizeof(int32_t), cudaMemcpyDeviceToHost));
  return removed;
}

int saMarkLowSignificancePeaks(double* x, double* y, double* sig, int32_t* status, double min_sig,
                               double r_neighbors, int np) {
  if (np <= 0) return 0;
  if (!x || !y || !sig || !status) {
    ferr("markLowSignificancePeaks: NULL argument");
    return -1;
  }
  CullBuf& b = cull_buf();
  PointGrid g;
  if (cull_setup(b, np, 0, x, y, sig, status, nullptr, nullptr, r_neighbors, &g)) return -1;
  int32_t* st_in = b.i;
  int32_t* st_out = b.i + np;
  int32_t* marked = b.i + 2 * (size_t)np;
  int32_t* misc = b.i + 4 * (size_t)np + 3 * (size_t)b.T;
  k_mark_low_sig<<<grid_for(np), kThreads>>>(b.d + 2 * np, st_in, np, min_sig, marked, misc + 4);
  k_mark_apply<<<grid_for(np), kThreads>>>(g, marked, st_in, st_out, np, r_neighbors);
  FCK(cudaGetLastError());
  int32_t removed = 0;
  FCK(cudaMemcpy(status, st_out, sizeof(int32_t) * np, cudaMemcpyDeviceToHost));
  FCK(cudaMemcpy(&removed, misc + 4, sizeof(int32_t), cudaMemcpyDeviceToHost));
  return removed;
}

void saRunningIfHasNeighbors(double* c_x, double* c_y, double* n_x, double* n_y, int32_t* status, double radius,
                             int nc, int nn) {
  if (nc <= 0 || nn <= 0) return;
  if (!c_x || !c_y || !n_x || !n_y || !status) {
    ferr("runningIfHasNeighbors: NULL argument");
    return;
  }
  CullBuf& b = cull_buf();
  PointGrid g;
  // grid over the new peaks, queries are the current peaks
  if (cull_setup(b, nn, nc, n_x, n_y, nullptr, nullptr, c_x, c_y, radius, &g)) return;
  int32_t* st = b.i;
  if (cudaMemcpy(st, status, sizeof(int32_t) * nc, cudaMemcpyHostToDevice) != cudaSuccess) {
    ferr("runningIfHasNeighbors: copy failed");
    return;
  }
  k_running_if_neighbors<<<grid_for(nc), kThreads>>>(g, b.d + 3 * nn, b.d + 3 * nn + nc, st, nc, radius);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpy(status, st, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost) != cudaSuccess)
    ferr("runningIfHasNeighbors: device step failed");
}

// The "kd-tree" of createKDTree / nearestKDTree is the point set itself;
// the grid is built per query radius.
struct PointSet {
  int n = 0;
  std::vector<double> x, y;
};

void* saCreateKDTree(double* x, double* y, int n) {
  if (n < 0 || (n > 0 && (!x || !y))) {
    ferr("createKDTree: bad arguments");
    return nullptr;
  }
  PointSet* p = new PointSet();
  p->n = n;
  p->x.assign(x, x + n);
  p->y.assign(y, y + n);
  return p;
}

void saFreeKDTree(void* kd) { delete static_cast<PointSet*>(kd); }

void saNearestKDTree(void* kd, double* x, double* y, double* dist, int32_t* index, double radius, int n) {
  PointSet* p = static_cast<PointSet*>(kd);
  if (!p || n <= 0) return;
  if (p->n == 0) {
    for (int i = 0; i < n; ++i) {
      dist[i] = -1.0;
      index[i] = -1;
    }
    return;
  }
  CullBuf& b = cull_buf();
  PointGrid g;
  if (cull_setup(b, p->n, n, p->x.data(), p->y.data(), nullptr, nullptr, x, y, radius, &g)) return;
  double* qx = b.d + 3 * (size_t)p->n;
  double* qy = qx + n;
  int32_t* di = b.i + 2 * (size_t)std::max(p->n, n);
  k_nearest<<<grid_for(n), kThreads>>>(g, qx, qy, n, radius, b.dq, di);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpy(dist, b.dq, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(index, di, sizeof(int32_t) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
    ferr("nearestKDTree: device step failed");
}

void* saIngestCreate(int rows, int cols, int pad, const double* offset, const double* scale, double offset0,
                     double scale0, int clip) {
  if (rows < 1 || cols < 1 || pad < 0 || pad > rows || pad > cols) {
    ferr("saIngestCreate: bad frame size %d x %d or padding %d (padding must not exceed the frame)", rows, cols,
         pad);
    return nullptr;
  }
  Ingest* h = new Ingest();
  h->rows = rows;
  h->cols = cols;
  h->pad = pad;
  h->clip = clip ? 1 : 0;
  h->off0 = offset0;
  h->sc0 = scale0;
  const size_t bytes = sizeof(double) * (size_t)rows * cols;
  bool ok = true;
  if (offset)
    ok = ok && cudaMalloc(&h->d_offset, bytes) == cudaSuccess &&
         cudaMemcpy(h->d_offset, offset, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  if (scale)
    ok = ok && cudaMalloc(&h->d_scale, bytes) == cudaSuccess &&
         cudaMemcpy(h->d_scale, scale, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    ferr("saIngestCreate: device set-up failed: %s", cudaGetErrorString(cudaGetLastError()));
    ingest_free(h);
    delete h;
    return nullptr;
  }
  return h;
}

int saIngestFrames(void* ih, const void* frames, int n_frames, int dtype_bits, int big_endian, int on_device,
                   double* d_out) {
  Ingest* h = static_cast<Ingest*>(ih);
  if (!h || !frames || n_frames < 1 || (dtype_bits != 16 && dtype_bits != 32 && dtype_bits != 64)) {
    ferr("saIngestFrames: bad arguments (dtype bits must be 16, 32 or 64)");
    return -1;
  }
  const size_t raw_bytes = (size_t)n_frames * h->rows * h->cols * (dtype_bits / 8);
  const void* src = frames;
  if (!on_device) {
    if (raw_bytes > h->raw_bytes) {
      FCK(cudaStreamSynchronize(h->stream));
      dfree(h->d_raw);
      FCK(cudaMalloc(&h->d_raw, raw_bytes));
      h->raw_bytes = raw_bytes;
    }
    FCK(cudaMemcpyAsync(h->d_raw, frames, raw_bytes, cudaMemcpyHostToDevice, h->stream));
    src = h->d_raw;
  }
  const int prow = h->rows + 2 * h->pad, pcol = h->cols + 2 * h->pad;
  double* out = d_out;
  if (!out) {
    const size_t ob = sizeof(double) * (size_t)n_frames * prow * pcol;
    if (ob > h->out_bytes) {
      FCK(cudaStreamSynchronize(h->stream));
      dfree(h->d_out);
      FCK(cudaMalloc(&h->d_out, ob));
      h->out_bytes = ob;
    }
    out = h->d_out;
  }
  const dim3 grid((unsigned)(((size_t)prow * pcol + kThreads - 1) / kThreads), n_frames);
  k_ingest<<<grid, kThreads, 0, h->stream>>>(src, dtype_bits, big_endian && dtype_bits == 16,
                                                        h->rows, h->cols, h->pad, h->d_offset, h->d_scale,
                                                        h->off0, h->sc0, h->clip, out);
  h->launches += 1;
  FCK(cudaGetLastError());
  h->n_frames = n_frames;
  return 0;
}

const double* saIngestResultDevice(void* ih) {
  Ingest* h = static_cast<Ingest*>(ih);
  return h ? h->d_out : nullptr;
}

int saIngestGetFrames(void* ih, double* out) {
  Ingest* h = static_cast<Ingest*>(ih);
  if (!h || !out || !h->d_out) return -1;
  const size_t n = (size_t)h->n_frames * (h->rows + 2 * h->pad) * (h->cols + 2 * h->pad);
  FCK(cudaMemcpyAsync(out, h->d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
  FCK(cudaStreamSynchronize(h->stream));
  return h->n_frames;
}

int saIngestSetStream(void* ih, void* stream) {
  Ingest* h = static_cast<Ingest*>(ih);
  if (!h) return -1;
  h->stream = static_cast<cudaStream_t>(stream);
  return 0;
}

int64_t saIngestKernelLaunches(void* ih) {
  Ingest* h = static_cast<Ingest*>(ih);
  return h ? h->launches : -1;
}

void saIngestCleanup(void* ih) {
  Ingest* h = static_cast<Ingest*>(ih);
  if (!h) return;
  cudaStreamSynchronize(h->stream);
  ingest_free(h);
  delete h;
}

void* saFinderCreate(int rows, int cols, void* bg_filter, void* fg_filter, void* fv_filter, int margin,
                     double radius, double threshold, double z_value, double sigma) {
  MFilter* bg = static_cast<MFilter*>(bg_filter);
  MFilter* fm = static_cast<MFilter*>(fg_filter);
  MFilter* fv = static_cast<MFilter*>(fv_filter);
  if (rows < 1 || cols < 1 || !bg || (!fm) != (!fv)) {
    ferr("saFinderCreate: need a background filter and both or neither foreground filters");
    return nullptr;
  }
  for (MFilter* m : {bg, fm, fv})
    if (m && (m->R != rows || m->C != cols)) {
      ferr("saFinderCreate: a filter is %d x %d, the frames %d x %d", m->R, m->C, rows, cols);
      return nullptr;
    }
  Maxima* mx = maxima_create(margin + 1, 1, radius, threshold, &z_value, 1, 1);
  if (!mx) return nullptr;
  Finder* h = new Finder();
  h->R = rows;
  h->C = cols;
  h->bg = bg;
  if (fm) {
    h->fms.push_back(fm);
    h->fvs.push_back(fv);
  }
  h->mx = mx;
  h->sigma = sigma;
  return h;
}

void* saFinderCreateArbitrary(int rows, int cols, void* bg_filter, int n_planes, void** fg_filters,
                              void** fv_filters, const double* z_values, int margin, double radius,
                              double threshold) {
  MFilter* bg = static_cast<MFilter*>(bg_filter);
  if (rows < 1 || cols < 1 || !bg || n_planes < 1 || !fg_filters || !fv_filters || !z_values) {
    ferr("saFinderCreateArbitrary: need a background filter and a foreground and PSF-squared filter per plane");
    return nullptr;
  }
  std::vector<MFilter*> fms(n_planes), fvs(n_planes);
  for (int z = 0; z < n_planes; ++z) {
    fms[z] = static_cast<MFilter*>(fg_filters[z]);
    fvs[z] = static_cast<MFilter*>(fv_filters[z]);
    for (MFilter* m : {fms[z], fvs[z], bg})
      if (!m || m->R != rows || m->C != cols) {
        ferr("saFinderCreateArbitrary: filter of plane %d missing or not %d x %d", z, rows, cols);
        return nullptr;
      }
  }
  // MaximaFinder(margin, radius, threshold, z_values): z_range = n_planes
  Maxima* mx = maxima_create(margin + 1, n_planes, radius, threshold, z_values, n_planes, 1);
  if (!mx) return nullptr;
  Finder* h = new Finder();
  h->R = rows;
  h->C = cols;
  h->bg = bg;
  h->fms = fms;
  h->fvs = fvs;
  h->Z = n_planes;
  h->abs_fit = 1;
  h->mx = mx;
  h->sigma = 0.0;
  return h;
}

int saFinderSetVariance(void* fh, const double* camera_variance) {
  Finder* h = static_cast<Finder*>(fh);
  if (!h) return -1;
  if (!camera_variance) {
    dfree(h->d_camvar);
    return 0;
  }
  const size_t bytes = sizeof(double) * (size_t)h->R * h->C;
  if (!h->d_camvar) FCK(cudaMalloc(&h->d_camvar, bytes));
  FCK(cudaMemcpyAsync(h->d_camvar, camera_variance, bytes, cudaMemcpyHostToDevice, h->stream));
  FCK(cudaStreamSynchronize(h->stream));
  return 0;
}

int saFinderSetMask(void* fh, const double* peak_mask) {
  Finder* h = static_cast<Finder*>(fh);
  if (!h) return -1;
  if (!peak_mask) {
    dfree(h->d_mask);
    return 0;
  }
  const size_t bytes = sizeof(double) * (size_t)h->R * h->C;
  if (!h->d_mask) FCK(cudaMalloc(&h->d_mask, bytes));
  FCK(cudaMemcpyAsync(h->d_mask, peak_mask, bytes, cudaMemcpyHostToDevice, h->stream));
  FCK(cudaStreamSynchronize(h->stream));
  return 0;
}

int saFinderNewImages(void* fh, const double* images, int n_frames, int on_device) {
  Finder* h = static_cast<Finder*>(fh);
  if (!h || !images || n_frames < 1) {
    ferr("saFinderNewImages: bad arguments");
    return -1;
  }
  if (h->F > 0 && n_frames != h->F) {
    ferr("saFinderNewImages: the handle holds %d frames, got %d", h->F, n_frames);
    return -1;
  }
  if (finder_frames(h, n_frames)) return -1;
  const size_t bytes = sizeof(double) * (size_t)h->R * h->C * n_frames;
  FCK(cudaMemcpyAsync(h->d_image, images, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                      h->stream));
  if (maxima_frames(h->mx, h->R, h->C, n_frames, h->stream)) return -1;
  if (maxima_reset(h->mx, h->stream)) return -1;
  h->d_background = nullptr;
  return 0;
}

int saFinderEstimateBackground(void* fh, const double* fit, const double* bg_estimate, int on_device) {
  Finder* h = static_cast<Finder*>(fh);
  if (!h || h->F < 1) {
    ferr("saFinderEstimateBackground: no images");
    return -1;
  }
  const int n = h->F;
  const size_t total = (size_t)h->R * h->C * n;
  if (bg_estimate) {
    const double* b = finder_input(h, bg_estimate, on_device, &h->d_bgest, n);
    if (!b) return -1;
    h->d_background = b;
    return 0;
  }
  const double* f = finder_input(h, fit, on_device, &h->d_fit, n);
  if (fit && !f) return -1;
  k_sub<<<grid_for(total), kThreads, 0, h->stream>>>(h->d_image, f, h->d_a, total);
  h->launches += 1;
  FCK(cudaGetLastError());
  const int64_t l0 = h->bg->launches;
  if (filter_run(h->bg, h->d_a, n, 1, h->stream)) return -1;
  h->launches += h->bg->launches - l0;
  h->d_background = h->bg->d_last;
  return 0;
}

int saFinderFindPeaks(void* fh, const double* fit, int on_device, int32_t* counts) {
  Finder* h = static_cast<Finder*>(fh);
  if (!h || h->F < 1 || !h->d_background) {
    ferr("saFinderFindPeaks: call saFinderNewImages and saFinderEstimateBackground first");
    return -1;
  }
  const int n = h->F, npix = h->R * h->C;
  const size_t total = (size_t)npix * n;
  const double* f = finder_input(h, fit, on_device, &h->d_fit, n);
  if (fit && !f) return -1;
  k_find_prep<<<grid_for(total), kThreads, 0, h->stream>>>(h->d_image, h->d_background, f, h->d_camvar, h->d_a,
                                                           h->d_b, npix, total, h->abs_fit);
  h->launches += 1;
  FCK(cudaGetLastError());
  for (int z = 0; z < h->Z; ++z) {
    const double* bgv = h->d_a;
    const double* fg = h->d_b;
    if (!h->fvs.empty()) {
      MFilter* fv = h->fvs[z];
      MFilter* fm = h->fms[z];
      const int64_t l0 = fv->launches + fm->launches;
      if (filter_run(fv, h->d_a, n, 1, h->stream)) return -1;
      if (filter_run(fm, h->d_b, n, 1, h->stream)) return -1;
      h->launches += fv->launches + fm->launches - l0;
      bgv = fv->d_last;
      fg = fm->d_last;
    }
    k_find_ratio<<<grid_for(total), kThreads, 0, h->stream>>>(fg, bgv, h->d_mask, h->d_ratio, npix, total, z, h->Z);
    h->launches += 1;
    FCK(cudaGetLastError());
  }
  const int64_t l0 = h->mx->launches;
  const int found = maxima_find(h->mx, h->d_ratio, h->R, h->C, n, counts, h->sigma, h->stream);
  h->launches += h->mx->launches - l0;
  if (found < 0) return -1;
  h->n_peaks = found;
  return found;
}

const double* saFinderBackgroundDevice(void* fh) {
  Finder* h = static_cast<Finder*>(fh);
  return h ? h->d_background : nullptr;
}

const double* saFinderPeaksDevice(void* fh) {
  Finder* h = static_cast<Finder*>(fh);
  return h ? h->mx->d_out : nullptr;
}

int saFinderGetPeaks(void* fh, double* rows) {
  Finder* h = static_cast<Finder*>(fh);
  if (!h) return -1;
  return saMaximaGetPeaks(h->mx, rows);
}

int saFinderGetArray(void* fh, int which, double* out) {
  Finder* h = static_cast<Finder*>(fh);
  if (!h || !out || h->F < 1) return -1;
  const double* src = which == 0 ? h->d_background : which == 1 ? h->d_ratio : nullptr;
  if (!src) {
    ferr("saFinderGetArray: nothing to return for %d", which);
    return -1;
  }
  const size_t planes = which == 1 ? (size_t)h->Z : 1;
  FCK(cudaMemcpyAsync(out, src, sizeof(double) * (size_t)h->R * h->C * h->F * planes, cudaMemcpyDeviceToHost,
                      h->stream));
  FCK(cudaStreamSynchronize(h->stream));
  return 0;
}

int saFinderSetStream(void* fh, void* stream) {
  Finder* h = static_cast<Finder*>(fh);
  if (!h) return -1;
  h->stream = static_cast<cudaStream_t>(stream);
  h->mx->stream = h->stream;
  return 0;
}

int64_t saFinderKernelLaunches(void* fh) {
  Finder* h = static_cast<Finder*>(fh);
  return h ? h->launches : -1;
}

void saFinderCleanup(void* fh) {
  Finder* h = static_cast<Finder*>(fh);
  if (!h) return;
  cudaStreamSynchronize(h->stream);
  finder_free_frames(h);
  dfree(h->d_camvar);
  dfree(h->d_mask);
  maxima_free(h->mx);
  delete h->mx;
  delete h;
}

}  // extern "C"
