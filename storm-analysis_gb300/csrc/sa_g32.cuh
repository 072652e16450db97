// sa_g32.cuh -- the LM step of one peak in the FP32 engine for the Gaussian
// models (2dfixed, 2d, 3d, Z); one warp per peak.
//
// Precision plan.  The step's Hessian, its FP32 LDL^T factor and the
// per-pixel model shape are FP32; what decides the step -- the gradient and
// the change of the MLE error between the start of the step and a trial --
// is carried in float-float ("ff", ~48 bits) from exact inputs:
//   * the fit image and a copy of the data are fixed point, so f - x is
//     exact and becomes an ff residual without rounding;
//   * the shape factors exp(-t^2 w) are evaluated in ff per ROI row and
//     column (2 * roi exponentials per table, ff_exp) and kept as ff pairs;
//   * the change of the error for a trial at the same ROI anchor is
//     summed per pixel as  df * t1 + 2 x (r - log1p r),  t1 = 2 (f0 - x)/f0,
//     r = df / f0, with df = h1 psf1 - h0 psf0 (+ background change) in ff:
//     the first-order term, whose pixel sum cancels near convergence, is ff;
//     the second-order term is positive and FP32.
// This keeps the accept / reject / converged decisions of the reference
// (multi_fit.c:1229-1318, evaluated there in FP64) except where they sit
// within ~1e-12 of a threshold.
#pragma once

#include "sa_device.cuh"

namespace sa {

enum { ACT_EVAL = 0, ACT_CONTINUE = 1, ACT_BREAK = 2, ACT_BREAK_ADDED = 3, ACT_ESCAPE = 4 };

// Per-axis Jacobian factors of pass 1 in tab1 (ff pairs, stride ts):
// a1 = 2 h wx t_x, a2 = -h t_x^2 (x gx for Z), b1 = 2 h wy t_y, b2 = -h t_y^2
// (x gy), so that with ps = rqe * psf the Jacobian row is
//   2dfixed [ps, ps a1, ps b1, rqe]            (dao_fit.c:48-105)
//   2d      [ps, ps a1, ps b1, ps (a2+b2), rqe] (:409-467)
//   3d      [ps, ps a1, ps a2, ps b1, ps b2, rqe] (:811-871)
//   Z       [ps, ps a1, ps b1, ps (a2+b2), rqe] (:883-958)
template <int M>
__device__ inline void g32_grad_tables(const ModelCfg& cfg, const float* par, float* g, int ts, int lane) {
  G32Axes ax;
  ax.xo = gpar(par, GP_XO);
  ax.yo = gpar(par, GP_YO);
  ax.wx = gpar(par, GP_WX);
  ax.wy = gpar(par, GP_WY);
  constexpr bool one_width = (M == M_2DFIXED) || (M == M_2D);
  const ff H = gpar(par, GP_H);
  const ff H2 = ff{2.0f * H.h, 2.0f * H.l};
  const ff HX = ff_mul(H2, ax.wx), HY = ff_mul(H2, one_width ? ax.wx : ax.wy);   // 2 h w
  const ff NX = (M == M_Z) ? ff_neg(ff_mul(H, gpar(par, GP_GX))) : ff_neg(H);
  const ff NY = (M == M_Z) ? ff_neg(ff_mul(H, gpar(par, GP_GY))) : ff_neg(H);
  for (int i = lane; i < cfg.roi; i += 32) {
    const ff tx = ff_add_f(ax.xo, (float)i), ty = ff_add_f(ax.yo, (float)i);
    ff v = ff_mul(HX, tx);
    g[i] = v.h;
    g[ts + i] = v.l;
    v = ff_mul(NX, ff_mul(tx, tx));
    g[2 * ts + i] = v.h;
    g[3 * ts + i] = v.l;
    v = ff_mul(HY, ty);
    g[4 * ts + i] = v.h;
    g[5 * ts + i] = v.l;
    v = ff_mul(NY, ff_mul(ty, ty));
    g[6 * ts + i] = v.h;
    g[7 * ts + i] = v.l;
  }
}

// The normal equations of a step as float-float values, in the memory of
// ws.jh: hi parts at [0, 36), lo parts at [36, 72); gradient first, then
// the packed upper Hessian (hes_index).
__device__ __forceinline__ float* g32_jh(WarpWS<float>& ws) { return reinterpret_cast<float*>(ws.jh); }

__device__ __forceinline__ ff shfl_ff(ff v, int src) {
  return ff{__shfl_sync(0xffffffffu, v.h, src), __shfl_sync(0xffffffffu, v.l, src)};
}

// The FP64 Cholesky of the ff normal equations (lane 0), the rare path of
// solve_g32 (an FP32 pivot <= 0), with the arithmetic of solve_fp64_lane0 /
// chol_solve.  Its matrix lives in shared scratch s (MAX_JAC^2 + MAX_JAC
// doubles; the factor overwrites the lower triangle) and its loops are not
// unrolled, so it adds no registers to the step; an out-of-line call would
// make the compiler save the step's live registers to the stack around it.
__device__ inline int solve_g32_fallback(const float* jh, int k, double lam, double* s, double* out) {
  double* A = s;
  double* b = s + MAX_JAC * MAX_JAC;
  int id = k;
#pragma unroll 1
  for (int l = 0; l < k; l++) {
    b[l] = (double)jh[l] + (double)jh[36 + l];
#pragma unroll 1
    for (int m = l; m < k; m++) {
      const double v = (double)jh[id] + (double)jh[36 + id];
      A[l * MAX_JAC + m] = (l == m) ? (1.0 + lam) * v : v;
      id++;
    }
  }
#pragma unroll 1
  for (int j = 0; j < k; j++) {
    double d = A[j * MAX_JAC + j];
#pragma unroll 1
    for (int q = 0; q < j; q++) d = __dsub_rn(d, __dmul_rn(A[j * MAX_JAC + q], A[j * MAX_JAC + q]));
    if (!(d > 0.0)) return j + 1;
    d = sqrt(d);
    A[j * MAX_JAC + j] = d;
#pragma unroll 1
    for (int i = j + 1; i < k; i++) {
      double t = A[j * MAX_JAC + i];
#pragma unroll 1
      for (int q = 0; q < j; q++) t = __dsub_rn(t, __dmul_rn(A[i * MAX_JAC + q], A[j * MAX_JAC + q]));
      A[i * MAX_JAC + j] = t / d;
    }
  }
#pragma unroll 1
  for (int i = 0; i < k; i++) {
    double t = b[i];
#pragma unroll 1
    for (int q = 0; q < i; q++) t = __dsub_rn(t, __dmul_rn(A[i * MAX_JAC + q], b[q]));
    b[i] = t / A[i * MAX_JAC + i];
  }
#pragma unroll 1
  for (int i = k - 1; i >= 0; i--) {
    double t = b[i];
#pragma unroll 1
    for (int q = i + 1; q < k; q++) t = __dsub_rn(t, __dmul_rn(A[q * MAX_JAC + i], b[q]));
    b[i] = t / A[i * MAX_JAC + i];
  }
  int st = 0;
#pragma unroll 1
  for (int i = 0; i < k; i++) {
    out[i] = b[i];
    if (isnan(b[i])) st = 1;
  }
  return st;
}

// Damped solve (H + lam diag H) d = b of the FP32 Gaussian step
// (multi_fit.c:1174-1203 with dposv :1839-1883), FP32 instructions only.
// Every lane factors the Jacobi-scaled matrix (LDL^T) and substitutes on its
// own, so the factorisation needs no shuffles; the two refinements compute
// the residual in float-float a row per lane and gather it to every lane.
// A pivot <= 0 hands the system to the FP64 Cholesky on lane 0, which
// decides failure as dposv does.  Lane j < K returns component j of the
// solution in dl (the K conversions to double run lane-parallel); the
// status is returned on every lane.
template <int K>
__device__ inline int solve_g32(WarpWS<float>& ws, double lam, double& dl, int lane) {
  const float* jh = g32_jh(ws);
  const ff L1 = ff_from_double(1.0 + lam);
  float sc[K], D[K], R[K], L[K][K], c[K];
  int status = 0;
  dl = 0.0;
#pragma unroll
  for (int i = 0; i < K; i++) {
    const int id = hes_index(K, i, i);
    const float d = ff_mul(L1, ff{jh[id], jh[36 + id]}).h;
    if (!(d > 1.0e-30f && d < 1.0e30f)) status = 2;
    sc[i] = rsqrtf(d);
  }
  if (status == 0) {
#pragma unroll
    for (int j = 0; j < K; j++) {
      const int idj = hes_index(K, j, j);
      float dj = (ff_mul(L1, ff{jh[idj], jh[36 + idj]}).h * sc[j]) * sc[j];
#pragma unroll
      for (int m = 0; m < j; m++) dj = fmaf(-L[j][m] * L[j][m], D[m], dj);
      if (!(dj > 0.0f)) status = 2;
      D[j] = dj;
      const float inv = __frcp_rn(dj);
      R[j] = inv;
#pragma unroll
      for (int i = j + 1; i < K; i++) {
        float t = (jh[hes_index(K, i, j)] * sc[i]) * sc[j];
#pragma unroll
        for (int m = 0; m < j; m++) t = fmaf(-L[i][m] * L[j][m], D[m], t);
        L[i][j] = t * inv;
      }
    }
  }
  if (status == 0) {
    // L D L^T x = c, c = scaled right-hand side; d = x * scale
    auto substitute = [&](float (&v)[K]) {
#pragma unroll
      for (int i = 0; i < K; i++) {
#pragma unroll
        for (int m = 0; m < i; m++) v[i] = fmaf(-L[i][m], v[m], v[i]);
      }
#pragma unroll
      for (int i = 0; i < K; i++) v[i] = v[i] * R[i];
#pragma unroll
      for (int i = K - 1; i >= 0; i--) {
#pragma unroll
        for (int m = i + 1; m < K; m++) v[i] = fmaf(-L[m][i], v[m], v[i]);
      }
    };
    ff x[K];
#pragma unroll
    for (int i = 0; i < K; i++) c[i] = jh[i] * sc[i];
    substitute(c);
#pragma unroll
    for (int i = 0; i < K; i++) x[i] = two_prod(c[i], sc[i]);
    for (int it = 0; it < 2; it++) {
      // residual of row `lane` in float-float, then every row to every lane
      ff res{0.0f, 0.0f};
      if (lane < K) {
        res = ff{jh[lane], jh[36 + lane]};
#pragma unroll
        for (int j = 0; j < K; j++) {
          const int id = hes_index(K, lane, j);
          const ff a{jh[id], jh[36 + id]};
          res = ff_sub(res, ff_mul(j == lane ? ff_mul(L1, a) : a, x[j]));
        }
      }
#pragma unroll
      for (int i = 0; i < K; i++) c[i] = __shfl_sync(0xffffffffu, res.h, i) * sc[i];
      substitute(c);
#pragma unroll
      for (int i = 0; i < K; i++) x[i] = ff_add(x[i], two_prod(c[i], sc[i]));
    }
    ff xl = x[0];
#pragma unroll
    for (int j = 1; j < K; j++)
      if (lane == j) xl = x[j];
    dl = ff_to_double(xl);
    if (__any_sync(0xffffffffu, lane < K && isnan(xl.h))) status = 1;   // multi_fit.c:1857-1863
  }
  if (status == 2) {   // the same on every lane (the factorisation is)
    // scratch: the trial tables, rebuilt after every solve
    double* scr = reinterpret_cast<double*>(ws.tab1);
    int st = 0;
    if (lane == 0) st = solve_g32_fallback(jh, K, lam, scr, scr + MAX_JAC * MAX_JAC + MAX_JAC);
    __syncwarp();
    status = __shfl_sync(0xffffffffu, st, 0);
    dl = scr[MAX_JAC * MAX_JAC + MAX_JAC + (lane < K ? lane : 0)];
    __syncwarp();
  }
  return status;
}

struct G32Pix {
  long long F, B, X;
  float2 x;   // the data X 2^-36 as a float-float pair
  int C;
  float rq;
};

template <typename T>
__device__ __forceinline__ void g32_load(const ModelCfg& cfg, const FrameSet<T>& fs, long long fbase,
                                         const unsigned short* roi, int ax, int ay, int p, G32Pix& v) {
  int rx, ry;
  roi_rc(roi, p, rx, ry);
  const long long k = pix_index(cfg, ax, ay, rx, ry);
  v.F = __ldcg(fs.f + fbase + k);
  v.B = __ldcg(fs.bg + fbase + k);
  v.C = __ldcg(fs.cnt + fbase + k);
  v.X = __ldg(fs.xq + fbase + k);
  v.x = __ldg(fs.xff + fbase + k);
  v.rq = cfg.rqe_one ? 1.0f : (float)__ldg(fs.rqe + k);
}

// Per-pixel state of the step's start, from the loaded pixel: f0 = f + bg /
// cnt and rho = f0 - x, exact up to the division (multi_fit.c:143; the data
// are kept in fixed point for this), t1 = 2 rho / f0, the Hessian weight
// t2 = 2 x / f0^2 and the start error term.
//
// For the Z model t2 is (2 - t1) / f0 in float-float, rounded once to
// FP32.  Evaluated from the FP32-rounded x and f0 it carries ~2e-7 relative
// error per pixel, and that alone changes the reference's iteration count of
// ~0.2 % of the peaks of the astigmatic sCMOS workload (FP64 oracle with the
// same roundings emulated: 99.8 % of the peaks within the position
// tolerance); rounded once, 99.95 %.  The other Gaussian models keep the
// FP32 quotient (their fits match the oracle to 1e-5 px with it).
template <int M>
__device__ __forceinline__ void g32_pixel_state(const G32Pix& v, int p, WarpWS<float>& ws, float& devf,
                                                bool& fail) {
  // f0 = rho + x with the data's float-float copy: two int64 conversions
  // fewer per pixel than converting f as well
  const float vx = v.x.x;
  const float cf = fx_s22(v.C);
  const ff bgc = ff_div(ff_from_fixed(v.B), ff{cf, 0.0f});
  const ff rho = ff_add(ff_from_fixed(v.F - v.X), bgc);
  const ff f0 = ff_add(rho, ff{v.x.x, v.x.y});
  if (!(f0.h > 0.0f)) fail = true;
  else devf += dev_res(rho.h, vx);
  const ff t1 = ff_div(ff{2.0f * rho.h, 2.0f * rho.l}, f0);
  ws.t1h[p] = t1.h;
  ws.t1l[p] = t1.l;
  ws.f0g[p] = f0.h;
  if constexpr (M == M_Z) ws.T2s[p] = ff_div(ff_sub(ff{2.0f, 0.0f}, t1), f0).h;
  else {
    const float iv = rcp_approx(f0.h);
    ws.T2s[p] = (2.0f * vx) * (iv * iv);
  }
  ws.Rs[p] = v.rq;
  ws.Cs[p] = cf;
}

// Pass 1a: the start state of the ROI's pixels into the warp workspace;
// returns the lane's start error terms.  Software-pipelined: the loads of
// the lane's next pixel are in flight while this one is computed, which
// hides one L2 round trip per pixel at the cost of one pixel's loaded
// values in registers.
template <int M, typename T>
__device__ inline void g32_gather(const ModelCfg& cfg, const FrameSet<T>& fs, long long fbase,
                                  const PeakRec& o, WarpWS<T>& ws, int lane, float& devf, bool& fail) {
  if constexpr (sizeof(T) == 4) {
    int p = lane;
    if (p >= cfg.nroi) return;
    G32Pix cur;
    g32_load(cfg, fs, fbase, ws.roi, o.xi, o.yi, p, cur);
    for (;;) {
      const int pn = p + 32;
      const bool more = pn < cfg.nroi;
      G32Pix nxt;
      if (more) g32_load(cfg, fs, fbase, ws.roi, o.xi, o.yi, pn, nxt);
      g32_pixel_state<M>(cur, p, ws, devf, fail);
      if (!more) break;
      cur = nxt;
      p = pn;
    }
  }
}

// Pass 1b over the ROI for model M: ff gradient and Hessian partial sums of
// this lane, from the start state in the warp workspace.  Two loops: the
// Hessian's products do not hold registers across the float-float
// gradient's chains.
//
// Hessian: FP32 products and per-lane sums (acc[0, nhes)), except for the
// astigmatic Z model, whose fits turn on it: its iteration counts change
// on ~0.1 % of the peaks of the sCMOS workload when the Hessian carries
// FP32 rounding (measured against the FP64 oracle), so there the Jacobian
// row is float-float, every product is exact (two_prod) and the lane sums
// are float-float, hi words in acc[0, 15), lo words in acc[15, 30).
template <int M, typename T>
__device__ inline void g32_pass1(const ModelCfg& cfg, const FrameSet<T>& fs, long long fbase,
                                 const PeakRec& o, WarpWS<T>& ws, int lane, ff (&g)[8],
                                 float (&acc)[32]) {
  constexpr int K = (M == M_2DFIXED) ? 4 : ((M == M_3D) ? 6 : 5);
  const int ts = ws.ts;
  const float* t0 = ws.tab0;
  const float* gt = ws.tab1;
  // gradient (float-float)
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(ws.roi, p, rx, ry);
    const ff t1{ws.t1h[p], ws.t1l[p]};
    const float rq = ws.Rs[p];
    const ff u = ff_mul(t1, ff_mul_f(g32_psf(t0, ts, rx, ry), rq));
    const ff A1{gt[rx], gt[ts + rx]}, A2{gt[2 * ts + rx], gt[3 * ts + rx]};
    const ff B1{gt[4 * ts + ry], gt[5 * ts + ry]}, B2{gt[6 * ts + ry], gt[7 * ts + ry]};
    ff_acc(g[0], u);
    if constexpr (M == M_3D) {
      ff_acc(g[1], ff_mul_raw(u, A1));
      ff_acc(g[2], ff_mul_raw(u, A2));
      ff_acc(g[3], ff_mul_raw(u, B1));
      ff_acc(g[4], ff_mul_raw(u, B2));
    } else {
      ff_acc(g[1], ff_mul_raw(u, A1));
      ff_acc(g[2], ff_mul_raw(u, B1));
      if constexpr (M != M_2DFIXED) ff_acc(g[3], ff_mul_raw(u, ff_add(A2, B2)));
    }
    ff_acc(g[K - 1], ff_mul_f(t1, rq));
  }
#pragma unroll
  for (int l = 0; l < K; l++) g[l] = fast_two_sum(g[l].h, g[l].l);
  if constexpr (M == M_Z) {
    constexpr int NH = K * (K + 1) / 2;   // 15
    for (int p = lane; p < cfg.nroi; p += 32) {
      int rx, ry;
      roi_rc(ws.roi, p, rx, ry);
      const float t2 = ws.T2s[p], rq = ws.Rs[p];
      const ff ps = ff_mul_f(g32_psf(t0, ts, rx, ry), rq);
      const ff A1{gt[rx], gt[ts + rx]}, A2{gt[2 * ts + rx], gt[3 * ts + rx]};
      const ff B1{gt[4 * ts + ry], gt[5 * ts + ry]}, B2{gt[6 * ts + ry], gt[7 * ts + ry]};
      ff jf[K];
      jf[0] = ps;
      jf[1] = ff_mul(ps, A1);
      jf[2] = ff_mul(ps, B1);
      jf[3] = ff_mul(ps, ff_add(A2, B2));
      jf[4] = ff{rq, 0.0f};
#pragma unroll
      for (int l = 0; l < K; l++) {
        const ff u = ff_mul_f(jf[l], t2);
#pragma unroll
        for (int m = l; m < K; m++) {
          const int id = l * K - (l * (l - 1)) / 2 + (m - l);
          const ff x = ff_mul_raw(u, jf[m]);
          const ff sh = two_sum(acc[id], x.h);
          acc[id] = sh.h;
          acc[NH + id] = __fadd_rn(acc[NH + id], __fadd_rn(sh.l, x.l));
        }
      }
    }
    return;
  }
  // Hessian (FP32)
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(ws.roi, p, rx, ry);
    const float t2 = ws.T2s[p], rq = ws.Rs[p];
    const float ps = t0[rx] * t0[2 * ts + ry] * rq;
    const float a1 = gt[rx], a2 = gt[2 * ts + rx], b1 = gt[4 * ts + ry], b2 = gt[6 * ts + ry];
    float jf[K];
    jf[0] = ps;
    if constexpr (M == M_3D) {
      jf[1] = ps * a1;
      jf[2] = ps * a2;
      jf[3] = ps * b1;
      jf[4] = ps * b2;
    } else {
      jf[1] = ps * a1;
      jf[2] = ps * b1;
      if constexpr (M != M_2DFIXED) jf[3] = ps * (a2 + b2);
    }
    jf[K - 1] = rq;
#pragma unroll
    for (int l = 0; l < K; l++) {
#pragma unroll
      for (int m = l; m < K; m++) acc[l * K - (l * (l - 1)) / 2 + (m - l)] += t2 * jf[l] * jf[m];
    }
  }
}

// Change of the MLE error for a trial at the start anchor (see the header
// comment); the trial tables are in tab1.  Returns the lane's ff first-order
// sum in s1 and FP32 second-order sum in s2.
template <typename T>
__device__ inline void g32_delta(const ModelCfg& cfg, const FrameSet<T>& fs, long long fbase,
                                 const PeakRec& o, const PeakRec& t, WarpWS<T>& ws, int lane, ff& s1,
                                 float& s2, bool& fail) {
  const int ts = ws.ts;
  const ff H0 = gpar(ws.par0, GP_H), H1 = gpar(ws.par1, GP_H);
  const ff DBG = gpar(ws.par1, GP_DBG);
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(ws.roi, p, rx, ry);
    const float rq = ws.Rs[p];
    const ff d = ff_mul_f(ff_sub(ff_mul(H1, g32_psf(ws.tab1, ts, rx, ry)), ff_mul(H0, g32_psf(ws.tab0, ts, rx, ry))), rq);
    const ff bgd = ff_div(ff_mul_f(DBG, rq), ff{ws.Cs[p], 0.0f});
    const ff df = ff_add(d, bgd);
    const float f0 = ws.f0g[p];
    if (!(f0 + df.h > 0.0f)) {
      fail = true;
    } else {
      const float t1h = ws.t1h[p];
      ff_acc(s1, ff_mul_raw(df, ff{t1h, ws.t1l[p]}));
      // x = f0 (1 - t1 / 2); the second-order term is FP32 anyway
      const float xv = fmaf(-0.5f * t1h, f0, f0);
      s2 += 2.0f * xv * r_minus_log1p(df.h * rcp_approx(f0));
    }
  }
}

// Is ROI pixel (rx, ry) inside the circular ROI (multi_fit.c:1031-1060)?
// Exact in FP32: every term is a multiple of 1/4.
__device__ __forceinline__ bool in_roi(int rx, int ry, int roi) {
  if (rx < 0 || ry < 0 || rx >= roi || ry >= roi) return false;
  const float c = 0.5f * (float)roi;
  const float dx = (float)rx - c + 0.5f, dy = (float)ry - c + 0.5f;
  return dx * dx + dy * dy <= c * c;
}

// MLE error of a trial at another anchor (FP32 with the exact fixed-point
// residual).  The peak is still in the fit image at its start anchor o; its
// contribution is taken out here, pixel by pixel, exactly as the write-back
// will take it out.
template <typename T>
__device__ inline float g32_absolute(const ModelCfg& cfg, const FrameSet<T>& fs, long long fbase,
                                     const PeakRec& o, const PeakRec& t, WarpWS<T>& ws, int lane,
                                     bool& fail) {
  const int ts = ws.ts;
  const float h1 = ws.par1[2 * GP_H], bg1 = ws.par1[2 * GP_BG];   // (float) of the doubles
  const ff H0 = gpar(ws.par0, GP_H), BG0 = gpar(ws.par0, GP_BG);
  const int dx = t.xi - o.xi, dy = t.yi - o.yi;
  float devf = 0.0f;
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(ws.roi, p, rx, ry);
    const long long k = pix_index(cfg, t.xi, t.yi, rx, ry);
    long long F = __ldcg(fs.f + fbase + k), B = __ldcg(fs.bg + fbase + k);
    int C = __ldcg(fs.cnt + fbase + k);
    const float xv = (float)__ldg(fs.x + fbase + k);
    const float rq = cfg.rqe_one ? 1.0f : (float)__ldg(fs.rqe + k);
    const float sc = cfg.scmos_zero ? 0.0f : (float)__ldg(fs.scmos + k);
    const long long Xq = __ldg(fs.xq + fbase + k);
    const int ox = rx + dx, oy = ry + dy;   // the same image pixel in the start ROI
    if (in_roi(ox, oy, cfg.roi)) {
      Q2 qf, qb;
      g32_contrib(ws.tab0, ts, H0, BG0, ox, oy, rq, sc, qf, qb);
      F -= qf.h;
      B -= qb.h;
      C -= 1;
    }
    const float psf = g32_psf(ws.tab1, ts, rx, ry).h;
    const float res = fx_to_float(F - Xq) + h1 * psf * rq +
                      (fx_to_float(B) + bg1 * rq + sc) * rcp_approx(fx_s22(C + 1));
    if (!(xv + res > 0.0f)) fail = true;
    else devf += dev_res(res, xv);
  }
  return devf;
}

// Delta slot j of model M -> its parameter (apply_update's order,
// dao_fit.c:1777-1880).
template <int M>
__device__ __forceinline__ int g32_delta_param(int j) {
  if constexpr (M == M_3D) return j == 0 ? PH : j == 1 ? PX : j == 2 ? PXW : j == 3 ? PY : j == 4 ? PYW : PBG;
  if constexpr (M == M_Z) return j == 0 ? PH : j == 1 ? PX : j == 2 ? PY : j == 3 ? PZ : PBG;
  if constexpr (M == M_2D) return j == 0 ? PH : j == 1 ? PX : j == 2 ? PY : j == 3 ? PXW : PBG;
  return j == 0 ? PH : j == 1 ? PX : j == 2 ? PY : PBG;
}

// apply_update + check_for of model M on the trial record t (a copy of
// the working record, in the warp workspace), one parameter per lane:
// lane j < K applies delta j (dl) to its parameter with the same double
// operations -- the Z range clamp and widths from z (dao_fit.c:1828-1880),
// the ROI re-anchor (mFitUpdate multi_fit.c:1933-1946), mFitCheck and the
// width clamps of daoCheck2D / daoCheck3D (:1061-1119).  Each FP64
// instruction then runs once for all parameters.  Returns check_for's code
// (0 ok, 1 margin, 2 negative height) on every lane.
template <int M>
__device__ inline int g32_update(const ModelCfg& cfg, PeakRec& t, double dl, int lane) {
  constexpr int K = (M == M_2DFIXED) ? 4 : ((M == M_3D) ? 6 : 5);
  const bool act = lane < K;
  const int pi = g32_delta_param<M>(act ? lane : 0);
  double nv = t.p[pi] - dl;
  if constexpr (M == M_Z) {
    if (pi == PZ) {
      if (nv < cfg.zmin) nv = cfg.zmin;
      if (nv > cfg.zmax) nv = cfg.zmax;
    }
  }
  // re-anchor on the PX and PY lanes
  const bool axis = act && (pi == PX || pi == PY);
  int ai = (pi == PY) ? t.yi : t.xi;
  {
    const double d = nv - (double)ai;
    if (axis && ((d < -0.5) || (d > 1.5))) ai = (int)floor(nv);
  }
  // widths from the new z: wx on lane 0, wy on lane 1 (widths_from_z)
  double wt = 0.0, wv = 0.0;
  if constexpr (M == M_Z) {
    const double z = __shfl_sync(0xffffffffu, nv, 3);   // delta 3 is PZ
    const bool sy = (lane == 1);
    const double c0 = sy ? cfg.wy[0] : cfg.wx[0], c1 = sy ? cfg.wy[1] : cfg.wx[1];
    const double c2 = sy ? cfg.wy[2] : cfg.wx[2], c3 = sy ? cfg.wy[3] : cfg.wx[3];
    const double c4 = sy ? cfg.wy[4] : cfg.wx[4];
    const double z0 = (z - c1) / c2;
    const double z1 = z0 * z0, z2 = z1 * z0, z3 = z2 * z0;
    const double tt = 1.0 + z1 + c3 * z2 + c4 * z3;
    wt = tt * tt;
    wv = 2.0 / (c0 * tt);
  }
  // mFitCheck: the anchors in the image, a non-negative height
  const int lim = (pi == PY) ? (cfg.ny - cfg.roi) : (cfg.nx - cfg.roi);
  const bool margin = __any_sync(0xffffffffu, axis && ((ai < 0) || (ai >= lim)));
  const bool negh = __any_sync(0xffffffffu, act && pi == PH && (nv < 0.0));
  // width clamps (used only when the check passes; the record is dropped otherwise)
  double cv = nv;
  if constexpr (M == M_2D || M == M_3D) {
    if (pi == PXW || (M == M_3D && pi == PYW)) {
      if (cv < cfg.wmin) cv = cfg.wmin;
      else if (cv > cfg.wmax) cv = cfg.wmax;
    }
  }
  if (act) {
    t.p[pi] = cv;
    if (M == M_2D && pi == PXW) t.p[PYW] = nv;   // the unclamped x width
    if (pi == PX) t.xi = ai;
    if (pi == PY) t.yi = ai;
  }
  if constexpr (M == M_Z) {
    if (lane == 0) {
      t.wxt = wt;
      t.p[PXW] = wv;
    } else if (lane == 1) {
      t.wyt = wt;
      t.p[PYW] = wv;
    }
  }
  __syncwarp();
  return margin ? 1 : (negh ? 2 : 0);
}

// What the step of a peak needs before it reads the fit image: its record
// (ws.orig), its shape tables (tab0) and Jacobian factors (tab1).  Only the
// peak's own step changes its record, so this runs before the dependency
// waits of the sweep and overlaps them.
template <int M, typename T>
__device__ inline void g32_prologue(const ModelCfg& cfg, const PeakRec* recp, WarpWS<T>& ws, int lane) {
  if constexpr (sizeof(T) == 4 && M <= M_Z) {
    if (lane < 8) {
      reinterpret_cast<double2*>(ws.orig)[lane] = __ldcg(reinterpret_cast<const double2*>(recp) + lane);
    }
    __syncwarp();
    const PeakRec& orig = *ws.orig;
    g32_params(cfg, orig, nullptr, M == M_Z, ws.par0, lane);
    g32_tables_p(cfg, ws.par0, ws.tab0, ws.ts, lane);
    g32_grad_tables<M>(cfg, ws.par0, ws.tab1, ws.ts, lane);
    __syncwarp();
  }
}

// The step of a peak of Gaussian model M (cfg.model == M), after
// g32_prologue.  Returns true if the step escaped its footprint (nothing
// changed).
template <int M, typename T>
__device__ bool lm_step_g32(const ModelCfg& cfg, const FrameSet<T>& fs, long long fbase, PeakRec* recp,
                            bool unbounded, int dil, WarpWS<T>& ws, int* ctr_out, int lane) {
  if constexpr (sizeof(T) != 4 || M > M_Z) {
    return false;
  } else {
    const PeakRec& orig = *ws.orig;
    constexpr int k = (M == M_2DFIXED) ? 4 : ((M == M_3D) ? 6 : 5);
    constexpr int nhes = k * (k + 1) / 2;
    const int ts = ws.ts;

    // -- 1. starting error, gradient / Hessian, subtract (multi_fit.c:1107-1142)
    float devf = 0.0f;
    bool fail = false;
    g32_gather<M>(cfg, fs, fbase, orig, ws, lane, devf, fail);
    __syncwarp();
    ff g[8];
#pragma unroll
    for (int i = 0; i < 8; i++) g[i] = ff{0.0f, 0.0f};
    float acc[32];
#pragma unroll
    for (int i = 0; i < 32; i++) acc[i] = 0.0f;
    g32_pass1<M>(cfg, fs, fbase, orig, ws, lane, g, acc);
    // The reference subtracts the peak here (multi_fit.c:1141) and adds the
    // accepted trial back.  No other warp touches this ROI during the step,
    // so the subtraction is deferred to the write-back, which applies the
    // net change once; the trial evaluations account for it.
    const ff H0 = gpar(ws.par0, GP_H), BG0 = gpar(ws.par0, GP_BG);
    const double dev0 = warp_sum_ff(devf);
    fail = __any_sync(0xffffffffu, fail);
    {
      float* jh = g32_jh(ws);
      // Lane sums to warp totals: float-float for Z (the lo words' totals
      // come from lanes nhes .. 2 nhes - 1 and are added in), FP32 for the
      // other models (whose lo words stay zero).
      if constexpr (M == M_Z) {
        ff hv = warp_transpose_sum32_ff(acc, lane);
        const ff lo = shfl_ff(hv, (lane + nhes) & 31);
        hv = ff_add(hv, lo);
        if (lane < nhes) {
          jh[k + lane] = hv.h;
          jh[36 + k + lane] = hv.l;
        }
      } else {
        const float hv = warp_transpose_sum32(acc, lane);
        if (lane < nhes) {
          jh[k + lane] = hv;
          jh[36 + k + lane] = 0.0f;
        }
      }
      const ff gv = warp_reduce8_ff(g, lane);
      const int gi = reduce8_index(lane);
      if ((lane & 3) == 0 && gi < k) {
        jh[gi] = gv.h;
        jh[36 + gi] = gv.l;
      }
    }
    __syncwarp();

    // -- 2. LM loop (multi_fit.c:1145-1325); lane 0 holds the scalar state.
    PeakRec& w = *ws.w;
    double se = 0.0;
    // the step's counters (lane 0) live in the warp workspace, not in
    // registers that every lane would carry through the loop
    int* ctr = reinterpret_cast<int*>(ws.scratch);
    if (lane == 0) {
#pragma unroll
      for (int i = 0; i < NCOUNTERS; i++) ctr[i] = 0;
      w = orig;
      if (!fail) w.error = dev0;
      else ctr[C_STARTFAIL]++;
      se = w.error;
    }
    bool added_end = false, escaped = false;
    for (;;) {
      int act = ACT_EVAL;
      // lambda bound and iteration count (multi_fit.c:1153-1171)
      if (lane == 0) {
        if (w.lambda > LAMBDA_MAX) {
          ctr[C_LOST]++;
          w.status = ERROR;
          act = ACT_BREAK;
        } else {
          w.iterations++;
          ctr[C_ITER]++;
          w.status = RUNNING;
        }
      }
      act = __shfl_sync(0xffffffffu, act, 0);
      if (act == ACT_BREAK) break;
      // damped solve (multi_fit.c:1174-1203), warp-collective
      const double lam = __shfl_sync(0xffffffffu, w.lambda, 0);
      double dl;
      const int info = solve_g32<k>(ws, lam, dl, lane);
      int c = 0;
      if (info == 0) {
        PeakRec& t = *ws.t;
        if (lane == 0) t = w;
        __syncwarp();
        c = g32_update<M>(cfg, t, dl, lane);
      }
      if (lane == 0) {
        if (info != 0) {
          ctr[C_DPOSV]++;
          w.status = ERROR;
          w.lambda = w.lambda * LAMBDA_UP;
          act = ACT_CONTINUE;
        } else {
          const PeakRec& t = *ws.t;
          if (c) {
            if (c == 1) ctr[C_MARGIN]++;
            else ctr[C_NEGH]++;
            w = orig;                      // mFitResetPeak multi_fit.c:1788-1798
            w.lambda = lam * LAMBDA_UP;
            w.status = ERROR;
            act = ACT_CONTINUE;
          } else if (!unbounded && (abs(t.xi - orig.xi) > dil || abs(t.yi - orig.yi) > dil)) {
            act = ACT_ESCAPE;
          } else {
            w = t;
            act = ACT_EVAL;
          }
        }
      }
      act = __shfl_sync(0xffffffffu, act, 0);
      __syncwarp();
      if (act == ACT_CONTINUE) continue;
      if (act == ACT_BREAK) break;
      if (act == ACT_ESCAPE) {
        escaped = true;
        break;
      }
      // -- trial evaluation: shape, add, error (multi_fit.c:1229-1256)
      const PeakRec& wl = *ws.w;
      g32_params(cfg, wl, &orig, false, ws.par1, lane);
      g32_tables_p(cfg, ws.par1, ws.tab1, ts, lane);
      __syncwarp();
      const bool is_delta = (wl.xi == orig.xi) && (wl.yi == orig.yi);
      double dev;
      fail = false;
      if (is_delta) {
        ff s1{0.0f, 0.0f};
        float s2 = 0.0f;
        g32_delta(cfg, fs, fbase, orig, wl, ws, lane, s1, s2, fail);
        s1 = fast_two_sum(s1.h, s1.l);
        dev = ff_to_double(warp_sum_ffv(s1)) + warp_sum_ff(s2);
      } else {
        dev = warp_sum_ff(g32_absolute(cfg, fs, fbase, orig, wl, ws, lane, fail));
      }
      // A trial whose error overflows FP32 has an error astronomically above
      // the start error in the reference's FP64 too: reject it.
      if (!(fabs(dev) < 1.0e300)) dev = 1.0e300;
      fail = __any_sync(0xffffffffu, fail);
      if (lane == 0) {
        if (fail) {
          ctr[C_NEGFI]++;
          const double lm = w.lambda;
          w = orig;
          w.lambda = lm * LAMBDA_UP;
          w.status = ERROR;
          act = ACT_CONTINUE;
        } else {
          w.error = is_delta ? se + dev : dev;
          const double change = is_delta ? dev : w.error - se;
          // |change| / se < tol as a product for a positive start error (no
          // FP64 division on the step's critical path; the two forms differ
          // only within 1e-16 of the threshold, far below the engine's
          // float-float error change)
          const bool small = (se > 0.0) ? (fabs(change) < cfg.tol * se) : (fabs(change) / se < cfg.tol);
          if (change > 0.0) {
            if (small) {
              w.status = CONVERGED;
              act = ACT_BREAK_ADDED;
            } else {
              ctr[C_NONDECR]++;
              const double lm = w.lambda;
              w = orig;
              w.lambda = lm * LAMBDA_UP;
              act = ACT_CONTINUE;
            }
          } else {
            if (small) {
              w.status = CONVERGED;
            } else if (w.lambda > LAMBDA_MIN) {
              w.lambda = LAMBDA_DOWN * w.lambda;
            }
            act = ACT_BREAK_ADDED;
          }
        }
      }
      act = __shfl_sync(0xffffffffu, act, 0);
      if (act == ACT_BREAK_ADDED) {
        added_end = true;
        break;
      }
    }

    // -- 3. write back: the net change of the fit image (subtract the start
    // contribution, add the accepted one)
    if (escaped) return true;   // nothing was changed
    if (lane == 0) w.added = orig.added - 1 + (added_end ? 1 : 0);
    __syncwarp();
    const PeakRec& wl = *ws.w;
    // the accepted trial's slots (par1 is the last trial's, and a step
    // that adds back ends on an accepted trial)
    const ff H1 = gpar(ws.par1, GP_H), BG1 = gpar(ws.par1, GP_BG);
    if (added_end && wl.xi == orig.xi && wl.yi == orig.yi && cfg.rqe_one && cfg.scmos_zero) {
      // uniform calibration: BG * 1 + 0 at every pixel, quantised once
      // (bit-identical to g32_contrib with rqe 1 and sCMOS 0)
      Q2 b0, b1;
      b0.h = fixed_from_ff(BG0);
      b1.h = fixed_from_ff(BG1);
      b0.l = b1.l = 0;
      const Q2 db = q_sub(b1, b0);
      for (int p = lane; p < cfg.nroi; p += 32) {
        int rx, ry;
        roi_rc(ws.roi, p, rx, ry);
        const long long kk = pix_index(cfg, orig.xi, orig.yi, rx, ry);
        Q2 q0f, q1f;
        q0f.h = fixed_from_ff(ff_mul(H0, g32_psf(ws.tab0, ts, rx, ry)));
        q1f.h = fixed_from_ff(ff_mul(H1, g32_psf(ws.tab1, ts, rx, ry)));
        q0f.l = q1f.l = 0;
        acc_red<1>(fs.f, fbase + kk, q_sub(q1f, q0f), +1);
        acc_red<1>(fs.bg, fbase + kk, db, +1);
      }
    } else if (added_end && wl.xi == orig.xi && wl.yi == orig.yi) {
      for (int p = lane; p < cfg.nroi; p += 32) {
        int rx, ry;
        roi_rc(ws.roi, p, rx, ry);
        const long long kk = pix_index(cfg, orig.xi, orig.yi, rx, ry);
        const float rq = ws.Rs[p], sc = cfg.scmos_zero ? 0.0f : (float)__ldg(fs.scmos + kk);
        Q2 q0f, q0b, q1f, q1b;
        g32_contrib(ws.tab0, ts, H0, BG0, rx, ry, rq, sc, q0f, q0b);
        g32_contrib(ws.tab1, ts, H1, BG1, rx, ry, rq, sc, q1f, q1b);
        acc_red<1>(fs.f, fbase + kk, q_sub(q1f, q0f), +1);
        acc_red<1>(fs.bg, fbase + kk, q_sub(q1b, q0b), +1);
      }
    } else {
      for (int p = lane; p < cfg.nroi; p += 32) {
        int rx, ry;
        roi_rc(ws.roi, p, rx, ry);
        const long long kk = pix_index(cfg, orig.xi, orig.yi, rx, ry);
        Q2 qf, qb;
        g32_contrib(ws.tab0, ts, H0, BG0, rx, ry, ws.Rs[p], cfg.scmos_zero ? 0.0f : (float)__ldg(fs.scmos + kk),
                    qf, qb);
        acc_red<1>(fs.f, fbase + kk, qf, -1);
        acc_red<1>(fs.bg, fbase + kk, qb, -1);
        atomicAdd(fs.cnt + fbase + kk, -1);
      }
    }
    if (added_end && (wl.xi != orig.xi || wl.yi != orig.yi)) {
      for (int p = lane; p < cfg.nroi; p += 32) {
        int rx, ry;
        roi_rc(ws.roi, p, rx, ry);
        const long long kk = pix_index(cfg, wl.xi, wl.yi, rx, ry);
        Q2 qf, qb;
        g32_contrib(ws.tab1, ts, H1, BG1, rx, ry, cfg.rqe_one ? 1.0f : (float)__ldg(fs.rqe + kk),
                    cfg.scmos_zero ? 0.0f : (float)__ldg(fs.scmos + kk), qf, qb);
        acc_red<1>(fs.f, fbase + kk, qf, +1);
        acc_red<1>(fs.bg, fbase + kk, qb, +1);
        atomicAdd(fs.cnt + fbase + kk, 1);
      }
    }
    if (lane == 0) {
      *recp = w;
      for (int i = 0; i < NCOUNTERS; i++) ctr_out[i] = ctr[i];
    }
    return false;
  }
}

}  // namespace sa
