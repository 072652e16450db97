// sa_kernels.cuh -- kernels of the GB300 multi-emitter LM engine.
//
// One LM sweep (mFitIterateLM, multi_fit.c:1072-1349) over a frame set is
//   k_prepare   per frame: list RUNNING peaks in index order ("run ranks"),
//               snapshot them, bin their dilated footprints into a grid
//               (or, after an escape, roll back and mark barriers)
//   k_sweep     persistent warps; one warp runs one peak's LM step.  A peak
//               waits until every lower-index RUNNING peak whose dilated
//               footprint overlaps its own has finished, which reproduces
//               the reference's Gauss-Seidel order for every pixel.  A trial
//               step that would leave the footprint "escapes": the peak
//               restores itself, the frame's later peaks are rolled back and
//               re-run with the escaped peak as a barrier.
//   k_post      per frame: recenter (mFitRecenterPeaks :1644-1690), sum the
//               counters, count RUNNING peaks and decide whether the frame
//               needs another sweep (dao_fit_c.py:332-356).
#pragma once

#include "sa_g32.cuh"

namespace sa {

// ---------------------------------------------------------------------------
// block scan (blockDim.x == 1024)
// ---------------------------------------------------------------------------

__device__ inline int block_excl_scan(int v, int* smem32, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) smem32[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int s = smem32[lane];
    int si = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, si, o);
      if (lane >= o) si += t;
    }
    smem32[lane] = si - s;
    if (lane == 31) smem32[32] = si;
  }
  __syncthreads();
  int res = smem32[wid] + inc - v;
  total = smem32[32];
  __syncthreads();
  return res;
}

__device__ __forceinline__ unsigned pack_anchor(int xi, int yi) {
  return ((unsigned)xi & 0xffffu) | ((unsigned)yi << 16);
}

__device__ __forceinline__ void load_rec(const PeakRec* src, PeakRec& dst) {
  const double2* s = reinterpret_cast<const double2*>(src);
  double2* d = reinterpret_cast<double2*>(&dst);
#pragma unroll
  for (int i = 0; i < 8; i++) d[i] = __ldcg(s + i);
}

// ---------------------------------------------------------------------------
// the LM step of one peak (one warp)
// ---------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ T ic_store(int c) {
  // FP32 keeps 1/count and multiplies; FP64 keeps the count and divides as
  // the reference does (multi_fit.c:143).
  if (sizeof(T) == 4) return c > 0 ? (T)1 / (T)c : (T)0;
  return (T)c;
}
template <typename T>
__device__ __forceinline__ T bg_div(T b, T ic) {
  if (sizeof(T) == 4) return b * ic;
  return b / ic;
}

// Load the base pixel state (fit image without this peak) at anchor (ax, ay).
template <typename T>
__device__ inline void load_base(const ModelCfg& cfg, const FrameSet<T>& fs, long long fbase, int ax,
                                 int ay, WarpWS<T>& ws, int lane) {
  constexpr int W = AccW<T>::W;
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(ws.roi, p, rx, ry);
    const long long k = pix_index(cfg, ax, ay, rx, ry);
    const Q2 Fq = acc_load<W>(fs.f, fbase + k);
    const Q2 Bq = acc_load<W>(fs.bg, fbase + k);
    const int Cg = __ldcg(fs.cnt + fbase + k);
    const T sc = __ldg(fs.scmos + k);
    if constexpr (sizeof(T) == 4) {
      ws.Fb[p] = fx_to_float(Fq.h);
      ws.Bs[p] = fx_to_float(Bq.h) + sc;
    } else {
      ws.Fb[p] = (T)acc_value<W>(Fq);
      ws.Bs[p] = (T)(acc_value<W>(Bq) + (double)sc);
    }
    ws.R[p] = __ldg(fs.rqe + k);
    ws.X[p] = __ldg(fs.x + fbase + k);
    ws.IC[p] = ic_store<T>(Cg + 1);
  }
}


// Returns true if the step escaped its footprint (nothing changed).
template <typename T>
__device__ bool lm_step(const ModelCfg& cfg, const FrameSet<T>& fs, long long fbase, PeakRec* recp,
                        bool unbounded, int dil, WarpWS<T>& ws, int* ctr_out, int lane) {
  // The start-of-step, working and trial records live in the warp's shared
  // workspace; only lane 0 writes them.
  if (lane < 8) {
    reinterpret_cast<double2*>(ws.orig)[lane] = __ldcg(reinterpret_cast<const double2*>(recp) + lane);
  }
  __syncwarp();
  const PeakRec& orig = *ws.orig;
  const int k = cfg.jac;
  const int nh = k + k * (k + 1) / 2;

  // -- 1. starting error, Jacobian / Hessian, subtract (multi_fit.c:1107-1142)
  SplinePos s0 = shape_tables(cfg, orig, ws, lane);
  double gxd, gyd;
  z_factors(cfg, cfg.model, orig, gxd, gyd);
  const T gx = (T)gxd, gy = (T)gyd;
  T acc[32];
#pragma unroll
  for (int i = 0; i < 32; i++) acc[i] = (T)0;
  ff g[MAX_JAC];   // FP32 engine: per-lane float-float gradient
#pragma unroll
  for (int i = 0; i < MAX_JAC; i++) g[i] = ff{0.0f, 0.0f};
  double dev = 0.0;
  float devf = 0.0f;   // FP32 engine: per-lane partial sum
  bool fail = false;
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(ws.roi, p, rx, ry);
    const long long kk = pix_index(cfg, orig.xi, orig.yi, rx, ry);
    const Q2 Fq = acc_load<AccW<T>::W>(fs.f, fbase + kk);
    const Q2 Bq = acc_load<AccW<T>::W>(fs.bg, fbase + kk);
    const int Cg = __ldcg(fs.cnt + fbase + kk);
    const T xv = __ldg(fs.x + fbase + kk);
    const T rq = __ldg(fs.rqe + kk);
    const T sc = __ldg(fs.scmos + kk);
    T psf;
    ff psf_ff{0.0f, 0.0f};   // FP32: the model value as float-float
    if constexpr (sizeof(T) == 4) {
      psf_ff = spline_value_ff(cfg, fs.aij, ws, s0, rx, ry);
      psf = psf_ff.h;
    } else {
      psf = psf_at(cfg, fs.aij, ws, s0, rx, ry);
    }
    T t1, t2;
    float t1lo = 0.0f;
    if constexpr (sizeof(T) == 4) {
      // FP32 engine (spline models), float and integer instructions only.
      // The residual rho = f + bg/cnt - x is float-float: f - x is exact in
      // fixed point (the data's fixed-point copy), so t1 = 2 rho / f0 and
      // the Hessian weight t2 = 2 x / f0^2 = (2 - t1) / f0 are accurate to
      // ~1e-14 before their final rounding; t1 stays float-float for the
      // gradient and for the first-order error change of the trials.
      const long long Xq = __ldg(fs.xq + fbase + kk);
      const float2 xd = __ldg(fs.xff + fbase + kk);
      const ff rh = ff_add(ff_from_fixed(Fq.h - Xq), ff_div(ff_from_fixed(Bq.h), ff{(float)Cg, 0.0f}));
      const ff f0 = ff_add(rh, ff{xd.x, xd.y});
      const ff t1f = ff_div(ff{2.0f * rh.h, 2.0f * rh.l}, f0);
      ws.psf0[p] = psf;
      ws.f0[p] = f0.h;
      ws.rho[p] = t1f.h;   // the FP32 engine keeps t1 here (hi word)
      t1lo = t1f.l;
      if (!(f0.h > 0.0f)) fail = true;
      else devf += dev_res(rh.h, xd.x);
      t1 = t1f.h;
      t2 = ff_div(ff_sub(ff{2.0f, 0.0f}, t1f), f0).h;
    } else {
      const double fi0 = acc_value<AccW<T>::W>(Fq) + acc_value<AccW<T>::W>(Bq) / (double)Cg;
      if (!(fi0 > 0.0)) fail = true;
      else dev += (double)deviance((T)fi0, xv);
      // the reference's forms (dao_fit.c:454-460)
      t1 = (T)2 * ((T)1 - xv / (T)fi0);
      t2 = (T)2 * xv / ((T)fi0 * (T)fi0);
    }
    T jt[MAX_JAC];
    jt_row(cfg, fs.aij, ws, s0, orig, gx, gy, rx, ry, rq, psf, jt);
    int idx = 0;
#pragma unroll
    for (int l = 0; l < MAX_JAC; l++) {
      if constexpr (sizeof(T) == 4) {
        if (l < k) ff_acc(g[l], ff_mul_raw(ff{(float)t1, t1lo}, ff{(float)jt[l], 0.0f}));
      } else {
        if (l < k) acc[l] += t1 * jt[l];
      }
    }
    idx = k;
#pragma unroll
    for (int l = 0; l < MAX_JAC; l++) {
#pragma unroll
      for (int m = l; m < MAX_JAC; m++) {
        if (l < k && m < k) {
          // packed upper triangle, row-major
          const int id = k + l * k - (l * (l - 1)) / 2 + (m - l);
          if (id < 32) acc[id] += t2 * jt[l] * jt[m];
        }
      }
    }
    (void)idx;
    // subtract this peak (multi_fit.c:1141) and keep the base state
    Q2 cf, cb;
    if constexpr (sizeof(T) == 4) {
      spl32_contrib(psf_ff, ff_from_double(orig.p[PH]), ff_from_double(orig.p[PBG]), rq, sc, cf, cb);
    } else {
      cf = quant_t<T>(contrib_f(orig.p[PH], psf, rq));
      cb = quant_t<T>(contrib_bg(orig.p[PBG], rq, sc));
    }
    acc_red<AccW<T>::W>(fs.f, fbase + kk, cf, -1);
    acc_red<AccW<T>::W>(fs.bg, fbase + kk, cb, -1);
    atomicAdd(fs.cnt + fbase + kk, -1);
    if constexpr (sizeof(T) == 4) {
      ws.Fb[p] = fx_to_float(Fq.h - cf.h);
      ws.Bs[p] = fx_to_float(Bq.h - cb.h) + sc;
    } else {
      ws.Fb[p] = (T)acc_value<AccW<T>::W>(q_sub(Fq, cf));
      ws.Bs[p] = (T)(acc_value<AccW<T>::W>(q_sub(Bq, cb)) + (double)sc);
    }
    ws.R[p] = rq;
    // FP32: the low word of t1 until a trial reloads the base state (the
    // trials then take the absolute path, which reloads the data here)
    if constexpr (sizeof(T) == 4) ws.X[p] = t1lo;
    else ws.X[p] = xv;
    ws.IC[p] = ic_store<T>(Cg);   // (Cg - 1) + 1 once the peak is re-added
  }
  if constexpr (sizeof(T) == 4) dev = warp_sum_ff(devf);
  else dev = warp_sum(dev);
  fail = __any_sync(0xffffffffu, fail);
  if constexpr (sizeof(T) == 4) {
    // Per-lane partial sums (a few pixels each) are summed across the warp
    // in float-float arithmetic: the cross-lane sums are where the gradient
    // cancels.
    // The gradient's lo words go to columns nh .. nh + k - 1 (nh + k <= 25).
    float* red = ws.red;
#pragma unroll
    for (int i = 0; i < 32; i++) {
      if (i < k) {
        const ff gi = fast_two_sum(g[i < MAX_JAC ? i : 0].h, g[i < MAX_JAC ? i : 0].l);
        red[lane * 33 + i] = gi.h;
        red[lane * 33 + nh + i] = gi.l;
      } else if (i < nh) {
        red[lane * 33 + i] = acc[i];
      }
    }
    __syncwarp();
    if (lane < nh) {
      float hi = 0.0f, lo = 0.0f;
      for (int j = 0; j < 32; j++) ff_add(hi, lo, red[j * 33 + lane]);
      if (lane < k)
        for (int j = 0; j < 32; j++) ff_add(hi, lo, red[j * 33 + nh + lane]);
      ws.jh[lane] = (double)hi + (double)lo;
    }
  } else {
    T v = warp_transpose_sum32(acc, lane);
    if (lane < nh) ws.jh[lane] = (double)v;
  }
  if constexpr (sizeof(T) == 4) {
    // Gaussian start-of-step factors for the differential evaluation.
    if (!is_spline(cfg.model)) {
      for (int i = lane; i < cfg.roi; i += 32) {
        ws.ext[64 + i] = ws.ext[i];
        ws.eyt[64 + i] = ws.eyt[i];
      }
    }
  }
  __syncwarp();

  // -- 2. LM loop (multi_fit.c:1145-1325); lane 0 holds the scalar state.
  PeakRec& w = *ws.w;
  double se = 0.0;
  int ctr[NCOUNTERS];
#pragma unroll
  for (int i = 0; i < NCOUNTERS; i++) ctr[i] = 0;
  if (lane == 0) {
    w = orig;
    if (!fail) w.error = dev;
    else ctr[C_STARTFAIL]++;
    se = w.error;
  }
  int cax = orig.xi, cay = orig.yi;   // anchor of the cached base arrays
  bool reloaded = false;              // base arrays reloaded by a trial
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
    double b[MAX_JAC];
    const int info = solve_damped<T>(ws, k, lam, b, lane);
    if (lane == 0) {
      if (info != 0) {
        ctr[C_DPOSV]++;
        w.status = ERROR;
        w.lambda = w.lambda * LAMBDA_UP;
        act = ACT_CONTINUE;
      } else {
        PeakRec& t = *ws.t;
        t = w;
        apply_update(cfg, cfg.model, t, b);
        const int c = check_for(cfg, cfg.model, t);
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
    SplinePos s = shape_tables(cfg, wl, ws, lane, false);
    bool is_delta = false;
    if constexpr (sizeof(T) == 4) {
      // FP32: evaluate the change of the error from the start of the step
      // when the ROI and the spline cell are unchanged and the start state
      // is still in the workspace.
      is_delta = !reloaded && (wl.xi == orig.xi) && (wl.yi == orig.yi) &&
                 (!is_spline(cfg.model) || (s.xs == s0.xs && s.ys == s0.ys && s.zi == s0.zi));
    }
    if (sizeof(T) == 4 ? (!is_delta && (!reloaded || wl.xi != cax || wl.yi != cay))
                       : (wl.xi != cax || wl.yi != cay)) {
      __threadfence();
      __syncwarp();
      load_base(cfg, fs, fbase, wl.xi, wl.yi, ws, lane);
      __syncwarp();
      cax = wl.xi;
      cay = wl.yi;
      reloaded = true;
    }
    dev = 0.0;
    devf = 0.0f;
    fail = false;
    const double hh = wl.p[PH], bgv = wl.p[PBG];
    const T bgT = (T)bgv;
    if constexpr (sizeof(T) == 4) {
      if (is_delta) {
        diff_tables(cfg, orig, wl, s0, s, ws, lane);
        __syncwarp();
        const float h1 = (float)hh;
        const float dh = (float)(hh - orig.p[PH]);
        const float dbg = (float)(bgv - orig.p[PBG]);
        // first-order term df * t1 in float-float (its pixel sum cancels
        // near convergence), second-order term 2 x (r - log1p r) in FP32
        ff s1{0.0f, 0.0f};
        float s2 = 0.0f;
        for (int p = lane; p < cfg.nroi; p += 32) {
          int rx, ry;
          roi_rc(ws.roi, p, rx, ry);
          float psf, dpsf;
          psf_and_delta(cfg, fs.aij, ws, s, rx, ry, psf, dpsf);
          ws.psf[p] = psf;
          const float rq = ws.R[p];
          const float df = rq * fmaf(h1, dpsf, dh * ws.psf0[p]) + dbg * rq * ws.IC[p];
          const float f0 = ws.f0[p];
          if (!(f0 + df > 0.0f)) {
            fail = true;
          } else {
            const float t1h = ws.rho[p];
            ff_acc(s1, ff_mul_raw(ff{df, 0.0f}, ff{t1h, ws.X[p]}));
            const float xv = fmaf(-0.5f * t1h, f0, f0);
            s2 += 2.0f * xv * r_minus_log1p(__fdiv_rn(df, f0));
          }
        }
        s1 = fast_two_sum(s1.h, s1.l);
        devf = 0.0f;
        dev = ff_to_double(warp_sum_ffv(s1)) + warp_sum_ff(s2);
      } else {
        for (int p = lane; p < cfg.nroi; p += 32) {
          int rx, ry;
          roi_rc(ws.roi, p, rx, ry);
          const T psf = psf_at(cfg, fs.aij, ws, s, rx, ry);
          ws.psf[p] = psf;
          const T rq = ws.R[p];
          const T fi = ws.Fb[p] + contrib_f(hh, psf, rq) + bg_div(ws.Bs[p] + bgT * rq, ws.IC[p]);
          if (!(fi > (T)0)) fail = true;
          else devf += dev_res(fi - ws.X[p], ws.X[p]);
        }
      }
    } else {
      for (int p = lane; p < cfg.nroi; p += 32) {
        int rx, ry;
        roi_rc(ws.roi, p, rx, ry);
        const T psf = psf_at(cfg, fs.aij, ws, s, rx, ry);
        ws.psf[p] = psf;
        const T rq = ws.R[p];
        const T fi = ws.Fb[p] + contrib_f(hh, psf, rq) + bg_div(ws.Bs[p] + bgT * rq, ws.IC[p]);
        if (!(fi > (T)0)) fail = true;
        else dev += (double)deviance(fi, ws.X[p]);
      }
    }
    if constexpr (sizeof(T) == 4) {
      if (!is_delta) dev = warp_sum_ff(devf);
    } else {
      dev = warp_sum(dev);
    }
    fail = __any_sync(0xffffffffu, fail);
    if (lane == 0) {
      if (fail) {
        ctr[C_NEGFI]++;
        const double lam = w.lambda;
        w = orig;
        w.lambda = lam * LAMBDA_UP;
        w.status = ERROR;
        act = ACT_CONTINUE;
      } else {
        w.error = is_delta ? se + dev : dev;
        // change of the error, exact from the differential evaluation
        const double change = is_delta ? dev : w.error - se;
        if (is_delta ? (change > 0.0) : (w.error > se)) {
          if ((change / se) < cfg.tol) {
            w.status = CONVERGED;
            act = ACT_BREAK_ADDED;
          } else {
            ctr[C_NONDECR]++;
            const double lam = w.lambda;
            w = orig;
            w.lambda = lam * LAMBDA_UP;
            act = ACT_CONTINUE;
          }
        } else {
          if ((-change / se) < cfg.tol) {
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

  // -- 3. write back
  if (escaped) {
    // Restore the start-of-step contribution; the record is untouched.
    SplinePos so = shape_tables(cfg, orig, ws, lane);
    add_peak(cfg, fs, fbase, orig, so, ws, +1, lane);
    return true;
  }
  if (lane == 0) w.added = orig.added - 1 + (added_end ? 1 : 0);
  __syncwarp();
  if (added_end) {
    const PeakRec& wl = *ws.w;
    if constexpr (sizeof(T) == 4) {
      // the tables in the workspace are the accepted trial's
      const SplinePos sw = spline_pos(wl.p, wl.xi, wl.yi, wl.zi);
      const ff H = ff_from_double(wl.p[PH]), BG = ff_from_double(wl.p[PBG]);
      for (int p = lane; p < cfg.nroi; p += 32) {
        int rx, ry;
        roi_rc(ws.roi, p, rx, ry);
        const long long kk = pix_index(cfg, wl.xi, wl.yi, rx, ry);
        Q2 qf, qb;
        spl32_contrib(spline_value_ff(cfg, fs.aij, ws, sw, rx, ry), H, BG, __ldg(fs.rqe + kk),
                      __ldg(fs.scmos + kk), qf, qb);
        acc_red<1>(fs.f, fbase + kk, qf, +1);
        acc_red<1>(fs.bg, fbase + kk, qb, +1);
        atomicAdd(fs.cnt + fbase + kk, 1);
      }
    } else {
      for (int p = lane; p < cfg.nroi; p += 32) {
        int rx, ry;
        roi_rc(ws.roi, p, rx, ry);
        const long long kk = pix_index(cfg, wl.xi, wl.yi, rx, ry);
        const T rq = ws.R[p];
        const T sc = __ldg(fs.scmos + kk);
        acc_red<AccW<T>::W>(fs.f, fbase + kk, quant_t<T>(contrib_f(wl.p[PH], ws.psf[p], rq)), +1);
        acc_red<AccW<T>::W>(fs.bg, fbase + kk, quant_t<T>(contrib_bg(wl.p[PBG], rq, sc)), +1);
        atomicAdd(fs.cnt + fbase + kk, 1);
      }
    }
  }
  if (lane == 0) {
    *recp = w;
    for (int i = 0; i < NCOUNTERS; i++) ctr_out[i] = ctr[i];
  }
  return false;
}

// ---------------------------------------------------------------------------
// k_sweep: persistent warps over the run ranks of all frames in IN_SWEEP
// ---------------------------------------------------------------------------

// Can the steps of two peaks whose ROI anchors differ by (dx, dy) touch a
// common pixel, when each may move its anchor by up to dil in x and y?  A
// ROI pixel's centre lies within roi/2 of the ROI centre (the circular ROI,
// multi_fit.c:1031-1060), so two ROIs share no pixel when their centres are
// more than roi apart; the moves widen that by the distance between the two
// squares of reachable anchors.  The bounding-box test is kept as well.
__device__ __forceinline__ bool footprints_overlap(int dx, int dy, int roi, int dil) {
  const int span = roi + 2 * dil;
  dx = abs(dx);
  dy = abs(dy);
  if (dx >= span || dy >= span) return false;
  const int ex = max(dx - 2 * dil, 0), ey = max(dy - 2 * dil, 0);
  return ex * ex + ey * ey <= roi * roi;
}

// G32 >= 0: the FP32 Gaussian step (lm_step_g32) of model G32 (one
// instantiation per model); G32 < 0: lm_step.
template <typename T, int G32>
__global__ void __launch_bounds__(128, 5) k_sweep(ModelCfg cfg, FrameSet<T> fs) {
  extern __shared__ __align__(16) char smem[];
  // the tick's epoch: a done flag equal to it marks a rank done in this
  // launch (k_post of the previous tick advanced it)
  const int epoch = __ldcg(fs.epoch);
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  WarpWS<T> ws = warp_ws<T>(smem + (size_t)wib * warp_ws_bytes<T>(cfg, cfg.nroi), cfg, cfg.nroi);
  {
    // the ROI pixel table, shared by the CTA's warps, after their workspaces
    unsigned short* roi = reinterpret_cast<unsigned short*>(smem + (size_t)wpb * warp_ws_bytes<T>(cfg, cfg.nroi));
    for (int i = threadIdx.x; i < cfg.nroi; i += blockDim.x) roi[i] = fs.roi_xy[i];
    __syncthreads();
    ws.roi = roi;
  }
  const int gwarp = blockIdx.x * wpb + wib;
  int f = gwarp % fs.F;
  int misses = 0;
  while (misses < fs.F) {
    FrameCtl* c = fs.ctl + f;
    int r = -1;
    if (lane == 0) {
      // a plain read first: exhausted frames cost no atomic
      if (*((volatile int*)&c->phase) == PH_IN_SWEEP && *((volatile int*)&c->grab) < c->nrun) {
        r = atomicAdd(&c->grab, 1);
        if (r >= c->nrun) r = -1;
      }
    }
    r = __shfl_sync(0xffffffffu, r, 0);
    if (r < 0) {
      f = (f + 1) % fs.F;
      misses++;
      continue;
    }
    misses = 0;
    const int base = fs.pk_off[f];
    const int start = c->start;
    const int dil = c->dil;
    const unsigned a0 = fs.anchor0[base + r];
    const int ax = a0 & 0xffff, ay = a0 >> 16;
    const int li = fs.run[base + r];
    if constexpr (G32 >= 0) g32_prologue<G32>(cfg, fs.pk + base + li, ws, lane);
    bool barrier = c->serial != 0;
    bool ok = true;
    const int nb = c->n_barrier;
    // -- dependencies
    if (c->serial) {
      if (r - 1 >= start) ok = wait_epoch(fs.done + base + r - 1, epoch, fs.err_flag);
    } else {
      // Barriers (escaped peaks of earlier attempts, unbounded steps) are
      // ascending: the last one <= r decides.  A barrier waits until the
      // completed prefix reaches it (every lower rank done); a later rank
      // waits for the last barrier below it, which is done only after
      // every rank below that barrier.
      int lo = 0, hi = nb;   // first barrier index with barrier > r
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (c->barrier[mid] <= r) lo = mid + 1;
        else hi = mid;
      }
      const int bprev = lo > 0 ? c->barrier[lo - 1] : -1;
      if (bprev == r) barrier = true;
      if (barrier) {
        ok = wait_prefix(&c->frontier, r, fs.done + base, c->nrun, epoch, fs.err_flag, lane);
      } else {
        if (bprev >= start) ok = wait_epoch(fs.done + base + bprev, epoch, fs.err_flag);
        // lower-index RUNNING neighbours whose dilated footprints overlap:
        // lane l < 9 reads the range of neighbouring cell l, then the
        // candidates of all nine cells are checked 32 at a time
        const int cw = cfg.cell;
        const int cx = ax / cw, cy = ay / cw;
        const int* cs = fs.cell_start + (size_t)f * (cfg.gx * cfg.gy + 1);
        int c0 = 0, cnt = 0;
        if (lane < 9) {
          const int yy = cy - 1 + lane / 3, xx = cx - 1 + lane % 3;
          if (yy >= 0 && yy < cfg.gy && xx >= 0 && xx < cfg.gx) {
            c0 = cs[yy * cfg.gx + xx];
            cnt = cs[yy * cfg.gx + xx + 1] - c0;
          }
        }
        int off = cnt;   // inclusive prefix sum over the nine cells
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, off, o);
          if (lane >= o) off += t;
        }
        const int total = __shfl_sync(0xffffffffu, off, 8);
        off -= cnt;      // exclusive
        for (int j0 = 0; j0 < total && ok; j0 += 32) {
          const int j = j0 + lane;
          // the cell holding candidate j: the last cell whose offset is <= j
          int idx = -1;
#pragma unroll
          for (int k = 0; k < 9; k++) {
            const int ok_ = __shfl_sync(0xffffffffu, off, k);
            const int ck = __shfl_sync(0xffffffffu, c0, k);
            if (j < total && j >= ok_) idx = ck + (j - ok_);
          }
          int q = -1;
          if (idx >= 0) {
            const int2 e = fs.cell_items[base + idx];
            if (e.x < r && e.x >= start) {
              const unsigned b0 = (unsigned)e.y;
              const int bx = b0 & 0xffff, by = b0 >> 16;
              if (footprints_overlap(bx - ax, by - ay, cfg.roi, dil)) q = e.x;
            }
          }
          // each lane reads its own candidate's done flag (one round trip
          // for all of them); only the ranks not yet done are waited for,
          // one at a time by the whole warp.  The __syncwarp orders every
          // lane's later reads after the lanes' acquire loads.
          const bool pend = (q >= 0) && (ld_acquire(fs.done + base + q) != epoch);
          unsigned m = __ballot_sync(0xffffffffu, pend);
          while (m && ok) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const int qq = __shfl_sync(0xffffffffu, q, src);
            ok = wait_epoch(fs.done + base + qq, epoch, fs.err_flag);
          }
          __syncwarp();
        }
      }
    }
    if (!ok) return;   // a wait timed out: err_flag is set, the host reports it
    // A lower rank of this attempt escaped: every rank above it re-runs in
    // the next attempt, so this one is skipped now (record and image stay
    // as they are, nothing to roll back).
    if (*((volatile int*)&c->escaped_min) < r) {
      __syncwarp();
      if (lane == 0) st_release(fs.done + base + r, epoch);
      if (nb > 0) advance_prefix(&c->frontier, fs.done + base, c->nrun, epoch, lane);
      continue;
    }
    // No fence before the step: every lane made its own acquire load of each
    // dependency's done flag, which orders the step's reads after the
    // predecessors' writes (released after their own fence below).
    // -- the step
    bool esc;
    if constexpr (G32 >= 0)
      esc = lm_step_g32<G32>(cfg, fs, (long long)f * fs.npix, fs.pk + base + li, barrier, dil, ws,
                             fs.stepctr + (size_t)(base + li) * NCOUNTERS, lane);
    else
      esc = lm_step(cfg, fs, (long long)f * fs.npix, fs.pk + base + li, barrier, dil, ws,
                    fs.stepctr + (size_t)(base + li) * NCOUNTERS, lane);
    if (esc && lane == 0) {
      atomicMin(&c->escaped_min, r);
      int slot = atomicAdd(&c->n_escaped, 1);
      if (slot < MAX_ESCAPES) c->escaped[slot] = r;
    }
    __threadfence();
    __syncwarp();
    if (lane == 0) st_release(fs.done + base + r, epoch);
    if (nb > 0) advance_prefix(&c->frontier, fs.done + base, c->nrun, epoch, lane);
  }
}

// ---------------------------------------------------------------------------
// k_prepare: one CTA (1024 threads) per frame
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(1024) k_prepare(ModelCfg cfg, FrameSet<T> fs) {
  extern __shared__ __align__(16) char smem[];
  __shared__ int sc32[33];
  __shared__ int s_total;
  const int f = blockIdx.x;
  FrameCtl* c = fs.ctl + f;
  const int phase = c->phase;
  const int base = fs.pk_off[f];
  const int tid = threadIdx.x;
  if (phase == PH_SWEEP_PENDING) {
    // Within a fit a peak only leaves RUNNING, so after the first sweep the
    // candidates are the previous sweep's run list (compacted in place:
    // every kept entry moves to a lower or equal position, and a chunk is
    // read before any of it is written).
    const bool from_run = c->sweeps > 0;
    const int n = from_run ? c->nrun : fs.nfit[f];
    int nrun = 0;
    for (int c0 = 0; c0 < n; c0 += 1024) {
      const int k = c0 + tid;
      const int i = (k < n) ? (from_run ? fs.run[base + k] : k) : -1;
      __syncthreads();
      int flag = 0;
      if (i >= 0 && fs.pk[base + i].status == RUNNING) {
        // A RUNNING peak always has an in-image ROI, except one re-marked
        // RUNNING by the caller after a failed placement; it cannot be
        // fitted (its ROI is outside the image) and is set to ERROR.
        const PeakRec& q = fs.pk[base + i];
        if (q.xi < 0 || q.yi < 0 || q.xi >= cfg.nx - cfg.roi || q.yi >= cfg.ny - cfg.roi)
          fs.pk[base + i].status = ERROR;
        else
          flag = 1;
      }
      int tot;
      const int pos = block_excl_scan(flag, sc32, tot);
      if (flag) {
        const PeakRec& rec = fs.pk[base + i];
        fs.run[base + nrun + pos] = i;
        fs.snap[base + i] = rec;
        fs.anchor0[base + nrun + pos] = pack_anchor(rec.xi, rec.yi);
      }
      nrun += tot;
    }
    // grid of dilated-footprint anchors (counting sort by cell)
    const int ncell = cfg.gx * cfg.gy;
    int* cntc = reinterpret_cast<int*>(smem);
    for (int i = tid; i < ncell; i += 1024) cntc[i] = 0;
    __syncthreads();
    for (int r = tid; r < nrun; r += 1024) {
      const unsigned a = fs.anchor0[base + r];
      const int cell = ((a >> 16) / cfg.cell) * cfg.gx + (a & 0xffff) / cfg.cell;
      atomicAdd(&cntc[cell], 1);
    }
    __syncthreads();
    int* cs = fs.cell_start + (size_t)f * (ncell + 1);
    // exclusive scan of ncell counts: per-thread contiguous chunk
    const int per = (ncell + 1023) / 1024;
    const int lo = tid * per, hi = min(lo + per, ncell);
    int local = 0;
    for (int i = lo; i < hi; i++) local += cntc[i];
    int tot;
    int off = block_excl_scan(local, sc32, tot);
    for (int i = lo; i < hi; i++) {
      const int v = cntc[i];
      cs[i] = off;
      cntc[i] = off;   // becomes the fill cursor
      off += v;
    }
    if (tid == 0) cs[ncell] = tot;
    __syncthreads();
    for (int r = tid; r < nrun; r += 1024) {
      const unsigned a = fs.anchor0[base + r];
      const int cell = ((a >> 16) / cfg.cell) * cfg.gx + (a & 0xffff) / cfg.cell;
      const int slot = atomicAdd(&cntc[cell], 1);
      fs.cell_items[base + slot] = make_int2(r, (int)a);
    }
    if (tid == 0) {
      c->nrun = nrun;
      c->start = 0;
      c->grab = 0;
      c->frontier = 0;
      c->escaped_min = INT_MAX;
      c->n_escaped = 0;
      c->n_barrier = 0;
      c->serial = cfg.force_serial;
      // the late dilation from sweep dil_switch on, unless the previous
      // sweep of this frame re-ran more than once (anchors still moving
      // in many places: a dense frame then spends more on re-runs than
      // the wider footprints cost)
      c->dil = (c->sweeps >= cfg.dil_switch && c->attempts <= 2) ? cfg.dil_late : cfg.dil;
      c->attempts = 1;
      c->phase = nrun > 0 ? PH_IN_SWEEP : PH_IN_SWEEP;
    }
  } else if (phase == PH_RERUN_PENDING) {
    const int b = c->escaped_min;
    const int nrun = c->nrun;
    // barriers: merge the escaped run ranks
    if (tid == 0) {
      // merge the escaped run ranks into the ascending barrier list
      const int ne = min(c->n_escaped, MAX_ESCAPES);
      for (int e = 0; e < ne; e++) {
        const int r = c->escaped[e];
        int pos = 0;
        while (pos < c->n_barrier && c->barrier[pos] < r) pos++;
        if (pos < c->n_barrier && c->barrier[pos] == r) continue;
        if (c->n_barrier >= MAX_BARRIERS) {
          c->serial = 1;
          continue;
        }
        for (int q = c->n_barrier; q > pos; q--) c->barrier[q] = c->barrier[q - 1];
        c->barrier[pos] = r;
        c->n_barrier++;
      }
      if (c->n_escaped > MAX_ESCAPES) c->serial = 1;
      s_total = 0;
    }
    __syncthreads();
    // roll back run ranks > b: remove the current contribution, restore the snapshot
    const int lane = tid & 31, wid = tid >> 5;
    const int nws = cta_ws_warps(cfg);
    WarpWS<T> ws = warp_ws<T>(smem + (size_t)(wid < nws ? wid : 0) * warp_ws_bytes<T>(cfg, 0), cfg, 0);
    const long long fbase = (long long)f * fs.npix;
    for (int r = b + 1 + wid; wid < nws && r < nrun; r += nws) {
      const int li = fs.run[base + r];
      PeakRec cur, sn;
      load_rec(fs.pk + base + li, cur);
      load_rec(fs.snap + base + li, sn);
      // ranks skipped after the escape (or escaped themselves) are untouched
      bool same = true;
      const long long* wa = reinterpret_cast<const long long*>(&cur);
      const long long* wb = reinterpret_cast<const long long*>(&sn);
#pragma unroll
      for (int q = 0; q < (int)(sizeof(PeakRec) / 8); q++) same = same && (wa[q] == wb[q]);
      if (same) continue;
      if (cur.added > 0) {
        SplinePos s = shape_tables(cfg, cur, ws, lane);
        add_peak(cfg, fs, fbase, cur, s, ws, -1, lane);
      }
      __syncwarp();
      if (sn.added > 0) {
        SplinePos s = shape_tables(cfg, sn, ws, lane);
        add_peak(cfg, fs, fbase, sn, s, ws, +1, lane);
      }
      __syncwarp();
      if (lane == 0) fs.pk[base + li] = sn;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
      c->start = b;
      c->grab = b;
      c->frontier = b;
      c->escaped_min = INT_MAX;
      c->n_escaped = 0;
      c->attempts += 1;
      c->reruns_total += 1;
      c->barriers_total = c->barriers_total + c->n_barrier;
      c->phase = PH_IN_SWEEP;
    }
  }
}

// ---------------------------------------------------------------------------
// k_post: one CTA (1024 threads) per frame
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(1024) k_post(ModelCfg cfg, FrameSet<T> fs) {
  extern __shared__ __align__(16) char smem[];
  __shared__ long long s_ctr[NCOUNTERS];
  __shared__ int s_unconv;
  __shared__ int s_nmove;
  __shared__ int s_move[1024];
  const int f = blockIdx.x;
  FrameCtl* c = fs.ctl + f;
  // the next tick's epoch (every k_sweep of this tick has finished)
  if (f == 0 && threadIdx.x == 0) *fs.epoch += 1;
  if (c->phase != PH_IN_SWEEP) return;
  const int tid = threadIdx.x;
  if (c->escaped_min != INT_MAX) {
    __syncthreads();
    if (tid == 0) c->phase = PH_RERUN_PENDING;
    return;
  }
  if (tid < NCOUNTERS) s_ctr[tid] = 0;
  if (tid == 0) s_unconv = 0;
  __syncthreads();
  const int base = fs.pk_off[f];
  const int nrun = c->nrun;
  const int lane = tid & 31, wid = tid >> 5;
  const int nws = cta_ws_warps(cfg);
  WarpWS<T> ws = warp_ws<T>(smem + (size_t)(wid < nws ? wid : 0) * warp_ws_bytes<T>(cfg, 0), cfg, 0);
  const long long fbase = (long long)f * fs.npix;
  // recenter (mFitRecenterPeaks multi_fit.c:1644-1690); order-free with
  // fixed-point accumulation.  The run ranks are scanned a thread each; the
  // peaks that move their ROI are listed and then re-added a warp each.
  int lost = 0, margin = 0, negh = 0, unconv = 0;
  for (int c0 = 0; c0 < nrun; c0 += 1024) {
    if (tid == 0) s_nmove = 0;
    __syncthreads();
    const int rr = c0 + tid;
    if (rr < nrun) {
      const PeakRec* q = fs.pk + base + fs.run[base + rr];
      if (__ldcg(&q->status) == RUNNING) {
        const double dx = __ldcg(&q->p[PX]) - __ldcg(&q->xi), dy = __ldcg(&q->p[PY]) - __ldcg(&q->yi);
        if ((dx < -0.25) || (dx > 1.25) || (dy < -0.25) || (dy > 1.25)) s_move[atomicAdd(&s_nmove, 1)] = rr;
        else unconv++;
      }
    }
    __syncthreads();
    const int nmove = s_nmove;
    for (int m = wid; wid < nws && m < nmove; m += nws) {
      const int li = fs.run[base + s_move[m]];
      PeakRec rec;
      load_rec(fs.pk + base + li, rec);
      SplinePos s = shape_tables(cfg, rec, ws, lane);
      add_peak(cfg, fs, fbase, rec, s, ws, -1, lane);
      __syncwarp();
      rec.added -= 1;
      rec.xi = (int)floor(rec.p[PX]);
      rec.yi = (int)floor(rec.p[PY]);
      const int chk = base_check(cfg, rec);
      if (chk) {
        if (lane == 0) {
          lost++;
          if (chk == 1) margin++;
          else negh++;
        }
        rec.status = ERROR;
      } else {
        SplinePos s2 = shape_tables(cfg, rec, ws, lane);
        add_peak(cfg, fs, fbase, rec, s2, ws, +1, lane);
        rec.added += 1;
      }
      __syncwarp();
      if (lane == 0) {
        fs.pk[base + li] = rec;
        if (rec.status == RUNNING) unconv++;
      }
    }
    __syncthreads();
  }
  // counters of this sweep's steps
  long long loc[NCOUNTERS];
  for (int i = 0; i < NCOUNTERS; i++) loc[i] = 0;
  for (int r = tid; r < nrun; r += 1024) {
    const int li = fs.run[base + r];
    const int* sc = fs.stepctr + (size_t)(base + li) * NCOUNTERS;
    for (int i = 0; i < NCOUNTERS; i++) loc[i] += sc[i];
  }
  loc[C_LOST] += lost;
  loc[C_MARGIN] += margin;
  loc[C_NEGH] += negh;
  for (int i = 0; i < NCOUNTERS; i++) {
    long long v = loc[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0 && v) atomicAdd(reinterpret_cast<unsigned long long*>(&s_ctr[i]), (unsigned long long)v);
  }
  for (int o = 16; o > 0; o >>= 1) unconv += __shfl_xor_sync(0xffffffffu, unconv, o);
  if (lane == 0 && unconv) atomicAdd(&s_unconv, unconv);
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    for (int i = 0; i < NCOUNTERS; i++) c->ctr[i] += s_ctr[i];
    c->unconverged = s_unconv;
    c->sweeps += 1;
    c->phase = (s_unconv == 0 || c->sweeps >= c->max_sweeps) ? PH_DONE : PH_SWEEP_PENDING;
  }
}

// ---------------------------------------------------------------------------
// k_tail: the remaining sweeps of frames with few RUNNING peaks, one launch
// ---------------------------------------------------------------------------

// One warp (a 32-thread CTA) per frame.  A frame whose fit has made at least
// one sweep and has at most tail_peaks RUNNING peaks left runs all of its
// remaining sweeps here, each as k_prepare + k_sweep + k_post would: the
// RUNNING peaks of the previous sweep's run list, in index order, take their
// LM steps one after another -- the reference's own sequential order
// (mFitIterateLM multi_fit.c:1072-1349), so every step is unbounded and
// needs no dependency wait or escape -- then the moved peaks are recentered
// (mFitRecenterPeaks :1644-1690), the counters summed and the frame's
// next phase decided (dao_fit_c.py:332-356).  The results are the ones the
// normal ticks give; what goes is two launches and a host poll per sweep.
template <typename T, int G32>
__global__ void __launch_bounds__(32) k_tail(ModelCfg cfg, FrameSet<T> fs, int tail_peaks) {
  extern __shared__ __align__(16) char smem[];
  const int lane = threadIdx.x;
  const int f = blockIdx.x;
  FrameCtl* c = fs.ctl + f;
  if (c->phase != PH_SWEEP_PENDING || c->sweeps == 0 || c->unconverged > tail_peaks) return;
  WarpWS<T> ws = warp_ws<T>(smem, cfg, cfg.nroi);
  {
    unsigned short* roi = reinterpret_cast<unsigned short*>(smem + warp_ws_bytes<T>(cfg, cfg.nroi));
    for (int i = lane; i < cfg.nroi; i += 32) roi[i] = fs.roi_xy[i];
    __syncwarp();
    ws.roi = roi;
  }
  const int base = fs.pk_off[f];
  const long long fbase = (long long)f * fs.npix;
  int nrun = c->nrun;
  for (;;) {
    // run list: the previous run list's RUNNING peaks, in order (k_prepare)
    int m = 0;
    for (int k0 = 0; k0 < nrun; k0 += 32) {
      const int k = k0 + lane;
      const int i = (k < nrun) ? fs.run[base + k] : -1;
      bool flag = false;
      if (i >= 0 && fs.pk[base + i].status == RUNNING) {
        const PeakRec& q = fs.pk[base + i];
        if (q.xi < 0 || q.yi < 0 || q.xi >= cfg.nx - cfg.roi || q.yi >= cfg.ny - cfg.roi)
          fs.pk[base + i].status = ERROR;
        else
          flag = true;
      }
      const unsigned bal = __ballot_sync(0xffffffffu, flag);
      __syncwarp();
      if (flag) fs.run[base + m + __popc(bal & ((1u << lane) - 1u))] = i;
      m += __popc(bal);
      __syncwarp();
    }
    nrun = m;
    // the steps, one after another in index order (k_sweep)
    long long loc[NCOUNTERS];
#pragma unroll
    for (int i = 0; i < NCOUNTERS; i++) loc[i] = 0;
    for (int r = 0; r < nrun; r++) {
      const int li = fs.run[base + r];
      int* sc = fs.stepctr + (size_t)(base + li) * NCOUNTERS;
      if constexpr (G32 >= 0) {
        g32_prologue<G32>(cfg, fs.pk + base + li, ws, lane);
        lm_step_g32<G32>(cfg, fs, fbase, fs.pk + base + li, true, 0, ws, sc, lane);
      } else {
        lm_step(cfg, fs, fbase, fs.pk + base + li, true, 0, ws, sc, lane);
      }
      __threadfence();
      __syncwarp();
      if (lane == 0)
        for (int i = 0; i < NCOUNTERS; i++) loc[i] += sc[i];
      __syncwarp();
    }
    // recenter, count (k_post)
    int unconv = 0;
    for (int r = 0; r < nrun; r++) {
      const int li = fs.run[base + r];
      PeakRec rec;
      load_rec(fs.pk + base + li, rec);
      if (rec.status != RUNNING) continue;
      const double dx = rec.p[PX] - rec.xi, dy = rec.p[PY] - rec.yi;
      if (!((dx < -0.25) || (dx > 1.25) || (dy < -0.25) || (dy > 1.25))) {
        unconv++;
        continue;
      }
      SplinePos sp = shape_tables(cfg, rec, ws, lane);
      add_peak(cfg, fs, fbase, rec, sp, ws, -1, lane);
      __syncwarp();
      rec.added -= 1;
      rec.xi = (int)floor(rec.p[PX]);
      rec.yi = (int)floor(rec.p[PY]);
      const int chk = base_check(cfg, rec);
      if (chk) {
        if (lane == 0) {
          loc[C_LOST]++;
          loc[chk == 1 ? C_MARGIN : C_NEGH]++;
        }
        rec.status = ERROR;
      } else {
        SplinePos s2 = shape_tables(cfg, rec, ws, lane);
        add_peak(cfg, fs, fbase, rec, s2, ws, +1, lane);
        rec.added += 1;
        unconv++;
      }
      __threadfence();
      __syncwarp();
      if (lane == 0) fs.pk[base + li] = rec;
      __syncwarp();
    }
    if (lane == 0) {
      for (int i = 0; i < NCOUNTERS; i++) c->ctr[i] += loc[i];
      c->unconverged = unconv;
      c->sweeps += 1;
      c->nrun = nrun;
      c->attempts = 1;
      c->phase = (unconv == 0 || c->sweeps >= c->max_sweeps) ? PH_DONE : PH_SWEEP_PENDING;
    }
    __syncwarp();
    if (unconv == 0 || *((volatile int*)&c->sweeps) >= c->max_sweeps) break;
  }
}

// ---------------------------------------------------------------------------
// frame ingest
// ---------------------------------------------------------------------------

// mFitNewImage multi_fit.c:1382-1408: x = image * rqe + scmos; reset the fit.
template <typename T, typename I>
__global__ void k_new_image(FrameSet<T> fs, const I* img, int frame0, int nframes) {
  const long long n = fs.npix * nframes;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long k = i % fs.npix;
    const long long g = (long long)frame0 * fs.npix + i;
    const double v = (double)img[i] * (double)fs.rqe[k] + (double)fs.scmos[k];
    const_cast<T*>(fs.x)[g] = (T)v;
    if (fs.xq) {
      const long long q = __double2ll_rn(v * 68719476736.0);
      const_cast<long long*>(fs.xq)[g] = q;
      // q 2^-36 is exact in double for |v| < 2^17; its float-float pair
      const double d = (double)q * 1.4551915228366852e-11;
      const float h = __double2float_rn(d);
      const_cast<float2*>(fs.xff)[g] = make_float2(h, __double2float_rn(d - (double)h));
    }
    for (int w = 0; w < AccW<T>::W; w++) {
      fs.f[g * AccW<T>::W + w] = 0;
      fs.bg[g * AccW<T>::W + w] = 0;
    }
    fs.cnt[g] = 0;
  }
}

// mFitNewBackground multi_fit.c:1360-1370: bg_estimate = background * rqe.
template <typename T, typename I>
__global__ void k_new_background(FrameSet<T> fs, const I* bgin, int frame0, int nframes) {
  const long long n = fs.npix * nframes;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long k = i % fs.npix;
    const long long g = (long long)frame0 * fs.npix + i;
    const_cast<double*>(fs.bgest)[g] = (double)bgin[i] * (double)fs.rqe[k];
  }
}

// ---------------------------------------------------------------------------
// new peaks (daoNewPeaks dao_fit.c:1582-1766, cfNewPeaks cubic_fit.c:758-928)
// ---------------------------------------------------------------------------

// Parameters of a new peak from its input row; returns the record.
__device__ inline PeakRec new_peak_rec(const ModelCfg& cfg, const double* q, int ptype) {
  PeakRec w;
  for (int i = 0; i < 7; i++) w.p[i] = 0.0;
  w.error = 0.0;
  w.lambda = LAMBDA_START;
  w.wxt = w.wyt = 0.0;
  w.added = 0;
  w.iterations = 0;
  w.status = RUNNING;
  w.zi = 0;
  for (int i = 0; i < 4; i++) w.pad[i] = 0;
  const bool spl = is_arb(cfg.model);   // the arbitrary-PSF input formats
  w.p[PX] = q[0] - cfg.xoff;
  w.p[PY] = q[1] - cfg.yoff;
  w.p[PZ] = q[2] - cfg.zoff;
  if (ptype == PT_TEXT) {
    w.p[PBG] = q[3];
    w.p[PH] = q[4];
    if (!spl) {
      w.p[PXW] = 1.0 / (2.0 * q[5] * q[5]);
      w.p[PYW] = 1.0 / (2.0 * q[6] * q[6]);
      if (cfg.model == M_Z) widths_from_z(cfg, w);
    }
  } else if (!spl) {
    if (cfg.model == M_Z) {
      widths_from_z(cfg, w);
    } else {
      const double wd = 1.0 / (2.0 * q[3] * q[3]);
      w.p[PXW] = wd;
      w.p[PYW] = wd;
    }
  }
  w.xi = (int)floor(w.p[PX]);
  w.yi = (int)floor(w.p[PY]);
  if (is_spline(cfg.model)) w.zi = (int)w.p[PZ];
  if (ptype != PT_TEXT) {
    w.p[PBG] = 1.0;
    w.p[PH] = 1.0;
  }
  return w;
}

// Initialise (and for "testing"/"text" add) the new peaks; warp per peak.
// slots[i] = global peak slot; frames[i] = frame of peak i.
template <typename T>
__global__ void k_newpeaks(ModelCfg cfg, FrameSet<T> fs, const double* rows, int ncol, int ptype,
                           const int* slots, const int* frames, int n, int do_add) {
  extern __shared__ __align__(16) char smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  WarpWS<T> ws = warp_ws<T>(smem + (size_t)wib * warp_ws_bytes<T>(cfg, 0), cfg, 0);
  const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int i = gw; i < n; i += nw) {
    PeakRec w = new_peak_rec(cfg, rows + (size_t)i * ncol, ptype);
    const int f = frames[i];
    const long long fbase = (long long)f * fs.npix;
    const int chk = check_for(cfg, cfg.model, w);
    if (chk) {
      w.status = ERROR;
      if (lane == 0) {
        fs.pk[slots[i]] = w;
        atomicAdd(reinterpret_cast<unsigned long long*>(&fs.ctl[f].ctr[chk == 1 ? C_MARGIN : C_NEGH]), 1ull);
      }
      continue;
    }
    SplinePos s = shape_tables(cfg, w, ws, lane);
    if (ptype != PT_TEXT) {
      // mFitEstimatePeakBackground multi_fit.c:638-662
      double t = 0.0;
      for (int p = lane; p < cfg.nroi; p += 32) {
        int rx, ry;
        roi_rc(fs.roi_xy, p, rx, ry);
        const long long k = pix_index(cfg, w.xi, w.yi, rx, ry);
        t += fs.bgest[fbase + k] / (double)__ldg(fs.rqe + k);
      }
      t = warp_sum(t);
      w.p[PBG] = t / ((double)cfg.nroi);
    }
    if (do_add) {
      add_peak(cfg, fs, fbase, w, s, ws, +1, lane);
      w.added = 1;
    }
    if (lane == 0) fs.pk[slots[i]] = w;
    __syncwarp();
  }
}

// "finder" peaks, one warp per frame in input order: the height estimate
// (mFitEstimatePeakHeight multi_fit.c:678-700) reads the fit image that
// already holds the earlier new peaks.
template <typename T>
__global__ void k_newpeaks_finder(ModelCfg cfg, FrameSet<T> fs, const int* slots, const int* frame_first,
                                  const int* frame_n, int nframes) {
  extern __shared__ __align__(16) char smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  WarpWS<T> ws = warp_ws<T>(smem + (size_t)wib * warp_ws_bytes<T>(cfg, 0), cfg, 0);
  const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
  if (gw >= nframes) return;
  const int i0 = frame_first[gw], n = frame_n[gw];
  for (int j = 0; j < n; j++) {
    const int slot = slots[i0 + j];
    PeakRec w;
    load_rec(fs.pk + slot, w);
    if (w.status != RUNNING) continue;
    const int f = gw;
    const long long fbase = (long long)f * fs.npix;
    SplinePos s = shape_tables(cfg, w, ws, lane);
    double sp = 0.0, sx = 0.0;
    for (int p = lane; p < cfg.nroi; p += 32) {
      int rx, ry;
      roi_rc(fs.roi_xy, p, rx, ry);
      const long long k = pix_index(cfg, w.xi, w.yi, rx, ry);
      const double t = (double)psf_at(cfg, fs.aij, ws, s, rx, ry) * (double)__ldg(fs.rqe + k);
      sp += t * t * t;
      const double fv = acc_value<AccW<T>::W>(acc_load<AccW<T>::W>(fs.f, fbase + k));
      sx += t * t * ((double)__ldg(fs.x + fbase + k) - fv - fs.bgest[fbase + k]);
    }
    sp = warp_sum(sp);
    sx = warp_sum(sx);
    w.p[PH] = sx / sp;
    if (w.p[PH] < cfg.min_height) w.p[PH] = cfg.min_height;
    if (w.p[PH] <= 0.0) {
      w.status = ERROR;
    } else {
      add_peak(cfg, fs, fbase, w, s, ws, +1, lane);
      w.added = 1;
    }
    __threadfence();
    __syncwarp();
    if (lane == 0) fs.pk[slot] = w;
    __syncwarp();
  }
}

// Initial error of the new peaks (dao_fit.c:1757-1763), warp per peak.
template <typename T>
__global__ void k_peak_error(ModelCfg cfg, FrameSet<T> fs, const int* slots, const int* frames, int n) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = gw; i < n; i += nw) {
    const int slot = slots[i];
    PeakRec w;
    load_rec(fs.pk + slot, w);
    if (w.status != RUNNING) continue;
    const long long fbase = (long long)frames[i] * fs.npix;
    double dev = 0.0;
    bool fail = false;
    for (int p = lane; p < cfg.nroi; p += 32) {
      int rx, ry;
      roi_rc(fs.roi_xy, p, rx, ry);
      const long long k = pix_index(cfg, w.xi, w.yi, rx, ry);
      const double fi = fi_global(fs, fbase + k);
      const T xv = __ldg(fs.x + fbase + k);
      if (!(fi > 0.0)) fail = true;
      else dev += (double)deviance((T)fi, xv);
    }
    dev = warp_sum(dev);
    fail = __any_sync(0xffffffffu, fail);
    if (lane == 0) {
      if (fail) atomicAdd(reinterpret_cast<unsigned long long*>(&fs.ctl[frames[i]].ctr[C_NEGFI]), 1ull);
      else fs.pk[slot].error = dev;
    }
  }
}

// ---------------------------------------------------------------------------
// properties and status edits
// ---------------------------------------------------------------------------

// Per-peak sums (mFitPeakSum :1620-1632, mFitPeakFgSum :1578-1610,
// mFitPeakBgSum :1518-1565) and, optionally, the Jacobian with the current
// model values (mFitGetPeakPropertyDouble "jacobian", :791-805).
template <typename T>
__global__ void k_peak_props(ModelCfg cfg, FrameSet<T> fs, const int* slots, const int* frames, int n,
                             double* out_sum, double* out_fg, double* out_bg, double* out_jac) {
  extern __shared__ __align__(16) char smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  WarpWS<T> ws = warp_ws<T>(smem + (size_t)wib * warp_ws_bytes<T>(cfg, 0), cfg, 0);
  const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int i = gw; i < n; i += nw) {
    PeakRec w;
    load_rec(fs.pk + slots[i], w);
    const long long fbase = (long long)frames[i] * fs.npix;
    const bool inside = (w.xi >= 0) && (w.yi >= 0) && (w.xi + cfg.roi <= cfg.nx) && (w.yi + cfg.roi <= cfg.ny);
    if (!inside) {
      if (lane == 0) {
        if (out_sum) { out_sum[i] = 0.0; out_fg[i] = 1.0; out_bg[i] = 1.0; }
        if (out_jac) for (int l = 0; l < cfg.jac; l++) out_jac[(size_t)i * cfg.jac + l] = 0.0;
      }
      continue;
    }
    SplinePos s = shape_tables(cfg, w, ws, lane);
    double ps = 0.0, ps2 = 0.0, bs = 0.0;
    double gxd, gyd;
    z_factors(cfg, cfg.model, w, gxd, gyd);
    T acc[32];
    for (int q = 0; q < 32; q++) acc[q] = (T)0;
    for (int p = lane; p < cfg.nroi; p += 32) {
      int rx, ry;
      roi_rc(fs.roi_xy, p, rx, ry);
      const long long k = pix_index(cfg, w.xi, w.yi, rx, ry);
      const T psfT = psf_at(cfg, fs.aij, ws, s, rx, ry);
      const double psf = (double)psfT;
      ps += psf;
      ps2 += psf * psf;
      const double xv = (double)__ldg(fs.x + fbase + k);
      const double bgv = (xv - (double)__ldg(fs.scmos + k)) / (double)__ldg(fs.rqe + k) - w.p[PH] * psf;
      bs += bgv * psf * psf;
      if (out_jac) {
        const double fi = fi_global(fs, fbase + k);
        const T fiT = (T)fi;
        const T t1 = (T)2 * ((T)1 - (T)xv / fiT);
        T jt[MAX_JAC];
        jt_row(cfg, fs.aij, ws, s, w, (T)gxd, (T)gyd, rx, ry, __ldg(fs.rqe + k), psfT, jt);
        for (int l = 0; l < MAX_JAC; l++)
          if (l < cfg.jac) acc[l] += t1 * jt[l];
      }
    }
    ps = warp_sum(ps);
    ps2 = warp_sum(ps2);
    bs = warp_sum(bs);
    if (out_jac) {
      for (int l = 0; l < cfg.jac; l++) {
        T v = warp_sum(acc[l]);
        if (lane == 0) out_jac[(size_t)i * cfg.jac + l] = (double)v;
      }
    }
    if (lane == 0 && out_sum) {
      out_sum[i] = ps * w.p[PH];
      out_fg[i] = (ps > 0.0) ? (w.p[PH] * ps2) / ps : 1.0;
      out_bg[i] = ((bs > 0.0) && (ps > 0.0)) ? bs / (ps * ps) : 1.0;
    }
  }
}

// mFitSetPeakStatus multi_fit.c:1809-1831: ERROR peaks still in the image
// are subtracted first.
template <typename T>
__global__ void k_set_status(ModelCfg cfg, FrameSet<T> fs, const int* slots, const int* frames,
                             const int* status, int n) {
  extern __shared__ __align__(16) char smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  WarpWS<T> ws = warp_ws<T>(smem + (size_t)wib * warp_ws_bytes<T>(cfg, 0), cfg, 0);
  const int gw = blockIdx.x * (blockDim.x >> 5) + wib;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int i = gw; i < n; i += nw) {
    PeakRec w;
    load_rec(fs.pk + slots[i], w);
    const bool inside = (w.xi >= 0) && (w.yi >= 0) && (w.xi < cfg.nx - cfg.roi) && (w.yi < cfg.ny - cfg.roi);
    if (status[i] == ERROR && w.added > 0 && inside) {
      SplinePos s = shape_tables(cfg, w, ws, lane);
      add_peak(cfg, fs, (long long)frames[i] * fs.npix, w, s, ws, -1, lane);
      w.added -= 1;
    }
    w.status = status[i];
    __syncwarp();
    if (lane == 0) fs.pk[slots[i]] = w;
  }
}

// Fit image f / rqe (mFitGetFitImage :708-720) or residual x - f
// (mFitGetResidual :880-888).
template <typename T>
__global__ void k_fit_image(FrameSet<T> fs, int frame, double* out, int residual) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < fs.npix;
       k += (long long)gridDim.x * blockDim.x) {
    const long long g = (long long)frame * fs.npix + k;
    const double fv = acc_value<AccW<T>::W>(acc_load<AccW<T>::W>(fs.f, g));
    out[k] = residual ? ((double)fs.x[g] - fv) : fv / (double)fs.rqe[k];
  }
}

}  // namespace sa
