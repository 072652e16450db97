// sa_mp.cuh -- multi-plane fitting on the device: the coupled LM sweep of
// multi_plane/mp_fit.c (mpIterateLM) with the parameter updates of
// mp_fit_arb.c (spline, pupil-function and FFT PSFs) and mp_fit_dao.c (2D
// Gaussians), over channel engines that each hold one image plane.
//
// A group is one peak per channel at the same index.  Its channels share
// status and lambda; x / y are tied through the affine maps between the
// planes, z (and, unless the heights are independent) the height through
// z-dependent weighted averages of the channels' LM steps.  One warp runs a
// frame's groups in index order, the reference's Gauss-Seidel order, so a
// multi-frame batch is parallel over frames only.  The FP64 engine.
#pragma once

#include "sa_kernels.cuh"
#include "sa_mp_types.h"

namespace sa {

__device__ __forceinline__ long long mp_fbase(const MPChan& c, int f) { return (long long)f * c.fs.npix; }

__device__ __forceinline__ int warp_sum_int(int v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// mFitCalcErr multi_fit.c:111-195 from the global state: the deviance over
// the ROI; true (and no error) when some fi <= 0.
__device__ inline bool mp_error(const MPChan& c, long long fbase, const PeakRec& w, double& dev, int lane) {
  double d = 0.0;
  bool fail = false;
  for (int p = lane; p < c.cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(c.fs.roi_xy, p, rx, ry);
    const long long k = pix_index(c.cfg, w.xi, w.yi, rx, ry);
    const double fi = fi_global(c.fs, fbase + k);
    const double xv = __ldg(c.fs.x + fbase + k);
    if (!(fi > 0.0)) fail = true;
    else d += deviance(fi, xv);
  }
  dev = warp_sum(d);
  return __any_sync(0xffffffffu, fail);
}

// fn_calc_JH on the global state with the peak still added (the fi of the
// preceding mFitCalcErr): gradient and packed upper Hessian into jh.
__device__ inline SplinePos mp_jh(const MPChan& c, long long fbase, const PeakRec& w, WarpWS<double>& ws,
                                  double* jh, int lane) {
  const ModelCfg& cfg = c.cfg;
  const int k = cfg.jac;
  SplinePos s = shape_tables(cfg, w, ws, lane);
  double gxd, gyd;
  z_factors(cfg, cfg.model, w, gxd, gyd);
  double acc[32];
#pragma unroll
  for (int i = 0; i < 32; i++) acc[i] = 0.0;
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(c.fs.roi_xy, p, rx, ry);
    const long long kk = pix_index(cfg, w.xi, w.yi, rx, ry);
    const double fi = fi_global(c.fs, fbase + kk);
    const double xv = __ldg(c.fs.x + fbase + kk);
    const double rq = __ldg(c.fs.rqe + kk);
    const double psf = psf_at(cfg, c.fs.aij, ws, s, rx, ry);
    const double t1 = 2.0 * (1.0 - xv / fi);
    const double t2 = 2.0 * xv / (fi * fi);
    double jt[MAX_JAC];
    jt_row(cfg, c.fs.aij, ws, s, w, gxd, gyd, rx, ry, rq, psf, jt);
#pragma unroll
    for (int l = 0; l < MAX_JAC; l++)
      if (l < k) acc[l] += t1 * jt[l];
#pragma unroll
    for (int l = 0; l < MAX_JAC; l++) {
#pragma unroll
      for (int m = l; m < MAX_JAC; m++) {
        if (l < k && m < k) {
          const int id = k + l * k - (l * (l - 1)) / 2 + (m - l);
          if (id < 32) acc[id] += t2 * jt[l] * jt[m];
        }
      }
    }
  }
  const double v = warp_transpose_sum32(acc, lane);
  if (lane < k + k * (k + 1) / 2) jh[lane] = v;
  __syncwarp();
  return s;
}

// Subtract the peak (its shape tables current in ws) from the plane's image
// and keep the base state of its ROI -- the fit image and background
// without it, rqe, data, count with it -- in the workspace, as lm_step's
// first loop does: the trials are then evaluated from the workspace.
__device__ inline void mp_sub_base(const MPChan& c, long long fbase, const PeakRec& w, const SplinePos& s,
                                   WarpWS<double>& ws, int lane) {
  const ModelCfg& cfg = c.cfg;
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(ws.roi, p, rx, ry);
    const long long kk = pix_index(cfg, w.xi, w.yi, rx, ry);
    const Q2 Fq = acc_load<2>(c.fs.f, fbase + kk);
    const Q2 Bq = acc_load<2>(c.fs.bg, fbase + kk);
    const int Cg = __ldcg(c.fs.cnt + fbase + kk);
    const double rq = __ldg(c.fs.rqe + kk), sc = __ldg(c.fs.scmos + kk);
    const double psf = psf_at(cfg, c.fs.aij, ws, s, rx, ry);
    const Q2 cf = quant_t<double>(contrib_f(w.p[PH], psf, rq));
    const Q2 cb = quant_t<double>(contrib_bg(w.p[PBG], rq, sc));
    acc_red<2>(c.fs.f, fbase + kk, cf, -1);
    acc_red<2>(c.fs.bg, fbase + kk, cb, -1);
    atomicAdd(c.fs.cnt + fbase + kk, -1);
    ws.Fb[p] = acc_value<2>(q_sub(Fq, cf));
    ws.Bs[p] = acc_value<2>(q_sub(Bq, cb)) + sc;
    ws.R[p] = rq;
    ws.X[p] = __ldg(c.fs.x + fbase + kk);
    ws.IC[p] = ic_store<double>(Cg);
  }
  __syncwarp();
}

// The error of the trial w from the base state in ws (the peak added
// virtually; mp_fit.c:340-378 adds it and runs mFitCalcErr): true when some
// fi <= 0.  The shape goes to ws.psf for the final add.
__device__ inline bool mp_trial_error(const MPChan& c, const PeakRec& w, WarpWS<double>& ws, double& dev,
                                      int lane) {
  const ModelCfg& cfg = c.cfg;
  SplinePos s = shape_tables(cfg, w, ws, lane, false);
  const double hh = w.p[PH], bgv = w.p[PBG];
  double d = 0.0;
  bool fail = false;
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(ws.roi, p, rx, ry);
    const double psf = psf_at(cfg, c.fs.aij, ws, s, rx, ry);
    ws.psf[p] = psf;
    const double rq = ws.R[p];
    const double fi = ws.Fb[p] + contrib_f(hh, psf, rq) + bg_div(ws.Bs[p] + bgv * rq, ws.IC[p]);
    if (!(fi > 0.0)) fail = true;
    else d += deviance(fi, ws.X[p]);
  }
  dev = warp_sum(d);
  return __any_sync(0xffffffffu, fail);
}

// Add the accepted trial w (its shape in ws.psf) to the plane's image.
__device__ inline void mp_add_from_ws(const MPChan& c, long long fbase, const PeakRec& w, WarpWS<double>& ws,
                                      int lane) {
  const ModelCfg& cfg = c.cfg;
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(ws.roi, p, rx, ry);
    const long long kk = pix_index(cfg, w.xi, w.yi, rx, ry);
    const double rq = ws.R[p], sc = __ldg(c.fs.scmos + kk);
    acc_red<2>(c.fs.f, fbase + kk, quant_t<double>(contrib_f(w.p[PH], ws.psf[p], rq)), +1);
    acc_red<2>(c.fs.bg, fbase + kk, quant_t<double>(contrib_bg(w.p[PBG], rq, sc)), +1);
    atomicAdd(c.fs.cnt + fbase + kk, 1);
  }
  __syncwarp();
}

// Add (+1) or subtract (-1) channel c's working peak (its shape computed here).
__device__ inline void mp_add(const MPChan& c, long long fbase, const PeakRec& w, WarpWS<double>& ws, int sign,
                              int lane) {
  SplinePos s = shape_tables(c.cfg, w, ws, lane, false);
  add_peak(c.cfg, c.fs, fbase, w, s, ws, sign, lane);
  __syncwarp();
}

// mpWeightIndex mp_fit.c:703-725 (channel 0's working z) and
// mpWeightInterpolate :732-741.
__device__ inline void mp_weight_index(const MPParams& p, double z0, double& dz, int& zi) {
  const double t = p.w_z_scale * (z0 - p.w_z_offset);
  zi = (int)t;
  dz = t - (double)zi;
  if (zi < 0) zi = 0;
  if (zi > p.n_weights - 2) zi = p.n_weights - 2;
}
__device__ inline double mp_weight(const MPParams& p, int which, double dz, int zi, int ch) {
  const double* w = p.w + (size_t)which * p.n_weights * p.nc;
  const double w1 = w[p.nc * zi + ch], w2 = w[p.nc * (zi + 1) + ch];
  return w1 + (w2 - w1) * dz;
}
enum { MPW_BG = 0, MPW_H = 1, MPW_X = 2, MPW_Y = 3, MPW_Z = 4 };

// fn_zrange: ftFitZRangeCheck fft_fit.c:506-524, pfitZRangeCheck
// pupil_fit.c:555-570, cfZRangeCheck cubic_fit.c:987-1005 (which sets zi).
__device__ inline void mp_z_range(const ModelCfg& cfg, PeakRec& w) {
  if (cfg.model == M_FFT) {
    const double max_z = ((double)cfg.sz) * 0.5 - 1.0e-12;
    if (w.p[PZ] < -max_z) w.p[PZ] = -max_z;
    if (w.p[PZ] > max_z) w.p[PZ] = max_z;
  } else if (cfg.model == M_PUPIL) {
    if (w.p[PZ] < cfg.zmin) w.p[PZ] = cfg.zmin;
    if (w.p[PZ] > cfg.zmax) w.p[PZ] = cfg.zmax;
  } else if (cfg.model == M_SPLINE3D) {
    if (w.p[PZ] < 1.0e-12) w.p[PZ] = 1.0e-12;
    const double zmax = ((double)cfg.sz) - 1.0e-12;
    if (w.p[PZ] > zmax) w.p[PZ] = zmax;
    w.zi = (int)(w.p[PZ]);
  }
}

constexpr int MP_DIL = 2;     // ROI growth (pixels) that a bounded step may use

// Per-team coupling state beyond MPShared (the team leader writes).
struct MPCtl {
  double e[MP_MAXCH];          // the planes' errors of the latest evaluation
  int fail[MP_MAXCH];          // the planes' fi <= 0 / escape flags of that evaluation
  int act, undo, esc;
  long long ctr[MP_MAXCH][NCOUNTERS];   // the step's counters per plane (added at commit)
};

struct MPTeam {
  MPShared S;
  MPCtl K;
};

// fn_check of a channel (plane i of a team): daoCheck2D for the Gaussians,
// mFitCheck otherwise; counts the margin / height failures in the team's
// counters.
__device__ inline int mp_check_team(const MPChan& c, PeakRec& w, MPCtl& K, int i) {
  const int r = (c.cfg.model == M_2D) ? model_check(c.cfg, M_2D, w) : base_check(c.cfg, w);
  if (r == 1) K.ctr[i][C_MARGIN]++;
  else if (r == 2) K.ctr[i][C_NEGH]++;
  return r;
}

enum { MPA_EVAL = 0, MPA_CONTINUE = 1, MPA_BREAK = 2 };

// The channels' parameter update from their steps (lane 0): mpArbUpdateFixed
// mp_fit_arb.c:400-432 / mpArbUpdateIndependent :449-470 / mpDaoUpdate
// mp_fit_dao.c:164-209, each with mpUpdate mp_fit.c:626-696 and (arbitrary
// PSFs) mpArbUpdateZ mp_fit_arb.c:351-384.  The 2D Gaussian update moves the
// x width only (the y width keeps its value) and applies daoCheck2D (its
// clamp and counters) without using its result.
__device__ inline void mp_update_team(const MPChan* ch, const MPParams& p, MPShared& S, MPCtl& K) {
  const int nc = p.nc;
  double dz, p_ave, p_total, w;
  int zi;
  if (p.kind == MP_DAO || p.indep) {
    for (int i = 0; i < nc; i++) {
      S.w[i].p[PH] -= S.dl[i][0];
      if (S.w[i].p[PH] < 0.01) S.w[i].p[PH] = 0.01;
      S.heights[i] = S.w[i].p[PH];
    }
  }
  if (p.kind == MP_DAO) {
    for (int i = 0; i < nc; i++) {
      S.w[i].p[PXW] -= S.dl[i][3];
      (void)mp_check_team(ch[i], S.w[i], K, i);
    }
  } else if (!p.indep) {
    mp_weight_index(p, S.w[0].p[PZ], dz, zi);
    p_ave = 0.0;
    p_total = 0.0;
    for (int i = 0; i < nc; i++) {
      w = mp_weight(p, MPW_H, dz, zi, i);
      p_ave += S.dl[i][0] * w;
      p_total += w;
    }
    S.w[0].p[PH] -= p_ave / p_total;
    for (int i = 1; i < nc; i++) S.w[i].p[PH] = S.w[0].p[PH];
  }
  // mpUpdate: x, y
  mp_weight_index(p, S.w[0].p[PZ], dz, zi);
  p_ave = 0.0;
  p_total = 0.0;
  for (int i = 0; i < nc; i++) {
    w = mp_weight(p, MPW_X, dz, zi, i);
    double d = p.xtN0[i * 3 + 1] * S.dl[i][1];
    d += p.xtN0[i * 3 + 2] * S.dl[i][2];
    p_ave += d * w * S.heights[i];
    p_total += w * S.heights[i];
  }
  S.w[0].p[PX] -= p_ave / p_total;
  p_ave = 0.0;
  p_total = 0.0;
  for (int i = 0; i < nc; i++) {
    w = mp_weight(p, MPW_Y, dz, zi, i);
    double d = p.ytN0[i * 3 + 1] * S.dl[i][1];
    d += p.ytN0[i * 3 + 2] * S.dl[i][2];
    p_ave += d * w * S.heights[i];
    p_total += w * S.heights[i];
  }
  S.w[0].p[PY] -= p_ave / p_total;
  const double xoff = ch[0].cfg.xoff, yoff = ch[0].cfg.yoff;
  for (int i = 1; i < nc; i++) {
    double t = p.xt0N[i * 3];
    t += p.xt0N[i * 3 + 1] * (S.w[0].p[PX] + xoff);
    t += p.xt0N[i * 3 + 2] * (S.w[0].p[PY] + yoff);
    S.w[i].p[PX] = t - xoff;
    t = p.yt0N[i * 3];
    t += p.yt0N[i * 3 + 1] * (S.w[0].p[PX] + xoff);
    t += p.yt0N[i * 3 + 2] * (S.w[0].p[PY] + yoff);
    S.w[i].p[PY] = t - yoff;
  }
  for (int i = 0; i < nc; i++) anchor_update(S.w[i]);
  for (int i = 0; i < nc; i++) S.w[i].p[PBG] -= S.dl[i][4];
  if (p.kind == MP_ARB) {
    // mpArbUpdateZ (the weight index from the updated channel-0 z is not
    // needed: z has not moved yet)
    mp_weight_index(p, S.w[0].p[PZ], dz, zi);
    p_ave = 0.0;
    p_total = 0.0;
    for (int i = 0; i < nc; i++) {
      w = mp_weight(p, MPW_Z, dz, zi, i);
      p_ave += S.dl[i][3] * w * S.heights[i];
      p_total += w * S.heights[i];
    }
    const double delta = p_ave / p_total;
    for (int i = 0; i < nc; i++) {
      S.w[i].p[PZ] -= delta;
      mp_z_range(ch[i].cfg, S.w[i]);
    }
  }
}

// mpCheckError mp_fit.c:43-68 for group g.
__device__ inline void mp_check_error(const MPChan* ch, const MPParams& p, int f, int g, char* wsbase, int lane) {
  bool bad = false;
  for (int c = 0; c < p.nc; c++) bad |= (ch[c].fs.pk[ch[c].fs.pk_off[f] + g].status == ERROR);
  if (!bad) return;
  for (int c = 0; c < p.nc; c++) {
    PeakRec* q = ch[c].fs.pk + ch[c].fs.pk_off[f] + g;
    PeakRec r;
    load_rec(q, r);
    if (r.status != ERROR) {
      WarpWS<double> wc = warp_ws<double>(wsbase, ch[c].cfg, 0);
      mp_add(ch[c], mp_fbase(ch[c], f), r, wc, -1, lane);
      r.added -= 1;
    }
    r.status = ERROR;
    __syncwarp();
    if (lane == 0) *q = r;
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// The sweep, several groups at once.
//
// A frame's groups are taken in index order in batches of at most MP_TEAMS:
// a batch is a run of consecutive RUNNING groups whose ROIs, grown by
// MP_DIL pixels on every side, overlap in no plane.  Every group of a batch
// takes its step at once, one team of warps (a warp per plane) each, on
// its own copy of its ROIs' state: nothing is written to the planes'
// images or records until the batch commits.  A step that moves a ROI more
// than MP_DIL pixels from where it started "escapes" and stops.  The batch
// then commits the steps of its groups below the lowest escaped one (their
// regions are disjoint, so committing them together is what committing
// them one after another gives), drops the others, runs the escaped group
// alone on the committed state (unbounded) and commits it; the next batch
// starts after it.  So every group's step sees the state the reference's
// index-order sweep gives it, and the results are that sweep's.
// ---------------------------------------------------------------------------


__device__ __forceinline__ void team_sync(int team, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(team + 1), "r"(nthreads) : "memory");
}

// The base state of a ROI anchored at (ax, ay) without the peak's start
// contribution (rec0 anchored at its start, shape grid psfo[roi][roi]):
// the fit image and background less that contribution where the start ROI
// covers the pixel, rqe, data, and the count with the trial peak.
__device__ inline void mp_base_excl(const MPChan& c, long long fbase, int ax, int ay, const PeakRec& rec0,
                                    const double* psfo, WarpWS<double>& ws, int lane) {
  const ModelCfg& cfg = c.cfg;
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(ws.roi, p, rx, ry);
    const long long kk = pix_index(cfg, ax, ay, rx, ry);
    Q2 Fq = acc_load<2>(c.fs.f, fbase + kk);
    Q2 Bq = acc_load<2>(c.fs.bg, fbase + kk);
    int Cg = __ldcg(c.fs.cnt + fbase + kk);
    const double rq = __ldg(c.fs.rqe + kk), sc = __ldg(c.fs.scmos + kk);
    const int ox = ax + rx - rec0.xi, oy = ay + ry - rec0.yi;
    if (in_roi(ox, oy, cfg.roi)) {
      Fq = q_sub(Fq, quant_t<double>(contrib_f(rec0.p[PH], psfo[oy * cfg.roi + ox], rq)));
      Bq = q_sub(Bq, quant_t<double>(contrib_bg(rec0.p[PBG], rq, sc)));
      Cg -= 1;
    }
    ws.Fb[p] = acc_value<2>(Fq);
    ws.Bs[p] = acc_value<2>(Bq) + sc;
    ws.R[p] = rq;
    ws.X[p] = __ldg(c.fs.x + fbase + kk);
    ws.IC[p] = ic_store<double>(Cg + 1);
  }
  __syncwarp();
}

// One group's coupled LM step (mpIterateLM mp_fit.c:199-466) by one team:
// warp c of the team does plane c.  Nothing is written outside shared
// memory: the final records are in T.S.w, the final shape in ws.psf and the
// start shape in psfo (per plane).  Returns (on every thread of the team)
// 1 if a bounded step escaped.
__device__ inline int mp_team_step(const MPChan* ch, const MPParams& p, int f, int g, MPTeam& T,
                                   WarpWS<double>& wc, double* psfo, int c, int lane, int team, int nthr,
                                   bool bounded) {
  const int nc = p.nc;
  const bool lead = (c == 0 && lane == 0);
  MPShared& S = T.S;
  MPCtl& K = T.K;
  const MPChan& C = ch[c];
  const long long fb = mp_fbase(C, f);
  if (lane == 0)
    for (int i = 0; i < NCOUNTERS; i++) K.ctr[c][i] = 0;
  {
    PeakRec r;
    load_rec(C.fs.pk + C.fs.pk_off[f] + g, r);
    double dev;
    const bool fail = mp_error(C, fb, r, dev, lane);
    if (lane == 0) S.orig[c] = r;   // the stored peak (mpResetWorkingPeaks restores it)
    if (!fail) r.error = dev;       // the return value is ignored (mp_fit.c:220)
    else if (lane == 0) K.ctr[c][C_NEGFI]++;
    if (lane == 0) {
      S.orig_e[c] = r.error;
      r.added -= 1;
      S.w[c] = r;
    }
    const SplinePos sp = mp_jh(C, fb, r, wc, S.jh[c], lane);
    // the start shape on a roi x roi grid (for the exclusions and the commit)
    for (int q = lane; q < C.cfg.roi * C.cfg.roi; q += 32) psfo[q] = 0.0;
    __syncwarp();
    for (int q = lane; q < C.cfg.nroi; q += 32) {
      int rx, ry;
      roi_rc(wc.roi, q, rx, ry);
      psfo[ry * C.cfg.roi + rx] = psf_at(C.cfg, C.fs.aij, wc, sp, rx, ry);
    }
    __syncwarp();
    mp_base_excl(C, fb, r.xi, r.yi, r, psfo, wc, lane);
  }
  int cax = S.orig[c].xi, cay = S.orig[c].yi;
  const int x0 = S.orig[c].xi, y0 = S.orig[c].yi;
  for (;;) {
    team_sync(team, nthr);
    if (lead) {
      K.act = MPA_EVAL;
      if (S.w[0].lambda > LAMBDA_MAX) {
        for (int i = 0; i < nc; i++) {
          K.ctr[i][C_LOST]++;
          S.w[i].status = ERROR;
        }
        K.act = MPA_BREAK;
      } else {
        for (int i = 0; i < nc; i++) S.w[i].status = RUNNING;
      }
    }
    team_sync(team, nthr);
    if (K.act == MPA_BREAK) return 0;
    {
      double dl[MAX_JAC];
      const int info = solve_fp64_warp(S.jh[c], C.cfg.jac, S.w[c].lambda, dl, lane);
      if (lane == 0) {
        K.fail[c] = info;
        for (int m = 0; m < C.cfg.jac; m++) S.dl[c][m] = dl[m];
      }
    }
    team_sync(team, nthr);
    if (lead) {
      bool bad = false;
      for (int i = 0; i < nc; i++) {
        S.w[i].iterations++;
        K.ctr[i][C_ITER]++;
        if (K.fail[i] != 0) {
          K.ctr[i][C_DPOSV]++;
          bad = true;
          break;
        }
      }
      if (bad) {
        for (int i = 0; i < nc; i++) {
          S.w[i].status = ERROR;
          S.w[i].lambda = S.w[i].lambda * LAMBDA_UP;
        }
        K.act = MPA_CONTINUE;
      } else {
        mp_update_team(ch, p, S, K);
        for (int i = 0; i < nc; i++)
          if (mp_check_team(ch[i], S.w[i], K, i)) bad = true;
        if (bad) {
          for (int i = 0; i < nc; i++) {
            const int added = S.w[i].added;
            const double lam = S.w[i].lambda;
            S.w[i] = S.orig[i];
            S.w[i].added = added;
            S.w[i].lambda = lam * LAMBDA_UP;
            S.w[i].status = ERROR;
          }
          K.act = MPA_CONTINUE;
        }
      }
    }
    team_sync(team, nthr);
    if (K.act == MPA_CONTINUE) continue;
    // the trial: escape check, base at a moved ROI, error
    {
      const PeakRec r = S.w[c];
      const int esc = bounded && (abs(r.xi - x0) > MP_DIL || abs(r.yi - y0) > MP_DIL);
      if (lane == 0) K.fail[c] = esc;
    }
    team_sync(team, nthr);
    if (lead) {
      int e = 0;
      for (int i = 0; i < nc; i++) e |= K.fail[i];
      K.esc = e;
    }
    team_sync(team, nthr);
    if (K.esc) return 1;
    {
      const PeakRec r = S.w[c];
      if (r.xi != cax || r.yi != cay) {
        mp_base_excl(C, fb, r.xi, r.yi, S.orig[c], psfo, wc, lane);
        cax = r.xi;
        cay = r.yi;
      }
      double dev;
      const bool fail = mp_trial_error(C, r, wc, dev, lane);
      if (lane == 0) {
        S.w[c].added += 1;
        K.fail[c] = fail;
        K.e[c] = dev;
        if (fail) K.ctr[c][C_NEGFI]++;
        else S.w[c].error = dev;
      }
    }
    team_sync(team, nthr);
    if (lead) {
      double e0 = 0.0, e1 = 0.0;
      bool bad = false;
      for (int i = 0; i < nc; i++) {
        e0 += S.orig_e[i];
        if (K.fail[i]) bad = true;
        else e1 += K.e[i];
      }
      K.undo = 0;
      if (bad) {
        K.undo = 1;
        K.act = MPA_CONTINUE;
      } else if (e1 > e0) {
        if (((e1 - e0) / e0) < p.tol) {
          for (int i = 0; i < nc; i++) S.w[i].status = CONVERGED;
          K.act = MPA_BREAK;
        } else {
          for (int i = 0; i < nc; i++) K.ctr[i][C_NONDECR]++;
          K.undo = 1;
          K.act = MPA_CONTINUE;
        }
      } else {
        if (((e0 - e1) / e0) < p.tol) {
          for (int i = 0; i < nc; i++) S.w[i].status = CONVERGED;
        } else if (S.w[0].lambda > LAMBDA_MIN) {
          for (int i = 0; i < nc; i++) S.w[i].lambda = S.w[i].lambda * LAMBDA_DOWN;
        }
        K.act = MPA_BREAK;
      }
      if (K.undo) {
        // the trial was never added to the image: only the records go back
        for (int i = 0; i < nc; i++) {
          const int added = S.w[i].added - 1;
          const double lam = S.w[i].lambda;
          S.w[i] = S.orig[i];
          S.w[i].added = added;
          S.w[i].lambda = lam * LAMBDA_UP;
          S.w[i].status = ERROR;
        }
      }
    }
    team_sync(team, nthr);
    if (K.act == MPA_BREAK) return 0;
  }
}

// Commit a team's step (warp c, plane c): the start contribution out of the
// image, the accepted trial in (its shape in ws.psf), the record (with
// channel 0's status, mpCopyFromWorking mp_fit.c:124-134) and the counters.
__device__ inline void mp_commit(const MPChan& C, int f, int g, const MPTeam& T, const WarpWS<double>& wc,
                                 const double* psfo, int c, int lane) {
  const ModelCfg& cfg = C.cfg;
  const long long fb = mp_fbase(C, f);
  const PeakRec& r0 = T.S.orig[c];
  PeakRec r = T.S.w[c];
  r.status = T.S.w[0].status;
  for (int q = lane; q < cfg.nroi; q += 32) {
    int rx, ry;
    roi_rc(wc.roi, q, rx, ry);
    const long long kk = pix_index(cfg, r0.xi, r0.yi, rx, ry);
    const double rq = __ldg(C.fs.rqe + kk), sc = __ldg(C.fs.scmos + kk);
    acc_red<2>(C.fs.f, fb + kk, quant_t<double>(contrib_f(r0.p[PH], psfo[ry * cfg.roi + rx], rq)), -1);
    acc_red<2>(C.fs.bg, fb + kk, quant_t<double>(contrib_bg(r0.p[PBG], rq, sc)), -1);
    atomicAdd(C.fs.cnt + fb + kk, -1);
  }
  if (r.status != ERROR) {
    for (int q = lane; q < cfg.nroi; q += 32) {
      int rx, ry;
      roi_rc(wc.roi, q, rx, ry);
      const long long kk = pix_index(cfg, r.xi, r.yi, rx, ry);
      const double rq = wc.R[q], sc = __ldg(C.fs.scmos + kk);
      acc_red<2>(C.fs.f, fb + kk, quant_t<double>(contrib_f(r.p[PH], wc.psf[q], rq)), +1);
      acc_red<2>(C.fs.bg, fb + kk, quant_t<double>(contrib_bg(r.p[PBG], rq, sc)), +1);
      atomicAdd(C.fs.cnt + fb + kk, 1);
    }
  }
  __syncwarp();
  if (lane == 0) {
    C.fs.pk[C.fs.pk_off[f] + g] = r;
    for (int i = 0; i < NCOUNTERS; i++)
      if (T.K.ctr[c][i]) atomicAdd(reinterpret_cast<unsigned long long*>(&C.fs.ctl[f].ctr[i]),
                                   (unsigned long long)T.K.ctr[c][i]);
  }
}

// mpIterateLM mp_fit.c:183-478 for frame blockIdx.x (batches of groups as
// above; blockDim.x = 32 * nc * p.teams), then mFitRecenterPeaks per plane
// and mpCheckError per group.
__global__ void __launch_bounds__(32 * MP_MAXCH * 2) k_mp_sweep(const MPChan* chans, MPParams p) {
  extern __shared__ __align__(16) char smem[];
  const int nc = p.nc;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int team = warp / nc, c = warp - team * nc;
  const int nthr = 32 * nc;
  const int f = blockIdx.x;
  const size_t wstride = (size_t)p.ws_bytes + (((size_t)p.grid_doubles * 8 + 15) & ~(size_t)15);
  char* const ws_c = smem + (size_t)warp * wstride;
  double* const psfo = reinterpret_cast<double*>(ws_c + p.ws_bytes);
  size_t off = (size_t)nc * p.teams * wstride;
  MPTeam* teams = reinterpret_cast<MPTeam*>(smem + off);
  off += ((sizeof(MPTeam) * p.teams + 15) & ~(size_t)15);
  MPChan* ch = reinterpret_cast<MPChan*>(smem + off);
  off += ((sizeof(MPChan) * nc + 15) & ~(size_t)15);
  int* bgrp = reinterpret_cast<int*>(smem + off);           // the batch's groups
  int* bbox = bgrp + MP_TEAMS;                               // their grown ROIs per plane: x0, y0, x1, y1
  int* sh = bbox + 4 * MP_TEAMS * MP_MAXCH;                  // nb, next, esc_min
  for (int i = threadIdx.x; i < (int)(nc * sizeof(MPChan) / 4); i += blockDim.x)
    reinterpret_cast<int*>(ch)[i] = reinterpret_cast<const int*>(chans)[i];
  if (threadIdx.x < p.teams * MP_MAXCH) teams[threadIdx.x / MP_MAXCH].S.heights[threadIdx.x % MP_MAXCH] = 1.0;
  __syncthreads();
  const MPChan& C = ch[c];
  WarpWS<double> wc = warp_ws<double>(ws_c, C.cfg, C.cfg.nroi);
  wc.roi = C.fs.roi_xy;
  const int nfit = ch[0].fs.nfit[f];
  int base = 0;
  while (base < nfit) {
    if (threadIdx.x == 0) {
      // the batch: consecutive RUNNING groups, grown ROIs disjoint in every plane
      int nb = 0, g = base;
      while (nb < p.teams && g < nfit) {
        if (ch[0].fs.pk[ch[0].fs.pk_off[f] + g].status != RUNNING) {
          g++;
          continue;
        }
        bool clash = false;
        int box[MP_MAXCH][4];
        for (int i = 0; i < nc; i++) {
          const PeakRec* q = ch[i].fs.pk + ch[i].fs.pk_off[f] + g;
          const int xi = q->xi, yi = q->yi, roi = ch[i].cfg.roi;
          box[i][0] = xi - MP_DIL;
          box[i][1] = yi - MP_DIL;
          box[i][2] = xi + roi + MP_DIL;
          box[i][3] = yi + roi + MP_DIL;
          for (int m = 0; m < nb && !clash; m++) {
            const int* o = bbox + 4 * (m * MP_MAXCH + i);
            if (box[i][0] < o[2] && o[0] < box[i][2] && box[i][1] < o[3] && o[1] < box[i][3]) clash = true;
          }
        }
        if (clash) break;
        for (int i = 0; i < nc; i++)
          for (int k = 0; k < 4; k++) bbox[4 * (nb * MP_MAXCH + i) + k] = box[i][k];
        bgrp[nb++] = g++;
      }
      sh[0] = nb;
      sh[1] = g;
      sh[2] = INT_MAX;
    }
    __syncthreads();
    const int nb = sh[0];
    if (nb == 0) {
      base = sh[1];
      __syncthreads();
      continue;
    }
    // a lone group's step cannot meet another's: unbounded (no escape)
    int esc = 0;
    if (team < nb) {
      esc = mp_team_step(ch, p, f, bgrp[team], teams[team], wc, psfo, c, lane, team, nthr, nb > 1);
      if (esc && c == 0 && lane == 0) atomicMin(&sh[2], team);
    }
    __syncthreads();
    const int emin = sh[2];
    if (team < nb && team < emin) mp_commit(C, f, bgrp[team], teams[team], wc, psfo, c, lane);
    __syncthreads();
    if (emin < nb) {
      // the escaped group alone, on the committed state
      if (team == 0) {
        mp_team_step(ch, p, f, bgrp[emin], teams[0], wc, psfo, c, lane, 0, nthr, false);
        mp_commit(C, f, bgrp[emin], teams[0], wc, psfo, c, lane);
      }
      base = bgrp[emin] + 1;
    } else {
      base = sh[1];
    }
    __syncthreads();
  }
  // mFitRecenterPeaks multi_fit.c:1644-1690: team 0, a warp per plane
  if (team == 0) {
    const long long fb = mp_fbase(C, f);
    for (int g = 0; g < nfit; g++) {
      PeakRec* q = C.fs.pk + C.fs.pk_off[f] + g;
      PeakRec r;
      load_rec(q, r);
      if (r.status != RUNNING) continue;
      const double dx = r.p[PX] - r.xi, dy = r.p[PY] - r.yi;
      if (!((dx < -0.25) || (dx > 1.25) || (dy < -0.25) || (dy > 1.25))) continue;
      mp_add(C, fb, r, wc, -1, lane);
      r.added -= 1;
      r.xi = (int)floor(r.p[PX]);
      r.yi = (int)floor(r.p[PY]);
      const int chk = base_check(C.cfg, r);
      if (chk) {
        if (lane == 0) {
          C.fs.ctl[f].ctr[C_LOST]++;
          C.fs.ctl[f].ctr[chk == 1 ? C_MARGIN : C_NEGH]++;
        }
        r.status = ERROR;
      } else {
        mp_add(C, fb, r, wc, +1, lane);
        r.added += 1;
      }
      __syncwarp();
      if (lane == 0) *q = r;
      __syncwarp();
    }
  }
  __syncthreads();
  // mpCheckError mp_fit.c:43-68 for every group: team 0, a warp per plane
  for (int g = 0; g < nfit; g++) {
    if (threadIdx.x == 0) {
      bool bad = false;
      for (int i = 0; i < nc; i++) bad |= (ch[i].fs.pk[ch[i].fs.pk_off[f] + g].status == ERROR);
      sh[0] = bad;
    }
    __syncthreads();
    if (sh[0] && team == 0) {
      PeakRec* q = C.fs.pk + C.fs.pk_off[f] + g;
      PeakRec r;
      load_rec(q, r);
      if (r.status != ERROR) {
        mp_add(C, mp_fbase(C, f), r, wc, -1, lane);
        r.added -= 1;
      }
      r.status = ERROR;
      __syncwarp();
      if (lane == 0) *q = r;
    }
    __syncthreads();
  }
  if (p.unconv && warp == 0) {
    int n = 0;
    for (int g = lane; g < nfit; g += 32) n += (ch[0].fs.pk[ch[0].fs.pk_off[f] + g].status == RUNNING);
    n = warp_sum_int(n);
    if (lane == 0) p.unconv[f] = n;
  }
}

// After the channels' own new-peak passes (mpArbNewPeaks mp_fit_arb.c:180-340,
// mpDaoNewPeaks mp_fit_dao.c:82-152): with fixed heights the new "finder" /
// "testing" groups take their channels' mean height (their peaks subtracted,
// re-added at that height and their error recomputed), then every new group
// with an ERROR peak is made ERROR in all channels (mpCheckError).
__global__ void __launch_bounds__(32) k_mp_newpeaks(const MPChan* chans, MPParams p) {
  extern __shared__ __align__(16) char smem[];
  const int lane = threadIdx.x;
  const int f = blockIdx.x;
  MPChan* ch = reinterpret_cast<MPChan*>(smem + p.ws_bytes + ((sizeof(MPShared) + 15) & ~(size_t)15));
  for (int i = lane; i < (int)(p.nc * sizeof(MPChan) / 4); i += 32)
    reinterpret_cast<int*>(ch)[i] = reinterpret_cast<const int*>(chans)[i];
  __syncwarp();
  const int nc = p.nc;
  const int stop = p.stop < 0 ? ch[0].fs.nfit[f] : p.stop;
  for (int g = p.start; g < stop; g++) {
    if (p.fix_heights) {
      double height = 0.0;
      for (int c = 0; c < nc; c++) height += ch[c].fs.pk[ch[c].fs.pk_off[f] + g].p[PH];
      height = height / ((double)nc);
      for (int c = 0; c < nc; c++) {
        PeakRec* q = ch[c].fs.pk + ch[c].fs.pk_off[f] + g;
        PeakRec r;
        load_rec(q, r);
        const long long fb = mp_fbase(ch[c], f);
        WarpWS<double> wc = warp_ws<double>(smem, ch[c].cfg, 0);
        if (r.status != ERROR) mp_add(ch[c], fb, r, wc, -1, lane);
        r.p[PH] = height;
        if (r.status != ERROR) {
          mp_add(ch[c], fb, r, wc, +1, lane);
          if (r.status == RUNNING) {
            double dev;
            if (mp_error(ch[c], fb, r, dev, lane)) {
              if (lane == 0) ch[c].fs.ctl[f].ctr[C_NEGFI]++;
            } else {
              r.error = dev;
            }
          }
        }
        __syncwarp();
        if (lane == 0) *q = r;
        __syncwarp();
      }
    }
  }
  for (int g = p.start; g < stop; g++) mp_check_error(ch, p, f, g, smem, lane);
}

}  // namespace sa
