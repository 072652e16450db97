// sa_mp_types.h -- the multi-plane kernels' parameter blocks (sa_mp.cuh),
// shared with the host code that fills them.
#pragma once

#include "sa_common.cuh"

namespace sa {

constexpr int MP_MAXCH = 8;
constexpr int MP_TEAMS = 8;   // groups of a frame stepping at once (a batch) at most
enum { MP_ARB = 0, MP_DAO = 1 };

// One channel: its engine's model and frame set.
struct MPChan {
  ModelCfg cfg;
  FrameSet<double> fs;
};

struct MPParams {
  int nc, indep, kind, n_weights;
  double tol, w_z_offset, w_z_scale;
  double xt0N[3 * MP_MAXCH], yt0N[3 * MP_MAXCH], xtN0[3 * MP_MAXCH], ytN0[3 * MP_MAXCH];
  const double* w;   // weights bg, h, x, y, z: 5 x [n_weights][nc] (z the slow index)
  int ws_bytes;      // a channel workspace (the largest of the channels')
  int start, stop;   // k_mp_newpeaks: the new groups (stop < 0: to the frame's last)
  int fix_heights;   // k_mp_newpeaks: give the new groups their channels' mean height
  int* unconv;       // k_mp_sweep: RUNNING groups per frame after the sweep (may be null)
  int teams;         // k_mp_sweep: groups of a frame stepped at once (1 .. 8)
  int grid_doubles;  // k_mp_sweep: a plane's roi x roi shape grid (the largest of the planes')
};

// Per-frame state in shared memory (lane 0 writes the records).
struct MPShared {
  PeakRec orig[MP_MAXCH];
  PeakRec w[MP_MAXCH];
  double jh[MP_MAXCH][36];   // gradient (k) and packed upper Hessian per channel
  double dl[MP_MAXCH][8];    // the channels' LM steps
  double heights[MP_MAXCH];
  double orig_e[MP_MAXCH];   // the planes' starting errors of the group
};

}  // namespace sa
