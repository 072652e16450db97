// sa_solve.cu -- the engine's damped normal-equation solvers over a batch
// of systems (saSolveDamped): the same device functions the LM step calls,
// one warp per system, so that they can be checked against LAPACK dposv.
#include "sa_kernels.cuh"
#include "sa_launch.h"

namespace sa {

namespace {

// Workspace of one warp: room for either solver's view of the normal
// equations (36 doubles, or 72 floats of float-float hi / lo words), and the
// shared scratch of the FP32 Gaussian solver's FP64 fallback (which the LM
// step lends from its trial tables).
struct SolveWS {
  double jh[36];
  double scr[MAX_JAC * MAX_JAC + 2 * MAX_JAC];
};

// The FP32 Gaussian solver returns component j on lane j: gather it into
// out on lane 0.
template <int K>
__device__ int solve_g32_k(WarpWS<float>& ws, double lam, double* out, int lane) {
  double dl;
  const int st = solve_g32<K>(ws, lam, dl, lane);
#pragma unroll
  for (int j = 0; j < K; j++) {
    const double v = __shfl_sync(0xffffffffu, dl, j);
    if (lane == 0) out[j] = v;
  }
  return st;
}

// engine 0: FP64 Cholesky (the FP64 engine and the fallback of both FP32
// solvers); 1: the FP32 Gaussian step's per-lane LDL^T with two float-float
// refinements, given the Hessian rounded to FP32 as that step keeps it;
// 2: the FP32 spline step's Jacobi-scaled LU with FP64 refinements.
__global__ void k_solve_batch(const double* a, const double* b, int n_sys, int k, double lam, int engine,
                              double* x, int* info) {
  __shared__ SolveWS sws[4];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int sys = blockIdx.x * 4 + wib;
  if (sys >= n_sys) return;
  SolveWS& w = sws[wib];
  const double* A = a + (size_t)sys * k * k;
  const double* B = b + (size_t)sys * k;
  if (lane == 0) {
    if (engine == 1) {
      float* jf = reinterpret_cast<float*>(w.jh);
      for (int i = 0; i < 72; i++) jf[i] = 0.0f;
      for (int l = 0; l < k; l++) {
        const ff g = ff_from_double(B[l]);
        jf[l] = g.h;
        jf[36 + l] = g.l;
        for (int m = l; m < k; m++) jf[hes_index(k, l, m)] = (float)A[l * k + m];
      }
    } else {
      for (int l = 0; l < k; l++) {
        w.jh[l] = B[l];
        for (int m = l; m < k; m++) w.jh[hes_index(k, l, m)] = A[l * k + m];
      }
    }
  }
  __syncwarp();
  double out[MAX_JAC];
  for (int i = 0; i < MAX_JAC; i++) out[i] = 0.0;
  int st = 0;
  if (engine == 0) {
    if (lane == 0) st = solve_fp64_lane0(w.jh, k, lam, out);
  } else if (engine == 1) {
    WarpWS<float> ws{};
    ws.jh = w.jh;
    ws.tab1 = reinterpret_cast<float*>(w.scr);
    switch (k) {
      case 4: st = solve_g32_k<4>(ws, lam, out, lane); break;
      case 5: st = solve_g32_k<5>(ws, lam, out, lane); break;
      default: st = solve_g32_k<6>(ws, lam, out, lane); break;
    }
  } else {
    WarpWS<float> ws{};
    ws.jh = w.jh;
    st = solve_damped<float>(ws, k, lam, out, lane);
  }
  if (lane == 0) {
    info[sys] = st;
    for (int l = 0; l < k; l++) x[(size_t)sys * k + l] = out[l];
  }
}

}  // namespace

cudaError_t solve_batch(const double* a, const double* b, int n_sys, int k, double lam, int engine,
                        double* x, int* info, cudaStream_t s) {
  if (n_sys <= 0) return cudaSuccess;
  k_solve_batch<<<(n_sys + 3) / 4, 128, 0, s>>>(a, b, n_sys, k, lam, engine, x, info);
  return cudaGetLastError();
}

}  // namespace sa
