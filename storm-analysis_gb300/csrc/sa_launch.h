// sa_launch.h -- host-side launchers of the engine kernels, one explicit
// instantiation per pixel type (sa_launch_f32.cu, sa_launch_f64.cu).
#pragma once

#include <cuda_runtime.h>
#include "sa_common.cuh"

namespace sa {

// Print msg and keep it for saGetLastError (defined in sa_api.cu).
void record_error(const char* msg);

// The engine's damped solves (H + lam diag H) x = b on n_sys systems of
// size k (a: n_sys row-major k x k matrices, upper triangle read; b, x:
// n_sys x k; info: 0 or the solver's failure code).  engine 0: FP64
// Cholesky; 1: FP32 Gaussian step solver (k 4-6); 2: FP32 spline step
// solver.  Device pointers (sa_solve.cu).
cudaError_t solve_batch(const double* a, const double* b, int n_sys, int k, double lam, int engine,
                        double* x, int* info, cudaStream_t s);

template <typename T>
struct Launch {
  // Set shared-memory limits of the kernels; returns the sweep CTA count
  // that keeps every SM busy (persistent grid).
  static cudaError_t configure(const ModelCfg& cfg, int* sweep_grid, size_t* sweep_smem,
                               size_t* cta_smem, size_t* warp_smem);
  static cudaError_t prepare(const ModelCfg& cfg, const FrameSet<T>& fs, size_t smem, cudaStream_t s);
  static cudaError_t sweep(const ModelCfg& cfg, const FrameSet<T>& fs, int grid,
                           size_t smem, cudaStream_t s);
  static cudaError_t post(const ModelCfg& cfg, const FrameSet<T>& fs, size_t smem, cudaStream_t s);
  // The remaining sweeps of every frame with at most tail_peaks RUNNING
  // peaks left, one warp per frame, in one launch (k_tail).
  static cudaError_t tail(const ModelCfg& cfg, const FrameSet<T>& fs, int tail_peaks, cudaStream_t s);
  static cudaError_t new_image(const FrameSet<T>& fs, const void* img, int bits, int frame0,
                               int nframes, cudaStream_t s);
  static cudaError_t new_background(const FrameSet<T>& fs, const void* bg, int bits, int frame0,
                                    int nframes, cudaStream_t s);
  static cudaError_t new_peaks(const ModelCfg& cfg, const FrameSet<T>& fs, const double* rows,
                               int ncol, int ptype, const int* slots, const int* frames, int n,
                               int do_add, size_t warp_smem, cudaStream_t s);
  static cudaError_t new_peaks_finder(const ModelCfg& cfg, const FrameSet<T>& fs, const int* slots,
                                      const int* frame_first, const int* frame_n, int nframes,
                                      size_t warp_smem, cudaStream_t s);
  static cudaError_t peak_error(const ModelCfg& cfg, const FrameSet<T>& fs, const int* slots,
                                const int* frames, int n, cudaStream_t s);
  static cudaError_t peak_props(const ModelCfg& cfg, const FrameSet<T>& fs, const int* slots,
                                const int* frames, int n, double* sum, double* fg, double* bg,
                                double* jac, size_t warp_smem, cudaStream_t s);
  static cudaError_t set_status(const ModelCfg& cfg, const FrameSet<T>& fs, const int* slots,
                                const int* frames, const int* status, int n, size_t warp_smem,
                                cudaStream_t s);
  static cudaError_t fit_image(const FrameSet<T>& fs, int frame, double* out, int residual,
                               cudaStream_t s);
};

}  // namespace sa
