// sa_launch_impl.cuh -- definitions of the launchers; included once per
// pixel type by sa_launch_f32.cu / sa_launch_f64.cu.
#pragma once

#include "sa_kernels.cuh"
#include "sa_launch.h"

namespace sa {

constexpr int SWEEP_BLOCK = 128;    // 4 warps, one peak each (fewer where their workspaces do not fit)
constexpr int CTA_BLOCK = 1024;     // per-frame kernels
constexpr int AUX_BLOCK = 256;      // warp-per-peak auxiliary kernels without a workspace

// Threads of a warp-per-peak auxiliary CTA with a workspace per warp.
static inline int aux_block(const ModelCfg& cfg) { return 32 * aux_warps(cfg); }

// Shared bytes of the sweep CTA's ROI pixel table (after the workspaces).
static inline size_t roi_table_bytes(int nroi) { return ((size_t)nroi * 2 + 15) & ~(size_t)15; }

// Warps of a sweep CTA whose dynamic shared memory is smem (configure
// chooses 4, 3, 2 or 1 so that their workspaces fit).
template <typename T>
static inline int sweep_warps(const ModelCfg& cfg, size_t smem) {
  const size_t ws = warp_ws_bytes<T>(cfg, cfg.nroi);
  const size_t w = (smem - roi_table_bytes(cfg.nroi)) / ws;
  return w >= 4 ? 4 : (w >= 1 ? (int)w : 1);
}

// The sweep kernel of a configuration: the FP32 Gaussian models have one
// instantiation each, everything else shares the generic step.
template <typename T>
void (*sweep_kernel(const ModelCfg& cfg))(ModelCfg, FrameSet<T>) {
  if constexpr (sizeof(T) == 4) {
    if (gauss32<T>(cfg)) {
      switch (cfg.model) {
        case M_2DFIXED: return k_sweep<T, M_2DFIXED>;
        case M_2D: return k_sweep<T, M_2D>;
        case M_3D: return k_sweep<T, M_3D>;
        default: return k_sweep<T, M_Z>;
      }
    }
  }
  return k_sweep<T, -1>;
}

template <typename T>
void (*tail_kernel(const ModelCfg& cfg))(ModelCfg, FrameSet<T>, int) {
  if constexpr (sizeof(T) == 4) {
    if (gauss32<T>(cfg)) {
      switch (cfg.model) {
        case M_2DFIXED: return k_tail<T, M_2DFIXED>;
        case M_2D: return k_tail<T, M_2D>;
        case M_3D: return k_tail<T, M_3D>;
        default: return k_tail<T, M_Z>;
      }
    }
  }
  return k_tail<T, -1>;
}

template <typename T>
cudaError_t Launch<T>::configure(const ModelCfg& cfg, int* sweep_grid, size_t* sweep_smem,
                                 size_t* cta_smem, size_t* warp_smem) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int nsm = 0, max_smem = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t ws = warp_ws_bytes<T>(cfg, cfg.nroi);
  // four warps per sweep CTA, or as many as fit where their workspaces
  // (large ROIs in the FP64 engine, the pupil model) do not
  int wpc = SWEEP_BLOCK / 32;
  while (wpc > 1 && ws * wpc + roi_table_bytes(cfg.nroi) > (size_t)max_smem) wpc--;
  const size_t s_sweep = ws * wpc + roi_table_bytes(cfg.nroi);
  const size_t ws0 = warp_ws_bytes<T>(cfg, 0);
  const size_t grid_bytes = (size_t)(cfg.gx * cfg.gy + 1) * sizeof(int);
  const size_t s_cta_ws = ws0 * (size_t)cta_ws_warps(cfg);
  const size_t s_cta = s_cta_ws > grid_bytes ? s_cta_ws : grid_bytes;
  const size_t s_aux = ws0 * (size_t)aux_warps(cfg);
  if (s_sweep > (size_t)max_smem || s_cta > (size_t)max_smem || s_aux > (size_t)max_smem)
    return cudaErrorInvalidConfiguration;
  // The limit is a property of the kernel, shared by every handle of the
  // process (handles of different models and ROI sizes may run side by
  // side), so it is raised to the device maximum rather than to this
  // handle's need.
  auto raise_limit = [max_smem](const void* fn) {
    cudaFuncAttributes a;
    cudaError_t r = cudaFuncGetAttributes(&a, fn);
    if (r != cudaSuccess) return r;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                max_smem - (int)a.sharedSizeBytes);
  };
  e = raise_limit((const void*)sweep_kernel<T>(cfg));
  if (e != cudaSuccess) return e;
  e = raise_limit((const void*)k_prepare<T>);
  if (e != cudaSuccess) return e;
  e = raise_limit((const void*)k_post<T>);
  if (e != cudaSuccess) return e;
  e = raise_limit((const void*)tail_kernel<T>(cfg));
  if (e != cudaSuccess) return e;
  // the warp-per-peak auxiliary kernels (their workspace is above the
  // default 48 KB for the FFT PSF model)
  for (const void* fn : {(const void*)k_newpeaks<T>, (const void*)k_newpeaks_finder<T>, (const void*)k_peak_props<T>,
                         (const void*)k_set_status<T>}) {
    e = raise_limit(fn);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_kernel<T>(cfg), 32 * wpc, s_sweep);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  *sweep_grid = nsm * per_sm;
  *sweep_smem = s_sweep;
  *cta_smem = s_cta;
  *warp_smem = s_aux;
  return cudaSuccess;
}

template <typename T>
cudaError_t Launch<T>::prepare(const ModelCfg& cfg, const FrameSet<T>& fs, size_t smem, cudaStream_t s) {
  k_prepare<T><<<fs.F, CTA_BLOCK, smem, s>>>(cfg, fs);
  return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::sweep(const ModelCfg& cfg, const FrameSet<T>& fs, int grid, size_t smem,
                             cudaStream_t s) {
  sweep_kernel<T>(cfg)<<<grid, 32 * sweep_warps<T>(cfg, smem), smem, s>>>(cfg, fs);
  return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::post(const ModelCfg& cfg, const FrameSet<T>& fs, size_t smem, cudaStream_t s) {
  k_post<T><<<fs.F, CTA_BLOCK, smem, s>>>(cfg, fs);
  return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::tail(const ModelCfg& cfg, const FrameSet<T>& fs, int tail_peaks, cudaStream_t s) {
  const size_t smem = warp_ws_bytes<T>(cfg, cfg.nroi) + roi_table_bytes(cfg.nroi);
  tail_kernel<T>(cfg)<<<fs.F, 32, smem, s>>>(cfg, fs, tail_peaks);
  return cudaGetLastError();
}

static inline int grid_for(long long n, int block) {
  long long g = (n + block - 1) / block;
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  return (int)g;
}

template <typename T>
cudaError_t Launch<T>::new_image(const FrameSet<T>& fs, const void* img, int bits, int frame0,
                                 int nframes, cudaStream_t s) {
  const int g = grid_for(fs.npix * nframes, 256);
  if (bits == 32) k_new_image<T, float><<<g, 256, 0, s>>>(fs, (const float*)img, frame0, nframes);
  else if (bits == 16) k_new_image<T, unsigned short><<<g, 256, 0, s>>>(fs, (const unsigned short*)img, frame0, nframes);
  else k_new_image<T, double><<<g, 256, 0, s>>>(fs, (const double*)img, frame0, nframes);
  return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::new_background(const FrameSet<T>& fs, const void* bg, int bits, int frame0,
                                      int nframes, cudaStream_t s) {
  const int g = grid_for(fs.npix * nframes, 256);
  if (bits == 32) k_new_background<T, float><<<g, 256, 0, s>>>(fs, (const float*)bg, frame0, nframes);
  else k_new_background<T, double><<<g, 256, 0, s>>>(fs, (const double*)bg, frame0, nframes);
  return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::new_peaks(const ModelCfg& cfg, const FrameSet<T>& fs, const double* rows,
                                 int ncol, int ptype, const int* slots, const int* frames, int n,
                                 int do_add, size_t warp_smem, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int g = grid_for((long long)n * 32, aux_block(cfg));
  k_newpeaks<T><<<g, aux_block(cfg), warp_smem, s>>>(cfg, fs, rows, ncol, ptype, slots, frames, n, do_add);
  return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::new_peaks_finder(const ModelCfg& cfg, const FrameSet<T>& fs, const int* slots,
                                        const int* frame_first, const int* frame_n, int nframes,
                                        size_t warp_smem, cudaStream_t s) {
  const int g = (nframes * 32 + aux_block(cfg) - 1) / aux_block(cfg);
  k_newpeaks_finder<T><<<g, aux_block(cfg), warp_smem, s>>>(cfg, fs, slots, frame_first, frame_n, nframes);
  return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::peak_error(const ModelCfg& cfg, const FrameSet<T>& fs, const int* slots,
                                  const int* frames, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int g = grid_for((long long)n * 32, AUX_BLOCK);
  k_peak_error<T><<<g, AUX_BLOCK, 0, s>>>(cfg, fs, slots, frames, n);
  return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::peak_props(const ModelCfg& cfg, const FrameSet<T>& fs, const int* slots,
                                  const int* frames, int n, double* sum, double* fg, double* bg,
                                  double* jac, size_t warp_smem, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int g = grid_for((long long)n * 32, aux_block(cfg));
  k_peak_props<T><<<g, aux_block(cfg), warp_smem, s>>>(cfg, fs, slots, frames, n, sum, fg, bg, jac);
  return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::set_status(const ModelCfg& cfg, const FrameSet<T>& fs, const int* slots,
                                  const int* frames, const int* status, int n, size_t warp_smem,
                                  cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int g = grid_for((long long)n * 32, aux_block(cfg));
  k_set_status<T><<<g, aux_block(cfg), warp_smem, s>>>(cfg, fs, slots, frames, status, n);
  return cudaGetLastError();
}

template <typename T>
cudaError_t Launch<T>::fit_image(const FrameSet<T>& fs, int frame, double* out, int residual,
                                 cudaStream_t s) {
  const int g = grid_for(fs.npix, 256);
  k_fit_image<T><<<g, 256, 0, s>>>(fs, frame, out, residual);
  return cudaGetLastError();
}

}  // namespace sa
