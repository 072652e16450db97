// sa_mp.cu -- launchers of the multi-plane kernels (sa_mp.cuh).
#include "sa_mp.cuh"
#include "sa_mp.h"

namespace sa {

int mp_ws_bytes(const ModelCfg& cfg) { return (int)warp_ws_bytes<double>(cfg, cfg.nroi); }

static size_t al16(size_t b) { return (b + 15) & ~(size_t)15; }

// k_mp_sweep: a workspace per plane's warp, the coupling state, the channels.
static size_t mp_smem_sweep(const MPParams& p) {
  return (size_t)p.nc * p.ws_bytes + al16(sizeof(MPShared)) + al16(sizeof(MPCtl)) + (size_t)p.nc * sizeof(MPChan);
}

// k_mp_newpeaks: one warp.
size_t mp_smem(const MPParams& p) { return (size_t)p.ws_bytes + al16(sizeof(MPShared)) + (size_t)p.nc * sizeof(MPChan); }

static int g_max_smem = 0;

static cudaError_t mp_limits() {
  static bool done = false;
  if (done) return cudaSuccess;
  int dev = 0, max_smem = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  for (const void* fn : {(const void*)k_mp_sweep, (const void*)k_mp_newpeaks}) {
    cudaFuncAttributes a;
    e = cudaFuncGetAttributes(&a, fn);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem - (int)a.sharedSizeBytes);
    if (e != cudaSuccess) return e;
  }
  g_max_smem = max_smem - 1024;
  done = true;
  return cudaSuccess;
}

cudaError_t mp_sweep(const MPChan* d_chans, const MPParams& p, int frames, cudaStream_t s) {
  cudaError_t e = mp_limits();
  if (e != cudaSuccess) return e;
  // a workspace per plane: too many planes of a large PSF do not fit
  if (mp_smem_sweep(p) > (size_t)g_max_smem) return cudaErrorInvalidConfiguration;
  k_mp_sweep<<<frames, 32 * p.nc, mp_smem_sweep(p), s>>>(d_chans, p);
  return cudaGetLastError();
}

cudaError_t mp_newpeaks(const MPChan* d_chans, const MPParams& p, int frames, cudaStream_t s) {
  cudaError_t e = mp_limits();
  if (e != cudaSuccess) return e;
  k_mp_newpeaks<<<frames, 32, mp_smem(p), s>>>(d_chans, p);
  return cudaGetLastError();
}

}  // namespace sa
