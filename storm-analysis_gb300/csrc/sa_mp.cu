// sa_mp.cu -- launchers of the multi-plane kernels (sa_mp.cuh).
#include "sa_mp.cuh"
#include "sa_mp.h"

namespace sa {

int mp_ws_bytes(const ModelCfg& cfg) { return (int)warp_ws_bytes<double>(cfg, 0); }

size_t mp_smem(const MPParams& p) {
  return (size_t)p.ws_bytes + ((sizeof(MPShared) + 15) & ~(size_t)15) + (size_t)p.nc * sizeof(MPChan);
}

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
  done = true;
  return cudaSuccess;
}

cudaError_t mp_sweep(const MPChan* d_chans, const MPParams& p, int frames, cudaStream_t s) {
  cudaError_t e = mp_limits();
  if (e != cudaSuccess) return e;
  k_mp_sweep<<<frames, 32, mp_smem(p), s>>>(d_chans, p);
  return cudaGetLastError();
}

cudaError_t mp_newpeaks(const MPChan* d_chans, const MPParams& p, int frames, cudaStream_t s) {
  cudaError_t e = mp_limits();
  if (e != cudaSuccess) return e;
  k_mp_newpeaks<<<frames, 32, mp_smem(p), s>>>(d_chans, p);
  return cudaGetLastError();
}

}  // namespace sa
