// sa_mp.cu -- launchers of the multi-plane kernels (sa_mp.cuh).
#include "sa_mp.cuh"
#include "sa_mp.h"

namespace sa {

int mp_ws_bytes(const ModelCfg& cfg) { return (int)warp_ws_bytes<double>(cfg, cfg.nroi); }

static size_t al16(size_t b) { return (b + 15) & ~(size_t)15; }

// k_mp_sweep: per warp a workspace and a shape grid, per team its coupling
// state, the channels, the batch table.
static size_t mp_smem_sweep(const MPParams& p) {
  const size_t wstride = (size_t)p.ws_bytes + al16((size_t)p.grid_doubles * 8);
  return (size_t)p.nc * p.teams * wstride + al16(sizeof(MPTeam) * p.teams) + al16(sizeof(MPChan) * p.nc) +
         sizeof(int) * (MP_TEAMS + 4 * MP_TEAMS * MP_MAXCH + 4);
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
  // as many teams as fit (a workspace per plane each); none: too many planes
  // of a large PSF
  MPParams q = p;
  q.teams = MP_TEAMS;
  while (q.teams > 1 && (mp_smem_sweep(q) > (size_t)g_max_smem || 32 * q.nc * q.teams > 32 * MP_MAXCH * 2)) q.teams--;
  if (mp_smem_sweep(q) > (size_t)g_max_smem) return cudaErrorInvalidConfiguration;
  k_mp_sweep<<<frames, 32 * q.nc * q.teams, mp_smem_sweep(q), s>>>(d_chans, q);
  return cudaGetLastError();
}

cudaError_t mp_newpeaks(const MPChan* d_chans, const MPParams& p, int frames, cudaStream_t s) {
  cudaError_t e = mp_limits();
  if (e != cudaSuccess) return e;
  k_mp_newpeaks<<<frames, 32, mp_smem(p), s>>>(d_chans, p);
  return cudaGetLastError();
}

}  // namespace sa
