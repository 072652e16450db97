// sa_mp.cu -- launchers of the multi-plane kernels (sa_mp.cuh).
#include <algorithm>

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
  // Teams (groups stepping at once) per frame: the caller's number, else
  // enough for about MP_TEAMS teams per SM over all frames, at least 2 -- a
  // lone frame gets MP_TEAMS, a batch of 4 x SMs frames or more 2 each (the
  // SMs then fill with frames, with fewer of the teams' barriers and
  // escapes; on 512 and 1,024 two-plane 256 x 256 frames of 200 emitters, 2
  // or 3 teams fitted 15-30 % faster than 8, and 1 team 10 % slower than 2);
  // then as many as fit (a workspace per plane each); none: too many planes
  // of a large PSF
  MPParams q = p;
  if (p.teams > 0) {
    q.teams = std::min(p.teams, MP_TEAMS);
  } else {
    int dev = 0, sms = 1;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = ((long long)MP_TEAMS * sms + frames - 1) / std::max(frames, 1);
    q.teams = (int)std::max(2LL, std::min((long long)MP_TEAMS, want));
  }
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
