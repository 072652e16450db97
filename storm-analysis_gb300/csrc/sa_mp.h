// sa_mp.h -- host-side launchers of the multi-plane kernels (sa_mp.cu).
#pragma once

#include <cuda_runtime.h>
#include "sa_mp_types.h"

namespace sa {

// A channel's workspace bytes in a multi-plane CTA.
int mp_ws_bytes(const ModelCfg& cfg);
// Dynamic shared memory of a multi-plane CTA.
size_t mp_smem(const MPParams& p);
// mpIterateLM on frames 0 .. frames-1 (one warp each); d_chans: p.nc
// channel descriptors on the device.
cudaError_t mp_sweep(const MPChan* d_chans, const MPParams& p, int frames, cudaStream_t s);
// The new groups [p.start, p.stop) after the channels' own new-peak passes.
cudaError_t mp_newpeaks(const MPChan* d_chans, const MPParams& p, int frames, cudaStream_t s);

}  // namespace sa
