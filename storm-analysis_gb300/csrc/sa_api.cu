// sa_api.cu -- host side of libsa_cuda.so: handles, device memory, the
// device-driven sweep loop and the reference-named C ABI (include/sa_cuda.h).
#include <algorithm>
#include <climits>
#include <cstddef>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sa_launch.h"
#include "sa_psf_fft.h"
#include "sa_pupil_fn.h"
#include "sa_mp.h"
#include "sa_cuda.h"

using namespace sa;

namespace {

thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  fprintf(stderr, "libsa_cuda: %s\n", buf);
}

#define CK(call)                                                              \
  do {                                                                        \
    cudaError_t e__ = (call);                                                 \
    if (e__ != cudaSuccess) {                                                 \
      set_error("%s failed: %s", #call, cudaGetErrorString(e__));             \
      return -1;                                                              \
    }                                                                         \
  } while (0)

// Spline handle.  Its fields have the layout of the reference's splineData
// (spliner/cubic_spline.h:16-26): cfInitialize reads type, sizes and aij,
// so it accepts a spline made by this library's initSpline2D/3D or by the
// reference's libcubic_spline.  splineCleanup frees every array the struct
// points to, whichever library allocated it (both use malloc).
struct SplineH {
  int type;  // 0: 2D, 1: 3D (S2D / S3D)
  int xs, ys, zs;
  double* aij;
  double* reserved[4];   // the reference's delta tables; unused here
};

template <typename P>
void dfree(P*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}

}  // namespace

// Device scratch of saGetFitImageNoAlloc: 8 MiB compiled into the library
// (one copy per device), enough for a 1024 x 1024 frame of doubles.  It is
// reached through cudaGetSymbolAddress, never allocated or freed.
constexpr size_t kNoAllocPixels = (size_t)1 << 20;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocPixels];

namespace {

// The scratch's device address on the current device, looked up once per
// device.  Handle creation (new_handle: daoInitialize / cfInitialize) makes
// this set-up call with the handle's device current; the lookup loads this
// file's device module on that device, so saGetFitImageNoAlloc itself only
// launches a kernel and copies.  Returns nullptr (the caller reports it)
// when there is no usable device.
double* noalloc_scratch() {
  static double* addr[64] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return nullptr;
    addr[dev] = static_cast<double*>(p);
  }
  return addr[dev];
}

struct Engine {
  ModelCfg cfg{};
  bool model_set = false;
  bool unsupported = false;
  int prec = 32;
  std::vector<double> rqe_h, scmos_h;
  std::vector<double> aij_h;
  std::vector<unsigned short> roi_xy;
  std::vector<int> roi_x, roi_y;
  SplineH* spline = nullptr;
  // saGetFitImageNoAlloc's scratch on the device current at creation
  double* noalloc = nullptr;

  // frames
  int F = 0;
  long long npix = 0;
  void* d_x = nullptr;
  long long* d_xq = nullptr;   // FP32: data in fixed point
  float2* d_xff = nullptr;     // FP32: the fixed-point data as float-float
  void* d_rqe = nullptr;
  void* d_scmos = nullptr;
  void* d_aij = nullptr;
  long long* d_f = nullptr;
  long long* d_bg = nullptr;
  int* d_cnt = nullptr;
  double* d_bgest = nullptr;
  FrameCtl* d_ctl = nullptr;
  int* d_cellstart = nullptr;
  unsigned* d_err = nullptr;
  int* d_epoch = nullptr;   // the sweep epoch, advanced on the device by k_post
  unsigned short* d_roi = nullptr;
  void* d_stage = nullptr;
  size_t stage_bytes = 0;

  // peaks
  int cap_total = 0;
  std::vector<int> pk_off, cap_f, nfit;
  PeakRec* d_pk = nullptr;
  PeakRec* d_snap = nullptr;
  int* d_pkoff = nullptr;
  int* d_nfit = nullptr;
  int* d_run = nullptr;
  unsigned* d_anchor = nullptr;
  int* d_done = nullptr;
  int2* d_cellitems = nullptr;
  int* d_stepctr = nullptr;

  // scheduling
  cudaStream_t stream = 0;
  cudaStream_t own_stream = nullptr;   // created for graph capture when no stream was set
  int sweep_grid = 0;
  int sweep_ctas_cap = 0;   // 0: the full persistent grid
  int tail_peaks = 8;       // k_tail for frames with at most this many RUNNING peaks (0: never)
  size_t sweep_smem = 0, cta_smem = 0, warp_smem = 0;
  bool configured = false;

  // host mirrors
  std::vector<PeakRec> host_pk;   // frame 0 records (valid when host_valid)
  bool host_valid = false;
  long long ctr_seen[NCOUNTERS] = {0};
  int unconv_cache = -1;

  // timing: a pool of event pairs around the sweep launches, read once at
  // saGetTiming so that timing adds no synchronisation
  bool timing = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> pool;
  size_t pool_used = 0;
  double sweep_ms = 0.0;
  std::vector<float> sweep_times;   // per sweep launch, ms
  long long sweep_launches = 0, ticks = 0;
  long long launches = 0;   // kernels launched by this handle

  // serving slots: frame control blocks copied back after each launched
  // burst of ticks (pinned, read once the event has completed)
  FrameCtl* h_ctl = nullptr;
  int h_ctl_n = 0;
  cudaEvent_t ev_poll = nullptr;

  ~Engine() {
    release();
    release_poll_buffers();
    if (own_stream) {
      cudaStreamSynchronize(own_stream);
      cudaStreamDestroy(own_stream);
    }
    if (h_ctl) cudaFreeHost(h_ctl);
    if (ev_poll) cudaEventDestroy(ev_poll);
  }

  void release_peaks() {
    dfree(d_pk); dfree(d_snap); dfree(d_pkoff); dfree(d_nfit); dfree(d_run); dfree(d_anchor);
    dfree(d_done); dfree(d_cellitems); dfree(d_stepctr);
    cap_total = 0;
  }
  void release() {
    release_peaks();
    dfree(d_x); dfree(d_xq); dfree(d_xff); dfree(d_rqe); dfree(d_scmos); dfree(d_aij); dfree(d_f); dfree(d_bg); dfree(d_cnt);
    dfree(d_bgest); dfree(d_ctl); dfree(d_cellstart); dfree(d_err); dfree(d_epoch); dfree(d_roi); dfree(d_stage);
    release_graphs();
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    ev0 = ev1 = nullptr;
    for (cudaEvent_t ev : pool) cudaEventDestroy(ev);
    pool.clear();
    pool_used = 0;
    F = 0;
  }

  size_t tsize() const { return prec == 32 ? sizeof(float) : sizeof(double); }

  template <typename T>
  FrameSet<T> fs() const {
    FrameSet<T> s{};   // zeroed padding: the burst graphs compare it bytewise
    s.F = F;
    s.npix = npix;
    s.x = (const T*)d_x;
    s.xq = d_xq;
    s.xff = d_xff;
    s.rqe = (const T*)d_rqe;
    s.scmos = (const T*)d_scmos;
    s.f = d_f;
    s.bg = d_bg;
    s.cnt = d_cnt;
    s.bgest = d_bgest;
    s.aij = (const T*)d_aij;
    s.pk = d_pk;
    s.snap = d_snap;
    s.pk_off = d_pkoff;
    s.nfit = d_nfit;
    s.run = d_run;
    s.anchor0 = d_anchor;
    s.done = d_done;
    s.epoch = d_epoch;
    s.cell_start = d_cellstart;
    s.cell_items = d_cellitems;
    s.stepctr = d_stepctr;
    s.ctl = d_ctl;
    s.err_flag = d_err;
    s.roi_xy = d_roi;
    return s;
  }

  int stage(size_t bytes) {
    if (bytes <= stage_bytes) return 0;
    dfree(d_stage);
    CK(cudaMalloc(&d_stage, bytes));
    stage_bytes = bytes;
    return 0;
  }

  // Convert a double host array to the pixel type on the device.
  int upload_t(void** dst, const double* src, size_t n) {
    dfree(*dst);
    CK(cudaMalloc(dst, n * tsize()));
    if (prec == 32) {
      std::vector<float> tmp(src, src + n);
      CK(cudaMemcpy(*dst, tmp.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    } else {
      CK(cudaMemcpy(*dst, src, n * sizeof(double), cudaMemcpyHostToDevice));
    }
    return 0;
  }

  int configure() {
    if (configured) return 0;
    if (!model_set) {
      set_error("the fitting model has not been initialised");
      return -1;
    }
    // the FFT PSF and pupil-function models run in the FP64 engine only
    if (cfg.model == M_FFT || cfg.model == M_PUPIL) prec = 64;
    cudaError_t e = (prec == 32) ? Launch<float>::configure(cfg, &sweep_grid, &sweep_smem, &cta_smem, &warp_smem)
                                 : Launch<double>::configure(cfg, &sweep_grid, &sweep_smem, &cta_smem, &warp_smem);
    if (e != cudaSuccess) {
      set_error("kernel configuration failed (ROI %d, %d pixels): %s", cfg.roi, cfg.nroi,
                cudaGetErrorString(e));
      return -1;
    }
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));
    configured = true;
    return 0;
  }

  // Allocate the frame arrays for n frames (keeps contents when unchanged).
  int set_frames(int n) {
    if (configure()) return -1;
    if (n == F && d_x) return 0;
    dfree(d_x); dfree(d_xq); dfree(d_xff); dfree(d_f); dfree(d_bg); dfree(d_cnt); dfree(d_bgest); dfree(d_ctl);
    dfree(d_cellstart);
    const size_t np = (size_t)npix * n;
    const size_t words = (prec == 64) ? 2 : 1;   // accumulator words per pixel
    CK(cudaMalloc(&d_x, np * tsize()));
    if (prec == 32) CK(cudaMalloc(&d_xq, np * sizeof(long long)));
    if (prec == 32) CK(cudaMalloc(&d_xff, np * sizeof(float2)));
    CK(cudaMalloc(&d_f, np * words * sizeof(long long)));
    CK(cudaMalloc(&d_bg, np * words * sizeof(long long)));
    CK(cudaMalloc(&d_cnt, np * sizeof(int)));
    CK(cudaMalloc(&d_bgest, np * sizeof(double)));
    CK(cudaMemset(d_f, 0, np * words * sizeof(long long)));
    CK(cudaMemset(d_bg, 0, np * words * sizeof(long long)));
    CK(cudaMemset(d_cnt, 0, np * sizeof(int)));
    CK(cudaMemset(d_bgest, 0, np * sizeof(double)));
    CK(cudaMalloc(&d_ctl, sizeof(FrameCtl) * n));
    CK(cudaMemset(d_ctl, 0, sizeof(FrameCtl) * n));
    CK(cudaMalloc(&d_cellstart, sizeof(int) * (size_t)n * (cfg.gx * cfg.gy + 1)));
    if (!d_err) {
      CK(cudaMalloc(&d_err, sizeof(unsigned)));
      CK(cudaMemset(d_err, 0, sizeof(unsigned)));
    }
    if (!d_epoch) {
      // done flags start at -1 (d_done is memset to 0xff), epochs at 1
      const int one = 1;
      CK(cudaMalloc(&d_epoch, sizeof(int)));
      CK(cudaMemcpy(d_epoch, &one, sizeof(int), cudaMemcpyHostToDevice));
    }
    if (!d_rqe) {
      if (upload_t(&d_rqe, rqe_h.data(), npix)) return -1;
      if (upload_t(&d_scmos, scmos_h.data(), npix)) return -1;
      if (!aij_h.empty() && upload_t(&d_aij, aij_h.data(), aij_h.size())) return -1;
      // the FFT and pupil models' tables (FP64: d_aij holds them as doubles)
      if (cfg.model == M_FFT || cfg.model == M_PUPIL) cfg.fft = static_cast<const double*>(d_aij);
      CK(cudaMalloc(&d_roi, roi_xy.size() * sizeof(unsigned short)));
      CK(cudaMemcpy(d_roi, roi_xy.data(), roi_xy.size() * sizeof(unsigned short), cudaMemcpyHostToDevice));
    }
    F = n;
    pk_off.assign(n, 0);
    cap_f.assign(n, 0);
    nfit.assign(n, 0);
    release_peaks();
    host_pk.clear();
    host_valid = true;
    return 0;
  }

  // Peak storage: capacity caps[f] per frame (contents dropped).
  int set_peak_caps(const std::vector<int>& caps) {
    release_peaks();
    int tot = 0;
    for (int f = 0; f < F; f++) {
      pk_off[f] = tot;
      cap_f[f] = caps[f];
      tot += caps[f];
    }
    cap_total = std::max(tot, 1);
    const size_t c = cap_total;
    CK(cudaMalloc(&d_pk, c * sizeof(PeakRec)));
    CK(cudaMalloc(&d_snap, c * sizeof(PeakRec)));
    CK(cudaMalloc(&d_run, c * sizeof(int)));
    CK(cudaMalloc(&d_anchor, c * sizeof(unsigned)));
    CK(cudaMalloc(&d_done, c * sizeof(int)));
    CK(cudaMalloc(&d_cellitems, c * sizeof(int2)));
    CK(cudaMalloc(&d_stepctr, c * NCOUNTERS * sizeof(int)));
    CK(cudaMemset(d_pk, 0, c * sizeof(PeakRec)));
    CK(cudaMemset(d_done, 0xff, c * sizeof(int)));
    CK(cudaMemset(d_stepctr, 0, c * NCOUNTERS * sizeof(int)));
    CK(cudaMalloc(&d_pkoff, F * sizeof(int)));
    CK(cudaMalloc(&d_nfit, F * sizeof(int)));
    CK(cudaMemcpy(d_pkoff, pk_off.data(), F * sizeof(int), cudaMemcpyHostToDevice));
    return sync_nfit();
  }

  int sync_nfit() {
    if (!d_nfit || F == 0) return 0;
    CK(cudaMemcpyAsync(d_nfit, nfit.data(), F * sizeof(int), cudaMemcpyHostToDevice, stream));
    return 0;
  }

  int check_err_flag() {
    unsigned e = 0;
    CK(cudaMemcpy(&e, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (e) {
      cudaMemset(d_err, 0, sizeof(unsigned));
      set_error("device wait timed out (flag 0x%x); results of this call are invalid", e);
      return -1;
    }
    return 0;
  }

  // Next pair of timing events from the pool.
  int timing_pair(cudaEvent_t* a, cudaEvent_t* b) {
    while (pool.size() < pool_used + 2) {
      cudaEvent_t ev;
      CK(cudaEventCreate(&ev));
      pool.push_back(ev);
    }
    *a = pool[pool_used];
    *b = pool[pool_used + 1];
    pool_used += 2;
    return 0;
  }

  // Read and forget the recorded sweep timings (synchronises on the last).
  int drain_timing() {
    if (pool_used == 0) return 0;
    CK(cudaEventSynchronize(pool[pool_used - 1]));
    for (size_t i = 0; i + 1 < pool_used; i += 2) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, pool[i], pool[i + 1]));
      sweep_ms += ms;
      sweep_launches++;
      sweep_times.push_back(ms);
    }
    pool_used = 0;
    return 0;
  }

  int grid() const {
    return (sweep_ctas_cap > 0 && sweep_ctas_cap < sweep_grid) ? sweep_ctas_cap : sweep_grid;
  }

  int tick() {
    ticks++;
    launches += 3;
    cudaEvent_t ta = nullptr, tb = nullptr;
    if (timing && timing_pair(&ta, &tb)) return -1;
    if (prec == 32) {
      FrameSet<float> s = fs<float>();
      CK(Launch<float>::prepare(cfg, s, cta_smem, stream));
      if (timing) CK(cudaEventRecord(ta, stream));
      CK(Launch<float>::sweep(cfg, s, grid(), sweep_smem, stream));
      if (timing) CK(cudaEventRecord(tb, stream));
      CK(Launch<float>::post(cfg, s, cta_smem, stream));
    } else {
      FrameSet<double> s = fs<double>();
      CK(Launch<double>::prepare(cfg, s, cta_smem, stream));
      if (timing) CK(cudaEventRecord(ta, stream));
      CK(Launch<double>::sweep(cfg, s, grid(), sweep_smem, stream));
      if (timing) CK(cudaEventRecord(tb, stream));
      CK(Launch<double>::post(cfg, s, cta_smem, stream));
    }
    return 0;
  }

  // Run ticks until no frame is pending.  Frames start in SWEEP_PENDING
  // with max_sweeps set by the caller.
  // Two bursts are kept in flight: the next two ticks are queued before the
  // host reads the frame control blocks of the previous burst, so the
  // device never idles on the host's poll.  Ticks queued after the last
  // frame has finished change nothing (every kernel skips DONE frames).
  // Fits of one or two sweeps (a host-driven sweep loop) keep one burst in
  // flight, so that no tick is launched past their end.
  int run_until_done(std::vector<FrameCtl>& ctl, int max_sweeps) {
    if (ensure_poll_buffers()) return -1;
    bool tail_queued = false;
    const bool ahead = max_sweeps > 2;
    if (burst_poll(0)) return -1;
    int cur = 0;
    for (;;) {
      if (ahead && burst_poll(1 - cur)) return -1;
      CK(cudaEventSynchronize(ev_pb[cur]));
      if (h_perr[cur]) {
        CK(cudaStreamSynchronize(stream));
        return check_err_flag() ? -1 : 0;
      }
      bool active = false;
      for (int f = 0; f < F; f++)
        if (h_pctl[cur][f].phase != PH_DONE && h_pctl[cur][f].phase != PH_IDLE) active = true;
      if (!active) {
        for (int f = 0; f < F; f++) ctl[f] = h_pctl[cur][f];
        CK(cudaStreamSynchronize(stream));
        return check_err_flag() ? -1 : 0;
      }
      // Once every frame still fitting has at most tail_peaks RUNNING peaks
      // (a count that only falls during a fit), their remaining sweeps run
      // in one launch after the ticks already queued; a frame that is not
      // ready for it when it runs is left to the ticks.
      if (ahead && tail_peaks > 0 && !tail_queued) {
        bool all = true, any = false;
        for (int f = 0; f < F && all; f++) {
          const FrameCtl& c = h_pctl[cur][f];
          if (c.phase == PH_DONE || c.phase == PH_IDLE) continue;
          if (c.phase == PH_SWEEP_PENDING && c.sweeps > 0 && c.unconverged <= tail_peaks) any = true;
          else all = false;
        }
        if (all && any) {
          if (prec == 32) CK(Launch<float>::tail(cfg, fs<float>(), tail_peaks, stream));
          else CK(Launch<double>::tail(cfg, fs<double>(), tail_peaks, stream));
          launches += 1;
          tail_queued = true;
        }
      }
      if (ahead) {
        cur = 1 - cur;
      } else if (burst_poll(cur)) {
        return -1;
      }
    }
  }

  // Pinned buffers and events of the two bursts in flight.
  FrameCtl* h_pctl[2] = {nullptr, nullptr};
  unsigned* h_perr = nullptr;
  cudaEvent_t ev_pb[2] = {nullptr, nullptr};
  int pctl_n = 0;

  int ensure_poll_buffers() {
    if (!h_perr) {
      CK(cudaMallocHost((void**)&h_perr, 2 * sizeof(unsigned)));
      for (int b = 0; b < 2; b++) CK(cudaEventCreateWithFlags(&ev_pb[b], cudaEventDisableTiming));
    }
    if (pctl_n < F) {
      for (int b = 0; b < 2; b++) {
        if (h_pctl[b]) cudaFreeHost(h_pctl[b]);
        h_pctl[b] = nullptr;
        CK(cudaMallocHost((void**)&h_pctl[b], sizeof(FrameCtl) * F));
      }
      pctl_n = F;
    }
    return 0;
  }

  void release_poll_buffers() {
    release_graphs();
    for (int b = 0; b < 2; b++) {
      if (h_pctl[b]) cudaFreeHost(h_pctl[b]);
      if (ev_pb[b]) cudaEventDestroy(ev_pb[b]);
      h_pctl[b] = nullptr;
      ev_pb[b] = nullptr;
    }
    if (h_perr) cudaFreeHost(h_perr);
    h_perr = nullptr;
    pctl_n = 0;
  }

  // Bursts as CUDA graphs: the two ticks, the poll copies and the event of
  // poll buffer b are captured once and relaunched as one graph while
  // nothing they were captured with changes (model configuration, the frame
  // set's device arrays, launch shapes, poll buffers); anything else
  // re-captures.  The sweep epoch lives on the device (k_post advances
  // it), so the captured launches need no per-tick arguments.  With timing
  // on, or SA_CUDA_GRAPHS=0 in the environment, bursts are launched
  // kernel by kernel.
  cudaGraphExec_t burst_exec[2] = {nullptr, nullptr};
  std::vector<unsigned char> burst_sig[2];
  bool use_graphs = !(getenv("SA_CUDA_GRAPHS") && getenv("SA_CUDA_GRAPHS")[0] == '0');

  void release_graphs() {
    for (int b = 0; b < 2; b++) {
      if (burst_exec[b]) cudaGraphExecDestroy(burst_exec[b]);
      burst_exec[b] = nullptr;
      burst_sig[b].clear();
    }
  }

  std::vector<unsigned char> burst_signature(int b) const {
    std::vector<unsigned char> v;
    auto put = [&v](const void* p, size_t n) {
      const unsigned char* c = static_cast<const unsigned char*>(p);
      v.insert(v.end(), c, c + n);
    };
    put(&cfg, sizeof(cfg));
    if (prec == 32) {
      const FrameSet<float> s = fs<float>();
      put(&s, sizeof(s));
    } else {
      const FrameSet<double> s = fs<double>();
      put(&s, sizeof(s));
    }
    const int g = grid();
    put(&g, sizeof(g));
    put(&prec, sizeof(prec));
    put(&sweep_smem, sizeof(sweep_smem));
    put(&cta_smem, sizeof(cta_smem));
    put(&h_pctl[b], sizeof(h_pctl[b]));
    put(&h_perr, sizeof(h_perr));
    put(&ev_pb[b], sizeof(ev_pb[b]));
    put(&stream, sizeof(stream));
    return v;
  }

  // The stream work of one burst (captured; no early return, so that the
  // capture is always ended).
  cudaError_t enqueue_burst(int b) {
    cudaError_t err = cudaSuccess;
    auto keep = [&err](cudaError_t e) {
      if (err == cudaSuccess) err = e;
    };
    for (int i = 0; i < 2; i++) {
      if (prec == 32) {
        const FrameSet<float> s = fs<float>();
        keep(Launch<float>::prepare(cfg, s, cta_smem, stream));
        keep(Launch<float>::sweep(cfg, s, grid(), sweep_smem, stream));
        keep(Launch<float>::post(cfg, s, cta_smem, stream));
      } else {
        const FrameSet<double> s = fs<double>();
        keep(Launch<double>::prepare(cfg, s, cta_smem, stream));
        keep(Launch<double>::sweep(cfg, s, grid(), sweep_smem, stream));
        keep(Launch<double>::post(cfg, s, cta_smem, stream));
      }
    }
    keep(cudaMemcpy2DAsync(h_pctl[b], sizeof(FrameCtl), d_ctl, sizeof(FrameCtl), offsetof(FrameCtl, escaped), F,
                           cudaMemcpyDeviceToHost, stream));
    keep(cudaMemcpyAsync(h_perr + b, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    // an event record node (a plain record under capture only marks the
    // capture's dependencies and cannot be waited on afterwards)
    keep(cudaEventRecordWithFlags(ev_pb[b], stream, cudaEventRecordExternal));
    return err;
  }

  // Launch burst b as a graph; 1 when graphs are not available here (the
  // caller launches kernel by kernel), -1 on error.
  int burst_graph(int b) {
    if (stream == 0) {
      // the legacy default stream cannot be captured: a blocking stream of
      // our own keeps the same ordering with work on the legacy stream
      if (!own_stream && cudaStreamCreate(&own_stream) != cudaSuccess) {
        cudaGetLastError();
        use_graphs = false;
        return 1;
      }
      stream = own_stream;
    }
    std::vector<unsigned char> sig = burst_signature(b);
    if (!burst_exec[b] || sig != burst_sig[b]) {
      if (burst_exec[b]) cudaGraphExecDestroy(burst_exec[b]);
      burst_exec[b] = nullptr;
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        use_graphs = false;
        return 1;
      }
      cudaError_t err = enqueue_burst(b);
      const cudaError_t e2 = cudaStreamEndCapture(stream, &g);
      if (err == cudaSuccess) err = e2;
      if (err == cudaSuccess) err = cudaGraphInstantiate(&burst_exec[b], g, 0);
      if (g) cudaGraphDestroy(g);
      if (err != cudaSuccess) {
        cudaGetLastError();
        burst_exec[b] = nullptr;
        use_graphs = false;
        return 1;
      }
      burst_sig[b] = sig;
    }
    CK(cudaGraphLaunch(burst_exec[b], stream));
    ticks += 2;
    launches += 6;
    return 0;
  }

  // Two ticks, then the frame control blocks and the error flag into
  // pinned buffer b, then its event.
  int burst_poll(int b) {
    if (use_graphs && !timing) {
      const int r = burst_graph(b);
      if (r <= 0) return r;
    }
    for (int i = 0; i < 2; i++)
      if (tick()) return -1;
    // the fields before the device-only lists of every frame's block
    CK(cudaMemcpy2DAsync(h_pctl[b], sizeof(FrameCtl), d_ctl, sizeof(FrameCtl), offsetof(FrameCtl, escaped), F,
                         cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(h_perr + b, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    CK(cudaEventRecord(ev_pb[b], stream));
    return 0;
  }

  // Start a fit (max_sweeps sweeps at most) on all frames, or on the frames
  // with active[f] != 0, and run it.  Inactive frames stay DONE: every
  // kernel skips them.
  int fit(int max_sweeps, int* sweeps_out, const int32_t* active = nullptr) {
    if (!d_pk) {
      if (sweeps_out) *sweeps_out = 0;
      return 0;
    }
    std::vector<FrameCtl> ctl(F);
    CK(cudaMemcpy(ctl.data(), d_ctl, sizeof(FrameCtl) * F, cudaMemcpyDeviceToHost));
    for (int f = 0; f < F; f++) {
      ctl[f].phase = (active && !active[f]) ? PH_DONE : PH_SWEEP_PENDING;
      ctl[f].sweeps = 0;
      ctl[f].max_sweeps = max_sweeps;
    }
    CK(cudaMemcpy(d_ctl, ctl.data(), sizeof(FrameCtl) * F, cudaMemcpyHostToDevice));
    if (run_until_done(ctl, max_sweeps)) return -1;
    int sw = 0;
    for (int f = 0; f < F; f++) sw = std::max(sw, ctl[f].sweeps);
    unconv_cache = (F == 1) ? ctl[0].unconverged : -1;
    host_valid = false;
    if (sweeps_out) *sweeps_out = sw;
    return 0;
  }

  int pull_records() {
    if (host_valid) return 0;
    host_pk.resize(nfit[0]);
    if (nfit[0] > 0)
      CK(cudaMemcpy(host_pk.data(), d_pk + pk_off[0], sizeof(PeakRec) * nfit[0], cudaMemcpyDeviceToHost));
    host_valid = true;
    return 0;
  }

  int push_records() {
    if (!host_pk.empty())
      CK(cudaMemcpy(d_pk + pk_off[0], host_pk.data(), sizeof(PeakRec) * host_pk.size(), cudaMemcpyHostToDevice));
    nfit[0] = (int)host_pk.size();
    if (sync_nfit()) return -1;
    CK(cudaStreamSynchronize(stream));
    host_valid = true;
    unconv_cache = -1;
    return 0;
  }

  int read_counters(long long* out) {
    std::vector<FrameCtl> ctl(F);
    CK(cudaMemcpy(ctl.data(), d_ctl, sizeof(FrameCtl) * F, cudaMemcpyDeviceToHost));
    for (int i = 0; i < NCOUNTERS; i++) out[i] = 0;
    for (int f = 0; f < F; f++)
      for (int i = 0; i < NCOUNTERS; i++) out[i] += ctl[f].ctr[i];
    return 0;
  }
};

Engine* E(saFitData* h) { return h ? reinterpret_cast<Engine*>(h->engine) : nullptr; }

// Fold new device counter totals into the reference-layout fields.
void sync_counters(saFitData* h) {
  Engine* e = E(h);
  if (!e || !e->d_ctl) return;
  long long tot[NCOUNTERS];
  if (e->read_counters(tot)) return;
  int* fields[8] = {&h->n_dposv, &h->n_iterations, &h->n_lost, &h->n_margin,
                    &h->n_neg_fi, &h->n_neg_height, &h->n_non_converged, &h->n_non_decr};
  for (int i = 0; i < 8; i++) {
    *fields[i] += (int)(tot[i] - e->ctr_seen[i]);
    e->ctr_seen[i] = tot[i];
  }
  e->ctr_seen[C_STARTFAIL] = tot[C_STARTFAIL];
}

// Circular ROI, mFitInitializeROIIndexing multi_fit.c:1031-1060.
void roi_index(Engine* e, int roi) {
  const double c = 0.5 * (double)roi, rr = c * c;
  e->roi_x.clear();
  e->roi_y.clear();
  e->roi_xy.clear();
  for (int i = 0; i < roi; i++) {
    const double dy = (double)i - c + 0.5;
    for (int j = 0; j < roi; j++) {
      const double dx = (double)j - c + 0.5;
      if ((dx * dx + dy * dy) <= rr) {
        e->roi_x.push_back(j);
        e->roi_y.push_back(i);
        e->roi_xy.push_back((unsigned short)(j | (i << 8)));
      }
    }
  }
  e->cfg.roi = roi;
  e->cfg.nroi = (int)e->roi_x.size();
}

void finish_geometry(Engine* e) {
  ModelCfg& c = e->cfg;
  if (c.dil < 0) c.dil = 3;
  if (c.dil_late < 0 || c.dil_late > c.dil) c.dil_late = c.dil;
  c.cell = c.roi + 2 * c.dil;
  // keep the grid small enough for shared memory
  while ((long long)((c.nx + c.cell - 1) / c.cell) * ((c.ny + c.cell - 1) / c.cell) > 40000) c.cell *= 2;
  c.gx = (c.nx + c.cell - 1) / c.cell;
  c.gy = (c.ny + c.cell - 1) / c.cell;
}

saFitData* new_handle(const double* rqe, const double* scmos, double tol, int nx, int ny) {
  if (nx <= 0 || ny <= 0 || nx > 65535 || ny > 65535) {
    set_error("unsupported image size %d x %d", nx, ny);
    return nullptr;
  }
  saFitData* h = (saFitData*)calloc(1, sizeof(saFitData));
  Engine* e = new Engine();
  h->engine = e;
  {
    // set-up of saGetFitImageNoAlloc (no device: the entry point reports it)
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0) e->noalloc = noalloc_scratch();
    cudaGetLastError();
  }
  e->cfg.nx = nx;
  e->cfg.ny = ny;
  e->cfg.tol = tol;
  e->cfg.min_height = -1.0;   // multi_fit.c:965
  e->cfg.dil = -1;                // 3 pixels (finish_geometry) unless set
  // After 10 sweeps peaks move by hundredths of a pixel per sweep:
  // dependencies then use the undilated footprint (an anchor move escapes).
  // Measured on the 64-frame 3d workload: switching after 5, 10 or 20
  // sweeps is within 1 %, a late dilation of 1 costs 3 %.
  e->cfg.dil_late = 0;
  e->cfg.dil_switch = 10;
  e->npix = (long long)nx * ny;
  e->rqe_h.assign(rqe, rqe + e->npix);
  e->scmos_h.assign(scmos, scmos + e->npix);
  // uniform calibration (rqe 1, sCMOS 0 everywhere) enables the FP32 step's
  // per-peak background quantisation; SA_CUDA_CAL_FAST=0 keeps the
  // per-pixel form (the results are the same)
  const char* pc = getenv("SA_CUDA_CAL_FAST");
  const bool cal_fast = !(pc && atoi(pc) == 0);
  e->cfg.rqe_one = cal_fast && std::all_of(e->rqe_h.begin(), e->rqe_h.end(), [](double v) { return v == 1.0; }) ? 1 : 0;
  e->cfg.scmos_zero = cal_fast && std::all_of(e->scmos_h.begin(), e->scmos_h.end(), [](double v) { return v == 0.0; }) ? 1 : 0;
  const char* pe = getenv("SA_CUDA_PRECISION");
  if (pe && atoi(pe) == 64) e->prec = 64;
  const char* ps = getenv("SA_CUDA_SERIAL");
  e->cfg.force_serial = (ps && atoi(ps) == 1) ? 1 : 0;
  h->image_size_x = nx;
  h->image_size_y = ny;
  h->tolerance = tol;
  h->minimum_height = -1.0;
  return h;
}

void publish_geometry(saFitData* h) {
  Engine* e = E(h);
  h->fit_size_x = e->cfg.roi;
  h->fit_size_y = e->cfg.roi;
  h->roi_n_index = e->cfg.nroi;
  h->roi_x_index = e->roi_x.data();
  h->roi_y_index = e->roi_y.data();
  h->xoff = e->cfg.xoff;
  h->yoff = e->cfg.yoff;
  h->zoff = e->cfg.zoff;
}

void set_model(saFitData* h, int model, int jac) {
  Engine* e = E(h);
  if (!e) return;
  e->cfg.model = model;
  e->cfg.jac = jac;
  e->model_set = true;
  h->jac_size = jac;
  finish_geometry(e);
}

void unsupported(saFitData* h, const char* what) {
  Engine* e = E(h);
  if (e) e->unsupported = true;
  set_error("%s: only the MLE error model is implemented by this engine", what);
}

int parse_ptype(const char* t) {
  if (!t) return -1;
  if (!strcmp(t, "finder")) return PT_FINDER;
  if (!strcmp(t, "testing")) return PT_TESTING;
  if (!strcmp(t, "text") || !strcmp(t, "hdf5")) return PT_TEXT;
  return -1;
}

int ncol_for(const Engine* e, int ptype) {
  const bool spl = e->cfg.model >= M_SPLINE2D;
  if (ptype == PT_TEXT) return spl ? 5 : 7;
  return spl ? 3 : 4;
}

// Insert new peaks for frames [0, nframes) (rows concatenated per frame).
int insert_peaks(Engine* e, const double* rows, const std::vector<int>& counts, int ptype,
                 bool rows_on_device = false) {
  const int ncol = ncol_for(e, ptype);
  int n = 0;
  for (int c : counts) n += c;
  if (n == 0) return 0;
  std::vector<int> slots(n), frames(n), ffirst(counts.size()), fn(counts.size());
  int i = 0;
  for (size_t f = 0; f < counts.size(); f++) {
    ffirst[f] = i;
    fn[f] = counts[f];
    for (int j = 0; j < counts[f]; j++, i++) {
      slots[i] = e->pk_off[f] + e->nfit[f] + j;
      frames[i] = (int)f;
    }
  }
  const size_t rb = (size_t)n * ncol * sizeof(double);
  const size_t ib = (size_t)n * sizeof(int);
  const size_t fb = counts.size() * sizeof(int);
  if (e->stage(rb + 2 * ib + 2 * fb + 64)) return -1;
  char* st = (char*)e->d_stage;
  double* d_rows = (double*)st;
  int* d_slots = (int*)(st + rb);
  int* d_frames = (int*)(st + rb + ib);
  int* d_ff = (int*)(st + rb + 2 * ib);
  int* d_fn = (int*)(st + rb + 2 * ib + fb);
  if (rows_on_device) d_rows = const_cast<double*>(rows);
  else CK(cudaMemcpyAsync(d_rows, rows, rb, cudaMemcpyHostToDevice, e->stream));
  CK(cudaMemcpyAsync(d_slots, slots.data(), ib, cudaMemcpyHostToDevice, e->stream));
  CK(cudaMemcpyAsync(d_frames, frames.data(), ib, cudaMemcpyHostToDevice, e->stream));
  CK(cudaMemcpyAsync(d_ff, ffirst.data(), fb, cudaMemcpyHostToDevice, e->stream));
  CK(cudaMemcpyAsync(d_fn, fn.data(), fb, cudaMemcpyHostToDevice, e->stream));
  if (e->prec == 32) {
    FrameSet<float> s = e->fs<float>();
    CK(Launch<float>::new_peaks(e->cfg, s, d_rows, ncol, ptype, d_slots, d_frames, n,
                                ptype != PT_FINDER, e->warp_smem, e->stream));
    if (ptype == PT_FINDER)
      CK(Launch<float>::new_peaks_finder(e->cfg, s, d_slots, d_ff, d_fn, (int)counts.size(), e->warp_smem, e->stream));
    CK(Launch<float>::peak_error(e->cfg, s, d_slots, d_frames, n, e->stream));
  } else {
    FrameSet<double> s = e->fs<double>();
    CK(Launch<double>::new_peaks(e->cfg, s, d_rows, ncol, ptype, d_slots, d_frames, n,
                                 ptype != PT_FINDER, e->warp_smem, e->stream));
    if (ptype == PT_FINDER)
      CK(Launch<double>::new_peaks_finder(e->cfg, s, d_slots, d_ff, d_fn, (int)counts.size(), e->warp_smem, e->stream));
    CK(Launch<double>::peak_error(e->cfg, s, d_slots, d_frames, n, e->stream));
  }
  e->launches += (ptype == PT_FINDER) ? 3 : 2;
  for (size_t f = 0; f < counts.size(); f++) e->nfit[f] += counts[f];
  if (e->sync_nfit()) return -1;
  CK(cudaStreamSynchronize(e->stream));
  e->host_valid = false;
  e->unconv_cache = -1;
  return 0;
}

// mFitNewPeaks storage growth with ERROR compaction (multi_fit.c:1428-1477),
// single frame.
int grow_frame0(Engine* e, int n_new) {
  const int nf = e->nfit[0];
  if (e->d_pk && nf + n_new <= e->cap_f[0]) return 0;
  const int n_alloc = 500 * ((nf + n_new) / 500 + 1);
  std::vector<PeakRec> keep;
  if (e->d_pk && nf > 0) {
    if (e->pull_records()) return -1;
    for (const PeakRec& r : e->host_pk)
      if (r.status != ERROR) keep.push_back(r);
  }
  std::vector<int> caps(1, n_alloc);
  if (e->set_peak_caps(caps)) return -1;
  e->host_pk = keep;
  return e->push_records();
}

int new_peaks_single(saFitData* h, double* peaks, const char* p_type, int n) {
  Engine* e = E(h);
  if (!e) return -1;
  if (e->unsupported) {
    set_error("handle uses an unsupported error model");
    return -1;
  }
  const int pt = parse_ptype(p_type);
  if (pt < 0) {
    set_error("Unrecognized peak type '%s'!", p_type ? p_type : "(null)");
    return -1;
  }
  if (!e->d_x) {
    set_error("newPeaks before newImage");
    return -1;
  }
  if (n <= 0) return 0;
  if (grow_frame0(e, n)) return -1;
  std::vector<int> counts(1, n);
  if (insert_peaks(e, peaks, counts, pt)) return -1;
  h->nfit = e->nfit[0];
  h->max_nfit = e->cap_f[0];
  sync_counters(h);
  return 0;
}

int image_single(saFitData* h, const double* img, bool background) {
  Engine* e = E(h);
  if (!e) return -1;
  if (e->set_frames(e->F > 0 ? e->F : 1)) return -1;
  const size_t bytes = (size_t)e->npix * sizeof(double);
  if (e->stage(bytes)) return -1;
  CK(cudaMemcpyAsync(e->d_stage, img, bytes, cudaMemcpyHostToDevice, e->stream));
  if (e->prec == 32) {
    FrameSet<float> s = e->fs<float>();
    CK(background ? Launch<float>::new_background(s, e->d_stage, 64, 0, 1, e->stream)
                  : Launch<float>::new_image(s, e->d_stage, 64, 0, 1, e->stream));
  } else {
    FrameSet<double> s = e->fs<double>();
    CK(background ? Launch<double>::new_background(s, e->d_stage, 64, 0, 1, e->stream)
                  : Launch<double>::new_image(s, e->d_stage, 64, 0, 1, e->stream));
  }
  CK(cudaStreamSynchronize(e->stream));
  if (!background) {
    // mFitNewImage resets nfit (multi_fit.c:1407)
    e->nfit[0] = 0;
    if (e->sync_nfit()) return -1;
    e->host_pk.clear();
    e->host_valid = true;
    e->unconv_cache = -1;
    h->nfit = 0;
  }
  return 0;
}

int props_device(Engine* e, int frame0, const std::vector<int>& counts, double* sum, double* fg,
                 double* bg, double* jac) {
  int n = 0;
  for (int c : counts) n += c;
  if (n == 0) return 0;
  std::vector<int> slots(n), frames(n);
  int i = 0;
  for (size_t f = 0; f < counts.size(); f++)
    for (int j = 0; j < counts[f]; j++, i++) {
      slots[i] = e->pk_off[frame0 + f] + j;
      frames[i] = frame0 + (int)f;
    }
  const int k = e->cfg.jac;
  const size_t ib = (size_t)n * sizeof(int);
  const size_t db = (size_t)n * sizeof(double);
  const size_t jb = (size_t)n * k * sizeof(double);
  if (e->stage(2 * ib + 3 * db + jb + 64)) return -1;
  char* st = (char*)e->d_stage;
  int* d_slots = (int*)st;
  int* d_frames = (int*)(st + ib);
  double* d_sum = (double*)(st + 2 * ib);
  double* d_fg = d_sum + n;
  double* d_bg = d_fg + n;
  double* d_jac = d_bg + n;
  CK(cudaMemcpyAsync(d_slots, slots.data(), ib, cudaMemcpyHostToDevice, e->stream));
  CK(cudaMemcpyAsync(d_frames, frames.data(), ib, cudaMemcpyHostToDevice, e->stream));
  if (e->prec == 32)
    CK(Launch<float>::peak_props(e->cfg, e->fs<float>(), d_slots, d_frames, n, d_sum, d_fg, d_bg,
                                 jac ? d_jac : nullptr, e->warp_smem, e->stream));
  else
    CK(Launch<double>::peak_props(e->cfg, e->fs<double>(), d_slots, d_frames, n, d_sum, d_fg, d_bg,
                                  jac ? d_jac : nullptr, e->warp_smem, e->stream));
  if (sum) CK(cudaMemcpyAsync(sum, d_sum, db, cudaMemcpyDeviceToHost, e->stream));
  if (fg) CK(cudaMemcpyAsync(fg, d_fg, db, cudaMemcpyDeviceToHost, e->stream));
  if (bg) CK(cudaMemcpyAsync(bg, d_bg, db, cudaMemcpyDeviceToHost, e->stream));
  if (jac) CK(cudaMemcpyAsync(jac, d_jac, jb, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return 0;
}

// Property of one record (multi_fit.c:754-868); returns false if unknown.
bool record_prop(const Engine* e, const PeakRec& r, const char* what, double* v) {
  if (!strcmp(what, "background")) *v = r.p[PBG];
  else if (!strcmp(what, "error")) *v = r.error;
  else if (!strcmp(what, "height")) *v = r.p[PH];
  else if (!strcmp(what, "x")) *v = r.p[PX] + e->cfg.xoff;
  else if (!strcmp(what, "xsigma")) *v = sqrt(1.0 / (2.0 * r.p[PXW]));
  else if (!strcmp(what, "y")) *v = r.p[PY] + e->cfg.yoff;
  else if (!strcmp(what, "ysigma")) *v = sqrt(1.0 / (2.0 * r.p[PYW]));
  else if (!strcmp(what, "z")) *v = r.p[PZ] + e->cfg.zoff;
  else return false;
  return true;
}

int get_double_props(Engine* e, int frame0, int nframes, double* values, const char* what) {
  std::vector<int> counts(e->nfit.begin() + frame0, e->nfit.begin() + frame0 + nframes);
  int n = 0;
  for (int c : counts) n += c;
  if (!strcmp(what, "bg_sum") || !strcmp(what, "fg_sum") || !strcmp(what, "fg_sum_sc") ||
      !strcmp(what, "sum") || !strcmp(what, "jacobian")) {
    std::vector<double> a(n), b(n), c(n);
    std::vector<double> jac;
    const bool jj = !strcmp(what, "jacobian");
    if (jj) jac.resize((size_t)n * e->cfg.jac);
    if (props_device(e, frame0, counts, a.data(), b.data(), c.data(), jj ? jac.data() : nullptr)) return -1;
    const std::vector<double>& src = jj ? jac : (!strcmp(what, "sum") ? a : (!strcmp(what, "bg_sum") ? c : b));
    memcpy(values, src.data(), src.size() * sizeof(double));
    return 0;
  }
  std::vector<PeakRec> recs(n);
  size_t o = 0;
  for (int f = 0; f < nframes; f++) {
    if (counts[f] > 0)
      CK(cudaMemcpy(recs.data() + o, e->d_pk + e->pk_off[frame0 + f], sizeof(PeakRec) * counts[f],
                    cudaMemcpyDeviceToHost));
    o += counts[f];
  }
  for (int i = 0; i < n; i++) {
    if (!record_prop(e, recs[i], what, values + i)) {
      set_error("Unrecognized parameter '%s'!", what);
      return -1;
    }
  }
  return 0;
}

}  // namespace

// Error recorder shared with the peak finder's translation unit.
void sa::record_error(const char* msg) { set_error("%s", msg); }

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

int saGetLastError(char* buf, int len) {
  const int n = (int)g_last_error.size();
  if (buf && len > 0) {
    strncpy(buf, g_last_error.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return n;
}

void saClearLastError(void) { g_last_error.clear(); }

int saDeviceCount(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

saFitData* daoInitialize(double* rqe, double* scmos, double tol, int nx, int ny, int roi) {
  if (roi < 2 || roi > MAX_ROI || roi > 255) {
    set_error("unsupported ROI size %d (2..%d)", roi, MAX_ROI);
    return nullptr;
  }
  saFitData* h = new_handle(rqe, scmos, tol, nx, ny);
  if (!h) return nullptr;
  Engine* e = E(h);
  roi_index(e, roi);
  // dao_fit.c:1264-1271: the same offset for even and odd ROI sizes.
  e->cfg.xoff = 0.5 * ((double)roi) - 1.0;
  e->cfg.yoff = e->cfg.xoff;
  publish_geometry(h);
  return h;
}

void daoInitialize2DFixed(saFitData* h) { set_model(h, M_2DFIXED, 4); }

void daoInitialize2D(saFitData* h, double wmin, double wmax) {
  if (!E(h)) return;
  E(h)->cfg.wmin = wmin;
  E(h)->cfg.wmax = wmax;
  set_model(h, M_2D, 5);
}

void daoInitialize3D(saFitData* h, double wmin, double wmax) {
  if (!E(h)) return;
  E(h)->cfg.wmin = wmin;
  E(h)->cfg.wmax = wmax;
  set_model(h, M_3D, 6);
}

void daoInitializeZ(saFitData* h, double* wx, double* wy, double zmin, double zmax) {
  Engine* e = E(h);
  if (!e) return;
  for (int i = 0; i < 5; i++) {
    e->cfg.wx[i] = wx[i];
    e->cfg.wy[i] = wy[i];
  }
  // dao_fit.c:1566-1567: w0 squared
  e->cfg.wx[0] = e->cfg.wx[0] * e->cfg.wx[0];
  e->cfg.wy[0] = e->cfg.wy[0] * e->cfg.wy[0];
  e->cfg.zmin = zmin;
  e->cfg.zmax = zmax;
  set_model(h, M_Z, 5);
}

void daoInitialize2DFixedALS(saFitData* h) { unsupported(h, "daoInitialize2DFixedALS"); }
void daoInitialize2DFixedLS(saFitData* h) { unsupported(h, "daoInitialize2DFixedLS"); }
void daoInitialize2DFixedDWLS(saFitData* h) { unsupported(h, "daoInitialize2DFixedDWLS"); }
void daoInitialize2DFixedFWLS(saFitData* h) { unsupported(h, "daoInitialize2DFixedFWLS"); }
void daoInitialize2DALS(saFitData* h, double, double) { unsupported(h, "daoInitialize2DALS"); }
void daoInitialize2DLS(saFitData* h, double, double) { unsupported(h, "daoInitialize2DLS"); }
void daoInitialize2DDWLS(saFitData* h, double, double) { unsupported(h, "daoInitialize2DDWLS"); }
void daoInitialize2DFWLS(saFitData* h, double, double) { unsupported(h, "daoInitialize2DFWLS"); }
void cfInitialize3DALS(saFitData* h) { unsupported(h, "cfInitialize3DALS"); }
void cfInitialize3DLS(saFitData* h) { unsupported(h, "cfInitialize3DLS"); }
void cfInitialize3DFWLS(saFitData* h) { unsupported(h, "cfInitialize3DFWLS"); }
void mFitAnscombeTransformImage(saFitData* h) { unsupported(h, "mFitAnscombeTransformImage"); }

void daoNewPeaks(saFitData* h, double* peaks, char* p_type, int n) { new_peaks_single(h, peaks, p_type, n); }
void cfNewPeaks(saFitData* h, double* peaks, char* p_type, int n) { new_peaks_single(h, peaks, p_type, n); }

void daoCleanup(saFitData* h) {
  if (!h) return;
  delete E(h);
  free(h);
}

static void* new_spline(int type, const double* aij, int xs, int ys, int zs, size_t n) {
  SplineH* s = static_cast<SplineH*>(calloc(1, sizeof(SplineH)));
  if (!s) return nullptr;
  s->aij = static_cast<double*>(malloc(sizeof(double) * (n > 0 ? n : 1)));
  if (!s->aij) {
    free(s);
    return nullptr;
  }
  if (n) memcpy(s->aij, aij, sizeof(double) * n);
  s->type = type;
  s->xs = xs;
  s->ys = ys;
  s->zs = zs;
  return s;
}

void* initSpline2D(double* aij, int xs, int ys) {
  return new_spline(0, aij, xs, ys, 0, (size_t)xs * ys * 16);
}

void* initSpline3D(double* aij, int xs, int ys, int zs) {
  return new_spline(1, aij, xs, ys, zs, (size_t)xs * ys * zs * 64);
}

void splineCleanup(void* sp) {
  SplineH* s = reinterpret_cast<SplineH*>(sp);
  if (!s) return;
  free(s->aij);
  for (double* r : s->reserved) free(r);
  free(s);
}
int getXSize(void* sp) { return sp ? reinterpret_cast<SplineH*>(sp)->xs : 0; }
int getYSize(void* sp) { return sp ? reinterpret_cast<SplineH*>(sp)->ys : 0; }
int getZSize(void* sp) { return sp ? reinterpret_cast<SplineH*>(sp)->zs : 0; }

saFitData* cfInitialize(void* spline, double* rqe, double* scmos, double tol, int nx, int ny) {
  SplineH* s = reinterpret_cast<SplineH*>(spline);
  if (!s) {
    set_error("cfInitialize: NULL spline");
    return nullptr;
  }
  const int sx = s->xs - 1, sy = s->ys - 1;
  if (sx != sy) {
    // The reference exits the process here (cubic_fit.c:646-649).
    set_error("PSF must be square in X/Y!");
    return nullptr;
  }
  if (sx < 2 || sx > MAX_ROI) {
    set_error("unsupported spline size %d", s->xs);
    return nullptr;
  }
  saFitData* h = new_handle(rqe, scmos, tol, nx, ny);
  if (!h) return nullptr;
  Engine* e = E(h);
  e->spline = s;
  e->cfg.sx = s->xs;
  e->cfg.sy = s->ys;
  e->cfg.sz = s->zs;
  const size_t ncoef = (size_t)s->xs * s->ys * (s->type == 1 ? (size_t)s->zs * 64 : 16);
  e->aij_h.assign(s->aij, s->aij + ncoef);
  // cubic_fit.c:627-641
  if ((sx % 2) == 1) {
    e->cfg.xoff = (double)(sx / 2) - 0.5;
    e->cfg.yoff = (double)(sy / 2) - 0.5;
  } else {
    e->cfg.xoff = (double)(sx / 2) - 1.0;
    e->cfg.yoff = (double)(sy / 2) - 1.0;
  }
  roi_index(e, sx);
  publish_geometry(h);
  return h;
}

void cfInitialize2D(saFitData* h) {
  Engine* e = E(h);
  if (!e) return;
  if (e->spline && e->spline->type != 0) {
    set_error("cfInitialize2D needs a 2D spline");
    e->unsupported = true;
    return;
  }
  set_model(h, M_SPLINE2D, 4);
}

void cfInitialize3D(saFitData* h) {
  Engine* e = E(h);
  if (!e) return;
  if (e->spline && e->spline->type != 1) {
    set_error("cfInitialize3D needs a 3D spline");
    e->unsupported = true;
    return;
  }
  set_model(h, M_SPLINE3D, 5);
}

void cfCleanup(saFitData* h) {
  if (!h) return;
  Engine* e = E(h);
  if (e && e->spline) {
    splineCleanup(e->spline);   // cubic_fit.c:528-530
    e->spline = nullptr;
  }
  daoCleanup(h);
}

// ---- the FFT PSF fitter (psf_fft/fft_fit.c; psf_fft/fft_fit_c.py binds it) ----

// ftFitInitialize fft_fit.c:254-310: the ROI is the PSF's x size (square in
// x / y), xoff = x_size / 2 - 1, yoff = y_size / 2 - 1, five parameters
// (height, x, y, z, background).  The handle keeps the PSF's device tables;
// the FFT model runs in the FP64 engine.
saFitData* ftFitInitialize(void* psf_fft, double* rqe, double* scmos, double tol, int nx, int ny) {
  const PsfFFTH* p = reinterpret_cast<const PsfFFTH*>(psf_fft);
  if (!p) {
    set_error("ftFitInitialize: NULL psf_fft");
    return nullptr;
  }
  if (p->nx != p->ny) {
    // The reference exits the process here (fft_fit.c:283-286).
    set_error("PSF must be square in X/Y!");
    return nullptr;
  }
  if (p->nx < 2 || p->nx > MAX_ROI || p->nz < 1 || p->nz > 64) {
    set_error("unsupported PSF size %d x %d x %d", p->nz, p->ny, p->nx);
    return nullptr;
  }
  saFitData* h = new_handle(rqe, scmos, tol, nx, ny);
  if (!h) return nullptr;
  Engine* e = E(h);
  e->prec = 64;
  e->cfg.sx = p->nx;
  e->cfg.sy = p->ny;
  e->cfg.sz = p->nz;
  psf_fft_tables(*p, e->aij_h);
  e->cfg.xoff = 0.5 * (double)p->nx - 1.0;
  e->cfg.yoff = 0.5 * (double)p->ny - 1.0;
  roi_index(e, p->nx);
  publish_geometry(h);
  set_model(h, M_FFT, 5);
  return h;
}

// ftFitNewPeaks fft_fit.c:318-470 ("finder" / "testing": x, y, z;
// "text" / "hdf5": x, y, z, background, height).
void ftFitNewPeaks(saFitData* h, double* peaks, char* p_type, int n) { new_peaks_single(h, peaks, p_type, n); }

// ftFitCleanup fft_fit.c:165-192 (the PSF object is the caller's, freed by
// pFTCleanup).
void ftFitCleanup(saFitData* h) { daoCleanup(h); }

// ---- the pupil-function fitter (pupilfn/pupil_fit.c; pupilfn/pupil_fit_c.py binds it) ----

// pfitInitialize pupil_fit.c:288-332: the ROI is the pupil size,
// xoff = yoff = size / 2, five parameters (height, x, y, z, background).
// The handle keeps the pupil function's device tables as they are at this
// call (the reference reads the pupil data at each evaluation; its Python
// sets the pupil function before creating the fitter and not after); the
// pupil model runs in the FP64 engine.  The z range is open until
// pfitSetZRange.
saFitData* pfitInitialize(void* pupil_data, double* rqe, double* scmos, double tol, int nx, int ny) {
  const PupilH* p = reinterpret_cast<const PupilH*>(pupil_data);
  if (!p) {
    set_error("pfitInitialize: NULL pupil_data");
    return nullptr;
  }
  if (p->n < 2 || p->n > MAX_ROI || (p->n % 2) != 0) {
    set_error("unsupported pupil function size %d", p->n);
    return nullptr;
  }
  if (!pupil_rows_separable(*p)) {
    // pfnTranslate takes the x shift from kx's first column; the engine's
    // x derivative does the same
    set_error("pfitInitialize: kx must be constant along the pupil function's rows");
    return nullptr;
  }
  saFitData* h = new_handle(rqe, scmos, tol, nx, ny);
  if (!h) return nullptr;
  Engine* e = E(h);
  e->prec = 64;
  e->cfg.sx = p->n;
  e->cfg.sy = p->n;
  e->cfg.zmin = -1.0e300;
  e->cfg.zmax = 1.0e300;
  // the support band's rows size the per-warp row sums (pupil_scratch_doubles)
  e->cfg.sz = std::max(1, pupil_tables(*p, e->aij_h));
  e->cfg.xoff = 0.5 * (double)p->n;
  e->cfg.yoff = 0.5 * (double)p->n;
  roi_index(e, p->n);
  publish_geometry(h);
  set_model(h, M_PUPIL, 5);
  return h;
}

// pfitNewPeaks pupil_fit.c:342-503 ("finder" / "testing": x, y, z;
// "text" / "hdf5": x, y, z, background, height).
void pfitNewPeaks(saFitData* h, double* peaks, char* p_type, int n) { new_peaks_single(h, peaks, p_type, n); }

// pfitSetZRange pupil_fit.c:511-518: the clamp of pfitZRangeCheck :555-570.
void pfitSetZRange(saFitData* h, double min_z, double max_z) {
  Engine* e = E(h);
  if (!e) return;
  e->cfg.zmin = min_z;
  e->cfg.zmax = max_z;
}

// pfitCleanup pupil_fit.c:180-211 (the pupil data is the caller's, freed by
// pfnCleanup).
void pfitCleanup(saFitData* h) { daoCleanup(h); }

void mFitNewImage(saFitData* h, double* img) { image_single(h, img, false); }
void mFitNewBackground(saFitData* h, double* bg) { image_single(h, bg, true); }

void mFitIterateLM(saFitData* h) {
  Engine* e = E(h);
  if (!e || !e->d_x) return;
  int sw = 0;
  e->fit(1, &sw);
  sync_counters(h);
}

int saDoFit(saFitData* h, int max_iterations) {
  Engine* e = E(h);
  if (!e) return -1;
  if (!e->d_x) {
    set_error("doFit before newImage");
    return -1;
  }
  int sw = 0;
  if (e->fit(max_iterations + 1, &sw)) return -1;
  sync_counters(h);
  return sw;
}

int mFitGetUnconverged(saFitData* h) {
  Engine* e = E(h);
  if (!e || !e->d_pk) return 0;
  if (e->unconv_cache >= 0) return e->unconv_cache;
  if (e->pull_records()) return 0;
  int c = 0;
  for (const PeakRec& r : e->host_pk) c += (r.status == RUNNING);
  e->unconv_cache = c;
  return c;
}

int mFitGetNError(saFitData* h) {
  Engine* e = E(h);
  if (!e || !e->d_pk) return 0;
  if (e->pull_records()) return 0;
  int c = 0;
  for (const PeakRec& r : e->host_pk) c += (r.status == ERROR);
  return c;
}

void mFitGetPeakPropertyDouble(saFitData* h, double* values, char* what) {
  Engine* e = E(h);
  if (!e || !e->d_pk || e->nfit[0] == 0) return;
  get_double_props(e, 0, 1, values, what);
}

void mFitGetPeakPropertyInt(saFitData* h, int32_t* values, char* what) {
  Engine* e = E(h);
  if (!e || !e->d_pk || e->nfit[0] == 0) return;
  const bool it = !strcmp(what, "iterations");
  if (!it && strcmp(what, "status")) {
    set_error("Unrecognized parameter '%s'!", what);
    return;
  }
  if (e->pull_records()) return;
  for (size_t i = 0; i < e->host_pk.size(); i++)
    values[i] = it ? e->host_pk[i].iterations : e->host_pk[i].status;
}

static void fit_image_common(saFitData* h, double* out, int residual) {
  Engine* e = E(h);
  if (!e || !e->d_x) return;
  const size_t bytes = (size_t)e->npix * sizeof(double);
  if (e->stage(bytes)) return;
  cudaError_t err = (e->prec == 32)
                        ? Launch<float>::fit_image(e->fs<float>(), 0, (double*)e->d_stage, residual, e->stream)
                        : Launch<double>::fit_image(e->fs<double>(), 0, (double*)e->d_stage, residual, e->stream);
  if (err != cudaSuccess) {
    set_error("fit image: %s", cudaGetErrorString(err));
    return;
  }
  cudaMemcpyAsync(out, e->d_stage, bytes, cudaMemcpyDeviceToHost, e->stream);
  cudaStreamSynchronize(e->stream);
}

void mFitGetFitImage(saFitData* h, double* out) { fit_image_common(h, out, 0); }
void mFitGetResidual(saFitData* h, double* out) { fit_image_common(h, out, 1); }

int saGetFitImageNoAlloc(saFitData* h, int frame, double* out, int residual) {
  Engine* e = E(h);
  if (!e) return -1;
  if ((size_t)e->npix > kNoAllocPixels) {
    set_error("saGetFitImageNoAlloc: %lld pixels exceed the scratch capacity of %zu",
              (long long)e->npix, kNoAllocPixels);
    return -1;
  }
  if (!e->d_x || frame < 0 || frame >= e->F) {
    set_error("saGetFitImageNoAlloc: no image or frame %d out of range", frame);
    return -1;
  }
  double* scratch = e->noalloc;
  if (!scratch) {
    set_error("saGetFitImageNoAlloc: the device scratch was not found when the handle was created");
    return -1;
  }
  // The kernel writes every element that is copied out: nothing in the
  // scratch has to start at zero.
  cudaError_t err = (e->prec == 32)
                        ? Launch<float>::fit_image(e->fs<float>(), frame, scratch, residual, e->stream)
                        : Launch<double>::fit_image(e->fs<double>(), frame, scratch, residual, e->stream);
  if (err != cudaSuccess) {
    set_error("saGetFitImageNoAlloc: %s", cudaGetErrorString(err));
    return -1;
  }
  e->launches += 1;
  CK(cudaMemcpyAsync(out, scratch, (size_t)e->npix * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  return 0;
}

void mFitSetPeakStatus(saFitData* h, int32_t* status) {
  Engine* e = E(h);
  if (!e || !e->d_pk) return;
  const int n = e->nfit[0];
  if (n == 0) return;
  std::vector<int> slots(n), frames(n, 0);
  for (int i = 0; i < n; i++) slots[i] = e->pk_off[0] + i;
  const size_t ib = (size_t)n * sizeof(int);
  if (e->stage(3 * ib)) return;
  int* d_slots = (int*)e->d_stage;
  int* d_frames = d_slots + n;
  int* d_status = d_frames + n;
  cudaMemcpyAsync(d_slots, slots.data(), ib, cudaMemcpyHostToDevice, e->stream);
  cudaMemcpyAsync(d_frames, frames.data(), ib, cudaMemcpyHostToDevice, e->stream);
  cudaMemcpyAsync(d_status, status, ib, cudaMemcpyHostToDevice, e->stream);
  cudaError_t err = (e->prec == 32)
                        ? Launch<float>::set_status(e->cfg, e->fs<float>(), d_slots, d_frames, d_status, n, e->warp_smem, e->stream)
                        : Launch<double>::set_status(e->cfg, e->fs<double>(), d_slots, d_frames, d_status, n, e->warp_smem, e->stream);
  if (err != cudaSuccess) set_error("set status: %s", cudaGetErrorString(err));
  cudaStreamSynchronize(e->stream);
  e->host_valid = false;
  e->unconv_cache = -1;
}

static void remove_peaks(saFitData* h, int drop_status) {
  Engine* e = E(h);
  if (!e || !e->d_pk) return;
  if (e->pull_records()) return;
  std::vector<PeakRec> keep;
  keep.reserve(e->host_pk.size());
  for (const PeakRec& r : e->host_pk) {
    if (r.status != drop_status) keep.push_back(r);
    else if (drop_status == RUNNING) h->n_non_converged++;   // multi_fit.c:1775
  }
  e->host_pk = keep;
  e->push_records();
  h->nfit = e->nfit[0];
}

void mFitRemoveErrorPeaks(saFitData* h) { remove_peaks(h, ERROR); }
void mFitRemoveRunningPeaks(saFitData* h) { remove_peaks(h, RUNNING); }

int saSolveDamped(const double* a, const double* b, int n_sys, int k, double lam, int engine, double* x,
                  int32_t* info) {
  if (n_sys < 0 || k < 1 || k > MAX_JAC || engine < 0 || engine > 2 || (engine == 1 && (k < 4 || k > 6))) {
    set_error("saSolveDamped: unsupported n_sys %d, k %d, engine %d", n_sys, k, engine);
    return -1;
  }
  if (n_sys == 0) return 0;
  const size_t na = (size_t)n_sys * k * k, nb = (size_t)n_sys * k;
  double *da = nullptr, *db = nullptr, *dx = nullptr;
  int* di = nullptr;
  cudaError_t err = cudaMalloc(&da, na * sizeof(double));
  if (err == cudaSuccess) err = cudaMalloc(&db, nb * sizeof(double));
  if (err == cudaSuccess) err = cudaMalloc(&dx, nb * sizeof(double));
  if (err == cudaSuccess) err = cudaMalloc(&di, (size_t)n_sys * sizeof(int));
  if (err == cudaSuccess) err = cudaMemcpy(da, a, na * sizeof(double), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemcpy(db, b, nb * sizeof(double), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = solve_batch(da, db, n_sys, k, lam, engine, dx, di, 0);
  if (err == cudaSuccess) err = cudaMemcpy(x, dx, nb * sizeof(double), cudaMemcpyDeviceToHost);
  if (err == cudaSuccess) err = cudaMemcpy(info, di, (size_t)n_sys * sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(da);
  cudaFree(db);
  cudaFree(dx);
  cudaFree(di);
  if (err != cudaSuccess) {
    set_error("saSolveDamped: %s", cudaGetErrorString(err));
    return -1;
  }
  return 0;
}

int saSetPrecision(saFitData* h, int bits) {
  Engine* e = E(h);
  if (!e) return -1;
  if (bits != 32 && bits != 64) {
    set_error("precision must be 32 or 64");
    return -1;
  }
  if (e->configured && e->prec != bits) {
    set_error("precision must be set before the first image");
    return -1;
  }
  e->prec = bits;
  return 0;
}

int saSetDilation(saFitData* h, int pixels) {
  Engine* e = E(h);
  if (!e) return -1;
  if (e->configured || pixels < 0 || pixels > 16) {
    set_error("dilation must be 0..16 and set before the first image");
    return -1;
  }
  e->cfg.dil = pixels;
  if (e->model_set) finish_geometry(e);
  return 0;
}

int saSetSchedule(saFitData* h, int dil_late, int dil_switch) {
  Engine* e = E(h);
  if (!e) return -1;
  const int dil = e->cfg.dil < 0 ? 3 : e->cfg.dil;
  if (dil_late < 0 || dil_late > dil || dil_switch < 0) {
    set_error("saSetSchedule: late dilation must be 0..%d and the switch sweep >= 0", dil);
    return -1;
  }
  e->cfg.dil_late = dil_late;
  e->cfg.dil_switch = dil_switch;
  return 0;
}

int saGetSweepGrid(saFitData* h) {
  Engine* e = E(h);
  if (!e || !e->configured) return -1;
  return e->sweep_grid;
}

int saSetTailPeaks(saFitData* h, int peaks) {
  Engine* e = E(h);
  if (!e || peaks < 0) return -1;
  e->tail_peaks = peaks;
  return 0;
}

int saSetSweepCTAs(saFitData* h, int ctas) {
  Engine* e = E(h);
  if (!e || ctas < 0) return -1;
  e->sweep_ctas_cap = ctas;
  return 0;
}

int saSetStream(saFitData* h, void* stream) {
  Engine* e = E(h);
  if (!e) return -1;
  e->stream = (cudaStream_t)stream;
  return 0;
}

int saGetCounters(saFitData* h, int64_t* out) {
  Engine* e = E(h);
  if (!e || !e->d_ctl) {
    for (int i = 0; i < NCOUNTERS; i++) out[i] = 0;
    return 0;
  }
  long long tot[NCOUNTERS];
  if (e->read_counters(tot)) return -1;
  for (int i = 0; i < NCOUNTERS; i++) out[i] = tot[i];
  return 0;
}

int saGetSchedStats(saFitData* h, int64_t* out2) {
  Engine* e = E(h);
  if (!e || !e->d_ctl) {
    out2[0] = out2[1] = 0;
    return 0;
  }
  std::vector<FrameCtl> ctl(e->F);
  CK(cudaMemcpy(ctl.data(), e->d_ctl, sizeof(FrameCtl) * e->F, cudaMemcpyDeviceToHost));
  long long reruns = 0, barriers = 0;
  for (const FrameCtl& c : ctl) {
    reruns += c.reruns_total;
    barriers += c.barriers_total;
  }
  out2[0] = reruns;
  out2[1] = barriers;
  return 0;
}

int saSetFrames(saFitData* h, int n_frames, int cap) {
  Engine* e = E(h);
  if (!e) return -1;
  if (n_frames <= 0) {
    set_error("n_frames must be positive");
    return -1;
  }
  if (e->set_frames(n_frames)) return -1;
  std::vector<int> caps(n_frames, std::max(cap, 1));
  if (e->set_peak_caps(caps)) return -1;
  h->nfit = 0;
  h->max_nfit = caps[0];
  return 0;
}

int saNewImages(saFitData* h, const void* images, int n_frames, int bits, int on_device) {
  Engine* e = E(h);
  if (!e) return -1;
  if (n_frames != e->F) {
    set_error("saNewImages: %d frames given, frame set holds %d", n_frames, e->F);
    return -1;
  }
  if (bits != 16 && bits != 32 && bits != 64) {
    set_error("saNewImages: dtype bits must be 16, 32 or 64");
    return -1;
  }
  const void* src = images;
  if (!on_device) {
    const size_t bytes = (size_t)e->npix * n_frames * (bits / 8);
    if (e->stage(bytes)) return -1;
    CK(cudaMemcpyAsync(e->d_stage, images, bytes, cudaMemcpyHostToDevice, e->stream));
    src = e->d_stage;
  }
  if (e->prec == 32) CK(Launch<float>::new_image(e->fs<float>(), src, bits, 0, n_frames, e->stream));
  else CK(Launch<double>::new_image(e->fs<double>(), src, bits, 0, n_frames, e->stream));
  e->launches += 1;
  std::fill(e->nfit.begin(), e->nfit.end(), 0);
  if (e->sync_nfit()) return -1;
  e->host_pk.clear();
  e->host_valid = true;
  e->unconv_cache = -1;
  h->nfit = 0;
  return 0;
}

int saNewBackgrounds(saFitData* h, const void* bgs, int n_frames, int bits, int on_device) {
  Engine* e = E(h);
  if (!e) return -1;
  if (n_frames != e->F || (bits != 32 && bits != 64)) {
    set_error("saNewBackgrounds: bad frame count or dtype");
    return -1;
  }
  const void* src = bgs;
  if (!on_device) {
    const size_t bytes = (size_t)e->npix * n_frames * (bits / 8);
    if (e->stage(bytes)) return -1;
    CK(cudaMemcpyAsync(e->d_stage, bgs, bytes, cudaMemcpyHostToDevice, e->stream));
    src = e->d_stage;
  }
  if (e->prec == 32) CK(Launch<float>::new_background(e->fs<float>(), src, bits, 0, n_frames, e->stream));
  else CK(Launch<double>::new_background(e->fs<double>(), src, bits, 0, n_frames, e->stream));
  e->launches += 1;
  CK(cudaStreamSynchronize(e->stream));
  return 0;
}

static int new_peaks_batch(saFitData* h, const double* peaks, const int32_t* counts, int n_frames,
                           const char* p_type, bool on_device) {
  Engine* e = E(h);
  if (!e) return -1;
  const int pt = parse_ptype(p_type);
  if (pt < 0) {
    set_error("Unrecognized peak type '%s'!", p_type ? p_type : "(null)");
    return -1;
  }
  if (n_frames != e->F || !e->d_pk) {
    set_error("saNewPeaksBatch: frame set not prepared (saSetFrames)");
    return -1;
  }
  std::vector<int> cnt(counts, counts + n_frames);
  for (int f = 0; f < n_frames; f++) {
    if (e->nfit[f] + cnt[f] > e->cap_f[f]) {
      set_error("saNewPeaksBatch: frame %d needs %d peaks, capacity %d", f, e->nfit[f] + cnt[f], e->cap_f[f]);
      return -1;
    }
  }
  if (insert_peaks(e, peaks, cnt, pt, on_device)) return -1;
  h->nfit = e->nfit[0];
  return 0;
}

int saNewPeaksBatch(saFitData* h, const double* peaks, const int32_t* counts, int n_frames,
                    const char* p_type) {
  return new_peaks_batch(h, peaks, counts, n_frames, p_type, false);
}

int saNewPeaksBatchDevice(saFitData* h, const double* d_peaks, const int32_t* counts, int n_frames,
                          const char* p_type) {
  return new_peaks_batch(h, d_peaks, counts, n_frames, p_type, true);
}

int saDoFitBatch(saFitData* h, int max_iterations) {
  Engine* e = E(h);
  if (!e) return -1;
  int sw = 0;
  if (e->fit(max_iterations + 1, &sw)) return -1;
  sync_counters(h);
  return sw;
}

int saDoFitBatchFrames(saFitData* h, int max_iterations, const int32_t* active) {
  Engine* e = E(h);
  if (!e || !active) return -1;
  int sw = 0;
  if (e->fit(max_iterations + 1, &sw, active)) return -1;
  sync_counters(h);
  return sw;
}

// All frames' peak records to the host (frame-major, nfit[f] each).
static int pull_all(Engine* e, std::vector<std::vector<PeakRec>>& out) {
  out.assign(e->F, {});
  for (int f = 0; f < e->F; f++) {
    out[f].resize(e->nfit[f]);
    if (e->nfit[f] > 0)
      CK(cudaMemcpy(out[f].data(), e->d_pk + e->pk_off[f], sizeof(PeakRec) * e->nfit[f], cudaMemcpyDeviceToHost));
  }
  return 0;
}

static int push_all(Engine* e, const std::vector<std::vector<PeakRec>>& in) {
  for (int f = 0; f < e->F; f++) {
    if (!in[f].empty())
      CK(cudaMemcpy(e->d_pk + e->pk_off[f], in[f].data(), sizeof(PeakRec) * in[f].size(), cudaMemcpyHostToDevice));
    e->nfit[f] = (int)in[f].size();
  }
  if (e->sync_nfit()) return -1;
  CK(cudaStreamSynchronize(e->stream));
  e->host_valid = false;
  e->unconv_cache = -1;
  return 0;
}

int saSetPeakStatusBatch(saFitData* h, const int32_t* status) {
  Engine* e = E(h);
  if (!e || !e->d_pk || !status) return -1;
  std::vector<int> slots, frames;
  for (int f = 0; f < e->F; f++)
    for (int i = 0; i < e->nfit[f]; i++) {
      slots.push_back(e->pk_off[f] + i);
      frames.push_back(f);
    }
  const int n = (int)slots.size();
  if (n == 0) return 0;
  const size_t ib = (size_t)n * sizeof(int);
  if (e->stage(3 * ib)) return -1;
  int* d_slots = (int*)e->d_stage;
  int* d_frames = d_slots + n;
  int* d_status = d_frames + n;
  CK(cudaMemcpyAsync(d_slots, slots.data(), ib, cudaMemcpyHostToDevice, e->stream));
  CK(cudaMemcpyAsync(d_frames, frames.data(), ib, cudaMemcpyHostToDevice, e->stream));
  CK(cudaMemcpyAsync(d_status, status, ib, cudaMemcpyHostToDevice, e->stream));
  CK((e->prec == 32)
         ? Launch<float>::set_status(e->cfg, e->fs<float>(), d_slots, d_frames, d_status, n, e->warp_smem, e->stream)
         : Launch<double>::set_status(e->cfg, e->fs<double>(), d_slots, d_frames, d_status, n, e->warp_smem,
                                      e->stream));
  e->launches += 1;
  CK(cudaStreamSynchronize(e->stream));
  e->host_valid = false;
  e->unconv_cache = -1;
  return 0;
}

int saRemovePeaksBatch(saFitData* h, int status) {
  Engine* e = E(h);
  if (!e || !e->d_pk) return -1;
  std::vector<std::vector<PeakRec>> recs;
  if (pull_all(e, recs)) return -1;
  for (auto& v : recs) {
    std::vector<PeakRec> keep;
    keep.reserve(v.size());
    for (const PeakRec& r : v) {
      if (r.status != status) keep.push_back(r);
      else if (status == RUNNING) h->n_non_converged++;
    }
    v.swap(keep);
  }
  if (push_all(e, recs)) return -1;
  h->nfit = e->nfit[0];
  return 0;
}

int saReservePeaksBatch(saFitData* h, int capacity_per_frame) {
  Engine* e = E(h);
  if (!e || e->F < 1) return -1;
  bool need = !e->d_pk;
  for (int f = 0; f < e->F && !need; f++) need = e->cap_f[f] < capacity_per_frame;
  if (!need) return 0;
  std::vector<std::vector<PeakRec>> recs;
  if (e->d_pk && pull_all(e, recs)) return -1;
  std::vector<int> caps(e->F);
  for (int f = 0; f < e->F; f++) caps[f] = std::max(capacity_per_frame, e->d_pk ? e->cap_f[f] : 0);
  if (e->set_peak_caps(caps)) return -1;
  if (!recs.empty() && push_all(e, recs)) return -1;
  h->max_nfit = e->cap_f[0];
  return 0;
}

int saGetFitImagesDevice(saFitData* h, double* d_out, int residual) {
  Engine* e = E(h);
  if (!e || !d_out || !e->d_x) return -1;
  for (int f = 0; f < e->F; f++) {
    CK((e->prec == 32) ? Launch<float>::fit_image(e->fs<float>(), f, d_out + (size_t)f * e->npix, residual, e->stream)
                       : Launch<double>::fit_image(e->fs<double>(), f, d_out + (size_t)f * e->npix, residual,
                                                   e->stream));
    e->launches += 1;
  }
  CK(cudaStreamSynchronize(e->stream));
  return 0;
}

int saGetNFitBatch(saFitData* h, int32_t* counts) {
  Engine* e = E(h);
  if (!e) return -1;
  for (int f = 0; f < e->F; f++) counts[f] = e->nfit[f];
  return 0;
}

int saGetPeakPropertyBatch(saFitData* h, double* values, const char* what) {
  Engine* e = E(h);
  if (!e || !e->d_pk) return -1;
  return get_double_props(e, 0, e->F, values, what);
}

int saGetPeakPropertyIntBatch(saFitData* h, int32_t* values, const char* what) {
  Engine* e = E(h);
  if (!e || !e->d_pk) return -1;
  const bool it = !strcmp(what, "iterations");
  if (!it && strcmp(what, "status")) {
    set_error("Unrecognized parameter '%s'!", what);
    return -1;
  }
  size_t o = 0;
  for (int f = 0; f < e->F; f++) {
    std::vector<PeakRec> recs(e->nfit[f]);
    if (e->nfit[f] > 0)
      CK(cudaMemcpy(recs.data(), e->d_pk + e->pk_off[f], sizeof(PeakRec) * e->nfit[f], cudaMemcpyDeviceToHost));
    for (const PeakRec& r : recs) values[o++] = it ? r.iterations : r.status;
  }
  return 0;
}

int saSetDevice(int device) {
  CK(cudaSetDevice(device));
  return 0;
}

int saGetResultsBatch(saFitData* h, double* values, int32_t* ints) {
  Engine* e = E(h);
  if (!e || !e->d_pk) return -1;
  int n = 0;
  for (int f = 0; f < e->F; f++) n += e->nfit[f];
  if (n == 0) return 0;
  // one device-to-host copy of the records of all frames
  const size_t rb = (size_t)e->cap_total * sizeof(PeakRec);
  std::vector<PeakRec> recs(e->cap_total);
  CK(cudaMemcpyAsync(recs.data(), e->d_pk, rb, cudaMemcpyDeviceToHost, e->stream));
  CK(cudaStreamSynchronize(e->stream));
  const char* names[8] = {"x", "y", "z", "height", "background", "xsigma", "ysigma", "error"};
  size_t o = 0;
  for (int f = 0; f < e->F; f++) {
    for (int j = 0; j < e->nfit[f]; j++, o++) {
      const PeakRec& r = recs[(size_t)e->pk_off[f] + j];
      for (int q = 0; q < 8; q++) record_prop(e, r, names[q], values + o * 8 + q);
      ints[o * 2] = r.status;
      ints[o * 2 + 1] = r.iterations;
    }
  }
  return n;
}

int saSetTiming(saFitData* h, int on) {
  Engine* e = E(h);
  if (!e) return -1;
  e->drain_timing();
  e->timing = on != 0;
  e->sweep_ms = 0.0;
  e->sweep_times.clear();
  e->sweep_launches = 0;
  e->ticks = 0;
  return 0;
}

int saGetTiming(saFitData* h, double* total_ms, int64_t* launches, int64_t* ticks) {
  Engine* e = E(h);
  if (!e) return -1;
  if (e->drain_timing()) return -1;
  *total_ms = e->sweep_ms;
  *launches = e->sweep_launches;
  *ticks = e->ticks;
  return 0;
}

int saGetSweepTimes(saFitData* h, float* out, int max_n) {
  Engine* e = E(h);
  if (!e) return -1;
  if (e->drain_timing()) return -1;
  const int n = (int)std::min<size_t>(e->sweep_times.size(), (size_t)max_n);
  for (int i = 0; i < n; i++) out[i] = e->sweep_times[i];
  return n;
}

int64_t saGetKernelLaunches(saFitData* h) {
  Engine* e = E(h);
  return e ? e->launches : -1;
}

// ---- serving slots ---------------------------------------------------------

int saSlotLoad(saFitData* h, int slot, const void* image, const void* background, int bits,
               const double* peaks, int n_peaks, const char* p_type, int max_iterations) {
  Engine* e = E(h);
  if (!e) return -1;
  if (!e->d_pk || slot < 0 || slot >= e->F) {
    set_error("saSlotLoad: slot %d is not in the frame set (saSetFrames first)", slot);
    return -1;
  }
  if (bits != 32 && bits != 64) {
    set_error("saSlotLoad: dtype bits must be 32 or 64");
    return -1;
  }
  const int pt = parse_ptype(p_type);
  if (pt < 0) {
    set_error("Unrecognized peak type '%s'!", p_type ? p_type : "(null)");
    return -1;
  }
  if (n_peaks < 0 || n_peaks > e->cap_f[slot]) {
    set_error("saSlotLoad: %d peaks, slot capacity %d", n_peaks, e->cap_f[slot]);
    return -1;
  }
  // the slot is idle while its frame and peaks are replaced
  FrameCtl c;
  memset(&c, 0, sizeof(c));
  c.phase = PH_IDLE;
  c.escaped_min = INT_MAX;
  CK(cudaMemcpyAsync(e->d_ctl + slot, &c, sizeof(c), cudaMemcpyHostToDevice, e->stream));
  const size_t bytes = (size_t)e->npix * (bits / 8);
  if (e->stage(2 * bytes)) return -1;
  char* st = (char*)e->d_stage;
  CK(cudaMemcpyAsync(st, image, bytes, cudaMemcpyHostToDevice, e->stream));
  CK(cudaMemcpyAsync(st + bytes, background, bytes, cudaMemcpyHostToDevice, e->stream));
  if (e->prec == 32) {
    CK(Launch<float>::new_image(e->fs<float>(), st, bits, slot, 1, e->stream));
    CK(Launch<float>::new_background(e->fs<float>(), st + bytes, bits, slot, 1, e->stream));
  } else {
    CK(Launch<double>::new_image(e->fs<double>(), st, bits, slot, 1, e->stream));
    CK(Launch<double>::new_background(e->fs<double>(), st + bytes, bits, slot, 1, e->stream));
  }
  e->launches += 2;
  CK(cudaStreamSynchronize(e->stream));   // the stage buffer is reused below
  e->nfit[slot] = 0;
  std::vector<int> counts(e->F, 0);
  counts[slot] = n_peaks;
  if (insert_peaks(e, peaks, counts, pt)) return -1;
  c.phase = PH_SWEEP_PENDING;
  c.max_sweeps = max_iterations + 1;   // dao_fit_c.py:340-346
  CK(cudaMemcpyAsync(e->d_ctl + slot, &c, sizeof(c), cudaMemcpyHostToDevice, e->stream));
  return 0;
}

int saSlotLaunch(saFitData* h, int n_ticks) {
  Engine* e = E(h);
  if (!e || !e->d_ctl) return -1;
  if (!e->h_ctl || e->h_ctl_n < e->F) {
    if (e->h_ctl) cudaFreeHost(e->h_ctl);
    e->h_ctl = nullptr;
    CK(cudaMallocHost((void**)&e->h_ctl, sizeof(FrameCtl) * e->F));
    e->h_ctl_n = e->F;
  }
  if (!e->ev_poll) CK(cudaEventCreateWithFlags(&e->ev_poll, cudaEventDisableTiming));
  for (int i = 0; i < n_ticks; i++)
    if (e->tick()) return -1;
  CK(cudaMemcpy2DAsync(e->h_ctl, sizeof(FrameCtl), e->d_ctl, sizeof(FrameCtl), offsetof(FrameCtl, escaped), e->F,
                       cudaMemcpyDeviceToHost, e->stream));
  CK(cudaEventRecord(e->ev_poll, e->stream));
  return 0;
}

int saSlotReady(saFitData* h) {
  Engine* e = E(h);
  if (!e || !e->ev_poll) return -1;
  const cudaError_t q = cudaEventQuery(e->ev_poll);
  if (q == cudaSuccess) return 1;
  if (q == cudaErrorNotReady) return 0;
  set_error("CUDA error: %s", cudaGetErrorString(q));
  return -1;
}

int saSlotPoll(saFitData* h, int32_t* phases, int32_t* sweeps) {
  Engine* e = E(h);
  if (!e || !e->h_ctl || !e->ev_poll) return -1;
  CK(cudaEventSynchronize(e->ev_poll));
  if (e->check_err_flag()) return -1;
  int active = 0;
  for (int f = 0; f < e->F; f++) {
    const int ph = e->h_ctl[f].phase;
    if (phases) phases[f] = ph;
    if (sweeps) sweeps[f] = e->h_ctl[f].sweeps;
    if (ph != PH_DONE && ph != PH_IDLE) active++;
  }
  e->host_valid = false;
  return active;
}

int saSlotResults(saFitData* h, int slot, double* values, int32_t* ints) {
  Engine* e = E(h);
  if (!e || !e->d_pk || slot < 0 || slot >= e->F) return -1;
  const int n = e->nfit[slot];
  if (n == 0) return 0;
  std::vector<PeakRec> recs(n);
  CK(cudaMemcpyAsync(recs.data(), e->d_pk + e->pk_off[slot], sizeof(PeakRec) * n, cudaMemcpyDeviceToHost,
                     e->stream));
  CK(cudaStreamSynchronize(e->stream));
  const char* names[8] = {"x", "y", "z", "height", "background", "xsigma", "ysigma", "error"};
  for (int j = 0; j < n; j++) {
    for (int q = 0; q < 8; q++) record_prop(e, recs[j], names[q], values + (size_t)j * 8 + q);
    ints[j * 2] = recs[j].status;
    ints[j * 2 + 1] = recs[j].iterations;
  }
  return n;
}


// ---- multi-plane fitting (multi_plane/mp_fit.c, mp_fit_arb.c, mp_fit_dao.c;
// multi_plane/mp_fit_c.py, mp_fit_arb_c.py, mp_fit_dao_c.py bind them) ----
//
// The channels are ordinary handles of this library (one image plane
// each, FP64 engine); the coupled sweep runs on the device (sa_mp.cuh).

struct MPState {
  int kind = -1;                 // MP_ARB / MP_DAO once a channel is set
  std::vector<double> xt0N, yt0N, xtN0, ytN0;
  std::vector<double> w;         // bg, h, x, y, z weights, each [n_weights][nc]
  double* d_w = nullptr;
  MPChan* d_chans = nullptr;
  int* d_unconv = nullptr;       // RUNNING groups per frame after a batched sweep
  int unconv_n = 0;
  int teams = 0;                 // groups stepping at once per frame (0: chosen from the frame count)
  std::vector<saFitData*> fit;   // the channels (also in saMPFit.fit_data)
};

static MPState* MPS(saMPFit* mp) { return mp ? reinterpret_cast<MPState*>(mp->engine) : nullptr; }

// A channel's own cleanup (a spline channel frees its spline: cfCleanup).
static void mp_channel_cleanup(saFitData* h) {
  Engine* e = E(h);
  if (e && e->spline) cfCleanup(h);
  else daoCleanup(h);
}

// mpInitialize mp_fit.c:146-175.
saMPFit* mpInitialize(double tolerance, int n_channels, int independent_heights, int im_size_x, int im_size_y) {
  if (n_channels < 1 || n_channels > MP_MAXCH) {
    set_error("mpInitialize: %d channels (1..%d)", n_channels, MP_MAXCH);
    return nullptr;
  }
  saMPFit* mp = static_cast<saMPFit*>(calloc(1, sizeof(saMPFit)));
  MPState* st = new MPState();
  mp->engine = st;
  mp->im_size_x = im_size_x;
  mp->im_size_y = im_size_y;
  mp->independent_heights = independent_heights;
  mp->n_channels = n_channels;
  mp->tolerance = tolerance;
  const int n3 = 3 * n_channels;
  st->xt0N.assign(n3, 0.0);
  st->yt0N.assign(n3, 0.0);
  st->xtN0.assign(n3, 0.0);
  st->ytN0.assign(n3, 0.0);
  mp->xt_0toN = st->xt0N.data();
  mp->yt_0toN = st->yt0N.data();
  mp->xt_Nto0 = st->xtN0.data();
  mp->yt_Nto0 = st->ytN0.data();
  st->fit.assign(n_channels, nullptr);
  mp->fit_data = st->fit.data();
  return mp;
}

// A channel handle made by one of the fitters' initialisers: the FP64
// engine, minimum height 1 (mp_fit_arb.c / mp_fit_dao.c set it).
static int mp_attach(saMPFit* mp, saFitData* h, int channel, int kind) {
  MPState* st = MPS(mp);
  if (!h) return -1;
  if (channel < 0 || channel >= mp->n_channels) {
    set_error("channel %d out of range (%d channels)", channel, mp->n_channels);
    mp_channel_cleanup(h);
    return -1;
  }
  if (st->kind >= 0 && st->kind != kind) {
    set_error("multi-plane channels must all be Gaussian or all arbitrary-PSF");
    mp_channel_cleanup(h);
    return -1;
  }
  if (st->fit[channel]) mp_channel_cleanup(st->fit[channel]);
  st->kind = kind;
  Engine* e = E(h);
  e->prec = 64;
  e->cfg.min_height = 1.0;
  h->minimum_height = 1.0;
  st->fit[channel] = h;
  return 0;
}

// mpArbInitializePSFFFTChannel mp_fit_arb.c:36-77.
void mpArbInitializePSFFFTChannel(saMPFit* mp, void* psf_fft, double* rqe, double* variance, int channel) {
  if (!MPS(mp)) return;
  mp_attach(mp, ftFitInitialize(psf_fft, rqe, variance, mp->tolerance, mp->im_size_x, mp->im_size_y), channel,
            MP_ARB);
}

// mpArbInitializePupilFnChannel mp_fit_arb.c:85-128.
void mpArbInitializePupilFnChannel(saMPFit* mp, void* pupil_data, double* rqe, double* variance, double zmin,
                                   double zmax, int channel) {
  if (!MPS(mp)) return;
  saFitData* h = pfitInitialize(pupil_data, rqe, variance, mp->tolerance, mp->im_size_x, mp->im_size_y);
  if (mp_attach(mp, h, channel, MP_ARB) == 0) pfitSetZRange(h, zmin, zmax);
}

// mpArbInitializeSplineChannel mp_fit_arb.c:135-172.
void mpArbInitializeSplineChannel(saMPFit* mp, void* spline, double* rqe, double* variance, int channel) {
  if (!MPS(mp)) return;
  saFitData* h = cfInitialize(spline, rqe, variance, mp->tolerance, mp->im_size_x, mp->im_size_y);
  if (h) cfInitialize3D(h);
  mp_attach(mp, h, channel, MP_ARB);
}

// mpDaoInitialize2DChannel mp_fit_dao.c:28-73.
void mpDaoInitialize2DChannel(saMPFit* mp, double* rqe, double* variance, double width_min, double width_max,
                              int roi_size, int channel) {
  if (!MPS(mp)) return;
  saFitData* h = daoInitialize(rqe, variance, mp->tolerance, mp->im_size_x, mp->im_size_y, roi_size);
  if (h) daoInitialize2D(h, width_min, width_max);
  mp_attach(mp, h, channel, MP_DAO);
}

// mpSetTransforms mp_fit.c:535-548.
void mpSetTransforms(saMPFit* mp, double* xt_0toN, double* yt_0toN, double* xt_Nto0, double* yt_Nto0) {
  MPState* st = MPS(mp);
  if (!st) return;
  for (int i = 0; i < 3 * mp->n_channels; i++) {
    st->xt0N[i] = xt_0toN[i];
    st->yt0N[i] = yt_0toN[i];
    st->xtN0[i] = xt_Nto0[i];
    st->ytN0[i] = yt_Nto0[i];
  }
}

// mpSetWeights mp_fit.c:561-592.
void mpSetWeights(saMPFit* mp, double* w_bg, double* w_h, double* w_x, double* w_y, double* w_z, int z_size) {
  MPState* st = MPS(mp);
  if (!st) return;
  const size_t n = (size_t)mp->n_channels * z_size;
  st->w.assign(5 * n, 0.0);
  const double* src[5] = {w_bg, w_h, w_x, w_y, w_z};
  for (int k = 0; k < 5; k++) std::memcpy(st->w.data() + k * n, src[k], sizeof(double) * n);
  mp->n_weights = z_size;
  mp->w_bg = st->w.data();
  mp->w_h = st->w.data() + n;
  mp->w_x = st->w.data() + 2 * n;
  mp->w_y = st->w.data() + 3 * n;
  mp->w_z = st->w.data() + 4 * n;
  if (st->d_w) {
    cudaFree(st->d_w);
    st->d_w = nullptr;
  }
}

// mpSetWeightsIndexing mp_fit.c:600-604.
void mpSetWeightsIndexing(saMPFit* mp, double z_offset, double z_scale) {
  if (!mp) return;
  mp->w_z_offset = z_offset;
  mp->w_z_scale = z_scale;
}

// How many groups of a frame may step at once (1..8; 0: chosen from the
// frame count, 2..8).  The results do not depend on it.
int mpSetTeams(saMPFit* mp, int teams) {
  MPState* st = MPS(mp);
  if (!st || teams < 0 || teams > MP_TEAMS) {
    set_error("mpSetTeams: %d (0..%d)", teams, MP_TEAMS);
    return -1;
  }
  st->teams = teams;
  return 0;
}

// The channel descriptors and parameters of a multi-plane launch; all
// channels must be set, imaged and hold the same number of peaks.
static int mp_prepare(saMPFit* mp, MPParams& p, int& frames, cudaStream_t& stream) {
  MPState* st = MPS(mp);
  if (!st) return -1;
  const int nc = mp->n_channels;
  for (int c = 0; c < nc; c++) {
    if (!st->fit[c] || !E(st->fit[c])->d_x) {
      set_error("multi-plane channel %d is not initialised or has no image", c);
      return -1;
    }
  }
  if (st->w.empty()) {
    set_error("mpSetWeights has not been called");
    return -1;
  }
  Engine* e0 = E(st->fit[0]);
  std::vector<MPChan> chans(nc);
  int ws = 0;
  for (int c = 0; c < nc; c++) {
    Engine* e = E(st->fit[c]);
    if (e->F != e0->F || e->npix != e0->npix) {
      set_error("multi-plane channels must have the same frames");
      return -1;
    }
    chans[c].cfg = e->cfg;
    chans[c].fs = e->fs<double>();
    ws = std::max(ws, mp_ws_bytes(e->cfg));
    CK(cudaStreamSynchronize(e->stream));
  }
  if (!st->d_chans) CK(cudaMalloc(&st->d_chans, sizeof(MPChan) * MP_MAXCH));
  CK(cudaMemcpy(st->d_chans, chans.data(), sizeof(MPChan) * nc, cudaMemcpyHostToDevice));
  if (!st->d_w) {
    CK(cudaMalloc(&st->d_w, sizeof(double) * st->w.size()));
    CK(cudaMemcpy(st->d_w, st->w.data(), sizeof(double) * st->w.size(), cudaMemcpyHostToDevice));
  }
  std::memset(&p, 0, sizeof(p));
  p.nc = nc;
  p.indep = mp->independent_heights;
  p.kind = st->kind;
  p.n_weights = mp->n_weights;
  p.tol = mp->tolerance;
  p.w_z_offset = mp->w_z_offset;
  p.w_z_scale = mp->w_z_scale;
  for (int i = 0; i < 3 * nc; i++) {
    p.xt0N[i] = st->xt0N[i];
    p.yt0N[i] = st->yt0N[i];
    p.xtN0[i] = st->xtN0[i];
    p.ytN0[i] = st->ytN0[i];
  }
  p.w = st->d_w;
  p.ws_bytes = ws;
  for (int c = 0; c < nc; c++) p.grid_doubles = std::max(p.grid_doubles, E(st->fit[c])->cfg.roi * E(st->fit[c])->cfg.roi);
  p.teams = st->teams;
  frames = e0->F;
  stream = e0->stream;
  return 0;
}

// After a multi-plane kernel: the channels' host copies are stale.
static int mp_finish(saMPFit* mp, cudaStream_t stream) {
  MPState* st = MPS(mp);
  CK(cudaStreamSynchronize(stream));
  for (int c = 0; c < mp->n_channels; c++) {
    Engine* e = E(st->fit[c]);
    e->host_valid = false;
    e->unconv_cache = -1;
    sync_counters(st->fit[c]);
  }
  return 0;
}

// mpArbNewPeaks mp_fit_arb.c:180-340, mpDaoNewPeaks mp_fit_dao.c:82-152.
static void mp_new_peaks(saMPFit* mp, double* peaks, char* p_type, int n, bool arb) {
  MPState* st = MPS(mp);
  if (!st) return;
  const int pt = parse_ptype(p_type);
  if (pt < 0) {
    set_error("Unrecognized peak type '%s'!", p_type ? p_type : "(null)");
    return;
  }
  for (int c = 0; c < mp->n_channels; c++) {
    if (!st->fit[c]) {
      set_error("multi-plane channel %d is not initialised", c);
      return;
    }
  }
  const int start = st->fit[0]->nfit;
  const int ncol = (pt == PT_TEXT) ? (arb ? 5 : 7) : (arb ? 3 : 4);
  std::vector<double> mapped((size_t)ncol * std::max(n, 1));
  for (int c = 0; c < mp->n_channels; c++) {
    double* rows = peaks;
    if (c > 0) {
      for (int j = 0; j < n; j++) {
        const double* q = peaks + (size_t)ncol * j;
        double* o = mapped.data() + (size_t)ncol * j;
        const double tx = q[0], ty = q[1];
        for (int k = 0; k < ncol; k++) o[k] = q[k];
        o[0] = st->xt0N[c * 3] + tx * st->xt0N[c * 3 + 1] + ty * st->xt0N[c * 3 + 2];
        o[1] = st->yt0N[c * 3] + tx * st->yt0N[c * 3 + 1] + ty * st->yt0N[c * 3 + 2];
      }
      rows = mapped.data();
    }
    if (new_peaks_single(st->fit[c], rows, p_type, n)) return;
  }
  MPParams p;
  int frames = 0;
  cudaStream_t stream = nullptr;
  if (mp_prepare(mp, p, frames, stream)) return;
  p.start = start;
  p.stop = start + n;
  p.fix_heights = (arb && !mp->independent_heights && pt != PT_TEXT) ? 1 : 0;
  cudaError_t err = mp_newpeaks(st->d_chans, p, 1, stream);
  if (err != cudaSuccess) {
    set_error("multi-plane new peaks: %s", cudaGetErrorString(err));
    return;
  }
  mp_finish(mp, stream);
}

void mpArbNewPeaks(saMPFit* mp, double* peaks, char* p_type, int n_peaks) {
  mp_new_peaks(mp, peaks, p_type, n_peaks, true);
}

void mpDaoNewPeaks(saMPFit* mp, double* peaks, char* p_type, int n_peaks) {
  mp_new_peaks(mp, peaks, p_type, n_peaks, false);
}

// mpIterateLM mp_fit.c:183-478: one coupled sweep on the device.
void mpIterateLM(saMPFit* mp) {
  MPState* st = MPS(mp);
  if (!st) return;
  MPParams p;
  int frames = 0;
  cudaStream_t stream = nullptr;
  if (mp_prepare(mp, p, frames, stream)) return;
  for (int c = 1; c < mp->n_channels; c++) {
    if (st->fit[c]->nfit != st->fit[0]->nfit) {
      set_error("multi-plane channels hold different numbers of peaks");
      return;
    }
  }
  cudaError_t err = mp_sweep(st->d_chans, p, 1, stream);
  if (err != cudaSuccess) {
    set_error("mpIterateLM: %s", cudaGetErrorString(err));
    return;
  }
  mp_finish(mp, stream);
}

// mpCleanup mp_fit.c:76-115 (each channel's fitter cleanup).
void mpCleanup(saMPFit* mp) {
  MPState* st = MPS(mp);
  if (!st) return;
  for (saFitData* h : st->fit)
    if (h) mp_channel_cleanup(h);
  if (st->d_w) cudaFree(st->d_w);
  if (st->d_chans) cudaFree(st->d_chans);
  if (st->d_unconv) cudaFree(st->d_unconv);
  delete st;
  free(mp);
}

// ---- batched multi-plane fitting (no reference counterpart): many frames
// per channel handle, one warp per frame.  The channels' frames are set with
// mpSetFrames, their images with saNewImages / saNewBackgrounds on each
// fit_data[i]; the results are read per channel with saGetResultsBatch /
// saGetPeakPropertyBatch.

// saSetFrames on every channel.
int mpSetFrames(saMPFit* mp, int n_frames, int peaks_capacity) {
  MPState* st = MPS(mp);
  if (!st) return -1;
  for (int c = 0; c < mp->n_channels; c++) {
    if (!st->fit[c]) {
      set_error("multi-plane channel %d is not initialised", c);
      return -1;
    }
    if (saSetFrames(st->fit[c], n_frames, peaks_capacity)) return -1;
  }
  return 0;
}

// New peaks of every frame (counts[f] rows of the peak format in channel
// 0's coordinates, frames one after another) into frames whose images
// were just loaded: mapped into every plane, each channel's new-peak pass,
// then mpArbNewPeaks' / mpDaoNewPeaks' height and error synchronisation
// per frame.
int mpNewPeaksBatch(saMPFit* mp, const double* peaks, const int32_t* counts, const char* p_type) {
  MPState* st = MPS(mp);
  if (!st) return -1;
  const int pt = parse_ptype(p_type);
  if (pt < 0 || st->kind < 0) {
    set_error("mpNewPeaksBatch: unknown peak type or no channels");
    return -1;
  }
  const bool arb = st->kind == MP_ARB;
  const int F = E(st->fit[0])->F;
  long long total = 0;
  for (int f = 0; f < F; f++) total += counts[f];
  const int ncol = (pt == PT_TEXT) ? (arb ? 5 : 7) : (arb ? 3 : 4);
  std::vector<double> mapped((size_t)ncol * std::max<long long>(total, 1));
  for (int c = 0; c < mp->n_channels; c++) {
    const double* rows = peaks;
    if (c > 0) {
      for (long long j = 0; j < total; j++) {
        const double* q = peaks + (size_t)ncol * j;
        double* o = mapped.data() + (size_t)ncol * j;
        const double tx = q[0], ty = q[1];
        for (int k = 0; k < ncol; k++) o[k] = q[k];
        o[0] = st->xt0N[c * 3] + tx * st->xt0N[c * 3 + 1] + ty * st->xt0N[c * 3 + 2];
        o[1] = st->yt0N[c * 3] + tx * st->yt0N[c * 3 + 1] + ty * st->yt0N[c * 3 + 2];
      }
      rows = mapped.data();
    }
    if (saNewPeaksBatch(st->fit[c], rows, counts, F, p_type)) return -1;
  }
  MPParams p;
  int frames = 0;
  cudaStream_t stream = nullptr;
  if (mp_prepare(mp, p, frames, stream)) return -1;
  p.start = 0;
  p.stop = -1;
  p.fix_heights = (arb && !mp->independent_heights && pt != PT_TEXT) ? 1 : 0;
  cudaError_t err = mp_newpeaks(st->d_chans, p, frames, stream);
  if (err != cudaSuccess) {
    set_error("mpNewPeaksBatch: %s", cudaGetErrorString(err));
    return -1;
  }
  return mp_finish(mp, stream);
}

// MultiFitter.doFit (dao_fit_c.py:332-356) for every frame at once: one
// coupled sweep, then sweeps while any frame has RUNNING groups and fewer
// than max_iterations were made (a frame without RUNNING groups is left
// unchanged by a sweep).  Returns the number of sweeps, or -1.
int mpDoFitBatch(saMPFit* mp, int max_iterations) {
  MPState* st = MPS(mp);
  if (!st) return -1;
  MPParams p;
  int frames = 0;
  cudaStream_t stream = nullptr;
  if (mp_prepare(mp, p, frames, stream)) return -1;
  if (st->unconv_n < frames) {
    if (st->d_unconv) cudaFree(st->d_unconv);
    CK(cudaMalloc(&st->d_unconv, sizeof(int) * frames));
    st->unconv_n = frames;
  }
  p.unconv = st->d_unconv;
  std::vector<int> un(frames);
  int sweeps = 0;
  for (;;) {
    cudaError_t err = mp_sweep(st->d_chans, p, frames, stream);
    if (err != cudaSuccess) {
      set_error("mpDoFitBatch: %s", cudaGetErrorString(err));
      return -1;
    }
    sweeps++;
    CK(cudaMemcpyAsync(un.data(), st->d_unconv, sizeof(int) * frames, cudaMemcpyDeviceToHost, stream));
    CK(cudaStreamSynchronize(stream));
    long long running = 0;
    for (int f = 0; f < frames; f++) running += un[f];
    if (running == 0 || sweeps > max_iterations) break;
  }
  if (mp_finish(mp, stream)) return -1;
  return sweeps;
}

}  // extern "C"
