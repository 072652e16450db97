// sa_device.cuh -- device building blocks: memory-model helpers, warp
// reductions, the FP64 Cholesky solve, the MLE deviance and the PSF models.
#pragma once

#include <climits>
#include "sa_common.cuh"

namespace sa {

// ---------------------------------------------------------------------------
// memory model helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Polling load: no ordering, and unlike an acquire load it does not
// invalidate the SM's L1 on every poll.  A wait polls with it and acquires
// once, when it has seen what it waits for.
__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Sleep between polls: 32 ns doubling to 512 ns.  A waiter wakes at most
// about half a microsecond after its predecessor is done (an LM step takes
// tens of microseconds), and sleeping waiters leave the issue slots to the
// warps that are stepping.
__device__ __forceinline__ void poll_backoff(unsigned& ns) {
  __nanosleep(ns);
  if (ns < 512) ns <<= 1;
}

constexpr unsigned long long WAIT_LIMIT_NS = 4000000000ull;

// Wait (all lanes, warp-uniform) until done[idx] == epoch, with an acquire
// load at the end.  Bounded: after ~4 s the wait gives up, raises bit 0 of
// err_flag and returns false.
__device__ __forceinline__ bool wait_epoch(const int* done, int epoch, unsigned* err_flag) {
  if (ld_acquire(done) == epoch) return true;
  const unsigned long long t0 = global_ns();
  unsigned ns = 32;
  for (unsigned it = 1;; it++) {
    poll_backoff(ns);
    if (ld_relaxed(done) == epoch) return ld_acquire(done) == epoch;
    if ((it & 31) == 0 && global_ns() - t0 > WAIT_LIMIT_NS) {
      atomicOr(err_flag, 1u);
      return false;
    }
  }
}

// The completed prefix of a frame's sweep attempt: every run rank in
// [start, *frontier) is done.  advance_prefix (all lanes, warp-uniform)
// moves it over the done ranks at its end, 32 done flags per round trip
// (one per lane); any warp may move it, so a rank that completes while
// another warp is moving the prefix past it is never missed (that warp, or
// this one, sees its flag).  Before each move every lane fences (its
// relaxed observation of a done flag followed by the fence acquires that
// rank's writes, and the fence releases them again with the move), so a
// waiter that acquires the prefix sees the writes of every rank below it.
// Returns the prefix (a relaxed read: wait_prefix acquires it).
__device__ __forceinline__ int advance_prefix(int* frontier, const int* done, int nrun, int epoch, int lane) {
  int fr = __shfl_sync(0xffffffffu, lane == 0 ? ld_relaxed(frontier) : 0, 0);
  while (fr < nrun) {
    const int q = fr + lane;
    const bool d = (q < nrun) && (ld_relaxed(done + q) == epoch);
    const unsigned m = __ballot_sync(0xffffffffu, d);
    const int k = (~m != 0u) ? (__ffs(~m) - 1) : 32;
    if (k == 0) break;
    __threadfence();
    __syncwarp();
    int seen = 0;
    if (lane == 0) seen = atomicCAS(frontier, fr, fr + k);
    seen = __shfl_sync(0xffffffffu, seen, 0);
    fr = (seen == fr) ? fr + k : seen;
  }
  return fr;
}

// Wait (all lanes, warp-uniform) until the completed prefix reaches target,
// moving it along meanwhile; acquires the prefix at the end.  Bounded like
// wait_epoch.
__device__ __forceinline__ bool wait_prefix(int* frontier, int target, const int* done, int nrun, int epoch,
                                            unsigned* err_flag, int lane) {
  if (advance_prefix(frontier, done, nrun, epoch, lane) < target) {
    const unsigned long long t0 = global_ns();
    unsigned ns = 32;
    for (unsigned it = 1;; it++) {
      poll_backoff(ns);
      if (advance_prefix(frontier, done, nrun, epoch, lane) >= target) break;
      if ((it & 31) == 0 && global_ns() - t0 > WAIT_LIMIT_NS) {
        if (lane == 0) atomicOr(err_flag, 1u);
        return false;
      }
    }
  }
  return ld_acquire(frontier) >= target;
}

// ---------------------------------------------------------------------------
// warp reductions
// ---------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Float-float accumulation (Knuth's TwoSum): hi + lo carries about 48 bits.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float v) {
  const float s = hi + v;
  const float bb = s - hi;
  const float err = (hi - (s - bb)) + (v - bb);
  hi = s;
  lo += err;
}

// Warp sum of FP32 partials in float-float arithmetic, returned as double
// (three FP64 instructions per warp instead of a double reduction).
__device__ __forceinline__ double warp_sum_ff(float v) {
  float hi = v, lo = 0.0f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o);
    const float ol = __shfl_xor_sync(0xffffffffu, lo, o);
    const float s = hi + oh;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (oh - bb);
    hi = s;
    lo = lo + ol + err;
  }
  return (double)hi + (double)lo;
}

// Reduce 32 values held by every lane; afterwards lane l holds the warp
// total of value l.  31 shuffles instead of 32*5.
template <typename T>
__device__ __forceinline__ T warp_transpose_sum32(T (&v)[32], int lane) {
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool up = (lane & h) != 0;
#pragma unroll
    for (int i = 0; i < h; i++) {
      T send = up ? v[i] : v[i + h];
      T keep = up ? v[i + h] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, h);
    }
  }
  return v[0];
}

// ---------------------------------------------------------------------------
// float-float ("ff") arithmetic: a value is hi + lo with |lo| <= ulp(hi)/2,
// about 48 significant bits, from FP32 instructions only (Dekker's and
// Knuth's error-free transformations; Shewchuk 1997, Hida-Li-Bailey 2001).
// Every operation is explicitly rounded so the compiler cannot contract or
// reorder it.
// ---------------------------------------------------------------------------

struct ff {
  float h, l;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return ff{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.h, -a.l}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_add_f(ff a, float b) {
  const ff s = two_sum(a.h, b);
  return fast_two_sum(s.h, __fadd_rn(s.l, a.l));
}

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return fast_two_sum(p, e);
}

// a * b as an unnormalised pair (p, e) with p + e = a * b to ~2^-48.
__device__ __forceinline__ ff ff_mul_raw(ff a, ff b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return ff{p, e};
}

// Cascaded summation: acc += x with the rounding error of the high parts
// kept exactly and the low parts summed in FP32; acc is renormalised by the
// caller (fast_two_sum) once the sum is complete.
__device__ __forceinline__ void ff_acc(ff& acc, ff x) {
  const ff s = two_sum(acc.h, x.h);
  acc.h = s.h;
  acc.l = __fadd_rn(acc.l, __fadd_rn(s.l, x.l));
}

__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  const float p = __fmul_rn(a.h, b);
  const float e = __fmaf_rn(a.h, b, -p);
  return fast_two_sum(p, __fmaf_rn(a.l, b, e));
}

// Hardware reciprocal approximation (rcp.approx, about 1 ulp).  Where its
// result is corrected afterwards (ff_div) or only scales an FP32 term it
// replaces the correctly rounded reciprocal, whose slow-path check makes it
// several times longer on the dependency chain.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// a / b: one correction of the FP32 quotient q1 = a.h / b.h (relative error
// ~1e-14; the correction absorbs the approximate reciprocal's error).
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float inv = rcp_approx(b.h);
  const float q1 = __fmul_rn(a.h, inv);
  const ff r = ff_sub(a, ff_mul_f(b, q1));
  return fast_two_sum(q1, __fmul_rn(r.h, inv));
}

__device__ __forceinline__ ff ff_from_double(double d) {
  const float h = __double2float_rn(d);
  return ff{h, __double2float_rn(d - (double)h)};
}

__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.h + (double)a.l; }

// Fixed-point words (q * 2^-36) to and from FP32 with 32-bit instructions.
// The 64-bit integer <-> float conversions issue on the FP64 pipe, which
// runs at a small fraction of the FP32 rate on this part.  A word splits
// into its signed high word and the low word's bits 31..9 and 8..0; each
// piece converts exactly by the exponent-bias trick (an integer below 2^23
// placed in the mantissa of 2^23, or of 1.5 * 2^23 for a signed one).
// Words beyond the fast range (|q * 2^-36| >= 2^17) take the 64-bit
// conversions.

__device__ __forceinline__ float fx_u23(unsigned u) {   // 0 <= u < 2^23: exact
  return __fsub_rn(__int_as_float(0x4B000000u | u), 8388608.0f);
}

__device__ __forceinline__ float fx_s22(int s) {   // |s| < 2^22: exact
  return __fsub_rn(__int_as_float(0x4B400000 + s), 12582912.0f);
}

// q * 2^-36 = a + b + c exactly; false outside the fast range.
__device__ __forceinline__ bool fx_split(long long q, float& a, float& b, float& c) {
  const int hi = (int)(q >> 32);
  const unsigned lo = (unsigned)q;
  a = __fmul_rn(fx_s22(hi), 0.0625f);                           // hi * 2^-4
  b = __fmul_rn(fx_u23(lo >> 9), 7.450580596923828125e-9f);     // 2^-27
  c = __fmul_rn(fx_u23(lo & 511u), 1.4551915228366852e-11f);    // 2^-36
  return (unsigned)(hi + (1 << 21)) < (1u << 22);
}

// One-word fixed-point value q * 2^-36 as a float-float pair (~2^-48).
__device__ __forceinline__ ff ff_from_fixed(long long q) {
  float a, b, c;
  if (fx_split(q, a, b, c)) {
    // a + b is a multiple of 2^-27 and c < 2^-27: the renormalisation's
    // ordering condition holds
    const ff s = two_sum(a, b);
    return fast_two_sum(s.h, __fadd_rn(s.l, c));
  }
  const float h = __ll2float_rn(q);
  const long long r = q - __float2ll_rn(h);
  return ff{__fmul_rn(h, 1.4551915228366852e-11f), __fmul_rn(__ll2float_rn(r), 1.4551915228366852e-11f)};
}

// y rounded to the nearest integer (ties to even), as __float2ll_rn: y is
// split at a multiple of 2^31 (t, exact) and the remainder y - t (exact,
// |y - t| <= 2^30) rounded on its own.
__device__ __forceinline__ long long fx_round(float y) {
  if (!(fabsf(y) < 6.755399441055744e15f)) return __float2ll_rn(y);   // 1.5 * 2^52 (and NaN)
  const float t = __fsub_rn(__fadd_rn(y, 2.7021597764222976e16f), 2.7021597764222976e16f);   // 1.5 * 2^54
  const int hi = __float_as_int(__fadd_rn(__fmul_rn(t, 4.656612873077393e-10f), 12582912.0f)) - 0x4B400000;
  const int lo = __float2int_rn(__fsub_rn(y, t));
  return (long long)hi * 2147483648LL + (long long)lo;
}

// Float-float value rounded to the one-word fixed-point grid (2^-36).
__device__ __forceinline__ long long fixed_from_ff(ff a) {
  return fx_round(__fmul_rn(a.h, 68719476736.0f)) + fx_round(__fmul_rn(a.l, 68719476736.0f));
}

__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return ff{p, __fmaf_rn(a, b, -p)};
}

// exp(a) of a float-float a in [-87, 40], in FP32 instructions: Cody-Waite
// reduction a = k ln2 + r (ln2 split in three parts, the first with 16
// significant bits so that k * part1 is exact), the Taylor series of
// exp(r / 32) to degree 6 in Horner form, five squarings, and the exact
// scaling by 2^k.  Relative error <= 2.7e-13 for a in [-60, 0] (checked
// against 60-digit arithmetic and against FP64 exp on the GPU); a < -87
// (or NaN) returns 0; a > 40 is taken as 40.
__device__ __forceinline__ ff ff_exp(ff a) {
  if (!(a.h >= -87.0f)) return ff{0.0f, 0.0f};
  if (a.h > 40.0f) a = ff{40.0f, 0.0f};
  const float k = rintf(a.h * 1.44269504088896341f);
  ff r = ff_add_f(a, -k * 0.693145751953125f);
  const ff kc = two_prod(k, 1.428606765330187e-06f);
  r = ff_sub(r, kc);
  r = ff_add_f(r, -k * 5.497923148104107e-14f);
  const ff s{r.h * 0.03125f, r.l * 0.03125f};
  ff e{1.3888889225199819e-03f, -3.3631094437103215e-11f};                          // 1/6!
  e = ff_add(ff_mul(e, s), ff{8.333333767950535e-03f, -4.34617203337595e-10f});     // 1/5!
  e = ff_add(ff_mul(e, s), ff{4.16666679084301e-02f, -1.2417634698280722e-09f});    // 1/4!
  e = ff_add(ff_mul(e, s), ff{0.1666666716337204f, -4.967053879312289e-09f});       // 1/3!
  e = ff_add(ff_mul(e, s), ff{0.5f, 0.0f});
  e = ff_add(ff_mul(e, s), ff{1.0f, 0.0f});
  e = ff_add(ff_mul(e, s), ff{1.0f, 0.0f});
#pragma unroll
  for (int i = 0; i < 5; i++) e = ff_mul(e, e);
  const float scale = __int_as_float(((int)k + 127) << 23);   // 2^k, k in [-126, 58]
  return ff{e.h * scale, e.l * scale};
}

__device__ __forceinline__ ff shfl_xor_ff(ff v, int o) {
  return ff{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)};
}

// Warp total of a float-float value (every lane gets it: ff_add commutes).
__device__ __forceinline__ ff warp_sum_ffv(ff v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = ff_add(v, shfl_xor_ff(v, o));
  return v;
}

// Reduce 8 float-float values held by every lane: afterwards lane L holds
// the warp total of value 4*b4 + 2*b3 + b2 (b = bits of L).  9 additions
// instead of 40.
__device__ __forceinline__ ff warp_reduce8_ff(ff (&v)[8], int lane) {
#pragma unroll
  for (int h = 16, m = 8; h >= 4; h >>= 1, m >>= 1) {
    const bool up = (lane & h) != 0;
#pragma unroll
    for (int i = 0; i < m / 2; i++) {
      const ff send = up ? v[i] : v[i + m / 2];
      const ff keep = up ? v[i + m / 2] : v[i];
      v[i] = ff_add(keep, shfl_xor_ff(send, h));
    }
  }
  v[0] = ff_add(v[0], shfl_xor_ff(v[0], 2));
  v[0] = ff_add(v[0], shfl_xor_ff(v[0], 1));
  return v[0];
}
__device__ __forceinline__ int reduce8_index(int lane) {
  return ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
}

// warp_transpose_sum32 with float-float additions: lane l gets the warp
// total of float value l to ~1e-14 (no rounding beyond the inputs').
__device__ __forceinline__ ff warp_transpose_sum32_ff(float (&v)[32], int lane) {
  ff w[16];
  {
    const bool up = (lane & 16) != 0;
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const float send = up ? v[i] : v[i + 16];
      const float keep = up ? v[i + 16] : v[i];
      w[i] = two_sum(keep, __shfl_xor_sync(0xffffffffu, send, 16));
    }
  }
#pragma unroll
  for (int h = 8; h >= 1; h >>= 1) {
    const bool up = (lane & h) != 0;
#pragma unroll
    for (int i = 0; i < h; i++) {
      const ff send = up ? w[i] : w[i + h];
      const ff keep = up ? w[i + h] : w[i];
      w[i] = ff_add(keep, shfl_xor_ff(send, h));
    }
  }
  return w[0];
}

// ---------------------------------------------------------------------------
// FP64 Cholesky solve of the damped normal equations (replaces LAPACK
// dposv("Lower"), multi_fit.c:1839-1883).  a: k x k, only a[i*k+j] with
// j >= i is read.  Returns 0 on success; nonzero when not positive definite
// or the solution has a NaN (multi_fit.c:1857-1863).  Products, differences
// and divisions are separately rounded, in the unblocked Cholesky order, so
// ill-conditioned systems (a peak started at height 1) give the LAPACK
// result to the last bit as often as possible.
// ---------------------------------------------------------------------------

__device__ inline int chol_solve(const double* a, double* b, int n) {
  double L[MAX_JAC * MAX_JAC];
  for (int j = 0; j < n; j++) {
    double d = a[j * n + j];
    for (int k = 0; k < j; k++) d = __dsub_rn(d, __dmul_rn(L[j * MAX_JAC + k], L[j * MAX_JAC + k]));
    if (!(d > 0.0)) return j + 1;
    d = sqrt(d);
    L[j * MAX_JAC + j] = d;
    for (int i = j + 1; i < n; i++) {
      double s = a[j * n + i];
      for (int k = 0; k < j; k++) s = __dsub_rn(s, __dmul_rn(L[i * MAX_JAC + k], L[j * MAX_JAC + k]));
      L[i * MAX_JAC + j] = s / d;
    }
  }
  for (int i = 0; i < n; i++) {
    double s = b[i];
    for (int k = 0; k < i; k++) s = __dsub_rn(s, __dmul_rn(L[i * MAX_JAC + k], b[k]));
    b[i] = s / L[i * MAX_JAC + i];
  }
  for (int i = n - 1; i >= 0; i--) {
    double s = b[i];
    for (int k = i + 1; k < n; k++) s = __dsub_rn(s, __dmul_rn(L[k * MAX_JAC + i], b[k]));
    b[i] = s / L[i * MAX_JAC + i];
  }
  for (int i = 0; i < n; i++)
    if (isnan(b[i])) return 1;
  return 0;
}

// Packed upper-triangle index of (r, c) with r <= c after the k gradient
// entries: the layout of the normal equations in the warp workspace.
__device__ __forceinline__ int hes_index(int k, int r, int c) {
  if (r > c) {
    const int t = r;
    r = c;
    c = t;
  }
  return k + r * k - (r * (r - 1)) / 2 + (c - r);
}

// Damped normal equations (H + lam diag H) d = b, solved on lane 0 in FP64
// (multi_fit.c:1174-1203 with dposv).  Returns the solver status on lane 0.
__device__ inline int solve_fp64_lane0(const double* jh, int k, double lam, double* out) {
  double A[MAX_JAC * MAX_JAC], b[MAX_JAC];
  int id = k;
  for (int l = 0; l < k; l++) {
    b[l] = jh[l];
    for (int m = l; m < k; m++) {
      A[l * k + m] = (l == m) ? (1.0 + lam) * jh[id] : jh[id];
      id++;
    }
  }
  const int info = chol_solve(A, b, k);
  for (int l = 0; l < k; l++) out[l] = b[l];
  return info;
}

// solve_fp64_lane0 with one row per lane (all lanes call it): every element
// of the factor and of the solution is computed with chol_solve's
// operations in chol_solve's order -- lane i forms row i of L and, in turn,
// b[i]; the back substitution's products are formed on the lanes that hold
// them and subtracted in order -- so the result is chol_solve's to the bit,
// with O(k^2) instead of O(k^3) instructions on a single lane (each FP64
// instruction occupies the pipe for the whole warp however few lanes run).
// Returns the solver status on every lane; out[0..k) on every lane.
__device__ inline int solve_fp64_warp(const double* jh, int k, double lam, double* out, int lane) {
  const unsigned full = 0xffffffffu;
  double ac[MAX_JAC], L[MAX_JAC];
#pragma unroll
  for (int j = 0; j < MAX_JAC; j++) {
    ac[j] = 0.0;
    L[j] = 0.0;
    if (lane < k && j < k && j <= lane) {
      const int id = k + j * k - (j * (j - 1)) / 2 + (lane - j);
      ac[j] = (j == lane) ? (1.0 + lam) * jh[id] : jh[id];
    }
  }
  int info = 0;
#pragma unroll
  for (int j = 0; j < MAX_JAC; j++) {
    if (j < k && info == 0) {
      double Lj[MAX_JAC];
#pragma unroll
      for (int m = 0; m < MAX_JAC; m++) Lj[m] = (m < j) ? __shfl_sync(full, L[m], j) : 0.0;
      double d = ac[j];
#pragma unroll
      for (int m = 0; m < MAX_JAC; m++)
        if (m < j) d = __dsub_rn(d, __dmul_rn(L[m], L[m]));
      d = __shfl_sync(full, d, j);
      if (!(d > 0.0)) {
        info = j + 1;
      } else {
        d = sqrt(d);
        if (lane == j) L[j] = d;
        if (lane > j && lane < k) {
          double sum = ac[j];
#pragma unroll
          for (int m = 0; m < MAX_JAC; m++)
            if (m < j) sum = __dsub_rn(sum, __dmul_rn(L[m], Lj[m]));
          L[j] = sum / d;
        }
      }
    }
  }
  if (info != 0) return info;
  // forward substitution: lane i in turn, b[i] broadcast as it is found
  const double bl = lane < k ? jh[lane] : 0.0;
  double bb[MAX_JAC];
#pragma unroll
  for (int i = 0; i < MAX_JAC; i++) {
    bb[i] = 0.0;
    if (i < k) {
      double v = 0.0;
      if (lane == i) {
        double sum = bl;
#pragma unroll
        for (int m = 0; m < MAX_JAC; m++)
          if (m < i) sum = __dsub_rn(sum, __dmul_rn(L[m], bb[m]));
        v = sum / L[i];
      }
      bb[i] = __shfl_sync(full, v, i);
    }
  }
  // back substitution: the products L[m][i] x[m] formed on lane m
  double xs[MAX_JAC];
#pragma unroll
  for (int i = 0; i < MAX_JAC; i++) xs[i] = 0.0;
#pragma unroll
  for (int i = MAX_JAC - 1; i >= 0; i--) {
    if (i < k) {
      double sum = bb[i];
#pragma unroll
      for (int m = 0; m < MAX_JAC; m++) {
        if (m > i && m < k) {
          const double pr = __shfl_sync(full, __dmul_rn(L[i], xs[m]), m);
          sum = __dsub_rn(sum, pr);
        }
      }
      xs[i] = sum / __shfl_sync(full, L[i], i);
    }
  }
#pragma unroll
  for (int i = 0; i < MAX_JAC; i++) {
    if (i < k) {
      out[i] = xs[i];
      if (isnan(xs[i])) info = 1;
    }
  }
  return info;
}

// ---------------------------------------------------------------------------
// MLE per-pixel deviance 2((f - x) - x log(f/x))  (multi_fit.c:174)
// ---------------------------------------------------------------------------

__device__ __forceinline__ double deviance(double fi, double x) {
  return 2.0 * ((fi - x) - x * log(fi / x));
}

// FP32 form without the cancellation of the direct formula when f ~ x:
// with r = (f - x)/x,  dev = 2 x (r - log1p(r)).  For |r| < 1/2 the bracket
// is evaluated from the atanh series of log1p: with u = r/(2+r),
//   r - log1p(r) = u r - 2 u^3 (1/3 + u^2/5 + u^4/7 + ...),
// whose two terms do not cancel; elsewhere the direct form is well
// conditioned.
__device__ __forceinline__ float r_minus_log1p(float r) {
  if (fabsf(r) < 0.5f) {
    const float u = r * rcp_approx(2.0f + r);
    const float u2 = u * u;
    float s = 1.0f / 19.0f;
    s = fmaf(u2, s, 1.0f / 17.0f);
    s = fmaf(u2, s, 1.0f / 15.0f);
    s = fmaf(u2, s, 1.0f / 13.0f);
    s = fmaf(u2, s, 1.0f / 11.0f);
    s = fmaf(u2, s, 1.0f / 9.0f);
    s = fmaf(u2, s, 1.0f / 7.0f);
    s = fmaf(u2, s, 1.0f / 5.0f);
    s = fmaf(u2, s, 1.0f / 3.0f);
    return fmaf(u, r, -2.0f * u * u2 * s);
  }
  return r - log1pf(r);
}

// Deviance from the residual res = f - x, which the caller computes
// accurately: 2 x (r - log1p(r)) with r = res / x.
__device__ __forceinline__ float dev_res(float res, float x) {
  return 2.0f * x * r_minus_log1p(res * rcp_approx(x));
}

__device__ __forceinline__ float deviance(float fi, float x) { return dev_res(fi - x, x); }

// Explicitly rounded products so that a contribution computed in one
// kernel is bit-identical to the one recomputed in another.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float exp_t(float v) { return expf(v); }
__device__ __forceinline__ double exp_t(double v) { return exp(v); }

// Fit-image contribution of a peak at one pixel: h * psf * rqe
// (multi_fit.c:52) and its background term bg * rqe + scmos (:54).
template <typename T>
__device__ __forceinline__ T contrib_f(double h, T psf, T rqe) {
  return mul_rn(mul_rn((T)h, psf), rqe);
}
template <typename T>
__device__ __forceinline__ T contrib_bg(double bg, T rqe, T scmos) {
  return add_rn(mul_rn((T)bg, rqe), scmos);
}

// ---------------------------------------------------------------------------
// per-warp workspace in shared memory
// ---------------------------------------------------------------------------

__host__ __device__ __forceinline__ bool is_spline(int model) { return model == M_SPLINE2D || model == M_SPLINE3D; }
__host__ __device__ __forceinline__ bool is_fft(int model) { return model == M_FFT; }
// an arbitrary-PSF model: input formats (x, y, z [, background, height]) and
// mFitCheck alone as the check (cubic_fit.c:660, fft_fit.c:303)
__host__ __device__ __forceinline__ bool is_arb(int model) { return model >= M_SPLINE2D; }

// The FFT PSF model's device tables (doubles), for a PSF of nz x ny x nx
// (x fastest) and nk = nx/2 + 1 spectrum columns:
//   W  [nz][ny][nk] (re, im)  the spectrum, pFTInitialize psf_fft.c:310-365
//   Ex [nx][nk]     (re, im)  e^{2 pi i kx x / nx}
//   Ey [ny][ny]     (re, im)  e^{2 pi i ky y / ny}   (index [y][ky])
//   Ez [nz]         (re, im)  e^{2 pi i kz (nz/2) / nz}: the middle z plane
//   dkx [nk], dky [ny], dkz [nz]  pFTCalcShiftVectorDerivative :70-84
struct FFTLayout {
  int nk, w, ex, ey, ez, dkx, dky, dkz, total;
};
__host__ __device__ __forceinline__ FFTLayout fft_layout(int nx, int ny, int nz) {
  FFTLayout L;
  L.nk = nx / 2 + 1;
  L.w = 0;
  L.ex = L.w + 2 * nz * ny * L.nk;
  L.ey = L.ex + 2 * nx * L.nk;
  L.ez = L.ey + 2 * ny * ny;
  L.dkx = L.ez + 2 * nz;
  L.dky = L.dkx + L.nk;
  L.dkz = L.dky + ny;
  L.total = L.dkz + nz;
  return L;
}
__host__ __device__ __forceinline__ bool is_pupil(int model) { return model == M_PUPIL; }

// The pupil-function model's device tables (doubles), pupil size N (even),
// m = N / 2:
//   E   [N][N] (re, im)  e^{2 pi i a b / N}: the backward DFT's twiddles
//   PF  [N][N] (re, im)  the pupil function / N, negated where i + k is odd
//                        (pfnSetPF pupil_function.c:370-410)
//   KX  [N]              2 pi kx[i N]: the x and y shift multipliers of
//                        pfnTranslate :453-463 and the x derivative's
//   KY  [N][N]           2 pi ky: the y derivative's multiplier (:160-178)
//   KZ  [N][N]           2 pi kz: the z derivative's multiplier (:185-203)
//   KZS [m+1][m+1]       2 pi kz at (m - min(a, b), m - max(a, b)): the z
//                        shift multiplier of pixel offset (a, b) from the
//                        centre, pfnTranslate's pie slice :475-486
//   RNG [N][2]           per pupil row, the first and last column where the
//                        pupil function is not zero (first > last: none)
//   BAND [2]             the first and last row that is not all zero
// A pupil function is zero outside the objective's NA (a disk of a few
// pixels' radius in a pupil of tens), so the sums run over its support
// only; the terms left out are exact zeros.
struct PupilLayout {
  int e, pf, kx, ky, kz, kzs, rng, band, total;
};
__host__ __device__ __forceinline__ PupilLayout pupil_layout(int n) {
  PupilLayout L;
  const int m1 = n / 2 + 1;
  L.e = 0;
  L.pf = L.e + 2 * n * n;
  L.kx = L.pf + 2 * n * n;
  L.ky = L.kx + n;
  L.kz = L.ky + n * n;
  L.kzs = L.kz + n * n;
  L.rng = L.kzs + m1 * m1;
  L.band = L.rng + 2 * n;
  L.total = L.band + 2;
  return L;
}
// Rows of the pupil function's support band (first-index rows holding a
// nonzero value; set from the pupil's tables when the fitter is made), or
// all N rows when unknown.
__host__ __device__ __forceinline__ int pupil_band_rows(int n, int sz) { return (sz > 0 && sz <= n) ? sz : n; }
// Doubles of a warp's pupil scratch: B, By, Bz [band rows][N] (complex; the
// sums over the pupil's second index of the translated pupil function, and
// of it times -i ky and -i kz, for the band's rows only: the others are 0),
// three row buffers [N] (complex), the shift vectors sx, sy [N] (complex)
// and the z shift table [m+1][m+1] (complex).
__host__ __device__ __forceinline__ int pupil_scratch_doubles(int n, int sz) {
  const int m1 = n / 2 + 1;
  return 6 * pupil_band_rows(n, sz) * n + 10 * n + 2 * m1 * m1;
}
// Warps with a workspace in a per-frame CTA (k_prepare, k_post) and in an
// auxiliary CTA for the pupil model: its scratch is ~54 KB per warp at a
// 30-pixel pupil, ~110 KB at 44 pixels.
__host__ __device__ __forceinline__ int pupil_ws_warps(int n) { return n <= 30 ? 4 : (n <= 44 ? 2 : 1); }

// Warps of a 1024-thread per-frame CTA (k_prepare, k_post) that carry a
// workspace: all 32, 8 for the FFT PSF model, whose shape scratch is
// ~20 KB per warp, and pupil_ws_warps for the pupil model.
__host__ __device__ __forceinline__ int cta_ws_warps(const ModelCfg& cfg) {
  return cfg.model == M_FFT ? 8 : (cfg.model == M_PUPIL ? pupil_ws_warps(cfg.sx) : 32);
}
// Warps of the warp-per-peak auxiliary kernels' CTAs.
__host__ __device__ __forceinline__ int aux_warps(const ModelCfg& cfg) {
  return cfg.model == M_PUPIL ? pupil_ws_warps(cfg.sx) : 8;
}

// Doubles of a warp's FFT scratch: C, Cz [ny][nk], D, Dy, Dz [ny][nk]
// (complex), the shift vectors sx [nk], sy [ny], sz [nz] (complex).
__host__ __device__ __forceinline__ int fft_scratch_doubles(int nx, int ny, int nz) {
  const int nk = nx / 2 + 1;
  return 2 * (5 * ny * nk + nk + ny + nz);
}

// The FP32 engine fits the Gaussian models with compensated (float-float)
// arithmetic on the quantities that decide steps; it has its own, smaller
// workspace layout.
template <typename T>
__host__ __device__ __forceinline__ bool gauss32(const ModelCfg& cfg) {
  return sizeof(T) == 4 && !is_arb(cfg.model);
}

template <typename T>
struct WarpWS {
  T* Fb;      // base fit image (without this peak) at the cached anchor
  T* Bs;      // base background sum + this pixel's sCMOS term
  T* R;       // rqe
  T* X;       // data (FP32 splines: the low word of t1 until a trial reloads)
  T* IC;      // 1 / (base count + 1)
  T* psf;     // current peak shape
  T* psf0;    // FP32 only: shape at the start of the step
  T* f0;      // FP32 only: model value at the start of the step
  T* rho;     // FP32 only: t1 = 2 (f0 - x) / f0, high word
  T* ext;     // Gaussian x factors / spline deltas (4*64)
  T* eyt;
  T* xt;
  T* yt;
  double* jh; // 36: jacobian (7) + upper Hessian (up to 28)
  double* scratch;  // 16
  PeakRec* w;     // working record (lane 0 writes)
  PeakRec* orig;  // record at the start of the step
  PeakRec* t;     // trial record (lane 0)
  float* red; // FP32: 32 x 33 per-lane partial sums (splines) / solve scratch
  // FP32 Gaussian layout
  float* t1h;   // t1 = 2 (f0 - x) / f0 at the start of the step, float-float
  float* t1l;
  float* f0g;   // f0 (float)
  float* T2s;   // Hessian weight 2 x / f0^2, rqe and peak count (with this
  float* Rs;    // peak) at the start anchor
  float* Cs;
  float* tab0;  // shape tables of the step's start: ex hi, ex lo, ey hi, ey lo, xt, yt
  float* tab1;  // trial tables (same layout) / pass-1 gradient tables / solve scratch
  double* fw;   // M_FFT / M_PUPIL: the shape evaluation's scratch (fft_scratch_doubles,
                // pupil_scratch_doubles)
  float* par0;  // float-float parameter slots (g32_params) of the step's start record
  float* par1;  // ... and of the current trial
  int ts;       // table stride (ROI size rounded up to 32)
  const unsigned short* roi;   // ROI pixel table (packed rx | ry << 8)
};

template <typename T>
__host__ __device__ constexpr int ws_pixel_arrays() {
  return sizeof(T) == 4 ? 9 : 6;
}

__host__ __device__ __forceinline__ int table_stride(int roi) { return (roi + 31) & ~31; }

template <typename T>
__host__ __device__ inline size_t warp_ws_bytes(const ModelCfg& cfg, int nroi) {
  size_t n = (size_t)((nroi + 31) / 32) * 32;
  size_t b;
  if (gauss32<T>(cfg)) {
    b = 6 * n * sizeof(float) + 14 * (size_t)table_stride(cfg.roi) * sizeof(float) + 2 * 20 * sizeof(float);
  } else {
    b = ws_pixel_arrays<T>() * n * sizeof(T);
    b += 4 * 64 * sizeof(T) * 2;   // ext/eyt/xt/yt (Gaussian) or 4 delta tables (spline)
  }
  b = (b + 15) & ~(size_t)15;
  b += 36 * sizeof(double) + 16 * sizeof(double);
  b += 3 * sizeof(PeakRec);
  if (sizeof(T) == 4 && !gauss32<T>(cfg) && nroi > 0) b += 32 * 33 * sizeof(float);
  if (is_fft(cfg.model)) b = ((b + 15) & ~(size_t)15) + fft_scratch_doubles(cfg.sx, cfg.sy, cfg.sz) * sizeof(double);
  if (is_pupil(cfg.model)) b = ((b + 15) & ~(size_t)15) + pupil_scratch_doubles(cfg.sx, cfg.sz) * sizeof(double);
  return (b + 127) & ~(size_t)127;
}

template <typename T>
__device__ inline WarpWS<T> warp_ws(char* base, const ModelCfg& cfg, int nroi) {
  WarpWS<T> ws;
  size_t n = (size_t)((nroi + 31) / 32) * 32;
  size_t off;
  if (gauss32<T>(cfg)) {
    const int ts = table_stride(cfg.roi);
    float* t = reinterpret_cast<float*>(base);
    ws.t1h = t;
    ws.t1l = t + n;
    ws.f0g = t + 2 * n;
    ws.T2s = t + 3 * n;
    ws.Rs = t + 4 * n;
    ws.Cs = t + 5 * n;
    ws.tab0 = t + 6 * n;
    ws.tab1 = ws.tab0 + 6 * ts;
    ws.ts = ts;
    ws.roi = nullptr;
    // generic views used by the auxiliary kernels (jt_row reads xt / yt)
    ws.Fb = ws.Bs = ws.R = ws.X = ws.IC = ws.psf = ws.psf0 = ws.f0 = ws.rho = nullptr;
    ws.ext = reinterpret_cast<T*>(ws.tab0);
    ws.eyt = reinterpret_cast<T*>(ws.tab0 + 2 * ts);
    ws.xt = reinterpret_cast<T*>(ws.tab0 + 4 * ts);
    ws.yt = reinterpret_cast<T*>(ws.tab0 + 5 * ts);
    ws.red = ws.tab1;
    ws.par0 = ws.tab0 + 14 * ts;
    ws.par1 = ws.par0 + 20;
    off = 6 * n * sizeof(float) + 14 * (size_t)ts * sizeof(float) + 2 * 20 * sizeof(float);
  } else {
    T* t = reinterpret_cast<T*>(base);
    ws.Fb = t;
    ws.Bs = t + n;
    ws.R = t + 2 * n;
    ws.X = t + 3 * n;
    ws.IC = t + 4 * n;
    ws.psf = t + 5 * n;
    ws.psf0 = t + 6 * n;   // only valid when ws_pixel_arrays<T>() == 9
    ws.f0 = t + 7 * n;
    ws.rho = t + 8 * n;
    T* tab = t + ws_pixel_arrays<T>() * n;
    ws.ext = tab;
    ws.eyt = tab + 128;
    ws.xt = tab + 256;
    ws.yt = tab + 384;
    ws.t1h = ws.t1l = ws.f0g = ws.T2s = ws.Rs = ws.Cs = ws.tab0 = ws.tab1 = ws.par0 = ws.par1 = nullptr;
    ws.ts = 0;
    ws.roi = nullptr;
    off = ws_pixel_arrays<T>() * n * sizeof(T) + 4 * 64 * sizeof(T) * 2;
  }
  off = (off + 15) & ~(size_t)15;
  ws.jh = reinterpret_cast<double*>(base + off);
  ws.scratch = ws.jh + 36;
  ws.w = reinterpret_cast<PeakRec*>(base + off + 52 * sizeof(double));
  ws.orig = ws.w + 1;
  ws.t = ws.w + 2;
  if (!gauss32<T>(cfg))
    ws.red = reinterpret_cast<float*>(base + off + 52 * sizeof(double) + 3 * sizeof(PeakRec));
  ws.fw = nullptr;
  if (is_fft(cfg.model) || is_pupil(cfg.model)) {
    size_t o = off + 52 * sizeof(double) + 3 * sizeof(PeakRec);
    if (sizeof(T) == 4 && nroi > 0) o += 32 * 33 * sizeof(float);
    ws.fw = reinterpret_cast<double*>(base + ((o + 15) & ~(size_t)15));
  }
  return ws;
}

// ---------------------------------------------------------------------------
// model pieces (all lanes participate; results in the warp workspace)
// ---------------------------------------------------------------------------

// Offsets of the first ROI column / row from the peak centre
// (daoCalcPeakShape dao_fit.c:968-998; the y offset uses xoff, :979) and
// the widths, as float-float values.
struct G32Axes {
  ff xo, yo, wx, wy;
};
__device__ __forceinline__ G32Axes g32_axes(const ModelCfg& cfg, const PeakRec& w) {
  G32Axes a;
  a.xo = ff_from_double(-(w.p[PX] - (double)w.xi) - cfg.xoff);
  a.yo = ff_from_double(-(w.p[PY] - (double)w.yi) - cfg.xoff);
  a.wx = ff_from_double(w.p[PXW]);
  a.wy = ff_from_double(w.p[PYW]);
  return a;
}

// The float-float parameters of a Gaussian record that the FP32 step uses,
// converted lane-parallel into a shared slot table (two floats per slot):
// lane i computes slot i, so the set costs one pass of FP64 instructions
// instead of one per value.  An FP64 instruction takes 64 cycles of this
// part's FP64 pipe whether one lane or 32 execute it.  The values equal
// g32_axes' and ff_from_double's bit for bit (the same double operations).
enum { GP_XO = 0, GP_YO, GP_WX, GP_WY, GP_H, GP_BG, GP_GX, GP_GY, GP_DBG, GP_N };

// z_factors' gx (side 0) or gy (side 1), one lane each.
__device__ __forceinline__ double z_factor_side(const ModelCfg& cfg, const PeakRec& w, int side) {
  const double c0 = side ? cfg.wy[0] : cfg.wx[0], c1 = side ? cfg.wy[1] : cfg.wx[1];
  const double c2 = side ? cfg.wy[2] : cfg.wx[2], c3 = side ? cfg.wy[3] : cfg.wx[3];
  const double c4 = side ? cfg.wy[4] : cfg.wx[4];
  const double z0 = (w.p[PZ] - c1) / c2;
  const double z1 = z0 * z0, z2 = z1 * z0;
  const double zt = 2.0 * z0 + 3.0 * c3 * z1 + 4.0 * c4 * z2;
  return -2.0 * zt / (c0 * (side ? w.wyt : w.wxt));
}

// Slots of record w into par[2 * GP_N] (all lanes, warp-uniform).  ref is
// the record the background change GP_DBG is taken against (nullptr: no
// GP_DBG); zf: also the Z model's width derivatives GP_GX / GP_GY.
__device__ inline void g32_params(const ModelCfg& cfg, const PeakRec& w, const PeakRec* ref, bool zf,
                                  float* par, int lane) {
  const int sl = lane < GP_N ? lane : GP_H;
  const int pi = (sl == GP_XO) ? PX : (sl == GP_YO) ? PY : (sl == GP_WX) ? PXW : (sl == GP_WY) ? PYW
               : (sl == GP_BG || sl == GP_DBG) ? PBG : PH;
  double v = w.p[pi];
  double b = 0.0;   // v - 0 is v (a -0.0 stays -0.0)
  if (sl <= GP_YO) b = (double)(sl == GP_XO ? w.xi : w.yi);
  else if (sl == GP_DBG && ref) b = ref->p[PBG];
  v = v - b;
  if (sl <= GP_YO) v = -v - cfg.xoff;
  if (zf) {
    const double g = z_factor_side(cfg, w, sl == GP_GY ? 1 : 0);
    if (sl == GP_GX || sl == GP_GY) v = g;
  }
  const ff f = ff_from_double(v);
  if (lane < GP_N) {
    par[2 * lane] = f.h;
    par[2 * lane + 1] = f.l;
  }
  __syncwarp();
}

__device__ __forceinline__ ff gpar(const float* par, int slot) { return ff{par[2 * slot], par[2 * slot + 1]}; }

// FP32 Gaussian shape tables: per axis the factor exp(-t^2 w) as a
// float-float pair and the offset t as a float, all in FP32 instructions.
// dst layout (stride ts): ex hi, ex lo, ey hi, ey lo, xt, yt.
// A width can be negative: the '2d' model clamps XWIDTH only and copies the
// unclamped value to YWIDTH (dao_fit.c:1061-1085, :1801-1816).  Factors
// above e^30 are taken as e^30: a trial with such a factor has a model value
// of 1e13 or more at that pixel, an error far above any start error, and is
// rejected whatever the exact value (as the reference rejects it).
__device__ inline void g32_tables_ax(const ModelCfg& cfg, const G32Axes& ax, float* dst, int ts, int lane) {
  for (int i = lane; i < cfg.roi; i += 32) {
    const ff tx = ff_add_f(ax.xo, (float)i), ty = ff_add_f(ax.yo, (float)i);
    ff argx = ff_neg(ff_mul(ff_mul(tx, tx), ax.wx)), argy = ff_neg(ff_mul(ff_mul(ty, ty), ax.wy));
    if (argx.h > 30.0f) argx = ff{30.0f, 0.0f};
    if (argy.h > 30.0f) argy = ff{30.0f, 0.0f};
    const ff ex = ff_exp(argx);
    const ff ey = ff_exp(argy);
    dst[i] = ex.h;
    dst[ts + i] = ex.l;
    dst[2 * ts + i] = ey.h;
    dst[3 * ts + i] = ey.l;
    dst[4 * ts + i] = tx.h;
    dst[5 * ts + i] = ty.h;
  }
}

__device__ inline void g32_tables(const ModelCfg& cfg, const PeakRec& w, float* dst, int ts, int lane) {
  g32_tables_ax(cfg, g32_axes(cfg, w), dst, ts, lane);
}

// The same tables from a slot table of g32_params.
__device__ inline void g32_tables_p(const ModelCfg& cfg, const float* par, float* dst, int ts, int lane) {
  G32Axes ax;
  ax.xo = gpar(par, GP_XO);
  ax.yo = gpar(par, GP_YO);
  ax.wx = gpar(par, GP_WX);
  ax.wy = gpar(par, GP_WY);
  g32_tables_ax(cfg, ax, dst, ts, lane);
}

__device__ __forceinline__ ff g32_psf(const float* tab, int ts, int rx, int ry) {
  return ff_mul(ff{tab[rx], tab[ts + rx]}, ff{tab[2 * ts + ry], tab[3 * ts + ry]});
}

// Fit-image contributions of an FP32 Gaussian peak at one pixel, quantised:
// f: h * (psf * rqe), bg: bg * rqe + scmos (multi_fit.c:52-54), both
// float-float.  Every add and subtract of the same record goes through
// this one function, so they cancel exactly.
__device__ __forceinline__ void g32_contrib(const float* tab, int ts, ff H, ff BG, int rx, int ry,
                                            float rq, float sc, Q2& qf, Q2& qb) {
  const ff ps = ff_mul_f(g32_psf(tab, ts, rx, ry), rq);
  qf.h = fixed_from_ff(ff_mul(H, ps));
  qf.l = 0;
  qb.h = fixed_from_ff(ff_add_f(ff_mul_f(BG, rq), sc));
  qb.l = 0;
}

// Gaussian separable factors, daoCalcPeakShape dao_fit.c:968-998.  The y
// offset uses xoff as the reference does (:979).
template <typename T>
__device__ inline void gauss_tables(const ModelCfg& cfg, const double* p, int xi, int yi,
                                    WarpWS<T>& ws, int lane) {
  const double xo = -(p[PX] - (double)xi) - cfg.xoff;
  const double yo = -(p[PY] - (double)yi) - cfg.xoff;
  const T wx = (T)p[PXW], wy = (T)p[PYW];
  for (int i = lane; i < cfg.roi; i += 32) {
    T tx = (T)((double)i + xo);
    T ty = (T)((double)i + yo);
    ws.xt[i] = tx;
    ws.yt[i] = ty;
    ws.ext[i] = exp_t(mul_rn(mul_rn(-tx, tx), wx));
    ws.eyt[i] = exp_t(mul_rn(mul_rn(-ty, ty), wy));
  }
}

// Spline cell position of a peak, cfCalcPeakShape cubic_fit.c:455-480.
struct SplinePos {
  int xs, ys, zi;
  double xd, yd, zd;
};

__device__ inline SplinePos spline_pos(const double* p, int xi, int yi, int zi) {
  SplinePos s;
  double xd = 1.5 - (p[PX] - xi);
  double yd = 1.5 - (p[PY] - yi);
  s.xs = 0;
  if (xd >= 1.0) { xd -= 1.0; s.xs = 1; }
  s.ys = 0;
  if (yd >= 1.0) { yd -= 1.0; s.ys = 1; }
  s.zi = zi;
  s.xd = xd;
  s.yd = yd;
  s.zd = p[PZ] - zi;
  return s;
}

__device__ __forceinline__ double clamp01(double v) { return v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v); }

template <typename T>
__device__ __forceinline__ T pw(T v, int e) {
  T r = (T)1;
  for (int i = 0; i < e; i++) r = mul_rn(r, v);
  return r;
}

// Monomial tables for value / d/dx / d/dy / d/dz (computeDelta3D,
// cubic_spline.c:105-138; computeDelta2D :66-91).  Deltas are clamped to
// [0, 1] as rangeCheckD does (:798-826).
__device__ __forceinline__ ff ff_pow(ff v, int e) {
  ff r{1.0f, 0.0f};
  for (int i = 0; i < e; i++) r = ff_mul(r, v);
  return r;
}

// FP32 engine: the value monomials x^a y^b z^c as float-float (hi words in
// ext[0, 64), lo words in yt[0, 64)), from the FP64 deltas.  The spline's
// model value is evaluated from them with a compensated dot
// (spline_value_ff): FP32 rounding noise in the model value, which the fit
// image carries from one step to the next, moves the converged background
// of ~1 % of the peaks of the spline workload by more than 1e-4 relative
// (FP64 oracle with 1e-8 relative noise on the value; 1e-9: 0.1 %).
template <typename T>
__device__ inline void spline_value_monomials(const ModelCfg& cfg, const SplinePos& s, WarpWS<T>& ws,
                                              int lane) {
  const bool three = (cfg.model == M_SPLINE3D);
  const ff x = ff_from_double(clamp01(s.xd)), y = ff_from_double(clamp01(s.yd));
  const ff z = ff_from_double(three ? clamp01(s.zd) : 0.0);
  for (int id = lane; id < (three ? 64 : 16); id += 32) {
    const int a = three ? (id >> 4) : (id >> 2);
    const int b = three ? ((id >> 2) & 3) : (id & 3);
    const int c = three ? (id & 3) : 0;
    const ff m = ff_mul(ff_mul(ff_pow(x, a), ff_pow(y, b)), ff_pow(z, c));
    ws.ext[id] = (T)m.h;
    ws.yt[id] = (T)m.l;
  }
}

template <typename T>
__device__ inline void spline_tables(const ModelCfg& cfg, const SplinePos& s, WarpWS<T>& ws,
                                     int lane) {
  const T x = (T)clamp01(s.xd), y = (T)clamp01(s.yd);
  if (cfg.model == M_SPLINE3D) {
    const T z = (T)clamp01(s.zd);
    for (int id = lane; id < 64; id += 32) {
      const int a = id >> 4, b = (id >> 2) & 3, c = id & 3;
      const T px = pw(x, a), py = pw(y, b), pz = pw(z, c);
      if (sizeof(T) != 4) ws.ext[id] = mul_rn(mul_rn(px, py), pz);
      // derivative tables are indexed by the coefficient they multiply
      ws.ext[64 + id] = (a > 0) ? mul_rn(mul_rn(mul_rn((T)a, pw(x, a - 1)), py), pz) : (T)0;
      ws.eyt[id] = (b > 0) ? mul_rn(mul_rn(px, mul_rn((T)b, pw(y, b - 1))), pz) : (T)0;
      ws.eyt[64 + id] = (c > 0) ? mul_rn(mul_rn(px, py), mul_rn((T)c, pw(z, c - 1))) : (T)0;
    }
  } else {
    for (int id = lane; id < 16; id += 32) {
      const int a = id >> 2, b = id & 3;
      const T px = pw(x, a), py = pw(y, b);
      if (sizeof(T) != 4) ws.ext[id] = mul_rn(px, py);
      ws.ext[64 + id] = (a > 0) ? mul_rn(mul_rn((T)a, pw(x, a - 1)), py) : (T)0;
      ws.eyt[id] = (b > 0) ? mul_rn(px, mul_rn((T)b, pw(y, b - 1))) : (T)0;
    }
  }
  if constexpr (sizeof(T) == 4) spline_value_monomials(cfg, s, ws, lane);
}

__device__ __forceinline__ int clampi(int v, int hi_excl) {
  return v < 0 ? 0 : (v >= hi_excl ? hi_excl - 1 : v);
}

// Spline cell base (fAt3D index clamps, cubic_spline.c:509-522).
template <typename T>
__device__ __forceinline__ const T* spline_cell(const ModelCfg& cfg, const T* aij, int zc, int yc,
                                                int xc) {
  xc = clampi(xc, cfg.sx);
  yc = clampi(yc, cfg.sy);
  if (cfg.model == M_SPLINE3D) {
    zc = clampi(zc, cfg.sz);
    return aij + ((size_t)xc * (cfg.sy * cfg.sz) + (size_t)yc * cfg.sz + zc) * 64;
  }
  return aij + ((size_t)xc * cfg.sy + yc) * 16;
}

// Dot of a spline cell with one of the monomial tables, in a fixed order.
template <typename T>
__device__ __forceinline__ T spline_dot(const T* c, const T* tab, int n) {
  T acc = (T)0;
#pragma unroll 8
  for (int i = 0; i < n; i++) acc = fma_rn(__ldg(c + i), tab[i], acc);
  return acc;
}

// FP32 engine: the spline's value at ROI pixel (rx, ry) as float-float: a
// compensated dot (Ogita, Rump and Oishi's Dot2, with the float-float
// monomials' lo words folded into the error sum) of the cell's FP32
// coefficients with the value monomials of spline_value_monomials.
__device__ __forceinline__ ff spline_value_ff(const ModelCfg& cfg, const float* aij, const WarpWS<float>& ws,
                                              const SplinePos& s, int rx, int ry) {
  const int nc = (cfg.model == M_SPLINE3D) ? 64 : 16;
  const float* c = spline_cell(cfg, aij, s.zi, ry + s.ys, rx + s.xs);
  float hi = 0.0f, err = 0.0f;
#pragma unroll 8
  for (int i = 0; i < nc; i++) {
    const float ci = __ldg(c + i);
    const float p = __fmul_rn(ci, ws.ext[i]);
    const float pe = __fmaf_rn(ci, ws.ext[i], -p);
    const ff t = two_sum(hi, p);
    hi = t.h;
    err = __fmaf_rn(ci, ws.yt[i], __fadd_rn(err, __fadd_rn(t.l, pe)));
  }
  return fast_two_sum(hi, err);
}

// FP32 spline contributions at one pixel, quantised from float-float
// values: f: h * (psf * rqe), bg: bg * rqe + scmos (multi_fit.c:52-54).
// Every add and subtract of a spline peak in the FP32 engine goes through
// this function, so they cancel exactly.
__device__ __forceinline__ void spl32_contrib(ff psf, ff H, ff BG, float rq, float sc, Q2& qf, Q2& qb) {
  qf.h = fixed_from_ff(ff_mul(H, ff_mul_f(psf, rq)));
  qf.l = 0;
  qb.h = fixed_from_ff(ff_add_f(ff_mul_f(BG, rq), sc));
  qb.l = 0;
}

// ---------------------------------------------------------------------------
// FFT PSF model (M_FFT, the FP64 engine): ftFitCalcPeakShape fft_fit.c:127-155
// and ftFitCalcJH3D :43-117 through pFTTranslate / pFTGetPSF* (psf_fft.c).
// The PSF at the peak's offset (dx, dy, dz) is the middle z plane of the c2r
// inverse of the spectrum times the shift vectors, evaluated separably: for
// each (ky, kx) the z sum C of the shifted spectrum times the middle-plane
// twiddle (and Cz, the same times -i dkz); for each (y, kx) the y sums D of
// C, Dy of C times -i dky and Dz of Cz; a pixel (x, y) is then the c2r x sum
// of D[y] (weights 1 for the x DC and Nyquist bins, whose imaginary parts
// the c2r drops, 2 otherwise), and of D[y] times -i dkx, Dy[y], Dz[y] for
// the derivatives (dz negated, as pFTGetPSFdz).
// ---------------------------------------------------------------------------

constexpr double SA_PI = 3.14159265358979323846;   // the reference's M_PI

template <typename T>
__device__ inline void fft_tables(const ModelCfg& cfg, const PeakRec& w, WarpWS<T>& ws, int lane) {
  const int nx = cfg.sx, ny = cfg.sy, nz = cfg.sz;
  const FFTLayout L = fft_layout(nx, ny, nz);
  const int nk = L.nk;
  double* C = ws.fw;
  double* Cz = C + 2 * ny * nk;
  double* Dm = Cz + 2 * ny * nk;
  double* Dy = Dm + 2 * ny * nk;
  double* Dz = Dy + 2 * ny * nk;
  double* sxv = Dz + 2 * ny * nk;
  double* syv = sxv + 2 * nk;
  double* szv = syv + 2 * ny;
  const double ox = w.p[PX] - (double)w.xi, oy = w.p[PY] - (double)w.yi, oz = w.p[PZ];
  // shift vectors, pFTCalcShiftVector psf_fft.c:43-60 (the z one with -dz):
  // entry k is cos / sin of t1 * m with m = k up to size/2 (the sine kept
  // positive at size/2, the reference loop's second write) and m = size - k
  // with the sine negated above it
  for (int i = lane; i < nk + ny + nz; i += 32) {
    int size, k;
    double d;
    double* out;
    if (i < nk) {
      size = nx; k = i; d = ox; out = sxv + 2 * k;
    } else if (i < nk + ny) {
      size = ny; k = i - nk; d = oy; out = syv + 2 * k;
    } else {
      size = nz; k = i - nk - ny; d = -oz; out = szv + 2 * k;
    }
    double re = 1.0, im = 0.0;
    if (k > 0) {
      const double t1 = -SA_PI * 2.0 * d / ((double)size);
      const bool low = k <= size / 2;
      const double t2 = t1 * (double)(low ? k : size - k);
      re = cos(t2);
      im = low ? sin(t2) : -sin(t2);
    }
    out[0] = re;
    out[1] = im;
  }
  __syncwarp();
  const double* Wt = cfg.fft + L.w;
  const double* Ez = cfg.fft + L.ez;
  const double* dkz = cfg.fft + L.dkz;
  for (int q = lane; q < ny * nk; q += 32) {
    const int ky = q / nk, kx = q - ky * nk;
    const double syr = syv[2 * ky], syi = syv[2 * ky + 1], sxr = sxv[2 * kx], sxi = sxv[2 * kx + 1];
    double cr = 0.0, ci = 0.0, czr = 0.0, czi = 0.0;
    for (int kz = 0; kz < nz; kz++) {
      const double* wp = Wt + 2 * (((size_t)kz * ny + ky) * nk + kx);
      double r1 = __ldg(wp), c1 = __ldg(wp + 1), r2, c2;
      // z, y, x shifts in the reference's order (pFTTranslate :395-418)
      r2 = r1 * szv[2 * kz] - c1 * szv[2 * kz + 1];
      c2 = r1 * szv[2 * kz + 1] + c1 * szv[2 * kz];
      r1 = r2 * syr - c2 * syi;
      c1 = r2 * syi + c2 * syr;
      r2 = r1 * sxr - c1 * sxi;
      c2 = r1 * sxi + c1 * sxr;
      const double er = __ldg(Ez + 2 * kz), ei = __ldg(Ez + 2 * kz + 1);
      const double pr = r2 * er - c2 * ei, pi = r2 * ei + c2 * er;
      cr += pr;
      ci += pi;
      const double dk = __ldg(dkz + kz);
      czr += pi * dk;
      czi -= pr * dk;
    }
    C[2 * q] = cr;
    C[2 * q + 1] = ci;
    Cz[2 * q] = czr;
    Cz[2 * q + 1] = czi;
  }
  __syncwarp();
  const double* Ey = cfg.fft + L.ey;
  const double* dky = cfg.fft + L.dky;
  for (int q = lane; q < ny * nk; q += 32) {
    const int y = q / nk, kx = q - y * nk;
    double dr = 0.0, di = 0.0, dyr = 0.0, dyi = 0.0, dzr = 0.0, dzi = 0.0;
    for (int ky = 0; ky < ny; ky++) {
      const double er = __ldg(Ey + 2 * (y * ny + ky)), ei = __ldg(Ey + 2 * (y * ny + ky) + 1);
      const int c = 2 * (ky * nk + kx);
      const double ar = C[c], ai = C[c + 1];
      const double pr = ar * er - ai * ei, pi = ar * ei + ai * er;
      dr += pr;
      di += pi;
      const double dk = __ldg(dky + ky);
      dyr += pi * dk;
      dyi -= pr * dk;
      const double zr = Cz[c], zi = Cz[c + 1];
      dzr += zr * er - zi * ei;
      dzi += zr * ei + zi * er;
    }
    Dm[2 * q] = dr;
    Dm[2 * q + 1] = di;
    Dy[2 * q] = dyr;
    Dy[2 * q + 1] = dyi;
    Dz[2 * q] = dzr;
    Dz[2 * q + 1] = dzi;
  }
}

// The PSF at ROI pixel (rx, ry) from fft_tables' D arrays; with g non-null
// also its x, y and z derivatives (pFTGetPSFdx / dy / dz) in g[0..2].
__device__ inline double fft_pixel(const ModelCfg& cfg, const double* fw, int rx, int ry, double* g) {
  const int nx = cfg.sx, ny = cfg.sy;
  const FFTLayout L = fft_layout(nx, ny, cfg.sz);
  const int nk = L.nk;
  const double* Dm = fw + 4 * ny * nk;
  const double* Dy = Dm + 2 * ny * nk;
  const double* Dz = Dy + 2 * ny * nk;
  const double* Ex = cfg.fft + L.ex + 2 * rx * nk;
  const double* dkx = cfg.fft + L.dkx;
  double vp = 0.0, vx = 0.0, vy = 0.0, vz = 0.0;
  for (int kx = 0; kx < nk; kx++) {
    const double er = __ldg(Ex + 2 * kx), ei = __ldg(Ex + 2 * kx + 1);
    const double c = ((kx == 0) || (2 * kx == nx)) ? 1.0 : 2.0;
    const int o = 2 * (ry * nk + kx);
    const double pr = Dm[o] * er - Dm[o + 1] * ei, pi = Dm[o] * ei + Dm[o + 1] * er;
    vp += c * pr;
    if (g) {
      vx += c * pi * __ldg(dkx + kx);
      vy += c * (Dy[o] * er - Dy[o + 1] * ei);
      vz += c * (Dz[o] * er - Dz[o + 1] * ei);
    }
  }
  if (g) {
    g[0] = vx;
    g[1] = vy;
    g[2] = -vz;
  }
  return vp;
}

// ---------------------------------------------------------------------------
// Pupil-function model (M_PUPIL, the FP64 engine): pfitCalcPeakShape
// pupil_fit.c:133-170 and pfitCalcJH3D :45-123 through pfnTranslate /
// pfnGetPSF / pfnGetPSFdx / dy / dz (pupil_function.c).  The complex PSF at
// pixel (u, v) -- u along the pupil's first index, which is the ROI's x
// (pupil_fit.c reads psf_r[roi_x * fit_size_y + roi_y]) -- is FFTW's
// unnormalised backward 2D transform of the translated pupil function ws,
//   psf(u, v) = sum_i e^{2 pi i i u / N} sum_k ws[i][k] e^{2 pi i k v / N},
// evaluated separably: the inner sums B[i][v] (and By, Bz: the same of ws
// times -i ky and -i kz, for the y and z derivatives) in pupil_tables, the
// outer sum per pixel in pupil_pixel, where the x derivative is the outer
// sum of B times -i kx[i] (kx is constant along the pupil's rows, which
// pfitInitialize checks on the host).
// ---------------------------------------------------------------------------

template <typename T>
__device__ inline void pupil_tables(const ModelCfg& cfg, const PeakRec& w, WarpWS<T>& ws, int lane,
                                    bool deriv) {
  const int n = cfg.sx, m = n / 2, m1 = m + 1;
  const int hb = pupil_band_rows(n, cfg.sz);
  const PupilLayout L = pupil_layout(n);
  double* B = ws.fw;             // row i of the band at (i - i_lo) * n
  double* By = B + 2 * hb * n;
  double* Bz = By + 2 * hb * n;
  double* rw = Bz + 2 * hb * n;  // the translated pupil function's row i (complex)
  double* rwy = rw + 2 * n;      // ... times -i ky
  double* rwz = rwy + 2 * n;     // ... times -i kz
  double* sxv = rwz + 2 * n;     // x shift per first index (complex)
  double* syv = sxv + 2 * n;     // y shift per second index (complex)
  double* szt = syv + 2 * n;     // z shift per pie-slice offset [m+1][m+1] (complex)
  const double* E = cfg.fft + L.e;
  const double* PF = cfg.fft + L.pf;
  const double* KX = cfg.fft + L.kx;
  const double* KY = cfg.fft + L.ky;
  const double* KZ = cfg.fft + L.kz;
  const double* KZS = cfg.fft + L.kzs;
  // pfitCalcPeakShape :148-150
  const double dx = w.p[PX] - (double)w.xi, dy = w.p[PY] - (double)w.yi, dz = w.p[PZ];
  // shift vectors, pfnTranslate :453-463 (both from kx's first column)
  for (int i = lane; i < 2 * n; i += 32) {
    const int j = i < n ? i : i - n;
    const double dd = __ldg(KX + j) * (i < n ? dx : dy);
    double sv, cv;
    sincos(dd, &sv, &cv);
    double* o = (i < n ? sxv : syv) + 2 * j;
    o[0] = cv;
    o[1] = -sv;
  }
  // z shift over the pie slice, :475-486 (with -dz); symmetric in (a, b)
  for (int q = lane; q < m1 * m1; q += 32) {
    const int a = q / m1, b = q - a * m1;
    if (a <= b) {
      const double dd = -__ldg(KZS + q) * dz;
      double sv, cv;
      sincos(dd, &sv, &cv);
      szt[2 * q] = cv;
      szt[2 * q + 1] = -sv;
      szt[2 * (b * m1 + a)] = cv;
      szt[2 * (b * m1 + a) + 1] = -sv;
    }
  }
  __syncwarp();
  const int i_lo = (int)__ldg(cfg.fft + L.band), i_hi = (int)__ldg(cfg.fft + L.band + 1);
  for (int i = i_lo; i <= i_hi; i++) {
    const double xr = sxv[2 * i], xc = sxv[2 * i + 1];
    const int oa = abs(i - m) * m1;
    const int k_lo = (int)__ldg(cfg.fft + L.rng + 2 * i), k_hi = (int)__ldg(cfg.fft + L.rng + 2 * i + 1);
    for (int k = k_lo + lane; k <= k_hi; k += 32) {
      const int o = oa + abs(k - m);
      // the reference's products in its order, :488-505
      const double r2 = xr * syv[2 * k] - xc * syv[2 * k + 1];
      const double c2 = xr * syv[2 * k + 1] + xc * syv[2 * k];
      const double r1 = r2 * szt[2 * o] - c2 * szt[2 * o + 1];
      const double c1 = r2 * szt[2 * o + 1] + c2 * szt[2 * o];
      const double pr = __ldg(PF + 2 * (i * n + k)), pc = __ldg(PF + 2 * (i * n + k) + 1);
      const double wr = r1 * pr - c1 * pc, wc = r1 * pc + c1 * pr;
      rw[2 * k] = wr;
      rw[2 * k + 1] = wc;
      if (deriv) {
        // times -i k: (wr, wc) -> (wc k, -wr k), pfnGetPSFdy / dz :165-168, :190-193
        const double ky = __ldg(KY + i * n + k), kz = __ldg(KZ + i * n + k);
        rwy[2 * k] = wc * ky;
        rwy[2 * k + 1] = -wr * ky;
        rwz[2 * k] = wc * kz;
        rwz[2 * k + 1] = -wr * kz;
      }
    }
    __syncwarp();
    if (deriv) {
      for (int v = lane; v < n; v += 32) {
        double br = 0.0, bc = 0.0, yr = 0.0, yc = 0.0, zr = 0.0, zc = 0.0;
        for (int k = k_lo; k <= k_hi; k++) {
          const double er = __ldg(E + 2 * (k * n + v)), ei = __ldg(E + 2 * (k * n + v) + 1);
          br += rw[2 * k] * er - rw[2 * k + 1] * ei;
          bc += rw[2 * k] * ei + rw[2 * k + 1] * er;
          yr += rwy[2 * k] * er - rwy[2 * k + 1] * ei;
          yc += rwy[2 * k] * ei + rwy[2 * k + 1] * er;
          zr += rwz[2 * k] * er - rwz[2 * k + 1] * ei;
          zc += rwz[2 * k] * ei + rwz[2 * k + 1] * er;
        }
        const int o = 2 * ((i - i_lo) * n + v);
        B[o] = br;
        B[o + 1] = bc;
        By[o] = yr;
        By[o + 1] = yc;
        Bz[o] = zr;
        Bz[o + 1] = zc;
      }
    } else {
      for (int v = lane; v < n; v += 32) {
        double br = 0.0, bc = 0.0;
        for (int k = k_lo; k <= k_hi; k++) {
          const double er = __ldg(E + 2 * (k * n + v)), ei = __ldg(E + 2 * (k * n + v) + 1);
          br += rw[2 * k] * er - rw[2 * k + 1] * ei;
          bc += rw[2 * k] * ei + rw[2 * k + 1] * er;
        }
        B[2 * ((i - i_lo) * n + v)] = br;
        B[2 * ((i - i_lo) * n + v) + 1] = bc;
      }
    }
    __syncwarp();
  }
}

// The PSF |psf|^2 at ROI pixel (rx, ry) from pupil_tables' B arrays
// (pfitCalcPeakShape :164-169); with g non-null also Re(conj(psf) d) for the
// x, y and z derivatives d (pfitCalcJH3D :103-106 without the 2 h rqe
// factor; dz negated as pfnGetPSFdz :199-201).
__device__ inline double pupil_pixel(const ModelCfg& cfg, const double* fw, int rx, int ry, double* g) {
  const int n = cfg.sx;
  const int hb = pupil_band_rows(n, cfg.sz);
  const PupilLayout L = pupil_layout(n);
  const double* B = fw;          // row i of the band at (i - i_lo) * n
  const double* By = B + 2 * hb * n;
  const double* Bz = By + 2 * hb * n;
  const double* E = cfg.fft + L.e;
  const double* KX = cfg.fft + L.kx;
  const int i_lo = (int)__ldg(cfg.fft + L.band), i_hi = (int)__ldg(cfg.fft + L.band + 1);
  double pr = 0.0, pc = 0.0;
  if (!g) {
    for (int i = i_lo; i <= i_hi; i++) {
      const double er = __ldg(E + 2 * (i * n + rx)), ei = __ldg(E + 2 * (i * n + rx) + 1);
      const int o = 2 * ((i - i_lo) * n + ry);
      pr += B[o] * er - B[o + 1] * ei;
      pc += B[o] * ei + B[o + 1] * er;
    }
    return pr * pr + pc * pc;
  }
  double xr = 0.0, xc = 0.0, yr = 0.0, yc = 0.0, zr = 0.0, zc = 0.0;
  for (int i = i_lo; i <= i_hi; i++) {
    const double er = __ldg(E + 2 * (i * n + rx)), ei = __ldg(E + 2 * (i * n + rx) + 1);
    const int o = 2 * ((i - i_lo) * n + ry);
    const double tr = B[o] * er - B[o + 1] * ei, tc = B[o] * ei + B[o + 1] * er;
    pr += tr;
    pc += tc;
    // times -i kx[i] (pfnGetPSFdx :140-143)
    const double kx = __ldg(KX + i);
    xr += tc * kx;
    xc -= tr * kx;
    yr += By[o] * er - By[o + 1] * ei;
    yc += By[o] * ei + By[o + 1] * er;
    zr += Bz[o] * er - Bz[o + 1] * ei;
    zc += Bz[o] * ei + Bz[o + 1] * er;
  }
  g[0] = pr * xr + pc * xc;
  g[1] = pr * yr + pc * yc;
  g[2] = pr * (-zr) + pc * (-zc);
  return pr * pr + pc * pc;
}

// Peak shape at ROI pixel p for the tables currently in the workspace.
template <typename T>
__device__ __forceinline__ T psf_at(const ModelCfg& cfg, const T* aij, const WarpWS<T>& ws,
                                    const SplinePos& s, int rx, int ry) {
  if (is_fft(cfg.model)) return (T)fft_pixel(cfg, ws.fw, rx, ry, nullptr);
  if (is_pupil(cfg.model)) return (T)pupil_pixel(cfg, ws.fw, rx, ry, nullptr);
  if (!is_spline(cfg.model)) {
    if constexpr (sizeof(T) == 4) return g32_psf(ws.tab0, ws.ts, rx, ry).h;
    else return mul_rn(ws.eyt[ry], ws.ext[rx]);
  }
  if constexpr (sizeof(T) == 4) {
    return spline_value_ff(cfg, aij, ws, s, rx, ry).h;
  } else {
    const int nc = (cfg.model == M_SPLINE3D) ? 64 : 16;
    const T* c = spline_cell(cfg, aij, s.zi, ry + s.ys, rx + s.xs);
    return spline_dot(c, ws.ext, nc);
  }
}

// Widths from z for the Z model, daoCalcWidthsFromZ dao_fit.c:1009-1035.
__device__ inline void widths_from_z(const ModelCfg& cfg, PeakRec& w) {
  double z0 = (w.p[PZ] - cfg.wx[1]) / cfg.wx[2];
  double z1 = z0 * z0, z2 = z1 * z0, z3 = z2 * z0;
  double t = 1.0 + z1 + cfg.wx[3] * z2 + cfg.wx[4] * z3;
  w.wxt = t * t;
  w.p[PXW] = 2.0 / (cfg.wx[0] * t);
  z0 = (w.p[PZ] - cfg.wy[1]) / cfg.wy[2];
  z1 = z0 * z0;
  z2 = z1 * z0;
  z3 = z2 * z0;
  t = 1.0 + z1 + cfg.wy[3] * z2 + cfg.wy[4] * z3;
  w.wyt = t * t;
  w.p[PYW] = 2.0 / (cfg.wy[0] * t);
}

// ROI re-anchor, mFitUpdate multi_fit.c:1933-1946.
__device__ inline void anchor_update(PeakRec& w) {
  double dx = w.p[PX] - w.xi;
  if ((dx < -0.5) || (dx > 1.5)) w.xi = (int)floor(w.p[PX]);
  double dy = w.p[PY] - w.yi;
  if ((dy < -0.5) || (dy > 1.5)) w.yi = (int)floor(w.p[PY]);
}

// Apply the solved step in each model's delta order (dao_fit.c:1777-1880,
// cubic_fit.c:939-1005).  model is cfg.model (a constant where the caller
// is compiled for one model).
__device__ inline void apply_update(const ModelCfg& cfg, int model, PeakRec& w, const double* d) {
  switch (model) {
    case M_2DFIXED:
    case M_SPLINE2D:
      w.p[PH] -= d[0]; w.p[PX] -= d[1]; w.p[PY] -= d[2]; w.p[PBG] -= d[3];
      anchor_update(w);
      break;
    case M_2D:
      w.p[PH] -= d[0]; w.p[PX] -= d[1]; w.p[PY] -= d[2]; w.p[PXW] -= d[3]; w.p[PBG] -= d[4];
      w.p[PYW] = w.p[PXW];
      anchor_update(w);
      break;
    case M_3D:
      w.p[PH] -= d[0]; w.p[PX] -= d[1]; w.p[PXW] -= d[2]; w.p[PY] -= d[3]; w.p[PYW] -= d[4];
      w.p[PBG] -= d[5];
      anchor_update(w);
      break;
    case M_Z:
      w.p[PH] -= d[0]; w.p[PX] -= d[1]; w.p[PY] -= d[2]; w.p[PZ] -= d[3]; w.p[PBG] -= d[4];
      if (w.p[PZ] < cfg.zmin) w.p[PZ] = cfg.zmin;
      if (w.p[PZ] > cfg.zmax) w.p[PZ] = cfg.zmax;
      anchor_update(w);
      widths_from_z(cfg, w);
      break;
    case M_FFT: {
      // ftFitUpdate3D fft_fit.c:481-497 with ftFitZRangeCheck :506-524
      w.p[PH] -= d[0]; w.p[PX] -= d[1]; w.p[PY] -= d[2]; w.p[PZ] -= d[3]; w.p[PBG] -= d[4];
      anchor_update(w);
      const double max_z = ((double)cfg.sz) * 0.5 - 1.0e-12;
      if (w.p[PZ] < -max_z) w.p[PZ] = -max_z;
      if (w.p[PZ] > max_z) w.p[PZ] = max_z;
      break;
    }
    case M_PUPIL:
      // pfitUpdate3D pupil_fit.c:529-546 with pfitZRangeCheck :555-570
      w.p[PH] -= d[0]; w.p[PX] -= d[1]; w.p[PY] -= d[2]; w.p[PZ] -= d[3]; w.p[PBG] -= d[4];
      anchor_update(w);
      if (w.p[PZ] < cfg.zmin) w.p[PZ] = cfg.zmin;
      if (w.p[PZ] > cfg.zmax) w.p[PZ] = cfg.zmax;
      break;
    default: {  // M_SPLINE3D, with cfZRangeCheck
      w.p[PH] -= d[0]; w.p[PX] -= d[1]; w.p[PY] -= d[2]; w.p[PZ] -= d[3]; w.p[PBG] -= d[4];
      anchor_update(w);
      if (w.p[PZ] < 1.0e-12) w.p[PZ] = 1.0e-12;
      const double zmax = ((double)cfg.sz) - 1.0e-12;
      if (w.p[PZ] > zmax) w.p[PZ] = zmax;
      w.zi = (int)(w.p[PZ]);
      break;
    }
  }
}

// mFitCheck multi_fit.c:470-502; returns 0 (ok), 1 (margin), 2 (height).
__device__ inline int base_check(const ModelCfg& cfg, const PeakRec& w) {
  if ((w.xi < 0) || (w.xi >= (cfg.nx - cfg.roi)) || (w.yi < 0) || (w.yi >= (cfg.ny - cfg.roi)))
    return 1;
  if (w.p[PH] < 0.0) return 2;
  return 0;
}

// Model check with the width clamps of daoCheck2D / daoCheck3D
// (dao_fit.c:1061-1119).
__device__ inline int model_check(const ModelCfg& cfg, int model, PeakRec& w) {
  int c = base_check(cfg, w);
  if (c) return c;
  if ((model == M_2D) || (model == M_3D)) {
    if (w.p[PXW] < cfg.wmin) w.p[PXW] = cfg.wmin;
    else if (w.p[PXW] > cfg.wmax) w.p[PXW] = cfg.wmax;
  }
  if (model == M_3D) {
    if (w.p[PYW] < cfg.wmin) w.p[PYW] = cfg.wmin;
    else if (w.p[PYW] > cfg.wmax) w.p[PYW] = cfg.wmax;
  }
  return 0;
}

__device__ __forceinline__ int check_for(const ModelCfg& cfg, int model, PeakRec& w) {
  return is_arb(model) ? base_check(cfg, w) : model_check(cfg, model, w);
}

// Prepare the shape tables of peak w (all lanes) and return its spline
// position (unused for Gaussians).  deriv false: only the shape will be
// read (the pupil model then skips its derivative sums).
template <typename T>
__device__ inline SplinePos shape_tables(const ModelCfg& cfg, const PeakRec& w, WarpWS<T>& ws,
                                         int lane, bool deriv = true) {
  SplinePos s;
  if (is_fft(cfg.model)) {
    s.xs = s.ys = s.zi = 0;
    s.xd = s.yd = s.zd = 0.0;
    fft_tables(cfg, w, ws, lane);
  } else if (is_pupil(cfg.model)) {
    s.xs = s.ys = s.zi = 0;
    s.xd = s.yd = s.zd = 0.0;
    pupil_tables(cfg, w, ws, lane, deriv);
  } else if (is_spline(cfg.model)) {
    s = spline_pos(w.p, w.xi, w.yi, w.zi);
    spline_tables(cfg, s, ws, lane);
  } else {
    s.xs = s.ys = s.zi = 0;
    s.xd = s.yd = s.zd = 0.0;
    if constexpr (sizeof(T) == 4) g32_tables(cfg, w, ws.tab0, ws.ts, lane);
    else gauss_tables(cfg, w.p, w.xi, w.yi, ws, lane);
  }
  __syncwarp();
  return s;
}

__device__ __forceinline__ void roi_rc(const unsigned short* roi_xy, int p, int& rx, int& ry) {
  unsigned short v = roi_xy[p];
  rx = v & 0xff;
  ry = v >> 8;
}

// Per-pixel Jacobian row jt (MLE models): daoCalcJH2DFixed dao_fit.c:48-105,
// daoCalcJH2D :409-467, daoCalcJH3D :811-871, daoCalcJHZ :883-958,
// cfCalcJH2D cubic_fit.c:48-108, cfCalcJH3D :120-182.
template <typename T>
__device__ __forceinline__ void jt_row(const ModelCfg& cfg, const T* aij, const WarpWS<T>& ws,
                                       const SplinePos& s, const PeakRec& w, T gx, T gy, int rx,
                                       int ry, T rq, T psf, T* jt) {
  const T h = (T)w.p[PH];
  switch (cfg.model) {
    case M_2DFIXED: {
      const T e_t = psf, wd = (T)w.p[PXW];
      jt[0] = rq * e_t;
      jt[1] = rq * (T)2 * h * wd * ws.xt[rx] * e_t;
      jt[2] = rq * (T)2 * h * wd * ws.yt[ry] * e_t;
      jt[3] = rq;
      break;
    }
    case M_2D: {
      const T e_t = psf, wd = (T)w.p[PXW], xt = ws.xt[rx], yt = ws.yt[ry];
      jt[0] = rq * e_t;
      jt[1] = rq * (T)2 * h * wd * xt * e_t;
      jt[2] = rq * (T)2 * h * wd * yt * e_t;
      jt[3] = rq * (-h * xt * xt * e_t - h * yt * yt * e_t);
      jt[4] = rq;
      break;
    }
    case M_3D: {
      const T e_t = psf, xt = ws.xt[rx], yt = ws.yt[ry];
      jt[0] = rq * e_t;
      jt[1] = rq * (T)2 * h * (T)w.p[PXW] * xt * e_t;
      jt[2] = rq * (-h * xt * xt * e_t);
      jt[3] = rq * (T)2 * h * (T)w.p[PYW] * yt * e_t;
      jt[4] = rq * (-h * yt * yt * e_t);
      jt[5] = rq;
      break;
    }
    case M_Z: {
      const T e_t = psf, xt = ws.xt[rx], yt = ws.yt[ry];
      jt[0] = rq * e_t;
      jt[1] = rq * (T)2 * h * (T)w.p[PXW] * xt * e_t;
      jt[2] = rq * (T)2 * h * (T)w.p[PYW] * yt * e_t;
      jt[3] = rq * (-h * xt * xt * gx * e_t - h * yt * yt * gy * e_t);
      jt[4] = rq;
      break;
    }
    case M_FFT: {
      // ftFitCalcJH3D fft_fit.c:90-100
      double g[3];
      fft_pixel(cfg, ws.fw, rx, ry, g);
      jt[0] = rq * psf;
      jt[1] = rq * h * (T)g[0];
      jt[2] = rq * h * (T)g[1];
      jt[3] = rq * h * (T)g[2];
      jt[4] = rq;
      break;
    }
    case M_PUPIL: {
      // pfitCalcJH3D pupil_fit.c:103-107
      double g[3];
      pupil_pixel(cfg, ws.fw, rx, ry, g);
      jt[0] = rq * psf;
      jt[1] = rq * (T)2 * h * (T)g[0];
      jt[2] = rq * (T)2 * h * (T)g[1];
      jt[3] = rq * (T)2 * h * (T)g[2];
      jt[4] = rq;
      break;
    }
    case M_SPLINE3D: {
      const T* c = spline_cell(cfg, aij, s.zi, ry + s.ys, rx + s.xs);
      T dx = (T)0, dy = (T)0, dz = (T)0;
#pragma unroll 8
      for (int i = 0; i < 64; i++) {
        const T ci = __ldg(c + i);
        dx = fma_rn(ci, ws.ext[64 + i], dx);
        dy = fma_rn(ci, ws.eyt[i], dy);
        dz = fma_rn(ci, ws.eyt[64 + i], dz);
      }
      jt[0] = rq * psf;
      jt[1] = -rq * h * dx;
      jt[2] = -rq * h * dy;
      jt[3] = rq * h * dz;
      jt[4] = rq;
      break;
    }
    default: {  // M_SPLINE2D
      const T* c = spline_cell(cfg, aij, 0, ry + s.ys, rx + s.xs);
      T dx = (T)0, dy = (T)0;
#pragma unroll 8
      for (int i = 0; i < 16; i++) {
        const T ci = __ldg(c + i);
        dx = fma_rn(ci, ws.ext[64 + i], dx);
        dy = fma_rn(ci, ws.eyt[i], dy);
      }
      jt[0] = rq * psf;
      jt[1] = -rq * h * dx;
      jt[2] = -rq * h * dy;
      jt[3] = rq;
      break;
    }
  }
}

// ---------------------------------------------------------------------------
// differential shape evaluation (FP32 engine)
//
// For a trial at the same ROI anchor the change of the peak shape is
// computed from differences that are accurate relative to the step:
//  Gaussian: ext1 - ext0 = ext0 * expm1(a1 - a0), a = -t^2 w, with
//            a1 - a0 = -[dt (2 t0 + dt) w1 + t0^2 (w1 - w0)], dt = -(x1 - x0);
//  spline:   m1 - m0 for each monomial x^a y^b z^c, telescoped as
//            d(x^a) y1^b z1^c + x0^a d(y^b) z1^c + x0^a y0^b d(z^c),
//            d(p^n) = dp * sum_j p1^j p0^(n-1-j).
// Tables: Gaussian start factors at ext[64+i] / eyt[64+i], differences at
// xt[64+i] / yt[64+i]; spline monomial differences at xt[0..63].
// ---------------------------------------------------------------------------

template <typename T>
__device__ inline void diff_tables(const ModelCfg& cfg, const PeakRec& w0, const PeakRec& w1,
                                   const SplinePos& s0, const SplinePos& s1, WarpWS<T>& ws, int lane) {
  if (!is_spline(cfg.model)) {
    // per-warp scalars from the FP64 parameters (differences taken in FP64)
    const float xo0 = (float)(-(w0.p[PX] - (double)w0.xi) - cfg.xoff);
    const float yo0 = (float)(-(w0.p[PY] - (double)w0.yi) - cfg.xoff);
    const float dtx = (float)(w0.p[PX] - w1.p[PX]);
    const float dty = (float)(w0.p[PY] - w1.p[PY]);
    const float wx1 = (float)w1.p[PXW], dwx = (float)(w1.p[PXW] - w0.p[PXW]);
    const float wy1 = (float)w1.p[PYW], dwy = (float)(w1.p[PYW] - w0.p[PYW]);
    for (int i = lane; i < cfg.roi; i += 32) {
      const float tx = (float)i + xo0, ty = (float)i + yo0;
      const float dax = -(dtx * (2.0f * tx + dtx) * wx1 + tx * tx * dwx);
      const float day = -(dty * (2.0f * ty + dty) * wy1 + ty * ty * dwy);
      ws.xt[64 + i] = ws.ext[64 + i] * (T)expm1f(dax);
      ws.yt[64 + i] = ws.eyt[64 + i] * (T)expm1f(day);
    }
  } else {
    const double x0 = clamp01(s0.xd), x1 = clamp01(s1.xd);
    const double y0 = clamp01(s0.yd), y1 = clamp01(s1.yd);
    const double z0 = clamp01(s0.zd), z1 = clamp01(s1.zd);
    const T dx = (T)(x1 - x0), dy = (T)(y1 - y0), dz = (T)(z1 - z0);
    const T X0 = (T)x0, X1 = (T)x1, Y0 = (T)y0, Y1 = (T)y1, Z0 = (T)z0, Z1 = (T)z1;
    const bool three = (cfg.model == M_SPLINE3D);
    const int nmono = three ? 64 : 16;
    for (int id = lane; id < nmono; id += 32) {
      const int a = three ? (id >> 4) : (id >> 2);
      const int b = three ? ((id >> 2) & 3) : (id & 3);
      const int c = three ? (id & 3) : 0;
      // d(p^n) via the telescoped sum
      T sx = (T)0, sy = (T)0, sz = (T)0;
      for (int j = 0; j < a; j++) sx += pw(X1, j) * pw(X0, a - 1 - j);
      for (int j = 0; j < b; j++) sy += pw(Y1, j) * pw(Y0, b - 1 - j);
      for (int j = 0; j < c; j++) sz += pw(Z1, j) * pw(Z0, c - 1 - j);
      ws.xt[id] = (dx * sx) * pw(Y1, b) * pw(Z1, c) + pw(X0, a) * (dy * sy) * pw(Z1, c) +
                  pw(X0, a) * pw(Y0, b) * (dz * sz);
    }
  }
}

// Trial shape (canonical, from the trial tables) and its change from the
// start of the step at ROI pixel (rx, ry).
template <typename T>
__device__ __forceinline__ void psf_and_delta(const ModelCfg& cfg, const T* aij, const WarpWS<T>& ws,
                                              const SplinePos& s, int rx, int ry, T& psf, T& dpsf) {
  if (!is_spline(cfg.model)) {
    psf = mul_rn(ws.eyt[ry], ws.ext[rx]);
    const T ex0 = ws.ext[64 + rx], dex = ws.xt[64 + rx];
    const T ey0 = ws.eyt[64 + ry], dey = ws.yt[64 + ry];
    dpsf = ey0 * dex + dey * (ex0 + dex);
    return;
  }
  const int nc = (cfg.model == M_SPLINE3D) ? 64 : 16;
  const T* c = spline_cell(cfg, aij, s.zi, ry + s.ys, rx + s.xs);
  T acc = (T)0, dacc = (T)0;
#pragma unroll 8
  for (int i = 0; i < nc; i++) {
    const T ci = __ldg(c + i);
    acc = fma_rn(ci, ws.ext[i], acc);
    dacc = fma_rn(ci, ws.xt[i], dacc);
  }
  psf = acc;
  dpsf = dacc;
}

// ---------------------------------------------------------------------------
// Damped solve of the FP32 engine (warp-collective).
//
// The reference solves (H + lam diag H) d = b in FP64 with dposv
// (multi_fit.c:1839-1883).  Here lane i (< k) holds row i of the system:
// the rows are Jacobi-scaled to unit diagonal and eliminated in FP32
// without pivoting (the matrix is symmetric positive definite; a pivot
// <= 0 means it is not, numerically), pivot rows broadcast by shuffles.
// The solution is refined twice with the residual b - A d evaluated in
// FP64 (one row per lane), which leaves an error of about
// (cond(A_scaled) * 2^-24)^3.  When a pivot is not positive the FP64
// Cholesky on lane 0 decides, exactly as dposv does.  The solution
// (lane 0) is written to out[0..k).
// ---------------------------------------------------------------------------

template <typename T>
__device__ inline int solve_damped(WarpWS<T>& ws, int k, double lam, double* out, int lane) {
  return solve_fp64_warp(ws.jh, k, lam, out, lane);
}

// Forward and back substitution with the factors held in r (multipliers
// left of the diagonal, U from the diagonal on), one row per lane.
__device__ __forceinline__ float lu_substitute(const float (&r)[MAX_JAC], float c, int k, int lane) {
#pragma unroll
  for (int j = 0; j < MAX_JAC; j++) {
    if (j < k) {
      const float cj = __shfl_sync(0xffffffffu, c, j);
      if (lane > j && lane < k) c = fmaf(-r[j], cj, c);
    }
  }
#pragma unroll
  for (int j = MAX_JAC - 1; j >= 0; j--) {
    if (j < k) {
      if (lane == j) c = __fdiv_rn(c, r[j]);
      const float xj = __shfl_sync(0xffffffffu, c, j);
      if (lane < j) c = fmaf(-r[j], xj, c);
    }
  }
  return c;
}

template <>
__device__ inline int solve_damped<float>(WarpWS<float>& ws, int k, double lam, double* out, int lane) {
  const double* jh = ws.jh;
  const bool act = lane < k;
  double Ai[MAX_JAC];
  float r[MAX_JAC];
  double bi = 0.0, dii = 1.0;
#pragma unroll
  for (int j = 0; j < MAX_JAC; j++) {
    Ai[j] = 0.0;
    if (act && j < k) {
      const double a = jh[hes_index(k, lane, j)];
      Ai[j] = (j == lane) ? (1.0 + lam) * a : a;
      if (j == lane) dii = Ai[j];
    }
  }
  if (act) bi = jh[lane];
  const float dfl = (float)dii;
  const bool bad = act && (!(dii > 0.0) || !(dfl > 1.0e-30f) || !(dfl < 1.0e30f));
  int status = __any_sync(0xffffffffu, bad) ? 2 : 0;
  const float si = act && !bad ? rsqrtf(dfl) : 0.0f;
  if (status == 0) {
#pragma unroll
    for (int j = 0; j < MAX_JAC; j++) {
      const float sj = __shfl_sync(0xffffffffu, si, j);
      r[j] = (act && j < k) ? ((float)Ai[j] * si) * sj : 0.0f;
    }
    // elimination, pivot row j broadcast from lane j
#pragma unroll
    for (int j = 0; j < MAX_JAC; j++) {
      if (j < k && status == 0) {
        const float piv = __shfl_sync(0xffffffffu, r[j], j);
        if (!(piv > 0.0f)) {
          status = 2;
        } else {
          const bool below = act && lane > j;
          const float m = below ? __fdiv_rn(r[j], piv) : 0.0f;
#pragma unroll
          for (int l = j + 1; l < MAX_JAC; l++) {
            if (l < k) {
              const float pl = __shfl_sync(0xffffffffu, r[l], j);
              if (below) r[l] = fmaf(-m, pl, r[l]);
            }
          }
          if (below) r[j] = m;
        }
      }
    }
  }
  if (status == 0) {
    float c = act ? (float)bi * si : 0.0f;
    c = lu_substitute(r, c, k, lane);
    double xs = act ? (double)(c * si) : 0.0;
    for (int it = 0; it < 2; it++) {
      double res = bi;
#pragma unroll
      for (int j = 0; j < MAX_JAC; j++) {
        if (j < k) {
          const double dj = __shfl_sync(0xffffffffu, xs, j);
          if (act) res = fma(-Ai[j], dj, res);
        }
      }
      c = act ? (float)res * si : 0.0f;
      c = lu_substitute(r, c, k, lane);
      if (act) xs += (double)(c * si);
    }
#pragma unroll
    for (int j = 0; j < MAX_JAC; j++) {
      if (j < k) {
        const double v = __shfl_sync(0xffffffffu, xs, j);
        if (lane == 0) {
          out[j] = v;
          if (isnan(v)) status = 1;   // multi_fit.c:1857-1863
        }
      }
    }
  }
  if (lane == 0 && status == 2) status = solve_fp64_lane0(jh, k, lam, out);
  return status;
}

// d width / dz factors of the Z model (dao_fit.c:904-916).
__device__ inline void z_factors(const ModelCfg& cfg, int model, const PeakRec& w, double& gx,
                                 double& gy) {
  gx = gy = 0.0;
  if (model != M_Z) return;
  double z0 = (w.p[PZ] - cfg.wx[1]) / cfg.wx[2];
  double z1 = z0 * z0, z2 = z1 * z0;
  double zt = 2.0 * z0 + 3.0 * cfg.wx[3] * z1 + 4.0 * cfg.wx[4] * z2;
  gx = -2.0 * zt / (cfg.wx[0] * w.wxt);
  z0 = (w.p[PZ] - cfg.wy[1]) / cfg.wy[2];
  z1 = z0 * z0;
  z2 = z1 * z0;
  zt = 2.0 * z0 + 3.0 * cfg.wy[3] * z1 + 4.0 * cfg.wy[4] * z2;
  gy = -2.0 * zt / (cfg.wy[0] * w.wyt);
}

__device__ __forceinline__ long long pix_index(const ModelCfg& cfg, int xi, int yi, int rx, int ry) {
  return (long long)(yi + ry) * cfg.nx + (xi + rx);
}

// Quantisation of a contribution in the pixel type: FP32 contributions go
// to one word with float-only instructions (the value v * 2^36 is exact in
// float, so rounding it to an integer equals acc_quant<1>), FP64 ones to two.
template <typename T>
__device__ __forceinline__ Q2 quant_t(T v);
template <>
__device__ __forceinline__ Q2 quant_t<float>(float v) {
  Q2 q;
  q.h = fx_round(v * 68719476736.0f);
  q.l = 0;
  return q;
}
template <>
__device__ __forceinline__ Q2 quant_t<double>(double v) {
  return acc_quant<2>(v);
}

// One-word accumulator value as float (FP32 engine).
__device__ __forceinline__ float fx_to_float(long long q) {
  float a, b, c;
  if (fx_split(q, a, b, c)) return __fadd_rn(a, __fadd_rn(b, c));
  return __ll2float_rn(q) * 1.4551915228366852e-11f;   // 2^-36
}

// Accumulator access: pixel i of a W-word array (see acc_quant).
template <int W>
__device__ __forceinline__ Q2 acc_load(const long long* a, long long i) {
  Q2 q;
  q.h = __ldcg(a + i * W);
  q.l = (W == 2) ? __ldcg(a + i * W + 1) : 0;
  return q;
}

template <int W>
__device__ __forceinline__ void acc_red(long long* a, long long i, Q2 q, int sign) {
  unsigned long long* p = reinterpret_cast<unsigned long long*>(a + i * W);
  atomicAdd(p, (unsigned long long)(sign > 0 ? q.h : -q.h));
  if (W == 2) atomicAdd(p + 1, (unsigned long long)(sign > 0 ? q.l : -q.l));
}

__device__ __forceinline__ Q2 q_sub(Q2 a, Q2 b) {
  Q2 r;
  r.h = a.h - b.h;
  r.l = a.l - b.l;
  return r;
}

// Add (sign +1) or subtract (sign -1) a peak's contribution over its ROI
// with integer atomics (mFitAddPeak multi_fit.c:28-57, mFitSubtractPeak
// :1894-1922).  The shape tables of w must be in the workspace.
template <typename T>
__device__ inline void add_peak(const ModelCfg& cfg, const FrameSet<T>& fs, long long fbase,
                                const PeakRec& w, const SplinePos& s, const WarpWS<T>& ws,
                                int sign, int lane) {
  constexpr int W = AccW<T>::W;
  if constexpr (sizeof(T) == 4) {
    if (!is_spline(cfg.model)) {
      const ff H = ff_from_double(w.p[PH]), BG = ff_from_double(w.p[PBG]);
      for (int p = lane; p < cfg.nroi; p += 32) {
        int rx, ry;
        roi_rc(fs.roi_xy, p, rx, ry);
        const long long k = pix_index(cfg, w.xi, w.yi, rx, ry);
        Q2 qf, qb;
        g32_contrib(ws.tab0, ws.ts, H, BG, rx, ry, __ldg(fs.rqe + k), __ldg(fs.scmos + k), qf, qb);
        acc_red<1>(fs.f, fbase + k, qf, sign);
        acc_red<1>(fs.bg, fbase + k, qb, sign);
        atomicAdd(fs.cnt + fbase + k, sign);
      }
      return;
    }
  }
  if constexpr (sizeof(T) == 4) {
    // FP32 splines
    const ff H = ff_from_double(w.p[PH]), BG = ff_from_double(w.p[PBG]);
    for (int p = lane; p < cfg.nroi; p += 32) {
      int rx, ry;
      roi_rc(fs.roi_xy, p, rx, ry);
      const long long k = pix_index(cfg, w.xi, w.yi, rx, ry);
      Q2 qf, qb;
      spl32_contrib(spline_value_ff(cfg, fs.aij, ws, s, rx, ry), H, BG, __ldg(fs.rqe + k), __ldg(fs.scmos + k),
                    qf, qb);
      acc_red<1>(fs.f, fbase + k, qf, sign);
      acc_red<1>(fs.bg, fbase + k, qb, sign);
      atomicAdd(fs.cnt + fbase + k, sign);
    }
    return;
  }
  for (int p = lane; p < cfg.nroi; p += 32) {
    int rx, ry;
    roi_rc(fs.roi_xy, p, rx, ry);
    const long long k = pix_index(cfg, w.xi, w.yi, rx, ry);
    const T rq = __ldg(fs.rqe + k), sc = __ldg(fs.scmos + k);
    const T psf = psf_at(cfg, fs.aij, ws, s, rx, ry);
    acc_red<W>(fs.f, fbase + k, quant_t<T>(contrib_f(w.p[PH], psf, rq)), sign);
    acc_red<W>(fs.bg, fbase + k, quant_t<T>(contrib_bg(w.p[PBG], rq, sc)), sign);
    atomicAdd(fs.cnt + fbase + k, sign);
  }
}

// Pixel model value from the global accumulator state (f + bg/cnt, multi_fit.c:143).
template <typename T>
__device__ __forceinline__ double fi_global(const FrameSet<T>& fs, long long g) {
  constexpr int W = AccW<T>::W;
  return acc_value<W>(acc_load<W>(fs.f, g)) + acc_value<W>(acc_load<W>(fs.bg, g)) / (double)__ldcg(fs.cnt + g);
}

}  // namespace sa
