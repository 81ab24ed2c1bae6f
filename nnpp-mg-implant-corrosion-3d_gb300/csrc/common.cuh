// common.cuh -- device helpers and internal data structures of the GB300 NNPP library.
#ifndef NNPP_COMMON_CUH
#define NNPP_COMMON_CUH

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "nnpp_gb300.h"
#include "nnpp_internal.h"

namespace nnpp {

// A named range of a C-ABI call for profilers and tracers (NVTX; nothing is recorded unless a
// tool is attached).
struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

constexpr int S = NNPP_NSPECIES;
constexpr int kReduceSlots = 24;   // values reduced per block by the step kernels
constexpr int kHistMax = 6;        // potentials kept for the warm start of the solve
constexpr int kMaxPartialBlocks = 4096;

// CUDA call check inside functions returning nnpp_status.
#define NNPP_CUDA(call)                                                                     \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return ::nnpp::set_error(NNPP_ERR_CUDA, std::string(#call) + ": " +                   \
                                                  cudaGetErrorString(e_));                  \
  } while (0)

#define NNPP_TRY(call)                  \
  do {                                  \
    nnpp_status s_ = (call);            \
    if (s_ != NNPP_OK) return s_;       \
  } while (0)

// ---------------------------------------------------------------------------------------
// Node records gathered by the bond kernels: one 32-byte (FP32) or 64-byte (FP64) aligned
// record per node, so that a neighbour costs one or two sectors.
struct __align__(32) Rec32 {
  float c[S];     // concentrations (high word of the compensated pair)
  float phi_hi;   // potential, high word
  float phi_lo;   // potential, low word (phi = phi_hi + phi_lo to ~1e-14 absolute)
  float phase;    // 1 solid, 0 liquid
  float pad;
};

struct __align__(32) Rec64 {
  double c[S];
  double phi;
  double phase;
  double pad[2];
};

// Scalars that live on the device for the whole run (diagnostics, CG state, counters).
struct DevState {
  // diagnostics (nnpp_diag)
  long long steps;
  long long solid_count;
  double voln1rel;
  double vol0rel;
  double BV;  // 10^(-vol_red (1 - voln1rel)), refreshed with voln1rel
  double mass[S];
  double mg_mass_t0;
  double dissolved;
  long long cg_iters;
  long long cg_solves;
  long long cg_nc;
  double last_relres;
  long long outer_total;
  int nonfinite;
  int wait_timeout;   // a bounded device wait gave up (the step's results are invalid)
  int bounds_error;   // a device index check (nnpp_set_checks) found an index out of range
  int nflip;          // nodes the last transport turned liquid (listed in flip_list; reset
                      // by the next-guess pass that follows the transport)
  // potential solve
  double bnorm2;      // ||b_eff||^2
  double rnorm2;      // ||r||^2 of the outer (FP64) residual
  double rr0;         // inner: ||r||^2 at start
  double rr;          // inner: current ||r||^2
  double rz;          // inner: r.z
  double alpha, beta;
  double pq;          // inner: p.A p of the current direction (deflated CG's step length)
  double tol;         // relative tolerance of the solve
  double inner_rel;   // inner relative reduction per refinement sweep
  double inner_target;  // inner: stop when ||r||^2 <= inner_target
  int inner_it;
  int outer_it;
  int max_iter;
  int max_outer;
  int solve_iters;    // inner iterations of the current solve
  int outer_active;   // this instance still refines its potential
  int inner_active;   // this instance still iterates its inner CG
  int op_valid;       // freem, dsum, dinv, d32 and the Dirichlet coupling hold the current
                      // phases' values (cleared by a flip or a state change)
  // per-step mass-curve sampling (adjoint forward)
  double mg_mass_now;
  // adjoint accumulators: dL/dD_liquid[0..3], dL/dk_diss
  double adj_g[5];
  // warm start of the potential solve from the last hist_n solutions (ring, newest at
  // hist_head): coefficients of their divided differences for the next initial guess
  int hist_n;
  int hist_head;
  int warm_nd;        // differences used by the next guess (0: keep the extrapolation)
  int defl;           // 1: the coarse operator and A P match the current phases (the mixed
                      // inner CG runs deflated); cleared by a flip or a phase change
  double warm_coef[kHistMax];
  // block tickets for last-block reductions
  unsigned int ticket[8];
};

// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void two_sum_d(double a, double b, double& s, double& e) {
  s = a + b;
  double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (hi, lo) += a * b on FP32 pairs: the product's rounding error from an FMA, the sum's
// from TwoSum.  A dot product accumulated this way is as accurate as an FP64 one and runs
// on the FP32 pipes (the GB300's FP64 rate is a small fraction of its FP32 rate).
__device__ __forceinline__ void pair_fma(float& hi, float& lo, float a, float b) {
  const float p = a * b;
  const float pe = fmaf(a, b, -p);
  float s, e;
  two_sum(hi, p, s, e);
  hi = s;
  lo += e + pe;
}

// warp sum of FP32 pairs (hi, lo) with TwoSum at each level; lane 0 holds the pair sum to
// ~2^-48 relative (as good as an FP64 sum of 32 terms, on the FP32 pipes)
__device__ __forceinline__ void pair_warp_sum(float& hi, float& lo) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float oh = __shfl_down_sync(0xffffffffu, hi, off);
    const float ol = __shfl_down_sync(0xffffffffu, lo, off);
    float sum, err;
    two_sum(hi, oh, sum, err);
    hi = sum;
    lo = lo + ol + err;
  }
}

// FP32 pairs (hi, lo) standing in for FP64 where GB300's FP64 rate would bound a bond pass:
// products by FMA-based TwoProd, sums by TwoSum; ~2^-46 relative per operation.
__device__ __forceinline__ void pair_add(float& sh, float& sl, float ah, float al) {
  float s, e;
  two_sum(sh, ah, s, e);
  sh = s;
  sl += e + al;
}
__device__ __forceinline__ void pair_mul(float ah, float al, float bh, float bl, float& ph, float& pl) {
  ph = ah * bh;
  pl = fmaf(ah, bh, -ph) + fmaf(ah, bl, al * bh);
}
// FP32 pair (hi, lo) of a double by bit manipulation, with no FP64 arithmetic: hi keeps the
// leading 24 significant bits (truncated), lo the rest rounded to 24 bits, so that
// |t - hi - lo| <= 2^-48 |t|.  Zero and subnormals give (0, 0); magnitudes outside
// [2^-60, 2^100) and non-finite values take the FP64 conversion.
__device__ __forceinline__ void split_pair(double t, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(t);
  const int e = (int)((b >> 52) & 0x7ffu);
  if (e == 0) {
    hi = lo = 0.0f;
    return;
  }
  if (e < 1023 - 60 || e >= 1023 + 100) {
    hi = (float)t;
    lo = isfinite(hi) ? (float)(t - (double)hi) : 0.0f;
    return;
  }
  const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
  const unsigned long long m = b & 0xfffffffffffffull;
  hi = __uint_as_float(sign | ((unsigned int)(e - 1023 + 127) << 23) | (unsigned int)(m >> 29));
  const float r = (float)(unsigned int)(m & 0x1fffffffu) * 0x1p-29f;            // in [0, 1)
  const float sc = __uint_as_float((unsigned int)(e - 1023 - 23 + 127) << 23);  // 2^(E-23)
  lo = __uint_as_float(__float_as_uint(r * sc) | sign);
}
// (ah, al) - (bh, bl), renormalised (|lo| <= half an ulp of hi)
__device__ __forceinline__ void pair_sub(float ah, float al, float bh, float bl, float& dh, float& dl) {
  float s, e;
  two_sum(ah, -bh, s, e);
  e += al - bl;
  dh = s + e;
  dl = e - (dh - s);
}
// Sum of products a*b of one thread: FP64 on the FP64 path, FP32 pairs on the FP32 path.
template <typename P>
struct DotAcc;
template <>
struct DotAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double a, double b) { s += a * b; }
  __device__ __forceinline__ void warp_sum() {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  }
  __device__ __forceinline__ double value() const { return s; }
};
template <>
struct DotAcc<float> {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add(float a, float b) { pair_fma(hi, lo, a, b); }
  // += (ah + al) * (bh + bl), the product of two pairs to ~2^-46 relative
  __device__ __forceinline__ void add_pair(float ah, float al, float bh, float bl) {
    const float p = ah * bh;
    const float pe = fmaf(ah, bh, -p) + fmaf(ah, bl, al * bh);
    float s, e;
    two_sum(hi, p, s, e);
    hi = s;
    lo += e + pe;
  }
  __device__ __forceinline__ void warp_sum() { pair_warp_sum(hi, lo); }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Compensated reduction of (value, error) pairs over `width` lanes of a warp segment.
template <int WIDTH>
__device__ __forceinline__ float comp_reduce(float v) {
  float err = 0.0f;
#pragma unroll
  for (int off = WIDTH / 2; off > 0; off >>= 1) {
    float ov = __shfl_down_sync(0xffffffffu, v, off, WIDTH);
    float oe = __shfl_down_sync(0xffffffffu, err, off, WIDTH);
    float s, e;
    two_sum(v, ov, s, e);
    v = s;
    err = err + oe + e;
  }
  return v + err;
}

template <int WIDTH>
__device__ __forceinline__ double seg_reduce_d(double v) {
#pragma unroll
  for (int off = WIDTH / 2; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off, WIDTH);
  return v;
}

template <int WIDTH>
__device__ __forceinline__ int seg_or(int v) {
#pragma unroll
  for (int off = WIDTH / 2; off > 0; off >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, off, WIDTH);
  return v;
}

// Block-wide sum of NV doubles per thread into block_out[NV] (thread 0 holds the result).
template <int NV, int BLOCK>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem /* NV*BLOCK/32 */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = v[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    if (lane == 0) smem[k * (BLOCK / 32) + wid] = x;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = (lane < BLOCK / 32) ? smem[k * (BLOCK / 32) + lane] : 0.0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
      v[k] = x;
    }
  }
  __syncthreads();
}

// Last-block pattern: every block writes its partials, the block that takes the final
// ticket reduces them in block order (deterministic) and resets the ticket.
// Returns true in the last block (all threads).
__device__ __forceinline__ bool take_last_ticket(unsigned int* ticket, int* s_flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int t = atomicAdd(ticket, 1u);
    *s_flag = (t == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  bool last = *s_flag != 0;
  if (last) __threadfence();
  return last;
}

// Reduce NV partials per block (layout partials[k * nblk + b]) in the last block.
template <int NV, int BLOCK>
__device__ __forceinline__ void reduce_partials(const double* partials, int nblk, double (&out)[NV],
                                                double* smem) {
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = 0.0;
    for (int b = threadIdx.x; b < nblk; b += BLOCK) x += partials[k * nblk + b];
    out[k] = x;
  }
  block_sum<NV, BLOCK>(out, smem);
}

// beta of utils.h:17-25
template <typename T>
__device__ __forceinline__ T beta_fn(T xi, T delta, T dx) {
  T h = dx / T(2);
  if (xi <= delta - h) return T(1);
  if (xi > delta - h && xi <= delta + h) return (delta + h - xi) / dx;
  return T(0);
}

}  // namespace nnpp

#endif  // NNPP_COMMON_CUH
