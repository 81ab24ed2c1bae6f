// coarse.cu -- the coarse space of the two-level preconditioner of the potential solve.
//
// Aggregates are blocks of f x f x f bins (bins of side >= the horizon radius, so every bond
// joins the same or an adjacent aggregate).  The preconditioner is
//   M^-1 r = D^-1 r + P A_c^-1 P^T r,   P = the aggregate indicator of the unknowns,
// A_c = P^T A P the Galerkin coarse operator (27 nonzeros per row), stored with its inverse
// as dense n x n FP32 matrices (n <= kCoarseMax).  The inverse comes from the Newton-Schulz
// iteration X <- X (2I - A_c X), X_0 = I / ||A_c||_inf (every iterate is a positive
// polynomial of A_c, so the preconditioner stays symmetric positive definite even when the
// iteration is stopped early).  Its GEMMs are FP32 products that cuBLAS runs on the BF16
// tensor cores by the BF16x9 split (each FP32 operand as three BF16 parts, nine partial
// products accumulated in FP32: FP32 accuracy, not TF32's).  A periodic rebuild within a run starts
// instead from the previous inverse when ||I - A_c X_0||_F < 1/2: the error then squares
// every step, and a few steps replace the 18 of the cold start.  The coarse operator is
// rebuilt when the state is replaced, and every `coarse_every` steps (counted from the last
// replacement) if a phase changed since the last rebuild; in between a stale one is still a
// valid preconditioner.  The schedule depends only on the step count and the phases, so it is
// reproducible, and forward_ckpt records each rebuilt inverse for backward to replay.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include <cublas_v2.h>

#include "engine.cuh"

namespace nnpp {

namespace {

constexpr int kNsIterations = 18;
constexpr int kNormBlocks = 128;      // block partials of the warm start's residual norm
constexpr double kNsWarmMax = 0.5;    // warm start when ||I - A_c X_0||_F is below this
constexpr double kNsTarget = 1e-8;    // warm start: steps until the bound ||.||^(2^m) meets this

// C = A B for n x n column-major FP32 matrices, emulated FP32 on the BF16 tensor cores (the
// handle's emulation strategy is EAGER, so cuBLAS takes the emulated kernels wherever they
// exist and its FP32 kernels elsewhere)
cublasStatus_t ns_gemm(cublasHandle_t hb, int n, const float* a, const float* b, float* c) {
  const float one = 1.0f, zero = 0.0f;
  return cublasGemmEx(hb, CUBLAS_OP_N, CUBLAS_OP_N, n, n, n, &one, a, CUDA_R_32F, n, b, CUDA_R_32F, n, &zero, c,
                      CUDA_R_32F, n, CUBLAS_COMPUTE_32F_EMULATED_16BFX9, CUBLAS_GEMM_DEFAULT);
}

// block partials of ||I - T||_F^2 (T n x n): FP32 sums per thread, FP64 across the block
__global__ void k_resid_sq(int n, const float* T, double* partials) {
  __shared__ double sm[256 / 32];
  const size_t nn = (size_t)n * n;
  float s = 0.0f;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nn; e += (size_t)gridDim.x * blockDim.x) {
    const float d = ((e / n == e % n) ? 1.0f : 0.0f) - T[e];
    s = fmaf(d, d, s);
  }
  double x = s;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 256 / 32; ++w) t += sm[w];
    partials[blockIdx.x] = t;
  }
}

// aggregate of every node (internal order), from the bins' node ranges
__global__ void k_agg_fill(const int* bin_start, int nb0, int nb1, int nb2, int f, int na0, int na1,
                           int* agg) {
  const int nbins = nb0 * nb1 * nb2;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbins; b += gridDim.x * blockDim.x) {
    const int bx = b % nb0, by = (b / nb0) % nb1, bz = b / (nb0 * nb1);
    const int I = bx / f + na0 * (by / f + na1 * (bz / f));
    for (int i = bin_start[b]; i < bin_start[b + 1]; ++i) agg[i] = I;
  }
}

__device__ __forceinline__ bool node_liquid(const KParams& k, int i, int mixed) {
  return (mixed ? k.rec32_cur[i].phase : (float)k.rec64_cur[i].phase) == 0.0f;
}

// Warp per aggregate row I: the 27 entries of A_c = P^T A P from the current phases (an
// unknown is a liquid node off the potential's Dirichlet set with a liquid neighbour; its
// diagonal is the sum of its liquid bonds, its off-diagonals -w to unknown neighbours).
// Lanes own fixed node subsets and reduce in a fixed order, so the matrix is reproducible.
__global__ void k_coarse_assemble(KParams k, const int* bin_start, int nb0, int nb1, int nb2, int f,
                                  int na0, int na1, int na2, int mixed, float* mat, float* rowabs) {
  const int lane = threadIdx.x & 31;
  const int n = na0 * na1 * na2;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < n; I += warps) {
    const int ax = I % na0, ay = (I / na0) % na1, az = I / (na0 * na1);
    float acc[27];
#pragma unroll
    for (int q = 0; q < 27; ++q) acc[q] = 0.0f;
    int unknowns = 0;
    for (int bz = az * f; bz < min(az * f + f, nb2); ++bz)
      for (int by = ay * f; by < min(ay * f + f, nb1); ++by)
        for (int bx = ax * f; bx < min(ax * f + f, nb0); ++bx) {
          const int b = bx + nb0 * (by + nb1 * bz);
          for (int i = bin_start[b] + lane; i < bin_start[b + 1]; i += 32) {
            if (!node_liquid(k, i, mixed) || ((k.dirmask[i] >> S) & 1)) continue;
            float d = 0.0f;
            bool ll = false;
            for (int j = k.row[i]; j < k.row[i + 1]; ++j) {
              const int m = k.col[j];
              if (!node_liquid(k, m, mixed)) continue;
              const float w = k.w32[j];
              d += w;
              ll = true;
              if ((k.dirmask[m] >> S) & 1) continue;
              const int J = k.agg[m];
              const int jx = J % na0, jy = (J / na0) % na1, jz = J / (na0 * na1);
              const int q = (jx - ax + 1) + 3 * ((jy - ay + 1) + 3 * (jz - az + 1));
#pragma unroll
              for (int t = 0; t < 27; ++t)
                if (t == q) acc[t] -= w;
            }
            if (ll) {
              acc[13] += d;
              ++unknowns;
            }
          }
        }
    unknowns = __reduce_add_sync(0xffffffffu, unknowns);
    float ra = 0.0f;
#pragma unroll
    for (int q = 0; q < 27; ++q) {
      float x = acc[q];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
      acc[q] = x;
      ra += fabsf(x);
    }
    if (lane == 0) {
      // no unknown in the aggregate: an identity row keeps A_c regular (rowabs -1 marks it:
      // the inverse's diagonal entry there is zeroed after the iteration)
      if (unknowns == 0) {
        mat[(size_t)I * n + I] = 1.0f;
        ra = -1.0f;
      } else {
        for (int q = 0; q < 27; ++q) {
          const int jx = ax + q % 3 - 1, jy = ay + (q / 3) % 3 - 1, jz = az + q / 9 - 1;
          if (jx < 0 || jy < 0 || jz < 0 || jx >= na0 || jy >= na1 || jz >= na2) continue;
          mat[(size_t)I * n + (jx + na0 * (jy + na1 * jz))] = acc[q];
        }
      }
      rowabs[I] = ra;
    }
  }
}

// Rows of A P off the diagonal term, for the deflated CG: for an unknown i and an aggregate
// J, -sum of w_ij over the unknowns j of J (liquid, off the Dirichlet set).  Thread per node,
// the 27 neighbour aggregates accumulated in fixed slots in the row's bond order.  fill == 0
// takes the largest number of touched slots (kmax); fill == 1 writes them in slot order into
// the K-slot layout col/val[s * N + i], the unused slots with value 0 (sliced like ELLPACK:
// the threads of a warp read consecutive words).
__global__ void k_ap_rows(KParams k, int mixed, int na0, int na1, int na2, int fill, int K, int* kmax,
                          int* col, float* val) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k.N; i += gridDim.x * blockDim.x) {
    float acc[27];
    unsigned int touched = 0u;
#pragma unroll
    for (int q = 0; q < 27; ++q) acc[q] = 0.0f;
    const bool unk = node_liquid(k, i, mixed) && !((k.dirmask[i] >> S) & 1);
    const int I = k.agg[i];
    const int ax = I % na0, ay = (I / na0) % na1, az = I / (na0 * na1);
    if (unk) {
      for (int j = k.row[i]; j < k.row[i + 1]; ++j) {
        const int m = k.col[j];
        if (!node_liquid(k, m, mixed) || ((k.dirmask[m] >> S) & 1)) continue;
        const int J = k.agg[m];
        const int jx = J % na0, jy = (J / na0) % na1, jz = J / (na0 * na1);
        const int q = (jx - ax + 1) + 3 * ((jy - ay + 1) + 3 * (jz - az + 1));
        const float w = k.w32[j];
#pragma unroll
        for (int t = 0; t < 27; ++t)
          if (t == q) acc[t] -= w;
        touched |= 1u << q;
      }
    }
    if (!fill) {
      const int c = __popc(touched);
      if (c) atomicMax(kmax, c);
      continue;
    }
    int o = 0;
#pragma unroll
    for (int q = 0; q < 27; ++q)
      if ((touched >> q) & 1u) {
        col[(size_t)o * k.N + i] = (ax + q % 3 - 1) + na0 * ((ay + (q / 3) % 3 - 1) + na1 * (az + q / 9 - 1));
        val[(size_t)o * k.N + i] = acc[q];
        ++o;
      }
    for (; o < K; ++o) {
      col[(size_t)o * k.N + i] = I;
      val[(size_t)o * k.N + i] = 0.0f;
    }
  }
}

// X = I / max_i rowabs[i]  (column-major n x n)
__global__ void k_ns_init(int n, const float* rowabs, float* X) {
  __shared__ float smax;
  if (threadIdx.x == 0) {
    float m = 0.0f;
    for (int i = 0; i < n; ++i) m = fmaxf(m, fabsf(rowabs[i]));  // identity rows count 1
    smax = m > 0.0f ? m : 1.0f;
  }
  __syncthreads();
  const float inv = 1.0f / smax;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n; e += (size_t)gridDim.x * blockDim.x)
    X[e] = (e / n == e % n) ? inv : 0.0f;
}

// T = 2I - T
__global__ void k_two_i_minus(int n, float* T) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n; e += (size_t)gridDim.x * blockDim.x)
    T[e] = ((e / n == e % n) ? 2.0f : 0.0f) - T[e];
}

// Y = (X + X^T) / 2, Y with rows of stride ld; the diagonal entry of an aggregate that held
// no unknown (rowabs < 0) is zero.  Its row and column of X are those of the identity; once
// a front reaches the aggregate, a coarse inverse that has not been rebuilt yet would scale
// the aggregate's residual sum by 1 instead of by the inverse of its new diagonal, so the
// stale additive correction leaves such aggregates to the diagonal part.
__global__ void k_symmetrize(int n, int ld, const float* X, const float* rowabs, float* Y) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n * n; e += (size_t)gridDim.x * blockDim.x) {
    const size_t i = e / n, j = e % n;
    Y[i * ld + j] = (i == j && rowabs[i] < 0.0f) ? 0.0f : 0.5f * (X[e] + X[j * n + i]);
  }
}

// phases in internal order (1: solid) from the current records
__global__ void k_phase_snap(KParams k, int mixed, unsigned char* snap) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k.N; i += gridDim.x * blockDim.x)
    snap[i] = node_liquid(k, i, mixed) ? 0 : 1;
}

// number of nodes whose phase differs from snap
__global__ void k_phase_diff(KParams k, int mixed, const unsigned char* snap, int* count) {
  int c = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k.N; i += gridDim.x * blockDim.x)
    c += (node_liquid(k, i, mixed) ? 0 : 1) != snap[i];
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

// deflation flag from a phase comparison: on when no node differs from the operator's phases
__global__ void k_defl_from_count(DevState* ds, const int* count) { ds->defl = *count == 0 ? 1 : 0; }

}  // namespace

Coarse::~Coarse() {
  if (cublas) cublasDestroy(static_cast<cublasHandle_t>(cublas));
}

nnpp_status coarse_build(Handle& h) {
  Coarse& c = h.coarse;
  c.valid = false;
  c.n = 0;
  if (!h.coarse_enabled) return NNPP_OK;
  const Layout& L = h.lay;
  int f = 1;
  auto count = [&](int ff) {
    long long n = 1;
    for (int d = 0; d < 3; ++d) n *= (L.nb[d] + ff - 1) / ff;
    return n;
  };
  while (count(f) > kCoarseMax) ++f;
  c.f = f;
  for (int d = 0; d < 3; ++d) c.na[d] = (L.nb[d] + f - 1) / f;
  c.n = (int)count(f);
  c.ld = (c.n + 3) & ~3;
  // A P rows hold at most 27 aggregates each: allocated once, so that no pointer the
  // kernels hold changes when the operator is rebuilt or replayed
  if (!c.agg.alloc(h.N) || !c.inv.alloc(c.inv_elems()) || !c.rc.alloc(c.ld) || !c.xc.alloc(c.n) ||
      !c.dots.alloc(3 * (size_t)c.n) || !c.rowabs.alloc(c.n) || !c.ap_col.alloc(27 * (size_t)h.N) ||
      !c.ap_val.alloc(27 * (size_t)h.N))
    return set_error(NNPP_ERR_NOMEM, "coarse space");
  NNPP_CUDA(cudaMemsetAsync(c.dots.get(), 0, sizeof(double) * 3 * (size_t)c.n, h.st));
  NNPP_CUDA(cudaMemsetAsync(c.rc.get(), 0, sizeof(float) * c.ld, h.st));  // padding to ld stays 0
  c.ap_k = 1;
  NNPP_CUDA(cudaMemsetAsync(c.inv.get(), 0, sizeof(float) * c.inv_elems(), h.st));  // padding stays 0
  k_agg_fill<<<std::max(1, std::min((L.nbins + 255) / 256, 4096)), 256, 0, h.st>>>(
      L.bin_start.get(), L.nb[0], L.nb[1], L.nb[2], f, c.na[0], c.na[1], c.agg.get());
  NNPP_CUDA(cudaGetLastError());
  if (!c.cublas) {
    cublasHandle_t hb = nullptr;
    if (cublasCreate(&hb) != CUBLAS_STATUS_SUCCESS) return set_error(NNPP_ERR_CUDA, "cublasCreate");
    c.cublas = hb;
    if (cublasSetEmulationStrategy(hb, CUBLAS_EMULATION_STRATEGY_EAGER) != CUBLAS_STATUS_SUCCESS)
      return set_error(NNPP_ERR_CUDA, "cublasSetEmulationStrategy");
  }
  c.stale = true;
  return NNPP_OK;
}

nnpp_status coarse_refresh(Handle& h) {
  Coarse& c = h.coarse;
  if (!h.coarse_enabled || c.n == 0) return NNPP_OK;
  const Layout& L = h.lay;
  const int n = c.n;
  const size_t nn = (size_t)n * n;
  // work matrices on first use (ensemble members never refresh and never hold them)
  if (!c.a.alloc(nn) || !c.t.alloc(nn) || !c.x.alloc(nn) || !c.y.alloc(nn))
    return set_error(NNPP_ERR_NOMEM, "coarse inverse");
  DBuf<float>& A = c.a;
  DBuf<float>& T = c.t;
  DBuf<float>& X = c.x;
  NNPP_CUDA(cudaMemsetAsync(A.get(), 0, sizeof(float) * nn, h.st));
  KParams kp = make_kparams(h, h.cur);
  k_coarse_assemble<<<std::max(1, std::min((n * 32 + 255) / 256, 152 * 32)), 256, 0, h.st>>>(
      kp, L.bin_start.get(), L.nb[0], L.nb[1], L.nb[2], c.f, c.na[0], c.na[1], c.na[2],
      h.state_prec == NNPP_MIXED ? 1 : 0, A.get(), c.rowabs.get());
  NNPP_CUDA(cudaGetLastError());
  const int eg = (int)std::min<size_t>((nn + 255) / 256, 152 * 64);
  cublasHandle_t hb = static_cast<cublasHandle_t>(c.cublas);
  if (cublasSetStream(hb, h.st) != CUBLAS_STATUS_SUCCESS) return set_error(NNPP_ERR_CUDA, "cublasSetStream");
  float* x = X.get();
  float* y = c.y.get();
  // a rebuild within a run (phases changed since the last one, the state not replaced)
  // starts from the last inverse if it is close enough: T = A X_0 is then the first step's
  // product already.  The residual norm is summed on the host in block order, so the
  // number of steps is reproducible.
  int steps = kNsIterations;
  bool warm = false;
  if (c.valid && !c.stale && h.coarse_event_cur < 0) {
    if (!c.nrm.alloc(kNormBlocks)) return set_error(NNPP_ERR_NOMEM, "coarse inverse");
    NNPP_CUDA(cudaMemcpy2DAsync(x, sizeof(float) * n, c.inv.get(), sizeof(float) * c.ld, sizeof(float) * n, n,
                                cudaMemcpyDeviceToDevice, h.st));
    if (ns_gemm(hb, n, A.get(), x, T.get()) != CUBLAS_STATUS_SUCCESS)
      return set_error(NNPP_ERR_CUDA, "coarse inverse: GEMM");
    k_resid_sq<<<kNormBlocks, 256, 0, h.st>>>(n, T.get(), c.nrm.get());
    NNPP_CUDA(cudaGetLastError());
    std::vector<double> part(kNormBlocks);
    NNPP_CUDA(cudaMemcpyAsync(part.data(), c.nrm.get(), sizeof(double) * kNormBlocks, cudaMemcpyDeviceToHost, h.st));
    NNPP_CUDA(cudaStreamSynchronize(h.st));
    double ss = 0.0;
    for (double v : part) ss += v;
    const double r0 = std::sqrt(ss);
    if (std::isfinite(r0) && r0 < kNsWarmMax) {
      warm = true;
      steps = 1;
      while (steps < kNsIterations && std::pow(r0, std::ldexp(1.0, steps)) > kNsTarget) ++steps;
    }
  }
  if (!warm) {
    k_ns_init<<<eg, 256, 0, h.st>>>(n, c.rowabs.get(), X.get());
    NNPP_CUDA(cudaGetLastError());
  }
  for (int it = 0; it < steps; ++it) {
    // T = A X ; T = 2I - T ; X <- X T
    if (!(warm && it == 0) && ns_gemm(hb, n, A.get(), x, T.get()) != CUBLAS_STATUS_SUCCESS)
      return set_error(NNPP_ERR_CUDA, "coarse inverse: GEMM");
    k_two_i_minus<<<eg, 256, 0, h.st>>>(n, T.get());
    NNPP_CUDA(cudaGetLastError());
    if (ns_gemm(hb, n, x, T.get(), y) != CUBLAS_STATUS_SUCCESS) return set_error(NNPP_ERR_CUDA, "coarse inverse: GEMM");
    std::swap(x, y);
  }
  // x holds the last iterate; its symmetrised copy goes to c.inv (rows of stride ld)
  k_symmetrize<<<eg, 256, 0, h.st>>>(n, c.ld, x, c.rowabs.get(), c.inv.get());
  NNPP_CUDA(cudaGetLastError());
  if (!c.snap.alloc(h.N) || !c.count.alloc(1)) return set_error(NNPP_ERR_NOMEM, "coarse phase snapshot");
  // A P for the deflated CG (the same phases as A_c)
  {
    const int gb = std::max(1, std::min((h.N + 255) / 256, 152 * 16));
    const int mixed = h.state_prec == NNPP_MIXED ? 1 : 0;
    NNPP_CUDA(cudaMemsetAsync(c.count.get(), 0, sizeof(int), h.st));
    k_ap_rows<<<gb, 256, 0, h.st>>>(kp, mixed, c.na[0], c.na[1], c.na[2], 0, 0, c.count.get(), nullptr, nullptr);
    NNPP_CUDA(cudaGetLastError());
    int K = 0;
    NNPP_CUDA(cudaMemcpyAsync(&K, c.count.get(), sizeof(int), cudaMemcpyDeviceToHost, h.st));
    NNPP_CUDA(cudaStreamSynchronize(h.st));
    c.ap_k = std::max(1, std::min(K, 27));  // at most 27: within the arrays allocated at build
    k_ap_rows<<<gb, 256, 0, h.st>>>(kp, mixed, c.na[0], c.na[1], c.na[2], 1, c.ap_k, nullptr, c.ap_col.get(),
                                    c.ap_val.get());
    NNPP_CUDA(cudaGetLastError());
  }

  k_phase_snap<<<std::max(1, std::min((h.N + 255) / 256, 152 * 16)), 256, 0, h.st>>>(
      kp, h.state_prec == NNPP_MIXED ? 1 : 0, c.snap.get());
  NNPP_CUDA(cudaGetLastError());
  c.valid = true;
  c.stale = false;
  c.rebuilds += 1;
  c.warm_rebuilds += warm ? 1 : 0;
  c.ns_steps = steps;
  h.coarse_event_cur = -1;
  // the coarse operator and A P match the phases now
  static const int kOne = 1;
  NNPP_CUDA(cudaMemcpyAsync(&h.dstate.get()->defl, &kOne, sizeof(int), cudaMemcpyHostToDevice, h.st));
  return NNPP_OK;
}

nnpp_status coarse_check(Handle& h) {
  Coarse& c = h.coarse;
  if (!h.coarse_enabled || !c.valid || h.coarse_replay) return NNPP_OK;
  KParams kp = make_kparams(h, h.cur);
  NNPP_CUDA(cudaMemsetAsync(c.count.get(), 0, sizeof(int), h.st));
  k_phase_diff<<<std::max(1, std::min((h.N + 255) / 256, 152 * 16)), 256, 0, h.st>>>(
      kp, h.state_prec == NNPP_MIXED ? 1 : 0, c.snap.get(), c.count.get());
  NNPP_CUDA(cudaGetLastError());
  int changed = 0;
  NNPP_CUDA(cudaMemcpyAsync(&changed, c.count.get(), sizeof(int), cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  if (changed == 0) return NNPP_OK;
  const auto t0 = std::chrono::steady_clock::now();
  NNPP_TRY(coarse_refresh(h));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  c.rebuild_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  c.timed_rebuilds += 1;
  if (h.coarse_record) NNPP_TRY(coarse_record_event(h, h.nstep - h.coarse_base));
  return NNPP_OK;
}

nnpp_status coarse_record_event(Handle& h, long long step) {
  const Coarse& c = h.coarse;
  h.coarse_events.emplace_back();
  Handle::CoarseEvent& ev = h.coarse_events.back();
  ev.step = step;
  const size_t nn = c.inv_elems();
  const size_t na = (size_t)c.ap_k * h.N;
  ev.ap_k = c.ap_k;
  if (!ev.inv.alloc(nn) || !ev.ap_col.alloc(na) || !ev.ap_val.alloc(na) || !ev.snap.alloc(h.N))
    return set_error(NNPP_ERR_NOMEM, "recorded coarse operator");
  NNPP_CUDA(cudaMemcpyAsync(ev.snap.get(), c.snap.get(), (size_t)h.N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(ev.inv.get(), c.inv.get(), sizeof(float) * nn, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(ev.ap_col.get(), c.ap_col.get(), sizeof(int) * na, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(ev.ap_val.get(), c.ap_val.get(), sizeof(float) * na, cudaMemcpyDeviceToDevice, h.st));
  return NNPP_OK;
}

nnpp_status coarse_select(Handle& h, long long step, bool recompute) {
  if (h.coarse_events.empty()) return NNPP_OK;
  int e = 0;
  while (e + 1 < (int)h.coarse_events.size() && h.coarse_events[e + 1].step <= step) ++e;
  if (e != h.coarse_event_cur) {
    Coarse& c = h.coarse;
    const Handle::CoarseEvent& ev = h.coarse_events[e];
    const size_t nn = c.inv_elems();
    const size_t na = (size_t)ev.ap_k * h.N;
    c.ap_k = ev.ap_k;
    NNPP_CUDA(cudaMemcpyAsync(c.inv.get(), ev.inv.get(), sizeof(float) * nn, cudaMemcpyDeviceToDevice, h.st));
    NNPP_CUDA(cudaMemcpyAsync(c.ap_col.get(), ev.ap_col.get(), sizeof(int) * na, cudaMemcpyDeviceToDevice, h.st));
    NNPP_CUDA(cudaMemcpyAsync(c.ap_val.get(), ev.ap_val.get(), sizeof(float) * na, cudaMemcpyDeviceToDevice, h.st));
    NNPP_CUDA(cudaMemcpyAsync(c.snap.get(), ev.snap.get(), (size_t)h.N, cudaMemcpyDeviceToDevice, h.st));
    h.coarse_event_cur = e;
  }
  // recomputing the step the forward rebuilt the operator before: the deflation resumed there
  if (recompute && step > 0 && h.coarse_events[e].step == step) {
    static const int kOn = 1;
    NNPP_CUDA(cudaMemcpyAsync(&h.dstate.get()->defl, &kOn, sizeof(int), cudaMemcpyHostToDevice, h.st));
  }
  return NNPP_OK;
}

nnpp_status coarse_defl_check(Handle& h) {
  Coarse& c = h.coarse;
  if (!h.coarse_enabled || !c.valid) {
    NNPP_CUDA(cudaMemsetAsync(&h.dstate.get()->defl, 0, sizeof(int), h.st));
    return NNPP_OK;
  }
  KParams kp = make_kparams(h, h.cur);
  NNPP_CUDA(cudaMemsetAsync(c.count.get(), 0, sizeof(int), h.st));
  k_phase_diff<<<std::max(1, std::min((h.N + 255) / 256, 152 * 16)), 256, 0, h.st>>>(
      kp, h.state_prec == NNPP_MIXED ? 1 : 0, c.snap.get(), c.count.get());
  k_defl_from_count<<<1, 1, 0, h.st>>>(h.dstate.get(), c.count.get());
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

}  // namespace nnpp
