// implicit.cu -- the reference's production time step on the GPU: backward Euler with one
// tangent per step and modified Newton iterations, each solving every field's correction by
// left-Jacobi GMRES(30) (main.cpp:640-922, utils::NewtonMatrices utils.h:844-1849,
// Eigen::GMRES GMRES.h:56-203).  FP64 throughout, node order of the reference (the user's).
//
//   per step   tangents K_f at U^n: species k (utils.h:900-1102) off-diagonal
//              -(K1 D(BV) + K2 D(BV) z F/(RT) (phi^n_n - phi^n_i)) w per bond, diagonal
//              1/dt + sum K1 D(BV) w; the potential K11 (utils.h:1797-1848) -w on
//              liquid-liquid bonds, their sum on the diagonal; Dirichlet rows (and potential
//              rows without liquid-liquid bonds) identity; w = beta dV / xi^3.
//   Newton     F = Residuals(U^{n+1}, U^n) with the migration on phi^n (utils.h:126), F11's
//              charge from U^n (utils.h:829-831), and
//              F = U - bc on Dirichlet rows (main.cpp:676-712); K_f dU_f = -F_f by GMRES for
//              the S species and the potential at once (five independent Krylov solves
//              advanced together: one gather of a bond serves all five); U += dU; the clamp
//              (main.cpp:805-837); stop when max_f | ||dU_f|| - ||dU_f||_prev | < EPS.
//   then       the phase flip (main.cpp:914-922) and the volume every sub_step_no steps.
//
// GMRES follows Eigen's (GMRES.h:56-203): initial guess x = b (GMRES.h:330-334), the
// diagonal preconditioner on the left, restarts every 30 steps, iterations counted across
// restarts up to MAX_ITER, stop when |g_k| / ||M^-1 (b - K x_0)|| < EPS.  The Arnoldi basis is
// orthogonalised by classical Gram-Schmidt applied twice (the same Krylov space and
// least-squares problem as Eigen's Householder form; one reduction pass per sweep instead of
// k dependent ones).  Reductions are block partials summed in a fixed order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.cuh"

using namespace nnpp;

struct nnpp_handle {
  Handle h;
};

namespace {

constexpr int F5 = S + 1;          // fields: the species and the potential
constexpr int kRestart = 30;       // Eigen::GMRES's default restart (GMRES.h:282)
constexpr double kEps = 10E-6;     // EPS, main.cpp:33-36
constexpr int kMaxIter = 200;      // MAX_ITER, main.cpp:33-36
constexpr int kTB = 256;
constexpr int kDotBlocks = 304;    // two per SM

struct ImpCtx {
  int N;
  const int* ptr;                  // CSR over user indices, self excluded
  const int* col;
  const double* w;                 // per bond: beta dV / xi^3
  const unsigned char* dir;        // F5 * N Dirichlet flags
  const double* bc;                // F5 * N boundary values (species / CSolid)
  const int* phase;                // N
  const double* u0;                // F5 * N: U^n (its potential is the migration's phi^n)
  const double* diag;              // F5 * N: the tangents' diagonals
  double dt, bvmix, csat, k_diss, sw, lam, kphis;
  double K1[S], K2zF[S], DL[S], DSo[S], z[S];
};

// bond coefficients of species k between nodes of phases pi, pn (utils.h:100-153,
// 202-239): false when the bond is absent (solid-solid for k >= 1)
__device__ __forceinline__ bool species_bond(const ImpCtx& c, int k, int pi, int pn, double* a1,
                                             double* a2zf) {
  double D, BV = 1.0;
  if (k == 0) {
    if (pi != pn) BV = c.bvmix;
    D = (pi == 0 && pn == 0) ? c.DL[0] : c.DSo[0];
  } else {
    if (pi == 1 && pn == 1) return false;
    D = (pi == 0 && pn == 0) ? c.DL[k] : c.DSo[k];
  }
  *a1 = c.K1[k] * D * BV;
  *a2zf = c.K2zF[k] * D * BV;
  return true;
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// per bond w = beta dV / xi^3 (utils.h:17-25, the bond terms' xi^(3+2s) beta dV with s = 0)
__global__ void k_imp_weights(int N, const int* ptr, const int* col, const double* x, const double* y,
                              const double* z, double delta, double dx, double dV, double* w) {
  const int lane = threadIdx.x & 31;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N; i += (gridDim.x * blockDim.x) >> 5)
    for (int j = ptr[i] + lane; j < ptr[i + 1]; j += 32) {
      const int n = col[j];
      const double a = x[n] - x[i], b = y[n] - y[i], d = z[n] - z[i];
      const double xi = sqrt(a * a + b * b + d * d);
      w[j] = beta_fn<double>(xi, delta, dx) * dV / (xi * xi * xi);
    }
}

// the tangents' diagonals (warp per node)
__global__ void k_imp_diag(ImpCtx c, double* diag) {
  const int lane = threadIdx.x & 31;
  const int N = c.N;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N; i += (gridDim.x * blockDim.x) >> 5) {
    const int pi = c.phase[i];
    double sk[S] = {0.0, 0.0, 0.0, 0.0}, sp = 0.0, ll = 0.0;
    for (int j = c.ptr[i] + lane; j < c.ptr[i + 1]; j += 32) {
      const int n = c.col[j];
      const int pn = c.phase[n];
      const double w = c.w[j];
#pragma unroll
      for (int k = 0; k < S; ++k) {
        double a1, a2;
        if (species_bond(c, k, pi, pn, &a1, &a2)) sk[k] += a1 * w;
      }
      if (pi == 0 && pn == 0) {
        sp += w;
        ll += 1.0;
      }
    }
#pragma unroll
    for (int k = 0; k < S; ++k) sk[k] = warp_sum(sk[k]);
    sp = warp_sum(sp);
    ll = warp_sum(ll);
    if (lane == 0) {
      for (int k = 0; k < S; ++k)
        diag[(size_t)k * N + i] = c.dir[(size_t)k * N + i] ? 1.0 : 1.0 / c.dt + sk[k];
      diag[(size_t)S * N + i] = (c.dir[(size_t)S * N + i] || ll == 0.0) ? 1.0 : sp;
    }
  }
}

// Residual of the implicit step (utils.h:72-257, 798-841; Dirichlet rows main.cpp:676-712)
__global__ void k_imp_residual(ImpCtx c, const double* u1, double* F) {
  const int lane = threadIdx.x & 31;
  const int N = c.N;
  const double* phi0 = c.u0 + (size_t)S * N;
  const double* phi1 = u1 + (size_t)S * N;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N; i += (gridDim.x * blockDim.x) >> 5) {
    const int pi = c.phase[i];
    double ci[S];
#pragma unroll
    for (int k = 0; k < S; ++k) ci[k] = u1[(size_t)k * N + i];
    double s1[S] = {0, 0, 0, 0}, s2[S] = {0, 0, 0, 0}, sp = 0.0;
    int iface = 0, ll = 0;
    for (int j = c.ptr[i] + lane; j < c.ptr[i + 1]; j += 32) {
      const int n = c.col[j];
      const int pn = c.phase[n];
      const double w = c.w[j];
      iface |= (pi == 1 && pn == 0) ? 1 : 0;
      const double dphi0 = phi0[n] - phi0[i];
#pragma unroll
      for (int k = 0; k < S; ++k) {
        double a1, a2;
        if (!species_bond(c, k, pi, pn, &a1, &a2)) continue;
        const double cn = u1[(size_t)k * N + n];
        s1[k] += -(a1 * (cn - ci[k])) * w;
        s2[k] += -(a2 * cn * dphi0) * w;
      }
      if (pi == 0 && pn == 0) {
        sp += -(c.kphis * (phi1[n] - phi1[i])) * w;
        ll = 1;
      }
    }
#pragma unroll
    for (int k = 0; k < S; ++k) {
      s1[k] = warp_sum(s1[k]);
      s2[k] = warp_sum(s2[k]);
    }
    sp = warp_sum(sp);
    iface = __any_sync(0xffffffffu, iface) ? 1 : 0;
    ll = __any_sync(0xffffffffu, ll) ? 1 : 0;
    if (lane == 0) {
      for (int k = 0; k < S; ++k) {
        double R = 0.0;
        if (k == 0 && iface) {
          const double sw = c.sw > 0.0 ? 1.0 / (1.0 + exp(-(ci[0] - c.csat) / c.sw)) : (ci[0] > c.csat ? 1.0 : 0.0);
          R = -c.k_diss * sw;
        }
        double f = ((ci[k] - c.u0[(size_t)k * N + i]) / c.dt) + s1[k] + s2[k] - R;
        if (c.dir[(size_t)k * N + i]) f = ci[k] - c.bc[(size_t)k * N + i];
        F[(size_t)k * N + i] = f;
      }
      // F11 from phi^{n+1} and the charge of U^n (utils.h:829-831)
      double f11 = 0.0;
      if (ll) {
        double r11 = 0.0;
        for (int k = 0; k < S; ++k) r11 += c.z[k] * c.u0[(size_t)k * N + i];
        f11 = (1.0 / c.kphis) * sp - c.lam * r11;
      }
      if (c.dir[(size_t)S * N + i]) f11 = phi1[i] - c.bc[(size_t)S * N + i];
      F[(size_t)S * N + i] = f11;
    }
  }
}

// out_f = M^-1 K_f v_f for the fields in mask (bit f): the tangents applied to the five
// fields at once, one pass over the bonds (warp per node)
__global__ void k_imp_apply(ImpCtx c, const double* v, double* out, int mask) {
  const int lane = threadIdx.x & 31;
  const int N = c.N;
  const double* phi0 = c.u0 + (size_t)S * N;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N; i += (gridDim.x * blockDim.x) >> 5) {
    const int pi = c.phase[i];
    double acc[F5] = {0, 0, 0, 0, 0};
    for (int j = c.ptr[i] + lane; j < c.ptr[i + 1]; j += 32) {
      const int n = c.col[j];
      const int pn = c.phase[n];
      const double w = c.w[j];
      const double dphi0 = phi0[n] - phi0[i];
#pragma unroll
      for (int k = 0; k < S; ++k) {
        if (!((mask >> k) & 1)) continue;
        double a1, a2;
        if (!species_bond(c, k, pi, pn, &a1, &a2)) continue;
        acc[k] += -(a1 + a2 * dphi0) * w * v[(size_t)k * N + n];
      }
      if (((mask >> S) & 1) && pi == 0 && pn == 0) acc[S] += -w * v[(size_t)S * N + n];
    }
#pragma unroll
    for (int f = 0; f < F5; ++f) acc[f] = warp_sum(acc[f]);
    if (lane == 0)
      for (int f = 0; f < F5; ++f) {
        if (!((mask >> f) & 1)) continue;
        const size_t q = (size_t)f * N + i;
        const double d = c.diag[q];
        // identity rows: Dirichlet, and potential rows without liquid-liquid bonds (diag 1 and
        // no off-diagonal term then; a Dirichlet row's bonds are dropped here)
        const double off = c.dir[q] ? 0.0 : acc[f];
        out[q] = (d * v[q] + off) / d;
      }
  }
}

// block partials of the dot products <a_f, B_{q,f}> for q < nq and the fields of mask:
// part[(q * F5 + f) * gridDim.x + block]; B_q at B + q * F5 * N
__global__ void k_imp_dots(int N, const double* a, const double* B, int nq, int mask, double* part) {
  __shared__ double sm[kTB / 32];
  for (int q = 0; q < nq; ++q)
    for (int f = 0; f < F5; ++f) {
      if (!((mask >> f) & 1)) continue;
      const double* x = a + (size_t)f * N;
      const double* y = B + ((size_t)q * F5 + f) * N;
      double s = 0.0;
      for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) s += x[i] * y[i];
      s = warp_sum(s);
      if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
      __syncthreads();
      if (threadIdx.x == 0) {
        double t = 0.0;
        for (int u = 0; u < kTB / 32; ++u) t += sm[u];
        part[((size_t)q * F5 + f) * gridDim.x + blockIdx.x] = t;
      }
      __syncthreads();
    }
}

// out[v] = sum of the nb partials of value v, in block order
__global__ void k_imp_reduce(const double* part, int nb, int nv, double* out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double t = 0.0;
  for (int b = 0; b < nb; ++b) t += part[(size_t)v * nb + b];
  out[v] = t;
}

// y_f += sign * sum_{q < nq} coef[q * F5 + f] B_{q,f} for the fields of mask
__global__ void k_imp_combine(int N, double* y, const double* B, int nq, const double* coef, double sign, int mask) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    for (int f = 0; f < F5; ++f) {
      if (!((mask >> f) & 1)) continue;
      double s = 0.0;
      for (int q = 0; q < nq; ++q) s += coef[q * F5 + f] * B[((size_t)q * F5 + f) * N + i];
      y[(size_t)f * N + i] += sign * s;
    }
}

// dst_f = src_f * scale[f] for the fields of mask
__global__ void k_imp_scale(int N, const double* src, double* dst, const double* scale, int mask) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    for (int f = 0; f < F5; ++f)
      if ((mask >> f) & 1) dst[(size_t)f * N + i] = src[(size_t)f * N + i] * scale[f];
}

// r_f = b_f / diag_f - t_f (t = M^-1 K x) for the fields of mask
__global__ void k_imp_presid(int N, const double* b, const double* diag, const double* t, double* r, int mask) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    for (int f = 0; f < F5; ++f)
      if ((mask >> f) & 1) {
        const size_t q = (size_t)f * N + i;
        r[q] = b[q] / diag[q] - t[q];
      }
}

// U += dU, then the clamp of the species (main.cpp:805-837; the model's species are the
// always-clamped U1..U4)
__global__ void k_imp_update(int N, double* u1, const double* du, double floor_c) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    for (int f = 0; f < F5; ++f) {
      const size_t q = (size_t)f * N + i;
      double v = u1[q] + du[q];
      if (f < S && v < floor_c) v = floor_c;
      u1[q] = v;
    }
}

// phase flip (main.cpp:914-922); flip step into the handle's record (internal order); the
// solid volume sum of main.cpp:944-949 into per-block partials
__global__ void k_imp_flip(int N, const double* u1, int* phase, double csat, int step, const int* iperm,
                           int* flip_step, double* part) {
  __shared__ double sm[kTB / 32];
  double v = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    if (phase[i] == 1 && u1[i] <= csat) {
      phase[i] = 0;
      flip_step[iperm[i]] = step;
    }
    if (phase[i] == 1) v += u1[i] - csat;
  }
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int u = 0; u < kTB / 32; ++u) t += sm[u];
    part[blockIdx.x] = t;
  }
}

// Device buffers of the implicit solver (one set per call; a handle keeps its weights).
struct Work {
  int N = 0;
  DBuf<double> u0, u1, F, b, dU, x, t, r, diag, V, part, red, coef;
  DBuf<unsigned char> dir;
  DBuf<double> bc;
  DBuf<int> phase;
};

int grid_for(long long items, int per_block) {
  long long g = (items + per_block - 1) / per_block;
  return (int)std::max<long long>(1, std::min<long long>(g, 152 * 16));
}

// dots <a_f, B_{q,f}> (q < nq, fields of mask) into host h[q * F5 + f]
nnpp_status dots(cudaStream_t st, Work& wk, const double* a, const double* B, int nq, int mask, double* h) {
  const int N = wk.N;
  k_imp_dots<<<kDotBlocks, kTB, 0, st>>>(N, a, B, nq, mask, wk.part.get());
  const int nv = nq * F5;
  k_imp_reduce<<<(nv + 127) / 128, 128, 0, st>>>(wk.part.get(), kDotBlocks, nv, wk.red.get());
  NNPP_CUDA(cudaGetLastError());
  NNPP_CUDA(cudaMemcpyAsync(h, wk.red.get(), sizeof(double) * nv, cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  return NNPP_OK;
}

nnpp_status apply(cudaStream_t st, const ImpCtx& c, const double* v, double* out, int mask) {
  k_imp_apply<<<grid_for((long long)c.N * 32, kTB), kTB, 0, st>>>(c, v, out, mask);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

// Five independent GMRES solves K_f x_f = b_f (wk.b -> wk.x), as Eigen's; iterations summed
nnpp_status gmres5(cudaStream_t st, const ImpCtx& c, Work& wk, long long* iters_total) {
  const int N = wk.N;
  const size_t FN = (size_t)F5 * N;
  double* V = wk.V.get();
  std::vector<double> bb(F5), r0n(F5), beta(F5), h1((kRestart + 1) * F5), h2((kRestart + 1) * F5);
  std::vector<double> H((size_t)F5 * (kRestart + 1) * kRestart), g((size_t)F5 * (kRestart + 1)),
      cs((size_t)F5 * kRestart), sn((size_t)F5 * kRestart);
  std::vector<int> it(F5, 0);
  // x = b (GMRES.h:330-334); b = 0 gives x = 0
  NNPP_CUDA(cudaMemcpyAsync(wk.x.get(), wk.b.get(), sizeof(double) * FN, cudaMemcpyDeviceToDevice, st));
  NNPP_TRY(dots(st, wk, wk.b.get(), wk.b.get(), 1, 0x1f, bb.data()));
  int active = 0;
  for (int f = 0; f < F5; ++f)
    if (bb[f] != 0.0) active |= 1 << f;
  if (!active) return NNPP_OK;
  // r = M^-1 (b - K x)
  NNPP_TRY(apply(st, c, wk.x.get(), wk.t.get(), active));
  k_imp_presid<<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.b.get(), c.diag, wk.t.get(), wk.r.get(), active);
  NNPP_TRY(dots(st, wk, wk.r.get(), wk.r.get(), 1, active, r0n.data()));
  for (int f = 0; f < F5; ++f) {
    r0n[f] = std::sqrt(r0n[f]);
    if ((active >> f) & 1 && r0n[f] == 0.0) active &= ~(1 << f);
  }
  std::vector<double> scale(F5), coef((size_t)(kRestart + 1) * F5);
  while (active) {
    // a cycle: V_0 = r / ||r||
    NNPP_TRY(dots(st, wk, wk.r.get(), wk.r.get(), 1, active, beta.data()));
    for (int f = 0; f < F5; ++f) {
      beta[f] = std::sqrt(beta[f]);
      scale[f] = beta[f] != 0.0 ? 1.0 / beta[f] : 0.0;
      for (int q = 0; q <= kRestart; ++q) g[(size_t)f * (kRestart + 1) + q] = 0.0;
      g[(size_t)f * (kRestart + 1)] = beta[f];
    }
    NNPP_CUDA(cudaMemcpyAsync(wk.coef.get(), scale.data(), sizeof(double) * F5, cudaMemcpyHostToDevice, st));
    k_imp_scale<<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.r.get(), V, wk.coef.get(), active);
    int cycle = active;  // fields still iterating in this cycle
    int restart_set = 0;
    for (int k = 1; k <= kRestart && cycle; ++k) {
      double* w = V + (size_t)k * FN;
      NNPP_TRY(apply(st, c, V + (size_t)(k - 1) * FN, w, cycle));
      // classical Gram-Schmidt, twice
      for (int pass = 0; pass < 2; ++pass) {
        std::vector<double>& hh = pass == 0 ? h1 : h2;
        NNPP_TRY(dots(st, wk, w, V, k, cycle, hh.data()));
        NNPP_CUDA(cudaMemcpyAsync(wk.coef.get(), hh.data(), sizeof(double) * k * F5, cudaMemcpyHostToDevice, st));
        k_imp_combine<<<grid_for(N, kTB), kTB, 0, st>>>(N, w, V, k, wk.coef.get(), -1.0, cycle);
      }
      std::vector<double> nrm(F5);
      NNPP_TRY(dots(st, wk, w, w, 1, cycle, nrm.data()));
      for (int f = 0; f < F5; ++f) {
        scale[f] = 0.0;
        if (!((cycle >> f) & 1)) continue;
        double* Hf = H.data() + (size_t)f * (kRestart + 1) * kRestart;
        double* gf = g.data() + (size_t)f * (kRestart + 1);
        double* csf = cs.data() + (size_t)f * kRestart;
        double* snf = sn.data() + (size_t)f * kRestart;
        for (int q = 0; q < k; ++q) Hf[(size_t)q * kRestart + (k - 1)] = h1[q * F5 + f] + h2[q * F5 + f];
        const double hk = std::sqrt(nrm[f]);
        Hf[(size_t)k * kRestart + (k - 1)] = hk;
        scale[f] = hk != 0.0 ? 1.0 / hk : 0.0;
        for (int q = 0; q < k - 1; ++q) {
          const double a = Hf[(size_t)q * kRestart + (k - 1)], b = Hf[(size_t)(q + 1) * kRestart + (k - 1)];
          Hf[(size_t)q * kRestart + (k - 1)] = csf[q] * a + snf[q] * b;
          Hf[(size_t)(q + 1) * kRestart + (k - 1)] = -snf[q] * a + csf[q] * b;
        }
        const double a = Hf[(size_t)(k - 1) * kRestart + (k - 1)], b = Hf[(size_t)k * kRestart + (k - 1)];
        const double den = std::hypot(a, b);
        csf[k - 1] = den == 0.0 ? 1.0 : a / den;
        snf[k - 1] = den == 0.0 ? 0.0 : b / den;
        Hf[(size_t)(k - 1) * kRestart + (k - 1)] = den;
        Hf[(size_t)k * kRestart + (k - 1)] = 0.0;
        gf[k] = -snf[k - 1] * gf[k - 1];
        gf[k - 1] = csf[k - 1] * gf[k - 1];
        it[f] += 1;
        const bool stop = k == N || std::abs(gf[k]) / r0n[f] < kEps || it[f] == kMaxIter;
        if (stop || k == kRestart) {
          // x_f += V y, y = H^-1 g (upper triangular)
          std::vector<double> y(k);
          for (int q = k - 1; q >= 0; --q) {
            double s = gf[q];
            for (int u = q + 1; u < k; ++u) s -= Hf[(size_t)q * kRestart + u] * y[u];
            y[q] = s / Hf[(size_t)q * kRestart + q];
          }
          for (int q = 0; q <= kRestart; ++q) coef[q * F5 + f] = 0.0;
          for (int q = 0; q < k; ++q) coef[q * F5 + f] = y[q];
          NNPP_CUDA(cudaMemcpyAsync(wk.coef.get(), coef.data(), sizeof(double) * k * F5, cudaMemcpyHostToDevice, st));
          k_imp_combine<<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.x.get(), V, k, wk.coef.get(), 1.0, 1 << f);
          NNPP_CUDA(cudaStreamSynchronize(st));  // coef is reused by the next field
          cycle &= ~(1 << f);
          if (stop)
            active &= ~(1 << f);
          else
            restart_set |= 1 << f;
        }
      }
      if (cycle) {
        NNPP_CUDA(cudaMemcpyAsync(wk.coef.get(), scale.data(), sizeof(double) * F5, cudaMemcpyHostToDevice, st));
        k_imp_scale<<<grid_for(N, kTB), kTB, 0, st>>>(N, w, w, wk.coef.get(), cycle);
      }
    }
    if (restart_set) {
      NNPP_TRY(apply(st, c, wk.x.get(), wk.t.get(), restart_set));
      k_imp_presid<<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.b.get(), c.diag, wk.t.get(), wk.r.get(), restart_set);
      NNPP_CUDA(cudaGetLastError());
    }
  }
  for (int f = 0; f < F5; ++f) *iters_total += it[f];
  return NNPP_OK;
}

__global__ void k_imp_negate(size_t n, const double* a, double* b) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = -a[i];
}

}  // namespace

extern "C" nnpp_status nnpp_forward_implicit(nnpp_handle* hp, int n_steps, int64_t* newton_iterations,
                                             int64_t* krylov_iterations) {
  clear_error();
  if (!hp) return set_error(NNPP_ERR_INVALID, "handle is NULL");
  Handle& h = hp->h;
  if (!h.built) return set_error(NNPP_ERR_STATE, "neighbour lists not built (call nnpp_build_neighbours)");
  if (n_steps < 0) return set_error(NNPP_ERR_INVALID, "forward_implicit: negative step count");
  NNPP_CUDA(cudaSetDevice(h.device));
  const nnpp_params& p = h.p;
  if (p.s_phi != 0.0) return set_error(NNPP_ERR_UNSUPPORTED, "forward_implicit: kernel exponent s must be 0");
  const int N = h.N;
  const size_t FN = (size_t)F5 * N;
  const long long nnz = h.ref.nnz;
  cudaStream_t st = h.st;
  // per-bond weights in the reference's node order, kept with the handle's solver buffers
  Work wk;
  wk.N = N;
  DBuf<double> w;
  if (!w.alloc(std::max<long long>(nnz, 1)) || !wk.u0.alloc(FN) || !wk.u1.alloc(FN) || !wk.F.alloc(FN) ||
      !wk.b.alloc(FN) || !wk.x.alloc(FN) || !wk.t.alloc(FN) || !wk.r.alloc(FN) || !wk.diag.alloc(FN) ||
      !wk.V.alloc((size_t)(kRestart + 1) * FN) || !wk.part.alloc((size_t)kDotBlocks * (kRestart + 1) * F5) ||
      !wk.red.alloc((size_t)(kRestart + 1) * F5) || !wk.coef.alloc((size_t)(kRestart + 1) * F5) ||
      !wk.dir.alloc(FN) || !wk.bc.alloc(FN) || !wk.phase.alloc(N))
    return set_error(NNPP_ERR_NOMEM, "forward_implicit buffers");
  k_imp_weights<<<grid_for((long long)N * 32, kTB), kTB, 0, st>>>(
      N, h.ref.ptr.get(), h.ref.col.get(), h.ux.get(), h.uy.get(), h.uz.get(), p.delta, p.dx,
      p.dx * p.dy * p.dz, w.get());
  NNPP_CUDA(cudaGetLastError());
  {
    // Dirichlet flags and values in the reference's order (main.cpp:676-712)
    std::vector<unsigned char> dir(FN, 0);
    std::vector<double> bc(FN, 0.0);
    for (int f = 0; f <= S; ++f)
      for (int i = 0; i < N; ++i) {
        const double v = h.h_bcv[(size_t)f * N + i];
        if (h.h_bctypes[i] == 0 && v != -1) {
          dir[(size_t)f * N + i] = 1;
          bc[(size_t)f * N + i] = f < S ? v / p.CSolid : v;
        }
      }
    NNPP_CUDA(cudaMemcpyAsync(wk.dir.get(), dir.data(), FN, cudaMemcpyHostToDevice, st));
    NNPP_CUDA(cudaMemcpyAsync(wk.bc.get(), bc.data(), sizeof(double) * FN, cudaMemcpyHostToDevice, st));
  }
  // the handle's state (FP64, user order)
  NNPP_TRY(store_state(h, wk.u0.get(), wk.u0.get() + (size_t)S * N, wk.phase.get()));
  DevState ds;
  NNPP_CUDA(cudaMemcpyAsync(&ds, h.dstate.get(), sizeof(DevState), cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  ImpCtx c;
  std::memset(&c, 0, sizeof(c));
  c.N = N;
  c.ptr = h.ref.ptr.get();
  c.col = h.ref.col.get();
  c.w = w.get();
  c.dir = wk.dir.get();
  c.bc = wk.bc.get();
  c.phase = wk.phase.get();
  c.u0 = wk.u0.get();
  c.diag = wk.diag.get();
  c.dt = p.dt;
  c.csat = p.CSat / p.CSolid;
  c.k_diss = p.k_diss;
  c.sw = p.switch_width;
  c.kphis = p.K_phi * p.sigma;
  c.lam = (1. / (p.K_phi * p.sigma)) * p.F * p.CSolid;
  for (int k = 0; k < S; ++k) {
    c.K1[k] = p.K1[k];
    c.K2zF[k] = p.K2[k] * p.z[k] * p.F / (p.R * p.T);
    c.DL[k] = p.D_liquid[k];
    c.DSo[k] = p.D_solid[k];
    c.z[k] = p.z[k];
  }
  double voln1rel = ds.voln1rel;
  long long steps_done = ds.steps;
  long long newton_total = 0, krylov_total = 0;
  std::vector<double> res(F5), res_old(F5), part(kDotBlocks);
  for (int s = 0; s < n_steps; ++s) {
    c.bvmix = std::pow(10., -p.vol_red * (1. - voln1rel));  // utils.h:100-116
    // the tangents' diagonals at U^n (main.cpp:657-662), U^{n+1} = U^n to start
    k_imp_diag<<<grid_for((long long)N * 32, kTB), kTB, 0, st>>>(c, wk.diag.get());
    NNPP_CUDA(cudaMemcpyAsync(wk.u1.get(), wk.u0.get(), sizeof(double) * FN, cudaMemcpyDeviceToDevice, st));
    std::fill(res_old.begin(), res_old.end(), 0.0);
    int it = 0;
    for (it = 0; it < kMaxIter; ++it) {
      k_imp_residual<<<grid_for((long long)N * 32, kTB), kTB, 0, st>>>(c, wk.u1.get(), wk.F.get());
      k_imp_negate<<<grid_for((long long)FN, kTB), kTB, 0, st>>>(FN, wk.F.get(), wk.b.get());
      NNPP_CUDA(cudaGetLastError());
      NNPP_TRY(gmres5(st, c, wk, &krylov_total));
      NNPP_TRY(dots(st, wk, wk.x.get(), wk.x.get(), 1, 0x1f, res.data()));
      k_imp_update<<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.u1.get(), wk.x.get(), 1.0e-8 / p.CSolid);
      NNPP_CUDA(cudaGetLastError());
      double resMax = 0.0;
      for (int f = 0; f < F5; ++f) {
        res[f] = std::sqrt(res[f]);
        resMax = std::max(resMax, std::abs(res[f] - res_old[f]));
      }
      if (!std::isfinite(resMax)) return set_error(NNPP_ERR_NONFINITE, "forward_implicit: non-finite update");
      if (resMax < kEps) {
        ++it;
        break;
      }
      res_old = res;
    }
    newton_total += it;
    // flip, volume (main.cpp:914-922, 944-949)
    steps_done += 1;
    k_imp_flip<<<kDotBlocks, kTB, 0, st>>>(N, wk.u1.get(), wk.phase.get(), c.csat, (int)steps_done,
                                           h.lay.iperm.get(), h.flip_step.get(), wk.part.get());
    NNPP_CUDA(cudaGetLastError());
    NNPP_CUDA(cudaMemcpyAsync(part.data(), wk.part.get(), sizeof(double) * kDotBlocks, cudaMemcpyDeviceToHost, st));
    NNPP_CUDA(cudaStreamSynchronize(st));
    if (p.sub_step_no > 0 && steps_done % p.sub_step_no == 0) {
      double v = 0.0;
      for (double x : part) v += x;
      voln1rel = ds.vol0rel != 0.0 ? v / ds.vol0rel : 0.0;
    }
    // time-level swap (main.cpp:1002-1024)
    NNPP_CUDA(cudaMemcpyAsync(wk.u0.get(), wk.u1.get(), sizeof(double) * FN, cudaMemcpyDeviceToDevice, st));
  }
  // the result into the handle's state (FP64), its diagnostics and step count
  NNPP_TRY(load_state(h, wk.u0.get(), wk.u0.get() + (size_t)S * N, wk.phase.get(), NNPP_FP64, true));
  NNPP_TRY(init_diag(h, true));
  DevState d2;
  NNPP_CUDA(cudaMemcpyAsync(&d2, h.dstate.get(), sizeof(DevState), cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  d2.steps = steps_done;
  d2.voln1rel = voln1rel;
  d2.BV = std::pow(10., -p.vol_red * (1. - voln1rel));
  NNPP_CUDA(cudaMemcpyAsync(h.dstate.get(), &d2, sizeof(DevState), cudaMemcpyHostToDevice, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  h.coarse.stale = true;
  h.nstep = 0;
  if (newton_iterations) *newton_iterations = newton_total;
  if (krylov_iterations) *krylov_iterations = krylov_total;
  return NNPP_OK;
}
