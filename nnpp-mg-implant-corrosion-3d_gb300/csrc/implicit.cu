// implicit.cu -- the reference's production time step on the GPU: backward Euler with one
// tangent per step and modified Newton iterations, each solving every field's correction by
// left-Jacobi GMRES(30) (main.cpp:640-922, utils::NewtonMatrices utils.h:844-1849,
// Eigen::GMRES GMRES.h:56-203).  FP64 throughout, node order of the reference (the user's).
//
//   per step   tangents K_f at U^n: species k (utils.h:900-1102) off-diagonal
//              -(K1 D(BV) + K2 D(BV) z F/(RT) (phi^n_n - phi^n_i)) w per bond, diagonal
//              1/dt + sum K1 D(BV) w; the potential K11 (utils.h:1797-1848) -w on
//              liquid-liquid bonds, their sum on the diagonal; Dirichlet rows (and potential
//              rows without liquid-liquid bonds) identity; w = beta dV / xi^3.  The species'
//              off-diagonals are stored per bond for the step (the GB300's FP64 rate made
//              forming them in every GMRES product the product's bound).
//   Newton     F = Residuals(U^{n+1}, U^n) with the migration on phi^n (utils.h:126), F11's
//              charge from U^n (utils.h:829-831), and
//              F = U - bc on Dirichlet rows (main.cpp:676-712); K_f dU_f = -F_f by GMRES for
//              the species and the potential at once (independent Krylov solves advanced
//              together: one pass over the bonds serves every field); U += dU; the clamp
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

template <int NS>
struct ImpCtxT {
  int N;
  const int* ptr;                  // CSR over user indices, self excluded
  const int* col;
  const double* w;                 // per bond: beta dV / xi^3
  const unsigned char* dir;        // (NS + 1) * N Dirichlet flags
  const double* bc;                // (NS + 1) * N boundary values (species / CSolid)
  const int* phase;                // N
  const double* u0;                // (NS + 1) * N: U^n (its potential is the migration's phi^n)
  const double* diag;              // (NS + 1) * N: the tangents' diagonals
  const double* toff;              // NS * nnz: the species tangents' off-diagonals per bond
  long long nnz;
  double dt, bvmix, csat, k_diss, sw, lam, kphis;
  double K1[NS], K2zF[NS], DL[NS], DSo[NS], z[NS];
  double k7b, k8b, k9b;            // the complete model's rates in its tangents' diagonals
};
using ImpCtx = ImpCtxT<S>;

// bond coefficients of species k between nodes of phases pi, pn (utils.h:100-153,
// 202-239): false when the bond is absent (solid-solid for k >= 1)
template <int NS>
__device__ __forceinline__ bool species_bond(const ImpCtxT<NS>& c, int k, int pi, int pn, double* a1,
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

// the tangents' diagonals (warp per node).  The complete model (NS = 10) adds the linearised
// reaction terms of utils::NewtonMatrices at U^n: H+ on interface and liquid nodes
// (utils.h:1089-1098), species 3, 4, 5 and 7 on liquid nodes (1176-1182, 1266-1271,
// 1356-1361, 1546-1551).
template <int NS>
__global__ void k_imp_diag(ImpCtxT<NS> c, double* diag) {
  const int lane = threadIdx.x & 31;
  const int N = c.N;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N; i += (gridDim.x * blockDim.x) >> 5) {
    const int pi = c.phase[i];
    double sk[NS], sp = 0.0, ll = 0.0;
    int iface = 0;
#pragma unroll
    for (int k = 0; k < NS; ++k) sk[k] = 0.0;
    for (int j = c.ptr[i] + lane; j < c.ptr[i + 1]; j += 32) {
      const int n = c.col[j];
      const int pn = c.phase[n];
      const double w = c.w[j];
      iface |= (pi == 1 && pn == 0) ? 1 : 0;
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        double a1, a2;
        if (species_bond(c, k, pi, pn, &a1, &a2)) sk[k] += a1 * w;
      }
      if (pi == 0 && pn == 0) {
        sp += w;
        ll += 1.0;
      }
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) sk[k] = warp_sum(sk[k]);
    sp = warp_sum(sp);
    ll = warp_sum(ll);
    iface = __any_sync(0xffffffffu, iface) ? 1 : 0;
    if (lane == 0) {
      for (int k = 0; k < NS; ++k) {
        double R = 0.0;
        if (NS == 10) {
          const bool liq = pi == 0;
          auto u = [&](int f) { return c.u0[(size_t)f * N + i]; };
          if (k == 1 && (iface || liq))
            R = c.k7b * (-u(2)) + c.k8b * (-u(4)) + c.k9b * (-u(6));
          else if (k == 2 && liq)
            R = c.k7b * (-u(1));
          else if ((k == 3 || k == 4) && liq)
            R = c.k8b * (-u(1));
          else if (k == 6 && liq)
            R = c.k9b * (-u(1));
        }
        diag[(size_t)k * N + i] = c.dir[(size_t)k * N + i] ? 1.0 : 1.0 / c.dt + sk[k] - R;
      }
      diag[(size_t)NS * N + i] = (c.dir[(size_t)NS * N + i] || ll == 0.0) ? 1.0 : sp;
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

// the species tangents' off-diagonals of every bond (utils.h:900-1792):
// -(K1 D(BV) + K2 D(BV) z F/(RT) (phi^n_n - phi^n_i)) w, zero where the bond is absent;
// formed once a step, read by every GMRES iteration's product (warp per node)
template <int NS>
__global__ void k_imp_tangent(ImpCtxT<NS> c, double* toff) {
  const int lane = threadIdx.x & 31;
  const int N = c.N;
  const double* phi0 = c.u0 + (size_t)NS * N;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N; i += (gridDim.x * blockDim.x) >> 5) {
    const int pi = c.phase[i];
    for (int j = c.ptr[i] + lane; j < c.ptr[i + 1]; j += 32) {
      const int n = c.col[j];
      const int pn = c.phase[n];
      const double w = c.w[j];
      const double dphi0 = phi0[n] - phi0[i];
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        double a1, a2;
        toff[(size_t)k * c.nnz + j] = species_bond(c, k, pi, pn, &a1, &a2) ? -(a1 + a2 * dphi0) * w : 0.0;
      }
    }
  }
}

// out_f = M^-1 K_f v_f for the fields in mask (bit f): the tangents applied to every field at
// once, one pass over the bonds (warp per node), the species' off-diagonals from toff
template <int NS>
__global__ void k_imp_apply(ImpCtxT<NS> c, const double* v, double* out, int mask) {
  constexpr int NF = NS + 1;
  const int lane = threadIdx.x & 31;
  const int N = c.N;
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N; i += (gridDim.x * blockDim.x) >> 5) {
    const int pi = c.phase[i];
    double acc[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) acc[f] = 0.0;
    for (int j = c.ptr[i] + lane; j < c.ptr[i + 1]; j += 32) {
      const int n = c.col[j];
#pragma unroll
      for (int k = 0; k < NS; ++k)
        if ((mask >> k) & 1) acc[k] += c.toff[(size_t)k * c.nnz + j] * v[(size_t)k * N + n];
      if (((mask >> NS) & 1) && pi == 0 && c.phase[n] == 0) acc[NS] += -c.w[j] * v[(size_t)NS * N + n];
    }
#pragma unroll
    for (int f = 0; f < NF; ++f) acc[f] = warp_sum(acc[f]);
    if (lane == 0)
      for (int f = 0; f < NF; ++f) {
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

// block partials of the dot products <a_f, B_{q,f}> for q < nq and the fields of mask, every
// product at once (blockIdx.y = q * NF + f): part[(q * NF + f) * gridDim.x + block]; B_q at
// B + q * NF * N
template <int NF>
__global__ void k_imp_dots(int N, const double* a, const double* B, int nq, int mask, double* part) {
  __shared__ double sm[kTB / 32];
  const int v = blockIdx.y;
  const int q = v / NF, f = v - q * NF;
  if (q >= nq || !((mask >> f) & 1)) return;
  const double* x = a + (size_t)f * N;
  const double* y = B + ((size_t)q * NF + f) * N;
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) s += x[i] * y[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int u = 0; u < kTB / 32; ++u) t += sm[u];
    part[(size_t)v * gridDim.x + blockIdx.x] = t;
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

// y_f += sign * sum_{q < nq} coef[q * NF + f] B_{q,f} for the fields of mask
template <int NF>
__global__ void k_imp_combine(int N, double* y, const double* B, int nq, const double* coef, double sign, int mask) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    for (int f = 0; f < NF; ++f) {
      if (!((mask >> f) & 1)) continue;
      double s = 0.0;
      for (int q = 0; q < nq; ++q) s += coef[q * NF + f] * B[((size_t)q * NF + f) * N + i];
      y[(size_t)f * N + i] += sign * s;
    }
}

// dst_f = src_f * scale[f] for the fields of mask
template <int NF>
__global__ void k_imp_scale(int N, const double* src, double* dst, const double* scale, int mask) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    for (int f = 0; f < NF; ++f)
      if ((mask >> f) & 1) dst[(size_t)f * N + i] = src[(size_t)f * N + i] * scale[f];
}

// r_f = b_f / diag_f - t_f (t = M^-1 K x) for the fields of mask
template <int NF>
__global__ void k_imp_presid(int N, const double* b, const double* diag, const double* t, double* r, int mask) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    for (int f = 0; f < NF; ++f)
      if ((mask >> f) & 1) {
        const size_t q = (size_t)f * N + i;
        r[q] = b[q] / diag[q] - t[q];
      }
}

// U += dU, then the clamp of the species (main.cpp:805-837: U1..U9 always, U10 on liquid
// nodes; the four-species model's species are the always-clamped U1..U4)
template <int NS>
__global__ void k_imp_update(int N, double* u1, const double* du, double floor_c, const int* phase) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    for (int f = 0; f <= NS; ++f) {
      const size_t q = (size_t)f * N + i;
      double v = u1[q] + du[q];
      if (f < NS && v < floor_c && (f < 9 || phase[i] == 0)) v = floor_c;
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
      if (flip_step) flip_step[iperm[i]] = step;
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
// pinned host memory (the GMRES's reduction results come back by asynchronous copies)
struct HostPinned {
  double* p = nullptr;
  HostPinned() = default;
  HostPinned(const HostPinned&) = delete;
  HostPinned& operator=(const HostPinned&) = delete;
  ~HostPinned() {
    if (p) cudaFreeHost(p);
  }
  bool alloc(size_t n) { return cudaMallocHost(reinterpret_cast<void**>(&p), n * sizeof(double)) == cudaSuccess; }
};

struct Work {
  int N = 0;
  DBuf<double> u0, u1, F, b, dU, x, t, r, diag, V, part, red, coef, toff;
  HostPinned hpin;
  DBuf<unsigned char> dir;
  DBuf<double> bc;
  DBuf<int> phase;
};

int grid_for(long long items, int per_block) {
  long long g = (items + per_block - 1) / per_block;
  return (int)std::max<long long>(1, std::min<long long>(g, 152 * 16));
}

// dots <a_f, B_{q,f}> (q < nq, fields of mask) into the device array wk.red[q * NF + f]
template <int NF>
nnpp_status dots_dev(cudaStream_t st, Work& wk, const double* a, const double* B, int nq, int mask) {
  const int N = wk.N;
  // blocks of 8 elements a thread per product (at most kDotBlocks)
  const int nb = std::max(1, std::min(kDotBlocks, (N + kTB * 8 - 1) / (kTB * 8)));
  const int nv = nq * NF;
  k_imp_dots<NF><<<dim3((unsigned)nb, (unsigned)nv), kTB, 0, st>>>(N, a, B, nq, mask, wk.part.get());
  k_imp_reduce<<<(nv + 127) / 128, 128, 0, st>>>(wk.part.get(), nb, nv, wk.red.get());
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

// the same into host h[q * NF + f]
template <int NF>
nnpp_status dots(cudaStream_t st, Work& wk, const double* a, const double* B, int nq, int mask, double* h) {
  NNPP_TRY(dots_dev<NF>(st, wk, a, B, nq, mask));
  const int nv = nq * NF;
  NNPP_CUDA(cudaMemcpyAsync(h, wk.red.get(), sizeof(double) * nv, cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  return NNPP_OK;
}

template <int NS>
nnpp_status apply(cudaStream_t st, const ImpCtxT<NS>& c, const double* v, double* out, int mask) {
  k_imp_apply<NS><<<grid_for((long long)c.N * 32, kTB), kTB, 0, st>>>(c, v, out, mask);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

// NS + 1 independent GMRES solves K_f x_f = b_f (wk.b -> wk.x), as Eigen's; iterations summed
template <int NS>
nnpp_status gmres_fields(cudaStream_t st, const ImpCtxT<NS>& c, Work& wk, long long* iters_total) {
  constexpr int F5 = NS + 1;
  constexpr int kAll = (1 << F5) - 1;
  const int N = wk.N;
  const size_t FN = (size_t)F5 * N;
  double* V = wk.V.get();
  std::vector<double> bb(F5), r0n(F5), beta(F5), h1((kRestart + 1) * F5), h2((kRestart + 1) * F5);
  std::vector<double> H((size_t)F5 * (kRestart + 1) * kRestart), g((size_t)F5 * (kRestart + 1)),
      cs((size_t)F5 * kRestart), sn((size_t)F5 * kRestart);
  std::vector<int> it(F5, 0);
  if (!wk.hpin.p && !wk.hpin.alloc((size_t)3 * (kRestart + 1) * F5))
    return set_error(NNPP_ERR_NOMEM, "implicit step: pinned reduction buffer");
  // x = b (GMRES.h:330-334); b = 0 gives x = 0
  NNPP_CUDA(cudaMemcpyAsync(wk.x.get(), wk.b.get(), sizeof(double) * FN, cudaMemcpyDeviceToDevice, st));
  NNPP_TRY(dots<F5>(st, wk, wk.b.get(), wk.b.get(), 1, kAll, bb.data()));
  int active = 0;
  for (int f = 0; f < F5; ++f)
    if (bb[f] != 0.0) active |= 1 << f;
  if (!active) return NNPP_OK;
  // r = M^-1 (b - K x)
  NNPP_TRY(apply(st, c, wk.x.get(), wk.t.get(), active));
  k_imp_presid<F5><<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.b.get(), c.diag, wk.t.get(), wk.r.get(), active);
  NNPP_TRY(dots<F5>(st, wk, wk.r.get(), wk.r.get(), 1, active, r0n.data()));
  for (int f = 0; f < F5; ++f) {
    r0n[f] = std::sqrt(r0n[f]);
    if ((active >> f) & 1 && r0n[f] == 0.0) active &= ~(1 << f);
  }
  std::vector<double> scale(F5), coef((size_t)(kRestart + 1) * F5);
  while (active) {
    // a cycle: V_0 = r / ||r||
    NNPP_TRY(dots<F5>(st, wk, wk.r.get(), wk.r.get(), 1, active, beta.data()));
    for (int f = 0; f < F5; ++f) {
      beta[f] = std::sqrt(beta[f]);
      scale[f] = beta[f] != 0.0 ? 1.0 / beta[f] : 0.0;
      for (int q = 0; q <= kRestart; ++q) g[(size_t)f * (kRestart + 1) + q] = 0.0;
      g[(size_t)f * (kRestart + 1)] = beta[f];
    }
    NNPP_CUDA(cudaMemcpyAsync(wk.coef.get(), scale.data(), sizeof(double) * F5, cudaMemcpyHostToDevice, st));
    k_imp_scale<F5><<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.r.get(), V, wk.coef.get(), active);
    int cycle = active;  // fields still iterating in this cycle
    int restart_set = 0;
    for (int k = 1; k <= kRestart && cycle; ++k) {
      double* w = V + (size_t)k * FN;
      NNPP_TRY(apply(st, c, V + (size_t)(k - 1) * FN, w, cycle));
      // classical Gram-Schmidt, twice: each pass's coefficients stay on the device (the
      // combination reads the reduction's output) and come back with the new vector's norm by
      // asynchronous copies, one synchronisation an iteration
      const size_t hs = (size_t)(kRestart + 1) * F5;
      for (int pass = 0; pass < 2; ++pass) {
        NNPP_TRY(dots_dev<F5>(st, wk, w, V, k, cycle));
        NNPP_CUDA(cudaMemcpyAsync(wk.hpin.p + pass * hs, wk.red.get(), sizeof(double) * k * F5,
                                  cudaMemcpyDeviceToHost, st));
        k_imp_combine<F5><<<grid_for(N, kTB), kTB, 0, st>>>(N, w, V, k, wk.red.get(), -1.0, cycle);
      }
      NNPP_TRY(dots_dev<F5>(st, wk, w, w, 1, cycle));
      NNPP_CUDA(cudaMemcpyAsync(wk.hpin.p + 2 * hs, wk.red.get(), sizeof(double) * F5, cudaMemcpyDeviceToHost, st));
      NNPP_CUDA(cudaStreamSynchronize(st));
      std::copy(wk.hpin.p, wk.hpin.p + (size_t)k * F5, h1.begin());
      std::copy(wk.hpin.p + hs, wk.hpin.p + hs + (size_t)k * F5, h2.begin());
      std::vector<double> nrm(wk.hpin.p + 2 * hs, wk.hpin.p + 2 * hs + F5);
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
          k_imp_combine<F5><<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.x.get(), V, k, wk.coef.get(), 1.0, 1 << f);
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
        k_imp_scale<F5><<<grid_for(N, kTB), kTB, 0, st>>>(N, w, w, wk.coef.get(), cycle);
      }
    }
    if (restart_set) {
      NNPP_TRY(apply(st, c, wk.x.get(), wk.t.get(), restart_set));
      k_imp_presid<F5><<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.b.get(), c.diag, wk.t.get(), wk.r.get(), restart_set);
      NNPP_CUDA(cudaGetLastError());
    }
  }
  for (int f = 0; f < F5; ++f) *iters_total += it[f];
  return NNPP_OK;
}

// F = U - bc on the Dirichlet rows of every field (main.cpp:676-712)
template <int NF>
__global__ void k_imp_dirichlet(int N, const double* u1, const double* bc, const unsigned char* dir, double* F) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    for (int f = 0; f < NF; ++f) {
      const size_t q = (size_t)f * N + i;
      if (dir[q]) F[q] = u1[q] - bc[q];
    }
}

__global__ void k_imp_negate(size_t n, const double* a, double* b) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = -a[i];
}

}  // namespace

extern "C" nnpp_status nnpp_forward_implicit(nnpp_handle* hp, int n_steps, int64_t* newton_iterations,
                                             int64_t* krylov_iterations) {
  nnpp::TraceRange trace_("nnpp_forward_implicit");
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
      !wk.dir.alloc(FN) || !wk.bc.alloc(FN) || !wk.phase.alloc(N) ||
      !wk.toff.alloc((size_t)S * std::max<long long>(nnz, 1)))
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
  c.toff = wk.toff.get();
  c.nnz = nnz;
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
    k_imp_diag<S><<<grid_for((long long)N * 32, kTB), kTB, 0, st>>>(c, wk.diag.get());
    k_imp_tangent<S><<<grid_for((long long)N * 32, kTB), kTB, 0, st>>>(c, wk.toff.get());
    NNPP_CUDA(cudaMemcpyAsync(wk.u1.get(), wk.u0.get(), sizeof(double) * FN, cudaMemcpyDeviceToDevice, st));
    std::fill(res_old.begin(), res_old.end(), 0.0);
    int it = 0;
    for (it = 0; it < kMaxIter; ++it) {
      k_imp_residual<<<grid_for((long long)N * 32, kTB), kTB, 0, st>>>(c, wk.u1.get(), wk.F.get());
      k_imp_negate<<<grid_for((long long)FN, kTB), kTB, 0, st>>>(FN, wk.F.get(), wk.b.get());
      NNPP_CUDA(cudaGetLastError());
      NNPP_TRY(gmres_fields<S>(st, c, wk, &krylov_total));
      NNPP_TRY(dots<F5>(st, wk, wk.x.get(), wk.x.get(), 1, 0x1f, res.data()));
      k_imp_update<S><<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.u1.get(), wk.x.get(), 1.0e-8 / p.CSolid, wk.phase.get());
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

// ---------------------------------------------------------------- the complete model -----
// The reference's time step with all eleven fields (main.cpp:640-922 as written: ten species
// and the potential).  The tangents of utils::NewtonMatrices (utils.h:846-1849) at U^n,
// applied matrix-free like the four-species step's (eleven fields in one pass over the bonds;
// the species' own constants, the linearised reaction terms on the diagonals), the residual
// of utils::Residuals (utils.h:29-842: nnpp_residuals_full_device) with the Dirichlet rows of
// main.cpp:676-712, eleven GMRES corrections advanced together, the clamp of
// main.cpp:805-837 (U10 on liquid nodes only), the update-norm test, the flip of
// main.cpp:914-922 and the relative volume every sub_step_no steps (main.cpp:944-949).
struct nnpp_chem {
  int N = 0, ml = 0, device = 0;
  long long nnz = 0;
  cudaStream_t st = nullptr;
  DBuf<double> xyz, w;
  DBuf<int> ptr, col, hz, hl;
  Work wk;
  std::vector<double> d2, dc, d11;
  double voln1rel = 0.0, vol0rel = 0.0;
  long long steps = 0;
  bool has_state = false;
  ~nnpp_chem() {
    if (st) cudaStreamDestroy(st);
  }
};

namespace {
constexpr int kChemNS = 10;
constexpr int kChemNF = 11;
constexpr int kChemSubSteps = 8;  // sub_step_no, main.cpp:39
}  // namespace

extern "C" nnpp_status nnpp_chem_create(nnpp_chem** out, int n_nodes, const double* nodes_colmajor,
                                        const int* clouds_colmajor, int max_node_no, const int* cloud_lengths,
                                        const int* bctypes, const double* bcvalues, const double* data2,
                                        const double* datac, const double* datac11) {
  clear_error();
  if (!out) return set_error(NNPP_ERR_INVALID, "chem_create: out is NULL");
  *out = nullptr;
  if (n_nodes <= 0 || max_node_no < 1 || !nodes_colmajor || !clouds_colmajor || !cloud_lengths || !bctypes ||
      !bcvalues || !data2 || !datac || !datac11)
    return set_error(NNPP_ERR_INVALID, "chem_create: bad argument");
  for (int k = 0; k < kChemNS; ++k)
    if (datac[7 * k + 3] != 0.0 || datac[7 * k + 4] != 0.0)
      return set_error(NNPP_ERR_UNSUPPORTED, "chem_create: the bond weights need the kernel exponents s = 0");
  if (datac11[2] != 0.0) return set_error(NNPP_ERR_UNSUPPORTED, "chem_create: the potential's exponent s must be 0");
  if (!(data2[2] != 0.0) || !(data2[3] > 0.0) || !(data2[7] > 0.0) || !(datac11[1] * datac11[3] != 0.0))
    return set_error(NNPP_ERR_INVALID, "chem_create: dt, dx, CSolid or K11prop1 sigma1 is zero");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return set_error(NNPP_ERR_CUDA, "chem_create: no CUDA device");
  }
  const int N = n_nodes;
  int ml = 1;
  long long nnz = 0;
  for (int i = 0; i < N; ++i) {
    const int l = cloud_lengths[i];
    if (l < 1 || l > max_node_no) return set_error(NNPP_ERR_INVALID, "chem_create: cloud length out of range");
    ml = std::max(ml, l);
    nnz += l - 1;
  }
  if (nnz > 0x7fffffffLL) return set_error(NNPP_ERR_UNSUPPORTED, "chem_create: more than 2^31 bonds");
  // CSR without the node itself (the tangents) and the padded clouds (the residual)
  std::vector<int> ptr(N + 1), col(std::max<long long>(nnz, 1));
  ptr[0] = 0;
  for (int i = 0; i < N; ++i) {
    int q = ptr[i];
    for (int j = 1; j < cloud_lengths[i]; ++j) {
      const int n = clouds_colmajor[(size_t)j * N + i];
      if (n < 0 || n >= N) return set_error(NNPP_ERR_INVALID, "chem_create: cloud index out of range");
      col[q++] = n;
    }
    ptr[i + 1] = q;
  }
  nnpp_chem* c = new nnpp_chem();
  c->N = N;
  c->ml = ml;
  c->nnz = nnz;
  cudaGetDevice(&c->device);
  c->d2.assign(data2, data2 + 51);
  c->dc.assign(datac, datac + 70);
  c->d11.assign(datac11, datac11 + 4);
  const size_t FN = (size_t)kChemNF * N;
  Work& wk = c->wk;
  wk.N = N;
  bool ok = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && c->xyz.alloc(3 * (size_t)N) && c->w.alloc(std::max<long long>(nnz, 1)) && c->ptr.alloc(N + 1) &&
       c->col.alloc(col.size()) && c->hz.alloc((size_t)ml * N) && c->hl.alloc(N) && wk.u0.alloc(FN) &&
       wk.u1.alloc(FN) && wk.F.alloc(FN) && wk.b.alloc(FN) && wk.x.alloc(FN) && wk.t.alloc(FN) &&
       wk.r.alloc(FN) && wk.diag.alloc(FN) && wk.V.alloc((size_t)(kRestart + 1) * FN) &&
       wk.part.alloc((size_t)kDotBlocks * (kRestart + 1) * kChemNF) && wk.red.alloc((size_t)(kRestart + 1) * kChemNF) &&
       wk.coef.alloc((size_t)(kRestart + 1) * kChemNF) && wk.dir.alloc(FN) && wk.bc.alloc(FN) && wk.phase.alloc(N) &&
       wk.toff.alloc((size_t)kChemNS * std::max<long long>(nnz, 1));
  if (!ok) {
    cudaGetLastError();
    delete c;
    return set_error(NNPP_ERR_NOMEM, "chem_create buffers");
  }
  cudaStream_t st = c->st;
  std::vector<unsigned char> dir(FN, 0);
  std::vector<double> bc(FN, 0.0);
  const double CSolid = data2[7];
  for (int f = 0; f < kChemNF; ++f)
    for (int i = 0; i < N; ++i) {
      const double v = bcvalues[(size_t)f * N + i];
      if (bctypes[i] == 0 && v != -1) {
        dir[(size_t)f * N + i] = 1;
        bc[(size_t)f * N + i] = f < kChemNS ? v / CSolid : v;
      }
    }
  nnpp_status rs = NNPP_OK;
  auto cp = [&](void* d, const void* h, size_t bytes) {
    if (rs == NNPP_OK && cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
      rs = set_error(NNPP_ERR_CUDA, "chem_create: copy");
  };
  cp(c->xyz.get(), nodes_colmajor, sizeof(double) * 3 * N);
  cp(c->ptr.get(), ptr.data(), sizeof(int) * (N + 1));
  cp(c->col.get(), col.data(), sizeof(int) * col.size());
  cp(c->hz.get(), clouds_colmajor, sizeof(int) * (size_t)ml * N);
  cp(c->hl.get(), cloud_lengths, sizeof(int) * N);
  cp(wk.dir.get(), dir.data(), FN);
  cp(wk.bc.get(), bc.data(), sizeof(double) * FN);
  if (rs == NNPP_OK) {
    const double dx = data2[3], dy = data2[4], dz = data2[5], delta = data2[6];
    k_imp_weights<<<grid_for((long long)N * 32, kTB), kTB, 0, st>>>(N, c->ptr.get(), c->col.get(), c->xyz.get(),
                                                                    c->xyz.get() + N, c->xyz.get() + 2 * (size_t)N,
                                                                    delta, dx, dx * dy * dz, c->w.get());
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
      rs = set_error(NNPP_ERR_CUDA, "chem_create: weights");
  }
  if (rs != NNPP_OK) {
    delete c;
    return rs;
  }
  *out = c;
  return NNPP_OK;
}

extern "C" void nnpp_chem_destroy(nnpp_chem* c) { delete c; }

extern "C" nnpp_status nnpp_chem_set_state(nnpp_chem* c, const double* U, const int* phase, double voln1rel,
                                           double vol0rel) {
  clear_error();
  if (!c || !U || !phase) return set_error(NNPP_ERR_INVALID, "chem_set_state: NULL argument");
  const int N = c->N;
  NNPP_CUDA(cudaSetDevice(c->device));
  for (int i = 0; i < N; ++i)
    if (phase[i] != 0 && phase[i] != 1) return set_error(NNPP_ERR_INVALID, "chem_set_state: phase must be 0 or 1");
  if (!(vol0rel > 0.0)) {
    // the initial volume (main.cpp:472-480): the solid nodes' Mg above saturation
    const double csat = c->d2[8] / c->d2[7];
    double v = 0.0;
    for (int i = 0; i < N; ++i)
      if (phase[i] == 1) v += U[i] - csat;
    vol0rel = v;
  }
  NNPP_CUDA(cudaMemcpyAsync(c->wk.u0.get(), U, sizeof(double) * kChemNF * N, cudaMemcpyHostToDevice, c->st));
  NNPP_CUDA(cudaMemcpyAsync(c->wk.phase.get(), phase, sizeof(int) * N, cudaMemcpyHostToDevice, c->st));
  NNPP_CUDA(cudaStreamSynchronize(c->st));
  c->voln1rel = voln1rel;
  c->vol0rel = vol0rel;
  c->steps = 0;
  c->has_state = true;
  return NNPP_OK;
}

extern "C" nnpp_status nnpp_chem_get_state(nnpp_chem* c, double* U, int* phase, double* voln1rel) {
  clear_error();
  if (!c) return set_error(NNPP_ERR_INVALID, "chem_get_state: NULL handle");
  if (!c->has_state) return set_error(NNPP_ERR_STATE, "chem_get_state: no state (call nnpp_chem_set_state)");
  NNPP_CUDA(cudaSetDevice(c->device));
  const int N = c->N;
  if (U) NNPP_CUDA(cudaMemcpyAsync(U, c->wk.u0.get(), sizeof(double) * kChemNF * N, cudaMemcpyDeviceToHost, c->st));
  if (phase) NNPP_CUDA(cudaMemcpyAsync(phase, c->wk.phase.get(), sizeof(int) * N, cudaMemcpyDeviceToHost, c->st));
  NNPP_CUDA(cudaStreamSynchronize(c->st));
  if (voln1rel) *voln1rel = c->voln1rel;
  return NNPP_OK;
}

extern "C" nnpp_status nnpp_chem_step(nnpp_chem* c, int n_steps, int64_t* newton_iterations,
                                      int64_t* krylov_iterations) {
  nnpp::TraceRange trace_("nnpp_chem_step");
  clear_error();
  if (!c) return set_error(NNPP_ERR_INVALID, "chem_step: NULL handle");
  if (n_steps < 0) return set_error(NNPP_ERR_INVALID, "chem_step: negative step count");
  if (!c->has_state) return set_error(NNPP_ERR_STATE, "chem_step: no state (call nnpp_chem_set_state)");
  NNPP_CUDA(cudaSetDevice(c->device));
  const int N = c->N;
  const size_t FN = (size_t)kChemNF * N;
  const std::vector<double>& d2 = c->d2;
  const std::vector<double>& dc = c->dc;
  Work& wk = c->wk;
  cudaStream_t st = c->st;
  const double CSolid = d2[7], CSat = d2[8], T = d2[47], R = d2[48], Fc = d2[49], vol_red = d2[50];
  ImpCtxT<kChemNS> x;
  std::memset(&x, 0, sizeof(x));
  x.N = N;
  x.ptr = c->ptr.get();
  x.col = c->col.get();
  x.w = c->w.get();
  x.dir = wk.dir.get();
  x.bc = wk.bc.get();
  x.phase = wk.phase.get();
  x.u0 = wk.u0.get();
  x.diag = wk.diag.get();
  x.toff = wk.toff.get();
  x.nnz = c->nnz;
  x.dt = d2[2];
  x.csat = CSat / CSolid;
  x.k7b = d2[41];
  x.k8b = d2[43];
  x.k9b = d2[45];
  for (int k = 0; k < kChemNS; ++k) {
    x.z[k] = dc[7 * k];
    x.DSo[k] = dc[7 * k + 1];
    x.DL[k] = dc[7 * k + 2];
    x.K1[k] = dc[7 * k + 5];
    x.K2zF[k] = dc[7 * k + 6] * dc[7 * k] * Fc / (R * T);
  }
  long long newton_total = 0, krylov_total = 0;
  std::vector<double> res(kChemNF), res_old(kChemNF), part(kDotBlocks);
  constexpr int kAll = (1 << kChemNF) - 1;
  for (int s = 0; s < n_steps; ++s) {
    x.bvmix = std::pow(10., -vol_red * (1. - c->voln1rel));  // utils.h:100-116
    k_imp_diag<kChemNS><<<grid_for((long long)N * 32, kTB), kTB, 0, st>>>(x, wk.diag.get());
    k_imp_tangent<kChemNS><<<grid_for((long long)N * 32, kTB), kTB, 0, st>>>(x, wk.toff.get());
    NNPP_CUDA(cudaMemcpyAsync(wk.u1.get(), wk.u0.get(), sizeof(double) * FN, cudaMemcpyDeviceToDevice, st));
    std::fill(res_old.begin(), res_old.end(), 0.0);
    int it = 0;
    for (it = 0; it < kMaxIter; ++it) {
      NNPP_TRY(nnpp_residuals_full_device(N, c->xyz.get(), c->hz.get(), c->hl.get(), wk.u1.get(), wk.u0.get(),
                                          wk.phase.get(), c->voln1rel, d2.data(), dc.data(), c->d11.data(),
                                          wk.F.get(), st));
      k_imp_dirichlet<kChemNF><<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.u1.get(), wk.bc.get(), wk.dir.get(), wk.F.get());
      k_imp_negate<<<grid_for((long long)FN, kTB), kTB, 0, st>>>(FN, wk.F.get(), wk.b.get());
      NNPP_CUDA(cudaGetLastError());
      NNPP_TRY(gmres_fields<kChemNS>(st, x, wk, &krylov_total));
      NNPP_TRY(dots<kChemNF>(st, wk, wk.x.get(), wk.x.get(), 1, kAll, res.data()));
      k_imp_update<kChemNS><<<grid_for(N, kTB), kTB, 0, st>>>(N, wk.u1.get(), wk.x.get(), 1.0e-8 / CSolid,
                                                             wk.phase.get());
      NNPP_CUDA(cudaGetLastError());
      double resMax = 0.0;
      for (int f = 0; f < kChemNF; ++f) {
        res[f] = std::sqrt(res[f]);
        resMax = std::max(resMax, std::abs(res[f] - res_old[f]));
      }
      if (!std::isfinite(resMax)) return set_error(NNPP_ERR_NONFINITE, "chem_step: non-finite update");
      if (resMax < kEps) {
        ++it;
        break;
      }
      res_old = res;
    }
    newton_total += it;
    c->steps += 1;
    k_imp_flip<<<kDotBlocks, kTB, 0, st>>>(N, wk.u1.get(), wk.phase.get(), x.csat, (int)c->steps, nullptr, nullptr,
                                           wk.part.get());
    NNPP_CUDA(cudaGetLastError());
    NNPP_CUDA(cudaMemcpyAsync(part.data(), wk.part.get(), sizeof(double) * kDotBlocks, cudaMemcpyDeviceToHost, st));
    NNPP_CUDA(cudaStreamSynchronize(st));
    if (c->steps % kChemSubSteps == 0) {
      double v = 0.0;
      for (double q : part) v += q;
      c->voln1rel = c->vol0rel != 0.0 ? v / c->vol0rel : 0.0;
    }
    NNPP_CUDA(cudaMemcpyAsync(wk.u0.get(), wk.u1.get(), sizeof(double) * FN, cudaMemcpyDeviceToDevice, st));
  }
  NNPP_CUDA(cudaStreamSynchronize(st));
  if (newton_iterations) *newton_iterations = newton_total;
  if (krylov_iterations) *krylov_iterations = krylov_total;
  return NNPP_OK;
}
