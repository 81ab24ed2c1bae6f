// step.cu -- the explicit NNPP step on the GPU: potential solve (K11, utils.h:1794-1848 /
// F11, utils.h:798-841) and transport (bond sums utils.h:72-257, Dirichlet main.cpp:676-712,
// clamp main.cpp:805-837, phase flip main.cpp:914-922, volume main.cpp:944-949).
//
// Two precisions share one structure:
//   FP64  : FP64 records and weights, FP64 Jacobi-preconditioned CG.
//   mixed : FP32 bond sums over 32-byte records with FP64-computed FP32 weights, per-lane
//           FP32 accumulation and a compensated (TwoSum) cross-lane reduction per node;
//           concentrations kept as compensated FP32 pairs (hi + lo) so that the time
//           accumulation and the FP64 saturation test see ~48 significant bits; the
//           potential is refined in FP64 (FP64 residual b - A phi on FP64 weights) with
//           FP32 CG for the corrections.
//
// Every kernel that reduces writes one partial per block; the block that takes the last
// ticket reduces them in block order, so results are bitwise reproducible.
#include <cmath>

#include "handle.cuh"

namespace nnpp {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ void node_range(int N, int& beg, int& end) {
  const int chunk = (N + gridDim.x - 1) / gridDim.x;
  beg = blockIdx.x * chunk;
  end = min(N, beg + chunk);
}

template <typename P>
struct VecSel;
template <>
struct VecSel<float> {
  __device__ static float* rin(const KParams& k) { return k.rin32; }
  __device__ static float* z(const KParams& k) { return k.z32; }
  __device__ static float* p(const KParams& k) { return k.p32; }
  __device__ static float* q(const KParams& k) { return k.q32; }
  __device__ static float* e(const KParams& k) { return k.e32; }
  __device__ static const float* dinv(const KParams& k) { return k.dinv32; }
  __device__ static const float* w(const KParams& k) { return k.w32; }
};
template <>
struct VecSel<double> {
  __device__ static double* rin(const KParams& k) { return k.rin64; }
  __device__ static double* z(const KParams& k) { return k.z64; }
  __device__ static double* p(const KParams& k) { return k.p64; }
  __device__ static double* q(const KParams& k) { return k.q64; }
  __device__ static double* e(const KParams& k) { return k.e64; }
  __device__ static const double* dinv(const KParams& k) { return k.dinv64; }
  __device__ static const double* w(const KParams& k) { return k.w64; }
};

template <typename P>
__device__ __forceinline__ float phase_of(const KParams& k, int a);
template <>
__device__ __forceinline__ float phase_of<float>(const KParams& k, int a) {
  return k.rec32_cur[a].phase;
}
template <>
__device__ __forceinline__ float phase_of<double>(const KParams& k, int a) {
  return (float)k.rec64_cur[a].phase;
}

// FP64 concentration of species s at node a in the current state
template <typename P>
__device__ __forceinline__ double conc_of(const KParams& k, int a, int s);
template <>
__device__ __forceinline__ double conc_of<float>(const KParams& k, int a, int s) {
  const float4 lo = k.clo[a];
  const float l = s == 0 ? lo.x : s == 1 ? lo.y : s == 2 ? lo.z : lo.w;
  return (double)k.rec32_cur[a].c[s] + (double)l;
}
template <>
__device__ __forceinline__ double conc_of<double>(const KParams& k, int a, int s) {
  return k.rec64_cur[a].c[s];
}

__device__ __forceinline__ void set_phi_rec(const KParams& k, int a, double phi, bool mixed) {
  if (mixed) {
    const float hi = (float)phi;
    k.rec32_cur[a].phi_hi = hi;
    k.rec32_cur[a].phi_lo = (float)(phi - (double)hi);
  } else {
    k.rec64_cur[a].phi = phi;
  }
}

// ------------------------------------------------------------------- potential: prep ----
// Per node: diagonal of K11 (sum of liquid-liquid weights), unknown mask, right-hand side
// b = (1/(K sigma)) F CSolid sum_k z_k c_k, FP64 residual r = b - A phi.  With F11_out set,
// writes the reference's F11 (utils.h:798-841) for every node instead and changes nothing.
template <typename P, int W>
__global__ void __launch_bounds__(kBlock) k_prep(KParams k, cudaGraphConditionalHandle hc,
                                                 double* F11_out) {
  __shared__ double sm[2 * kBlock / 32];
  __shared__ int s_last;
  const int sub = threadIdx.x % W, seg = threadIdx.x / W, nseg = kBlock / W;
  int beg, end;
  node_range(k.N, beg, end);
  double part[2] = {0.0, 0.0};  // ||b_eff||^2, ||r||^2
  for (int a0 = beg; a0 < end; a0 += nseg) {
    const int a = a0 + seg;
    const bool act = a < end;
    const float pa = act ? phase_of<P>(k, a) : 1.0f;
    const bool dirp = act && ((k.dirmask[a] >> S) & 1);
    const bool scan = act && pa == 0.0f && (F11_out != nullptr || !dirp);
    double dsum = 0.0, swphi = 0.0, cpl = 0.0;
    int anyll = 0;
    if (scan) {
      for (int j = k.row[a] + sub; j < k.row[a + 1]; j += W) {
        const int n = k.col[j];
        if (phase_of<P>(k, n) == 0.0f) {
          const double w = k.w64[j];
          const double ph = k.phi64[n];
          dsum += w;
          swphi += w * ph;
          anyll = 1;
          if ((k.dirmask[n] >> S) & 1) cpl += w * ph;
        }
      }
    }
    dsum = seg_reduce_d<W>(dsum);
    swphi = seg_reduce_d<W>(swphi);
    cpl = seg_reduce_d<W>(cpl);
    anyll = seg_or<W>(anyll);
    if (act && sub == 0) {
      double R11 = 0.0;
      for (int s = 0; s < S; ++s) R11 += k.z[s] * conc_of<P>(k, a, s);
      const double b = k.lam * R11;
      if (F11_out) {
        F11_out[a] = anyll ? (dsum * k.phi64[a] - swphi) - b : 0.0;
      } else {
        const bool fr = !dirp && pa == 0.0f && anyll;
        k.freem[a] = fr ? 1 : 0;
        k.dsum64[a] = fr ? dsum : 1.0;
        k.dinv64[a] = fr ? 1.0 / dsum : 0.0;
        k.d32[a] = fr ? (float)dsum : 1.0f;
        k.dinv32[a] = fr ? (float)(1.0 / dsum) : 0.0f;
        const double bb = fr ? b : 0.0;
        const double r = fr ? bb - (dsum * k.phi64[a] - swphi) : 0.0;
        k.b64[a] = bb;
        k.r64[a] = r;
        part[0] += (bb + (fr ? cpl : 0.0)) * (bb + (fr ? cpl : 0.0));
        part[1] += r * r;
      }
    }
  }
  if (F11_out) return;
  block_sum<2, kBlock>(part, sm);
  if (threadIdx.x == 0) {
    k.partials[0 * gridDim.x + blockIdx.x] = part[0];
    k.partials[1 * gridDim.x + blockIdx.x] = part[1];
  }
  if (!take_last_ticket(&k.ds->ticket[0], &s_last)) return;
  double tot[2];
  reduce_partials<2, kBlock>(k.partials, gridDim.x, tot, sm);
  if (threadIdx.x == 0) {
    DevState* ds = k.ds;
    ds->ticket[0] = 0;
    double bn = tot[0] > 0.0 ? tot[0] : 1.0;
    ds->bnorm2 = bn;
    ds->rnorm2 = tot[1];
    ds->outer_it = 0;
    ds->solve_iters = 0;
    const bool go = tot[1] > ds->tol * ds->tol * bn && ds->max_outer > 0;
    if (!go) {
      ds->cg_solves += 1;
      ds->last_relres = sqrt(tot[1] / bn);
    }
    if (k.in_graph) cudaGraphSetConditional(hc, go ? 1u : 0u);
  }
}

// ------------------------------------------------------------------- potential: CG -------
// Inner PCG on A e = r (r: FP64 outer residual rounded to P).  Jacobi preconditioner
// (the reference's Eigen::DiagonalPreconditioner, main.cpp:714-768).
template <typename P>
__global__ void __launch_bounds__(kBlock) k_cg_init(KParams k, cudaGraphConditionalHandle hc,
                                                    int fp64) {
  __shared__ double sm[2 * kBlock / 32];
  __shared__ int s_last;
  P* rin = VecSel<P>::rin(k);
  P* z = VecSel<P>::z(k);
  P* p = VecSel<P>::p(k);
  P* q = VecSel<P>::q(k);
  P* e = VecSel<P>::e(k);
  const P* dinv = VecSel<P>::dinv(k);
  double part[2] = {0.0, 0.0};
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x) {
    const P r = (P)k.r64[a];
    const P zz = r * dinv[a];
    rin[a] = r;
    z[a] = zz;
    p[a] = P(0);
    q[a] = P(0);
    e[a] = P(0);
    part[0] += (double)r * (double)zz;
    part[1] += (double)r * (double)r;
  }
  block_sum<2, kBlock>(part, sm);
  if (threadIdx.x == 0) {
    k.partials[0 * gridDim.x + blockIdx.x] = part[0];
    k.partials[1 * gridDim.x + blockIdx.x] = part[1];
  }
  if (!take_last_ticket(&k.ds->ticket[0], &s_last)) return;
  double tot[2];
  reduce_partials<2, kBlock>(k.partials, gridDim.x, tot, sm);
  if (threadIdx.x == 0) {
    DevState* ds = k.ds;
    ds->ticket[0] = 0;
    ds->rz = tot[0];
    ds->rr0 = tot[1];
    ds->rr = tot[1];
    ds->beta = 0.0;
    ds->alpha = 0.0;
    ds->inner_it = 0;
    // FP64: solve to the final tolerance in one sweep; mixed: reduce by inner_rel
    const double target = fp64 ? 0.25 * ds->tol * ds->tol * ds->bnorm2
                               : ds->inner_rel * ds->inner_rel * tot[1];
    ds->inner_target = target;
    if (k.in_graph) cudaGraphSetConditional(hc, (tot[1] > target && ds->max_iter > 0) ? 1u : 0u);
  }
}

// q = A z + beta q, p = z + beta p (so that q = A p), partial p.q -> alpha
template <typename P, int W>
__global__ void __launch_bounds__(kBlock) k_cg_spmv(KParams k) {
  __shared__ double sm[kBlock / 32];
  __shared__ int s_last;
  const int sub = threadIdx.x % W, seg = threadIdx.x / W, nseg = kBlock / W;
  const P* z = VecSel<P>::z(k);
  P* p = VecSel<P>::p(k);
  P* q = VecSel<P>::q(k);
  const P* w = VecSel<P>::w(k);
  const P beta = (P)k.ds->beta;
  int beg, end;
  node_range(k.N, beg, end);
  double part[1] = {0.0};
  for (int a0 = beg; a0 < end; a0 += nseg) {
    const int a = a0 + seg;
    const bool act = a < end && k.freem[a];
    P acc = P(0);
    if (act)
      for (int j = k.row[a] + sub; j < k.row[a + 1]; j += W) acc += w[j] * z[k.col[j]];
#pragma unroll
    for (int off = W / 2; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off, W);
    if (act && sub == 0) {
      const P dg = sizeof(P) == 4 ? (P)k.d32[a] : (P)k.dsum64[a];
      const P s = dg * z[a] - acc;
      const P qn = s + beta * q[a];
      const P pn = z[a] + beta * p[a];
      q[a] = qn;
      p[a] = pn;
      part[0] += (double)pn * (double)qn;
    }
  }
  block_sum<1, kBlock>(part, sm);
  if (threadIdx.x == 0) k.partials[blockIdx.x] = part[0];
  if (!take_last_ticket(&k.ds->ticket[0], &s_last)) return;
  double tot[1];
  reduce_partials<1, kBlock>(k.partials, gridDim.x, tot, sm);
  if (threadIdx.x == 0) {
    DevState* ds = k.ds;
    ds->ticket[0] = 0;
    ds->alpha = (tot[0] > 0.0 && isfinite(tot[0])) ? ds->rz / tot[0] : 0.0;
  }
}

// e += alpha p, r -= alpha q, z = D^-1 r, partial r.z and r.r -> beta, stop test
template <typename P>
__global__ void __launch_bounds__(kBlock) k_cg_update(KParams k, cudaGraphConditionalHandle hc) {
  __shared__ double sm[2 * kBlock / 32];
  __shared__ int s_last;
  P* rin = VecSel<P>::rin(k);
  P* z = VecSel<P>::z(k);
  const P* p = VecSel<P>::p(k);
  const P* q = VecSel<P>::q(k);
  P* e = VecSel<P>::e(k);
  const P* dinv = VecSel<P>::dinv(k);
  const double alpha_d = k.ds->alpha;
  const P alpha = (P)alpha_d;
  double part[2] = {0.0, 0.0};
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x) {
    const P di = dinv[a];
    if (di == P(0)) continue;
    const P ee = e[a] + alpha * p[a];
    const P r = rin[a] - alpha * q[a];
    const P zz = r * di;
    e[a] = ee;
    rin[a] = r;
    z[a] = zz;
    part[0] += (double)r * (double)zz;
    part[1] += (double)r * (double)r;
  }
  block_sum<2, kBlock>(part, sm);
  if (threadIdx.x == 0) {
    k.partials[0 * gridDim.x + blockIdx.x] = part[0];
    k.partials[1 * gridDim.x + blockIdx.x] = part[1];
  }
  if (!take_last_ticket(&k.ds->ticket[0], &s_last)) return;
  double tot[2];
  reduce_partials<2, kBlock>(k.partials, gridDim.x, tot, sm);
  if (threadIdx.x == 0) {
    DevState* ds = k.ds;
    ds->ticket[0] = 0;
    ds->beta = ds->rz != 0.0 ? tot[0] / ds->rz : 0.0;
    ds->rz = tot[0];
    ds->rr = tot[1];
    ds->inner_it += 1;
    ds->solve_iters += 1;
    ds->cg_iters += 1;
    const bool go = alpha_d != 0.0 && isfinite(tot[1]) && tot[1] > ds->inner_target &&
                    ds->inner_it < ds->max_iter && ds->solve_iters < ds->max_iter;
    if (k.in_graph) cudaGraphSetConditional(hc, go ? 1u : 0u);
  }
}

// phi += e on the unknowns; FP64 residual r -= A e (FP64 weights); outer stop test.
template <typename P, int W>
__global__ void __launch_bounds__(kBlock) k_ir_update(KParams k, cudaGraphConditionalHandle hc) {
  __shared__ double sm[kBlock / 32];
  __shared__ int s_last;
  const int sub = threadIdx.x % W, seg = threadIdx.x / W, nseg = kBlock / W;
  const P* e = VecSel<P>::e(k);
  const bool mixed = sizeof(P) == 4;
  int beg, end;
  node_range(k.N, beg, end);
  double part[1] = {0.0};
  for (int a0 = beg; a0 < end; a0 += nseg) {
    const int a = a0 + seg;
    const bool act = a < end && k.freem[a];
    double acc = 0.0;
    if (act)
      for (int j = k.row[a] + sub; j < k.row[a + 1]; j += W) acc += k.w64[j] * (double)e[k.col[j]];
    acc = seg_reduce_d<W>(acc);
    if (act && sub == 0) {
      const double ea = (double)e[a];
      const double r = k.r64[a] - (k.dsum64[a] * ea - acc);
      k.r64[a] = r;
      const double ph = k.phi64[a] + ea;
      k.phi64[a] = ph;
      set_phi_rec(k, a, ph, mixed);
      part[0] += r * r;
    }
  }
  block_sum<1, kBlock>(part, sm);
  if (threadIdx.x == 0) k.partials[blockIdx.x] = part[0];
  if (!take_last_ticket(&k.ds->ticket[0], &s_last)) return;
  double tot[1];
  reduce_partials<1, kBlock>(k.partials, gridDim.x, tot, sm);
  if (threadIdx.x == 0) {
    DevState* ds = k.ds;
    ds->ticket[0] = 0;
    ds->rnorm2 = tot[0];
    ds->outer_it += 1;
    ds->outer_total += 1;
    const bool conv = tot[0] <= ds->tol * ds->tol * ds->bnorm2;
    const bool go = !conv && ds->outer_it < ds->max_outer && ds->solve_iters < ds->max_iter &&
                    isfinite(tot[0]);
    if (!go) {
      ds->cg_solves += 1;
      ds->last_relres = sqrt(tot[0] / ds->bnorm2);
      if (!conv) ds->cg_nc += 1;
    }
    if (k.in_graph) cudaGraphSetConditional(hc, go ? 1u : 0u);
  }
}

// ------------------------------------------------------------------- transport -----------
__device__ __forceinline__ float sel4(const float4& v, int s) {
  return s == 0 ? v.x : s == 1 ? v.y : s == 2 ? v.z : v.w;
}

__device__ __forceinline__ double dissolve_switch(double c0, double csat, double sw) {
  if (sw > 0.0) return 1.0 / (1.0 + exp(-(c0 - csat) / sw));
  return c0 > csat ? 1.0 : 0.0;
}

constexpr int kDiagSlots = 9;  // mass[4], solid, vol, dissolved, nonfinite, mg

// Finishes a transport launch: block partials -> DevState (last block).
__device__ __forceinline__ void transport_epilogue(const KParams& k, double (&part)[kDiagSlots],
                                                   double* sm, int* s_last) {
  block_sum<kDiagSlots, kBlock>(part, sm);
  if (threadIdx.x == 0)
    for (int v = 0; v < kDiagSlots; ++v) k.partials[v * gridDim.x + blockIdx.x] = part[v];
  if (!take_last_ticket(&k.ds->ticket[0], s_last)) return;
  double tot[kDiagSlots];
  reduce_partials<kDiagSlots, kBlock>(k.partials, gridDim.x, tot, sm);
  if (threadIdx.x == 0) {
    DevState* ds = k.ds;
    ds->ticket[0] = 0;
    const double dV = 1.0;  // multiplied on the host
    (void)dV;
    for (int s = 0; s < S; ++s) ds->mass[s] = tot[s];
    ds->solid_count = (long long)tot[4];
    ds->steps += 1;
    if (k.dissolve_count) ds->dissolved += tot[6];
    if (tot[7] != 0.0) ds->nonfinite = 1;
    ds->mg_mass_now = tot[0];
    if (k.sub_step_no > 0 && ds->steps % k.sub_step_no == 0)
      ds->voln1rel = ds->vol0rel != 0.0 ? tot[5] / ds->vol0rel : 0.0;
  }
}

// Mixed transport.  RESID: write F_k = sum_KRk1 + sum_KRk2 - R_k (utils.h:177) to F_out
// and change nothing; otherwise advance the state into rec32_nxt / clo.
template <int W, bool RESID>
__global__ void __launch_bounds__(kBlock) k_transport32(KParams k, double* F_out) {
  __shared__ double sm[kDiagSlots * kBlock / 32];
  __shared__ int s_last;
  const int sub = threadIdx.x % W, seg = threadIdx.x / W, nseg = kBlock / W;
  const double voln1rel = *k.voln1rel_ptr;
  const double BV = pow(10., -k.vol_red * (1. - voln1rel));
  float cLL[S], cX[S], cSS[S], K1f[S], K2f[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    cLL[s] = (float)k.DL[s];
    cX[s] = (float)(s == 0 ? k.DSo[0] * BV : k.DSo[s]);
    cSS[s] = s == 0 ? (float)k.DSo[0] : 0.0f;
    K1f[s] = (float)k.K1[s];
    K2f[s] = (float)k.K2zF[s];
  }
  const float dtf = (float)k.dt;
  const long long step_no = k.ds->steps + 1;
  int beg, end;
  node_range(k.N, beg, end);
  double part[kDiagSlots];
#pragma unroll
  for (int v = 0; v < kDiagSlots; ++v) part[v] = 0.0;
  for (int a0 = beg; a0 < end; a0 += nseg) {
    const int a = a0 + seg;
    const bool act = a < end;
    Rec32 ra;
    if (act) ra = k.rec32_cur[a];
    const float pa = act ? ra.phase : 0.0f;
    float a1[S], a2[S];
#pragma unroll
    for (int s = 0; s < S; ++s) a1[s] = a2[s] = 0.0f;
    int iface = 0;
    if (act) {
      const int jb = k.row[a], je = k.row[a + 1];
      for (int j = jb + sub; j < je; j += W) {
        const int n = k.col[j];
        const float w = k.w32[j];
        const Rec32 rn = k.rec32_cur[n];
        const float pn = rn.phase;
        const float dphi = (rn.phi_hi - ra.phi_hi) + (rn.phi_lo - ra.phi_lo);
        const bool ll = (pa == 0.0f) && (pn == 0.0f);
        const bool ss = (pa != 0.0f) && (pn != 0.0f);
        iface |= (pa != 0.0f && pn == 0.0f) ? 1 : 0;
#pragma unroll
        for (int s = 0; s < S; ++s) {
          const float coef = ll ? cLL[s] : (ss ? cSS[s] : cX[s]);
          const float cw = coef * w;
          a1[s] = fmaf(cw, rn.c[s] - ra.c[s], a1[s]);
          a2[s] = fmaf(cw * rn.c[s], dphi, a2[s]);
        }
      }
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
      a1[s] = comp_reduce<W>(a1[s]);
      a2[s] = comp_reduce<W>(a2[s]);
    }
    iface = seg_or<W>(iface);
    if (!act || sub != 0) continue;
    const unsigned char dm = k.dirmask[a];
    const float4 lo4 = k.clo[a];
    const double c0old = (double)ra.c[0] + (double)lo4.x;
    const bool src_on = iface && !(dm & 1);
    const double sw = src_on ? dissolve_switch(c0old, k.csat, k.sw) : 0.0;
    const float Rmg = src_on ? (float)(-k.k_diss * sw) : 0.0f;
    if (RESID) {
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const double f = -(double)K1f[s] * a1[s] - (double)K2f[s] * a2[s] - (s == 0 ? (double)Rmg : 0.0);
        F_out[(size_t)s * k.N + a] = f;
      }
      continue;
    }
    float hi[S], lo[S];
    double v[S];
    bool bad = false;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const float inc = dtf * (K1f[s] * a1[s] + K2f[s] * a2[s] + (s == 0 ? Rmg : 0.0f));
      float t, e1, sh;
      two_sum(sel4(lo4, s), inc, t, e1);
      float e2;
      two_sum(ra.c[s], t, sh, e2);
      float sl = e1 + e2;
      float h2 = sh + sl;  // renormalise
      sl = sl - (h2 - sh);
      double val = (double)h2 + (double)sl;
      if ((dm >> s) & 1) val = k.bcval[(size_t)s * k.N + a];
      if (val < k.c_floor) val = k.c_floor;
      if (!isfinite(val)) bad = true;
      const float vh = (float)val;
      hi[s] = vh;
      lo[s] = (float)(val - (double)vh);
      v[s] = val;
    }
    float pnew = pa;
    if (pa != 0.0f && v[0] <= k.csat) {
      pnew = 0.0f;
      k.flip_step[a] = (int)step_no;
    }
    Rec32 out;
#pragma unroll
    for (int s = 0; s < S; ++s) out.c[s] = hi[s];
    out.phi_hi = ra.phi_hi;
    out.phi_lo = ra.phi_lo;
    out.phase = pnew;
    out.pad = 0.0f;
    k.rec32_nxt[a] = out;
    k.clo[a] = make_float4(lo[0], lo[1], lo[2], lo[3]);
#pragma unroll
    for (int s = 0; s < S; ++s) part[s] += v[s];
    if (pnew != 0.0f) {
      part[4] += 1.0;
      part[5] += v[0] - k.csat;
    }
    part[6] += k.k_diss * sw;
    part[7] += bad ? 1.0 : 0.0;
  }
  if (RESID) return;
  transport_epilogue(k, part, sm, &s_last);
}

// FP64 transport, same structure.
template <int W, bool RESID>
__global__ void __launch_bounds__(kBlock) k_transport64(KParams k, double* F_out) {
  __shared__ double sm[kDiagSlots * kBlock / 32];
  __shared__ int s_last;
  const int sub = threadIdx.x % W, seg = threadIdx.x / W, nseg = kBlock / W;
  const double voln1rel = *k.voln1rel_ptr;
  const double BV = pow(10., -k.vol_red * (1. - voln1rel));
  double cLL[S], cX[S], cSS[S];
#pragma unroll
  for (int s = 0; s < S; ++s) {
    cLL[s] = k.DL[s];
    cX[s] = s == 0 ? k.DSo[0] * BV : k.DSo[s];
    cSS[s] = s == 0 ? k.DSo[0] : 0.0;
  }
  const long long step_no = k.ds->steps + 1;
  int beg, end;
  node_range(k.N, beg, end);
  double part[kDiagSlots];
#pragma unroll
  for (int v = 0; v < kDiagSlots; ++v) part[v] = 0.0;
  for (int a0 = beg; a0 < end; a0 += nseg) {
    const int a = a0 + seg;
    const bool act = a < end;
    Rec64 ra;
    if (act) ra = k.rec64_cur[a];
    const double pa = act ? ra.phase : 0.0;
    double a1[S], a2[S];
#pragma unroll
    for (int s = 0; s < S; ++s) a1[s] = a2[s] = 0.0;
    int iface = 0;
    if (act) {
      const int jb = k.row[a], je = k.row[a + 1];
      for (int j = jb + sub; j < je; j += W) {
        const int n = k.col[j];
        const double w = k.w64[j];
        const Rec64 rn = k.rec64_cur[n];
        const double pn = rn.phase;
        const double dphi = rn.phi - ra.phi;
        const bool ll = (pa == 0.0) && (pn == 0.0);
        const bool ss = (pa != 0.0) && (pn != 0.0);
        iface |= (pa != 0.0 && pn == 0.0) ? 1 : 0;
#pragma unroll
        for (int s = 0; s < S; ++s) {
          const double coef = ll ? cLL[s] : (ss ? cSS[s] : cX[s]);
          const double cw = coef * w;
          a1[s] += cw * (rn.c[s] - ra.c[s]);
          a2[s] += cw * rn.c[s] * dphi;
        }
      }
    }
#pragma unroll
    for (int s = 0; s < S; ++s) {
      a1[s] = seg_reduce_d<W>(a1[s]);
      a2[s] = seg_reduce_d<W>(a2[s]);
    }
    iface = seg_or<W>(iface);
    if (!act || sub != 0) continue;
    const unsigned char dm = k.dirmask[a];
    const bool src_on = iface && !(dm & 1);
    const double sw = src_on ? dissolve_switch(ra.c[0], k.csat, k.sw) : 0.0;
    const double Rmg = src_on ? -k.k_diss * sw : 0.0;
    if (RESID) {
#pragma unroll
      for (int s = 0; s < S; ++s)
        F_out[(size_t)s * k.N + a] = -k.K1[s] * a1[s] - k.K2zF[s] * a2[s] - (s == 0 ? Rmg : 0.0);
      continue;
    }
    double v[S];
    bool bad = false;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const double F = -k.K1[s] * a1[s] - k.K2zF[s] * a2[s] - (s == 0 ? Rmg : 0.0);
      double val = ra.c[s] - k.dt * F;
      if ((dm >> s) & 1) val = k.bcval[(size_t)s * k.N + a];
      if (val < k.c_floor) val = k.c_floor;
      if (!isfinite(val)) bad = true;
      v[s] = val;
    }
    double pnew = pa;
    if (pa != 0.0 && v[0] <= k.csat) {
      pnew = 0.0;
      k.flip_step[a] = (int)step_no;
    }
    Rec64 out;
#pragma unroll
    for (int s = 0; s < S; ++s) out.c[s] = v[s];
    out.phi = ra.phi;
    out.phase = pnew;
    out.pad[0] = out.pad[1] = 0.0;
    k.rec64_nxt[a] = out;
#pragma unroll
    for (int s = 0; s < S; ++s) part[s] += v[s];
    if (pnew != 0.0) {
      part[4] += 1.0;
      part[5] += v[0] - k.csat;
    }
    part[6] += k.k_diss * sw;
    part[7] += bad ? 1.0 : 0.0;
  }
  if (RESID) return;
  transport_epilogue(k, part, sm, &s_last);
}

// ------------------------------------------------------------------- state transfer -----
__global__ void k_load_state(KParams k, const int* perm, const double* c_user, const double* phi_user,
                             const int* phase_user, int mixed, int dirichlet_phi) {
  const int N = k.N;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += gridDim.x * blockDim.x) {
    const int u = perm[a];
    double c[S];
    for (int s = 0; s < S; ++s) c[s] = c_user[(size_t)s * N + u];
    double phi = phi_user ? phi_user[u] : k.phi64[a];
    if (dirichlet_phi && ((k.dirmask[a] >> S) & 1)) phi = k.bcval[(size_t)S * N + a];
    float ph;
    if (phase_user)
      ph = phase_user[u] != 0 ? 1.0f : 0.0f;
    else
      ph = mixed ? k.rec32_cur[a].phase : (float)k.rec64_cur[a].phase;
    k.phi64[a] = phi;
    if (mixed) {
      Rec32 r;
      float lo[S];
      for (int s = 0; s < S; ++s) {
        r.c[s] = (float)c[s];
        lo[s] = (float)(c[s] - (double)r.c[s]);
      }
      r.phi_hi = (float)phi;
      r.phi_lo = (float)(phi - (double)r.phi_hi);
      r.phase = ph;
      r.pad = 0.0f;
      k.rec32_cur[a] = r;
      k.clo[a] = make_float4(lo[0], lo[1], lo[2], lo[3]);
    } else {
      Rec64 r;
      for (int s = 0; s < S; ++s) r.c[s] = c[s];
      r.phi = phi;
      r.phase = ph;
      r.pad[0] = r.pad[1] = 0.0;
      k.rec64_cur[a] = r;
    }
  }
}

__global__ void k_store_state(KParams k, const int* perm, double* c_user, double* phi_user,
                              int* phase_user, int mixed) {
  const int N = k.N;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += gridDim.x * blockDim.x) {
    const int u = perm[a];
    if (mixed) {
      const Rec32 r = k.rec32_cur[a];
      const float4 lo = k.clo[a];
      if (c_user)
        for (int s = 0; s < S; ++s) c_user[(size_t)s * N + u] = (double)r.c[s] + (double)sel4(lo, s);
      if (phase_user) phase_user[u] = r.phase != 0.0f ? 1 : 0;
    } else {
      const Rec64 r = k.rec64_cur[a];
      if (c_user)
        for (int s = 0; s < S; ++s) c_user[(size_t)s * N + u] = r.c[s];
      if (phase_user) phase_user[u] = r.phase != 0.0 ? 1 : 0;
    }
    if (phi_user) phi_user[u] = k.phi64[a];
  }
}

// convert the current state between the two representations
__global__ void k_convert(KParams k, int to_mixed) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x) {
    const double phi = k.phi64[a];
    if (to_mixed) {
      const Rec64 s64 = k.rec64_cur[a];
      Rec32 r;
      float lo[S];
      for (int s = 0; s < S; ++s) {
        r.c[s] = (float)s64.c[s];
        lo[s] = (float)(s64.c[s] - (double)r.c[s]);
      }
      r.phi_hi = (float)phi;
      r.phi_lo = (float)(phi - (double)r.phi_hi);
      r.phase = (float)s64.phase;
      r.pad = 0.0f;
      k.rec32_cur[a] = r;
      k.clo[a] = make_float4(lo[0], lo[1], lo[2], lo[3]);
    } else {
      const Rec32 s32 = k.rec32_cur[a];
      const float4 lo = k.clo[a];
      Rec64 r;
      for (int s = 0; s < S; ++s) r.c[s] = (double)s32.c[s] + (double)sel4(lo, s);
      r.phi = phi;
      r.phase = (double)s32.phase;
      r.pad[0] = r.pad[1] = 0.0;
      k.rec64_cur[a] = r;
    }
  }
}

// initial diagnostics (main.cpp:472-480): solid count, vol0rel, masses
__global__ void k_init_diag(KParams k, int mixed) {
  __shared__ double sm[7 * kBlock / 32];
  __shared__ int s_last;
  double part[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x) {
    double c[S];
    float ph;
    if (mixed) {
      const Rec32 r = k.rec32_cur[a];
      const float4 lo = k.clo[a];
      for (int s = 0; s < S; ++s) c[s] = (double)r.c[s] + (double)sel4(lo, s);
      ph = r.phase;
    } else {
      const Rec64 r = k.rec64_cur[a];
      for (int s = 0; s < S; ++s) c[s] = r.c[s];
      ph = (float)r.phase;
    }
    for (int s = 0; s < S; ++s) part[s] += c[s];
    if (ph != 0.0f) {
      part[4] += 1.0;
      part[5] += c[0] - k.csat;
    }
  }
  block_sum<7, kBlock>(part, sm);
  if (threadIdx.x == 0)
    for (int v = 0; v < 7; ++v) k.partials[v * gridDim.x + blockIdx.x] = part[v];
  if (!take_last_ticket(&k.ds->ticket[0], &s_last)) return;
  double tot[7];
  reduce_partials<7, kBlock>(k.partials, gridDim.x, tot, sm);
  if (threadIdx.x == 0) {
    DevState* ds = k.ds;
    ds->ticket[0] = 0;
    for (int s = 0; s < S; ++s) ds->mass[s] = tot[s];
    ds->mg_mass_t0 = tot[0];
    ds->mg_mass_now = tot[0];
    ds->solid_count = (long long)tot[4];
    ds->vol0rel = tot[5];
    ds->voln1rel = 0.0;
  }
}

template <typename F>
nnpp_status dispatch_lanes(int lanes, F&& f) {
  switch (lanes) {
    case 4: return f(std::integral_constant<int, 4>());
    case 8: return f(std::integral_constant<int, 8>());
    case 16: return f(std::integral_constant<int, 16>());
    case 32: return f(std::integral_constant<int, 32>());
    default: return set_error(NNPP_ERR_INVALID, "lanes per node must be 4, 8, 16 or 32");
  }
}

}  // namespace

// ---------------------------------------------------------------------------------------
nnpp_status step_alloc(Handle& h) {
  const size_t N = (size_t)h.N;
  bool ok = h.dirmask.alloc(N) && h.bcval.alloc((S + 1) * N) && h.rec32[0].alloc(N) &&
            h.rec32[1].alloc(N) && h.clo.alloc(N) && h.rec64[0].alloc(N) && h.rec64[1].alloc(N) &&
            h.phi64.alloc(N) && h.flip_step.alloc(N) && h.b64.alloc(N) && h.r64.alloc(N) &&
            h.dsum64.alloc(N) && h.dinv64.alloc(N) && h.rin64.alloc(N) && h.z64.alloc(N) &&
            h.p64.alloc(N) && h.q64.alloc(N) && h.e64.alloc(N) && h.d32.alloc(N) &&
            h.dinv32.alloc(N) && h.rin32.alloc(N) && h.z32.alloc(N) && h.p32.alloc(N) &&
            h.q32.alloc(N) && h.e32.alloc(N) && h.freem.alloc(N) &&
            h.partials.alloc((size_t)kReduceSlots * kMaxPartialBlocks) && h.dstate.alloc(1) &&
            h.scratch_d.alloc(16) && h.user_stage.alloc((S + 1) * N) && h.user_stage_i.alloc(N);
  if (!ok) return set_error(NNPP_ERR_NOMEM, "device state allocation");
  NNPP_CUDA(cudaMemsetAsync(h.freem.get(), 0, N, h.st));
  NNPP_CUDA(cudaMemsetAsync(h.rec32[1].get(), 0, N * sizeof(Rec32), h.st));
  NNPP_CUDA(cudaMemsetAsync(h.rec64[1].get(), 0, N * sizeof(Rec64), h.st));
  NNPP_CUDA(cudaMemsetAsync(h.e32.get(), 0, N * sizeof(float), h.st));
  NNPP_CUDA(cudaMemsetAsync(h.e64.get(), 0, N * sizeof(double), h.st));
  NNPP_CUDA(cudaMemsetAsync(h.flip_step.get(), 0xff, N * sizeof(int), h.st));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h.device);
  if (sms <= 0) sms = 152;
  long long want = ((long long)h.N + 63) / 64;
  long long g = std::min<long long>(want, (long long)sms * 8);
  if (g > kMaxPartialBlocks) g = kMaxPartialBlocks;
  if (g < 1) g = 1;
  h.grid = (int)g;
  return NNPP_OK;
}

KParams make_kparams(Handle& h, int cur) {
  KParams k;
  const nnpp_params& p = h.p;
  k.N = h.N;
  k.grid = h.grid;
  k.row = h.lay.row.get();
  k.col = h.lay.col.get();
  k.w64 = h.lay.w64.get();
  k.w32 = h.lay.w32.get();
  k.dirmask = h.dirmask.get();
  k.bcval = h.bcval.get();
  k.rec32_cur = h.rec32[cur].get();
  k.rec32_nxt = h.rec32[cur ^ 1].get();
  k.clo = h.clo.get();
  k.rec64_cur = h.rec64[cur].get();
  k.rec64_nxt = h.rec64[cur ^ 1].get();
  k.phi64 = h.phi64.get();
  k.flip_step = h.flip_step.get();
  k.b64 = h.b64.get();
  k.r64 = h.r64.get();
  k.dsum64 = h.dsum64.get();
  k.freem = h.freem.get();
  k.d32 = h.d32.get();
  k.dinv32 = h.dinv32.get();
  k.dinv64 = h.dinv64.get();
  k.rin32 = h.rin32.get();
  k.z32 = h.z32.get();
  k.p32 = h.p32.get();
  k.q32 = h.q32.get();
  k.e32 = h.e32.get();
  k.rin64 = h.rin64.get();
  k.z64 = h.z64.get();
  k.p64 = h.p64.get();
  k.q64 = h.q64.get();
  k.e64 = h.e64.get();
  k.partials = h.partials.get();
  k.ds = h.dstate.get();
  k.voln1rel_ptr = &h.dstate.get()->voln1rel;
  k.dt = p.dt;
  k.csat = p.CSat / p.CSolid;
  k.c_floor = p.c_floor;
  k.k_diss = p.k_diss;
  k.sw = p.switch_width;
  k.vol_red = p.vol_red;
  k.lam = (1. / (p.K_phi * p.sigma)) * p.F * p.CSolid;
  for (int s = 0; s < S; ++s) {
    k.K1[s] = p.K1[s];
    k.K2zF[s] = p.K2[s] * p.z[s] * p.F / (p.R * p.T);
    k.DL[s] = p.D_liquid[s];
    k.DSo[s] = p.D_solid[s];
    k.z[s] = p.z[s];
  }
  k.sub_step_no = p.sub_step_no;
  k.dissolve_count = 1;
  k.in_graph = 1;
  return k;
}

nnpp_status launch_prep(Handle& h, const KParams& kp, int prec, cudaStream_t st,
                        cudaGraphConditionalHandle hc, double* F11_out) {
  return dispatch_lanes(h.lanes, [&](auto wc) -> nnpp_status {
    constexpr int W = decltype(wc)::value;
    if (prec == NNPP_MIXED)
      k_prep<float, W><<<kp.grid, kBlock, 0, st>>>(kp, hc, F11_out);
    else
      k_prep<double, W><<<kp.grid, kBlock, 0, st>>>(kp, hc, F11_out);
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  });
}

nnpp_status launch_cg_init(Handle& h, const KParams& kp, int prec, cudaStream_t st,
                           cudaGraphConditionalHandle hc) {
  (void)h;
  if (prec == NNPP_MIXED)
    k_cg_init<float><<<kp.grid, kBlock, 0, st>>>(kp, hc, 0);
  else
    k_cg_init<double><<<kp.grid, kBlock, 0, st>>>(kp, hc, 1);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status launch_cg_iter(Handle& h, const KParams& kp, int prec, cudaStream_t st,
                           cudaGraphConditionalHandle hc) {
  return dispatch_lanes(h.lanes, [&](auto wc) -> nnpp_status {
    constexpr int W = decltype(wc)::value;
    if (prec == NNPP_MIXED) {
      k_cg_spmv<float, W><<<kp.grid, kBlock, 0, st>>>(kp);
      k_cg_update<float><<<kp.grid, kBlock, 0, st>>>(kp, hc);
    } else {
      k_cg_spmv<double, W><<<kp.grid, kBlock, 0, st>>>(kp);
      k_cg_update<double><<<kp.grid, kBlock, 0, st>>>(kp, hc);
    }
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  });
}

nnpp_status launch_cg_spmv(Handle& h, const KParams& kp, int prec, cudaStream_t st) {
  return dispatch_lanes(h.lanes, [&](auto wc) -> nnpp_status {
    constexpr int W = decltype(wc)::value;
    if (prec == NNPP_MIXED)
      k_cg_spmv<float, W><<<kp.grid, kBlock, 0, st>>>(kp);
    else
      k_cg_spmv<double, W><<<kp.grid, kBlock, 0, st>>>(kp);
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  });
}

nnpp_status launch_ir_update(Handle& h, const KParams& kp, int prec, cudaStream_t st,
                             cudaGraphConditionalHandle hc) {
  return dispatch_lanes(h.lanes, [&](auto wc) -> nnpp_status {
    constexpr int W = decltype(wc)::value;
    if (prec == NNPP_MIXED)
      k_ir_update<float, W><<<kp.grid, kBlock, 0, st>>>(kp, hc);
    else
      k_ir_update<double, W><<<kp.grid, kBlock, 0, st>>>(kp, hc);
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  });
}

nnpp_status launch_transport(Handle& h, const KParams& kp, int prec, cudaStream_t st,
                             double* F_out) {
  return dispatch_lanes(h.lanes, [&](auto wc) -> nnpp_status {
    constexpr int W = decltype(wc)::value;
    if (prec == NNPP_MIXED) {
      if (F_out)
        k_transport32<W, true><<<kp.grid, kBlock, 0, st>>>(kp, F_out);
      else
        k_transport32<W, false><<<kp.grid, kBlock, 0, st>>>(kp, nullptr);
    } else {
      if (F_out)
        k_transport64<W, true><<<kp.grid, kBlock, 0, st>>>(kp, F_out);
      else
        k_transport64<W, false><<<kp.grid, kBlock, 0, st>>>(kp, nullptr);
    }
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  });
}

nnpp_status load_state(Handle& h, const double* d_c_user, const double* d_phi_user,
                       const int* d_phase_user, int prec, bool dirichlet_phi) {
  KParams kp = make_kparams(h, h.cur);
  k_load_state<<<kp.grid, kBlock, 0, h.st>>>(kp, h.lay.perm.get(), d_c_user, d_phi_user,
                                             d_phase_user, prec == NNPP_MIXED ? 1 : 0,
                                             dirichlet_phi ? 1 : 0);
  NNPP_CUDA(cudaGetLastError());
  h.state_prec = prec;
  return NNPP_OK;
}

nnpp_status store_state(Handle& h, double* d_c_user, double* d_phi_user, int* d_phase_user) {
  KParams kp = make_kparams(h, h.cur);
  k_store_state<<<kp.grid, kBlock, 0, h.st>>>(kp, h.lay.perm.get(), d_c_user, d_phi_user,
                                              d_phase_user, h.state_prec == NNPP_MIXED ? 1 : 0);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status convert_state(Handle& h, int to_prec) {
  if (h.state_prec == to_prec) return NNPP_OK;
  KParams kp = make_kparams(h, h.cur);
  k_convert<<<kp.grid, kBlock, 0, h.st>>>(kp, to_prec == NNPP_MIXED ? 1 : 0);
  NNPP_CUDA(cudaGetLastError());
  h.state_prec = to_prec;
  return NNPP_OK;
}

nnpp_status init_diag(Handle& h) {
  KParams kp = make_kparams(h, h.cur);
  k_init_diag<<<kp.grid, kBlock, 0, h.st>>>(kp, h.state_prec == NNPP_MIXED ? 1 : 0);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

}  // namespace nnpp
