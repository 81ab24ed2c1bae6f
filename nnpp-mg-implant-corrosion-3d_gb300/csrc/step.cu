// step.cu -- the explicit NNPP step on the GPU for one or many instances: potential solve
// (K11, utils.h:1794-1848 / F11, utils.h:798-841) and transport (bond sums utils.h:72-257,
// Dirichlet main.cpp:676-712, clamp main.cpp:805-837, phase flip main.cpp:914-922, volume
// main.cpp:944-949).
//
// Work is a list of tiles (bond kernels) or node chunks (vector kernels) over all instances
// of a batch; each CTA loops over the list (persistent grid).  A tile kernel stages the
// tile's halo into shared memory and reaches every neighbour through a 16-bit slot, so the
// per-bond stream is 2 bytes (+ the stored weight where one is used).
//
// Precision:
//   FP64  : FP64 records and stored FP64 weights, FP64 Jacobi-preconditioned CG.
//   mixed : transport in FP32 with stored FP32 weights (computed in FP64), per-lane FP32
//           accumulation and a compensated (TwoSum) cross-lane reduction per node;
//           concentrations kept as compensated FP32 pairs (hi + lo), the saturation test on
//           hi + lo in FP64; potential: FP64 residual b - A phi (stored FP64 weights) with
//           FP32 CG corrections whose operator recomputes the weights in FP32 from
//           tile-relative coordinates.
//
// Reductions: every work item writes one partial per value; the CTA that completes an
// instance's last item reduces that instance's partials in item order (deterministic), and
// the last instance to finish sets the graph's loop condition (any instance still active).
#include <cmath>
#include <cstring>

#include "engine.cuh"
#include "tma.cuh"

namespace nnpp {

namespace {

constexpr int kBlock = 256;

// ---------------------------------------------------------------- work-item plumbing ----
struct TileSmem {
  int off[10];  // prefix offsets of the 9 halo rows, off[9] = halo size
  int hb[9];
  int flag;
};

__device__ __forceinline__ void load_tile(const TileDesc& t, TileSmem& ts) {
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int r = 0; r < 9; ++r) {
      ts.off[r] = acc;
      ts.hb[r] = t.hb[r];
      acc += t.hl[r];
    }
    ts.off[9] = acc;
  }
  __syncthreads();
}

__host__ __device__ __forceinline__ size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }

// Copy the tile's bond slots [bond0, bond1) into shared memory with 16-byte loads (bond0 is
// a multiple of 8, the slot array is padded); bond j is then at dst[j - bond0].
__device__ __forceinline__ const unsigned short* stage_slots(const unsigned short* slot16,
                                                             const TileDesc& t, unsigned char* dst) {
  const int n = (t.bond1 - t.bond0 + 7) >> 3;
  const uint4* src = reinterpret_cast<const uint4*>(slot16 + t.bond0);
  uint4* d = reinterpret_cast<uint4*>(dst);
  for (int i = threadIdx.x; i < n; i += blockDim.x) d[i] = src[i];
  return reinterpret_cast<const unsigned short*>(dst);
}

// node of halo index s
__device__ __forceinline__ int halo_node(const TileSmem& ts, int s) {
  int r = 0;
#pragma unroll
  for (int q = 1; q < 9; ++q) r += (s >= ts.off[q]) ? 1 : 0;
  return ts.hb[r] + (s - ts.off[r]);
}

// Records that an item of an instance is done; true in the CTA that completed the
// instance's last one (all threads).  `count` = number of items of the instance.
__device__ __forceinline__ bool item_done(unsigned int* ticket, int count, int* s_flag) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int t = atomicAdd(ticket, 1u);
    *s_flag = (t == (unsigned int)(count - 1)) ? 1 : 0;
  }
  __syncthreads();
  const bool last = *s_flag != 0;
  if (last) __threadfence();
  return last;
}

// thread 0 of an instance's finishing CTA: reset its ticket, count the instance as done and,
// in the last instance, set the loop condition to "any instance active".
__device__ __forceinline__ void instance_finished(const EngineView& v, int inst, int which,
                                                  cudaGraphConditionalHandle hc) {
  v.ticket[inst] = 0;
  __threadfence();
  const unsigned int g = atomicAdd(&v.ticket[v.M], 1u);
  if (g == (unsigned int)(v.M - 1)) {
    __threadfence();
    v.ticket[v.M] = 0;
    int any = 0;
    for (int i = 0; i < v.M; ++i) {
      const DevState* ds = v.inst[i].ds;
      any |= (which == 0) ? *((volatile const int*)&ds->outer_active)
                          : *((volatile const int*)&ds->inner_active);
    }
    if (v.in_graph) cudaGraphSetConditional(hc, any ? 1u : 0u);
  }
}

// reduce NV partials of items [first, first+count) (layout partials[k*stride + item])
template <int NV>
__device__ __forceinline__ void reduce_items(const double* partials, int stride, int first, int count,
                                             double (&out)[NV], double* sm) {
  // eight independent accumulators per thread (loads in flight together), combined in a
  // fixed order: the sum does not depend on timing
  constexpr int U = 8;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double* p = partials + (size_t)k * stride + first;
    double x[U];
#pragma unroll
    for (int u = 0; u < U; ++u) x[u] = 0.0;
    int b = threadIdx.x;
    for (; b + (U - 1) * kBlock < count; b += U * kBlock)
#pragma unroll
      for (int u = 0; u < U; ++u) x[u] += p[b + u * kBlock];
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (b + u * kBlock < count) x[u] += p[b + u * kBlock];
    out[k] = ((x[0] + x[1]) + (x[2] + x[3])) + ((x[4] + x[5]) + (x[6] + x[7]));
  }
  block_sum<NV, kBlock>(out, sm);
}

template <int NV>
__device__ __forceinline__ void write_partials(const EngineView& v, int item, double (&part)[NV], double* sm) {
  block_sum<NV, kBlock>(part, sm);
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) v.partials[(size_t)k * v.stride + item] = part[k];
}

// Pair partials: the FP32 path's item partials are FP32 pairs (hi, lo) stored in the 8-byte
// slots of the partials buffer, so that the last CTA sums them on the FP32 pipes (an FP64
// sum of the ~19k slice partials of a 512k-node pass would hold one SM's FP64 pipe for
// microseconds).
__device__ __forceinline__ void store_pair(double* partials, size_t idx, float hi, float lo) {
  reinterpret_cast<float2*>(partials)[idx] = make_float2(hi, lo);
}

// FP32 pair of an FP64 value x*x (x split into a pair, the square to ~2^-46 relative)
__device__ __forceinline__ void pair_square(double x, float& h, float& l) {
  float xh, xl;
  split_pair(x, xh, xl);
  h = xh * xh;
  l = fmaf(xh, xh, -h) + 2.0f * xh * xl;
}

// block sums of NV pairs per thread; thread 0 gets the FP64 values (sm: NV * BLK / 32
// doubles, used as pairs)
template <int NV, int BLK = kBlock>
__device__ __forceinline__ void block_pair_sum(float (&h)[NV], float (&l)[NV], double (&out)[NV], double* sm) {
  float2* smf = reinterpret_cast<float2*>(sm);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    pair_warp_sum(h[q], l[q]);
    if (lane == 0) smf[q * (BLK / 32) + wid] = make_float2(h[q], l[q]);
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      float th = 0.0f, tl = 0.0f;
      if (lane < BLK / 32) {
        th = smf[q * (BLK / 32) + lane].x;
        tl = smf[q * (BLK / 32) + lane].y;
      }
      pair_warp_sum(th, tl);
      out[q] = (double)th + (double)tl;
    }
  }
  __syncthreads();
}

// reduce NV pair partials of items [first, first+count) (layout partials[k*stride + item]);
// four independent pair accumulators per thread, combined in a fixed order
template <int NV, int BLK = kBlock>
__device__ __forceinline__ void reduce_pair_items(const double* partials, int stride, int first, int count,
                                                  double (&out)[NV], double* sm) {
  constexpr int U = 4;
  const float2* pp = reinterpret_cast<const float2*>(partials);
  float hh[NV], ll[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const float2* p = pp + (size_t)k * stride + first;
    float h[U], l[U];
#pragma unroll
    for (int u = 0; u < U; ++u) h[u] = l[u] = 0.0f;
    int b = threadIdx.x;
    for (; b + (U - 1) * BLK < count; b += U * BLK) {
      float2 x[U];
#pragma unroll
      for (int u = 0; u < U; ++u) x[u] = p[b + u * BLK];
#pragma unroll
      for (int u = 0; u < U; ++u) pair_add(h[u], l[u], x[u].x, x[u].y);
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (b + u * BLK < count) pair_add(h[u], l[u], p[b + u * BLK].x, p[b + u * BLK].y);
    pair_add(h[0], l[0], h[1], l[1]);
    pair_add(h[2], l[2], h[3], l[3]);
    pair_add(h[0], l[0], h[2], l[2]);
    hh[k] = h[0];
    ll[k] = l[0];
  }
  block_pair_sum<NV, BLK>(hh, ll, out, sm);
}

// the last CTA's reduction of items written by write_dot_partials
template <int NV, typename P>
__device__ __forceinline__ void reduce_dot_items(const double* partials, int stride, int first, int count,
                                                 double (&out)[NV], double* sm) {
  if constexpr (sizeof(P) == 8)
    reduce_items<NV>(partials, stride, first, count, out, sm);
  else
    reduce_pair_items<NV>(partials, stride, first, count, out, sm);
}

// Item partials of per-thread dot accumulators: FP64 block sums on the FP64 path; on the
// FP32 path FP32-pair warp sums, then warp 0 sums the warps' pairs (sm: NV * kBlock / 32
// doubles, reused as pairs) and stores the pair partials (reduce_dot_items sums them).
template <int NV, typename P>
__device__ __forceinline__ void write_dot_partials(const EngineView& v, int item, DotAcc<P> (&acc)[NV], double* sm) {
  if constexpr (sizeof(P) == 8) {
    double part[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) part[q] = acc[q].s;
    write_partials<NV>(v, item, part, sm);
  } else {
    float2* smf = reinterpret_cast<float2*>(sm);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      acc[q].warp_sum();
      if (lane == 0) smf[q * (kBlock / 32) + wid] = make_float2(acc[q].hi, acc[q].lo);
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        DotAcc<float> t;
        if (lane < kBlock / 32) {
          t.hi = smf[q * (kBlock / 32) + lane].x;
          t.lo = smf[q * (kBlock / 32) + lane].y;
        }
        t.warp_sum();
        if (lane == 0) store_pair(v.partials, (size_t)q * v.stride + item, t.hi, t.lo);
      }
    }
    __syncthreads();
  }
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
};
template <>
struct VecSel<double> {
  __device__ static double* rin(const KParams& k) { return k.rin64; }
  __device__ static double* z(const KParams& k) { return k.z64; }
  __device__ static double* p(const KParams& k) { return k.p64; }
  __device__ static double* q(const KParams& k) { return k.q64; }
  __device__ static double* e(const KParams& k) { return k.e64; }
  __device__ static const double* dinv(const KParams& k) { return k.dinv64; }
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

__device__ __forceinline__ float sel4(const float4& v, int s) {
  return s == 0 ? v.x : s == 1 ? v.y : s == 2 ? v.z : v.w;
}

// sum of pairs over the W lanes of a node's segment (lane 0 of the segment holds it)
template <int WIDTH>
__device__ __forceinline__ double seg_reduce_pair(float h, float l) {
#pragma unroll
  for (int off = WIDTH / 2; off > 0; off >>= 1) {
    const float oh = __shfl_down_sync(0xffffffffu, h, off, WIDTH);
    const float ol = __shfl_down_sync(0xffffffffu, l, off, WIDTH);
    pair_add(h, l, oh, ol);
  }
  return (double)h + (double)l;
}

// ------------------------------------------------------------------- potential: prep ----
// Per node: K11 diagonal (sum of liquid-liquid weights), unknown mask, right-hand side
// b = (1/(K sigma)) F CSolid sum_k z_k c_k and the FP64 residual r = b - A phi.  With F11_out
// (single instance), writes the reference's F11 (utils.h:798-841) for every node instead.
template <typename P, int W>
__global__ void __launch_bounds__(kBlock) k_prep(EngineView v, cudaGraphConditionalHandle hc,
                                                 double* F11_out) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ TileSmem ts;
  __shared__ double sm[2 * kBlock / 32];
  __shared__ int s_last;
  const int sub = threadIdx.x % W, seg = threadIdx.x / W, nseg = kBlock / W;
  for (int item = blockIdx.x; item < v.ntiles; item += gridDim.x) {
    const TileDesc t = v.tiles[item];
    const KParams& k = v.inst[t.inst];
    load_tile(t, ts);
    constexpr bool kPair = sizeof(P) == 4;  // mixed path: FP32-pair arithmetic on the bonds
    double* sphi = reinterpret_cast<double*>(dsm);
    float2* sphi2 = reinterpret_cast<float2*>(dsm);
    unsigned char* sfl = dsm + sizeof(double) * (size_t)t.halo;
    const unsigned short* sslot = stage_slots(k.slot16, t, dsm + align16(sizeof(double) * (size_t)t.halo + t.halo));
    const double* phi64 = k.phi64;
    const unsigned char* dm = k.dirmask;
    for (int s = threadIdx.x; s < t.halo; s += kBlock) {
      const int n = halo_node(ts, s);
      const double ph = phi64[n];
      if (kPair) {
        const float hi = (float)ph;
        sphi2[s] = make_float2(hi, (float)(ph - (double)hi));
      } else {
        sphi[s] = ph;
      }
      sfl[s] = (unsigned char)((phase_of<P>(k, n) == 0.0f ? 1 : 0) | (((dm[n] >> S) & 1) ? 2 : 0));
    }
    __syncthreads();
    double part[2] = {0.0, 0.0};
    const int* row = k.row;
    const double* w64 = k.w64;
    const int own0 = ts.off[4] + (t.own_begin - t.hb[4]);
    // the mask-only sums (diagonal, Dirichlet coupling, unknown flag) are kept from the
    // last prep while no phase changed: only sum_j w phi_j is formed then
    const bool cached = F11_out == nullptr && k.ds->op_valid != 0;
    for (int a0 = t.own_begin; a0 < t.own_end; a0 += nseg) {
      const int a = a0 + seg;
      const bool act = a < t.own_end;
      const int so = own0 + (a - t.own_begin);
      const unsigned char fa = act ? sfl[so] : 0;
      const bool scan = act && (fa & 1) && (F11_out != nullptr || !(fa & 2));
      double dsum = 0.0, swphi = 0.0, cpl = 0.0;
      int anyll = 0;
      if (cached) {
        if (kPair) {
          float sh = 0.f, sl = 0.f;
          if (scan && k.freem[a]) {
            for (int j = row[a] + sub; j < row[a + 1]; j += W) {
              const int s = sslot[j - t.bond0];
              if (sfl[s] & 1) {
                const float2 ph = sphi2[s];
                float ph_, pl_;
                pair_mul(k.w32[j], k.wlo32[j], ph.x, ph.y, ph_, pl_);
                pair_add(sh, sl, ph_, pl_);
              }
            }
          }
          swphi = seg_reduce_pair<W>(sh, sl);
        } else {
          if (scan && k.freem[a]) {
            for (int j = row[a] + sub; j < row[a + 1]; j += W) {
              const int s = sslot[j - t.bond0];
              if (sfl[s] & 1) swphi += w64[j] * sphi[s];
            }
          }
          swphi = seg_reduce_d<W>(swphi);
        }
      } else if (kPair) {
        float dh = 0.f, dl = 0.f, sh = 0.f, sl = 0.f, ch = 0.f, cl = 0.f;
        if (scan) {
          for (int j = row[a] + sub; j < row[a + 1]; j += W) {
            const int s = sslot[j - t.bond0];
            const unsigned char f = sfl[s];
            if (f & 1) {
              const float wh = k.w32[j], wl = k.wlo32[j];
              const float2 ph = sphi2[s];
              float ph_, pl_;
              pair_mul(wh, wl, ph.x, ph.y, ph_, pl_);
              pair_add(dh, dl, wh, wl);
              pair_add(sh, sl, ph_, pl_);
              anyll = 1;
              if (f & 2) pair_add(ch, cl, ph_, pl_);
            }
          }
        }
        dsum = seg_reduce_pair<W>(dh, dl);
        swphi = seg_reduce_pair<W>(sh, sl);
        cpl = seg_reduce_pair<W>(ch, cl);
      } else {
        if (scan) {
          for (int j = row[a] + sub; j < row[a + 1]; j += W) {
            const int s = sslot[j - t.bond0];
            const unsigned char f = sfl[s];
            if (f & 1) {
              const double w = w64[j];
              const double ph = sphi[s];
              dsum += w;
              swphi += w * ph;
              anyll = 1;
              if (f & 2) cpl += w * ph;
            }
          }
        }
        dsum = seg_reduce_d<W>(dsum);
        swphi = seg_reduce_d<W>(swphi);
        cpl = seg_reduce_d<W>(cpl);
      }
      anyll = seg_or<W>(anyll);
      if (act && sub == 0) {
        double b;
        if (k.b_override) {
          b = k.b_override[a];
        } else {
          double R11 = 0.0;
          for (int s = 0; s < S; ++s) R11 += k.z[s] * conc_of<P>(k, a, s);
          b = k.lam * R11;
        }
        const double pha = kPair ? (double)sphi2[so].x + (double)sphi2[so].y : sphi[so];
        if (F11_out) {
          F11_out[a] = anyll ? (dsum * pha - swphi) - b : 0.0;
        } else {
          bool fr;
          if (cached) {
            fr = k.freem[a] != 0;
            dsum = k.dsum64[a];
            cpl = k.cpl64[a];
          } else {
            fr = !(fa & 2) && (fa & 1) && anyll;
            k.freem[a] = fr ? 1 : 0;
            k.dsum64[a] = fr ? dsum : 1.0;
            k.cpl64[a] = fr ? cpl : 0.0;
            k.dinv64[a] = fr ? 1.0 / dsum : 0.0;
            k.d32[a] = fr ? (float)dsum : 1.0f;
            k.dinv32[a] = fr ? (float)(1.0 / dsum) : 0.0f;
          }
          const double bb = fr ? b : 0.0;
          const double r = fr ? bb - (dsum * pha - swphi) : 0.0;
          k.b64[a] = bb;
          k.r64[a] = r;
          const double be = bb + (fr ? cpl : 0.0);
          part[0] += be * be;
          part[1] += r * r;
        }
      }
    }
    if (!F11_out) {
      write_partials<2>(v, item, part, sm);
      if (item_done(&v.ticket[t.inst], v.tile_count[t.inst], &s_last)) {
        double tot[2];
        reduce_items<2>(v.partials, v.stride, v.tile_first[t.inst], v.tile_count[t.inst], tot, sm);
        if (threadIdx.x == 0) {
          DevState* ds = k.ds;
          ds->op_valid = 1;
          const double bn = tot[0] > 0.0 ? tot[0] : 1.0;
          ds->bnorm2 = bn;
          ds->rnorm2 = tot[1];
          ds->outer_it = 0;
          ds->solve_iters = 0;
          const bool go = tot[1] > ds->tol * ds->tol * bn && ds->max_outer > 0;
          if (!go) {
            ds->cg_solves += 1;
            ds->last_relres = sqrt(tot[1] / bn);
          }
          ds->outer_active = go ? 1 : 0;
          ds->inner_active = 0;
          instance_finished(v, t.inst, 0, hc);
        }
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------- potential: CG -------
// Inner PCG on A e = r (r: FP64 outer residual rounded to P).  Jacobi preconditioner
// (the reference's Eigen::DiagonalPreconditioner, main.cpp:714-768).
template <typename P>
__global__ void __launch_bounds__(kBlock) k_cg_init(EngineView v, cudaGraphConditionalHandle hc,
                                                    int fp64, int split) {
  __shared__ double sm[2 * kBlock / 32];
  __shared__ int s_last;
  for (int item = blockIdx.x; item < v.nchunks; item += gridDim.x) {
    const Chunk c = v.chunks[item];
    const KParams& k = v.inst[c.inst];
    const bool active = *((volatile int*)&k.ds->outer_active) != 0;
    DotAcc<P> part[2];
    if (split) {
      // two-level preconditioner: r, p, q, e here; z and the dots after the coarse solve
      if (active) {
        P* rin = VecSel<P>::rin(k);
        P* p = VecSel<P>::p(k);
        P* q = VecSel<P>::q(k);
        P* e = VecSel<P>::e(k);
        for (int a = c.begin + threadIdx.x; a < c.end; a += kBlock) {
          rin[a] = (P)k.r64[a];
          p[a] = P(0);
          q[a] = P(0);
          e[a] = P(0);
          if (sizeof(P) == 4) {  // the deflated solve's right-hand side and t = A e^
            k.r0_32[a] = (float)k.r64[a];
            k.t32[a] = 0.0f;
          }
        }
      }
      continue;
    }
    if (active) {
      P* rin = VecSel<P>::rin(k);
      P* z = VecSel<P>::z(k);
      P* p = VecSel<P>::p(k);
      P* q = VecSel<P>::q(k);
      P* e = VecSel<P>::e(k);
      const P* dinv = VecSel<P>::dinv(k);
      for (int a = c.begin + threadIdx.x; a < c.end; a += kBlock) {
        const P r = (P)k.r64[a];
        const P zz = r * dinv[a];
        rin[a] = r;
        z[a] = zz;
        p[a] = P(0);
        q[a] = P(0);
        e[a] = P(0);
        part[0].add(r, zz);
        part[1].add(r, r);
      }
    }
    write_dot_partials<2, P>(v, item, part, sm);
    if (item_done(&v.ticket[c.inst], v.chunk_count[c.inst], &s_last)) {
      double tot[2];
      reduce_dot_items<2, P>(v.partials, v.stride, v.chunk_first[c.inst], v.chunk_count[c.inst], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = k.ds;
        if (ds->outer_active) {
          ds->rz = tot[0];
          ds->rr = tot[1];
          ds->beta = 0.0;
          ds->alpha = 0.0;
          ds->inner_it = 0;
          // FP64: solve to the final tolerance in one sweep; mixed: reduce by inner_rel, but
          // not below what the outer tolerance needs (0.3 tol: the last sweep stops early)
          const double target = fp64 ? 0.25 * ds->tol * ds->tol * ds->bnorm2
                                     : fmax(ds->inner_rel * ds->inner_rel * tot[1],
                                            0.09 * ds->tol * ds->tol * ds->bnorm2);
          ds->inner_target = target;
          ds->inner_active = (tot[1] > target && ds->max_iter > 0) ? 1 : 0;
        } else {
          ds->inner_active = 0;
        }
        instance_finished(v, c.inst, 1, hc);
      }
    }
    __syncthreads();
  }
}

// Work split of the slice list: warp gw of nw takes the contiguous range [s0, s1), so the
// warps of one CTA walk neighbouring slices and share their neighbours in L1.
__device__ __forceinline__ void warp_slices(const EngineView& v, int* s0, int* s1) {
  const long long nw = (long long)gridDim.x * (kBlock / 32);
  const long long gw = (long long)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5);
  *s0 = (int)(((long long)v.nslices * gw) / nw);
  *s1 = (int)(((long long)v.nslices * (gw + 1)) / nw);
}

// the next slice of a kernel whose warps claim slices one at a time from the grid-wide
// counter ticket[M + 2] (reset by the kernel's last CTA); lane 0 claims, the warp shares it
__device__ __forceinline__ int claim_slice(const EngineView& v, int lane) {
  int s = 0;
  if (lane == 0) s = (int)atomicAdd(&v.ticket[v.M + 2], 1u);
  return __shfl_sync(0xffffffffu, s, 0);
}

__device__ __forceinline__ double warp_sum_d(double x) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
  return x;
}


// Interleaved sliced operator: bond column c of a slice holds 32 FP32 weights then 32 16-bit
// slot codes (kSellW floats = 192 bytes), so one contiguous copy moves both.
constexpr int kSellW = 48;      // stride of a column in floats
constexpr int kSellC = 96;      // stride of a column in 16-bit codes
__device__ __forceinline__ const float* sell_w(const KParams& k, const SliceDesc& d) {
  return k.sell + (size_t)(d.off >> 5) * kSellW;
}
__device__ __forceinline__ const unsigned short* sell_code(const KParams& k, const SliceDesc& d) {
  return reinterpret_cast<const unsigned short*>(sell_w(k, d) + 32);
}

// the CG operator's compacted copy (same layout and offsets; columns in use: cg_width)
__device__ __forceinline__ const float* sell_cg_w(const KParams& k, const SliceDesc& d) {
  return k.sell_cg + (size_t)(d.off >> 5) * kSellW;
}
__device__ __forceinline__ const unsigned short* sell_cg_code(const KParams& k, const SliceDesc& d) {
  return reinterpret_cast<const unsigned short*>(sell_cg_w(k, d) + 32);
}

// the inner-loop flag of a slice's instance (constant while the operator runs)
__device__ __forceinline__ bool slice_active(const EngineView& v, int sg) {
  return __ldg(&v.inst[__ldg(&v.slices[sg].inst)].ds->inner_active) != 0;
}

// node of a slot code: window row start (per-warp table of the slice's lo[]) + offset
// streamed operator loads: no L1 allocation (L1 stays with the gathered vectors) and L2
// evict-first (the operator is read once per pass; the vectors and the coarse inverse the
// other kernels of the iteration read stay in L2)
__device__ __forceinline__ uint64_t stream_policy() {
  uint64_t pol;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
__device__ __forceinline__ float ld_stream(const float* p) {
  float v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(stream_policy()));
  return v;
}
__device__ __forceinline__ unsigned int ld_stream(const unsigned short* p) {
  unsigned short v;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.u16 %0, [%1], %2;" : "=h"(v) : "l"(p), "l"(stream_policy()));
  return v;
}

__device__ __forceinline__ int code_node(const int* hb, unsigned int code) {
  return hb[code >> 12] + (int)(code & 4095u);
}

// q = A z + beta q, p = z + beta p (so that q = A p), partial p.q -> alpha.
// FP32, on the CG operator's slices (32 of a bin row's nodes without a potential Dirichlet
// value; each row holds only its bonds to possible unknowns, in bond order, zero-padded to
// the slice's longest; codes and weights column-major: one coalesced load per bond column),
// one lane per row.  WIN: the warp first copies the slice's window (the z values of its 9 window rows)
// into its shared-memory buffer with asynchronous 16-byte copies and gathers from there (the
// code's low 12 bits are the position in the window); otherwise it gathers from L1/L2.
// PF > 0: lane 0 keeps bulk L2 prefetches of the warp's operator stream PF batches ahead of
// the batch being read (the warp's slices are contiguous in the sliced array), so that the
// batch loads hit L2.  Slice partials are reduced per instance by the last CTA.
template <int W, bool WIN, int B, bool PIPE, int MINB, int PF = 0>
__global__ void __launch_bounds__(kBlock, MINB) k_cg_spmv32(EngineView v) {
  extern __shared__ __align__(16) float zwin[];
  __shared__ int s_hb[kBlock / 32][12];
  __shared__ double sm[kBlock / 32];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // PF == 0: warps claim slices one at a time (slices of solid nodes and narrow ones cost
  // less than full ones, and a static split leaves warps idle at the end of the single
  // wave); PF > 0 keeps each warp's contiguous range for its prefetch stream
  constexpr bool kClaim = PF == 0;
  const int ns = v.ncslices;
  int s0, s1;
  if (kClaim) {
    s0 = claim_slice(v, lane);
    s1 = ns;
  } else {
    const long long nw = (long long)gridDim.x * (kBlock / 32);
    const long long gw = (long long)blockIdx.x * (kBlock / 32) + warp;
    s0 = (int)(((long long)ns * gw) / nw);
    s1 = (int)(((long long)ns * (gw + 1)) / nw);
  }
  float* zw = zwin + (WIN ? (size_t)warp * kWinCap : 0);
  // prefetch window of the operator stream: [pf_next, pf_end) of the warp's byte range
  const char* pf_next = nullptr;
  const char* pf_end = nullptr;
  if (PF > 0 && s0 < s1) {
    const SliceDesc& da = v.cslices[s0];
    const SliceDesc& db = v.cslices[s1 - 1];
    pf_next = reinterpret_cast<const char*>(sell_cg_w(v.inst[da.inst], da));
    pf_end = reinterpret_cast<const char*>(sell_cg_w(v.inst[db.inst], db)) + (size_t)db.width * kSellW * 4;
    if (da.inst != db.inst) pf_end = pf_next;  // the range spans instances: no prefetch
    if (lane == 0) {
      const char* stop = pf_next + (size_t)PF * B * kSellW * 4;
      if (stop > pf_end) stop = pf_end;
      for (; pf_next < stop; pf_next += B * kSellW * 4)
        bulk_prefetch_l2(pf_next, (unsigned)min((size_t)B * kSellW * 4, (size_t)(pf_end - pf_next)));
    }
  }
  for (int sg = s0; sg < s1; sg = kClaim ? claim_slice(v, lane) : sg + 1) {
    const SliceDesc& d = v.cslices[sg];
    const int inst = __ldg(&d.inst);
    const KParams& k = v.inst[inst];
    DotAcc<float> part;
    if (__ldg(&k.ds->inner_active) != 0) {
      const int cs = sg - __ldg(&v.cslice_first[inst]);
      const int width = k.cg_width[cs];
      const int a = k.cg_rows[__ldg(&d.row0) + lane];
      const bool live = a >= 0 && k.freem[a];
      if (WIN && width > 0) {
        // the window (z of the 9 window rows, 16-byte aligned row segments) by 16-byte
        // cp.async, all copies in flight before the one wait
        const float* zg = k.z32;
#pragma unroll 1
        for (int r = 0; r < 9; ++r) {
          const int n = d.wlen[r], lo = d.lo[r], wo = d.woff[r];
          for (int i = 4 * lane; i < n; i += 128)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(zw + wo + i)), "l"(zg + lo + i)
                         : "memory");
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
      } else if (lane < 9) {
        s_hb[warp][lane] = d.gbase[lane];
      }
      __syncwarp();
      if (PF > 0 && lane == 0) {
        // keep the prefetches at least PF batches ahead of this slice's first column
        const char* target = reinterpret_cast<const char*>(sell_cg_w(k, d)) + (size_t)PF * B * kSellW * 4;
        if (target > pf_end) target = pf_end;
        for (; pf_next < target; pf_next += B * kSellW * 4)
          bulk_prefetch_l2(pf_next, (unsigned)min((size_t)B * kSellW * 4, (size_t)(pf_end - pf_next)));
      }
      // every lane of a slice with a live row runs the slice's columns (the shorter rows hold
      // code 0, weight 0), so that lane 0 can issue the prefetches
      if (PF > 0 ? __any_sync(0xffffffffu, live) : live) {
        const int* hb = s_hb[warp];
        const float* ws = sell_cg_w(k, d) + lane;
        const unsigned short* cs16 = sell_cg_code(k, d) + lane;
        const float* z = k.z32;
        // B columns per batch; PIPE: the next batch of streamed columns is in flight while
        // the current batch's neighbour values are gathered (more registers, fewer warps)
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        const int nb = width / B;
        float w[B];
        unsigned int code[B];
        if (PIPE && nb > 0) {
#pragma unroll
          for (int u = 0; u < B; ++u) {
            w[u] = ld_stream(ws + kSellW * u);
            code[u] = ld_stream(cs16 + kSellC * u);
          }
        }
        for (int b = 0; b < nb; ++b) {
          if (PF > 0 && lane == 0 && pf_next < pf_end) {
            bulk_prefetch_l2(pf_next, (unsigned)min((size_t)B * kSellW * 4, (size_t)(pf_end - pf_next)));
            pf_next += B * kSellW * 4;
          }
          if (!PIPE) {
#pragma unroll
            for (int u = 0; u < B; ++u) {
              w[u] = ld_stream(ws + kSellW * (b * B + u));
              code[u] = ld_stream(cs16 + kSellC * (b * B + u));
            }
          }
          float zv[B];
#pragma unroll
          for (int u = 0; u < B; ++u) zv[u] = WIN ? zw[code[u] & 4095u] : __ldg(z + code_node(hb, code[u]));
          float wc[B];
#pragma unroll
          for (int u = 0; u < B; ++u) wc[u] = w[u];
          if (PIPE && b + 1 < nb) {
            const int c1 = (b + 1) * B;
#pragma unroll
            for (int u = 0; u < B; ++u) {
              w[u] = ld_stream(ws + kSellW * (c1 + u));
              code[u] = ld_stream(cs16 + kSellC * (c1 + u));
            }
          }
#pragma unroll
          for (int u = 0; u < B; ++u) acc[u & 3] = fmaf(wc[u], zv[u], acc[u & 3]);
        }
        for (int c = nb * B; c < width; ++c) {
          const unsigned int cc = ld_stream(cs16 + kSellC * c);
          acc[0] = fmaf(ld_stream(ws + kSellW * c), WIN ? zw[cc & 4095u] : __ldg(z + code_node(hb, cc)), acc[0]);
        }
        if (live) {
          const float za = z[a];
          const float sa = k.d32[a] * za - ((acc[0] + acc[1]) + (acc[2] + acc[3]));
          const float beta = (float)k.ds->beta;
          const float qn = sa + beta * k.q32[a];
          const float pn = za + beta * k.p32[a];
          k.q32[a] = qn;
          k.p32[a] = pn;
          part.add(pn, qn);
        }
      }
      __syncwarp();
    }
    part.warp_sum();
    if (lane == 0) store_pair(v.partials, sg, part.hi, part.lo);
  }
  if (take_last_ticket(&v.ticket[v.M + 1], &s_last)) {
    for (int i = 0; i < v.M; ++i) {
      double tot[1];
      reduce_pair_items<1>(v.partials, v.stride, v.cslice_first[i], v.cslice_count[i], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = v.inst[i].ds;
        if (ds->inner_active) {
          ds->alpha = (tot[0] > 0.0 && isfinite(tot[0])) ? ds->rz / tot[0] : 0.0;
          ds->pq = tot[0];
        }
      }
    }
    if (threadIdx.x == 0) {
      v.ticket[v.M + 1] = 0;
      v.ticket[v.M + 2] = 0;
    }
  }
}

// Halo-staged FP32 CG operator with recomputed weights (variant 8): the product of
// k_cg_spmv32 (q = A z + beta q, p = z + beta p, partial p.q) over the rows and columns that
// can be unknowns of the potential solve (no Dirichlet value of the potential; the other
// columns hold z = 0).  A CTA claims tiles one at a time; for each it
//   - starts one bulk copy of the tile's code block into shared memory (an mbarrier wait,
//     bounded: a timeout is recorded in the instance's state and reported as NNPP_ERR_CUDA),
//   - stages the tile's halo as float4 {X, Y, Z, z}: the node's position in units of the bin
//     side, relative to the centre of the halo's box (|X| <= T/2 + 1, |Y|, |Z| <= 1.5, so
//     FP32 keeps it to ~1e-7 of a bin), and the CG vector z,
//   - then its warps take the tile's quads (longest first, from a shared counter); eight
//     lanes per row walk the row's codes (halo slots) and recompute each bond's weight
//     beta(xi) dV / xi^3 (utils.h:17-25, s = 0) from the two staged positions.
// HBM sees the 2-byte codes; positions and z of the halo come through L2.
constexpr unsigned kHaloWaitPolls = 1u << 22;  // polls of the tile copies' mbarrier
// z staging of a halo of hal_cap - 1 nodes: every row rounded out to 16-byte boundaries
__host__ __device__ constexpr int halo_zcap(int hal_cap) { return ((hal_cap - 1 + 9 * 8) + 3) & ~3; }

__device__ __forceinline__ float halo_bond(const float4& pa, const float4& pb, float hc0, float hc1) {
  const float dx = pb.x - pa.x, dy = pb.y - pa.y, dz = pb.z - pa.z;
  const float x2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float ri = rsqrtf(x2);
  const float be = fminf(1.0f, fmaf(-hc1, x2 * ri, hc0));
  return be * (ri * ri) * ri * pb.w;
}

// CHECK (nnpp_set_checks): every quad, row and code is checked against its bounds before
// it indexes an array (a bad one is recorded in bounds_error and replaced by the padding
// slot or an empty row), and with NNPP_CHECK_WAIT_PROBE the kernel also waits, bounded, on a
// barrier that nothing completes after each tile's copies have landed -- the timeout path
// without a copy in flight.
template <bool CHECK>
__global__ void __launch_bounds__(kBlock, 3) k_cg_spmv32h(EngineView v, int hal_cap, int quad_cap) {
  extern __shared__ __align__(16) float4 hal[];
  // after the halo: the z rows (each from a 16-byte aligned node, kHaloZPad floats of slack
  // per row), then the code block
  float* zst = reinterpret_cast<float*>(hal + hal_cap);
  // per quad of the tile: its rows' p.q as an FP32 pair (reduced in quad order, so that the
  // sum does not depend on which warp took which quad)
  float2* qpart = reinterpret_cast<float2*>(zst + halo_zcap(hal_cap));
  unsigned short* cod = reinterpret_cast<unsigned short*>(qpart + quad_cap);
  __shared__ __align__(8) uint64_t bar, probe_bar;
  __shared__ int s_tile, s_quad, s_last, s_stop;
  __shared__ int s_hb[9], s_pre[10], s_zb[9];
  __shared__ double sm[kBlock / 32];
  const int lane = threadIdx.x & 31;
  const int g = lane >> 3, j = lane & 7;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    if (CHECK) mbar_init(&probe_bar, 1);  // one arrival expected, none ever made
    fence_mbar_init();
    s_stop = 0;
  }
  __syncthreads();
  unsigned phase = 0;
  for (;;) {
    if (threadIdx.x == 0) {
      s_tile = s_stop ? v.ntiles : (int)atomicAdd(&v.ticket[v.M + 2], 1u);
      s_quad = 0;
    }
    __syncthreads();
    const int t = s_tile;
    if (t >= v.ntiles) break;
    const int inst = v.tiles[t].inst;
    const KParams& k = v.inst[inst];
    const HTile ht = v.htiles[t];
    const bool run = ht.nq > 0 && __ldg(&k.ds->inner_active) != 0;
    if (run) {
      if (threadIdx.x == 0) {
        // every row of the halo by bulk copies on one mbarrier: the position records (16
        // bytes a node, rows start 16-byte aligned) into their slots, the row's z values
        // from the 16-byte boundary at or below its first node (z is padded past N), and the
        // tile's code block
        int acc = 0, zacc = 0;
        unsigned bytes = (unsigned)ht.clen16 * 16u;
        for (int r = 0; r < 9; ++r) {
          const int hb = v.tiles[t].hb[r], hl = v.tiles[t].hl[r];
          s_hb[r] = hb;
          s_pre[r] = acc;
          const int a0 = hb & ~3;
          s_zb[r] = zacc - a0;  // z of node n of row r at zst[s_zb[r] + n]
          if (hl > 0) {
            bytes += (unsigned)hl * 16u + (unsigned)(((hb + hl + 3) & ~3) - a0) * 4u;
            zacc += ((hb + hl + 3) & ~3) - a0;
          }
          acc += hl;
        }
        s_pre[9] = acc;
        // the previous tile's reads and writes of these buffers come before the copies
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bar, bytes);
        for (int r = 0; r < 9; ++r) {
          const int hb = s_hb[r], hl = s_pre[r + 1] - s_pre[r];
          if (hl <= 0) continue;
          const int a0 = hb & ~3;
          bulk_g2s(hal + s_pre[r], k.posrec + hb, (unsigned)hl * 16u, &bar);
          bulk_g2s(zst + s_zb[r] + a0, k.z32 + a0, (unsigned)(((hb + hl + 3) & ~3) - a0) * 4u, &bar);
        }
        if (ht.clen16 > 0) bulk_g2s(cod, k.hcode + (size_t)ht.cstart16 * 8, (unsigned)ht.clen16 * 16u, &bar);
      }
      __syncthreads();
      if (!mbar_wait_bounded(&bar, phase, kHaloWaitPolls)) {
        k.ds->wait_timeout = 1;
        s_stop = 1;
      }
      phase ^= 1u;
      if (CHECK && (k.checks & NNPP_CHECK_WAIT_PROBE) && !mbar_wait_bounded(&probe_bar, 0, 1u << 10)) {
        k.ds->wait_timeout = 1;
        s_stop = 1;
      }
      // the records as float4 {X, Y, Z, z} in the halo's frame, in place
      const float hinv = k.hinv;
      const float xoff = 0.5f * (float)ht.T;
      const int halo = s_pre[9];
      for (int i = threadIdx.x; i < halo; i += kBlock) {
        int r = 0;
#pragma unroll
        for (int q = 1; q < 9; ++q) r += i >= s_pre[q] ? 1 : 0;
        const float4 pr = hal[i];
        const int pb = __float_as_int(pr.w);
        float4 o;
        o.x = fmaf(pr.x, hinv, (float)((pb & 1023) - ht.bx0) - xoff);
        o.y = fmaf(pr.y, hinv, (float)(((pb >> 10) & 1023) - ht.by) - 0.5f);
        o.z = fmaf(pr.z, hinv, (float)(((pb >> 20) & 1023) - ht.bz) - 0.5f);
        o.w = zst[s_zb[r] + s_hb[r] + (i - s_pre[r])];
        hal[i] = o;
      }
      // the padding slot: far away (weight 0) and z = 0
      if (threadIdx.x == 0) hal[halo] = make_float4(1e18f, 0.0f, 0.0f, 0.0f);
      __syncthreads();
      const int own = s_pre[4] - s_hb[4];  // slot of own node a: own + a
      const float hc0 = k.hc0, hc1 = k.hc1, hsw = k.hsw;
      const float beta = (float)k.ds->beta;
      for (;;) {
        int qi = 0;
        if (lane == 0) qi = atomicAdd(&s_quad, 1);
        qi = __shfl_sync(0xffffffffu, qi, 0);
        if (qi >= ht.nq) break;
        if (CHECK && (ht.q0 + qi < 0 || ht.q0 + qi >= k.hquad_n)) {
          if (lane == 0) k.ds->bounds_error = 1;
          break;
        }
        const HQuad* qd = k.hquad + ht.q0 + qi;
        int a = __ldg(&qd->rows[g]);
        int npass = __ldg(&qd->npass);
        if (CHECK) {
          const TileDesc& td = v.tiles[t];
          const int coff = __ldg(&qd->coff_rel);
          const bool bad_row = a != -1 && (a < td.own_begin || a >= td.own_end);
          const bool bad_codes = npass < 0 || coff < 0 || coff + 32 * npass > 8 * ht.clen16;
          if (bad_row || bad_codes) k.ds->bounds_error = 1;
          if (bad_row) a = -1;
          if (__any_sync(0xffffffffu, bad_codes)) npass = 0;
        }
        const bool live = a >= 0 && k.freem[a] != 0;
        if (!__any_sync(0xffffffffu, live)) {
          if (lane == 0) qpart[qi] = make_float2(0.0f, 0.0f);
          continue;
        }
        const float4 pa = a >= 0 ? hal[own + a] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const unsigned short* cq = cod + __ldg(&qd->coff_rel) + lane;
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        int p = 0;
        for (; p + 4 <= npass; p += 4) {
          unsigned sl[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) sl[u] = cq[32 * (p + u)];
          if (CHECK)
#pragma unroll
            for (int u = 0; u < 4; ++u)
              if (sl[u] > (unsigned)halo) {
                k.ds->bounds_error = 1;
                sl[u] = (unsigned)halo;
              }
          float4 pb[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) pb[u] = hal[sl[u]];
#pragma unroll
          for (int u = 0; u < 4; ++u) acc[u] += halo_bond(pa, pb[u], hc0, hc1);
        }
        for (; p < npass; ++p) {
          unsigned sl = cq[32 * p];
          if (CHECK && sl > (unsigned)halo) {
            k.ds->bounds_error = 1;
            sl = (unsigned)halo;
          }
          acc[0] += halo_bond(pa, hal[sl], hc0, hc1);
        }
        float sum = (acc[0] + acc[1]) + (acc[2] + acc[3]);
        sum += __shfl_xor_sync(0xffffffffu, sum, 4);
        sum += __shfl_xor_sync(0xffffffffu, sum, 2);
        sum += __shfl_xor_sync(0xffffffffu, sum, 1);
        float ph = 0.0f, pl = 0.0f;  // this row's p.q, TwoProd
        if (j == 0 && live) {
          const float za = pa.w;
          const float sa = __ldg(k.d32 + a) * za - hsw * sum;
          const float qn = sa + beta * k.q32[a];
          const float pn = za + beta * k.p32[a];
          k.q32[a] = qn;
          k.p32[a] = pn;
          ph = pn * qn;
          pl = fmaf(pn, qn, -ph);
        }
        // the quad's sum, rows in order
        float qh = __shfl_sync(0xffffffffu, ph, 0), ql = __shfl_sync(0xffffffffu, pl, 0);
#pragma unroll
        for (int r = 1; r < 4; ++r)
          pair_add(qh, ql, __shfl_sync(0xffffffffu, ph, 8 * r), __shfl_sync(0xffffffffu, pl, 8 * r));
        if (lane == 0) qpart[qi] = make_float2(qh, ql);
      }
    }
    __syncthreads();
    // the tile's partial: its quads' sums in quad order (lane l takes quads l, l + 32, ...,
    // then a fixed shuffle tree)
    if (threadIdx.x < 32) {
      float th = 0.0f, tl = 0.0f;
      if (run)
        for (int q = lane; q < ht.nq; q += 32) pair_add(th, tl, qpart[q].x, qpart[q].y);
      pair_warp_sum(th, tl);
      if (lane == 0) store_pair(v.partials, t, th, tl);
    }
  }
  if (take_last_ticket(&v.ticket[v.M + 1], &s_last)) {
    for (int i = 0; i < v.M; ++i) {
      double tot[1];
      reduce_pair_items<1>(v.partials, v.stride, v.tile_first[i], v.tile_count[i], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = v.inst[i].ds;
        if (ds->inner_active) {
          ds->alpha = (tot[0] > 0.0 && isfinite(tot[0])) ? ds->rz / tot[0] : 0.0;
          ds->pq = tot[0];
        }
      }
    }
    if (threadIdx.x == 0) {
      v.ticket[v.M + 1] = 0;
      v.ticket[v.M + 2] = 0;
    }
  }
}

// Staged FP32 CG operator (the same product as k_cg_spmv32, same work split).  Every warp
// owns, in shared memory,
//   - a ring of kTmaStages stages of kTmaCol interleaved bond columns of its slices (one
//     cp.async.bulk per stage, completed on an mbarrier), refilled by lane 0 as soon as the
//     warp has consumed the stage, and
//   - two window buffers: the z values of the current slice's 9 window rows (the only nodes
//     its bonds reach) and, in flight, the next slice's, copied by the lanes with 16-byte
//     cp.async.
// The gathers are shared-memory loads; HBM only sees the streamed operator.  Waits are
// bounded: a timeout is recorded in the instance's state (reported as NNPP_ERR_CUDA).
constexpr int kTmaCol = 32;
constexpr int kTmaStages = 2;
constexpr int kStageBytes = kTmaCol * kSellW * 4;  // 6 KB
constexpr int kWarpsCta = kBlock / 32;
constexpr size_t kTmaRingBytes = (size_t)kWarpsCta * kTmaStages * kStageBytes;
constexpr size_t kTmaWinBytes = (size_t)kWarpsCta * 2 * kWinCap * sizeof(float);
constexpr size_t kTmaBarBytes = (size_t)kWarpsCta * kTmaStages * sizeof(uint64_t);
constexpr unsigned kWaitPolls = 1u << 22;

__device__ __forceinline__ int tma_chunks(int width) { return width > 0 ? (width + kTmaCol - 1) / kTmaCol : 1; }

// a warp's operator producer (lane 0): position in its slice range and the current slice's
// descriptors, loaded once per slice so that issuing a chunk costs no dependent loads
struct TmaCursor {
  int sg, ch;
  int loaded;  // slice whose fields below are valid (-1: none)
  int width, nch;
  const float* base;
};

// lane 0: issue the cursor's chunk into `stage` and advance; false when the range is done
__device__ __forceinline__ bool tma_produce(const EngineView& v, TmaCursor& c, int s1, int warp, int stage,
                                            unsigned char* ring, uint64_t* bars, uint64_t pol) {
  if (c.loaded != c.sg) {
    while (c.sg < s1 && !slice_active(v, c.sg)) {
      ++c.sg;  // inactive instance: the consumer skips its slices too
      c.ch = 0;
    }
    if (c.sg >= s1) return false;
    const SliceDesc& d = v.slices[c.sg];
    c.width = d.width;
    c.nch = tma_chunks(c.width);
    c.base = sell_w(v.inst[d.inst], d);
    c.loaded = c.sg;
  }
  const int c0 = c.ch * kTmaCol;
  const int cc = min(kTmaCol, max(c.width - c0, 0));
  unsigned char* buf = ring + (size_t)(warp * kTmaStages + stage) * kStageBytes;
  uint64_t* bar = bars + warp * kTmaStages + stage;
  fence_proxy_async_smem();
  mbar_arrive_expect_tx(bar, (unsigned)(cc * kSellW * 4));
  if (cc > 0) bulk_g2s_hint(buf, c.base + (size_t)c0 * kSellW, (unsigned)(cc * kSellW * 4), bar, pol);
  if (++c.ch >= c.nch) {
    c.ch = 0;
    ++c.sg;
  }
  return true;
}

// all lanes: 16-byte cp.async copies of the window of the next active slice at or after *ws
// into zw, then one commit group (empty when no slice is left); advances *ws past it
__device__ __forceinline__ void win_copy(const EngineView& v, int* ws, int s1, float* zw, int lane) {
  while (*ws < s1 && !slice_active(v, *ws)) ++*ws;
  if (*ws < s1) {
    const SliceDesc& d = v.slices[*ws];
    const float* z = v.inst[d.inst].z32;
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
      const int n = d.wlen[r], lo = d.lo[r], wo = d.woff[r];
      for (int i = 4 * lane; i < n; i += 128)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(zw + wo + i)), "l"(z + lo + i)
                     : "memory");
    }
    ++*ws;
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

template <int W>
__global__ void __launch_bounds__(kBlock, 1) k_cg_spmv32t(EngineView v) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ double sm[kBlock / 32];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* ring = dsm;
  float* wins = reinterpret_cast<float*>(dsm + kTmaRingBytes);
  uint64_t* bars = reinterpret_cast<uint64_t*>(dsm + kTmaRingBytes + kTmaWinBytes);
  if (threadIdx.x < kWarpsCta * kTmaStages) mbar_init(bars + threadIdx.x, 1);
  fence_mbar_init();
  __syncthreads();
  int s0, s1;
  warp_slices(v, &s0, &s1);
  float* mywin = wins + (size_t)warp * 2 * kWinCap;
  TmaCursor pc{s0, 0, -1, 0, 0, nullptr};
  int wsrc = s0;  // next slice whose window is to be copied
  const uint64_t pol = l2_evict_first_policy();  // the operator is read once per launch
  if (lane == 0)
    for (int st = 0; st < kTmaStages; ++st)
      if (!tma_produce(v, pc, s1, warp, st, ring, bars, pol)) break;
  win_copy(v, &wsrc, s1, mywin, lane);
  int stage = 0, wb = 0;
  unsigned phases = 0u;
  int timed_out = -1;  // instance whose wait gave up
  for (int sg = s0; sg < s1; ++sg) {
    const SliceDesc& d = v.slices[sg];
    const KParams& k = v.inst[d.inst];
    DotAcc<float> part;
    if (slice_active(v, sg)) {
      // the next slice's window goes to the other buffer (free: its slice is done), then
      // this slice's window (the older commit group) is waited for
      win_copy(v, &wsrc, s1, mywin + (wb ^ 1) * kWinCap, lane);
      const int width = d.width;
      const int a = d.row0 + lane;
      const bool live = lane < d.nrows && k.freem[a];
      float za = 0.0f, da = 0.0f, qa = 0.0f, pa = 0.0f;
      if (live) {
        za = k.z32[a];
        da = k.d32[a];
        qa = k.q32[a];
        pa = k.p32[a];
      }
      asm volatile("cp.async.wait_group 1;" ::: "memory");
      __syncwarp();
      const float* zw = mywin + wb * kWinCap;
      float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      const int nch = tma_chunks(width);
      for (int ch = 0; ch < nch; ++ch) {
        uint64_t* bar = bars + warp * kTmaStages + stage;
        if (!mbar_wait_bounded(bar, (phases >> stage) & 1u, kWaitPolls)) timed_out = d.inst;
        phases ^= 1u << stage;
        const float* sw = reinterpret_cast<const float*>(ring + (size_t)(warp * kTmaStages + stage) * kStageBytes) + lane;
        const unsigned short* sc = reinterpret_cast<const unsigned short*>(sw - lane + 32) + lane;
        const int cc = min(kTmaCol, width - ch * kTmaCol);
        if (cc == kTmaCol) {
#pragma unroll 8
          for (int c = 0; c < kTmaCol; ++c) {
            const unsigned q = sc[kSellC * c];
            acc[c & 3] = fmaf(sw[kSellW * c], zw[q & 4095u], acc[c & 3]);
          }
        } else {
          for (int c = 0; c < cc; ++c) {
            const unsigned q = sc[kSellC * c];
            acc[c & 3] = fmaf(sw[kSellW * c], zw[q & 4095u], acc[c & 3]);
          }
        }
        __syncwarp();
        if (lane == 0) tma_produce(v, pc, s1, warp, stage, ring, bars, pol);
        stage = stage + 1 == kTmaStages ? 0 : stage + 1;
      }
      if (live) {
        const float sa = da * za - ((acc[0] + acc[1]) + (acc[2] + acc[3]));
        const float beta = (float)k.ds->beta;
        const float qn = sa + beta * qa;
        const float pn = za + beta * pa;
        k.q32[a] = qn;
        k.p32[a] = pn;
        part.add(pn, qn);
      }
      __syncwarp();
      wb ^= 1;
    }
    part.warp_sum();
    if (lane == 0) store_pair(v.partials, sg, part.hi, part.lo);
  }
  asm volatile("cp.async.wait_all;" ::: "memory");
  if (timed_out >= 0 && lane == 0) v.inst[timed_out].ds->wait_timeout = 1;
  if (take_last_ticket(&v.ticket[v.M + 1], &s_last)) {
    for (int i = 0; i < v.M; ++i) {
      double tot[1];
      reduce_pair_items<1>(v.partials, v.stride, v.slice_first[i], v.slice_count[i], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = v.inst[i].ds;
        if (ds->inner_active) {
          ds->alpha = (tot[0] > 0.0 && isfinite(tot[0])) ? ds->rz / tot[0] : 0.0;
          ds->pq = tot[0];
        }
      }
    }
    if (threadIdx.x == 0) v.ticket[v.M + 1] = 0;
  }
}

// Streamed FP32 CG operator for single-instance engines (the same product and work split as
// k_cg_spmv32).  A warp's slices are consecutive in the sliced array, so its whole share of
// the operator is one contiguous byte range: lane 0 streams it through a ring of `stages`
// shared-memory stages of kTmaCol bond columns with cp.async.bulk (completed on mbarriers,
// refilled as soon as a stage is consumed), independently of the slice boundaries.  The
// lanes consume the columns slice by slice and gather from double-buffered slice windows.
// Nothing on a slice's path waits on a dependent global load: the slice descriptors arrive
// by cp.async three slices ahead into a shared-memory ring of four, and each slice's window
// one slice ahead (one cp.async group per slice: the window of slice s + 1 and the
// descriptor of slice s + 3).
// Dynamic shared memory: ring [warps][stages][kStageBytes], windows [warps][2][win_cap]
// floats, barriers [warps][stages], descriptors [warps][4].  Waits are bounded (timeout
// recorded in the state).
constexpr int kDescRing = 4;

// lanes 0..11: 16-byte cp.async copies of slice sg's descriptor into dst (no-op past s1)
__device__ __forceinline__ void desc_copy(const EngineView& v, int sg, int s1, SliceDesc* dst, int lane) {
  static_assert(sizeof(SliceDesc) % 16 == 0, "slice descriptor copied in 16-byte pieces");
  if (sg < s1 && lane < (int)(sizeof(SliceDesc) / 16))
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(reinterpret_cast<char*>(dst) + 16 * lane)),
                 "l"(reinterpret_cast<const char*>(v.slices + sg) + 16 * lane)
                 : "memory");
}

// all lanes: 16-byte cp.async copies of the window of the slice described by d into zw
__device__ __forceinline__ void win_copy_desc(const SliceDesc& d, const float* z, float* zw, int lane) {
#pragma unroll 1
  for (int r = 0; r < 9; ++r) {
    const int n = d.wlen[r], lo = d.lo[r], wo = d.woff[r];
    for (int i = 4 * lane; i < n; i += 128)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(zw + wo + i)), "l"(z + lo + i)
                   : "memory");
  }
}

template <int W, int COL>
__global__ void __launch_bounds__(kBlock, 1) k_cg_spmv32s(EngineView v, int stages, int win_cap) {
  constexpr int SB = COL * kSellW * 4;  // bytes of a stage
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ double sm[kBlock / 32];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const size_t ring_bytes = (size_t)kWarpsCta * stages * SB;
  const size_t win_bytes = (size_t)kWarpsCta * 2 * win_cap * sizeof(float);
  unsigned char* ring = dsm;
  float* wins = reinterpret_cast<float*>(dsm + ring_bytes);
  uint64_t* bars = reinterpret_cast<uint64_t*>(dsm + ring_bytes + win_bytes);
  SliceDesc* descs = reinterpret_cast<SliceDesc*>(dsm + ring_bytes + win_bytes +
                                                  (size_t)kWarpsCta * stages * sizeof(uint64_t));
  if (threadIdx.x < kWarpsCta * stages) mbar_init(bars + threadIdx.x, 1);
  fence_mbar_init();
  __syncthreads();
  int s0, s1;
  warp_slices(v, &s0, &s1);
  const KParams& k = v.inst[0];
  int timed_out = 0;
  if (s0 < s1 && slice_active(v, s0)) {
    const SliceDesc& da = v.slices[s0];
    const SliceDesc& db = v.slices[s1 - 1];
    const char* base = reinterpret_cast<const char*>(sell_w(k, da));
    const size_t total = ((size_t)((db.off - da.off) >> 5) + (size_t)db.width) * kSellW * 4;
    const uint64_t pol = l2_evict_first_policy();  // the operator is read once per launch
    unsigned char* myring = ring + (size_t)warp * stages * SB;
    uint64_t* mybars = bars + warp * stages;
    SliceDesc* mydesc = descs + warp * kDescRing;
    size_t pos = 0;  // lane 0: bytes of the range issued so far
    if (lane == 0)
      for (int st = 0; st < stages && pos < total; ++st) {
        const unsigned bytes = (unsigned)min((size_t)SB, total - pos);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(mybars + st, bytes);
        bulk_g2s_hint(myring + (size_t)st * SB, base + pos, bytes, mybars + st, pol);
        pos += bytes;
      }
    const float* zg = k.z32;
    float* mywin = wins + (size_t)warp * 2 * win_cap;
    // descriptors of s0 and s0 + 1 now; then the window of s0 with the descriptor of s0 + 2
    desc_copy(v, s0, s1, mydesc, lane);
    desc_copy(v, s0 + 1, s1, mydesc + 1, lane);
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncwarp();
    win_copy_desc(mydesc[0], zg, mywin, lane);
    desc_copy(v, s0 + 2, s1, mydesc + 2, lane);
    asm volatile("cp.async.commit_group;" ::: "memory");
    int stage = 0, wb = 0;
    unsigned phases = 0u;
    bool ready = false;
    int cis = 0;  // column within the current stage
    for (int sg = s0; sg < s1; ++sg) {
      const int j = sg - s0;
      // this slice's window and the descriptors up to sg + 2 are in
      asm volatile("cp.async.wait_group 0;" ::: "memory");
      __syncwarp();
      const SliceDesc& d = mydesc[j & (kDescRing - 1)];
      if (sg + 1 < s1) win_copy_desc(mydesc[(j + 1) & (kDescRing - 1)], zg, mywin + (wb ^ 1) * win_cap, lane);
      desc_copy(v, sg + 3, s1, mydesc + ((j + 3) & (kDescRing - 1)), lane);
      asm volatile("cp.async.commit_group;" ::: "memory");
      const int width = d.width;
      const int a = d.row0 + lane;
      const bool row = lane < d.nrows;
      bool live = false;
      float za = 0.0f, dd = 0.0f, qa = 0.0f, pa = 0.0f;
      if (row) {
        live = k.freem[a] != 0;
        za = k.z32[a];
        dd = k.d32[a];
        qa = k.q32[a];
        pa = k.p32[a];
      }
      const float* zw = mywin + wb * win_cap;
      float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      int c = 0;
      while (c < width) {
        if (!ready) {
          if (!mbar_wait_bounded(mybars + stage, (phases >> stage) & 1u, kWaitPolls)) timed_out = 1;
          phases ^= 1u << stage;
          ready = true;
        }
        const float* sw = reinterpret_cast<const float*>(myring + (size_t)stage * SB) + lane;
        const unsigned short* sc = reinterpret_cast<const unsigned short*>(sw - lane + 32) + lane;
        const int n = min(COL - cis, width - c);
        if (n == COL) {
#pragma unroll 8
          for (int q = 0; q < COL; ++q) {
            const unsigned code = sc[kSellC * q];
            acc[q & 3] = fmaf(sw[kSellW * q], zw[code & 4095u], acc[q & 3]);
          }
        } else {
          for (int q = cis; q < cis + n; ++q) {
            const unsigned code = sc[kSellC * q];
            acc[q & 3] = fmaf(sw[kSellW * q], zw[code & 4095u], acc[q & 3]);
          }
        }
        c += n;
        cis += n;
        if (cis == COL) {
          // stage consumed: refill it with the range's next chunk
          __syncwarp();
          if (lane == 0 && pos < total) {
            const unsigned bytes = (unsigned)min((size_t)SB, total - pos);
            fence_proxy_async_smem();
            mbar_arrive_expect_tx(mybars + stage, bytes);
            bulk_g2s_hint(myring + (size_t)stage * SB, base + pos, bytes, mybars + stage, pol);
            pos += bytes;
          }
          stage = stage + 1 == stages ? 0 : stage + 1;
          ready = false;
          cis = 0;
        }
      }
      DotAcc<float> part;
      if (live) {
        const float sa = dd * za - ((acc[0] + acc[1]) + (acc[2] + acc[3]));
        const float beta = (float)k.ds->beta;
        const float qn = sa + beta * qa;
        const float pn = za + beta * pa;
        k.q32[a] = qn;
        k.p32[a] = pn;
        part.add(pn, qn);
      }
      __syncwarp();
      wb ^= 1;
      part.warp_sum();
      if (lane == 0) store_pair(v.partials, sg, part.hi, part.lo);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
  } else {
    for (int sg = s0; sg < s1; ++sg)
      if (lane == 0) store_pair(v.partials, sg, 0.0f, 0.0f);
  }
  if (timed_out && lane == 0) k.ds->wait_timeout = 1;
  if (take_last_ticket(&v.ticket[v.M + 1], &s_last)) {
    double tot[1];
    reduce_pair_items<1>(v.partials, v.stride, v.slice_first[0], v.slice_count[0], tot, sm);
    if (threadIdx.x == 0) {
      DevState* ds = k.ds;
      if (ds->inner_active) {
          ds->alpha = (tot[0] > 0.0 && isfinite(tot[0])) ? ds->rz / tot[0] : 0.0;
          ds->pq = tot[0];
        }
      v.ticket[v.M + 1] = 0;
    }
  }
}

// FP64 operator: stored FP64 weights, staged FP64 vector values
template <int W>
__global__ void __launch_bounds__(kBlock) k_cg_spmv64(EngineView v) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ TileSmem ts;
  __shared__ double sm[kBlock / 32];
  __shared__ int s_last;
  const int sub = threadIdx.x % W, seg = threadIdx.x / W, nseg = kBlock / W;
  for (int item = blockIdx.x; item < v.ntiles; item += gridDim.x) {
    const TileDesc t = v.tiles[item];
    const KParams& k = v.inst[t.inst];
    const bool active = *((volatile int*)&k.ds->inner_active) != 0;
    double part[1] = {0.0};
    if (active) {
      load_tile(t, ts);
      double* hs = reinterpret_cast<double*>(dsm);
      const unsigned short* sslot = stage_slots(k.slot16, t, dsm + align16(sizeof(double) * (size_t)t.halo));
      const double* z = k.z64;
      for (int s = threadIdx.x; s < t.halo; s += kBlock) hs[s] = z[halo_node(ts, s)];
      __syncthreads();
      const int* row = k.row;
      const double* w64 = k.w64;
      const unsigned char* freem = k.freem;
      double* p = k.p64;
      double* q = k.q64;
      const double beta = k.ds->beta;
      const int own0 = ts.off[4] + (t.own_begin - t.hb[4]);
      for (int a0 = t.own_begin; a0 < t.own_end; a0 += nseg) {
        const int a = a0 + seg;
        const bool act = a < t.own_end && freem[a];
        double acc = 0.0;
        if (act)
          for (int j = row[a] + sub; j < row[a + 1]; j += W) acc = fma(w64[j], hs[sslot[j - t.bond0]], acc);
        acc = seg_reduce_d<W>(acc);
        if (act && sub == 0) {
          const double za = hs[own0 + (a - t.own_begin)];
          const double s = k.dsum64[a] * za - acc;
          const double qn = s + beta * q[a];
          const double pn = za + beta * p[a];
          q[a] = qn;
          p[a] = pn;
          part[0] += pn * qn;
        }
      }
    }
    write_partials<1>(v, item, part, sm);
    if (item_done(&v.ticket[t.inst], v.tile_count[t.inst], &s_last)) {
      double tot[1];
      reduce_items<1>(v.partials, v.stride, v.tile_first[t.inst], v.tile_count[t.inst], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = k.ds;
        if (ds->inner_active) {
          ds->alpha = (tot[0] > 0.0 && isfinite(tot[0])) ? ds->rz / tot[0] : 0.0;
          ds->pq = tot[0];
        }
        v.ticket[t.inst] = 0;
      }
    }
    __syncthreads();
  }
}

// e += alpha p, r -= alpha q, z = D^-1 r, partial r.z and r.r -> beta, stop test
template <typename P>
__global__ void __launch_bounds__(kBlock) k_cg_update(EngineView v, cudaGraphConditionalHandle hc) {
  __shared__ double sm[2 * kBlock / 32];
  __shared__ int s_last;
  for (int item = blockIdx.x; item < v.nchunks; item += gridDim.x) {
    const Chunk c = v.chunks[item];
    const KParams& k = v.inst[c.inst];
    const bool active = *((volatile int*)&k.ds->inner_active) != 0;
    DotAcc<P> part[2];
    if (active) {
      P* rin = VecSel<P>::rin(k);
      P* z = VecSel<P>::z(k);
      const P* p = VecSel<P>::p(k);
      const P* q = VecSel<P>::q(k);
      P* e = VecSel<P>::e(k);
      const P* dinv = VecSel<P>::dinv(k);
      const P alpha = (P)k.ds->alpha;
      for (int a = c.begin + threadIdx.x; a < c.end; a += kBlock) {
        const P di = dinv[a];
        if (di == P(0)) continue;
        const P ee = e[a] + alpha * p[a];
        const P r = rin[a] - alpha * q[a];
        const P zz = r * di;
        e[a] = ee;
        rin[a] = r;
        z[a] = zz;
        part[0].add(r, zz);
        part[1].add(r, r);
      }
    }
    write_dot_partials<2, P>(v, item, part, sm);
    if (item_done(&v.ticket[c.inst], v.chunk_count[c.inst], &s_last)) {
      double tot[2];
      reduce_dot_items<2, P>(v.partials, v.stride, v.chunk_first[c.inst], v.chunk_count[c.inst], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = k.ds;
        if (ds->inner_active) {
          const double alpha_d = ds->alpha;
          ds->beta = ds->rz != 0.0 ? tot[0] / ds->rz : 0.0;
          ds->rz = tot[0];
          ds->rr = tot[1];
          ds->inner_it += 1;
          ds->solve_iters += 1;
          ds->cg_iters += 1;
          const bool go = alpha_d != 0.0 && isfinite(tot[1]) && tot[1] > ds->inner_target &&
                          ds->inner_it < ds->max_iter && ds->solve_iters < ds->max_iter;
          ds->inner_active = go ? 1 : 0;
        }
        instance_finished(v, c.inst, 1, hc);
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ two-level preconditioner ----
// Applied as z = D^-1 r + P A_c^-1 P^T r per instance (block diagonal over an ensemble; the
// coarse spaces and their inverses come from coarse.cu): the restriction sums r over each
// aggregate, the coarse solve is one product with the dense inverse, and k_cg_zdots forms z
// with the CG's dots and decisions.  Instances without a coarse space (k.coarse == 0) take
// z = D^-1 r.  All reductions run in a fixed order (reproducible iterates).
__device__ __forceinline__ bool coarse_active(const KParams& k, int which) {
  return (which ? *((volatile int*)&k.ds->inner_active) : *((volatile int*)&k.ds->outer_active)) != 0;
}

// The mixed inner CG runs deflated (DEF1: CG on P_d A e^ = P_d r with P_d = I - A Q,
// Q = P A_c^-1 P^T, e = Q r + e^ - Q A e^) while the coarse operator and A P match the
// phases; otherwise it takes the additive coarse correction.
template <typename P>
__device__ __forceinline__ bool deflating(const KParams& k) {
  return sizeof(P) == 4 && k.coarse && k.defl_ok && *((volatile const int*)&k.ds->defl) != 0;
}

// (A P x_c)_i of an unknown i: its diagonal term from the CG operator's diagonal, the rest
// from the stored rows.  Eight slots at a time (with aggregates two or more bins wide, a
// node's bonds reach at most 8 aggregates): their loads and gathers are in flight together,
// the sum runs in slot order.
__device__ __forceinline__ float ap_apply(const KParams& k, int i) {
  const float* xc = k.xc;
  float s = __ldg(k.d32 + i) * __ldg(xc + __ldg(k.agg + i));
  const size_t N = (size_t)k.N;
  int q = 0;
  for (; q + 8 <= k.ap_k; q += 8) {
    int col[8];
    float val[8], xv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      col[u] = __ldg(k.ap_col + (size_t)(q + u) * N + i);
      val[u] = __ldg(k.ap_val + (size_t)(q + u) * N + i);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) xv[u] = __ldg(xc + col[u]);
#pragma unroll
    for (int u = 0; u < 8; ++u) s = fmaf(val[u], xv[u], s);
  }
  for (; q < k.ap_k; ++q) {
    const size_t o = (size_t)q * N + i;
    s = fmaf(__ldg(k.ap_val + o), __ldg(xc + __ldg(k.ap_col + o)), s);
  }
  return s;
}

// warp per aggregate, the instances one after another
template <typename P>
__global__ void __launch_bounds__(kBlock) k_coarse_restrict(EngineView v, int which) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  for (int inst = 0; inst < v.M; ++inst) {
    const KParams& k = v.inst[inst];
    if (!k.coarse || !coarse_active(k, which == 2 ? 0 : which)) continue;
    if (which == 2 && !deflating<P>(k)) continue;  // the deflated solve's final correction only
    const P* r = VecSel<P>::rin(k);
    for (int I = gw; I < k.cn; I += warps) {
      const int ax = I % k.cna0, ay = (I / k.cna0) % k.cna1, az = I / (k.cna0 * k.cna1);
      const int bx0 = ax * k.cf, bx1 = min(bx0 + k.cf, k.nb0);
      float acc = 0.0f;
      for (int bz = az * k.cf; bz < min(az * k.cf + k.cf, k.nb2); ++bz)
        for (int by = ay * k.cf; by < min(ay * k.cf + k.cf, k.nb1); ++by) {
          // the aggregate's bins along x are one contiguous node range
          const int b0 = bx0 + k.nb0 * (by + k.nb1 * bz);
          const int i0 = k.bin_start[b0], i1 = k.bin_start[b0 + (bx1 - bx0)];
          for (int i = i0 + lane; i < i1; i += 32) acc += (float)r[i];
        }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
      if (lane == 0) k.rc[I] = acc;
    }
  }
}

// The CG update of the split (two-level) iteration fused with the restriction: e += alpha p,
// r -= alpha q on the unknowns, with a warp per aggregate walking its bins' node ranges, so
// that the new residual is summed into r_c[I] as it is written, with the aggregate's parts
// of r.D^-1 r and r.r.
template <typename P>
__global__ void __launch_bounds__(kBlock) k_cg_update_restrict(EngineView v) {
  __shared__ int2 s_runs[kBlock / 32][32];
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  for (int inst = 0; inst < v.M; ++inst) {
    const KParams& k = v.inst[inst];
    if (!coarse_active(k, 1)) continue;
    P* rin = VecSel<P>::rin(k);
    const P* p = VecSel<P>::p(k);
    const P* q = VecSel<P>::q(k);
    P* e = VecSel<P>::e(k);
    const P* dinv = VecSel<P>::dinv(k);
    const P alpha = (P)k.ds->alpha;
    if (!k.coarse) continue;  // engines run the split iteration only when every member has one
    const bool def = deflating<P>(k);
    for (int I = gw; I < k.cn; I += warps) {
      const int ax = I % k.cna0, ay = (I / k.cna0) % k.cna1, az = I / (k.cna0 * k.cna1);
      const int bx0 = ax * k.cf, bx1 = min(bx0 + k.cf, k.nb0);
      if (def) {
        // deflated iteration: restrict q = A p (the update follows the coarse product)
        float acc = 0.0f;
        const int y0 = ay * k.cf, ny = min(y0 + k.cf, k.nb1) - y0;
        const int z0 = az * k.cf, nr = ny * (min(z0 + k.cf, k.nb2) - z0);
        if (nr <= 32) {
          // the aggregate's runs (cf bins along x each): their bounds loaded one run a lane,
          // then the warp walks the runs' concatenation, eight elements a lane in flight
          int lo = 0, len = 0;
          if (lane < nr) {
            const int b0 = bx0 + k.nb0 * ((y0 + lane % ny) + k.nb1 * (z0 + lane / ny));
            lo = k.bin_start[b0];
            len = k.bin_start[b0 + (bx1 - bx0)] - lo;
          }
          int pre = len;
#pragma unroll
          for (int off = 1; off < 32; off <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, pre, off);
            if (lane >= off) pre += t;
          }
          const int total = __shfl_sync(0xffffffffu, pre, 31);
          int2* runs = s_runs[(threadIdx.x >> 5)];
          __syncwarp();
          if (lane < nr) runs[lane] = make_int2(pre - len, lo);  // (first position, first node)
          __syncwarp();
          for (int base = 0; base < total; base += 32 * 8) {
            P qv[8], dv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int idx = base + lane + 32 * u;
              qv[u] = dv[u] = P(0);
              if (idx < total) {
                int node = 0;
                for (int r = 0; r < nr; ++r) {
                  const int2 ru = runs[r];
                  if (idx >= ru.x) node = ru.y + (idx - ru.x);
                }
                dv[u] = dinv[node];
                qv[u] = q[node];
              }
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) acc += (float)(dv[u] != P(0) ? qv[u] : P(0));
          }
        } else {
          for (int bz = z0; bz < min(z0 + k.cf, k.nb2); ++bz)
            for (int by = y0; by < y0 + ny; ++by) {
              const int b0 = bx0 + k.nb0 * (by + k.nb1 * bz);
              const int i0 = k.bin_start[b0], i1 = k.bin_start[b0 + (bx1 - bx0)];
              for (int i = i0 + lane; i < i1; i += 32) acc += (float)(dinv[i] != P(0) ? q[i] : P(0));
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (lane == 0) k.rc[I] = acc;
        continue;
      }
      float acc = 0.0f;
      DotAcc<P> rzf, rr;  // r.D^-1 r and r.r of the aggregate's nodes
      for (int bz = az * k.cf; bz < min(az * k.cf + k.cf, k.nb2); ++bz)
        for (int by = ay * k.cf; by < min(ay * k.cf + k.cf, k.nb1); ++by) {
          // the aggregate's bins along x are one contiguous node range
          const int b0 = bx0 + k.nb0 * (by + k.nb1 * bz);
          const int i0 = k.bin_start[b0], i1 = k.bin_start[b0 + (bx1 - bx0)];
          // two nodes per lane per round (their loads in flight together), summed in order
          for (int i = i0 + lane; i < i1; i += 64) {
            const bool two = i + 32 < i1;
            P r0 = rin[i], r1 = two ? rin[i + 32] : P(0);
            const P d0 = dinv[i], d1 = two ? dinv[i + 32] : P(0);
            const P p0 = p[i], p1 = two ? p[i + 32] : P(0);
            const P q0 = q[i], q1 = two ? q[i + 32] : P(0);
            const P e0 = e[i], e1 = two ? e[i + 32] : P(0);
            if (d0 != P(0)) {
              e[i] = e0 + alpha * p0;
              r0 = r0 - alpha * q0;
              rin[i] = r0;
              rzf.add(r0, r0 * d0);
              rr.add(r0, r0);
            }
            acc += (float)r0;
            if (d1 != P(0)) {
              e[i + 32] = e1 + alpha * p1;
              r1 = r1 - alpha * q1;
              rin[i + 32] = r1;
              rzf.add(r1, r1 * d1);
              rr.add(r1, r1);
            }
            acc += (float)r1;
          }
        }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
      rzf.warp_sum();
      rr.warp_sum();
      if (lane == 0) {
        k.rc[I] = acc;
        k.cdots[I] = rzf.value();
        k.cdots[k.cn + I] = rr.value();
      }
    }
  }
}

// warp per row of an instance's inverse: x_c = A_c^-1 r_c (r_c in shared memory, 16-byte
// row loads, four accumulators combined in a fixed order).  With dots (the CG update of the
// split iteration), also r_c[I] x_c[I] = (P^T r).(x_c) per row, and the last CTA forms
// r.z = r.D^-1 r + r_c.x_c and r.r from the per-aggregate parts and makes the CG decisions.
// 16-byte loads per lane in flight (8 x 32 x 4 = 1024 floats a round); with at most 80
// registers three CTAs fit an SM, so the 343 CTAs of the 512k workload run in one wave
constexpr int kGemvU = 8;
__global__ void __launch_bounds__(kBlock, 3) k_coarse_gemv(EngineView v, int which, cudaGraphConditionalHandle hc,
                                                        int dots, int def_mixed) {
  extern __shared__ __align__(16) float srv[];
  __shared__ double sm[3 * kBlock / 32];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  for (int inst = 0; inst < v.M; ++inst) {
    const KParams& k = v.inst[inst];
    if (!k.coarse || !coarse_active(k, which == 2 ? 0 : which)) continue;
    if (which == 2 && !deflating<float>(k)) continue;  // the deflated solve's final correction only
    const int n = k.cn, ld = k.cld;
    const bool dm = def_mixed && k.defl_ok && *((volatile const int*)&k.ds->defl) != 0;
    __syncthreads();
    {
      // r_c into shared memory: 16-byte loads, four per thread in flight (rc holds ld
      // floats, its padding zero)
      const float4* rc4 = reinterpret_cast<const float4*>(k.rc);
      float4* sv4 = reinterpret_cast<float4*>(srv);
      const int nq = ld >> 2;
      for (int i0 = threadIdx.x; i0 < nq; i0 += 4 * kBlock) {
        float4 t[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (i0 + u * kBlock < nq) t[u] = rc4[i0 + u * kBlock];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (i0 + u * kBlock < nq) sv4[i0 + u * kBlock] = t[u];
      }
    }
    __syncthreads();
    const float4* sr4 = reinterpret_cast<const float4*>(srv);
    const int nq = ld >> 2;  // 16-byte groups per row
    for (int I = gw; I < n; I += warps) {
      const float4* row = reinterpret_cast<const float4*>(k.cinv + (size_t)I * ld);
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      // rounds of kGemvU 16-byte loads per lane, all in flight before their products
      for (int j0 = lane; j0 < nq; j0 += 32 * kGemvU) {
        float4 a[kGemvU];
#pragma unroll
        for (int u = 0; u < kGemvU; ++u)
          if (j0 + 32 * u < nq) a[u] = __ldg(row + j0 + 32 * u);
#pragma unroll
        for (int u = 0; u < kGemvU; ++u)
          if (j0 + 32 * u < nq) {
            const float4 b = sr4[j0 + 32 * u];
            acc[0] = fmaf(a[u].x, b.x, acc[0]);
            acc[1] = fmaf(a[u].y, b.y, acc[1]);
            acc[2] = fmaf(a[u].z, b.z, acc[2]);
            acc[3] = fmaf(a[u].w, b.w, acc[3]);
          }
      }
      float x = (acc[0] + acc[1]) + (acc[2] + acc[3]);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
      if (lane == 0) {
        k.xc[I] = x;
        if (dots) {
          if (dm) {
            // deflated (FP32 path): r_c[I] x_c[I] as an exact FP32 pair
            const float pr = srv[I] * x;
            store_pair(k.cdots, 2 * (size_t)n + I, pr, fmaf(srv[I], x, -pr));
          } else {
            k.cdots[2 * n + I] = (double)srv[I] * (double)x;
          }
        }
      }
    }
  }
  if (!dots) return;
  if (take_last_ticket(&v.ticket[v.M + 1], &s_last)) {
    for (int i = 0; i < v.M; ++i) {
      const KParams& k = v.inst[i];
      double tot[3] = {0.0, 0.0, 0.0};
      // the deflated iteration needs only r_c.x_c (the update kernel forms the dots)
      const bool dm = def_mixed && k.coarse && k.defl_ok && *((volatile const int*)&k.ds->defl) != 0;
      if (dm) {
        double t2[1];
        reduce_pair_items<1>(k.cdots + 2 * (size_t)k.cn, k.cn, 0, k.cn, t2, sm);
        tot[2] = t2[0];
      } else if (k.coarse) {
        reduce_items<3>(k.cdots, k.cn, 0, k.cn, tot, sm);
      }
      if (threadIdx.x == 0) {
        DevState* ds = k.ds;
        if (dm) {
          // deflated step length: p.P_d A p = p.q - r_c.x_c (r_c = P^T q); the update kernel
          // makes the decisions and drives the loop
          if (ds->inner_active) {
            const double pw = ds->pq - tot[2];
            ds->alpha = (pw > 0.0 && isfinite(pw)) ? ds->rz / pw : 0.0;
          }
        } else {
          if (!k.coarse) {
            ds->inner_active = 0;  // not reached: split engines have a coarse space per member
          } else if (ds->inner_active) {
            const double rz = tot[0] + tot[2];
            const double alpha_d = ds->alpha;
            ds->beta = ds->rz != 0.0 ? rz / ds->rz : 0.0;
            ds->rz = rz;
            ds->rr = tot[1];
            ds->inner_it += 1;
            ds->solve_iters += 1;
            ds->cg_iters += 1;
            const bool go = alpha_d != 0.0 && isfinite(tot[1]) && tot[1] > ds->inner_target &&
                            ds->inner_it < ds->max_iter && ds->solve_iters < ds->max_iter;
            ds->inner_active = go ? 1 : 0;
          }
          instance_finished(v, i, 1, hc);
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) v.ticket[v.M + 1] = 0;
  }
}

// Additive form: z = D^-1 r + x_c[agg] on the unknowns (after the decisions of
// k_coarse_gemv).  Deflated form: w = q - A P x_c, e^ += alpha p, r^ -= alpha w, t += alpha q,
// z = D^-1 r^, with the dots and the CG decisions (last chunk of the instance).
template <typename P>
__global__ void __launch_bounds__(kBlock) k_z_form(EngineView v, cudaGraphConditionalHandle hc) {
  __shared__ double sm[2 * kBlock / 32];
  __shared__ int s_last;
  for (int item = blockIdx.x; item < v.nchunks; item += gridDim.x) {
    const Chunk c = v.chunks[item];
    const KParams& k = v.inst[c.inst];
    const bool active = coarse_active(k, 1);
    P* rin = VecSel<P>::rin(k);
    P* z = VecSel<P>::z(k);
    const P* dinv = VecSel<P>::dinv(k);
    if (!deflating<P>(k)) {
      if (!active) continue;
      for (int a = c.begin + threadIdx.x; a < c.end; a += kBlock) {
        const P di = dinv[a];
        z[a] = di == P(0) ? P(0) : rin[a] * di + (P)k.xc[k.agg[a]];
      }
      continue;
    }
    DotAcc<float> part[2];
    if constexpr (sizeof(P) == 4) {
      if (active) {
        const float* p = k.p32;
        const float* q = k.q32;
        float* e = k.e32;
        float* t = k.t32;
        const float alpha = (float)k.ds->alpha;
        for (int a = c.begin + threadIdx.x; a < c.end; a += kBlock) {
          const float di = dinv[a];
          if (di == 0.0f) continue;
          // every load before the first store (loads are not moved across the stores)
          const float qa = __ldg(q + a);
          const float pa = __ldg(p + a);
          const float ea = e[a];
          const float ra = rin[a];
          const float ta = t[a];
          const float w = qa - ap_apply(k, a);
          e[a] = ea + alpha * pa;
          const float r = ra - alpha * w;
          rin[a] = r;
          t[a] = ta + alpha * qa;
          const float zz = r * di;
          z[a] = zz;
          part[0].add(r, zz);
          part[1].add(r, r);
        }
      }
    }
    write_dot_partials<2, float>(v, item, part, sm);
    if (item_done(&v.ticket[c.inst], v.chunk_count[c.inst], &s_last)) {
      double tot[2];
      reduce_dot_items<2, float>(v.partials, v.stride, v.chunk_first[c.inst], v.chunk_count[c.inst], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = k.ds;
        if (ds->inner_active) {
          const double alpha_d = ds->alpha;
          ds->beta = ds->rz != 0.0 ? tot[0] / ds->rz : 0.0;
          ds->rz = tot[0];
          ds->rr = tot[1];
          ds->inner_it += 1;
          ds->solve_iters += 1;
          ds->cg_iters += 1;
          const bool go = alpha_d != 0.0 && isfinite(tot[1]) && tot[1] > ds->inner_target &&
                          ds->inner_it < ds->max_iter && ds->solve_iters < ds->max_iter;
          ds->inner_active = go ? 1 : 0;
        }
        instance_finished(v, c.inst, 1, hc);
      }
    }
    __syncthreads();
  }
}

// Deflated solve, after the inner loop: e = e^ + Q (r0 - t).  Step 1 writes r0 - t into r
// (restricted and solved next), step 2 adds P x_c.
__global__ void __launch_bounds__(kBlock) k_def_final(EngineView v, int step) {
  for (int item = blockIdx.x; item < v.nchunks; item += gridDim.x) {
    const Chunk c = v.chunks[item];
    const KParams& k = v.inst[c.inst];
    if (!deflating<float>(k) || !coarse_active(k, 0)) continue;
    for (int a = c.begin + threadIdx.x; a < c.end; a += kBlock) {
      const bool unk = k.dinv32[a] != 0.0f;
      if (step == 1)
        k.rin32[a] = unk ? k.r0_32[a] - k.t32[a] : 0.0f;
      else if (unk)
        k.e32[a] = k.e32[a] + k.xc[k.agg[a]];
    }
  }
}

template <typename P>
__global__ void __launch_bounds__(kBlock) k_cg_zdots(EngineView v, cudaGraphConditionalHandle hc, int init,
                                                     int fp64) {
  __shared__ double sm[3 * kBlock / 32];
  __shared__ int s_last;
  for (int item = blockIdx.x; item < v.nchunks; item += gridDim.x) {
    const Chunk c = v.chunks[item];
    const KParams& k = v.inst[c.inst];
    const bool active = coarse_active(k, init ? 0 : 1);
    DotAcc<P> part[3];
    if (active) {
      P* rin = VecSel<P>::rin(k);
      P* z = VecSel<P>::z(k);
      const P* dinv = VecSel<P>::dinv(k);
      // deflated start (mixed, operator fresh): r^ = r - A P x_c, z = D^-1 r^
      const bool def = init && deflating<P>(k);
      for (int a = c.begin + threadIdx.x; a < c.end; a += kBlock) {
        const P di = dinv[a];
        P r = rin[a];
        part[2].add(r, r);
        P zz;
        if (def) {
          if (di != P(0)) {
            r = r - (P)ap_apply(k, a);
            rin[a] = r;
          }
          zz = r * di;
        } else {
          zz = di == P(0) ? P(0) : (k.coarse ? r * di + (P)k.xc[k.agg[a]] : r * di);
        }
        z[a] = zz;
        part[0].add(r, zz);
        part[1].add(r, r);
      }
    }
    write_dot_partials<3, P>(v, item, part, sm);
    if (item_done(&v.ticket[c.inst], v.chunk_count[c.inst], &s_last)) {
      double tot[3];
      reduce_dot_items<3, P>(v.partials, v.stride, v.chunk_first[c.inst], v.chunk_count[c.inst], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = k.ds;
        if (init) {
          if (ds->outer_active) {
            ds->rz = tot[0];
            ds->rr = tot[1];
            ds->beta = 0.0;
            ds->alpha = 0.0;
            ds->inner_it = 0;
            // the reduction is relative to the correction equation's residual r (before
            // the deflation), the stop test on the (deflated) iterated residual
            const double target = fp64 ? 0.25 * ds->tol * ds->tol * ds->bnorm2
                                       : fmax(ds->inner_rel * ds->inner_rel * tot[2],
                                              0.09 * ds->tol * ds->tol * ds->bnorm2);
            ds->inner_target = target;
            ds->inner_active = (tot[1] > target && ds->max_iter > 0) ? 1 : 0;
          } else {
            ds->inner_active = 0;
          }
        } else if (ds->inner_active) {
          const double alpha_d = ds->alpha;
          ds->beta = ds->rz != 0.0 ? tot[0] / ds->rz : 0.0;
          ds->rz = tot[0];
          ds->rr = tot[1];
          ds->inner_it += 1;
          ds->solve_iters += 1;
          ds->cg_iters += 1;
          const bool go = alpha_d != 0.0 && isfinite(tot[1]) && tot[1] > ds->inner_target &&
                          ds->inner_it < ds->max_iter && ds->solve_iters < ds->max_iter;
          ds->inner_active = go ? 1 : 0;
        }
        instance_finished(v, c.inst, 1, hc);
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------- warm start ---------
// Initial guess of the potential solve from the last H solutions x_n, ..., x_{n-H+1} and
// their images A x (the ring xh, bh; bh = b - r at the end of each solve):
//   x0 = x_n + sum_l a_l D^l x_n,   D^l: l-th backward difference at the newest solution,
// with the coefficients minimising the A-norm error of x0 over that affine space
// (Galerkin condition  (D^i x)^T A (D^j x) a_j = (D^i x)^T (b_new - A x_n)); A D^l x is the
// same difference of bh.  The differences are the well-conditioned basis of the span of
// the history; the linear extrapolation 2 x_n - x_{n-1} is the member a = (1, 0, ...).
constexpr int kWarmD = kHistMax - 1;                         // differences
constexpr int kWarmSlots = kWarmD * (kWarmD + 1) / 2 + kWarmD + 1;  // G (upper), rhs, x.Ax
static_assert(kWarmSlots <= kReduceSlots, "warm-start partials exceed the reduction buffer");

__device__ __forceinline__ int warm_history(const KParams& k) {
  if (k.hist_m < 3 || !k.extrapolate) return 0;
  const int n = k.ds->hist_n;
  return n < k.hist_m ? n : k.hist_m;
}

// Solve the scaled Galerkin system by Cholesky; differences whose pivot falls below 1e-12
// (near-dependent) or whose A-norm is below 1e-12 of the solution's (rounding level) end
// the basis.  Thread 0 of one CTA.
__device__ void warm_solve(const double (&tot)[kWarmSlots], int nd, DevState* ds) {
  double G[kWarmD][kWarmD], r[kWarmD], d[kWarmD], L[kWarmD][kWarmD], y[kWarmD];
  int q = 0;
  for (int i = 0; i < kWarmD; ++i)
    for (int j = i; j < kWarmD; ++j) G[i][j] = G[j][i] = tot[q++];
  for (int i = 0; i < kWarmD; ++i) r[i] = tot[q++];
  const double xax = tot[q];
  int n = 0;
  for (int i = 0; i < nd; ++i) {
    if (!(G[i][i] > 1e-24 * xax) || !isfinite(G[i][i])) break;
    d[i] = sqrt(G[i][i]);
    n = i + 1;
  }
  int m = 0;
  for (int j = 0; j < n; ++j) {
    double sj = 1.0;
    for (int k2 = 0; k2 < j; ++k2) sj -= L[j][k2] * L[j][k2];
    if (!(sj > 1e-12)) break;
    L[j][j] = sqrt(sj);
    for (int i = j + 1; i < n; ++i) {
      double si = G[i][j] / (d[i] * d[j]);
      for (int k2 = 0; k2 < j; ++k2) si -= L[i][k2] * L[j][k2];
      L[i][j] = si / L[j][j];
    }
    m = j + 1;
  }
  for (int i = 0; i < m; ++i) {
    double si = r[i] / d[i];
    for (int k2 = 0; k2 < i; ++k2) si -= L[i][k2] * y[k2];
    y[i] = si / L[i][i];
  }
  bool ok = m > 0;
  for (int i = m - 1; i >= 0; --i) {
    double si = y[i];
    for (int k2 = i + 1; k2 < m; ++k2) si -= L[k2][i] * y[k2];
    y[i] = si / L[i][i];
    ok = ok && isfinite(y[i]);
  }
  for (int i = 0; i < kWarmD; ++i) ds->warm_coef[i] = (ok && i < m) ? y[i] / d[i] : 0.0;
  ds->warm_nd = ok ? m : 0;
}

// backward differences D^1..D^{H-1} of the FP32 pairs t[0..H-1] (newest first) into d;
// t is consumed
__device__ __forceinline__ void pair_warm_diffs(float (&th)[kHistMax], float (&tl)[kHistMax], int H,
                                                float (&dh)[kWarmD], float (&dl)[kWarmD]) {
#pragma unroll
  for (int l = 1; l < kHistMax; ++l) {
#pragma unroll
    for (int j = 0; j + 1 < kHistMax; ++j)
      if (j + l < H) pair_sub(th[j], tl[j], th[j + 1], tl[j + 1], th[j], tl[j]);
    dh[l - 1] = l < H ? th[0] : 0.0f;
    dl[l - 1] = l < H ? tl[0] : 0.0f;
  }
}

// the history of node a as FP32 pairs, newest first (zero beyond H)
__device__ __forceinline__ void load_history_pairs(const double* ring, const int (&slot)[kHistMax], int H,
                                                   size_t N, int a, float (&th)[kHistMax], float (&tl)[kHistMax]) {
#pragma unroll
  for (int j = 0; j < kHistMax; ++j) {
    th[j] = tl[j] = 0.0f;
    if (j < H) split_pair(ring[(size_t)slot[j] * N + a], th[j], tl[j]);
  }
}

// The Galerkin system's dot products, on FP32 pairs (the FP64 rate of the GB300 would
// bound this pass): the history is split into pairs, differenced and multiplied with the
// pair operations, ~2^-46 relative per operation.
template <typename P>
__global__ void __launch_bounds__(kBlock) k_warm_dots(EngineView v) {
  __shared__ double sm[kWarmSlots * kBlock / 32];
  __shared__ int s_last;
  for (int item = blockIdx.x; item < v.nchunks; item += gridDim.x) {
    const Chunk c = v.chunks[item];
    const KParams& k = v.inst[c.inst];
    const int H = warm_history(k);
    DotAcc<float> part[kWarmSlots];
    if (H >= 3) {
      const int head = k.ds->hist_head, m = k.hist_m;
      const size_t N = (size_t)k.N;
      int slot[kHistMax];
#pragma unroll
      for (int j = 0; j < kHistMax; ++j) slot[j] = (head - j + 2 * m) % m;
      float lamh, laml, zh[S], zl[S];
      split_pair(k.lam, lamh, laml);
#pragma unroll
      for (int s2 = 0; s2 < S; ++s2) split_pair(k.z[s2], zh[s2], zl[s2]);
      for (int a = c.begin + threadIdx.x; a < c.end; a += kBlock) {
        if (!k.freem[a]) continue;
        float xh[kHistMax], xl[kHistMax], bh[kHistMax], bl[kHistMax];
        load_history_pairs(k.xh, slot, H, N, a, xh, xl);
        load_history_pairs(k.bh, slot, H, N, a, bh, bl);
        float bnh, bnl;
        if (k.b_override) {
          split_pair(k.b_override[a], bnh, bnl);  // adjoint solves: the given right-hand side
        } else {
          // b = lam sum_s z_s c_s
          float rh = 0.0f, rl = 0.0f;
#pragma unroll
          for (int s2 = 0; s2 < S; ++s2) {
            float ch, cl, ph, pl;
            if constexpr (sizeof(P) == 4) {
              const float4 lo4 = k.clo[a];
              ch = k.rec32_cur[a].c[s2];
              cl = sel4(lo4, s2);
            } else {
              split_pair(k.rec64_cur[a].c[s2], ch, cl);
            }
            pair_mul(zh[s2], zl[s2], ch, cl, ph, pl);
            pair_add(rh, rl, ph, pl);
          }
          pair_mul(lamh, laml, rh, rl, bnh, bnl);
        }
        float gh, gl;
        pair_sub(bnh, bnl, bh[0], bl[0], gh, gl);
        const float x0h = xh[0], x0l = xl[0], b0h = bh[0], b0l = bl[0];
        float dxh[kWarmD], dxl[kWarmD], dbh[kWarmD], dbl[kWarmD];
        pair_warm_diffs(xh, xl, H, dxh, dxl);
        pair_warm_diffs(bh, bl, H, dbh, dbl);
        int q = 0;
#pragma unroll
        for (int i = 0; i < kWarmD; ++i)
#pragma unroll
          for (int j = i; j < kWarmD; ++j) part[q++].add_pair(dxh[i], dxl[i], dbh[j], dbl[j]);
#pragma unroll
        for (int i = 0; i < kWarmD; ++i) part[q++].add_pair(dxh[i], dxl[i], gh, gl);
        part[q].add_pair(x0h, x0l, b0h, b0l);
      }
    }
    write_dot_partials<kWarmSlots, float>(v, item, part, sm);
    if (item_done(&v.ticket[c.inst], v.chunk_count[c.inst], &s_last)) {
      double tot[kWarmSlots];
      reduce_dot_items<kWarmSlots, float>(v.partials, v.stride, v.chunk_first[c.inst], v.chunk_count[c.inst], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = k.ds;
        ds->warm_nd = 0;
        if (H >= 3) warm_solve(tot, H - 1, ds);
        v.ticket[c.inst] = 0;
      }
    }
    __syncthreads();
  }
}

// the solution of a solve run outside a step (adjoint) and A x = b - r into ring slot `slot`
__global__ void k_record_solve(KParams k, int slot) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x) {
    const size_t o = (size_t)slot * k.N + a;
    k.xh[o] = k.phi64[a];
    k.bh[o] = k.freem[a] ? k.b64[a] - k.r64[a] : 0.0;
  }
}

// x0 = x_n + sum_l a_l D^l x_n on the unknowns, into phi64 and the state's potential
// (FP32-pair arithmetic as k_warm_dots; x0 is exact in FP64 as the sum of its pair)
template <typename P>
__global__ void __launch_bounds__(kBlock) k_warm_apply(EngineView v) {
  for (int item = blockIdx.x; item < v.nchunks; item += gridDim.x) {
    const Chunk c = v.chunks[item];
    const KParams& k = v.inst[c.inst];
    const int H = warm_history(k);
    if (H < 3) continue;
    const int nd = k.ds->warm_nd;
    if (nd <= 0) continue;
    float ch[kWarmD], cl[kWarmD];
#pragma unroll
    for (int i = 0; i < kWarmD; ++i) split_pair(k.ds->warm_coef[i], ch[i], cl[i]);
    const int head = k.ds->hist_head, m = k.hist_m;
    const size_t N = (size_t)k.N;
    int slot[kHistMax];
#pragma unroll
    for (int j = 0; j < kHistMax; ++j) slot[j] = (head - j + 2 * m) % m;
    for (int a = c.begin + threadIdx.x; a < c.end; a += kBlock) {
      if (!k.freem[a]) continue;
      float th[kHistMax], tl[kHistMax];
      load_history_pairs(k.xh, slot, H, N, a, th, tl);
      const float xh0 = th[0], xl0 = tl[0];
      float dh[kWarmD], dl[kWarmD];
      pair_warm_diffs(th, tl, H, dh, dl);
      float sh = 0.0f, sl = 0.0f;
#pragma unroll
      for (int i = 0; i < kWarmD; ++i) {
        float ph, pl;
        pair_mul(ch[i], cl[i], dh[i], dl[i], ph, pl);
        pair_add(sh, sl, ph, pl);
      }
      pair_add(sh, sl, xh0, xl0);
      // normalised pair: hi the FP32 rounding of the sum, lo its exact remainder
      const float hi = sh + sl;
      const float lo = sl - (hi - sh);
      k.phi64[a] = (double)hi + (double)lo;
      if constexpr (sizeof(P) == 4) {
        k.rec32_cur[a].phi_hi = hi;
        k.rec32_cur[a].phi_lo = lo;
      } else {
        k.rec64_cur[a].phi = (double)hi + (double)lo;
      }
    }
  }
}

// phi += e on the unknowns; FP64 residual r -= A e (FP64 weights); outer stop test.
template <typename P, int W>
__global__ void __launch_bounds__(kBlock) k_ir_update(EngineView v, cudaGraphConditionalHandle hc) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ TileSmem ts;
  __shared__ double sm[kBlock / 32];
  __shared__ int s_last;
  const int sub = threadIdx.x % W, seg = threadIdx.x / W, nseg = kBlock / W;
  const bool mixed = sizeof(P) == 4;
  for (int item = blockIdx.x; item < v.ntiles; item += gridDim.x) {
    const TileDesc t = v.tiles[item];
    const KParams& k = v.inst[t.inst];
    const bool active = *((volatile int*)&k.ds->outer_active) != 0;
    double part[1] = {0.0};
    if (active) {
      load_tile(t, ts);
      double* hs = reinterpret_cast<double*>(dsm);
      const unsigned short* sslot = stage_slots(k.slot16, t, dsm + align16(sizeof(double) * (size_t)t.halo));
      const P* e = VecSel<P>::e(k);
      for (int s = threadIdx.x; s < t.halo; s += kBlock) hs[s] = (double)e[halo_node(ts, s)];
      __syncthreads();
      const int* row = k.row;
      const double* w64 = k.w64;
      const unsigned char* freem = k.freem;
      const int own0 = ts.off[4] + (t.own_begin - t.hb[4]);
      for (int a0 = t.own_begin; a0 < t.own_end; a0 += nseg) {
        const int a = a0 + seg;
        const bool act = a < t.own_end && freem[a];
        double acc = 0.0;
        if (mixed) {
          // A e with the FP32 pair (w32, wlo32) and the FP32 correction e: exact products
          // (TwoProd), TwoSum accumulation
          float sh = 0.f, sl = 0.f;
          if (act)
            for (int j = row[a] + sub; j < row[a + 1]; j += W) {
              const float ev = (float)hs[sslot[j - t.bond0]];
              float ph, pl;
              pair_mul(k.w32[j], k.wlo32[j], ev, 0.0f, ph, pl);
              pair_add(sh, sl, ph, pl);
            }
          acc = seg_reduce_pair<W>(sh, sl);
        } else {
          if (act)
            for (int j = row[a] + sub; j < row[a + 1]; j += W) acc = fma(w64[j], hs[sslot[j - t.bond0]], acc);
          acc = seg_reduce_d<W>(acc);
        }
        if (act && sub == 0) {
          const double ea = hs[own0 + (a - t.own_begin)];
          const double r = k.r64[a] - (k.dsum64[a] * ea - acc);
          k.r64[a] = r;
          const double ph = k.phi64[a] + ea;
          k.phi64[a] = ph;
          set_phi_rec(k, a, ph, mixed);
          part[0] += r * r;
        }
      }
    }
    write_partials<1>(v, item, part, sm);
    if (item_done(&v.ticket[t.inst], v.tile_count[t.inst], &s_last)) {
      double tot[1];
      reduce_items<1>(v.partials, v.stride, v.tile_first[t.inst], v.tile_count[t.inst], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = k.ds;
        if (ds->outer_active) {
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
          ds->outer_active = go ? 1 : 0;
        }
        instance_finished(v, t.inst, 0, hc);
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------- potential residuals on the slices ----
// Mixed path: the prep and the refinement residual as slice kernels over the sliced operator
// (one lane per row, bond columns streamed in batches of 8, neighbour values gathered through
// L1/L2), with the FP64 weight carried as the FP32 pair (sell, sell_lo) and FP32-pair
// arithmetic (TwoProd, TwoSum) along each row.  Slice partials, one global ticket; the last
// CTA makes every instance's decisions.
constexpr int kResB = 8;

__device__ __forceinline__ const float* sell_lo_col(const KParams& k, const SliceDesc& d) {
  return k.sell_lo + (size_t)(d.off >> 5) * 32;
}

// per node {phi_hi, phi_lo} (zero on solid nodes), liquid flag, potential-Dirichlet flag
__global__ void __launch_bounds__(kBlock) k_phi4(EngineView v) {
  // a prep that forms the mask sums rewrites the CG operator's rows: their slices' longest
  // rows start from zero
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < v.ncslices; g += gridDim.x * blockDim.x) {
    const int inst = v.cslices[g].inst;
    const KParams& k = v.inst[inst];
    if (k.ds->op_valid == 0) k.cg_width[g - v.cslice_first[inst]] = 0;
  }
  for (int item = blockIdx.x; item < v.nchunks; item += gridDim.x) {
    const Chunk c = v.chunks[item];
    const KParams& k = v.inst[c.inst];
    for (int a = c.begin + threadIdx.x; a < c.end; a += kBlock) {
      const bool liq = k.rec32_cur[a].phase == 0.0f;
      const double ph = k.phi64[a];
      const float hi = (float)ph;
      const float lo = (float)(ph - (double)hi);
      k.phi4[a] = make_float4(liq ? hi : 0.0f, liq ? lo : 0.0f, liq ? 1.0f : 0.0f,
                              ((k.dirmask[a] >> S) & 1) ? 1.0f : 0.0f);
    }
  }
}

// prep: b, the FP64 residual r = b - A phi and the norms; the mask-only sums (diagonal,
// Dirichlet coupling, unknown flag) are formed only when the phases changed (op_valid == 0)
__global__ void __launch_bounds__(kBlock) k_prep_slices(EngineView v, cudaGraphConditionalHandle hc) {
  __shared__ int s_hb[kBlock / 32][12];
  __shared__ double sm[2 * kBlock / 32];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // warps claim slices one at a time (slices of solid nodes, narrow and partial slices
  // cost less than full ones)
  for (int sg = claim_slice(v, lane); sg < v.nslices; sg = claim_slice(v, lane)) {
    const SliceDesc& d = v.slices[sg];
    const KParams& k = v.inst[d.inst];
    const bool cached = k.ds->op_valid != 0;
    if (lane < 9) s_hb[warp][lane] = d.gbase[lane];
    __syncwarp();
    const int a = d.row0 + lane;
    const bool rowok = lane < d.nrows;
    float4 fa = make_float4(0.f, 0.f, 0.f, 0.f);
    int len = 0;
    if (rowok) {
      fa = k.phi4[a];
      len = k.row[a + 1] - k.row[a];
    }
    const bool scan = rowok && fa.z != 0.0f && fa.w == 0.0f;
    const int* hb = s_hb[warp];
    const float* ws = sell_w(k, d) + lane;
    const float* wls = sell_lo_col(k, d) + lane;
    const unsigned short* cs = sell_code(k, d) + lane;
    // sum_j w phi_j over the liquid columns as an FP32 pair in bond order (the cached pass
    // adds the solid columns' exact zeros, so both passes give the same bits).  The mask
    // sums also write the row into the CG operator's slices: its bonds to possible unknowns
    // (liquid, no potential Dirichlet value), codes relative to that slice's windows, zero
    // padding, and the slice's longest row.
    const int cpos = scan && !cached ? k.cg_pos[a] : -1;
    const SliceDesc* cd = nullptr;
    float* wcg = nullptr;
    float* wlcg = nullptr;
    unsigned short* ccg = nullptr;
    int cby = 0, cbz = 0;
    if (cpos >= 0) {
      cd = v.cslices + v.cslice_first[d.inst] + (cpos >> 5);
      const size_t col0 = (size_t)(cd->off >> 5);
      wcg = k.sell_cg + col0 * kSellW + (cpos & 31);
      wlcg = k.sell_cg_lo + col0 * 32 + (cpos & 31);
      ccg = reinterpret_cast<unsigned short*>(k.sell_cg + col0 * kSellW + 32) + (cpos & 31);
      cby = cd->tile & 0xffff;
      cbz = cd->tile >> 16;
    }
    int ncg = 0;
    float dh = 0.f, dl = 0.f, sh = 0.f, sl = 0.f, ch = 0.f, cl = 0.f;
    int anyll = 0;
    if (__any_sync(0xffffffffu, scan)) {
      const int width = d.width;
      for (int c0 = 0; c0 < width; c0 += kResB) {
        const int nc = min(kResB, width - c0);
        float w[kResB], wl[kResB];
        unsigned int code[kResB];
#pragma unroll
        for (int u = 0; u < kResB; ++u)
          if (u < nc) {
            w[u] = ld_stream(ws + kSellW * (c0 + u));
            wl[u] = ld_stream(wls + 32 * (c0 + u));
            code[u] = ld_stream(cs + kSellC * (c0 + u));
          }
        if (cached) {
          float2 f[kResB];
#pragma unroll
          for (int u = 0; u < kResB; ++u)
            if (u < nc) f[u] = __ldg(reinterpret_cast<const float2*>(k.phi4 + code_node(hb, code[u])));
#pragma unroll
          for (int u = 0; u < kResB; ++u)
            if (u < nc) {
              float ph, pl;
              pair_mul(w[u], wl[u], f[u].x, f[u].y, ph, pl);
              pair_add(sh, sl, ph, pl);
            }
          continue;
        }
        float4 f[kResB];
#pragma unroll
        for (int u = 0; u < kResB; ++u)
          if (u < nc) f[u] = __ldg(k.phi4 + code_node(hb, code[u]));
#pragma unroll
        for (int u = 0; u < kResB; ++u)
          if (u < nc && c0 + u < len && f[u].z != 0.0f) {
            float ph, pl;
            pair_mul(w[u], wl[u], f[u].x, f[u].y, ph, pl);
            pair_add(sh, sl, ph, pl);
            pair_add(dh, dl, w[u], wl[u]);
            anyll = 1;
            if (f[u].w != 0.0f) {
              pair_add(ch, cl, ph, pl);
            } else if (cpos >= 0) {
              const int m = code_node(hb, code[u]);
              const int xr = k.xrow[m];
              const int r = ((xr & 0xffff) - cby + 1) + 3 * ((xr >> 16) - cbz + 1);
              wcg[(size_t)kSellW * ncg] = w[u];
              wlcg[(size_t)32 * ncg] = wl[u];
              ccg[(size_t)kSellC * ncg] = (unsigned short)((r << 12) | (m - cd->gbase[r]));
              ++ncg;
            }
          }
      }
    }
    if (cpos >= 0) {
      // zero padding up to the slice's capacity (its longest full row)
      for (int c = ncg; c < cd->width; ++c) {
        wcg[(size_t)kSellW * c] = 0.0f;
        wlcg[(size_t)32 * c] = 0.0f;
        ccg[(size_t)kSellC * c] = 0;
      }
      atomicMax(&k.cg_width[cpos >> 5], ncg);
    }
    float b2h = 0.0f, b2l = 0.0f, r2h = 0.0f, r2l = 0.0f;  // b.b and r.r as FP32 pairs
    if (rowok) {
      double b;
      if (k.b_override) {
        b = k.b_override[a];
      } else {
        double R11 = 0.0;
        for (int s = 0; s < S; ++s) R11 += k.z[s] * conc_of<float>(k, a, s);
        b = k.lam * R11;
      }
      const double pha = (double)fa.x + (double)fa.y;
      const double swphi = scan ? (double)sh + (double)sl : 0.0;
      bool fr;
      double dsum, cpl;
      if (cached) {
        fr = k.freem[a] != 0;
        dsum = k.dsum64[a];
        cpl = k.cpl64[a];
      } else {
        dsum = scan ? (double)dh + (double)dl : 0.0;
        cpl = scan ? (double)ch + (double)cl : 0.0;
        fr = scan && anyll;
        k.freem[a] = fr ? 1 : 0;
        k.dsum64[a] = fr ? dsum : 1.0;
        k.cpl64[a] = fr ? cpl : 0.0;
        k.dinv64[a] = fr ? 1.0 / dsum : 0.0;
        k.d32[a] = fr ? (float)dsum : 1.0f;
        k.dinv32[a] = fr ? (float)(1.0 / dsum) : 0.0f;
      }
      const double bb = fr ? b : 0.0;
      const double r = fr ? bb - (dsum * pha - swphi) : 0.0;
      k.b64[a] = bb;
      k.r64[a] = r;
      const double be = bb + (fr ? cpl : 0.0);
      pair_square(be, b2h, b2l);
      pair_square(r, r2h, r2l);
    }
    pair_warp_sum(b2h, b2l);
    pair_warp_sum(r2h, r2l);
    if (lane == 0) {
      store_pair(v.partials, sg, b2h, b2l);
      store_pair(v.partials, (size_t)v.stride + sg, r2h, r2l);
    }
    __syncwarp();
  }
  if (take_last_ticket(&v.ticket[v.M + 1], &s_last)) {
    for (int i = 0; i < v.M; ++i) {
      double tot[2];
      reduce_pair_items<2>(v.partials, v.stride, v.slice_first[i], v.slice_count[i], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = v.inst[i].ds;
        ds->op_valid = 1;
        const double bn = tot[0] > 0.0 ? tot[0] : 1.0;
        ds->bnorm2 = bn;
        ds->rnorm2 = tot[1];
        ds->outer_it = 0;
        ds->solve_iters = 0;
        const bool go = tot[1] > ds->tol * ds->tol * bn && ds->max_outer > 0;
        if (!go) {
          ds->cg_solves += 1;
          ds->last_relres = sqrt(tot[1] / bn);
        }
        ds->outer_active = go ? 1 : 0;
        ds->inner_active = 0;
        instance_finished(v, i, 0, hc);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      v.ticket[v.M + 1] = 0;
      v.ticket[v.M + 2] = 0;
    }
  }
}

// refinement: phi += e on the unknowns, r -= A e (FP32 pairs of the FP64 weights times the
// FP32 correction), outer stop test
__global__ void __launch_bounds__(kBlock) k_ir_slices(EngineView v, cudaGraphConditionalHandle hc) {
  __shared__ int s_hb[kBlock / 32][12];
  __shared__ double sm[kBlock / 32];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // warps claim slices one at a time (slices of solid nodes, narrow and partial slices
  // cost less than full ones)
  for (int sg = claim_slice(v, lane); sg < v.ncslices; sg = claim_slice(v, lane)) {
    const SliceDesc& d = v.cslices[sg];
    const int inst = __ldg(&d.inst);
    const KParams& k = v.inst[inst];
    float rh = 0.0f, rl = 0.0f;  // r.r of the slice as an FP32 pair
    if (*((volatile int*)&k.ds->outer_active) != 0) {
      if (lane < 9) s_hb[warp][lane] = d.gbase[lane];
      __syncwarp();
      // the CG operator's slices: the correction e is zero off the unknowns
      const int a = k.cg_rows[__ldg(&d.row0) + lane];
      const bool live = a >= 0 && k.freem[a];
      const int len = __any_sync(0xffffffffu, live) ? k.cg_width[sg - __ldg(&v.cslice_first[inst])] : 0;
      const int* hb = s_hb[warp];
      const float* ws = sell_cg_w(k, d) + lane;
      const float* wls = k.sell_cg_lo + (size_t)(__ldg(&d.off) >> 5) * 32 + lane;
      const unsigned short* cs = sell_cg_code(k, d) + lane;
      const float* e = k.e32;
      float sh = 0.f, sl = 0.f;
      for (int c0 = 0; c0 < len; c0 += kResB) {
        const int nc = min(kResB, len - c0);
        float w[kResB], wl[kResB], ev[kResB];
        unsigned int code[kResB];
#pragma unroll
        for (int u = 0; u < kResB; ++u)
          if (u < nc) {
            w[u] = ld_stream(ws + kSellW * (c0 + u));
            wl[u] = ld_stream(wls + 32 * (c0 + u));
            code[u] = ld_stream(cs + kSellC * (c0 + u));
          }
#pragma unroll
        for (int u = 0; u < kResB; ++u)
          if (u < nc) ev[u] = __ldg(e + code_node(hb, code[u]));
#pragma unroll
        for (int u = 0; u < kResB; ++u)
          if (u < nc) {
            float ph, pl;
            pair_mul(w[u], wl[u], ev[u], 0.0f, ph, pl);
            pair_add(sh, sl, ph, pl);
          }
      }
      if (live) {
        const double ea = (double)e[a];
        const double r = k.r64[a] - (k.dsum64[a] * ea - ((double)sh + (double)sl));
        k.r64[a] = r;
        const double ph = k.phi64[a] + ea;
        k.phi64[a] = ph;
        set_phi_rec(k, a, ph, true);
        pair_square(r, rh, rl);
      }
      __syncwarp();
    }
    pair_warp_sum(rh, rl);
    if (lane == 0) store_pair(v.partials, sg, rh, rl);
  }
  if (take_last_ticket(&v.ticket[v.M + 1], &s_last)) {
    for (int i = 0; i < v.M; ++i) {
      double tot[1];
      reduce_pair_items<1>(v.partials, v.stride, v.cslice_first[i], v.cslice_count[i], tot, sm);
      if (threadIdx.x == 0) {
        DevState* ds = v.inst[i].ds;
        if (ds->outer_active) {
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
          ds->outer_active = go ? 1 : 0;
        }
        instance_finished(v, i, 0, hc);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      v.ticket[v.M + 1] = 0;
      v.ticket[v.M + 2] = 0;
    }
  }
}

// ------------------------------------------------------------------- transport -----------
__device__ __forceinline__ double dissolve_switch(double c0, double csat, double sw) {
  if (sw > 0.0) return 1.0 / (1.0 + exp(-(c0 - csat) / sw));
  return c0 > csat ? 1.0 : 0.0;
}

constexpr int kDiagSlots = 9;  // mass[4], solid, vol, dissolved, nonfinite, spare

// Per-step diagnostics of one instance from its reduced transport partials (thread 0).
__device__ __forceinline__ void finish_instance(const KParams& k, const double (&tot)[kDiagSlots]) {
  DevState* ds = k.ds;
  for (int s = 0; s < S; ++s) ds->mass[s] = tot[s];
  ds->solid_count = (long long)tot[4];
  ds->steps += 1;
  if (k.dissolve_count) ds->dissolved += tot[6];
  if (tot[7] != 0.0) ds->nonfinite = 1;
  ds->mg_mass_now = tot[0];
  if (k.hist_m >= 3) {
    ds->hist_head = (ds->hist_head + 1) % k.hist_m;
    ds->hist_n = ds->hist_n < k.hist_m ? ds->hist_n + 1 : k.hist_m;
  }
  if (k.sub_step_no > 0 && ds->steps % k.sub_step_no == 0) {
    ds->voln1rel = ds->vol0rel != 0.0 ? tot[5] / ds->vol0rel : 0.0;
    ds->BV = pow(10., -k.vol_red * (1. - ds->voln1rel));  // utils.h:100-116
  }
}

__device__ __forceinline__ void transport_finish(const EngineView& v, const TileDesc& t,
                                                 const KParams& k, int item,
                                                 double (&part)[kDiagSlots], double* sm,
                                                 int* s_last) {
  write_partials<kDiagSlots>(v, item, part, sm);
  if (!item_done(&v.ticket[t.inst], v.tile_count[t.inst], s_last)) return;
  double tot[kDiagSlots];
  reduce_items<kDiagSlots>(v.partials, v.stride, v.tile_first[t.inst], v.tile_count[t.inst], tot, sm);
  if (threadIdx.x == 0) {
    v.ticket[t.inst] = 0;
    finish_instance(k, tot);
  }
}

// The solution of this step's solve and its image A x = b - r into the warm-start ring.
__device__ __forceinline__ void record_history(const KParams& k, int a, int hslot) {
  if (k.hist_m < 3) return;
  const size_t o = (size_t)hslot * k.N + a;
  k.xh[o] = k.phi64[a];
  k.bh[o] = k.freem[a] ? k.b64[a] - k.r64[a] : 0.0;
}

// Warm start of the next solve: phi = 2 phi^n - phi^{n-1} on the unknowns (phi_prev keeps
// phi^n); the returned value also goes into the next record so that both agree.  A node the
// previous transport turned liquid (its phi^{n-1} is the solid's) is not extrapolated.
__device__ __forceinline__ double next_phi_guess(const KParams& k, int a) {
  const double ph = k.phi64[a];
  if (k.phi_keep) k.phi_keep[a] = ph;  // the step's solved potential (forward_ckpt)
  if (!k.extrapolate || !k.freem[a] || k.flip_step[a] == (int)k.ds->steps) {
    k.phi_prev[a] = ph;
    return ph;
  }
  const double g = 2.0 * ph - k.phi_prev[a];
  k.phi_prev[a] = ph;
  k.phi64[a] = g;
  return g;
}

// A neighbour's whole 32-byte record (c[4] | phi_hi, phi_lo, phase, pad) in one 256-bit
// read-only load (records are 32-byte aligned): half the gather instructions and L1 requests
// of two 16-byte loads of the same sector.
__device__ __forceinline__ void ld_rec32(const float4* p, float4& c, float4& t) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(c.x), "=f"(c.y), "=f"(c.z), "=f"(c.w), "=f"(t.x), "=f"(t.y), "=f"(t.z), "=f"(t.w)
      : "l"(p));
}

// Mixed transport of one 32-row slice sg.  RESID: write F_k = sum_KRk1 + sum_KRk2 - R_k
// (utils.h:177) to F_out (single instance) and change nothing; otherwise advance the state
// into rec32_nxt / clo and store the slice's diagnostics partials.  One lane per node streams
// the row's bond columns (codes and weights, column-major: one coalesced load per column) and
// gathers each neighbour's 32-byte record through rec(i), where i = hb[code >> 12] +
// (code & 4095) and hb[r] = gbase[r] - radj[r] (radj == nullptr: i is the node).  hb is the
// warp's 9-int table in shared memory.
// bond columns per batch of the FP32 transport: with 256-bit record loads 7 (128 registers,
// 2 CTAs an SM) measured 0.358 ms at 512k against 0.366 for 6 (8 spills); with two 16-byte
// loads a record 6 took 0.378 ms, 5 0.389, 4 0.405, 2 0.467
constexpr int kTrB = 7;
template <bool RESID, int B, bool EARLY, bool PIPE, typename Rec>
__device__ __forceinline__ void transport_slice(const EngineView& v, int sg, int lane, int* hbw,
                                                const int* radj, Rec rec, double* F_out) {
  const SliceDesc& d = v.slices[sg];
  const KParams& k = v.inst[__ldg(&d.inst)];
  if (lane < 9) hbw[lane] = __ldg(&d.gbase[lane]) - (radj ? radj[lane] : 0);
  __syncwarp();
  float ph_hi[6], ph_lo[6];  // masses[4], solid volume sum, dissolved (FP32 pairs)
#pragma unroll
  for (int q = 0; q < 6; ++q) ph_hi[q] = ph_lo[q] = 0.0f;
  int n_solid = 0, n_bad = 0;
  const int a = __ldg(&d.row0) + lane;
  if (lane < __ldg(&d.nrows)) {
    const float4* rc = reinterpret_cast<const float4*>(k.rec32_cur);
    const double BV = *k.bv_ptr;
    float cLL[S], cX[S], cSS[S], K1f[S], K2f[S];
#pragma unroll
    for (int s = 0; s < S; ++s) {
      cLL[s] = (float)k.DL[s];
      cX[s] = (float)(s == 0 ? k.DSo[0] * BV : k.DSo[s]);
      cSS[s] = s == 0 ? (float)k.DSo[0] : 0.0f;
      K1f[s] = (float)k.K1[s];
      K2f[s] = (float)k.K2zF[s];
    }
    const float4 ca = rc[2 * a];
    const float4 cb = rc[2 * a + 1];  // phi_hi, phi_lo, phase, pad
    const float pa = cb.z;
    // bond coefficient by the neighbour's phase (utils.h:100-153): liquid-liquid D_liquid,
    // mixed D_solid (BV for Mg), solid-solid D_solid for Mg only
    float cfL[S], cfS[S];
#pragma unroll
    for (int s = 0; s < S; ++s) {
      cfL[s] = pa == 0.0f ? cLL[s] : cX[s];
      cfS[s] = pa == 0.0f ? cX[s] : cSS[s];
    }
    float a1[S], a2[S];
#pragma unroll
    for (int s = 0; s < S; ++s) a1[s] = a2[s] = 0.0f;
    int iface = 0;
    const float* ws = sell_w(k, d) + lane;
    const unsigned short* cs = sell_code(k, d) + lane;
    const int len = k.row[a + 1] - k.row[a];
    // bonds in batches of B columns: the batch's streamed codes and weights, then its
    // neighbour records, all in flight before the arithmetic (column order is kept, so the
    // sums do not depend on the batch size)
    // PIPE: the next batch's codes and weights are loaded before the current batch's terms
    float wn[PIPE ? B : 1];
    unsigned int coden[PIPE ? B : 1];
    if (PIPE)
#pragma unroll
      for (int u = 0; u < B; ++u)
        if (u < len) {
          wn[PIPE ? u : 0] = ld_stream(ws + kSellW * u);
          coden[PIPE ? u : 0] = ld_stream(cs + kSellC * u);
        }
    for (int c0 = 0; c0 < len; c0 += B) {
      float w[B];
      unsigned int code[B];
#pragma unroll
      for (int u = 0; u < B; ++u)
        if (PIPE) {
          w[u] = wn[PIPE ? u : 0];
          code[u] = coden[PIPE ? u : 0];
        } else if (c0 + u < len) {
          w[u] = ld_stream(ws + kSellW * (c0 + u));
          code[u] = ld_stream(cs + kSellC * (c0 + u));
        }
      if (PIPE)
#pragma unroll
        for (int u = 0; u < B; ++u)
          if (c0 + B + u < len) {
            wn[PIPE ? u : 0] = ld_stream(ws + kSellW * (c0 + B + u));
            coden[PIPE ? u : 0] = ld_stream(cs + kSellC * (c0 + B + u));
          }
      // EARLY: the batch's records all in flight before the arithmetic (L1/L2 latency);
      // otherwise each one just before its bond's terms (shared memory)
      float4 cn[EARLY ? B : 1], nb[EARLY ? B : 1];
      if (EARLY)
#pragma unroll
        for (int u = 0; u < B; ++u)
          if (c0 + u < len) rec(code_node(hbw, code[u]), cn[EARLY ? u : 0], nb[EARLY ? u : 0]);
#pragma unroll
      for (int u = 0; u < B; ++u)
        if (c0 + u < len) {
          const int ur = EARLY ? u : 0;
          if (!EARLY) rec(code_node(hbw, code[u]), cn[0], nb[0]);
          const bool nsol = nb[ur].z != 0.0f;
          const float dphi = (nb[ur].x - cb.x) + (nb[ur].y - cb.y);
          iface |= (pa != 0.0f && !nsol) ? 1 : 0;
#pragma unroll
          for (int s = 0; s < S; ++s) {
            const float cw = (nsol ? cfS[s] : cfL[s]) * w[u];
            const float cns = sel4(cn[ur], s);
            a1[s] = fmaf(cw, cns - sel4(ca, s), a1[s]);
            a2[s] = fmaf(cw * cns, dphi, a2[s]);
          }
        }
    }
    const unsigned char dm = k.dirmask[a];
    const float4 lo4 = k.clo[a];
    const bool src_on = iface && !(dm & 1);
    const double swv = src_on ? dissolve_switch((double)ca.x + (double)lo4.x, k.csat, k.sw) : 0.0;
    const float Rmg = src_on ? (float)(-k.k_diss * swv) : 0.0f;
    if (RESID) {
#pragma unroll
      for (int s = 0; s < S; ++s)
        F_out[(size_t)s * k.N + a] =
            -(double)K1f[s] * a1[s] - (double)K2f[s] * a2[s] - (s == 0 ? (double)Rmg : 0.0);
    } else {
      // c + dt (K1 a1 + K2 a2 + R) on the compensated pair (hi, lo), renormalised: hi is
      // the FP32 rounding of the exact pair sum and lo its exact remainder
      const float dtf = (float)k.dt;
      float hi[S], lo[S];
      bool bad = false;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const float inc = dtf * (K1f[s] * a1[s] + K2f[s] * a2[s] + (s == 0 ? Rmg : 0.0f));
        float tt, e1, sh, e2;
        two_sum(sel4(lo4, s), inc, tt, e1);
        two_sum(sel4(ca, s), tt, sh, e2);
        two_sum(sh, e1 + e2, hi[s], lo[s]);
        if ((dm >> s) & 1) {
          const double x = k.bcval[(size_t)s * k.N + a];
          hi[s] = (float)x;
          lo[s] = (float)(x - (double)hi[s]);
        }
        // clamp c >= c_floor (main.cpp:805-837), compared on the normalised pairs
        if (hi[s] < k.cfl_hi || (hi[s] == k.cfl_hi && lo[s] < k.cfl_lo)) {
          hi[s] = k.cfl_hi;
          lo[s] = k.cfl_lo;
        }
        bad = bad || !isfinite(hi[s]);
      }
      float pnew = pa;
      // saturation test in FP64 (main.cpp:914-922)
      if (pa != 0.0f && (double)hi[0] + (double)lo[0] <= k.csat) {
        pnew = 0.0f;
        k.flip_step[a] = (int)(k.ds->steps + 1);
        k.flip_list[atomicAdd(&k.ds->nflip, 1)] = a;
        k.ds->op_valid = 0;
        k.ds->defl = 0;
      }
      record_history(k, a, k.hist_m >= 3 ? (k.ds->hist_head + 1) % k.hist_m : 0);
      const double g = next_phi_guess(k, a);
      Rec32 out;
#pragma unroll
      for (int s = 0; s < S; ++s) out.c[s] = hi[s];
      out.phi_hi = (float)g;
      out.phi_lo = (float)(g - (double)out.phi_hi);
      out.phase = pnew;
      out.pad = 0.0f;
      k.rec32_nxt[a] = out;
      k.clo[a] = make_float4(lo[0], lo[1], lo[2], lo[3]);
      // diagnostics as FP32 pairs: masses, solid volume sum (c_0 - CSat/CSolid), dissolved
#pragma unroll
      for (int s = 0; s < S; ++s) {
        ph_hi[s] = hi[s];
        ph_lo[s] = lo[s];
      }
      if (pnew != 0.0f) {
        n_solid = 1;
        float vs, ve;
        two_sum(hi[0], -k.csat_hi, vs, ve);
        ph_hi[4] = vs;
        ph_lo[4] = ve + (lo[0] - k.csat_lo);
      }
      if (src_on) {
        const double dv = k.k_diss * swv;
        ph_hi[5] = (float)dv;
        ph_lo[5] = (float)(dv - (double)ph_hi[5]);
      }
      n_bad = bad ? 1 : 0;
    }
  }
  __syncwarp();
  if (!RESID) {
#pragma unroll
    for (int q = 0; q < 6; ++q) pair_warp_sum(ph_hi[q], ph_lo[q]);
    n_solid = __reduce_add_sync(0xffffffffu, n_solid);
    n_bad = __reduce_add_sync(0xffffffffu, n_bad);
    if (lane == 0) {
      const size_t st = v.stride;
#pragma unroll
      for (int s = 0; s < S; ++s) store_pair(v.partials, s * st + sg, ph_hi[s], ph_lo[s]);
      store_pair(v.partials, 4 * st + sg, (float)n_solid, 0.0f);  // counts <= 32: exact
      store_pair(v.partials, 5 * st + sg, ph_hi[4], ph_lo[4]);
      store_pair(v.partials, 6 * st + sg, ph_hi[5], ph_lo[5]);
      store_pair(v.partials, 7 * st + sg, (float)n_bad, 0.0f);
      store_pair(v.partials, 8 * st + sg, 0.0f, 0.0f);
    }
  }
}

// the transport's last CTA: every instance's diagnostics from its slices' partials, then
// the counters' reset
template <int BLK>
__device__ __forceinline__ void transport_last_cta(const EngineView& v, double* sm, int* s_last) {
  if (!take_last_ticket(&v.ticket[v.M + 1], s_last)) return;
  for (int i = 0; i < v.M; ++i) {
    double tot[kDiagSlots];
    reduce_pair_items<kDiagSlots, BLK>(v.partials, v.stride, v.slice_first[i], v.slice_count[i], tot, sm);
    if (threadIdx.x == 0) finish_instance(v.inst[i], tot);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    v.ticket[v.M + 1] = 0;
    v.ticket[v.M + 2] = 0;
  }
}

// Mixed transport, neighbour records gathered from L1/L2.  Warps claim slices one at a time
// (slices of solid nodes, narrow and partial slices cost less than full ones); the residual
// form, which has no last CTA to reset the counter, keeps the static split.
template <int W, bool RESID>
__global__ void __launch_bounds__(kBlock, 2) k_transport32(EngineView v, double* F_out) {
  __shared__ int s_hb[kBlock / 32][12];
  __shared__ double sm[kDiagSlots * kBlock / 32];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr bool kClaim = !RESID;
  int s0, s1;
  if (kClaim) {
    s0 = claim_slice(v, lane);
    s1 = v.nslices;
  } else {
    warp_slices(v, &s0, &s1);
  }
  for (int sg = s0; sg < s1; sg = kClaim ? claim_slice(v, lane) : sg + 1) {
    const float4* rc = reinterpret_cast<const float4*>(v.inst[__ldg(&v.slices[sg].inst)].rec32_cur);
    transport_slice<RESID, kTrB, true, false>(v, sg, lane, s_hb[warp], nullptr,
                                 [rc](int n, float4& c, float4& t) { ld_rec32(rc + 2 * n, c, t); }, F_out);
  }
  if (RESID) return;
  transport_last_cta<kBlock>(v, sm, &s_last);
}

// Halo-staged mixed transport.  A CTA claims tiles one at a time; thread 0 copies the tile's
// halo records (its 9 halo rows: contiguous node ranges, 32-byte records) into shared memory
// by bulk copies on one mbarrier (a bounded wait: a timeout is recorded in the instance's state
// and reported as NNPP_ERR_CUDA), then the CTA's warps take the tile's slices and gather
// every neighbour's record from shared memory (its slot in the halo: the slice's window code
// rebased from the slice's window rows onto the tile's halo rows).  HBM and L2 see the
// streamed codes and weights and one copy of each halo; the per-bond gathers stay on chip.
constexpr int kTrHBlock = 128;
__host__ __device__ constexpr size_t smem_tr_halo(int halo_max) { return (size_t)halo_max * 32; }
// largest halo staged: two CTAs of 4 warps an SM at least
constexpr size_t kTrHaloSmemMax = 110 * 1024;

template <int B, bool PIPE, int MINB>
__global__ void __launch_bounds__(kTrHBlock, MINB) k_transport32h(EngineView v) {
  extern __shared__ __align__(16) float4 hrec[];  // 2 float4 a halo node
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_tile, s_stop, s_last;
  __shared__ int s_adj[9];  // halo row r: first node - its first slot
  __shared__ int s_hb[kTrHBlock / 32][12];
  __shared__ double sm[kDiagSlots * kTrHBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    s_stop = 0;
  }
  __syncthreads();
  unsigned phase = 0;
  for (;;) {
    if (threadIdx.x == 0) s_tile = s_stop ? v.ntiles : (int)atomicAdd(&v.ticket[v.M + 2], 1u);
    __syncthreads();
    const int t = s_tile;
    if (t >= v.ntiles) break;
    const TileDesc& td = v.tiles[t];
    const KParams& k = v.inst[td.inst];
    if (threadIdx.x == 0) {
      const float4* rc = reinterpret_cast<const float4*>(k.rec32_cur);
      unsigned bytes = 0;
      int acc = 0;
      for (int r = 0; r < 9; ++r) {
        s_adj[r] = td.hb[r] - acc;
        acc += td.hl[r];
        bytes += (unsigned)td.hl[r] * 32u;
      }
      // the previous tile's reads of the buffer come before the copies
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&bar, bytes);
      acc = 0;
      for (int r = 0; r < 9; ++r) {
        if (td.hl[r] > 0) bulk_g2s(hrec + 2 * acc, rc + 2 * (size_t)td.hb[r], (unsigned)td.hl[r] * 32u, &bar);
        acc += td.hl[r];
      }
    }
    __syncthreads();
    if (!mbar_wait_bounded(&bar, phase, kHaloWaitPolls)) {
      k.ds->wait_timeout = 1;
      s_stop = 1;
    }
    phase ^= 1u;
    const int nsl = (td.own_end - td.own_begin + 31) >> 5;
    for (int q = warp; q < nsl; q += kTrHBlock / 32)
      transport_slice<false, B, false, PIPE>(v, td.slice0 + q, lane, s_hb[warp], s_adj,
                                    [](int i, float4& c, float4& tt) {
                                      c = hrec[2 * i];
                                      tt = hrec[2 * i + 1];
                                    },
                                    nullptr);
    __syncthreads();
  }
  transport_last_cta<kTrHBlock>(v, sm, &s_last);
}

// Next-solve guess of the nodes a transport turned liquid.  As solids they carried no
// potential (zero); a potential solve started from that zero spends its first refinement
// sweeps on those few nodes.  Each listed node instead takes the w-weighted mean of the
// potentials that its liquid neighbours carry into the next solve, counting only neighbours
// that were liquid before this step (so every value read is one this pass does not write, and
// the result does not depend on the list's order), and the same value in every slot of the
// warm-start history, where the backward differences then vanish.  phi_prev keeps the step's
// potential (the adjoint's snapshots read it), and the next transport does not extrapolate
// these nodes.  Potential-Dirichlet nodes keep their boundary value.  The last CTA resets the
// count for the next transport.
template <typename P>
__global__ void __launch_bounds__(kBlock) k_flip_guess(EngineView v) {
  __shared__ int s_last;
  for (int i = 0; i < v.M; ++i) {
    const KParams& k = v.inst[i];
    const int n = k.ds->nflip;
    const int step_no = (int)k.ds->steps;  // the transport's last CTA has counted its step
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
      const int a = k.flip_list[q];
      if ((k.dirmask[a] >> S) & 1) continue;
      double sw = 0.0, swp = 0.0;
      for (int j = k.row[a]; j < k.row[a + 1]; ++j) {
        const int m = k.col[j];
        if (m == a || k.flip_step[m] == step_no) continue;
        const bool liq = sizeof(P) == 4 ? k.rec32_nxt[m].phase == 0.0f : k.rec64_nxt[m].phase == 0.0;
        if (!liq) continue;
        const double w = (double)k.w32[j];
        sw += w;
        swp += w * k.phi64[m];
      }
      if (!(sw > 0.0)) continue;
      const double g = swp / sw;
      k.phi64[a] = g;
      if constexpr (sizeof(P) == 4) {
        const float hi = (float)g;
        k.rec32_nxt[a].phi_hi = hi;
        k.rec32_nxt[a].phi_lo = (float)(g - (double)hi);
      } else {
        k.rec64_nxt[a].phi = g;
      }
      if (k.hist_m >= 3)
        for (int sl = 0; sl < k.hist_m; ++sl) k.xh[(size_t)sl * k.N + a] = g;
    }
  }
  if (take_last_ticket(&v.ticket[v.M + 3], &s_last) && threadIdx.x == 0) {
    for (int i = 0; i < v.M; ++i) v.inst[i].ds->nflip = 0;
    v.ticket[v.M + 3] = 0;
  }
}

// FP64 transport (the plain FP64 path)
template <int W, bool RESID>
__global__ void __launch_bounds__(kBlock) k_transport64(EngineView v, double* F_out) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ TileSmem ts;
  __shared__ double sm[kDiagSlots * kBlock / 32];
  __shared__ int s_last;
  const int sub = threadIdx.x % W, seg = threadIdx.x / W, nseg = kBlock / W;
  for (int item = blockIdx.x; item < v.ntiles; item += gridDim.x) {
    const TileDesc t = v.tiles[item];
    const KParams& k = v.inst[t.inst];
    load_tile(t, ts);
    double* hrec = reinterpret_cast<double*>(dsm);  // 6 doubles per halo node (SoA)
    const unsigned short* sslot = stage_slots(k.slot16, t, dsm + (size_t)6 * t.halo * sizeof(double));
    const Rec64* rc = k.rec64_cur;
    const int H = t.halo;
    for (int s = threadIdx.x; s < H; s += kBlock) {
      const Rec64 r = rc[halo_node(ts, s)];
#pragma unroll
      for (int q = 0; q < S; ++q) hrec[(size_t)q * H + s] = r.c[q];
      hrec[(size_t)S * H + s] = r.phi;
      hrec[(size_t)(S + 1) * H + s] = r.phase;
    }
    __syncthreads();
    const double BV = *k.bv_ptr;
    double cLL[S], cX[S], cSS[S];
#pragma unroll
    for (int s = 0; s < S; ++s) {
      cLL[s] = k.DL[s];
      cX[s] = s == 0 ? k.DSo[0] * BV : k.DSo[s];
      cSS[s] = s == 0 ? k.DSo[0] : 0.0;
    }
    const long long step_no = k.ds->steps + 1;
    const int hslot = k.hist_m >= 3 ? (k.ds->hist_head + 1) % k.hist_m : 0;
    const int* row = k.row;
    const double* w64 = k.w64;
    const int own0 = ts.off[4] + (t.own_begin - t.hb[4]);
    double part[kDiagSlots];
#pragma unroll
    for (int q = 0; q < kDiagSlots; ++q) part[q] = 0.0;
    for (int a0 = t.own_begin; a0 < t.own_end; a0 += nseg) {
      const int a = a0 + seg;
      const bool act = a < t.own_end;
      const int so = own0 + (a - t.own_begin);
      double ca[S], pha = 0.0, pa = 0.0;
#pragma unroll
      for (int s = 0; s < S; ++s) ca[s] = act ? hrec[(size_t)s * H + so] : 0.0;
      if (act) {
        pha = hrec[(size_t)S * H + so];
        pa = hrec[(size_t)(S + 1) * H + so];
      }
      double a1[S], a2[S];
#pragma unroll
      for (int s = 0; s < S; ++s) a1[s] = a2[s] = 0.0;
      int iface = 0;
      if (act) {
        for (int j = row[a] + sub; j < row[a + 1]; j += W) {
          const int sl = sslot[j - t.bond0];
          const double w = w64[j];
          const double pn = hrec[(size_t)(S + 1) * H + sl];
          const double dphi = hrec[(size_t)S * H + sl] - pha;
          const bool ll = (pa == 0.0) && (pn == 0.0);
          const bool ss = (pa != 0.0) && (pn != 0.0);
          iface |= (pa != 0.0 && pn == 0.0) ? 1 : 0;
#pragma unroll
          for (int s = 0; s < S; ++s) {
            const double coef = ll ? cLL[s] : (ss ? cSS[s] : cX[s]);
            const double cw = coef * w;
            const double cns = hrec[(size_t)s * H + sl];
            a1[s] += cw * (cns - ca[s]);
            a2[s] += cw * cns * dphi;
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
      const double swv = src_on ? dissolve_switch(ca[0], k.csat, k.sw) : 0.0;
      const double Rmg = src_on ? -k.k_diss * swv : 0.0;
      if (RESID) {
#pragma unroll
        for (int s = 0; s < S; ++s)
          F_out[(size_t)s * k.N + a] = -k.K1[s] * a1[s] - k.K2zF[s] * a2[s] - (s == 0 ? Rmg : 0.0);
        continue;
      }
      double val[S];
      bool bad = false;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const double F = -k.K1[s] * a1[s] - k.K2zF[s] * a2[s] - (s == 0 ? Rmg : 0.0);
        double x = ca[s] - k.dt * F;
        if ((dm >> s) & 1) x = k.bcval[(size_t)s * k.N + a];
        if (x < k.c_floor) x = k.c_floor;
        if (!isfinite(x)) bad = true;
        val[s] = x;
      }
      double pnew = pa;
      if (pa != 0.0 && val[0] <= k.csat) {
        pnew = 0.0;
        k.flip_step[a] = (int)step_no;
        k.flip_list[atomicAdd(&k.ds->nflip, 1)] = a;
        k.ds->op_valid = 0;
        k.ds->defl = 0;
      }
      record_history(k, a, hslot);
      const double g = next_phi_guess(k, a);
      Rec64 out;
#pragma unroll
      for (int s = 0; s < S; ++s) out.c[s] = val[s];
      out.phi = g;
      out.phase = pnew;
      out.pad[0] = out.pad[1] = 0.0;
      k.rec64_nxt[a] = out;
#pragma unroll
      for (int s = 0; s < S; ++s) part[s] += val[s];
      if (pnew != 0.0) {
        part[4] += 1.0;
        part[5] += val[0] - k.csat;
      }
      part[6] += k.k_diss * swv;
      part[7] += bad ? 1.0 : 0.0;
    }
    if (!RESID) transport_finish(v, t, k, item, part, sm, &s_last);
    __syncthreads();
  }
}

// ------------------------------------------------------------------- state transfer -----
__global__ void k_load_state(KParams k, const int* perm, const double* c_user, const double* phi_user,
                             const int* phase_user, int mixed, int dirichlet_phi, int keep_history) {
  const int N = k.N;
  // the history pairs (x, A x) stay valid guesses for the same operator; a new state
  // starts without them unless the caller continues a run (nnpp_step_host)
  if (blockIdx.x == 0 && threadIdx.x == 0 && !keep_history) k.ds->hist_n = 0;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += gridDim.x * blockDim.x) {
    const int u = perm[a];
    double c[S];
    for (int s = 0; s < S; ++s) c[s] = c_user[(size_t)s * N + u];
    double phi = phi_user ? phi_user[u] : k.phi_prev[a];
    if (dirichlet_phi && ((k.dirmask[a] >> S) & 1)) phi = k.bcval[(size_t)S * N + a];
    const float ph_old = mixed ? k.rec32_cur[a].phase : (float)k.rec64_cur[a].phase;
    const float ph = phase_user ? (phase_user[u] != 0 ? 1.0f : 0.0f) : ph_old;
    if (ph != ph_old) {  // a new liquid mask: the prep recomputes the diagonal, no deflation
      k.ds->op_valid = 0;
      k.ds->defl = 0;
    }
    k.phi64[a] = phi;
    k.phi_prev[a] = phi;
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

// The potential of the last solve is phi_prev (after a step phi64 holds the next warm
// start; before any step both agree).
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
    if (phi_user) phi_user[u] = k.phi_prev[a];
  }
}

// convert the current state between the two representations
__global__ void k_convert(KParams k, int to_mixed) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x) {
    if (to_mixed) {
      const Rec64 s64 = k.rec64_cur[a];
      Rec32 r;
      float lo[S];
      for (int s = 0; s < S; ++s) {
        r.c[s] = (float)s64.c[s];
        lo[s] = (float)(s64.c[s] - (double)r.c[s]);
      }
      r.phi_hi = (float)s64.phi;
      r.phi_lo = (float)(s64.phi - (double)r.phi_hi);
      r.phase = (float)s64.phase;
      r.pad = 0.0f;
      k.rec32_cur[a] = r;
      k.clo[a] = make_float4(lo[0], lo[1], lo[2], lo[3]);
    } else {
      const Rec32 s32 = k.rec32_cur[a];
      const float4 lo = k.clo[a];
      Rec64 r;
      for (int s = 0; s < S; ++s) r.c[s] = (double)s32.c[s] + (double)sel4(lo, s);
      r.phi = (double)s32.phi_hi + (double)s32.phi_lo;
      r.phase = (double)s32.phase;
      r.pad[0] = r.pad[1] = 0.0;
      k.rec64_cur[a] = r;
    }
  }
}

// initial diagnostics (main.cpp:472-480): solid count, vol0rel, masses; restart != 0 keeps
// vol0rel and the initial Mg mass and recomputes the relative volume of the current state
// instead (main.cpp:527-533, after a restart from file)
__global__ void k_init_diag(KParams k, int mixed, double* partials, int restart) {
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
    for (int q = 0; q < 7; ++q) partials[q * gridDim.x + blockIdx.x] = part[q];
  if (!take_last_ticket(&k.ds->ticket[0], &s_last)) return;
  double tot[7];
  reduce_partials<7, kBlock>(partials, gridDim.x, tot, sm);
  if (threadIdx.x == 0) {
    DevState* ds = k.ds;
    ds->ticket[0] = 0;
    for (int s = 0; s < S; ++s) ds->mass[s] = tot[s];
    ds->mg_mass_now = tot[0];
    ds->solid_count = (long long)tot[4];
    if (restart) {
      ds->voln1rel = ds->vol0rel != 0.0 ? tot[5] / ds->vol0rel : 0.0;
    } else {
      ds->mg_mass_t0 = tot[0];
      ds->vol0rel = tot[5];
      ds->voln1rel = 0.0;
    }
    ds->BV = pow(10., -k.vol_red * (1. - ds->voln1rel));
  }
}

template <typename F>
nnpp_status dispatch_lanes(int lanes, F&& f) {
  switch (lanes) {
    case 4: return f(std::integral_constant<int, 4>());
    case 8: return f(std::integral_constant<int, 8>());
    case 16: return f(std::integral_constant<int, 16>());
    default: return set_error(NNPP_ERR_INVALID, "lanes per node must be 4, 8 or 16");
  }
}

// Persistent grid: as many CTAs as fit on the device at once (at most one per item).
template <typename K>
int occ_grid_b(K kern, int block, size_t smem, int sms, int items) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, block, smem) != cudaSuccess) {
    cudaGetLastError();
    nb = 1;
  }
  if (nb < 1) nb = 1;
  const int g = sms * nb;
  return items < g ? (items > 0 ? items : 1) : g;
}

template <typename K>
int occ_grid(K kern, size_t smem, int sms, int items) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kBlock, smem) != cudaSuccess) {
    cudaGetLastError();
    nb = 1;
  }
  if (nb < 1) nb = 1;
  const int g = sms * nb;
  return items < g ? (items > 0 ? items : 1) : g;
}

// Grid of a slice kernel with several CTAs per SM: as many 8-warp CTAs as give every warp
// the same number of slices (the fewest rounds the resident warps need), so that no warp
// idles a whole slice at the end while the others of its CTA finish a second one.
template <typename K>
int slice_grid(K kern, size_t smem, int sms, int nslices) {
  const int g = occ_grid(kern, smem, sms, (nslices + 7) / 8);
  const int rounds = (nslices + 8 * g - 1) / (8 * g);
  const int g2 = (nslices + 8 * rounds - 1) / (8 * rounds);
  return g2 < 1 ? 1 : g2;
}

// kernels whose warps claim slices: as many CTAs as the SMs hold at once (fewer when the
// slices are fewer than the warps)
template <typename K>
int claim_grid(K kern, size_t smem, int sms, int nslices) {
  return occ_grid(kern, smem, sms, (nslices + 7) / 8);
}

size_t smem_slots(int B) { return (size_t)(B + 16) * sizeof(unsigned short); }
size_t smem_prep(int H, int B) { return align16((size_t)H * (sizeof(double) + 1)) + smem_slots(B); }
size_t smem_vec64(int H, int B) { return align16((size_t)H * sizeof(double)) + smem_slots(B); }
size_t smem_spmv_staged() { return kTmaRingBytes + kTmaWinBytes + kTmaBarBytes; }
// streamed operator: the deepest ring (2..4 stages) that fits beside windows of win_cap nodes
constexpr size_t kSmemCta = 225 * 1024;
// stages of kStreamCol columns (2 .. kStreamMaxStages)
constexpr int kStreamCol = 32;
constexpr int kStreamMaxStages = 4;
size_t smem_spmv_stream(int win_cap, int* stages) {
  const size_t win = (size_t)kWarpsCta * 2 * win_cap * sizeof(float) + (size_t)kWarpsCta * kDescRing * sizeof(SliceDesc);
  const size_t sb = (size_t)kStreamCol * kSellW * 4 + sizeof(uint64_t);
  int st = kStreamMaxStages;
  while (st > 2 && (size_t)kWarpsCta * st * sb + win > kSmemCta) --st;
  *stages = st;
  return (size_t)kWarpsCta * st * sb + win;
}
size_t smem_spmv_win() { return (size_t)(kBlock / 32) * kWinCap * sizeof(float); }
size_t smem_tr64(int H, int B) { return (size_t)H * 6 * sizeof(double) + smem_slots(B); }
size_t smem_adj(int H, int B) { return align16((size_t)H * (9 * sizeof(double) + 1)) + smem_slots(B) + 16; }

template <typename K>
nnpp_status allow_smem(K kern, size_t bytes) {
  if (bytes > 32 * 1024)  // the default limit counts static shared memory too
    NNPP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return NNPP_OK;
}

// ------------------------------------------------------------------- adjoint -------------
// Transpose of one explicit step (FP64).  For node m, with lh = lambda^{n+1} masked to zero
// on Dirichlet and clamped entries, a = dt K1 D w and b = dt K2 z F/(RT) D w:
//   mu_k,m = lh_k,m + sum_i a (lh_k,i - lh_k,m) + sum_i lh_k,i b (phi_m - phi_i)
//            [+ lh_0,m (-dt k S'(c_0,m)) on interface nodes]
//   nu_m   = sum_k dt K2zF_k (c_k,m sum_i D w lh_k,i - lh_k,m sum_i D w c_k,i)   (d/dphi)
// and the parameter sensitivities dL/dD_k = sum_m lh_k,m (transport increment)/D_k,
// dL/dk = sum_m lh_0,m (-dt S(c_0,m)) over interface nodes.  The bond terms are the
// off-diagonal weights of the reference's tangent (utils.h:955-963), applied transposed.
struct AdjArgs {
  const Rec64* snap;   // c^n, phi^n, phase^n
  const Rec64* snap1;  // c^{n+1} (clamp mask)
  const double* lam;   // lambda^{n+1}, S*N
  double* mu;          // S*N
  double* nu;          // N
  double* acc;         // 5 accumulators (dL/dD_k, dL/dk)
};

__device__ __forceinline__ double pair_D(const KParams& k, int s, bool pm, bool pi) {
  if (!pm && !pi) return k.DL[s];
  if (s == 0) return k.DSo[0];  // BV = 1: the adjoint requires vol_red = 0
  if (pm && pi) return 0.0;
  return k.DSo[s];
}

template <int W>
__global__ void __launch_bounds__(kBlock) k_adj_transport(EngineView v, AdjArgs ad) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ TileSmem ts;
  __shared__ double sm[5 * kBlock / 32];
  __shared__ int s_last;
  const int sub = threadIdx.x % W, seg = threadIdx.x / W, nseg = kBlock / W;
  for (int item = blockIdx.x; item < v.ntiles; item += gridDim.x) {
    const TileDesc t = v.tiles[item];
    const KParams& k = v.inst[t.inst];
    load_tile(t, ts);
    const int H = t.halo;
    const int N = k.N;
    double* hc = reinterpret_cast<double*>(dsm);  // c: S*H
    double* hl = hc + (size_t)S * H;              // masked lambda: S*H
    double* hphi = hl + (size_t)S * H;            // H
    unsigned char* hph = reinterpret_cast<unsigned char*>(hphi + H);
    const unsigned short* sslot = stage_slots(k.slot16, t, dsm + align16((size_t)9 * H * sizeof(double) + H));
    for (int s = threadIdx.x; s < H; s += kBlock) {
      const int n = halo_node(ts, s);
      const Rec64 r = ad.snap[n];
      const Rec64 r1 = ad.snap1[n];
      const unsigned char dm = k.dirmask[n];
#pragma unroll
      for (int q = 0; q < S; ++q) {
        hc[(size_t)q * H + s] = r.c[q];
        const bool zero = ((dm >> q) & 1) || r1.c[q] == k.c_floor;
        hl[(size_t)q * H + s] = zero ? 0.0 : ad.lam[(size_t)q * N + n];
      }
      hphi[s] = r.phi;
      hph[s] = r.phase != 0.0 ? 1 : 0;
    }
    __syncthreads();
    const int* row = k.row;
    const double* w64 = k.w64;
    const double dt = k.dt;
    const int own0 = ts.off[4] + (t.own_begin - t.hb[4]);
    double part[5] = {0, 0, 0, 0, 0};
    for (int a0 = t.own_begin; a0 < t.own_end; a0 += nseg) {
      const int a = a0 + seg;
      const bool act = a < t.own_end;
      const int so = own0 + (a - t.own_begin);
      double cm[S], lm[S];
      double phm = 0.0;
      bool pm = false;
#pragma unroll
      for (int q = 0; q < S; ++q) {
        cm[q] = act ? hc[(size_t)q * H + so] : 0.0;
        lm[q] = act ? hl[(size_t)q * H + so] : 0.0;
      }
      if (act) {
        phm = hphi[so];
        pm = hph[so] != 0;
      }
      double acc[S], a1[S], a2[S], sl[S], sc[S];
#pragma unroll
      for (int q = 0; q < S; ++q) acc[q] = a1[q] = a2[q] = sl[q] = sc[q] = 0.0;
      int iface = 0;
      if (act) {
        for (int j = row[a] + sub; j < row[a + 1]; j += W) {
          const int si = sslot[j - t.bond0];
          const double w = w64[j];
          const bool pi = hph[si] != 0;
          const double phi_i = hphi[si];
          iface |= (pm && !pi) ? 1 : 0;
#pragma unroll
          for (int q = 0; q < S; ++q) {
            const double Dw = pair_D(k, q, pm, pi) * w;
            const double li = hl[(size_t)q * H + si];
            const double ci = hc[(size_t)q * H + si];
            acc[q] += dt * k.K1[q] * Dw * (li - lm[q]) + li * dt * k.K2zF[q] * Dw * (phm - phi_i);
            a1[q] += Dw * (ci - cm[q]);
            a2[q] += Dw * ci * (phi_i - phm);
            sl[q] += Dw * li;
            sc[q] += Dw * ci;
          }
        }
      }
#pragma unroll
      for (int q = 0; q < S; ++q) {
        acc[q] = seg_reduce_d<W>(acc[q]);
        a1[q] = seg_reduce_d<W>(a1[q]);
        a2[q] = seg_reduce_d<W>(a2[q]);
        sl[q] = seg_reduce_d<W>(sl[q]);
        sc[q] = seg_reduce_d<W>(sc[q]);
      }
      iface = seg_or<W>(iface);
      if (!act || sub != 0) continue;
      const bool src = iface && !(k.dirmask[a] & 1);
      double nu = 0.0;
#pragma unroll
      for (int q = 0; q < S; ++q) {
        double m = lm[q] + acc[q];
        if (q == 0 && src) {
          const double sw = dissolve_switch(cm[0], k.csat, k.sw);
          const double dsw = k.sw > 0.0 ? sw * (1.0 - sw) / k.sw : 0.0;
          m += lm[0] * (-dt * k.k_diss * dsw);
          part[4] += lm[0] * (-dt * sw);
        }
        ad.mu[(size_t)q * N + a] = m;
        nu += dt * k.K2zF[q] * (cm[q] * sl[q] - lm[q] * sc[q]);
        part[q] += lm[q] * dt * (k.K1[q] * a1[q] + k.K2zF[q] * a2[q]) / k.DL[q];
      }
      ad.nu[a] = nu;
    }
    write_partials<5>(v, item, part, sm);
    if (item_done(&v.ticket[t.inst], v.tile_count[t.inst], &s_last)) {
      double tot[5];
      reduce_items<5>(v.partials, v.stride, v.tile_first[t.inst], v.tile_count[t.inst], tot, sm);
      if (threadIdx.x == 0) {
        for (int q = 0; q < 5; ++q) ad.acc[q] += tot[q];
        v.ticket[t.inst] = 0;
      }
    }
    __syncthreads();
  }
}

// Mixed adjoint transport: the same transpose in FP32 on the sliced operator.  k_adj_pack
// writes per node the 48-byte record {c[4], masked lambda[4], phi_hi, phi_lo, phase, 0};
// k_adj_transport32 streams the slices (one lane per node), gathers the neighbours' records
// from L1/L2, forms the differences directly (no cancellation of large sums) and
// accumulates the parameter sensitivities as FP32 pairs.
__global__ void k_adj_pack(KParams k, const Rec64* snap, const Rec64* snap1, const double* lam,
                           float4* rec) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x) {
    const Rec64 r = snap[a];
    const Rec64 r1 = snap1[a];
    const unsigned char dm = k.dirmask[a];
    float lh[S];
#pragma unroll
    for (int q = 0; q < S; ++q) {
      const bool zero = ((dm >> q) & 1) || r1.c[q] == k.c_floor;
      lh[q] = zero ? 0.0f : (float)lam[(size_t)q * k.N + a];
    }
    const float ph = (float)r.phi;
    rec[3 * a] = make_float4((float)r.c[0], (float)r.c[1], (float)r.c[2], (float)r.c[3]);
    rec[3 * a + 1] = make_float4(lh[0], lh[1], lh[2], lh[3]);
    rec[3 * a + 2] = make_float4(ph, (float)(r.phi - (double)ph), r.phase != 0.0 ? 1.0f : 0.0f, 0.0f);
  }
}

// bond columns per batch of the FP32 adjoint transport: 4 at 127 registers (2 CTAs an SM);
// the 400-step backward of the 262k calibration workload took 1014 ms against 1059 with 2
constexpr int kAdjB = 4;
template <int W>
__global__ void __launch_bounds__(kBlock, 2) k_adj_transport32(EngineView v, const float4* rec,
                                                               double* mu, double* nu, double* acc) {
  __shared__ int s_hb[kBlock / 32][12];
  __shared__ double sm[5 * kBlock / 32];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // warps claim slices one at a time (slices of solid nodes, narrow and partial slices
  // cost less than full ones)
  for (int sg = claim_slice(v, lane); sg < v.nslices; sg = claim_slice(v, lane)) {
    const SliceDesc d = v.slices[sg];
    const KParams& k = v.inst[d.inst];
    if (lane < 9) s_hb[warp][lane] = v.slices[sg].gbase[lane];
    __syncwarp();
    float gh[5], gl[5];  // dL/dD_k (4), dL/dk as FP32 pairs
#pragma unroll
    for (int q = 0; q < 5; ++q) gh[q] = gl[q] = 0.0f;
    const int a = d.row0 + lane;
    if (lane < d.nrows) {
      const int* hb = s_hb[warp];
      const float4 cm4 = rec[3 * a], lm4 = rec[3 * a + 1], pm4 = rec[3 * a + 2];
      const bool pm = pm4.z != 0.0f;
      float cfL[S], cfS[S];  // pair coefficient for a liquid / solid neighbour (BV = 1)
#pragma unroll
      for (int q = 0; q < S; ++q) {
        const float dl = (float)k.DL[q], ds = (float)k.DSo[q];
        cfL[q] = pm ? ds : dl;
        cfS[q] = pm ? (q == 0 ? ds : 0.0f) : ds;
      }
      float A1[S], A2[S], a1[S], a2[S], sl[S], sc[S];
#pragma unroll
      for (int q = 0; q < S; ++q) A1[q] = A2[q] = a1[q] = a2[q] = sl[q] = sc[q] = 0.0f;
      int iface = 0;
      const float* ws = sell_w(k, d) + lane;
      const unsigned short* cs = sell_code(k, d) + lane;
      const int len = k.row[a + 1] - k.row[a];
      // bonds in batches of kAdjB columns (codes, weights and records in flight together;
      // the column order of the sums is kept)
      for (int c0 = 0; c0 < len; c0 += kAdjB) {
        float wv[kAdjB];
        unsigned int code[kAdjB];
#pragma unroll
        for (int u = 0; u < kAdjB; ++u)
          if (c0 + u < len) {
            wv[u] = ld_stream(ws + kSellW * (c0 + u));
            code[u] = ld_stream(cs + kSellC * (c0 + u));
          }
        float4 cnv[kAdjB], lnv[kAdjB], pnv[kAdjB];
#pragma unroll
        for (int u = 0; u < kAdjB; ++u)
          if (c0 + u < len) {
            const int n = code_node(hb, code[u]);
            cnv[u] = __ldg(rec + 3 * n);
            lnv[u] = __ldg(rec + 3 * n + 1);
            pnv[u] = __ldg(rec + 3 * n + 2);
          }
#pragma unroll
        for (int u = 0; u < kAdjB; ++u)
          if (c0 + u < len) {
            const float w = wv[u];
            const float4 cn = cnv[u], ln = lnv[u], pn = pnv[u];
            const bool nsol = pn.z != 0.0f;
            iface |= (pm && !nsol) ? 1 : 0;
            const float dphi = (pm4.x - pn.x) + (pm4.y - pn.y);  // phi_m - phi_i
#pragma unroll
            for (int q = 0; q < S; ++q) {
              const float Dw = (nsol ? cfS[q] : cfL[q]) * w;
              const float li = sel4(ln, q), ci = sel4(cn, q);
              A1[q] = fmaf(Dw, li - sel4(lm4, q), A1[q]);
              a1[q] = fmaf(Dw, ci - sel4(cm4, q), a1[q]);
              const float tl = Dw * li, tc = Dw * ci;
              A2[q] = fmaf(tl, dphi, A2[q]);
              a2[q] = fmaf(-tc, dphi, a2[q]);
              sl[q] += tl;
              sc[q] += tc;
            }
          }
      }
      const unsigned char dm = k.dirmask[a];
      const bool src = iface && !(dm & 1);
      const float dt = (float)k.dt;
      float nu_a = 0.0f;
#pragma unroll
      for (int q = 0; q < S; ++q) {
        const float K1 = (float)k.K1[q], K2 = (float)k.K2zF[q];
        const float lmq = sel4(lm4, q), cmq = sel4(cm4, q);
        float m = lmq + dt * (K1 * A1[q] + K2 * A2[q]);
        if (q == 0 && src) {
          const double swd = dissolve_switch((double)cm4.x, k.csat, k.sw);
          const double dsw = k.sw > 0.0 ? swd * (1.0 - swd) / k.sw : 0.0;
          m += lmq * (float)(-k.dt * k.k_diss * dsw);
          const float gk = lmq * (float)(-k.dt * swd);
          float ek;
          two_sum(gh[4], gk, gh[4], ek);
          gl[4] += ek;
        }
        mu[(size_t)q * k.N + a] = (double)m;
        nu_a = fmaf(dt * K2, cmq * sl[q] - lmq * sc[q], nu_a);
        const float gq = lmq * dt * (K1 * a1[q] + K2 * a2[q]) / (float)k.DL[q];
        float e;
        two_sum(gh[q], gq, gh[q], e);
        gl[q] += e;
      }
      nu[a] = (double)nu_a;
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 5; ++q) pair_warp_sum(gh[q], gl[q]);
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 5; ++q) store_pair(v.partials, (size_t)q * v.stride + sg, gh[q], gl[q]);
  }
  if (take_last_ticket(&v.ticket[v.M + 1], &s_last)) {
    for (int i = 0; i < v.M; ++i) {
      double tot[5];
      reduce_pair_items<5>(v.partials, v.stride, v.slice_first[i], v.slice_count[i], tot, sm);
      if (threadIdx.x == 0)
        for (int q = 0; q < 5; ++q) acc[q] += tot[q];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      v.ticket[v.M + 1] = 0;
      v.ticket[v.M + 2] = 0;
    }
  }
}

// lambda^n = mu + (1/(K sigma)) F CSolid z_k psi on the unknowns, + the loss injection on
// species 0 (d(mass loss)/dc_0 = -dV times dL/d(sample))
__global__ void k_adj_combine(KParams k, const double* mu, double* lam, double inject) {
  const int N = k.N;
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < N; a += gridDim.x * blockDim.x) {
    const double psi = k.freem[a] ? k.phi64[a] : 0.0;
    for (int s = 0; s < S; ++s)
      lam[(size_t)s * N + a] = mu[(size_t)s * N + a] + k.lam * k.z[s] * psi + (s == 0 ? inject : 0.0);
  }
}

// snapshot c and phase of the current state (either representation)
__global__ void k_snap_state(KParams k, Rec64* dst, int mixed) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x) {
    Rec64 r = dst[a];
    if (mixed) {
      const Rec32 s32 = k.rec32_cur[a];
      const float4 lo = k.clo[a];
      for (int s = 0; s < S; ++s) r.c[s] = (double)s32.c[s] + (double)sel4(lo, s);
      r.phase = (double)s32.phase;
    } else {
      const Rec64 s64 = k.rec64_cur[a];
      for (int s = 0; s < S; ++s) r.c[s] = s64.c[s];
      r.phase = s64.phase;
    }
    dst[a] = r;
  }
}

// Recomputation without the potential solve: a step's solved potential (stored by
// forward_ckpt) as the solve leaves it -- phi64 and the current records' potential (the
// FP32 pair as set_phi_rec writes it) -- and into the step's snapshot.  On the nodes the
// solve does not change the stored value is the one the records already hold.
__global__ void k_load_phi(KParams k, const double* phi, Rec64* snap, int mixed) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x) {
    const double ph = phi[a];
    k.phi64[a] = ph;
    set_phi_rec(k, a, ph, mixed != 0);
    snap[a].phi = ph;
  }
}

// phi^n (the last solve's potential) into a snapshot
__global__ void k_snap_phi(KParams k, Rec64* dst) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x)
    dst[a].phi = k.phi_prev[a];
}

// adjoint solve set-up: phase^n into the current records, warm start psi (0 on Dirichlet
// and solid nodes)
__global__ void k_adj_solve_setup(KParams k, const Rec64* snap, const double* psi_prev) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x) {
    const double ph = snap[a].phase;
    k.rec32_cur[a].phase = (float)ph;
    k.rec64_cur[a].phase = ph;
    const bool zero = ph != 0.0 || ((k.dirmask[a] >> S) & 1);
    const double x = zero ? 0.0 : psi_prev[a];
    k.phi64[a] = x;
    k.phi_prev[a] = x;
    k.rec32_cur[a].phi_hi = (float)x;
    k.rec32_cur[a].phi_lo = (float)(x - (double)(float)x);
    k.rec64_cur[a].phi = x;
  }
}

__global__ void k_sum_c0(KParams k, int mixed, double* out) {
  __shared__ double sm[kBlock / 32];
  double part[1] = {0.0};
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < k.N; a += gridDim.x * blockDim.x) {
    if (mixed)
      part[0] += (double)k.rec32_cur[a].c[0] + (double)k.clo[a].x;
    else
      part[0] += k.rec64_cur[a].c[0];
  }
  block_sum<1, kBlock>(part, sm);
  if (threadIdx.x == 0) *out = part[0];
}

}  // namespace

nnpp_status launch_adj_transport(const Engine& e, const EngineView& v, const Rec64* snap,
                                 const Rec64* snap1, const double* lam, double* mu, double* nu,
                                 double* acc, cudaStream_t st) {
  AdjArgs ad{snap, snap1, lam, mu, nu, acc};
  const size_t sh = smem_adj(v.halo_max, v.bond_max);
  if (sh > 227 * 1024) return set_error(NNPP_ERR_UNSUPPORTED, "adjoint: tile halo too large");
  return dispatch_lanes(e.W, [&](auto wc) -> nnpp_status {
    constexpr int W = decltype(wc)::value;
    NNPP_TRY(allow_smem(k_adj_transport<W>, sh));
    k_adj_transport<W><<<occ_grid(k_adj_transport<W>, sh, e.sms, v.ntiles), kBlock, sh, st>>>(v, ad);
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  });
}

nnpp_status launch_adj_transport32(const Engine& e, const EngineView& v, Handle& h, const Rec64* snap,
                                   const Rec64* snap1, const double* lam, float4* rec, double* mu,
                                   double* nu, double* acc, cudaStream_t st) {
  KParams kp = make_kparams(h, h.cur);
  k_adj_pack<<<h.grid, kBlock, 0, st>>>(kp, snap, snap1, lam, rec);
  NNPP_CUDA(cudaGetLastError());
  k_adj_transport32<4><<<claim_grid(k_adj_transport32<4>, 0, e.sms, v.nslices), kBlock, 0, st>>>(
      v, rec, mu, nu, acc);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status launch_adj_combine(Handle& h, const double* mu, double* lam, double inject) {
  KParams kp = make_kparams(h, h.cur);
  k_adj_combine<<<h.grid, kBlock, 0, h.st>>>(kp, mu, lam, inject);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status launch_snap_state(Handle& h, Rec64* dst) {
  KParams kp = make_kparams(h, h.cur);
  k_snap_state<<<h.grid, kBlock, 0, h.st>>>(kp, dst, h.state_prec == NNPP_MIXED ? 1 : 0);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status launch_snap_phi(Handle& h, Rec64* dst) {
  KParams kp = make_kparams(h, h.cur);
  k_snap_phi<<<h.grid, kBlock, 0, h.st>>>(kp, dst);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status launch_load_phi(Handle& h, const double* phi, Rec64* snap) {
  KParams kp = make_kparams(h, h.cur);
  k_load_phi<<<h.grid, kBlock, 0, h.st>>>(kp, phi, snap, h.state_prec == NNPP_MIXED ? 1 : 0);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status launch_record_solve(Handle& h, int slot) {
  KParams kp = make_kparams(h, h.cur);
  k_record_solve<<<h.grid, kBlock, 0, h.st>>>(kp, slot);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status launch_adj_solve_setup(Handle& h, const Rec64* snap, const double* psi_prev) {
  NNPP_TRY(invalidate_operator(h));  // the adjoint solve's unknowns are those of step n
  KParams kp = make_kparams(h, h.cur);
  k_adj_solve_setup<<<h.grid, kBlock, 0, h.st>>>(kp, snap, psi_prev);
  NNPP_CUDA(cudaGetLastError());
  // deflated adjoint solve when the step's phases are those of the installed coarse operator
  return coarse_defl_check(h);
}

nnpp_status launch_sum_c0(Handle& h, double* out) {
  KParams kp = make_kparams(h, h.cur);
  // one block: a fixed summation order, so repeated runs give the same mass to the bit
  k_sum_c0<<<1, kBlock, 0, h.st>>>(kp, h.state_prec == NNPP_MIXED ? 1 : 0, out);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

// ---------------------------------------------------------------------------------------
nnpp_status prepare_kernels(int H, int B, int lanes) {
  // every tile kernel, the adjoint's included, must fit its staged halo
  if (smem_tr64(H, B) > 220 * 1024 || smem_adj(H, B) > 220 * 1024)
    return set_error(NNPP_ERR_UNSUPPORTED, "tile halo too large for shared memory");
  NNPP_TRY(allow_smem(k_cg_spmv32h<false>, 200 * 1024));  // spmv_halo_fits bounds the size used
  NNPP_TRY(allow_smem(k_cg_spmv32h<true>, 200 * 1024));
  // transport_halo_fits bounds the size used
  NNPP_TRY(allow_smem(k_transport32h<8, true, 4>, kTrHaloSmemMax));
  return dispatch_lanes(lanes, [&](auto wc) -> nnpp_status {
    constexpr int W = decltype(wc)::value;
    NNPP_TRY(allow_smem(k_prep<float, W>, smem_prep(H, B)));
    NNPP_TRY(allow_smem(k_prep<double, W>, smem_prep(H, B)));
    NNPP_TRY(allow_smem(k_cg_spmv64<W>, smem_vec64(H, B)));
    NNPP_TRY(allow_smem(k_cg_spmv32t<W>, smem_spmv_staged()));
    NNPP_TRY(allow_smem(k_cg_spmv32s<W, kStreamCol>, kSmemCta));
    NNPP_TRY(allow_smem(k_cg_spmv32<W, true, 8, true, 3>, smem_spmv_win()));
    NNPP_TRY(allow_smem(k_cg_spmv32<W, true, 16, false, 3>, smem_spmv_win()));
    NNPP_TRY(allow_smem(k_cg_spmv32<W, true, 16, false, 3, 3>, smem_spmv_win()));
    NNPP_TRY(allow_smem(k_cg_spmv32<W, true, 8, true, 3, 4>, smem_spmv_win()));
    NNPP_TRY(allow_smem(k_ir_update<float, W>, smem_vec64(H, B)));
    NNPP_TRY(allow_smem(k_ir_update<double, W>, smem_vec64(H, B)));
    NNPP_TRY(allow_smem(k_transport64<W, false>, smem_tr64(H, B)));
    NNPP_TRY(allow_smem(k_transport64<W, true>, smem_tr64(H, B)));
    return NNPP_OK;
  });
}

// FP32 CG operator variants without the staged ring (the autotuner's list): 0 L1/L2 gathers
// in batches of 16, pipelined (the next batch's weights and codes in flight while the current
// one gathers), 64 registers (32 warps per SM); 2 shared-memory windows, pipelined batches
// of 8; 3 L1/L2 gathers in batches of 16 (40 warps per SM); 4 shared-memory windows, batches
// of 16; 5, 6, 7: 4, 3, 2 with bulk L2 prefetches of the operator stream 3, 3, 4 batches ahead
template <int W>
void launch_spmv_gather(int variant, const EngineView& v, int sms, cudaStream_t st) {
  switch (variant) {
    case 2: {
      const size_t sh = smem_spmv_win();
      k_cg_spmv32<W, true, 8, true, 3><<<claim_grid(k_cg_spmv32<W, true, 8, true, 3>, sh, sms, v.ncslices), kBlock, sh, st>>>(v);
      break;
    }
    case 3:
      // 40 registers: six CTAs an SM (measured 0.087 ms at 512k; five CTAs 0.088, eight with
      // 32 registers 0.120, batches of 32 columns at four 0.089)
      k_cg_spmv32<W, false, 16, false, 6><<<claim_grid(k_cg_spmv32<W, false, 16, false, 6>, 0, sms, v.ncslices), kBlock, 0, st>>>(v);
      break;
    case 4: {
      const size_t sh = smem_spmv_win();
      k_cg_spmv32<W, true, 16, false, 3><<<claim_grid(k_cg_spmv32<W, true, 16, false, 3>, sh, sms, v.ncslices), kBlock, sh, st>>>(v);
      break;
    }
    case 5: {
      const size_t sh = smem_spmv_win();
      k_cg_spmv32<W, true, 16, false, 3, 3><<<slice_grid(k_cg_spmv32<W, true, 16, false, 3, 3>, sh, sms, v.ncslices), kBlock, sh, st>>>(v);
      break;
    }
    case 6:
      k_cg_spmv32<W, false, 16, false, 5, 3><<<slice_grid(k_cg_spmv32<W, false, 16, false, 5, 3>, 0, sms, v.ncslices), kBlock, 0, st>>>(v);
      break;
    case 7: {
      const size_t sh = smem_spmv_win();
      k_cg_spmv32<W, true, 8, true, 3, 4><<<slice_grid(k_cg_spmv32<W, true, 8, true, 3, 4>, sh, sms, v.ncslices), kBlock, sh, st>>>(v);
      break;
    }
    default:
      // measured 0.071 ms at 512k against 0.076 for 3; batches of 8 at 64 warps an SM took
      // 0.105, pipelined 16 at 3 CTAs 0.072, pipelined 24 at 3 CTAs (spilling) slower
      k_cg_spmv32<W, false, 16, true, 4><<<claim_grid(k_cg_spmv32<W, false, 16, true, 4>, 0, sms, v.ncslices), kBlock, 0, st>>>(v);
  }
}

bool spmv_staged_fits(const Engine& e) { return e.windows_fit && smem_spmv_staged() <= 227 * 1024; }

// the halo-staged operator's dynamic shared memory: the halo (plus the padding slot) as
// float4 and the largest tile code block
size_t smem_spmv_halo(int halo_max, int code_max16, int quad_max) {
  return (size_t)(halo_max + 1) * sizeof(float4) + (size_t)halo_zcap(halo_max + 1) * sizeof(float) +
         (size_t)((quad_max + 1) & ~1) * sizeof(float2) + (size_t)code_max16 * 16;
}
// the halo-staged transport runs when the largest tile halo fits a CTA's share
bool transport_halo_fits(const Engine& e) {
  return e.halo_max > 0 && smem_tr_halo(e.halo_max) <= kTrHaloSmemMax;
}

// variant 8 runs when every member has its layout, the tiles are at most 8 bins long (the
// halo-frame coordinates keep ~1e-7 of a bin) and a CTA's halo and code block fit
bool spmv_halo_fits(const Engine& e) {
  return e.halo_op && e.T <= 8 && smem_spmv_halo(e.halo_max, e.hcode_max16, e.hquad_max) <= 200 * 1024;
}

nnpp_status launch_warm_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st) {
  if (prec == NNPP_MIXED) {
    k_warm_dots<float><<<occ_grid(k_warm_dots<float>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v);
    k_warm_apply<float><<<occ_grid(k_warm_apply<float>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v);
  } else {
    k_warm_dots<double><<<occ_grid(k_warm_dots<double>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v);
    k_warm_apply<double><<<occ_grid(k_warm_apply<double>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v);
  }
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status launch_prep_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st,
                          cudaGraphConditionalHandle hc, double* F11_out) {
  if (prec == NNPP_MIXED && !F11_out) {
    k_phi4<<<occ_grid(k_phi4, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v);
    k_prep_slices<<<claim_grid(k_prep_slices, 0, e.sms, v.nslices), kBlock, 0, st>>>(v, hc);
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  }
  return dispatch_lanes(e.W, [&](auto wc) -> nnpp_status {
    constexpr int W = decltype(wc)::value;
    const size_t sh = smem_prep(v.halo_max, v.bond_max);
    if (prec == NNPP_MIXED)
      k_prep<float, W><<<occ_grid(k_prep<float, W>, sh, e.sms, v.ntiles), kBlock, sh, st>>>(v, hc, F11_out);
    else
      k_prep<double, W><<<occ_grid(k_prep<double, W>, sh, e.sms, v.ntiles), kBlock, sh, st>>>(v, hc, F11_out);
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  });
}

// largest row stride of the members' coarse inverses (shared memory of k_coarse_gemv)
int cld_max(const Engine& e) {
  int m = 4;
  for (const Handle* h : e.members) m = std::max(m, h->coarse.valid ? h->coarse.ld : 0);
  return m;
}

// z = M^-1 r with the two-level preconditioner: restriction, coarse solve, z and the dots
template <typename P>
nnpp_status launch_coarse_z(const Engine& e, const EngineView& v, cudaStream_t st, cudaGraphConditionalHandle hc,
                            int init) {
  int nmax = 1;
  for (const Handle* h : e.members) nmax = std::max(nmax, h->coarse.valid ? h->coarse.n : 0);
  const int which = init ? 0 : 1;
  const int rg = std::max(1, std::min((nmax * 32 + kBlock - 1) / kBlock, e.sms * 8));
  k_coarse_restrict<P><<<rg, kBlock, 0, st>>>(v, which);
  k_coarse_gemv<<<rg, kBlock, (size_t)cld_max(e) * sizeof(float), st>>>(v, which, 0, 0, 0);
  k_cg_zdots<P><<<occ_grid(k_cg_zdots<P>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v, hc, init,
                                                                               sizeof(P) == 8 ? 1 : 0);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

bool engine_coarse(const Engine& e) {
  for (const Handle* h : e.members)
    if (!h->coarse_enabled || !h->coarse.valid) return false;
  return !e.members.empty();
}

nnpp_status launch_cg_init_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st,
                             cudaGraphConditionalHandle hc) {
  const int split = engine_coarse(e) ? 1 : 0;
  if (prec == NNPP_MIXED)
    k_cg_init<float><<<occ_grid(k_cg_init<float>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v, split ? 0 : hc, 0, split);
  else
    k_cg_init<double><<<occ_grid(k_cg_init<double>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v, split ? 0 : hc, 1, split);
  NNPP_CUDA(cudaGetLastError());
  if (split) return prec == NNPP_MIXED ? launch_coarse_z<float>(e, v, st, hc, 1) : launch_coarse_z<double>(e, v, st, hc, 1);
  return NNPP_OK;
}

nnpp_status launch_cg_spmv_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st) {
  return dispatch_lanes(e.W, [&](auto wc) -> nnpp_status {
    constexpr int W = decltype(wc)::value;
    if (prec == NNPP_MIXED)
      if (e.spmv_variant == kSpmvHalo) {
        const size_t sh = smem_spmv_halo(e.halo_max, e.hcode_max16, e.hquad_max);
        const int qcap = (e.hquad_max + 1) & ~1;  // keeps the code block 16-byte aligned
        if (e.checks)
          k_cg_spmv32h<true><<<occ_grid(k_cg_spmv32h<true>, sh, e.sms, v.ntiles), kBlock, sh, st>>>(
              v, e.halo_max + 1, qcap);
        else
          k_cg_spmv32h<false><<<occ_grid(k_cg_spmv32h<false>, sh, e.sms, v.ntiles), kBlock, sh, st>>>(
              v, e.halo_max + 1, qcap);
      } else if (e.spmv_variant == 1 && e.members.size() == 1) {
        int stages = 2;
        const size_t sh = smem_spmv_stream(e.win_cap, &stages);
        k_cg_spmv32s<W, kStreamCol><<<occ_grid(k_cg_spmv32s<W, kStreamCol>, sh, e.sms, (v.nslices + 7) / 8), kBlock, sh, st>>>(
            v, stages, e.win_cap);
      } else if (e.spmv_variant == 1) {
        const size_t sh = smem_spmv_staged();
        k_cg_spmv32t<W><<<occ_grid(k_cg_spmv32t<W>, sh, e.sms, (v.nslices + 7) / 8), kBlock, sh, st>>>(v);
      } else {
        launch_spmv_gather<W>(e.spmv_variant, v, e.sms, st);
      }
    else
      { const size_t sh = smem_vec64(v.halo_max, v.bond_max); k_cg_spmv64<W><<<occ_grid(k_cg_spmv64<W>, sh, e.sms, v.ntiles), kBlock, sh, st>>>(v); }
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  });
}

// after the inner loop of a mixed solve: the deflated CG's final correction e = e^ + Q (r0 - t)
// (every kernel passes over instances that are not deflating)
nnpp_status launch_cg_final_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st) {
  if (prec != NNPP_MIXED || !engine_coarse(e) || e.members.size() != 1) return NNPP_OK;
  const int rg = std::max(1, std::min((cld_max(e) * 32 + kBlock - 1) / kBlock, e.sms * 8));
  const int cg = occ_grid(k_def_final, 0, e.sms, v.nchunks);
  k_def_final<<<cg, kBlock, 0, st>>>(v, 1);
  k_coarse_restrict<float><<<rg, kBlock, 0, st>>>(v, 2);
  k_coarse_gemv<<<rg, kBlock, (size_t)cld_max(e) * sizeof(float), st>>>(v, 2, 0, 0, 1);
  k_def_final<<<cg, kBlock, 0, st>>>(v, 2);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

// update fused with the restriction, coarse product, z and the dots
template <typename P>
nnpp_status launch_coarse_update(const Engine& e, const EngineView& v, cudaStream_t st, cudaGraphConditionalHandle hc) {
  int nmax = 1;
  for (const Handle* h : e.members) nmax = std::max(nmax, h->coarse.valid ? h->coarse.n : 0);
  const int rg = std::max(1, std::min((nmax * 32 + kBlock - 1) / kBlock, e.sms * 8));
  k_cg_update_restrict<P><<<rg, kBlock, 0, st>>>(v);
  if (e.members.size() == 1) {
    // one instance: the dots come from the aggregates, the decisions from the coarse product's
    // last CTA, and z is a plain elementwise pass
    k_coarse_gemv<<<rg, kBlock, (size_t)cld_max(e) * sizeof(float), st>>>(v, 1, hc, 1, sizeof(P) == 4 ? 1 : 0);
    k_z_form<P><<<occ_grid(k_z_form<P>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v, hc);
  } else {
    // ensembles: per-instance reductions in parallel (the last chunk of each instance)
    k_coarse_gemv<<<rg, kBlock, (size_t)cld_max(e) * sizeof(float), st>>>(v, 1, 0, 0, 0);
    k_cg_zdots<P><<<occ_grid(k_cg_zdots<P>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v, hc, 0, sizeof(P) == 8 ? 1 : 0);
  }
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

// one kernel of a single instance's split-iteration update (0 restriction and CG update,
// 1 coarse product, 2 z and the dots), for timing them one by one
nnpp_status launch_coarse_part_b(const Engine& e, const EngineView& v, int prec, int part, cudaStream_t st) {
  if (!engine_coarse(e) || e.members.size() != 1 || part < 0 || part > 2)
    return set_error(NNPP_ERR_INVALID, "time_kernel: the coarse update parts need one instance with a coarse space");
  const int n = std::max(1, e.members[0]->coarse.valid ? e.members[0]->coarse.n : 0);
  const int rg = std::max(1, std::min((n * 32 + kBlock - 1) / kBlock, e.sms * 8));
  const bool mixed = prec == NNPP_MIXED;
  if (part == 0) {
    if (mixed) k_cg_update_restrict<float><<<rg, kBlock, 0, st>>>(v);
    else k_cg_update_restrict<double><<<rg, kBlock, 0, st>>>(v);
  } else if (part == 1) {
    k_coarse_gemv<<<rg, kBlock, (size_t)cld_max(e) * sizeof(float), st>>>(v, 1, 0, 1, mixed ? 1 : 0);
  } else {
    if (mixed) k_z_form<float><<<occ_grid(k_z_form<float>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v, 0);
    else k_z_form<double><<<occ_grid(k_z_form<double>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v, 0);
  }
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status launch_cg_update_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st,
                               cudaGraphConditionalHandle hc) {
  if (engine_coarse(e))
    return prec == NNPP_MIXED ? launch_coarse_update<float>(e, v, st, hc) : launch_coarse_update<double>(e, v, st, hc);
  if (prec == NNPP_MIXED)
    k_cg_update<float><<<occ_grid(k_cg_update<float>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v, hc);
  else
    k_cg_update<double><<<occ_grid(k_cg_update<double>, 0, e.sms, v.nchunks), kBlock, 0, st>>>(v, hc);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status launch_ir_update_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st,
                               cudaGraphConditionalHandle hc) {
  if (prec == NNPP_MIXED) {
    k_ir_slices<<<claim_grid(k_ir_slices, 0, e.sms, v.ncslices), kBlock, 0, st>>>(v, hc);
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  }
  return dispatch_lanes(e.W, [&](auto wc) -> nnpp_status {
    constexpr int W = decltype(wc)::value;
    const size_t sh = smem_vec64(v.halo_max, v.bond_max);
    if (prec == NNPP_MIXED)
      k_ir_update<float, W><<<occ_grid(k_ir_update<float, W>, sh, e.sms, v.ntiles), kBlock, sh, st>>>(v, hc);
    else
      k_ir_update<double, W><<<occ_grid(k_ir_update<double, W>, sh, e.sms, v.ntiles), kBlock, sh, st>>>(v, hc);
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  });
}

// The halo-staged FP32 transport (form 1): batches of 8 bond columns, the next batch's codes
// and weights in flight.  Measured at 512k (bins per tile 4, ms a launch): 0.409, against
// 0.451 / 0.441 without the next batch in flight (batches of 8 / 16), 0.459 / 0.418 with it
// (16 / 4), 0.51-0.68 with tiles of 2 bins; the L1/L2 gathers of form 0 take 0.358.
void launch_transport_staged(const EngineView& v, int sms, cudaStream_t st) {
  const size_t sh = smem_tr_halo(v.halo_max);
  k_transport32h<8, true, 4><<<occ_grid_b(k_transport32h<8, true, 4>, kTrHBlock, sh, sms, v.ntiles), kTrHBlock, sh,
                               st>>>(v);
}

// CTAs of the next-guess pass (a step turns at most a few thousand nodes liquid)
constexpr int kFlipGuessCtas = 32;

nnpp_status launch_transport_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st,
                               double* F_out) {
  return dispatch_lanes(e.W, [&](auto wc) -> nnpp_status {
    constexpr int W = decltype(wc)::value;
    if (prec == NNPP_MIXED) {
      if (F_out)
        k_transport32<W, true><<<slice_grid(k_transport32<W, true>, 0, e.sms, v.nslices), kBlock, 0, st>>>(v, F_out);
      else {
        if (e.tr_variant > 0 && transport_halo_fits(e)) {
          launch_transport_staged(v, e.sms, st);
        } else {
          k_transport32<W, false><<<claim_grid(k_transport32<W, false>, 0, e.sms, v.nslices), kBlock, 0, st>>>(v, nullptr);
        }
        k_flip_guess<float><<<kFlipGuessCtas, kBlock, 0, st>>>(v);
      }
    } else {
      const size_t sh = smem_tr64(v.halo_max, v.bond_max);
      if (F_out)
        k_transport64<W, true><<<occ_grid(k_transport64<W, true>, sh, e.sms, v.ntiles), kBlock, sh, st>>>(v, F_out);
      else {
        k_transport64<W, false><<<occ_grid(k_transport64<W, false>, sh, e.sms, v.ntiles), kBlock, sh, st>>>(v, nullptr);
        k_flip_guess<double><<<kFlipGuessCtas, kBlock, 0, st>>>(v);
      }
    }
    NNPP_CUDA(cudaGetLastError());
    return NNPP_OK;
  });
}

// ---------------------------------------------------------------------------------------
nnpp_status step_alloc(Handle& h) {
  const size_t N = (size_t)h.N;
  bool ok = h.dirmask.alloc(N) && h.bcval.alloc((S + 1) * N) && h.rec32[0].alloc(N) &&
            h.rec32[1].alloc(N) && h.clo.alloc(N) && h.rec64[0].alloc(N) && h.rec64[1].alloc(N) &&
            h.phi64.alloc(N) && h.phi_prev.alloc(N) && h.flip_step.alloc(N) && h.flip_list.alloc(N) &&
            h.b64.alloc(N) &&
            h.r64.alloc(N) && h.dsum64.alloc(N) && h.cpl64.alloc(N) && h.dinv64.alloc(N) && h.rin64.alloc(N) &&
            h.z64.alloc(N) && h.p64.alloc(N) && h.q64.alloc(N) && h.e64.alloc(N) && h.d32.alloc(N) &&
            h.dinv32.alloc(N) && h.rin32.alloc(N) && h.z32.alloc(N + 16) && h.p32.alloc(N) &&
            h.q32.alloc(N) && h.e32.alloc(N) && h.r0_32.alloc(N) && h.t32.alloc(N) && h.freem.alloc(N) &&
            h.phi4.alloc(N) && h.dstate.alloc(1) &&
            h.scratch_d.alloc(16 + 7 * 4096) && h.user_stage.alloc((S + 1) * N) &&
            h.user_stage_i.alloc(N);
  if (ok && h.warm_hist >= 3) ok = h.xh.alloc((size_t)h.warm_hist * N) && h.bh.alloc((size_t)h.warm_hist * N);
  if (!ok) return set_error(NNPP_ERR_NOMEM, "device state allocation");
  NNPP_CUDA(cudaMemsetAsync(h.freem.get(), 0, N, h.st));
  NNPP_CUDA(cudaMemsetAsync(h.rec32[1].get(), 0, N * sizeof(Rec32), h.st));
  NNPP_CUDA(cudaMemsetAsync(h.rec64[1].get(), 0, N * sizeof(Rec64), h.st));
  NNPP_CUDA(cudaMemsetAsync(h.e32.get(), 0, N * sizeof(float), h.st));
  NNPP_CUDA(cudaMemsetAsync(h.e64.get(), 0, N * sizeof(double), h.st));
  // z32 is padded by 16 (read, never used) elements: window copies round their rows up to 4
  NNPP_CUDA(cudaMemsetAsync(h.z32.get(), 0, (N + 16) * sizeof(float), h.st));
  NNPP_CUDA(cudaMemsetAsync(h.z64.get(), 0, N * sizeof(double), h.st));
  NNPP_CUDA(cudaMemsetAsync(h.flip_step.get(), 0xff, N * sizeof(int), h.st));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h.device);
  if (sms <= 0) sms = 152;
  long long g = std::min<long long>(((long long)h.N + 255) / 256, (long long)sms * 8);
  if (g > 4096) g = 4096;
  if (g < 1) g = 1;
  h.grid = (int)g;
  return NNPP_OK;
}

KParams make_kparams(Handle& h, int cur) {
  KParams k;
  std::memset(&k, 0, sizeof(k));
  const nnpp_params& p = h.p;
  k.N = h.N;
  k.row = h.lay.row.get();
  k.col = h.lay.col.get();
  k.slot16 = h.slot16.get();
  k.sell = h.sell.get();
  k.sell_lo = h.sell_lo.get();
  k.sell_cg = h.sell_cg.get();
  k.sell_cg_lo = h.sell_cg_lo.get();
  k.cg_width = h.cg_width.get();
  k.cg_rows = h.cg_rows.get();
  k.cg_pos = h.cg_pos.get();
  k.xrow = h.xrow.get();
  k.phi4 = h.phi4.get();
  k.w64 = h.lay.w64.get();
  k.w32 = h.lay.w32.get();
  k.wlo32 = h.lay.wlo32.get();
  k.dirmask = h.dirmask.get();
  k.bcval = h.bcval.get();
  k.rec32_cur = h.rec32[cur].get();
  k.rec32_nxt = h.rec32[cur ^ 1].get();
  k.clo = h.clo.get();
  k.rec64_cur = h.rec64[cur].get();
  k.rec64_nxt = h.rec64[cur ^ 1].get();
  k.phi64 = h.phi64.get();
  k.phi_prev = h.phi_prev.get();
  k.phi_keep = h.phi_keep[cur & 1];
  k.flip_step = h.flip_step.get();
  k.flip_list = h.flip_list.get();
  k.b64 = h.b64.get();
  k.r64 = h.r64.get();
  k.dsum64 = h.dsum64.get();
  k.cpl64 = h.cpl64.get();
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
  k.ds = h.dstate.get();
  k.bv_ptr = &h.dstate.get()->BV;
  k.b_override = h.b_override;
  // halo-staged CG operator: weights in units of the bin side hb (FP32 of the bins' side)
  k.hquad = h.hquad.get();
  k.hquad_n = (int)h.hquad.size();
  k.checks = h.checks;
  k.hcode = h.hcode.get();
  k.posrec = h.posrec.get();
  {
    const double hb = (double)h.h32;
    k.hinv = (float)(1.0 / hb);
    k.hc0 = (float)((p.delta + 0.5 * p.dx) / p.dx);
    k.hc1 = (float)(hb / p.dx);
    k.hsw = (float)(p.dx * p.dy * p.dz / (hb * hb * hb));
  }
  k.dt = p.dt;
  k.csat = p.CSat / p.CSolid;
  k.c_floor = p.c_floor;
  k.csat_hi = (float)k.csat;
  k.csat_lo = (float)(k.csat - (double)k.csat_hi);
  k.cfl_hi = (float)k.c_floor;
  k.cfl_lo = (float)(k.c_floor - (double)k.cfl_hi);
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
  k.extrapolate = h.extrapolate;
  k.hist_m = (h.extrapolate && h.warm_hist >= 3 && h.xh.get()) ? h.warm_hist : 0;
  k.xh = h.warm_x_alt ? h.warm_x_alt : h.xh.get();
  k.bh = h.warm_b_alt ? h.warm_b_alt : h.bh.get();
  const Coarse& co = h.coarse;
  k.coarse = (h.coarse_enabled && co.valid) ? 1 : 0;
  k.defl_ok = 0;  // set by the engine for single-instance runs
  k.agg = co.agg.get();
  k.cinv = co.inv.get();
  k.rc = const_cast<float*>(co.rc.get());
  k.xc = const_cast<float*>(co.xc.get());
  k.bin_start = h.lay.bin_start.get();
  k.cn = co.n;
  k.cld = co.ld;
  k.cdots = co.dots.get();
  k.ap_k = co.ap_k;
  k.ap_col = co.ap_col.get();
  k.ap_val = co.ap_val.get();
  k.r0_32 = h.r0_32.get();
  k.t32 = h.t32.get();
  k.cf = co.f;
  k.cna0 = co.na[0];
  k.cna1 = co.na[1];
  k.cna2 = co.na[2];
  k.nb0 = h.lay.nb[0];
  k.nb1 = h.lay.nb[1];
  k.nb2 = h.lay.nb[2];
  return k;
}

nnpp_status load_state(Handle& h, const double* d_c_user, const double* d_phi_user,
                       const int* d_phase_user, int prec, bool dirichlet_phi,
                       bool keep_history) {
  // the cached operator arrays stay valid for the same phases, precision and Dirichlet
  // potentials (a changed phase is detected by the kernel)
  if (prec != h.state_prec || !dirichlet_phi) NNPP_TRY(invalidate_operator(h));
  KParams kp = make_kparams(h, h.cur);
  k_load_state<<<h.grid, kBlock, 0, h.st>>>(kp, h.lay.perm.get(), d_c_user, d_phi_user, d_phase_user,
                                            prec == NNPP_MIXED ? 1 : 0, dirichlet_phi ? 1 : 0,
                                            keep_history ? 1 : 0);
  NNPP_CUDA(cudaGetLastError());
  h.state_prec = prec;
  return NNPP_OK;
}

nnpp_status invalidate_operator(Handle& h) {
  NNPP_CUDA(cudaMemsetAsync(&h.dstate.get()->op_valid, 0, sizeof(int), h.st));
  return NNPP_OK;
}

nnpp_status store_state(Handle& h, double* d_c_user, double* d_phi_user, int* d_phase_user) {
  KParams kp = make_kparams(h, h.cur);
  k_store_state<<<h.grid, kBlock, 0, h.st>>>(kp, h.lay.perm.get(), d_c_user, d_phi_user, d_phase_user,
                                             h.state_prec == NNPP_MIXED ? 1 : 0);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status convert_state(Handle& h, int to_prec) {
  if (h.state_prec == to_prec) return NNPP_OK;
  KParams kp = make_kparams(h, h.cur);
  k_convert<<<h.grid, kBlock, 0, h.st>>>(kp, to_prec == NNPP_MIXED ? 1 : 0);
  NNPP_CUDA(cudaGetLastError());
  h.state_prec = to_prec;
  // the two precisions form the diagonal with different arithmetic
  return invalidate_operator(h);
}

nnpp_status init_diag(Handle& h, bool restart) {
  KParams kp = make_kparams(h, h.cur);
  k_init_diag<<<h.grid, kBlock, 0, h.st>>>(kp, h.state_prec == NNPP_MIXED ? 1 : 0,
                                           h.scratch_d.get() + 16, restart ? 1 : 0);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

}  // namespace nnpp
