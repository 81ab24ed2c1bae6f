// neighbours.cu -- GPU neighbour build that reproduces build_clouds_hash (grid.h:43-204),
// and the bin-sorted internal layout the step kernels run on.
//
// Exactness: the hash (grid.h:81-85), the cell corners (grid.h:137-139), the sphere-cube
// test (grid.h:27-41) and the horizon test (grid.h:186) are evaluated with explicitly
// rounded FP64 intrinsics (__dsub_rn, __dmul_rn, __dadd_rn, __ddiv_rn), which nvcc never
// contracts into FMAs, so every decision equals the host's ISO C++ evaluation.
#include <algorithm>
#include <climits>
#include <cmath>
#include <utility>
#include <vector>

#include "neighbours.cuh"

namespace nnpp {

namespace {

constexpr int kScanBlock = 1024;

template <typename T>
__global__ void k_scan_block(const T* in, T* out, T* block_sums, int n) {
  __shared__ T warp_tot[32];
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const T v = i < n ? in[i] : T(0);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    T t = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;
  }
  __syncthreads();
  const T excl = x - v + (w > 0 ? warp_tot[w - 1] : T(0));
  if (i < n) out[i] = excl;
  if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = excl + v;
}

template <typename T>
__global__ void k_scan_add(T* out, const T* offs, int n) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) out[i] += offs[blockIdx.x];
}

template <typename T>
__global__ void k_scan_tail(const T* in, T* out, int n) {
  out[n] = (n > 0) ? out[n - 1] + in[n - 1] : T(0);
}

// exclusive scan of n values (T) into out[0..n]
template <typename T>
nnpp_status scan_impl(cudaStream_t st, const T* in, T* out, int n) {
  if (n <= 0) {
    NNPP_CUDA(cudaMemsetAsync(out, 0, sizeof(T), st));
    return NNPP_OK;
  }
  const int nb = (n + kScanBlock - 1) / kScanBlock;
  DBuf<T> sums, sums_scan;
  if (!sums.alloc(nb) || !sums_scan.alloc(nb + 1)) return set_error(NNPP_ERR_NOMEM, "scan scratch");
  k_scan_block<T><<<nb, kScanBlock, 0, st>>>(in, out, sums.get(), n);
  if (nb > 1) {
    NNPP_TRY(scan_impl<T>(st, sums.get(), sums_scan.get(), nb));
    k_scan_add<T><<<nb, kScanBlock, 0, st>>>(out, sums_scan.get(), n);
  }
  k_scan_tail<T><<<1, 1, 0, st>>>(in, out, n);
  NNPP_CUDA(cudaGetLastError());
  // the scratch buffers are freed on return; make sure the kernels using them are done
  NNPP_CUDA(cudaStreamSynchronize(st));
  return NNPP_OK;
}

// ---------------------------------------------------------------- bounding box ----------
__global__ void k_bbox_partial(const double* x, const double* y, const double* z, int n,
                               double* part) {
  double mn[3] = {x[0], y[0], z[0]}, mx[3] = {x[0], y[0], z[0]};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v[3] = {x[i], y[i], z[i]};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      mn[d] = v[d] < mn[d] ? v[d] : mn[d];
      mx[d] = v[d] > mx[d] ? v[d] : mx[d];
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double a = __shfl_down_sync(0xffffffffu, mn[d], o);
      double b = __shfl_down_sync(0xffffffffu, mx[d], o);
      mn[d] = a < mn[d] ? a : mn[d];
      mx[d] = b > mx[d] ? b : mx[d];
    }
  __shared__ double sm[6][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0)
    for (int d = 0; d < 3; ++d) {
      sm[2 * d][w] = mn[d];
      sm[2 * d + 1][w] = mx[d];
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int d = 0; d < 3; ++d) {
      double a = sm[2 * d][0], b = sm[2 * d + 1][0];
      for (int k = 1; k < nw; ++k) {
        a = sm[2 * d][k] < a ? sm[2 * d][k] : a;
        b = sm[2 * d + 1][k] > b ? sm[2 * d + 1][k] : b;
      }
      part[blockIdx.x * 6 + 2 * d] = a;
      part[blockIdx.x * 6 + 2 * d + 1] = b;
    }
  }
}

__global__ void k_bbox_final(const double* part, int nblk, double* out) {
  if (threadIdx.x != 0) return;
  double r[6];
  for (int k = 0; k < 6; ++k) r[k] = part[k];
  for (int b = 1; b < nblk; ++b)
    for (int d = 0; d < 3; ++d) {
      double a = part[b * 6 + 2 * d], c = part[b * 6 + 2 * d + 1];
      r[2 * d] = a < r[2 * d] ? a : r[2 * d];
      r[2 * d + 1] = c > r[2 * d + 1] ? c : r[2 * d + 1];
    }
  for (int k = 0; k < 6; ++k) out[k] = r[k];
}

nnpp_status bbox_gpu(cudaStream_t st, const double* x, const double* y, const double* z, int n,
                     double* host6) {
  const int nblk = 128;
  DBuf<double> part, res;
  if (!part.alloc(nblk * 6) || !res.alloc(6)) return set_error(NNPP_ERR_NOMEM, "bbox scratch");
  k_bbox_partial<<<nblk, 256, 0, st>>>(x, y, z, n, part.get());
  k_bbox_final<<<1, 32, 0, st>>>(part.get(), nblk, res.get());
  NNPP_CUDA(cudaGetLastError());
  NNPP_CUDA(cudaMemcpyAsync(host6, res.get(), 6 * sizeof(double), cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  return NNPP_OK;
}

// ---------------------------------------------------------------- hashing ---------------
// grid.h:81-85: hash = (int)((x-x0)/dx) + mx*(int)((y-y0)/dy) + mx*my*(int)((z-z0)/dz)
__global__ void k_hash(const double* x, const double* y, const double* z, int n, double x0,
                       double y0, double z0, double cx, double cy, double cz, int mx, int my,
                       int* h, int* maxh) {
  int local_max = -1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int ix = (int)__ddiv_rn(__dsub_rn(x[i], x0), cx);
    const int iy = (int)__ddiv_rn(__dsub_rn(y[i], y0), cy);
    const int iz = (int)__ddiv_rn(__dsub_rn(z[i], z0), cz);
    const int v = ix + mx * iy + mx * my * iz;
    h[i] = v;
    local_max = v > local_max ? v : local_max;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    int b = __shfl_down_sync(0xffffffffu, local_max, o);
    local_max = b > local_max ? b : local_max;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(maxh, local_max);
}

__global__ void k_count(const int* key, int n, int* count) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    atomicAdd(&count[key[i]], 1);
}

__global__ void k_scatter(const int* key, int n, int* cursor, int* order) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int pos = atomicAdd(&cursor[key[i]], 1);
    order[pos] = i;
  }
}

// Sort every segment [seg[s], seg[s+1]) of `in` ascending into `out` (values distinct
// within a segment) by rank counting; one block per segment, 4 values per thread per
// chunk.  O(L^2 / blockDim) per segment, used for bins, cells and neighbour rows.
__global__ void k_sort_segments(const int* seg, int nseg, const int* in, int* out) {
  for (int s = blockIdx.x; s < nseg; s += gridDim.x) {
    const int b = seg[s];
    const int L = seg[s + 1] - b;
    for (int chunk = 0; chunk < L; chunk += 4 * blockDim.x) {
      int v[4], rank[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int t = chunk + threadIdx.x + e * blockDim.x;
        v[e] = t < L ? in[b + t] : INT_MAX;
        rank[e] = 0;
      }
      for (int u = 0; u < L; ++u) {
        const int vu = in[b + u];
#pragma unroll
        for (int e = 0; e < 4; ++e) rank[e] += (vu < v[e]) ? 1 : 0;
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int t = chunk + threadIdx.x + e * blockDim.x;
        if (t < L) out[b + rank[e]] = v[e];
      }
    }
  }
}

// ---------------------------------------------------------------- cell scan -------------
__device__ __forceinline__ double sqr_rn(double a) { return __dmul_rn(a, a); }

// grid.h:27-41 with the corner of grid.h:137-139
__device__ __forceinline__ bool sphere_cube_rn(double px, double py, double pz, double r2,
                                               double bx, double by, double bz, double w,
                                               double hh, double d) {
  const double bmin[3] = {bx, by, bz};
  const double bmax[3] = {__dadd_rn(bx, w), __dadd_rn(by, hh), __dadd_rn(bz, d)};
  const double c[3] = {px, py, pz};
  double dmin = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (c[i] < bmin[i])
      dmin = __dadd_rn(dmin, sqr_rn(__dsub_rn(c[i], bmin[i])));
    else if (c[i] > bmax[i])
      dmin = __dadd_rn(dmin, sqr_rn(__dsub_rn(c[i], bmax[i])));
  }
  return dmin <= r2;
}

// Warp per node.  Visits the cells within one cell of the sphere's bounding box in
// ascending hash order, keeps those that pass the reference's sphere-cube test, and
// appends the members of each (in the sorted order) that pass the horizon test, so the
// list equals the reference's scan over all cells (grid.h:157-196).  Pass FILL=false
// counts (lengths without self), FILL=true writes the CSR columns.
template <bool FILL>
__global__ void k_cell_scan(int n, const double* __restrict__ x, const double* __restrict__ y,
                            const double* __restrict__ z, double x0, double y0, double z0,
                            double cx, double cy, double cz, int mx, int my, int max_hash,
                            double r, const int* __restrict__ start,
                            const int* __restrict__ order, int max_node_no, int* len,
                            const int* __restrict__ row_ptr, int* cols, int* err) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const double r2 = __dmul_rn(r, r);
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const double px = x[i], py = y[i], pz = z[i];
    int lo[3], hi[3];
    const double q[3] = {px, py, pz}, o[3] = {x0, y0, z0}, w[3] = {cx, cy, cz};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      lo[d] = (int)floor((q[d] - r - o[d]) / w[d]) - 1;
      hi[d] = (int)floor((q[d] + r - o[d]) / w[d]) + 1;
      if (lo[d] < 0) lo[d] = 0;
    }
    if (hi[0] > mx - 1) hi[0] = mx - 1;
    if (hi[1] > my - 1) hi[1] = my - 1;
    int fill = 0;
    const int rbase = FILL ? row_ptr[i] : 0;
    const int cap = max_node_no - 1;
    for (int kz = lo[2]; kz <= hi[2]; ++kz) {
      const int mzo = mx * my * kz;
      if (mzo >= max_hash) break;
      for (int ky = lo[1]; ky <= hi[1]; ++ky)
        for (int kx = lo[0]; kx <= hi[0]; ++kx) {
          const int m = kx + mx * ky + mzo;
          if (m >= max_hash) continue;
          const double bx = __dadd_rn(x0, __dmul_rn((double)kx, cx));
          const double by = __dadd_rn(y0, __dmul_rn((double)ky, cy));
          const double bz = __dadd_rn(z0, __dmul_rn((double)kz, cz));
          if (!sphere_cube_rn(px, py, pz, r2, bx, by, bz, cx, cy, cz)) continue;
          const int s = start[m], e = start[m + 1];
          for (int base = s; base < e; base += 32) {
            const int k = base + lane;
            bool pass = false;
            int cand = -1;
            if (k < e) {
              cand = order[k];
              const double d2 = __dadd_rn(__dadd_rn(sqr_rn(__dsub_rn(px, x[cand])),
                                                    sqr_rn(__dsub_rn(py, y[cand]))),
                                          sqr_rn(__dsub_rn(pz, z[cand])));
              pass = (d2 <= r2) && (cand != i);
            }
            const unsigned int bal = __ballot_sync(0xffffffffu, pass);
            if (FILL && pass) {
              const int pos = fill + __popc(bal & ((1u << lane) - 1u));
              if (pos < cap) cols[rbase + pos] = cand;
            }
            fill += __popc(bal);
          }
        }
    }
    if (!FILL && lane == 0) {
      len[i] = fill;
      if (fill + 1 > max_node_no) atomicExch(err, 1);
    }
  }
}

// Variant of k_cell_scan for the allocation-free build: one pass that writes the padded
// column-major output directly (self at column 0, grid.h:170-171), the lengths (self
// included) and the running maximum length; raises the capacity flag where grid.h:187-189
// throws.
__global__ void k_cell_scan_padded(int n, const double* __restrict__ x, const double* __restrict__ y,
                                   const double* __restrict__ z, double x0, double y0, double z0,
                                   double cx, double cy, double cz, int mx, int my, int max_hash,
                                   double r, const int* __restrict__ start,
                                   const int* __restrict__ order, int max_node_no, int* clouds,
                                   int* lengths, int* misc) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const double r2 = __dmul_rn(r, r);
  for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const double px = x[i], py = y[i], pz = z[i];
    int lo[3], hi[3];
    const double q[3] = {px, py, pz}, o[3] = {x0, y0, z0}, w[3] = {cx, cy, cz};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      lo[d] = (int)floor((q[d] - r - o[d]) / w[d]) - 1;
      hi[d] = (int)floor((q[d] + r - o[d]) / w[d]) + 1;
      if (lo[d] < 0) lo[d] = 0;
    }
    if (hi[0] > mx - 1) hi[0] = mx - 1;
    if (hi[1] > my - 1) hi[1] = my - 1;
    int fill = 0;
    const int cap = max_node_no - 1;
    for (int kz = lo[2]; kz <= hi[2]; ++kz) {
      const int mzo = mx * my * kz;
      if (mzo >= max_hash) break;
      for (int ky = lo[1]; ky <= hi[1]; ++ky)
        for (int kx = lo[0]; kx <= hi[0]; ++kx) {
          const int m = kx + mx * ky + mzo;
          if (m >= max_hash) continue;
          const double bx = __dadd_rn(x0, __dmul_rn((double)kx, cx));
          const double by = __dadd_rn(y0, __dmul_rn((double)ky, cy));
          const double bz = __dadd_rn(z0, __dmul_rn((double)kz, cz));
          if (!sphere_cube_rn(px, py, pz, r2, bx, by, bz, cx, cy, cz)) continue;
          const int s = start[m], e = start[m + 1];
          for (int base = s; base < e; base += 32) {
            const int k = base + lane;
            bool pass = false;
            int cand = -1;
            if (k < e) {
              cand = order[k];
              const double d2 = __dadd_rn(__dadd_rn(sqr_rn(__dsub_rn(px, x[cand])),
                                                    sqr_rn(__dsub_rn(py, y[cand]))),
                                          sqr_rn(__dsub_rn(pz, z[cand])));
              pass = (d2 <= r2) && (cand != i);
            }
            const unsigned int bal = __ballot_sync(0xffffffffu, pass);
            if (pass) {
              const int pos = fill + __popc(bal & ((1u << lane) - 1u));
              if (pos < cap) clouds[(int64_t)(pos + 1) * n + i] = cand;
            }
            fill += __popc(bal);
          }
        }
    }
    if (lane == 0) {
      clouds[i] = i;
      lengths[i] = fill + 1 <= max_node_no ? fill + 1 : max_node_no;
      if (fill + 1 > max_node_no) atomicExch(&misc[1], 1);
      atomicMax(&misc[2], fill + 1);
    }
  }
}

__global__ void k_max_int(const int* v, int n, int* out) {
  int m = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    m = v[i] > m ? v[i] : m;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    int b = __shfl_down_sync(0xffffffffu, m, o);
    m = b > m ? b : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

__global__ void k_emit_padded(int n, const int* ptr, const int* col, int* clouds) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    clouds[i] = i;
    const int b = ptr[i], e = ptr[i + 1];
    for (int t = b; t < e; ++t) clouds[(int64_t)(t - b + 1) * n + i] = col[t];
  }
}

// ---------------------------------------------------------------- layout ----------------
__global__ void k_bin_of(const double* x, const double* y, const double* z, int n, double ox,
                         double oy, double oz, double hb, int nbx, int nby, int nbz, int* bin) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int bx = (int)((x[i] - ox) / hb), by = (int)((y[i] - oy) / hb), bz = (int)((z[i] - oz) / hb);
    bx = min(max(bx, 0), nbx - 1);
    by = min(max(by, 0), nby - 1);
    bz = min(max(bz, 0), nbz - 1);
    bin[i] = bx + nbx * (by + nby * bz);
  }
}

__global__ void k_invert(const int* perm, int n, int* iperm) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x)
    iperm[perm[a]] = a;
}

__global__ void k_gather_len(const int* perm, const int* ref_ptr, int n, int* len) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
    const int u = perm[a];
    len[a] = ref_ptr[u + 1] - ref_ptr[u];
  }
}

__global__ void k_fill_internal(const int* perm, const int* iperm, const int* ref_ptr,
                                const int* ref_col, const int* row, int n, int* col) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < n; a += warps) {
    const int u = perm[a];
    const int b = ref_ptr[u], L = ref_ptr[u + 1] - b, o = row[a];
    for (int t = lane; t < L; t += 32) col[o + t] = iperm[ref_col[b + t]];
  }
}

__global__ void k_gather_pos(const int* perm, const double* x, const double* y, const double* z,
                             int n, double* pos) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
    const int u = perm[a];
    pos[a] = x[u];
    pos[n + a] = y[u];
    pos[2 * n + a] = z[u];
  }
}

// w = beta(xi) dV / xi^(3+2s), FP64; same expression as the reference's bond terms
// (utils.h:122-124) without the K D factors.
__global__ void k_weights(int n, const int* row, const int* col, const double* pos, double delta,
                          double dx, double dV, double s_exp, double* w64, float* w32, float* wlo32) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const double ex = 3.0 + 2.0 * s_exp;
  for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < n; a += warps) {
    const double xa = pos[a], ya = pos[n + a], za = pos[2 * n + a];
    for (int j = row[a] + lane; j < row[a + 1]; j += 32) {
      const int b = col[j];
      const double dxv = pos[b] - xa, dyv = pos[n + b] - ya, dzv = pos[2 * n + b] - za;
      const double xi = sqrt(dxv * dxv + dyv * dyv + dzv * dzv);
      const double w = beta_fn<double>(xi, delta, dx) * dV / (s_exp == 0.0 ? xi * xi * xi : pow(xi, ex));
      w64[j] = w;
      w32[j] = (float)w;
      wlo32[j] = (float)(w - (double)w32[j]);  // w = w32 + wlo32 to ~2^-48
    }
  }
}

// The hash of grid.h:81-85 is an int; mx, my come from static_cast<int> of a double
// (grid.h:75-78).  A wide bounding box with small cells overflows both, after which
// wrapped hashes would index the cell arrays out of bounds.  The cell counts per axis are
// therefore formed in double first; the grid must hold at most `limit` cells (the int
// range for the allocating build, the scratch size for the allocation-free one).  A NaN
// extent (non-finite coordinates) fails the test as well.
nnpp_status check_hash_grid(const double bb[6], double cx, double cy, double cz, double limit) {
  const double ncx = std::floor((bb[1] - bb[0]) / cx) + 1.0;
  const double ncy = std::floor((bb[3] - bb[2]) / cy) + 1.0;
  const double ncz = std::floor((bb[5] - bb[4]) / cz) + 1.0;
  const double cells = ncx * ncy * ncz;
  if (!(cells <= limit))
    return set_error(NNPP_ERR_INVALID,
                     "build: hash grid of the bounding box has too many cells (cell sizes too "
                     "small for the node extent, or non-finite coordinates)");
  return NNPP_OK;
}

int grid_for(long long n, int block, int cap = 152 * 16) {
  long long g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

}  // namespace

nnpp_status scan_ints(cudaStream_t st, const int* in, int* out, int n, long long* total) {
  NNPP_TRY(scan_impl<int>(st, in, out, n));
  if (total) {
    int t = 0;
    NNPP_CUDA(cudaMemcpyAsync(&t, out + n, sizeof(int), cudaMemcpyDeviceToHost, st));
    NNPP_CUDA(cudaStreamSynchronize(st));
    *total = t;
  }
  return NNPP_OK;
}

// counting sort of keys in [0, nkeys): start[nkeys+1], order[n] with members of each key in
// ascending index order
static nnpp_status counting_sort(cudaStream_t st, const int* key, int n, int nkeys, DBuf<int>& start,
                                 DBuf<int>& order) {
  DBuf<int> count, cursor, tmp;
  if (!count.alloc(nkeys) || !start.alloc(nkeys + 1) || !cursor.alloc(nkeys + 1) ||
      !order.alloc(n) || !tmp.alloc(n))
    return set_error(NNPP_ERR_NOMEM, "counting sort buffers");
  NNPP_CUDA(cudaMemsetAsync(count.get(), 0, sizeof(int) * nkeys, st));
  k_count<<<grid_for(n, 256), 256, 0, st>>>(key, n, count.get());
  NNPP_TRY(scan_ints(st, count.get(), start.get(), nkeys, nullptr));
  NNPP_CUDA(cudaMemcpyAsync(cursor.get(), start.get(), sizeof(int) * (nkeys + 1),
                            cudaMemcpyDeviceToDevice, st));
  k_scatter<<<grid_for(n, 256), 256, 0, st>>>(key, n, cursor.get(), tmp.get());
  k_sort_segments<<<grid_for(nkeys, 1, 65535), 128, 0, st>>>(start.get(), nkeys, tmp.get(),
                                                             order.get());
  NNPP_CUDA(cudaGetLastError());
  NNPP_CUDA(cudaStreamSynchronize(st));
  return NNPP_OK;
}

nnpp_status build_ref_lists(cudaStream_t st, int N, const double* x, const double* y,
                            const double* z, int max_node_no, double r, double cx, double cy,
                            double cz, int order_mode, RefLists& out) {
  if (N <= 0) return set_error(NNPP_ERR_INVALID, "build: no nodes");
  if (!(r > 0.0) || !(cx > 0.0) || !(cy > 0.0) || !(cz > 0.0) || max_node_no < 1)
    return set_error(NNPP_ERR_INVALID, "build: r, cell sizes and max_node_no must be positive");
  if (order_mode != NNPP_ORDER_REFERENCE && order_mode != NNPP_ORDER_CANONICAL)
    return set_error(NNPP_ERR_INVALID, "build: unknown order mode");
  out.N = N;
  // Step 0 (grid.h:49-71)
  NNPP_TRY(bbox_gpu(st, x, y, z, N, out.bbox));
  const double x0 = out.bbox[0], x1 = out.bbox[1], y0 = out.bbox[2], y1 = out.bbox[3],
               z0 = out.bbox[4];
  NNPP_TRY(check_hash_grid(out.bbox, cx, cy, cz, (double)INT_MAX));
  // Step 1 (grid.h:75-86); multipliers computed on the host as in the reference
  const int mx = static_cast<int>((x1 - x0) / cx) + 1;
  const int my = static_cast<int>((y1 - y0) / cy) + 1;
  DBuf<int> hash, dmax;
  if (!hash.alloc(N) || !dmax.alloc(1)) return set_error(NNPP_ERR_NOMEM, "hash buffers");
  NNPP_CUDA(cudaMemsetAsync(dmax.get(), 0xff, sizeof(int), st));
  k_hash<<<grid_for(N, 256), 256, 0, st>>>(x, y, z, N, x0, y0, z0, cx, cy, cz, mx, my,
                                           hash.get(), dmax.get());
  NNPP_CUDA(cudaGetLastError());
  int hmax = -1;
  NNPP_CUDA(cudaMemcpyAsync(&hmax, dmax.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  if (hmax < 0) return set_error(NNPP_ERR_INVALID, "build: negative hash (non-finite coordinates?)");
  const int max_hash = hmax + 1;  // grid.h:94
  // Steps 2-3 (grid.h:88-124): order of the nodes by cell and the cell index
  DBuf<int> start, order;
  if (order_mode == NNPP_ORDER_CANONICAL) {
    NNPP_TRY(counting_sort(st, hash.get(), N, max_hash, start, order));
  } else {
    // The reference's within-cell order is the permutation that std::sort (unstable
    // introsort) leaves for (index, hash) pairs compared by hash only (grid.h:90).  The
    // same library call on the same input is made here; every other step runs on the GPU.
    std::vector<int> hh(N);
    NNPP_CUDA(cudaMemcpyAsync(hh.data(), hash.get(), sizeof(int) * N, cudaMemcpyDeviceToHost, st));
    NNPP_CUDA(cudaStreamSynchronize(st));
    std::vector<std::pair<int, int> > pairs(N);
    for (int i = 0; i < N; ++i) pairs[i] = std::make_pair(i, hh[i]);
    std::sort(pairs.begin(), pairs.end(),
              [](const std::pair<int, int>& a, const std::pair<int, int>& b) { return a.second < b.second; });
    std::vector<int> ord(N);
    for (int k = 0; k < N; ++k) ord[k] = pairs[k].first;
    DBuf<int> count;
    if (!count.alloc(max_hash) || !start.alloc(max_hash + 1) || !order.alloc(N))
      return set_error(NNPP_ERR_NOMEM, "cell index buffers");
    NNPP_CUDA(cudaMemcpyAsync(order.get(), ord.data(), sizeof(int) * N, cudaMemcpyHostToDevice, st));
    NNPP_CUDA(cudaMemsetAsync(count.get(), 0, sizeof(int) * max_hash, st));
    k_count<<<grid_for(N, 256), 256, 0, st>>>(hash.get(), N, count.get());
    NNPP_TRY(scan_ints(st, count.get(), start.get(), max_hash, nullptr));
  }
  // Step 5 (grid.h:143-196): count, then fill
  DBuf<int> len, err;
  if (!len.alloc(N) || !err.alloc(1) || !out.ptr.alloc(N + 1))
    return set_error(NNPP_ERR_NOMEM, "scan buffers");
  NNPP_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(int), st));
  const int warps_grid = grid_for((long long)N * 32, 256, 152 * 64);
  k_cell_scan<false><<<warps_grid, 256, 0, st>>>(N, x, y, z, x0, y0, z0, cx, cy, cz, mx, my,
                                                 max_hash, r, start.get(), order.get(),
                                                 max_node_no, len.get(), nullptr, nullptr,
                                                 err.get());
  NNPP_CUDA(cudaGetLastError());
  int herr = 0;
  NNPP_CUDA(cudaMemcpyAsync(&herr, err.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  if (herr)
    return set_error(NNPP_ERR_CAPACITY, "Not enough room to store clouds. Increase max_node_no.");
  long long nnz = 0;
  NNPP_TRY(scan_ints(st, len.get(), out.ptr.get(), N, &nnz));
  if (nnz < 0 || nnz > (long long)INT_MAX)
    return set_error(NNPP_ERR_UNSUPPORTED, "build: more than 2^31-1 bonds");
  if (!out.col.alloc(nnz > 0 ? nnz : 1)) return set_error(NNPP_ERR_NOMEM, "neighbour columns");
  k_cell_scan<true><<<warps_grid, 256, 0, st>>>(N, x, y, z, x0, y0, z0, cx, cy, cz, mx, my,
                                                max_hash, r, start.get(), order.get(),
                                                max_node_no, nullptr, out.ptr.get(),
                                                out.col.get(), err.get());
  NNPP_CUDA(cudaGetLastError());
  DBuf<int> dml;
  if (!dml.alloc(1)) return set_error(NNPP_ERR_NOMEM, "max length");
  NNPP_CUDA(cudaMemsetAsync(dml.get(), 0, sizeof(int), st));
  k_max_int<<<grid_for(N, 256), 256, 0, st>>>(len.get(), N, dml.get());
  int ml = 0;
  NNPP_CUDA(cudaMemcpyAsync(&ml, dml.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  out.nnz = nnz;
  out.max_len = ml + 1;  // self included, grid.h:198-203
  return NNPP_OK;
}

// exclusive scan of n <= 1024*1024 ints with the block sums in `sums` (3072 ints)
static nnpp_status scan_into(cudaStream_t st, const int* in, int* out, int n, int* sums) {
  const int nb = (n + kScanBlock - 1) / kScanBlock;
  if (nb > kScanBlock) return set_error(NNPP_ERR_UNSUPPORTED, "scan: too many elements");
  k_scan_block<int><<<nb, kScanBlock, 0, st>>>(in, out, sums, n);
  if (nb > 1) {
    k_scan_block<int><<<1, kScanBlock, 0, st>>>(sums, sums + 1024, sums + 2048, nb);
    k_scan_add<int><<<nb, kScanBlock, 0, st>>>(out, sums + 1024, n);
  }
  k_scan_tail<int><<<1, 1, 0, st>>>(in, out, n);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status build_canonical_into(cudaStream_t st, int N, const double* x, const double* y,
                                 const double* z, int max_node_no, double r, double cx,
                                 double cy, double cz, const BuildScratch& sc, int* clouds,
                                 int* lengths, int* max_len) {
  if (N <= 0 || N > sc.max_nodes)
    return set_error(NNPP_ERR_INVALID, "allocation-free build: node count beyond the scratch maximum");
  if (!(r > 0.0) || !(cx > 0.0) || !(cy > 0.0) || !(cz > 0.0) || max_node_no < 1)
    return set_error(NNPP_ERR_INVALID, "build: r, cell sizes and max_node_no must be positive");
  // bounding box (grid.h:49-71)
  k_bbox_partial<<<kBboxBlocks, 256, 0, st>>>(x, y, z, N, sc.bbox_part);
  k_bbox_final<<<1, 32, 0, st>>>(sc.bbox_part, kBboxBlocks, sc.bbox);
  NNPP_CUDA(cudaGetLastError());
  double bb[6];
  NNPP_CUDA(cudaMemcpyAsync(bb, sc.bbox, sizeof(bb), cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  // The whole grid, not only its occupied part, must fit the scratch cell arrays: then
  // no hash can wrap, and every hash indexes them in bounds.
  NNPP_TRY(check_hash_grid(bb, cx, cy, cz, (double)sc.max_cells));
  const int mx = static_cast<int>((bb[1] - bb[0]) / cx) + 1;
  const int my = static_cast<int>((bb[3] - bb[2]) / cy) + 1;
  // hashes (grid.h:81-85)
  NNPP_CUDA(cudaMemsetAsync(sc.misc, 0, 16 * sizeof(int), st));
  NNPP_CUDA(cudaMemsetAsync(sc.misc, 0xff, sizeof(int), st));
  k_hash<<<grid_for(N, 256), 256, 0, st>>>(x, y, z, N, bb[0], bb[2], bb[4], cx, cy, cz, mx, my,
                                           sc.hash, sc.misc);
  NNPP_CUDA(cudaGetLastError());
  int hmax = -1;
  NNPP_CUDA(cudaMemcpyAsync(&hmax, sc.misc, sizeof(int), cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  if (hmax < 0) return set_error(NNPP_ERR_INVALID, "build: negative hash (non-finite coordinates?)");
  const int max_hash = hmax + 1;
  if (max_hash > sc.max_cells)
    return set_error(NNPP_ERR_INVALID, "allocation-free build: cell count beyond the scratch maximum");
  // counting sort by cell, members by node index (the canonical order)
  NNPP_CUDA(cudaMemsetAsync(sc.count, 0, sizeof(int) * max_hash, st));
  k_count<<<grid_for(N, 256), 256, 0, st>>>(sc.hash, N, sc.count);
  NNPP_TRY(scan_into(st, sc.count, sc.start, max_hash, sc.scan_sums));
  NNPP_CUDA(cudaMemcpyAsync(sc.cursor, sc.start, sizeof(int) * (max_hash + 1), cudaMemcpyDeviceToDevice, st));
  k_scatter<<<grid_for(N, 256), 256, 0, st>>>(sc.hash, N, sc.cursor, sc.order_tmp);
  k_sort_segments<<<grid_for(max_hash, 1, 65535), 128, 0, st>>>(sc.start, max_hash, sc.order_tmp, sc.order);
  NNPP_CUDA(cudaGetLastError());
  // padded output: -1 everywhere, then self and neighbours (grid.h:145-196)
  NNPP_CUDA(cudaMemsetAsync(clouds, 0xff, sizeof(int) * (size_t)N * (size_t)max_node_no, st));
  k_cell_scan_padded<<<grid_for((long long)N * 32, 256, 152 * 64), 256, 0, st>>>(
      N, x, y, z, bb[0], bb[2], bb[4], cx, cy, cz, mx, my, max_hash, r, sc.start, sc.order,
      max_node_no, clouds, lengths, sc.misc);
  NNPP_CUDA(cudaGetLastError());
  int misc[3];
  NNPP_CUDA(cudaMemcpyAsync(misc, sc.misc, sizeof(misc), cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  if (misc[1])
    return set_error(NNPP_ERR_CAPACITY, "Not enough room to store clouds. Increase max_node_no.");
  if (max_len) *max_len = misc[2];
  return NNPP_OK;
}

nnpp_status emit_padded(cudaStream_t st, const RefLists& L, int max_node_no, int* host_clouds,
                        int* host_lengths) {
  const int N = L.N;
  if (host_lengths) {
    std::vector<int> ptr(N + 1);
    NNPP_CUDA(cudaMemcpyAsync(ptr.data(), L.ptr.get(), sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, st));
    NNPP_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < N; ++i) host_lengths[i] = ptr[i + 1] - ptr[i] + 1;
  }
  if (host_clouds) {
    DBuf<int> pad;
    const size_t total = (size_t)N * (size_t)max_node_no;
    if (!pad.alloc(total)) return set_error(NNPP_ERR_NOMEM, "padded clouds");
    NNPP_CUDA(cudaMemsetAsync(pad.get(), 0xff, total * sizeof(int), st));
    k_emit_padded<<<grid_for(N, 256), 256, 0, st>>>(N, L.ptr.get(), L.col.get(), pad.get());
    NNPP_CUDA(cudaGetLastError());
    NNPP_CUDA(cudaMemcpyAsync(host_clouds, pad.get(), total * sizeof(int), cudaMemcpyDeviceToHost, st));
    NNPP_CUDA(cudaStreamSynchronize(st));
  }
  return NNPP_OK;
}

nnpp_status build_layout(cudaStream_t st, const RefLists& L, const double* x, const double* y,
                         const double* z, double bin_side, double delta, double dx, double dV,
                         double s_exp, Layout& out) {
  const int N = L.N;
  out.N = N;
  const double ox = L.bbox[0], oy = L.bbox[2], oz = L.bbox[4];
  int nb[3];
  for (int d = 0; d < 3; ++d) {
    double ext = L.bbox[2 * d + 1] - L.bbox[2 * d];
    long long v = (long long)(ext / bin_side) + 1;
    if (v < 1) v = 1;
    if (v > 4096) return set_error(NNPP_ERR_UNSUPPORTED, "layout: too many bins per axis");
    nb[d] = (int)v;
  }
  long long nbins = (long long)nb[0] * nb[1] * nb[2];
  if (nbins > (1LL << 28)) return set_error(NNPP_ERR_UNSUPPORTED, "layout: too many bins");
  out.nbins = (int)nbins;
  for (int d = 0; d < 3; ++d) out.nb[d] = nb[d];
  DBuf<int> bin;
  if (!bin.alloc(N)) return set_error(NNPP_ERR_NOMEM, "bins");
  k_bin_of<<<grid_for(N, 256), 256, 0, st>>>(x, y, z, N, ox, oy, oz, bin_side, nb[0], nb[1], nb[2],
                                             bin.get());
  NNPP_TRY(counting_sort(st, bin.get(), N, out.nbins, out.bin_start, out.perm));
  if (!out.iperm.alloc(N)) return set_error(NNPP_ERR_NOMEM, "iperm");
  k_invert<<<grid_for(N, 256), 256, 0, st>>>(out.perm.get(), N, out.iperm.get());
  DBuf<int> len, tmpcol;
  if (!len.alloc(N) || !out.row.alloc(N + 1)) return set_error(NNPP_ERR_NOMEM, "rows");
  k_gather_len<<<grid_for(N, 256), 256, 0, st>>>(out.perm.get(), L.ptr.get(), N, len.get());
  long long nnz = 0;
  NNPP_TRY(scan_ints(st, len.get(), out.row.get(), N, &nnz));
  out.nnz = nnz;
  const size_t nz = nnz > 0 ? (size_t)nnz : 1;
  if (!tmpcol.alloc(nz) || !out.col.alloc(nz) || !out.w64.alloc(nz) || !out.w32.alloc(nz) ||
      !out.wlo32.alloc(nz) ||
      !out.pos.alloc(3 * (size_t)N))
    return set_error(NNPP_ERR_NOMEM, "layout bonds");
  const int wg = grid_for((long long)N * 32, 256, 152 * 64);
  k_fill_internal<<<wg, 256, 0, st>>>(out.perm.get(), out.iperm.get(), L.ptr.get(), L.col.get(),
                                      out.row.get(), N, tmpcol.get());
  k_sort_segments<<<grid_for(N, 1, 65535), 128, 0, st>>>(out.row.get(), N, tmpcol.get(), out.col.get());
  k_gather_pos<<<grid_for(N, 256), 256, 0, st>>>(out.perm.get(), x, y, z, N, out.pos.get());
  k_weights<<<wg, 256, 0, st>>>(N, out.row.get(), out.col.get(), out.pos.get(), delta, dx, dV, s_exp,
                                out.w64.get(), out.w32.get(), out.wlo32.get());
  NNPP_CUDA(cudaGetLastError());
  NNPP_CUDA(cudaStreamSynchronize(st));
  out.max_row = L.max_len - 1;
  return NNPP_OK;
}

}  // namespace nnpp
