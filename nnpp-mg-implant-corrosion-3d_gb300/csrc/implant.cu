// implant.cu -- the solid/liquid mask of the nodes from an implant point cloud.
//
// The reference marks a node solid when at least one point of the implant's surface-mesh
// cloud lies within r = 3 * 0.4 dx (1 + 1e-5) of it (main.cpp:316-325, 422-457): a kd-tree
// range query per node (kd_tree_interface.h:156-252 with libkdtree++'s find_within_range)
// returns the points inside the box c +- r (bounds c - r and c + r rounded in FP64,
// inclusive), of which those at Euclidean distance sqrt(x*x + y*y + z*z) <= r are counted.
// Here the points are binned on the host into a uniform grid of cells of side r; a thread
// per node walks the cells its box touches and applies the same two tests with explicitly
// rounded FP64 intrinsics (never contracted to FMA), so that every count equals the
// reference's.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "dbuf.cuh"

namespace nnpp {
namespace {

__global__ void k_implant_count(int n, const double* __restrict__ x, const double* __restrict__ y,
                                const double* __restrict__ z, double r, double gx0, double gy0,
                                double gz0, double cs, int gx, int gy, int gz,
                                const int* __restrict__ cstart, const double* __restrict__ px,
                                const double* __restrict__ py, const double* __restrict__ pz,
                                int* counts) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double c[3] = {x[i], y[i], z[i]};
    double lo[3], hi[3];
    int k0[3], k1[3];
    const double g0[3] = {gx0, gy0, gz0};
    const int gd[3] = {gx, gy, gz};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      lo[d] = __dsub_rn(c[d], r);  // the kd-tree region's bounds (region.hpp:50-51)
      hi[d] = __dadd_rn(c[d], r);
      // cells that can hold a point of the box, one cell of margin for the rounding of the
      // cell coordinate (the tests below decide)
      const double a = floor((lo[d] - g0[d]) / cs) - 1.0, b = floor((hi[d] - g0[d]) / cs) + 1.0;
      k0[d] = a < 0.0 ? 0 : (a > gd[d] - 1 ? gd[d] : (int)a);
      k1[d] = b < 0.0 ? -1 : (b > gd[d] - 1 ? gd[d] - 1 : (int)b);
    }
    int cnt = 0;
    for (int kz = k0[2]; kz <= k1[2]; ++kz)
      for (int ky = k0[1]; ky <= k1[1]; ++ky) {
        const int row = gx * (ky + gy * kz);
        const int s = cstart[row + k0[0]], e = k1[0] >= k0[0] ? cstart[row + k1[0] + 1] : s;
        for (int j = s; j < e; ++j) {
          const double qx = px[j], qy = py[j], qz = pz[j];
          // region.encloses (region.hpp:86-93): lo <= p <= hi in every coordinate
          if (qx < lo[0] || hi[0] < qx || qy < lo[1] || hi[1] < qy || qz < lo[2] || hi[2] < qz) continue;
          // Node::distance_euclidean (kd_tree_interface.h:42-48) <= r
          const double dx = __dsub_rn(qx, c[0]), dy = __dsub_rn(qy, c[1]), dz = __dsub_rn(qz, c[2]);
          const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
          if (__dsqrt_rn(d2) <= r) ++cnt;
        }
      }
    counts[i] = cnt;
  }
}

}  // namespace
}  // namespace nnpp

using namespace nnpp;

extern "C" nnpp_status nnpp_implant_mask(int n_nodes, const double* nodes_colmajor, int n_points,
                                         const double* points_colmajor, double r, int max_node_no,
                                         int* counts, int* phase) {
  clear_error();
  if (n_nodes <= 0 || n_points < 0 || !nodes_colmajor || (n_points > 0 && !points_colmajor))
    return set_error(NNPP_ERR_INVALID, "implant mask: missing nodes or points");
  if (!(r > 0.0) || !std::isfinite(r) || max_node_no < 0)
    return set_error(NNPP_ERR_INVALID, "implant mask: r must be positive and finite");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return set_error(NNPP_ERR_CUDA, "implant mask: no CUDA device");
  }
  const size_t N = (size_t)n_nodes, M = (size_t)n_points;
  // points binned by cell (host counting sort, cells of side r, x fastest)
  double b[6] = {0, 0, 0, 0, 0, 0};
  for (int d = 0; d < 3 && M > 0; ++d) {
    const double* p = points_colmajor + d * M;
    double mn = p[0], mx = p[0];
    for (size_t j = 1; j < M; ++j) {
      mn = std::min(mn, p[j]);
      mx = std::max(mx, p[j]);
    }
    if (!std::isfinite(mn) || !std::isfinite(mx)) return set_error(NNPP_ERR_INVALID, "implant mask: non-finite point");
    b[2 * d] = mn;
    b[2 * d + 1] = mx;
  }
  const double cs = r;
  long long g[3];
  for (int d = 0; d < 3; ++d) {
    const double ext = (b[2 * d + 1] - b[2 * d]) / cs;
    if (!(ext < 4.0e6)) return set_error(NNPP_ERR_UNSUPPORTED, "implant mask: point cloud too wide for r");
    g[d] = (long long)ext + 1;
  }
  const long long ncell = g[0] * g[1] * g[2];
  if (ncell > (1LL << 27)) return set_error(NNPP_ERR_UNSUPPORTED, "implant mask: more than 2^27 grid cells");
  std::vector<int> cell(M), start((size_t)ncell + 1, 0);
  for (size_t j = 0; j < M; ++j) {
    long long k[3];
    for (int d = 0; d < 3; ++d) {
      k[d] = (long long)((points_colmajor[d * M + j] - b[2 * d]) / cs);
      k[d] = std::min(std::max(k[d], 0LL), g[d] - 1);
    }
    cell[j] = (int)(k[0] + g[0] * (k[1] + g[1] * k[2]));
    start[cell[j] + 1] += 1;
  }
  for (long long c = 0; c < ncell; ++c) start[c + 1] += start[c];
  std::vector<double> sorted(3 * std::max<size_t>(M, 1));
  {
    std::vector<int> cur(start.begin(), start.end() - 1);
    for (size_t j = 0; j < M; ++j) {
      const int at = cur[cell[j]]++;
      for (int d = 0; d < 3; ++d) sorted[d * M + at] = points_colmajor[d * M + j];
    }
  }
  DBuf<double> dnodes, dpts;
  DBuf<int> dstart, dcount;
  if (!dnodes.alloc(3 * N) || !dpts.alloc(3 * std::max<size_t>(M, 1)) || !dstart.alloc((size_t)ncell + 1) ||
      !dcount.alloc(N))
    return set_error(NNPP_ERR_NOMEM, "implant mask buffers");
  cudaStream_t st = nullptr;
  NNPP_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } guard{st};
  NNPP_CUDA(cudaMemcpyAsync(dnodes.get(), nodes_colmajor, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, st));
  if (M > 0)
    NNPP_CUDA(cudaMemcpyAsync(dpts.get(), sorted.data(), sizeof(double) * 3 * M, cudaMemcpyHostToDevice, st));
  NNPP_CUDA(cudaMemcpyAsync(dstart.get(), start.data(), sizeof(int) * (ncell + 1), cudaMemcpyHostToDevice, st));
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>((N + 255) / 256, 152 * 16));
  k_implant_count<<<blocks, 256, 0, st>>>(n_nodes, dnodes.get(), dnodes.get() + N, dnodes.get() + 2 * N, r, b[0],
                                          b[2], b[4], cs, (int)g[0], (int)g[1], (int)g[2], dstart.get(),
                                          dpts.get(), dpts.get() + M, dpts.get() + 2 * M, dcount.get());
  NNPP_CUDA(cudaGetLastError());
  std::vector<int> cnt(N);
  NNPP_CUDA(cudaMemcpyAsync(cnt.data(), dcount.get(), sizeof(int) * N, cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  bool over = false;
  for (size_t i = 0; i < N; ++i) {
    over = over || cnt[i] > max_node_no;
    if (counts) counts[i] = cnt[i];
    if (phase) phase[i] = cnt[i] > 0 ? 1 : 0;
  }
  // kd_tree_interface.h:213-216
  if (over) return set_error(NNPP_ERR_CAPACITY, "found_node_no > max_node_no; increase max_node_no.");
  return NNPP_OK;
}
