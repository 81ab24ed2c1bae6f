// neighbours.cuh -- neighbour build (grid.h:43-204) and the internal bond layout.
#ifndef NNPP_NEIGHBOURS_CUH
#define NNPP_NEIGHBOURS_CUH

#include "common.cuh"
#include "dbuf.cuh"

namespace nnpp {

// Neighbour lists in the reference's order, user node indices, self excluded (CSR).
struct RefLists {
  int N = 0;
  long long nnz = 0;
  int max_len = 0;           // max cloud length, self included (grid.h:200-203)
  DBuf<int> ptr;             // N+1
  DBuf<int> col;             // nnz
  double bbox[6] = {0, 0, 0, 0, 0, 0};  // x0 x1 y0 y1 z0 z1
};

// Internal layout: nodes sorted into bins of side >= the horizon radius, bins in x-fastest
// order, nodes within a bin by user index; CSR rows over internal indices sorted ascending,
// with the per-bond weights beta(xi) dV / xi^(3+2s) in FP64 and FP32.
struct Layout {
  int N = 0;
  int nbins = 0;
  int nb[3] = {0, 0, 0};
  long long nnz = 0;
  int max_row = 0;
  DBuf<int> perm;        // internal -> user
  DBuf<int> iperm;       // user -> internal
  DBuf<int> bin_start;   // nbins + 1
  DBuf<int> row;         // N + 1
  DBuf<int> col;         // nnz, internal indices
  DBuf<double> pos;      // 3N SoA, internal order
  DBuf<double> w64;      // nnz
  DBuf<float> w32;       // nnz
  DBuf<float> wlo32;     // nnz: w64 - w32 (so that w32 + wlo32 carries w64 to ~2^-48)
};

// GPU exclusive scan of n ints into out[0..n] (out[n] = total).  Returns the total.
nnpp_status scan_ints(cudaStream_t st, const int* in, int* out, int n, long long* total);

// Reference-format build on the GPU from device coordinates (SoA x, y, z).
nnpp_status build_ref_lists(cudaStream_t st, int N, const double* x, const double* y,
                            const double* z, int max_node_no, double r, double cx, double cy,
                            double cz, int order_mode, RefLists& out);

// Padded column-major clouds (N x max_node_no, -1 padded, self at column 0) into host memory.
nnpp_status emit_padded(cudaStream_t st, const RefLists& L, int max_node_no, int* host_clouds,
                        int* host_lengths);

// Device scratch for the allocation-free build (every pointer provided by the caller).
struct BuildScratch {
  double* bbox_part;   // 6 * kBboxBlocks
  double* bbox;        // 6
  int* hash;           // max_nodes
  int* order_tmp;      // max_nodes
  int* order;          // max_nodes
  int* count;          // max_cells
  int* start;          // max_cells + 1
  int* cursor;         // max_cells + 1
  int* scan_sums;      // 4096
  int* misc;           // 16: [0] hash max, [1] capacity flag, [2] max length
  int max_nodes;
  int max_cells;
};
constexpr int kBboxBlocks = 128;

// Canonical-order build into caller device buffers (padded column-major clouds, lengths)
// without allocating: all temporaries live in `sc`.  Same kernels and decisions as the
// allocating path with NNPP_ORDER_CANONICAL.
nnpp_status build_canonical_into(cudaStream_t st, int N, const double* x, const double* y,
                                 const double* z, int max_node_no, double r, double cx,
                                 double cy, double cz, const BuildScratch& sc, int* clouds,
                                 int* lengths, int* max_len);

// Internal layout from the reference lists and user-order coordinates.
nnpp_status build_layout(cudaStream_t st, const RefLists& L, const double* x, const double* y,
                         const double* z, double bin_side, double delta, double dx,
                         double dV, double s_exp, Layout& out);

}  // namespace nnpp

#endif  // NNPP_NEIGHBOURS_CUH
