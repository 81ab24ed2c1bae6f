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

// Internal layout from the reference lists and user-order coordinates.
nnpp_status build_layout(cudaStream_t st, const RefLists& L, const double* x, const double* y,
                         const double* z, double bin_side, double delta, double dx,
                         double dV, double s_exp, Layout& out);

}  // namespace nnpp

#endif  // NNPP_NEIGHBOURS_CUH
