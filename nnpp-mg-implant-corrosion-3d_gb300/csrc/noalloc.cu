// noalloc.cu -- neighbour build for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code that runs under a host framework owning every
// device allocation (a fixed-size arena handed out by the application), real-time loops
// that must not hit the allocator, or an application already at its memory cap.  For them
// nnpp_build_clouds_hash_noalloc builds the neighbour lists into buffers the caller owns,
// with every temporary in one file-scope device array of fixed size.  That array exists on
// every GPU on which this library is loaded, for the life of the process.
#include <string>

#include "neighbours.cuh"

namespace {

constexpr int kMaxNodes = 1 << 18;  // 262,144 nodes
constexpr int kMaxCells = 1 << 18;  // 262,144 hash cells
constexpr size_t kDoubles = 6 * nnpp::kBboxBlocks + 8;
constexpr size_t kInts = 3 * (size_t)kMaxNodes + 3 * ((size_t)kMaxCells + 1) + 4096 + 16;
constexpr size_t kWords = kDoubles + (kInts + 1) / 2;  // 8-byte words, about 6.3 MB

// The shared scratch.  In host code this name is only a host-side stand-in for the device
// array; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned long long g_build_scratch[kWords];

// Device address of the scratch on the current device.  It is looked up on every call
// (cheap next to the call's stream synchronisations) rather than cached: after a
// cudaDeviceReset the module is loaded again and an address cached before it would be
// stale.
nnpp_status scratch_address(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_build_scratch);
  if (e != cudaSuccess || !p)
    return nnpp::set_error(NNPP_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  *out = p;
  return NNPP_OK;
}

}  // namespace

extern "C" nnpp_status nnpp_build_clouds_hash_noalloc(int max_node_no, double r, double dx,
                                                      double dy, double dz, int n_nodes,
                                                      const double* d_nodes_colmajor,
                                                      int* d_clouds_colmajor, int* d_cloud_lengths,
                                                      int* max_cloud_length, void* stream) {
  nnpp::clear_error();
  if (n_nodes <= 0 || !d_nodes_colmajor || !d_clouds_colmajor || !d_cloud_lengths)
    return nnpp::set_error(NNPP_ERR_INVALID, "noalloc build: missing buffers");
  if (n_nodes > kMaxNodes)
    return nnpp::set_error(NNPP_ERR_INVALID, "noalloc build: more than 262144 nodes (fixed scratch size)");
  void* base = nullptr;
  NNPP_TRY(scratch_address(&base));
  nnpp::BuildScratch sc;
  double* d = static_cast<double*>(base);
  sc.bbox_part = d;
  sc.bbox = d + 6 * nnpp::kBboxBlocks;
  int* i = reinterpret_cast<int*>(d + kDoubles);
  sc.hash = i;
  i += kMaxNodes;
  sc.order_tmp = i;
  i += kMaxNodes;
  sc.order = i;
  i += kMaxNodes;
  sc.count = i;
  i += kMaxCells + 1;
  sc.start = i;
  i += kMaxCells + 1;
  sc.cursor = i;
  i += kMaxCells + 1;
  sc.scan_sums = i;
  i += 4096;
  sc.misc = i;
  sc.max_nodes = kMaxNodes;
  sc.max_cells = kMaxCells;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t n = (size_t)n_nodes;
  return nnpp::build_canonical_into(st, n_nodes, d_nodes_colmajor, d_nodes_colmajor + n,
                                    d_nodes_colmajor + 2 * n, max_node_no, r, dx, dy, dz, sc,
                                    d_clouds_colmajor, d_cloud_lengths, max_cloud_length);
}
