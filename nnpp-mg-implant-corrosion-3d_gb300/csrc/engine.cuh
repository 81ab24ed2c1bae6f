// engine.cuh -- batched execution of one or many instances: tile and chunk work lists,
// per-instance reductions, the CUDA graph of a step.
#ifndef NNPP_ENGINE_CUH
#define NNPP_ENGINE_CUH

#include <vector>

#include "handle.cuh"

namespace nnpp {

// A tile: T consecutive bins along x of one instance (its "own" nodes) and the 3x3 rows of
// bins around them (its halo).  Bins have side >= the horizon radius, so every neighbour of
// an own node lies in the halo; halo rows are contiguous node ranges in the internal order.
struct TileDesc {
  int inst;
  int own_begin, own_end;  // own nodes (internal indices of the instance)
  int hb[9];               // halo row r: nodes [hb[r], hb[r] + hl[r])
  int hl[9];
  int halo;                // total halo nodes (sum of hl)
  int slice0;              // first 32-row slice of the own nodes (instance's sliced arrays)
  int pad[2];
  int bond0;               // first bond of the own nodes, rounded down to a multiple of 8
  int bond1;               // one past the last bond of the own nodes
};

// The halo-staged CG operator (variant 8) over the rows and columns that can be unknowns of
// the potential solve (nodes without a Dirichlet value of the potential; phases only change
// from solid to liquid, so the set is fixed for the run).  A tile's such rows are sorted by
// their number of such neighbours (initially solid rows last) and grouped in quads of four
// rows; a warp runs a quad with eight lanes per row.  A quad's codes (the 16-bit halo slot of
// each neighbour, the tile's padding slot after the row's end) lie pass-major: pass p, row g,
// lane j at coff + 32 p + 8 g + j, so that a pass of the warp reads 64 contiguous bytes.
struct HTile {             // parallel to the engine's tile list
  int q0, nq;              // the tile's quads (instance-local quad indices)
  int cstart16, clen16;    // its code block in the instance's code array, in 16-byte units
  int bx0, by, bz;         // first own bin along x, bin row (y, z)
  int T;                   // bins per tile
};
// (HQuad, the quad descriptor, is in handle.cuh)

// An elementwise work item: nodes [begin, end) of one instance.
struct Chunk {
  int inst;
  int begin, end;
  int pad;
};

// 32 consecutive rows of one tile in the sliced operator layout (bond c of row row0 + l at
// off + 32 c + l of the instance's sliced arrays).  The neighbours of a slice lie in 9 node
// ranges (its window rows, within the tile's 3x3 halo rows); a slot code is
// (window row r << 12 | node - lo[r]).  The window is what the staged kernels copy to shared
// memory: row r is wlen[r] nodes from lo[r] (both multiples of 4) at woff[r].
constexpr int kWinCap = 1536;  // nodes of one staged window
struct SliceDesc {
  int inst;
  int tile;    // global tile index
  int row0;    // first row (internal node index of the instance)
  int nrows;   // rows in the slice (<= 32)
  int off;     // offset in the instance's sliced arrays
  int width;   // columns (longest row of the slice)
  int wtotal;  // nodes of the window (sum of wlen)
  int pad;
  int lo[9];
  int woff[9];
  int wlen[9];
  // gather base of window row r: a bond's neighbour is gbase[code >> 12] + (code & 4095).
  // When the window fits 4096 nodes the 12-bit part is the neighbour's position in the
  // window (woff[r] + node - lo[r]) and gbase[r] = lo[r] - woff[r]; otherwise it is
  // node - lo[r] and gbase[r] = lo[r].
  int gbase[9];
  int pad2[4];
};

// What every batched kernel receives.
struct EngineView {
  const KParams* inst;      // per instance
  const TileDesc* tiles;    // grouped by instance
  const Chunk* chunks;      // grouped by instance
  const int* tile_first;    // per instance: first tile index
  const int* tile_count;    // per instance: number of tiles
  const int* chunk_first;
  const int* chunk_count;
  const HTile* htiles;      // parallel to tiles (halo-staged CG operator)
  const SliceDesc* slices;  // grouped by instance, tiles in order
  const int* slice_first;
  const int* slice_count;
  // the CG operator's slices: 32 of a bin row's nodes without a potential Dirichlet value
  // (row0: the first of its 32 slots in the instance's cg_rows; tile: the bin row, by | bz << 16)
  const SliceDesc* cslices; // grouped by instance
  const int* cslice_first;
  const int* cslice_count;
  unsigned int* ticket;     // per instance completion counters, + [M] global, + [M+1] grid,
                            // + [M+2] slice claims, + [M+3] the next-guess pass
  double* partials;         // kReduceSlots * stride
  int ntiles, nchunks, M, in_graph;
  int nslices;
  int ncslices;
  int stride;               // max(ntiles, nchunks, nslices, ncslices): slot stride of partials
  int halo_max;             // largest halo (dynamic shared memory sizing)
  int bond_max;             // largest staged bond range of a tile (bond1 - bond0)
  int hcode_max16;          // largest code block of a tile (16-byte units, variant 8)
};

constexpr int kChunk = 1024;  // nodes per elementwise work item
constexpr int kSpmvVariants = 9;  // FP32 CG operator variants the autotuner times
constexpr int kSpmvHalo = 8;      // the halo-staged variant with recomputed weights
constexpr int kTrVariants = 2;    // FP32 transport forms (0 L1/L2 gathers, 1 halo staged)

struct Engine {
  std::vector<Handle*> members;
  int T = 4;                // bins per tile (autotuned)
  int W = 8;                // lanes per node (autotuned)
  bool tuned = false;
  bool eager = false;       // NNPP_EAGER=1: launch kernel by kernel, loops driven by the host
  int spmv_variant = 0;     // FP32 CG operator: 0, 3 L1/L2 gathers (batches of 16, 0
                            // pipelined),
                            // 1 bulk-copy staged, 2, 4 shared-memory windows (8, 16),
                            // 5, 6, 7: 4, 3, 2 with L2 prefetch of the operator stream,
                            // 8 tile halo in shared memory, weights recomputed
  int tr_variant = 0;       // FP32 transport: 0 neighbour records gathered from L1/L2 (the
                            // faster), 1 the tile's halo records staged in shared memory
  bool halo_op = false;     // every member has the variant 8 layout
  int checks = 0;           // nnpp_set_checks flags of any member (the checked kernels run)
  int hcode_max16 = 0;      // largest tile code block (16-byte units)
  int hquad_max = 0;        // most quads of a tile
  bool windows_fit = false; // every slice window fits kWinCap (the staged operator runs)
  int win_cap = 0;          // largest slice window (nodes, multiple of 16)
  int grid = 0;
  int sms = 152;
  int halo_max = 0;
  int bond_max = 0;
  DBuf<KParams> d_inst[2];  // indexed by the parity of the current record buffer
  DBuf<TileDesc> d_tiles;
  DBuf<Chunk> d_chunks;
  DBuf<int> d_meta;         // tile/chunk/slice/CG slice first and count (8*M)
  DBuf<SliceDesc> d_slices;
  DBuf<SliceDesc> d_cslices;
  DBuf<HTile> d_htiles;
  DBuf<unsigned int> d_ticket;
  DBuf<double> d_partials;
  int ntiles = 0, nchunks = 0, nslices = 0, ncslices = 0;
  cudaStream_t st = nullptr, st_b1 = nullptr, st_b2 = nullptr;
  int device = 0;
  int cur = 0;              // record parity shared by all members
  bool coarse_graphs = false;  // graphs captured with the two-level preconditioner
  cudaGraphExec_t gexec[kGraphKinds][2][2] = {};
  cudaGraph_t graph[kGraphKinds][2][2] = {};
  ~Engine();
};

EngineView make_view(Engine& e, int parity, int in_graph);

// engine.cu
nnpp_status engine_build(Engine& e);             // tiles, work lists, autotune
nnpp_status engine_run(Engine& e, int n_steps, int prec, bool prepared = false);
nnpp_status engine_solve(Engine& e, int prec);   // potential solve only (current state)
nnpp_status engine_warm(Engine& e, int prec);    // tune, upload parameters, build graphs
nnpp_status engine_params(Engine& e);            // re-upload the members' KParams
void engine_destroy_graphs(Engine& e);

// tiles.cu: tile descriptors, 16-bit halo slots and FP32 position records of one instance
nnpp_status build_tiles(Handle& h, int T, std::vector<TileDesc>& tiles, std::vector<SliceDesc>& slices,
                        int inst, int* halo_max, int* bond_max, bool* windows_fit);
// the CG operator's slices of one instance (bin rows' nodes without a potential Dirichlet
// value, 32 a slice, with their windows) and its compacted arrays (filled by the prep); the
// slices are appended to cslices; false in *windows_fit when a window exceeds kWinCap
nnpp_status build_cg_slices(Handle& h, std::vector<SliceDesc>& cslices, int inst, bool* windows_fit);
// the variant 8 layout of one instance (after build_tiles, same T): its HTile entries are
// appended to htiles (parallel to the instance's tiles); false in *ok when the layout does
// not apply (a kernel exponent s != 0, a halo of 65535 nodes or more)
nnpp_status build_halo_op(Handle& h, int T, const std::vector<TileDesc>& tiles, int tile0,
                          std::vector<HTile>& htiles, int* code_max16, int* quad_max, bool* ok);

// step.cu launchers (batched)
nnpp_status launch_warm_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st);
bool spmv_staged_fits(const Engine& e);
// the halo-staged variant fits the shared memory of a CTA
bool spmv_halo_fits(const Engine& e);
bool transport_halo_fits(const Engine& e);
// the variant gathers from per-slice shared-memory windows (needs spmv_staged_fits)
inline bool spmv_needs_windows(int variant) {
  return variant == 1 || variant == 2 || variant == 4 || variant == 5 || variant == 7;
}
nnpp_status launch_prep_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st,
                          cudaGraphConditionalHandle hc, double* F11_out);
nnpp_status launch_cg_init_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st,
                             cudaGraphConditionalHandle hc);
nnpp_status launch_cg_spmv_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st);
nnpp_status launch_coarse_part_b(const Engine& e, const EngineView& v, int prec, int part, cudaStream_t st);
nnpp_status launch_cg_update_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st,
                               cudaGraphConditionalHandle hc);
bool engine_coarse(const Engine& e);  // the two-level preconditioner applies (every member has one)
nnpp_status launch_cg_final_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st);
nnpp_status launch_ir_update_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st,
                               cudaGraphConditionalHandle hc);
nnpp_status launch_transport_b(const Engine& e, const EngineView& v, int prec, cudaStream_t st,
                               double* F_out);
nnpp_status prepare_kernels(int halo_max, int bond_max, int W);
nnpp_status engine_set_tiles(Engine& e, int T);  // work lists for T bins per tile

// adjoint (step.cu)
nnpp_status launch_adj_transport(const Engine& e, const EngineView& v, const Rec64* snap,
                                 const Rec64* snap1, const double* lam, double* mu, double* nu,
                                 double* acc, cudaStream_t st);
nnpp_status launch_adj_combine(Handle& h, const double* mu, double* lam, double inject);
nnpp_status launch_snap_state(Handle& h, Rec64* dst);
nnpp_status launch_snap_phi(Handle& h, Rec64* dst);
// a stored solved potential into phi64, the current records and the snapshot dst
nnpp_status launch_load_phi(Handle& h, const double* phi, Rec64* dst);
nnpp_status launch_adj_solve_setup(Handle& h, const Rec64* snap, const double* psi_prev);
nnpp_status launch_record_solve(Handle& h, int slot);
nnpp_status launch_adj_transport32(const Engine& e, const EngineView& v, Handle& h, const Rec64* snap,
                                   const Rec64* snap1, const double* lam, float4* rec, double* mu,
                                   double* nu, double* acc, cudaStream_t st);
nnpp_status launch_sum_c0(Handle& h, double* out);

}  // namespace nnpp

#endif  // NNPP_ENGINE_CUH
