// handle.cuh -- the simulation handle and the parameter block of the step kernels.
#ifndef NNPP_HANDLE_CUH
#define NNPP_HANDLE_CUH

#include <vector>

#include "common.cuh"
#include "dbuf.cuh"
#include "neighbours.cuh"

namespace nnpp {

// A quad of the halo-staged CG operator (variant 8, see HTile in engine.cuh): four rows of
// one tile run by one warp, eight lanes per row.
struct HQuad {
  int rows[4];             // internal node index of row g, -1 for an empty row
  int npass;               // passes of eight codes per row
  int coff_abs;            // first code in the instance's code array
  int coff_rel;            // first code relative to the tile's code block
  int padcode;             // the tile's padding slot (its halo size)
};

// Everything a step kernel reads or writes for one instance; stored in device memory, one
// per instance of a batched launch.  Pointers are device pointers into the instance's
// buffers (internal node order).
struct KParams {
  int N;
  int pad0;
  const int* row;
  const int* col;
  const unsigned short* slot16;  // per bond: halo slot of the neighbour within its tile
  // sliced layout (32 consecutive rows of a tile per slice, bonds column-major within a
  // slice, rows padded to the slice's longest): per bond column 32 FP32 weights then 32
  // 16-bit slot codes (window row << 12 | offset)
  const float* sell;
  const float* sell_lo;          // sliced like sell's weights: wlo32 (32 floats per column)
  // the CG operator (and the refinement's residual update) on its own slices: 32 of a bin
  // row's nodes without a potential Dirichlet value a slice; each row holds its bonds to
  // columns that can be unknowns (liquid, no potential Dirichlet value) in bond order,
  // interleaved like sell (weights, codes relative to the CG slice's windows) and sell_lo
  float* sell_cg;
  float* sell_cg_lo;
  int* cg_width;                 // per CG slice of the handle: its longest row (the shorter
                                 // rows are zero-padded to the slice's capacity)
  const int* cg_rows;            // per slot: the node, -1 for padding
  const int* cg_pos;             // per node: its slot, -1 for potential-Dirichlet nodes
  const int* xrow;               // per node: its bin row, by | bz << 16
  float4* phi4;                  // per node {phi_hi, phi_lo} (zero on solid nodes), liquid, Dirichlet
  const double* w64;
  const float* w32;
  const float* wlo32;            // w64 - w32: the FP32 pair (w32, wlo32) carries w64
  const unsigned char* dirmask;  // bit k: species k Dirichlet, bit S: potential Dirichlet
  const double* bcval;           // (S+1)*N: species values already divided by CSolid
  Rec32* rec32_cur;
  Rec32* rec32_nxt;
  float4* clo;                   // compensation words of the FP32 concentrations
  Rec64* rec64_cur;
  Rec64* rec64_nxt;
  double* phi64;                 // potential (FP64, both precisions)
  double* phi_prev;              // potential of the previous step (linear extrapolation)
  double* phi_keep;              // non-null: the transport also writes the step's solved
                                 // potential here (forward_ckpt's per-step potentials)
  int* flip_step;
  int* flip_list;                // nodes this step's transport turned liquid (N capacity)
  // potential solve
  double* b64;
  double* r64;
  double* dsum64;                // sum of liquid-liquid weights (K11 diagonal)
  double* cpl64;                 // coupling to Dirichlet neighbours sum_j w phi_j (free rows)
  unsigned char* freem;          // unknown of the potential solve
  float* d32;
  float* dinv32;
  double* dinv64;
  float *rin32, *z32, *p32, *q32, *e32;
  double *rin64, *z64, *p64, *q64, *e64;
  DevState* ds;
  const double* bv_ptr;          // interface factor BV (ds->BV, or an override)
  const double* b_override;      // right-hand side of the potential solve instead of
                                 // (1/(K sigma)) F CSolid sum_k z_k c_k (adjoint solves)
  // physics
  double dt, csat, c_floor, k_diss, sw, vol_red, lam;
  float csat_hi, csat_lo, cfl_hi, cfl_lo;  // CSat/CSolid and c_floor as FP32 pairs
  double K1[S], K2zF[S], DL[S], DSo[S], z[S];
  int sub_step_no;
  int dissolve_count;            // 1: count the dissolution source into the diagnostics
  int extrapolate;               // 1: warm start phi = 2 phi^n - phi^{n-1}
  int hist_m;                    // >= 3: A-norm-optimal warm start from the last hist_m
                                 // solutions (history ring xh, bh = A xh); 0: off
  double* xh;                    // hist_m * N potentials of previous solves
  double* bh;                    // hist_m * N: A x of those (b - r at convergence)
  // two-level preconditioner (single-instance engines): node -> aggregate, the coarse
  // inverse (n x n), the restricted residual and the coarse correction
  const int* agg;
  const float* cinv;
  float* rc;
  float* xc;
  const int* bin_start;
  int coarse;                    // 1: z = D^-1 r + P A_c^-1 P^T r
  int cn;                        // coarse unknowns
  int cld;                       // row stride of cinv
  double* cdots;                 // 3 cn: per-aggregate dot contributions
  // deflated CG (mixed inner solves while k.ds->defl): A P without its diagonal term (ap_k
  // slots per node, slot-major: aggregate, -sum of the weights to the unknowns of that
  // aggregate), the correction equation's right-hand side r0 and t = A e
  int defl_ok;                   // single-instance engine (ensembles take the additive form)
  int ap_k;
  const int* ap_col;
  const float* ap_val;
  float* r0_32;
  float* t32;
  int cf, cna0, cna1, cna2, nb0, nb1, nb2;
  // halo-staged CG operator (variant 8): quads, codes, FP32 bin-local positions and the
  // weight in bin units w = beta / xi^3 with beta = min(1, hc0 - hc1 xi); the operator's
  // off-diagonal sum is hsw * sum w z (hsw = dV / h^3)
  const HQuad* hquad;
  const unsigned short* hcode;
  const float4* posrec;
  float hinv, hc0, hc1, hsw;
  int hquad_n;                   // quads of the instance
  int checks;                    // nnpp_set_checks flags
};

enum GraphKind { kGraphStep2 = 0, kGraphStep1 = 1, kGraphSolve = 2, kGraphKinds = 3 };

struct Engine;

constexpr int kCoarseMax = 3000;  // aggregates of the coarse space (dense inverse n^2 floats)

struct Coarse {
  int f = 0, n = 0, na[3] = {0, 0, 0};
  int ld = 0;         // row stride of inv: n rounded up to 4 (16-byte rows, zero padding)
  DBuf<int> agg;      // N: aggregate of each node
  DBuf<float> inv;    // n x ld: the coarse inverse (symmetric: row I = column I)
  DBuf<float> rc, xc; // restricted residual (ld, zero padding), coarse correction (n)
  DBuf<double> dots;  // 3n: per aggregate r.D^-1 r and r.r of the update, r_c x_c of the product
  DBuf<int> ap_col;   // A P off its diagonal term (27 N capacity, ap_k used): see KParams
  DBuf<float> ap_val;
  int ap_k = 1;
  DBuf<float> rowabs; // n: row sums of |A_c| (Newton-Schulz scaling)
  DBuf<float> a, t, x, y; // n x n: A_c and the Newton-Schulz work matrices
  DBuf<double> nrm;        // block partials of ||I - A_c X_0||_F^2 (warm-started rebuilds)
  size_t inv_elems() const { return (size_t)n * ld; }
  DBuf<unsigned char> snap;  // N: phases (internal order) the inverse was computed from
  DBuf<int> count;           // phase changes since (coarse_check)
  void* cublas = nullptr;
  bool valid = false; // inv holds an inverse
  bool stale = true;  // the phases changed since inv was computed
  long long rebuilds = 0;  // inverses computed since the handle was built
  long long warm_rebuilds = 0;  // of which Newton-Schulz started from the previous inverse
  int ns_steps = 0;        // Newton-Schulz steps of the last rebuild
  long long timed_rebuilds = 0;  // rebuilds triggered by phase changes within a run
  double rebuild_ms = 0.0;       // their host-observed duration (stream drained on both sides)
  ~Coarse();
};

struct Handle {
  nnpp_params p;
  int N = 0;
  int device = 0;
  cudaStream_t st = nullptr;
  // user-order inputs
  DBuf<double> ux, uy, uz;
  std::vector<int> h_bctypes;
  std::vector<double> h_bcv, h_ic;
  std::vector<int> h_phase0;
  // neighbour lists and internal layout
  RefLists ref;
  Layout lay;
  bool built = false;
  int max_node_no = 0;
  // tiles (built for tiles_T bins per tile)
  DBuf<unsigned short> slot16;
  DBuf<float> sell;
  DBuf<float> sell_lo;
  DBuf<float> sell_cg;          // the CG operator's slices (see KParams)
  DBuf<float> sell_cg_lo;
  DBuf<int> cg_width, cg_rows, cg_pos, xrow;
  DBuf<float4> phi4;
  DBuf<float4> posrec;
  float h32 = 0.f;
  DBuf<HQuad> hquad;     // halo-staged CG operator (variant 8) of the current tiles
  DBuf<unsigned short> hcode;
  bool halo_op_ok = false;
  int checks = 0;               // nnpp_set_checks flags
  int tiles_T = 0;
  // per-node constants, internal order
  DBuf<unsigned char> dirmask;
  DBuf<double> bcval;
  // state
  DBuf<Rec32> rec32[2];
  DBuf<float4> clo;
  DBuf<Rec64> rec64[2];
  int cur = 0;
  int state_prec = NNPP_FP64;
  DBuf<double> phi64, phi_prev;
  DBuf<int> flip_step;
  // solver
  DBuf<double> b64, r64, dsum64, cpl64, dinv64, rin64, z64, p64, q64, e64;
  DBuf<float> d32, dinv32, rin32, z32, p32, q32, e32, r0_32, t32;
  DBuf<unsigned char> freem;
  DBuf<int> flip_list;          // N: the nodes the last transport turned liquid
  DBuf<DevState> dstate;
  DBuf<double> scratch_d;       // small device scratch (voln1rel override, ...)
  DBuf<double> user_stage;      // (S+1)*N FP64 staging for host transfers
  DBuf<int> user_stage_i;       // N int staging
  double tol = 1e-10;
  int max_iter = 2000;
  int max_outer = 30;
  double inner_rel = 1e-4;
  int strict = 0;
  bool settings_pushed = false; // tol, max_iter, ... already in the device state
  int extrapolate = 1;
  int warm_hist = kHistMax;     // history length of the warm start (0: extrapolation only)
  bool coarse_enabled = true;   // two-level preconditioner (single-instance runs)
  Coarse coarse;
  int coarse_every = 64;        // check for phase changes every that many steps (0: never)
  long long nstep = 0;          // steps since the state was last replaced (refresh schedule)
  // refreshes during forward_ckpt (step relative to its start, the inverse from then on),
  // replayed by backward so that recomputed steps and adjoint solves see the same operator
  struct CoarseEvent {
    long long step = 0;
    DBuf<float> inv;
    DBuf<int> ap_col;
    DBuf<float> ap_val;
    int ap_k = 1;
    DBuf<unsigned char> snap;  // the phases it was built from
  };
  std::vector<CoarseEvent> coarse_events;
  bool coarse_record = false, coarse_replay = false;
  long long coarse_base = 0;    // nstep at the start of forward_ckpt
  long long fwd_nstep_end = 0;  // nstep at its end
  int coarse_event_cur = -1;    // event whose inverse coarse.inv holds during replay
  DBuf<double> xh, bh;          // warm-start history, warm_hist * N each
  double* warm_x_alt = nullptr; // another ring in place of xh, bh (the adjoint's solves)
  double* warm_b_alt = nullptr;
  const double* b_override = nullptr;  // set during adjoint solves
  int grid = 0;                 // CTAs of the per-handle elementwise kernels
  Engine* engine = nullptr;     // single-instance engine (owned)
  // adjoint checkpoints: the full device state at a step
  struct Ckpt {
    DBuf<Rec32> rec32;
    DBuf<float4> clo;
    DBuf<Rec64> rec64;
    DBuf<double> phi, phi_prev;
    DBuf<int> flip;
    DBuf<double> xh, bh;
    DevState ds;
    int cur = 0, prec = 0;
  };
  std::vector<Ckpt> ckpts;
  Ckpt fwd_end;
  // adjoint storage: 0 automatic (every step's snapshot when it fits a quarter of the free
  // device memory), 1 checkpoints and recomputation, 2 every step's snapshot
  int adjoint_store = 0;
  DBuf<Rec64> snap_all;         // (steps + 1) x N snapshots of the recorded forward
  bool snap_all_valid = false;
  // with checkpoints: every step's solved potential (steps x N), so that backward
  // recomputes a segment's steps without their potential solves
  DBuf<double> phi_all;
  bool phi_all_valid = false;
  double* phi_keep[2] = {nullptr, nullptr};  // KParams.phi_keep of each record parity
  // the last backward's adjoint potential solves: inner iterations, solves, refinement
  // sweeps, and the inner iterations of each step's solve (fwd_steps entries)
  long long adj_cg_iters = 0, adj_solves = 0, adj_sweeps = 0;
  DBuf<int> adj_log;
  double adj_tol = 0.0;         // relative tolerance of the adjoint solves (0: tol)
  int fwd_steps = 0, ck_every = 0, sample_every = 0, fwd_prec = NNPP_FP64;
  std::vector<double> curve;
  ~Handle();
};

// coarse.cu
nnpp_status coarse_build(Handle& h);
nnpp_status coarse_refresh(Handle& h);
// at a refresh point: recompute the inverse if a phase changed since the last refresh
nnpp_status coarse_check(Handle& h);
// during forward_ckpt: record the current coarse inverse and A P as used from `step` on
nnpp_status coarse_record_event(Handle& h, long long step);
// during backward: put the inverse and A P of the last recorded refresh at or before `step`
// (relative to the start of forward_ckpt) in place; recompute: `step` is about to be
// recomputed (a refresh recorded at it re-enables the deflation, as in the forward)
nnpp_status coarse_select(Handle& h, long long step, bool recompute = false);
// deflation on (device flag) exactly when the current phases are those of the installed
// coarse operator (asynchronous; the adjoint solves)
nnpp_status coarse_defl_check(Handle& h);

// step.cu
nnpp_status step_alloc(Handle& h);
KParams make_kparams(Handle& h, int cur);
// dirichlet_phi: put the boundary values of the potential on its Dirichlet nodes (state
// for stepping); false keeps the given values (inputs of the residual entry point).
nnpp_status load_state(Handle& h, const double* d_c_user, const double* d_phi_user,
                       const int* d_phase_user, int prec, bool dirichlet_phi,
                       bool keep_history = false);
nnpp_status store_state(Handle& h, double* d_c_user, double* d_phi_user, int* d_phase_user);
nnpp_status convert_state(Handle& h, int to_prec);
// the potential operator's mask-dependent arrays must be recomputed by the next prep
nnpp_status invalidate_operator(Handle& h);
// restart: keep vol0rel and the initial Mg mass, recompute voln1rel and BV of the current
// state (main.cpp:527-533)
nnpp_status init_diag(Handle& h, bool restart = false);

}  // namespace nnpp

#endif  // NNPP_HANDLE_CUH
