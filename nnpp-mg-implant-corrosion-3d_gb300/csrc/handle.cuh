// handle.cuh -- the simulation handle and the parameter block of the step kernels.
#ifndef NNPP_HANDLE_CUH
#define NNPP_HANDLE_CUH

#include <vector>

#include "common.cuh"
#include "dbuf.cuh"
#include "neighbours.cuh"

namespace nnpp {

// Everything a step kernel reads or writes, passed by value.  Pointers are device pointers
// into the handle's buffers (internal node order).
struct KParams {
  int N;
  int grid;                     // CTAs of every step kernel (layout of `partials`)
  const int* row;
  const int* col;
  const double* w64;
  const float* w32;
  const unsigned char* dirmask;  // bit k: species k Dirichlet, bit S: potential Dirichlet
  const double* bcval;          // (S+1)*N: species values already divided by CSolid
  Rec32* rec32_cur;
  Rec32* rec32_nxt;
  float4* clo;                  // compensation words of the FP32 concentrations
  Rec64* rec64_cur;
  Rec64* rec64_nxt;
  double* phi64;                // potential (FP64, both precisions)
  int* flip_step;
  // potential solve
  double* b64;
  double* r64;
  double* dsum64;               // sum of liquid-liquid weights (K11 diagonal)
  unsigned char* freem;         // unknown of the potential solve
  float* d32;
  float* dinv32;
  double* dinv64;
  float *rin32, *z32, *p32, *q32, *e32;
  double *rin64, *z64, *p64, *q64, *e64;
  double* partials;             // kReduceSlots * grid
  DevState* ds;
  const double* voln1rel_ptr;   // value entering BV (ds->voln1rel, or an override)
  // physics
  double dt, csat, c_floor, k_diss, sw, vol_red, lam;
  double K1[S], K2zF[S], DL[S], DSo[S], z[S];
  int sub_step_no;
  int dissolve_count;           // 1: count the dissolution source into the diagnostics
  int in_graph;                 // 1: kernels set the conditional handles of the graph
};

enum GraphKind { kGraphStep2 = 0, kGraphStep1 = 1, kGraphSolve = 2, kGraphKinds = 3 };

struct Handle {
  nnpp_params p;
  int N = 0;
  int device = 0;
  cudaStream_t st = nullptr;
  cudaStream_t st_b1 = nullptr, st_b2 = nullptr;  // capture streams for conditional bodies
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
  // per-node constants, internal order
  DBuf<unsigned char> dirmask;
  DBuf<double> bcval;
  // state
  DBuf<Rec32> rec32[2];
  DBuf<float4> clo;
  DBuf<Rec64> rec64[2];
  int cur = 0;
  int state_prec = NNPP_FP64;
  DBuf<double> phi64;
  DBuf<int> flip_step;
  // solver
  DBuf<double> b64, r64, dsum64, dinv64, rin64, z64, p64, q64, e64;
  DBuf<float> d32, dinv32, rin32, z32, p32, q32, e32;
  DBuf<unsigned char> freem;
  DBuf<double> partials;
  DBuf<DevState> dstate;
  DBuf<double> scratch_d;       // small device scratch (voln1rel override, ...)
  DBuf<double> user_stage;      // (S+1)*N FP64 staging for host transfers
  DBuf<int> user_stage_i;       // N int staging
  double tol = 1e-10;
  int max_iter = 2000;
  int max_outer = 30;
  double inner_rel = 1e-4;
  int strict = 0;
  int grid = 0;
  int lanes = 8;                // lanes per node of the bond kernels (autotuned)
  // graphs [kind][precision][cur]
  cudaGraphExec_t gexec[kGraphKinds][2][2] = {};
  cudaGraph_t graph[kGraphKinds][2][2] = {};
  // adjoint checkpoints (host-owned device buffers)
  struct Ckpt {
    DBuf<Rec64> rec;
    DBuf<double> phi;
    DevState ds;
  };
  std::vector<Ckpt> ckpts;
  int fwd_steps = 0, ck_every = 0, sample_every = 0, fwd_prec = NNPP_FP64;
  std::vector<double> curve;
  DevState ds_start;
  DBuf<Rec64> rec_start;
  DBuf<double> phi_start;
  DBuf<int> flip_start;
};

// step.cu
nnpp_status step_alloc(Handle& h);
KParams make_kparams(Handle& h, int cur);
nnpp_status launch_prep(Handle& h, const KParams& kp, int prec, cudaStream_t st,
                        cudaGraphConditionalHandle hc, double* F11_out);
nnpp_status launch_cg_init(Handle& h, const KParams& kp, int prec, cudaStream_t st,
                           cudaGraphConditionalHandle hc);
nnpp_status launch_cg_iter(Handle& h, const KParams& kp, int prec, cudaStream_t st,
                           cudaGraphConditionalHandle hc);
nnpp_status launch_cg_spmv(Handle& h, const KParams& kp, int prec, cudaStream_t st);
nnpp_status launch_ir_update(Handle& h, const KParams& kp, int prec, cudaStream_t st,
                             cudaGraphConditionalHandle hc);
nnpp_status launch_transport(Handle& h, const KParams& kp, int prec, cudaStream_t st,
                             double* F_out);
// dirichlet_phi: put the boundary values of the potential on its Dirichlet nodes (state
// for stepping); false keeps the given values (inputs of the residual entry point).
nnpp_status load_state(Handle& h, const double* d_c_user, const double* d_phi_user,
                       const int* d_phase_user, int prec, bool dirichlet_phi);
nnpp_status store_state(Handle& h, double* d_c_user, double* d_phi_user, int* d_phase_user);
nnpp_status convert_state(Handle& h, int to_prec);
nnpp_status init_diag(Handle& h);

}  // namespace nnpp

#endif  // NNPP_HANDLE_CUH
