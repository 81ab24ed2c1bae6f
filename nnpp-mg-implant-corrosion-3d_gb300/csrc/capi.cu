// capi.cu -- the C ABI (include/nnpp_gb300.h): handles, neighbour build, stepping through
// the batched engine (one instance per handle, many per ensemble), state transfer, the
// drop-in residual/solve entry points and measurement.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>

#include "engine.cuh"

using namespace nnpp;

struct nnpp_handle {
  Handle h;
};

struct nnpp_ensemble {
  Engine e;
  std::vector<nnpp_handle*> members;
};

namespace {

constexpr int kBlockHost = 256;

__global__ void k_unpermute(const int* perm, int n, int fields, const double* in, double* out) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
    const int u = perm[a];
    for (int f = 0; f < fields; ++f) out[(size_t)f * n + u] = in[(size_t)f * n + a];
  }
}

nnpp_status check_params(const nnpp_params* p) {
  if (!p) return set_error(NNPP_ERR_INVALID, "params is NULL");
  if (!(p->dt > 0) || !(p->dx > 0) || !(p->dy > 0) || !(p->dz > 0) || !(p->delta > 0))
    return set_error(NNPP_ERR_INVALID, "dt, dx, dy, dz and delta must be positive");
  if (p->CSolid == 0.0 || p->K_phi == 0.0 || p->sigma == 0.0 || p->R == 0.0 || p->T == 0.0)
    return set_error(NNPP_ERR_INVALID, "CSolid, K_phi, sigma, R and T must be non-zero");
  for (int s = 0; s < S; ++s)
    if (p->s1[s] != p->s_phi || p->s2[s] != p->s_phi)
      return set_error(NNPP_ERR_UNSUPPORTED,
                       "all kernel exponents s_k1, s_k2 and s111 must be equal (one weight per bond)");
  if (p->switch_width < 0) return set_error(NNPP_ERR_INVALID, "switch_width must be >= 0");
  return NNPP_OK;
}

nnpp_status read_state(Handle& h, DevState* ds) {
  NNPP_CUDA(cudaMemcpyAsync(ds, h.dstate.get(), sizeof(DevState), cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  return NNPP_OK;
}

nnpp_status check_after(Handle& h, long long nc_before) {
  DevState ds;
  NNPP_TRY(read_state(h, &ds));
  if (ds.wait_timeout) return set_error(NNPP_ERR_CUDA, "a bounded device wait timed out");
  if (ds.bounds_error) return set_error(NNPP_ERR_CUDA, "a device index check failed (nnpp_set_checks)");
  if (ds.nonfinite) return set_error(NNPP_ERR_NONFINITE, "non-finite concentration in the state");
  if (h.strict && ds.cg_nc > nc_before)
    return set_error(NNPP_ERR_CG_NO_CONVERGE, "potential solve hit its iteration cap");
  return NNPP_OK;
}

bool have_gpu() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return n > 0;
}

#define NNPP_GUARD(hp)                                                            \
  do {                                                                            \
    if (!(hp)) return set_error(NNPP_ERR_INVALID, "handle is NULL");              \
    clear_error();                                                                \
    if (cudaSetDevice((hp)->h.device) != cudaSuccess) {                           \
      cudaGetLastError();                                                         \
      return set_error(NNPP_ERR_CUDA, "cudaSetDevice failed");                    \
    }                                                                             \
  } while (0)

#define NNPP_NEED_BUILT(hp)                                                                   \
  do {                                                                                        \
    if (!(hp)->h.built)                                                                       \
      return set_error(NNPP_ERR_STATE, "neighbour lists not built (call nnpp_build_neighbours)"); \
  } while (0)

// Everything a one-off evaluation on scratch inputs changes, so that it can be undone.
struct StateBackup {
  int cur, prec;
  DBuf<double> phi, phi_prev;
  DBuf<double> xh, bh;  // the warm-start history ring (a timed transport records into it)
  DBuf<float4> clo;
  DBuf<Rec32> rec32;
  DBuf<Rec64> rec64;
  DBuf<int> flip;
  DevState ds;
};

nnpp_status backup(Handle& h, StateBackup& b) {
  const size_t N = h.N;
  b.cur = h.cur;
  b.prec = h.state_prec;
  if (!b.phi.alloc(N) || !b.phi_prev.alloc(N) || !b.clo.alloc(N) || !b.rec32.alloc(N) ||
      !b.rec64.alloc(N) || !b.flip.alloc(N))
    return set_error(NNPP_ERR_NOMEM, "backup");
  NNPP_CUDA(cudaMemcpyAsync(b.phi.get(), h.phi64.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(b.phi_prev.get(), h.phi_prev.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(b.clo.get(), h.clo.get(), sizeof(float4) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(b.rec32.get(), h.rec32[h.cur].get(), sizeof(Rec32) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(b.rec64.get(), h.rec64[h.cur].get(), sizeof(Rec64) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(b.flip.get(), h.flip_step.get(), sizeof(int) * N, cudaMemcpyDeviceToDevice, h.st));
  if (h.xh.size() > 0) {
    if (!b.xh.alloc(h.xh.size()) || !b.bh.alloc(h.bh.size())) return set_error(NNPP_ERR_NOMEM, "backup");
    NNPP_CUDA(cudaMemcpyAsync(b.xh.get(), h.xh.get(), h.xh.bytes(), cudaMemcpyDeviceToDevice, h.st));
    NNPP_CUDA(cudaMemcpyAsync(b.bh.get(), h.bh.get(), h.bh.bytes(), cudaMemcpyDeviceToDevice, h.st));
  }
  NNPP_TRY(read_state(h, &b.ds));
  return NNPP_OK;
}

nnpp_status restore(Handle& h, StateBackup& b) {
  const size_t N = h.N;
  h.cur = b.cur;
  h.state_prec = b.prec;
  NNPP_CUDA(cudaMemcpyAsync(h.phi64.get(), b.phi.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.phi_prev.get(), b.phi_prev.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.clo.get(), b.clo.get(), sizeof(float4) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.rec32[h.cur].get(), b.rec32.get(), sizeof(Rec32) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.rec64[h.cur].get(), b.rec64.get(), sizeof(Rec64) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.flip_step.get(), b.flip.get(), sizeof(int) * N, cudaMemcpyDeviceToDevice, h.st));
  if (b.xh.size() > 0 && b.xh.size() == h.xh.size() && b.bh.size() == h.bh.size()) {
    NNPP_CUDA(cudaMemcpyAsync(h.xh.get(), b.xh.get(), h.xh.bytes(), cudaMemcpyDeviceToDevice, h.st));
    NNPP_CUDA(cudaMemcpyAsync(h.bh.get(), b.bh.get(), h.bh.bytes(), cudaMemcpyDeviceToDevice, h.st));
  }
  NNPP_CUDA(cudaMemcpyAsync(h.dstate.get(), &b.ds, sizeof(DevState), cudaMemcpyHostToDevice, h.st));
  h.settings_pushed = false;
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  if (h.engine) NNPP_TRY(engine_params(*h.engine));
  return NNPP_OK;
}

// Upload user-order c (S*N), phi (N, may be NULL), phase (N, may be NULL) into the current
// buffers in precision prec.
nnpp_status upload_state(Handle& h, const double* c, const double* phi, const int* phase, int prec,
                         bool dirichlet_phi = true, bool keep_history = false) {
  const size_t N = h.N;
  NNPP_CUDA(cudaMemcpyAsync(h.user_stage.get(), c, sizeof(double) * S * N, cudaMemcpyHostToDevice, h.st));
  if (phi)
    NNPP_CUDA(cudaMemcpyAsync(h.user_stage.get() + S * N, phi, sizeof(double) * N, cudaMemcpyHostToDevice, h.st));
  if (phase)
    NNPP_CUDA(cudaMemcpyAsync(h.user_stage_i.get(), phase, sizeof(int) * N, cudaMemcpyHostToDevice, h.st));
  if (prec != h.state_prec && !phase) NNPP_TRY(convert_state(h, prec));
  return load_state(h, h.user_stage.get(), phi ? h.user_stage.get() + S * N : nullptr,
                    phase ? h.user_stage_i.get() : nullptr, prec, dirichlet_phi, keep_history);
}

// The initial state (main.cpp:398-420 with the given phase): concentrations and potential
// from the initial values, counters and diagnostics zeroed, no flipped node, no recorded run.
nnpp_status reset_initial(Handle& h) {
  const size_t N = h.N;
  DevState ds;
  std::memset(&ds, 0, sizeof(ds));
  ds.tol = h.tol;
  ds.max_iter = h.max_iter;
  ds.max_outer = h.max_outer;
  ds.inner_rel = h.inner_rel;
  NNPP_CUDA(cudaMemcpyAsync(h.dstate.get(), &ds, sizeof(DevState), cudaMemcpyHostToDevice, h.st));
  h.settings_pushed = false;
  h.cur = 0;
  NNPP_TRY(upload_state(h, h.h_ic.data(), h.h_ic.data() + S * N, h.h_phase0.data(), NNPP_FP64));
  NNPP_CUDA(cudaMemsetAsync(h.flip_step.get(), 0xff, sizeof(int) * N, h.st));
  NNPP_TRY(init_diag(h));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  h.fwd_steps = 0;
  h.ckpts.clear();
  h.nstep = 0;
  if (h.engine) NNPP_TRY(engine_params(*h.engine));
  return NNPP_OK;
}

// single-instance view of h's engine with a private KParams block (in_graph = 0)
struct OneView {
  DBuf<KParams> kp;
  EngineView v;
};

nnpp_status one_view(Handle& h, const KParams& k, OneView& ov) {
  if (!ov.kp.alloc(1)) return set_error(NNPP_ERR_NOMEM, "view");
  NNPP_CUDA(cudaMemcpyAsync(ov.kp.get(), &k, sizeof(KParams), cudaMemcpyHostToDevice, h.st));
  ov.v = make_view(*h.engine, 0, 0);
  ov.v.inst = ov.kp.get();
  return NNPP_OK;
}

}  // namespace

// ======================================================================== C ABI ==========
extern "C" {

int nnpp_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

nnpp_status nnpp_set_device(int device) {
  clear_error();
  if (device < 0 || device >= nnpp_device_count()) return set_error(NNPP_ERR_INVALID, "no such device");
  NNPP_CUDA(cudaSetDevice(device));
  return NNPP_OK;
}

nnpp_status nnpp_params_from_reference(const double* data2, const double* datac1, const double* datac2,
                                       const double* datac3, const double* datac4,
                                       const double* datac11, double k_diss, double switch_width,
                                       nnpp_params* out) {
  clear_error();
  if (!data2 || !datac1 || !datac2 || !datac3 || !datac4 || !datac11 || !out)
    return set_error(NNPP_ERR_INVALID, "params_from_reference: NULL input");
  std::memset(out, 0, sizeof(*out));
  // utils.h:2346-2395
  out->dt = data2[2];
  out->dx = data2[3];
  out->dy = data2[4];
  out->dz = data2[5];
  out->delta = data2[6];
  out->CSolid = data2[7];
  out->CSat = data2[8];
  out->T = data2[47];
  out->R = data2[48];
  out->F = data2[49];
  out->vol_red = data2[50];
  const double* dc[4] = {datac1, datac2, datac3, datac4};
  for (int s = 0; s < S; ++s) {  // utils.h:2397-2423
    out->z[s] = dc[s][0];
    out->D_solid[s] = dc[s][1];
    out->D_liquid[s] = dc[s][2];
    out->s1[s] = dc[s][3];
    out->s2[s] = dc[s][4];
    out->K1[s] = dc[s][5];
    out->K2[s] = dc[s][6];
  }
  out->sigma = datac11[1];  // utils.h:2480-2483
  out->s_phi = datac11[2];
  out->K_phi = datac11[3];
  out->k_diss = k_diss;
  out->switch_width = switch_width;
  out->c_floor = 1.0e-8 / out->CSolid;  // main.cpp:806
  out->sub_step_no = 8;                 // main.cpp:39
  return NNPP_OK;
}

nnpp_status nnpp_build_clouds_hash(int max_node_no, double r, double dx, double dy, double dz,
                                   int n_nodes, const double* nodes_colmajor, int order_mode,
                                   int* clouds_colmajor, int* cloud_lengths, int* max_cloud_length) {
  clear_error();
  if (n_nodes <= 0 || !nodes_colmajor) return set_error(NNPP_ERR_INVALID, "no nodes");
  if (!have_gpu()) return set_error(NNPP_ERR_CUDA, "no CUDA device");
  cudaStream_t st;
  NNPP_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  nnpp_status res = NNPP_OK;
  {
    DBuf<double> xyz;
    RefLists L;
    if (!xyz.alloc(3 * (size_t)n_nodes)) {
      res = set_error(NNPP_ERR_NOMEM, "nodes");
    } else {
      cudaMemcpyAsync(xyz.get(), nodes_colmajor, sizeof(double) * 3 * (size_t)n_nodes,
                      cudaMemcpyHostToDevice, st);
      res = build_ref_lists(st, n_nodes, xyz.get(), xyz.get() + n_nodes, xyz.get() + 2 * (size_t)n_nodes,
                            max_node_no, r, dx, dy, dz, order_mode, L);
      if (res == NNPP_OK) res = emit_padded(st, L, max_node_no, clouds_colmajor, cloud_lengths);
      if (res == NNPP_OK && max_cloud_length) *max_cloud_length = L.max_len;
    }
    cudaStreamSynchronize(st);
  }
  cudaStreamDestroy(st);
  return res;
}

nnpp_status nnpp_create(nnpp_handle** out, const nnpp_params* p, int n_nodes,
                        const double* nodes_colmajor, const int* bctypes, const double* bcvalues,
                        const double* icvalues, const int* phase0) {
  clear_error();
  if (!out) return set_error(NNPP_ERR_INVALID, "out is NULL");
  *out = nullptr;
  NNPP_TRY(check_params(p));
  if (n_nodes <= 0 || !nodes_colmajor || !bctypes || !bcvalues || !icvalues)
    return set_error(NNPP_ERR_INVALID, "create: missing inputs");
  if (!have_gpu()) return set_error(NNPP_ERR_CUDA, "no CUDA device");
  for (size_t i = 0; i < 3 * (size_t)n_nodes; ++i)
    if (!std::isfinite(nodes_colmajor[i])) return set_error(NNPP_ERR_INVALID, "non-finite node coordinate");
  nnpp_handle* hp = new nnpp_handle();
  Handle& h = hp->h;
  h.p = *p;
  h.N = n_nodes;
  cudaGetDevice(&h.device);
  auto fail = [&](nnpp_status st) {
    nnpp_destroy(hp);
    return st;
  };
  if (cudaStreamCreateWithFlags(&h.st, cudaStreamNonBlocking) != cudaSuccess)
    return fail(set_error(NNPP_ERR_CUDA, "stream creation"));
  const size_t N = n_nodes;
  if (!h.ux.alloc(N) || !h.uy.alloc(N) || !h.uz.alloc(N)) return fail(set_error(NNPP_ERR_NOMEM, "nodes"));
  if (cudaMemcpyAsync(h.ux.get(), nodes_colmajor, sizeof(double) * N, cudaMemcpyHostToDevice, h.st) ||
      cudaMemcpyAsync(h.uy.get(), nodes_colmajor + N, sizeof(double) * N, cudaMemcpyHostToDevice, h.st) ||
      cudaMemcpyAsync(h.uz.get(), nodes_colmajor + 2 * N, sizeof(double) * N, cudaMemcpyHostToDevice, h.st) ||
      cudaStreamSynchronize(h.st))
    return fail(set_error(NNPP_ERR_CUDA, "node upload"));
  h.h_bctypes.assign(bctypes, bctypes + N);
  h.h_bcv.assign(bcvalues, bcvalues + (S + 1) * N);
  h.h_ic.assign(icvalues, icvalues + (S + 1) * N);
  h.h_phase0.resize(N);
  for (size_t i = 0; i < N; ++i)
    h.h_phase0[i] = phase0 ? (phase0[i] != 0 ? 1 : 0) : (icvalues[i] > 0.0 + 10E-6 ? 1 : 0);
  *out = hp;
  return NNPP_OK;
}

nnpp_status nnpp_destroy(nnpp_handle* hp) {
  if (!hp) return NNPP_OK;
  Handle& h = hp->h;
  cudaSetDevice(h.device);
  if (h.st) cudaStreamSynchronize(h.st);
  if (h.engine) {
    delete h.engine;
    h.engine = nullptr;
  }
  cudaStream_t st = h.st;
  delete hp;
  if (st) cudaStreamDestroy(st);
  return NNPP_OK;
}

nnpp_status nnpp_build_neighbours(nnpp_handle* hp, int max_node_no, double r, double cx, double cy,
                                  double cz, int order_mode, int* clouds_colmajor, int* cloud_lengths,
                                  int* max_cloud_length) {
  nnpp::TraceRange trace_("nnpp_build_neighbours");
  NNPP_GUARD(hp);
  Handle& h = hp->h;
  if (h.engine) {
    delete h.engine;
    h.engine = nullptr;
  }
  h.built = false;
  NNPP_TRY(build_ref_lists(h.st, h.N, h.ux.get(), h.uy.get(), h.uz.get(), max_node_no, r, cx, cy, cz,
                           order_mode, h.ref));
  h.max_node_no = max_node_no;
  NNPP_TRY(emit_padded(h.st, h.ref, max_node_no, clouds_colmajor, cloud_lengths));
  if (max_cloud_length) *max_cloud_length = h.ref.max_len;
  const nnpp_params& p = h.p;
  // bins of side h32 >= r (an FP32 value, so that tile-relative FP32 coordinates are exact
  // multiples of it): every neighbour lies in an adjacent bin
  const double want = r * (1.0 + 1e-7);
  float h32 = (float)want;
  while ((double)h32 < want) h32 = nextafterf(h32, INFINITY);
  h.h32 = h32;
  NNPP_TRY(build_layout(h.st, h.ref, h.ux.get(), h.uy.get(), h.uz.get(), (double)h32, p.delta, p.dx,
                        p.dx * p.dy * p.dz, p.s_phi, h.lay));
  NNPP_TRY(step_alloc(h));
  // per-node constants in internal order (main.cpp:676-712: Dirichlet where bctypes == 0
  // and bcvalues != -1; species values divided by CSolid, the potential's not)
  const size_t N = h.N;
  std::vector<int> perm(N);
  NNPP_CUDA(cudaMemcpyAsync(perm.data(), h.lay.perm.get(), sizeof(int) * N, cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  std::vector<unsigned char> dm(N, 0);
  std::vector<double> bcv((S + 1) * N, 0.0);
  for (size_t a = 0; a < N; ++a) {
    const int u = perm[a];
    for (int f = 0; f <= S; ++f) {
      const double v = h.h_bcv[(size_t)f * N + u];
      if (h.h_bctypes[u] == 0 && v != -1) {
        dm[a] |= (unsigned char)(1u << f);
        bcv[(size_t)f * N + a] = (f < S) ? v / p.CSolid : v;
      }
    }
  }
  NNPP_CUDA(cudaMemcpyAsync(h.dirmask.get(), dm.data(), N, cudaMemcpyHostToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.bcval.get(), bcv.data(), sizeof(double) * (S + 1) * N, cudaMemcpyHostToDevice, h.st));
  NNPP_TRY(reset_initial(h));
  h.built = true;
  h.engine = new Engine();
  h.engine->members.push_back(&h);
  h.engine->st = h.st;
  nnpp_status st = engine_build(*h.engine);
  if (st == NNPP_OK) st = coarse_build(h);
  if (st != NNPP_OK) {
    h.built = false;
    return st;
  }
  return NNPP_OK;
}

nnpp_status nnpp_get_neighbours_csr(nnpp_handle* hp, int* row_ptr, int* cols, int64_t* nnz_out) {
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  Handle& h = hp->h;
  if (nnz_out) *nnz_out = h.ref.nnz;
  if (row_ptr)
    NNPP_CUDA(cudaMemcpyAsync(row_ptr, h.ref.ptr.get(), sizeof(int) * (h.N + 1), cudaMemcpyDeviceToHost, h.st));
  if (cols && h.ref.nnz > 0)
    NNPP_CUDA(cudaMemcpyAsync(cols, h.ref.col.get(), sizeof(int) * h.ref.nnz, cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  return NNPP_OK;
}

nnpp_status nnpp_set_solver(nnpp_handle* hp, double tol, int max_iter, int strict) {
  NNPP_GUARD(hp);
  if (!(tol > 0) || max_iter < 1) return set_error(NNPP_ERR_INVALID, "tol must be > 0, max_iter >= 1");
  Handle& h = hp->h;
  h.tol = tol;
  h.max_iter = max_iter;
  h.strict = strict;
  h.settings_pushed = false;
  return NNPP_OK;
}

nnpp_status nnpp_set_refinement(nnpp_handle* hp, double inner_rel, int max_outer) {
  NNPP_GUARD(hp);
  if (!(inner_rel > 0.0) || !(inner_rel < 1.0) || max_outer < 1)
    return set_error(NNPP_ERR_INVALID, "refinement: inner_rel in (0, 1), max_outer >= 1");
  Handle& h = hp->h;
  h.inner_rel = inner_rel;
  h.max_outer = max_outer;
  h.settings_pushed = false;
  return NNPP_OK;
}

nnpp_status nnpp_forward(nnpp_handle* hp, int n_steps, int precision) {
  nnpp::TraceRange trace_("nnpp_forward");
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  if (n_steps < 0) return set_error(NNPP_ERR_INVALID, "n_steps < 0");
  if (precision != NNPP_FP64 && precision != NNPP_MIXED) return set_error(NNPP_ERR_INVALID, "precision");
  Handle& h = hp->h;
  DevState before;
  NNPP_TRY(read_state(h, &before));
  NNPP_TRY(engine_run(*h.engine, n_steps, precision));
  return check_after(h, before.cg_nc);
}

nnpp_status nnpp_get_state(nnpp_handle* hp, double* c, double* phi, int* phase) {
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  Handle& h = hp->h;
  const size_t N = h.N;
  NNPP_TRY(store_state(h, h.user_stage.get(), h.user_stage.get() + S * N, h.user_stage_i.get()));
  if (c) NNPP_CUDA(cudaMemcpyAsync(c, h.user_stage.get(), sizeof(double) * S * N, cudaMemcpyDeviceToHost, h.st));
  if (phi)
    NNPP_CUDA(cudaMemcpyAsync(phi, h.user_stage.get() + S * N, sizeof(double) * N, cudaMemcpyDeviceToHost, h.st));
  if (phase) NNPP_CUDA(cudaMemcpyAsync(phase, h.user_stage_i.get(), sizeof(int) * N, cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  return NNPP_OK;
}

nnpp_status nnpp_set_state(nnpp_handle* hp, const double* c, const double* phi, const int* phase) {
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  if (!c) return set_error(NNPP_ERR_INVALID, "c is NULL");
  Handle& h = hp->h;
  NNPP_TRY(upload_state(h, c, phi, phase, h.state_prec));
  // the relative volume and the interface factor of the new state, as after the reference's
  // restart from file (main.cpp:527-533); vol0rel stays the initial state's
  NNPP_TRY(init_diag(h, true));
  h.coarse.stale = true;
  h.nstep = 0;
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  return NNPP_OK;
}

nnpp_status nnpp_get_diagnostics(nnpp_handle* hp, nnpp_diag* out) {
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  if (!out) return set_error(NNPP_ERR_INVALID, "out is NULL");
  Handle& h = hp->h;
  DevState ds;
  NNPP_TRY(read_state(h, &ds));
  const double dV = h.p.dx * h.p.dy * h.p.dz;
  std::memset(out, 0, sizeof(*out));
  out->steps_done = ds.steps;
  out->solid_count = ds.solid_count;
  out->voln1rel = ds.voln1rel;
  out->vol0rel = ds.vol0rel;
  for (int s = 0; s < S; ++s) out->mass[s] = ds.mass[s] * dV;
  out->mg_mass_lost = (ds.mg_mass_t0 - ds.mg_mass_now) * dV;
  out->dissolved_total = ds.dissolved * h.p.dt * dV;
  out->cg_iterations_total = ds.cg_iters;
  out->cg_solves = ds.cg_solves;
  out->cg_not_converged = ds.cg_nc;
  out->last_rel_residual = ds.last_relres;
  out->outer_iterations_total = ds.outer_total;
  return NNPP_OK;
}

nnpp_status nnpp_get_flip_steps(nnpp_handle* hp, int* flip_step) {
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  if (!flip_step) return set_error(NNPP_ERR_INVALID, "flip_step is NULL");
  Handle& h = hp->h;
  const size_t N = h.N;
  std::vector<int> perm(N), fs(N);
  NNPP_CUDA(cudaMemcpyAsync(perm.data(), h.lay.perm.get(), sizeof(int) * N, cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaMemcpyAsync(fs.data(), h.flip_step.get(), sizeof(int) * N, cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  for (size_t a = 0; a < N; ++a) flip_step[perm[a]] = fs[a];
  return NNPP_OK;
}

nnpp_status nnpp_step_host(nnpp_handle* hp, int precision, const double* c_in, const int* phase_in,
                           double* c_out, double* phi_out, int* phase_out) {
  nnpp::TraceRange trace_("nnpp_step_host");
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  if (precision != NNPP_FP64 && precision != NNPP_MIXED) return set_error(NNPP_ERR_INVALID, "precision");
  if (!c_in) return set_error(NNPP_ERR_INVALID, "c_in is NULL");
  Handle& h = hp->h;
  DevState before;
  NNPP_TRY(read_state(h, &before));
  NNPP_TRY(upload_state(h, c_in, nullptr, phase_in, precision, true, true));
  NNPP_TRY(engine_run(*h.engine, 1, precision));
  const size_t N = h.N;
  NNPP_TRY(store_state(h, h.user_stage.get(), h.user_stage.get() + S * N, h.user_stage_i.get()));
  if (c_out) NNPP_CUDA(cudaMemcpyAsync(c_out, h.user_stage.get(), sizeof(double) * S * N, cudaMemcpyDeviceToHost, h.st));
  if (phi_out)
    NNPP_CUDA(cudaMemcpyAsync(phi_out, h.user_stage.get() + S * N, sizeof(double) * N, cudaMemcpyDeviceToHost, h.st));
  if (phase_out)
    NNPP_CUDA(cudaMemcpyAsync(phase_out, h.user_stage_i.get(), sizeof(int) * N, cudaMemcpyDeviceToHost, h.st));
  return check_after(h, before.cg_nc);
}

nnpp_status nnpp_residuals(nnpp_handle* hp, int precision, const double* c, const double* phi,
                           const int* phase, double voln1rel, double* F) {
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  if (!c || !phi || !phase || !F) return set_error(NNPP_ERR_INVALID, "residuals: NULL argument");
  if (precision != NNPP_FP64 && precision != NNPP_MIXED) return set_error(NNPP_ERR_INVALID, "precision");
  Handle& h = hp->h;
  NNPP_TRY(engine_warm(*h.engine, precision));
  StateBackup b;
  NNPP_TRY(backup(h, b));
  nnpp_status st = upload_state(h, c, phi, phase, precision, false);
  DBuf<double> Fd;
  OneView ov;
  if (st == NNPP_OK && !Fd.alloc((S + 1) * (size_t)h.N)) st = set_error(NNPP_ERR_NOMEM, "residual output");
  if (st == NNPP_OK) {
    const double bv = std::pow(10., -h.p.vol_red * (1. - voln1rel));  // utils.h:100-116
    NNPP_CUDA(cudaMemcpyAsync(h.scratch_d.get(), &bv, sizeof(double), cudaMemcpyHostToDevice, h.st));
    KParams kp = make_kparams(h, h.cur);
    kp.bv_ptr = h.scratch_d.get();
    st = one_view(h, kp, ov);
    if (st == NNPP_OK) st = launch_transport_b(*h.engine, ov.v, precision, h.st, Fd.get());
    if (st == NNPP_OK) st = launch_prep_b(*h.engine, ov.v, precision, h.st, 0, Fd.get() + (size_t)S * h.N);
    if (st == NNPP_OK) {
      k_unpermute<<<h.grid, kBlockHost, 0, h.st>>>(h.lay.perm.get(), h.N, S + 1, Fd.get(), h.user_stage.get());
      if (cudaGetLastError() != cudaSuccess) st = set_error(NNPP_ERR_CUDA, "unpermute");
    }
    if (st == NNPP_OK)
      NNPP_CUDA(cudaMemcpyAsync(F, h.user_stage.get(), sizeof(double) * (S + 1) * h.N, cudaMemcpyDeviceToHost, h.st));
    cudaStreamSynchronize(h.st);
  }
  nnpp_status st2 = restore(h, b);
  return st != NNPP_OK ? st : st2;
}

nnpp_status nnpp_solve_potential(nnpp_handle* hp, int precision, const double* c, const int* phase,
                                 double* phi, int* iterations, double* rel_residual) {
  nnpp::TraceRange trace_("nnpp_solve_potential");
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  if (!c || !phase || !phi) return set_error(NNPP_ERR_INVALID, "solve_potential: NULL argument");
  if (precision != NNPP_FP64 && precision != NNPP_MIXED) return set_error(NNPP_ERR_INVALID, "precision");
  Handle& h = hp->h;
  StateBackup b;
  NNPP_TRY(backup(h, b));
  nnpp_status st = upload_state(h, c, phi, phase, precision);
  DevState ds0, ds1;
  if (st == NNPP_OK) st = read_state(h, &ds0);
  if (st == NNPP_OK) st = engine_solve(*h.engine, precision);
  if (st == NNPP_OK) st = read_state(h, &ds1);
  if (st == NNPP_OK) {
    k_unpermute<<<h.grid, kBlockHost, 0, h.st>>>(h.lay.perm.get(), h.N, 1, h.phi64.get(), h.user_stage.get());
    if (cudaGetLastError() != cudaSuccess) st = set_error(NNPP_ERR_CUDA, "unpermute");
    if (st == NNPP_OK) {
      NNPP_CUDA(cudaMemcpyAsync(phi, h.user_stage.get(), sizeof(double) * h.N, cudaMemcpyDeviceToHost, h.st));
      NNPP_CUDA(cudaStreamSynchronize(h.st));
    }
    if (iterations) *iterations = (int)(ds1.cg_iters - ds0.cg_iters);
    if (rel_residual) *rel_residual = ds1.last_relres;
    if (st == NNPP_OK && h.strict && ds1.cg_nc > ds0.cg_nc)
      st = set_error(NNPP_ERR_CG_NO_CONVERGE, "potential solve hit its iteration cap");
  }
  nnpp_status st2 = restore(h, b);
  return st != NNPP_OK ? st : st2;
}

nnpp_status nnpp_forward_timed(nnpp_handle* hp, int n_steps, int precision, double* ms) {
  nnpp::TraceRange trace_("nnpp_forward_timed");
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  if (n_steps < 0 || !ms) return set_error(NNPP_ERR_INVALID, "forward_timed: bad argument");
  if (precision != NNPP_FP64 && precision != NNPP_MIXED) return set_error(NNPP_ERR_INVALID, "precision");
  Handle& h = hp->h;
  DevState before;
  NNPP_TRY(read_state(h, &before));
  NNPP_TRY(engine_warm(*h.engine, precision));
  cudaEvent_t e0, e1;
  NNPP_CUDA(cudaEventCreate(&e0));
  NNPP_CUDA(cudaEventCreate(&e1));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  cudaEventRecord(e0, h.st);
  nnpp_status st = engine_run(*h.engine, n_steps, precision, true);
  cudaEventRecord(e1, h.st);
  cudaEventSynchronize(e1);
  float f = 0.0f;
  cudaEventElapsedTime(&f, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = f;
  NNPP_TRY(st);
  return check_after(h, before.cg_nc);
}

// kernel_id: 0 transport (bond sums), 1 CG SpMV (matrix-vector product on the
// liquid-liquid graph), 2 FP64 refinement residual.  The state is restored afterwards.
nnpp_status nnpp_time_kernel(nnpp_handle* hp, int kernel_id, int precision, int reps,
                             double* ms_per_launch) {
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  if (reps < 1 || !ms_per_launch || kernel_id < 0 || kernel_id > 6)
    return set_error(NNPP_ERR_INVALID, "time_kernel: bad argument");
  if (precision != NNPP_FP64 && precision != NNPP_MIXED) return set_error(NNPP_ERR_INVALID, "precision");
  Handle& h = hp->h;
  NNPP_TRY(engine_warm(*h.engine, precision));
  StateBackup b;
  NNPP_TRY(backup(h, b));
  Engine& e = *h.engine;
  EngineView v = make_view(e, 0, 0);
  nnpp_status st = launch_prep_b(e, v, precision, h.st, 0, nullptr);
  // every instance active so that the timed kernels do their full work
  DevState ds;
  if (st == NNPP_OK) st = read_state(h, &ds);
  ds.outer_active = 1;
  ds.inner_active = 1;
  ds.tol = 0.0;            // keep the refinement kernel's instance active across repetitions
  ds.max_outer = 1 << 30;
  if (st == NNPP_OK) {
    cudaMemcpyAsync(h.dstate.get(), &ds, sizeof(DevState), cudaMemcpyHostToDevice, h.st);
    st = launch_cg_init_b(e, v, precision, h.st, 0);
  }
  if (st == NNPP_OK) {
    ds.outer_active = 1;
    ds.inner_active = 1;
    cudaMemcpyAsync(&h.dstate.get()->outer_active, &ds.outer_active, 2 * sizeof(int), cudaMemcpyHostToDevice, h.st);
    static const double zero = 0.0;  // the CG update's stop test must not end the repetitions
    cudaMemcpyAsync(&h.dstate.get()->inner_target, &zero, sizeof(double), cudaMemcpyHostToDevice, h.st);
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto one = [&]() -> nnpp_status {
    if (kernel_id == 0) return launch_transport_b(e, v, precision, h.st, nullptr);
    if (kernel_id == 1) return launch_cg_spmv_b(e, v, precision, h.st);
    if (kernel_id == 3) return launch_cg_update_b(e, v, precision, h.st, 0);
    if (kernel_id >= 4) return launch_coarse_part_b(e, v, precision, kernel_id - 4, h.st);
    return launch_ir_update_b(e, v, precision, h.st, 0);
  };
  for (int w = 0; w < 3 && st == NNPP_OK; ++w) st = one();
  if (st == NNPP_OK) {
    cudaMemcpyAsync(&h.dstate.get()->outer_active, &ds.outer_active, 2 * sizeof(int), cudaMemcpyHostToDevice, h.st);
    cudaEventRecord(e0, h.st);
    for (int r = 0; r < reps && st == NNPP_OK; ++r) st = one();
    cudaEventRecord(e1, h.st);
    cudaEventSynchronize(e1);
    float f = 0.0f;
    cudaEventElapsedTime(&f, e0, e1);
    *ms_per_launch = (double)f / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  nnpp_status st2 = restore(h, b);
  return st != NNPP_OK ? st : st2;
}

nnpp_status nnpp_set_warm_start(nnpp_handle* hp, int history) {
  NNPP_GUARD(hp);
  if (history < 0 || history > kHistMax)
    return set_error(NNPP_ERR_INVALID, "warm start history must be in [0, 6]");
  Handle& h = hp->h;
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  h.extrapolate = history >= 1 ? 1 : 0;
  h.warm_hist = history >= 3 ? history : 0;
  h.xh.reset();
  h.bh.reset();
  if (h.warm_hist && h.built) {
    const size_t HN = (size_t)h.warm_hist * h.N;
    if (!h.xh.alloc(HN) || !h.bh.alloc(HN)) return set_error(NNPP_ERR_NOMEM, "warm-start history");
  }
  h.fwd_steps = 0;
  h.ckpts.clear();
  if (h.built) {
    static const int zero = 0;
    NNPP_CUDA(cudaMemcpyAsync(&h.dstate.get()->hist_n, &zero, sizeof(int), cudaMemcpyHostToDevice, h.st));
    NNPP_CUDA(cudaMemcpyAsync(&h.dstate.get()->hist_head, &zero, sizeof(int), cudaMemcpyHostToDevice, h.st));
    NNPP_CUDA(cudaStreamSynchronize(h.st));
  }
  if (h.engine) {
    engine_destroy_graphs(*h.engine);
    NNPP_TRY(engine_params(*h.engine));
  }
  return NNPP_OK;
}

nnpp_status nnpp_reset(nnpp_handle* hp) {
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  NNPP_TRY(reset_initial(hp->h));
  hp->h.coarse.stale = true;
  return NNPP_OK;
}

nnpp_status nnpp_set_preconditioner(nnpp_handle* hp, int kind, int refresh_every) {
  NNPP_GUARD(hp);
  if (kind != NNPP_PRECOND_JACOBI && kind != NNPP_PRECOND_TWO_LEVEL)
    return set_error(NNPP_ERR_INVALID, "preconditioner: 0 (Jacobi) or 1 (two-level)");
  if (refresh_every < 0) return set_error(NNPP_ERR_INVALID, "preconditioner: refresh_every < 0");
  Handle& h = hp->h;
  NNPP_CUDA(cudaSetDevice(h.device));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  const bool want = kind == NNPP_PRECOND_TWO_LEVEL;
  if (refresh_every != h.coarse_every) {
    h.coarse_every = refresh_every;
    h.fwd_steps = 0;
    h.ckpts.clear();
  }
  if (want == h.coarse_enabled) return NNPP_OK;
  h.coarse_enabled = want;
  h.coarse.valid = false;
  h.coarse.stale = true;
  h.fwd_steps = 0;
  h.ckpts.clear();
  if (h.built) {
    if (want && h.coarse.n == 0) NNPP_TRY(coarse_build(h));
    if (h.engine) NNPP_TRY(engine_params(*h.engine));
  }
  return NNPP_OK;
}

nnpp_status nnpp_get_preconditioner(nnpp_handle* hp, int* kind, int* coarse_unknowns, int* refresh_every,
                                    int64_t* rebuilds) {
  NNPP_GUARD(hp);
  const Handle& h = hp->h;
  if (kind) *kind = h.coarse_enabled ? NNPP_PRECOND_TWO_LEVEL : NNPP_PRECOND_JACOBI;
  if (coarse_unknowns) *coarse_unknowns = h.coarse_enabled ? h.coarse.n : 0;
  if (refresh_every) *refresh_every = h.coarse_every;
  if (rebuilds) *rebuilds = h.coarse.rebuilds;
  return NNPP_OK;
}

nnpp_status nnpp_set_checks(nnpp_handle* hp, int flags) {
  NNPP_GUARD(hp);
  if (flags & ~(NNPP_CHECK_BOUNDS | NNPP_CHECK_WAIT_PROBE))
    return set_error(NNPP_ERR_INVALID, "set_checks: unknown flag");
  Handle& h = hp->h;
  NNPP_CUDA(cudaSetDevice(h.device));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  h.checks = flags;
  if (h.engine && h.built) NNPP_TRY(engine_params(*h.engine));
  return NNPP_OK;
}

nnpp_status nnpp_set_transport_variant(nnpp_handle* hp, int variant) {
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  if (variant < 0 || variant > kTrVariants - 1)
    return set_error(NNPP_ERR_INVALID, "set_transport_variant: 0 or 1");
  Handle& h = hp->h;
  Engine& e = *h.engine;
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  if (variant > 0 && !transport_halo_fits(e))
    return set_error(NNPP_ERR_UNSUPPORTED, "set_transport_variant: a tile halo exceeds a CTA's shared memory");
  e.tr_variant = variant;
  engine_destroy_graphs(e);  // the captured steps launch the previous kernel
  return NNPP_OK;
}

nnpp_status nnpp_get_coarse_stats(nnpp_handle* hp, int64_t* rebuilds, int64_t* warm_rebuilds,
                                  int64_t* run_rebuilds, double* run_rebuild_ms, int* last_ns_steps) {
  NNPP_GUARD(hp);
  const Coarse& c = hp->h.coarse;
  if (rebuilds) *rebuilds = c.rebuilds;
  if (warm_rebuilds) *warm_rebuilds = c.warm_rebuilds;
  if (run_rebuilds) *run_rebuilds = c.timed_rebuilds;
  if (run_rebuild_ms) *run_rebuild_ms = c.rebuild_ms;
  if (last_ns_steps) *last_ns_steps = c.ns_steps;
  return NNPP_OK;
}

nnpp_status nnpp_set_params(nnpp_handle* hp, const nnpp_params* p) {
  NNPP_GUARD(hp);
  NNPP_TRY(check_params(p));
  Handle& h = hp->h;
  const nnpp_params& o = h.p;
  bool same = p->dx == o.dx && p->dy == o.dy && p->dz == o.dz && p->delta == o.delta &&
              p->s_phi == o.s_phi && p->CSolid == o.CSolid;
  for (int s = 0; s < S; ++s) same = same && p->s1[s] == o.s1[s] && p->s2[s] == o.s2[s];
  if (!same)
    return set_error(NNPP_ERR_INVALID, "set_params: geometry fields or CSolid differ from the handle's");
  NNPP_CUDA(cudaSetDevice(h.device));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  h.p = *p;
  h.fwd_steps = 0;
  h.ckpts.clear();
  if (h.engine) NNPP_TRY(engine_params(*h.engine));
  return NNPP_OK;
}

nnpp_status nnpp_get_tuning(nnpp_handle* hp, int* bins_per_tile, int* lanes_per_node,
                            int* cg_operator) {
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  const Engine& e = *hp->h.engine;
  if (bins_per_tile) *bins_per_tile = e.tuned ? e.T : 0;
  if (lanes_per_node) *lanes_per_node = e.tuned ? e.W : 0;
  if (cg_operator) *cg_operator = e.tuned ? e.spmv_variant : -1;
  return NNPP_OK;
}

nnpp_status nnpp_set_tuning(nnpp_handle* hp, int bins_per_tile, int lanes_per_node, int cg_operator) {
  NNPP_GUARD(hp);
  NNPP_NEED_BUILT(hp);
  const int T = bins_per_tile, W = lanes_per_node;
  if ((T != 2 && T != 4 && T != 8 && T != 16) || (W != 4 && W != 8 && W != 16) ||
      cg_operator < 0 || cg_operator >= kSpmvVariants)
    return set_error(NNPP_ERR_INVALID, "set_tuning: bins per tile in {2,4,8,16}, lanes in {4,8,16}, operator 0..8");
  Handle& h = hp->h;
  Engine& e = *h.engine;
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  NNPP_TRY(engine_set_tiles(e, T));
  NNPP_TRY(prepare_kernels(e.halo_max, e.bond_max, W));
  if (spmv_needs_windows(cg_operator) && !spmv_staged_fits(e))
    return set_error(NNPP_ERR_UNSUPPORTED, "set_tuning: a slice window exceeds the staged operators' capacity");
  if (cg_operator == kSpmvHalo && !spmv_halo_fits(e))
    return set_error(NNPP_ERR_UNSUPPORTED,
                     "set_tuning: the halo-staged operator needs s = 0, tiles of at most 8 bins and a "
                     "tile halo and code block within a CTA's shared memory");
  e.W = W;
  e.spmv_variant = cg_operator;
  e.tuned = true;
  NNPP_TRY(engine_params(e));
  return NNPP_OK;
}

// ---- ensembles ------------------------------------------------------------------------------
nnpp_status nnpp_ensemble_create(nnpp_ensemble** out, nnpp_handle* const* members, int n) {
  clear_error();
  if (!out || !members || n < 1) return set_error(NNPP_ERR_INVALID, "ensemble: no members");
  *out = nullptr;
  nnpp_ensemble* es = new nnpp_ensemble();
  for (int i = 0; i < n; ++i) {
    if (!members[i] || !members[i]->h.built) {
      delete es;
      return set_error(NNPP_ERR_STATE, "ensemble member without neighbour lists");
    }
    for (int j = 0; j < i; ++j)
      if (members[j] == members[i]) {
        delete es;
        return set_error(NNPP_ERR_INVALID, "ensemble: a handle appears twice");
      }
    es->members.push_back(members[i]);
    es->e.members.push_back(&members[i]->h);
  }
  if (cudaSetDevice(es->e.members[0]->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&es->e.st, cudaStreamNonBlocking) != cudaSuccess) {
    delete es;
    return set_error(NNPP_ERR_CUDA, "ensemble stream");
  }
  nnpp_status st = engine_build(es->e);
  if (st != NNPP_OK) {
    nnpp_ensemble_destroy(es);
    return st;
  }
  *out = es;
  return NNPP_OK;
}

nnpp_status nnpp_ensemble_forward(nnpp_ensemble* es, int n_steps, int precision) {
  clear_error();
  if (!es) return set_error(NNPP_ERR_INVALID, "ensemble is NULL");
  if (n_steps < 0) return set_error(NNPP_ERR_INVALID, "n_steps < 0");
  if (precision != NNPP_FP64 && precision != NNPP_MIXED) return set_error(NNPP_ERR_INVALID, "precision");
  NNPP_CUDA(cudaSetDevice(es->e.device));
  std::vector<long long> nc(es->members.size());
  for (size_t i = 0; i < es->members.size(); ++i) {
    DevState ds;
    NNPP_TRY(read_state(es->members[i]->h, &ds));
    nc[i] = ds.cg_nc;
  }
  NNPP_TRY(engine_run(es->e, n_steps, precision));
  for (size_t i = 0; i < es->members.size(); ++i) {
    Handle& h = es->members[i]->h;
    NNPP_TRY(check_after(h, nc[i]));
    if (h.engine) NNPP_TRY(engine_params(*h.engine));
  }
  return NNPP_OK;
}

nnpp_status nnpp_ensemble_forward_timed(nnpp_ensemble* es, int n_steps, int precision, double* ms) {
  clear_error();
  if (!es || !ms) return set_error(NNPP_ERR_INVALID, "ensemble_forward_timed: bad argument");
  NNPP_CUDA(cudaSetDevice(es->e.device));
  NNPP_TRY(engine_warm(es->e, precision));
  cudaEvent_t e0, e1;
  NNPP_CUDA(cudaEventCreate(&e0));
  NNPP_CUDA(cudaEventCreate(&e1));
  NNPP_CUDA(cudaStreamSynchronize(es->e.st));
  cudaEventRecord(e0, es->e.st);
  nnpp_status st = engine_run(es->e, n_steps, precision, true);
  cudaEventRecord(e1, es->e.st);
  cudaEventSynchronize(e1);
  float f = 0.0f;
  cudaEventElapsedTime(&f, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = f;
  NNPP_TRY(st);
  for (auto* m : es->members)
    if (m->h.engine) NNPP_TRY(engine_params(*m->h.engine));
  return NNPP_OK;
}

nnpp_status nnpp_ensemble_tuning(nnpp_ensemble* es, int* bins_per_tile, int* lanes_per_node) {
  clear_error();
  if (!es) return set_error(NNPP_ERR_INVALID, "ensemble is NULL");
  if (bins_per_tile) *bins_per_tile = es->e.T;
  if (lanes_per_node) *lanes_per_node = es->e.W;
  return NNPP_OK;
}

nnpp_status nnpp_ensemble_destroy(nnpp_ensemble* es) {
  if (!es) return NNPP_OK;
  cudaSetDevice(es->e.device);
  cudaStream_t st = es->e.st;
  if (st) cudaStreamSynchronize(st);
  delete es;
  if (st) cudaStreamDestroy(st);
  return NNPP_OK;
}

}  // extern "C"
