// engine.cu -- batched execution: work lists over one or many instances, the autotuner
// (bins per tile T, lanes per node W), CUDA-graph capture of the step with device-side loop
// control (conditional while nodes) and the run loop.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "engine.cuh"

namespace nnpp {

namespace {

nnpp_status push_settings(Handle& h) {
  if (h.settings_pushed) return NNPP_OK;
  DevState ds;
  NNPP_CUDA(cudaMemcpyAsync(&ds, h.dstate.get(), sizeof(DevState), cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  ds.tol = h.tol;
  ds.max_iter = h.max_iter;
  ds.max_outer = h.max_outer;
  ds.inner_rel = h.inner_rel;
  NNPP_CUDA(cudaMemcpyAsync(h.dstate.get(), &ds, sizeof(DevState), cudaMemcpyHostToDevice, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  h.settings_pushed = true;
  return NNPP_OK;
}

// KParams of every member for the current record parity (block 0) and the flipped one.
nnpp_status refresh_params(Engine& e) {
  const int M = (int)e.members.size();
  std::vector<KParams> k0(M), k1(M);
  for (int i = 0; i < M; ++i) {
    k0[i] = make_kparams(*e.members[i], e.members[i]->cur);
    k1[i] = make_kparams(*e.members[i], e.members[i]->cur ^ 1);
    k0[i].defl_ok = k1[i].defl_ok = M == 1 ? 1 : 0;
  }
  // pageable sources: the copies are staged before the calls return, and the kernels that
  // read the blocks are ordered after them on e.st
  NNPP_CUDA(cudaMemcpyAsync(e.d_inst[0].get(), k0.data(), sizeof(KParams) * M, cudaMemcpyHostToDevice, e.st));
  NNPP_CUDA(cudaMemcpyAsync(e.d_inst[1].get(), k1.data(), sizeof(KParams) * M, cudaMemcpyHostToDevice, e.st));
  return NNPP_OK;
}

nnpp_status sync_members(Engine& e) {
  for (Handle* h : e.members)
    if (h->st != e.st) NNPP_CUDA(cudaStreamSynchronize(h->st));
  return NNPP_OK;
}

// Work lists for bins-per-tile T (rebuilds every member's slots).
nnpp_status build_lists(Engine& e, int T) {
  const int M = (int)e.members.size();
  std::vector<TileDesc> tiles;
  std::vector<Chunk> chunks;
  std::vector<SliceDesc> slices;
  std::vector<HTile> htiles;
  std::vector<SliceDesc> cslices;
  std::vector<int> meta(8 * M);
  bool fit = true, hop = true;
  int hm = 0, bmax = 0, cmax = 0, qmax = 0;
  for (int i = 0; i < M; ++i) {
    Handle& h = *e.members[i];
    meta[i] = (int)tiles.size();
    int hmi = 0, bmi = 0;
    meta[4 * M + i] = (int)slices.size();
    bool wf = false;
    const int tile0 = (int)tiles.size();
    NNPP_TRY(build_tiles(h, T, tiles, slices, i, &hmi, &bmi, &wf));
    fit = fit && wf;
    int cmi = 0, qmi = 0;
    bool hok = false;
    NNPP_TRY(build_halo_op(h, T, tiles, tile0, htiles, &cmi, &qmi, &hok));
    hop = hop && hok;
    cmax = std::max(cmax, cmi);
    qmax = std::max(qmax, qmi);
    meta[5 * M + i] = (int)slices.size() - meta[4 * M + i];
    meta[6 * M + i] = (int)cslices.size();
    bool cf = false;
    NNPP_TRY(build_cg_slices(h, cslices, i, &cf));
    fit = fit && cf;
    meta[7 * M + i] = (int)cslices.size() - meta[6 * M + i];
    meta[M + i] = (int)tiles.size() - meta[i];
    hm = std::max(hm, hmi);
    bmax = std::max(bmax, bmi);
    meta[2 * M + i] = (int)chunks.size();
    for (int b = 0; b < h.N; b += kChunk) {
      Chunk c;
      c.inst = i;
      c.begin = b;
      c.end = std::min(h.N, b + kChunk);
      c.pad = 0;
      chunks.push_back(c);
    }
    meta[3 * M + i] = (int)chunks.size() - meta[2 * M + i];
  }
  e.ntiles = (int)tiles.size();
  e.nchunks = (int)chunks.size();
  e.nslices = (int)slices.size();
  e.ncslices = (int)cslices.size();
  e.windows_fit = fit;
  e.halo_op = hop;
  e.hcode_max16 = cmax;
  e.hquad_max = qmax;
  int wmax = 16;
  for (const SliceDesc& d : slices) wmax = std::max(wmax, d.wtotal);
  for (const SliceDesc& d : cslices) wmax = std::max(wmax, d.wtotal);
  e.win_cap = (wmax + 15) & ~15;
  e.halo_max = hm;
  e.bond_max = bmax;
  e.T = T;
  const int stride = std::max(std::max(e.ntiles, e.nchunks), std::max(e.nslices, e.ncslices));
  if (!e.d_tiles.alloc(tiles.size()) || !e.d_chunks.alloc(chunks.size()) || !e.d_meta.alloc(meta.size()) ||
      !e.d_slices.alloc(std::max<size_t>(slices.size(), 1)) || !e.d_htiles.alloc(std::max<size_t>(htiles.size(), 1)) ||
      !e.d_cslices.alloc(std::max<size_t>(cslices.size(), 1)) ||
      !e.d_ticket.alloc(M + 4) ||
      !e.d_partials.alloc((size_t)kReduceSlots * stride) ||
      !e.d_inst[0].alloc(M) || !e.d_inst[1].alloc(M))
    return set_error(NNPP_ERR_NOMEM, "engine work lists");
  NNPP_CUDA(cudaMemcpyAsync(e.d_tiles.get(), tiles.data(), sizeof(TileDesc) * tiles.size(), cudaMemcpyHostToDevice, e.st));
  NNPP_CUDA(cudaMemcpyAsync(e.d_chunks.get(), chunks.data(), sizeof(Chunk) * chunks.size(), cudaMemcpyHostToDevice, e.st));
  NNPP_CUDA(cudaMemcpyAsync(e.d_meta.get(), meta.data(), sizeof(int) * meta.size(), cudaMemcpyHostToDevice, e.st));
  if (!slices.empty())
    NNPP_CUDA(cudaMemcpyAsync(e.d_slices.get(), slices.data(), sizeof(SliceDesc) * slices.size(), cudaMemcpyHostToDevice, e.st));
  if (!htiles.empty())
    NNPP_CUDA(cudaMemcpyAsync(e.d_htiles.get(), htiles.data(), sizeof(HTile) * htiles.size(), cudaMemcpyHostToDevice, e.st));
  if (!cslices.empty())
    NNPP_CUDA(cudaMemcpyAsync(e.d_cslices.get(), cslices.data(), sizeof(SliceDesc) * cslices.size(), cudaMemcpyHostToDevice, e.st));
  NNPP_CUDA(cudaMemsetAsync(e.d_ticket.get(), 0, e.d_ticket.bytes(), e.st));
  NNPP_CUDA(cudaStreamSynchronize(e.st));
  engine_destroy_graphs(e);
  return NNPP_OK;
}

nnpp_status set_active(Engine& e, int outer, int inner) {
  NNPP_CUDA(cudaStreamSynchronize(e.st));
  for (Handle* h : e.members) {
    DevState ds;
    NNPP_CUDA(cudaMemcpyAsync(&ds, h->dstate.get(), sizeof(DevState), cudaMemcpyDeviceToHost, e.st));
    NNPP_CUDA(cudaStreamSynchronize(e.st));
    ds.outer_active = outer;
    ds.inner_active = inner;
    NNPP_CUDA(cudaMemcpyAsync(h->dstate.get(), &ds, sizeof(DevState), cudaMemcpyHostToDevice, e.st));
  }
  NNPP_CUDA(cudaStreamSynchronize(e.st));
  return NNPP_OK;
}

// Autotuner: bins per tile T and lanes per node W that minimise the CG operator on the
// current state (run tens of times per step) plus, for the mixed path, one FP64 tile
// operator (the refinement residual and the prep use the W lanes per node).
nnpp_status tune(Engine& e, int prec) {
  std::vector<DevState> saved(e.members.size());
  NNPP_CUDA(cudaStreamSynchronize(e.st));
  for (size_t i = 0; i < e.members.size(); ++i)
    NNPP_CUDA(cudaMemcpy(&saved[i], e.members[i]->dstate.get(), sizeof(DevState), cudaMemcpyDeviceToHost));
  const int Ts[4] = {2, 4, 8, 16};
  const int Ws[3] = {4, 8, 16};
  float best = 1e30f;
  int bT = 4, bW = 8;
  int bS = 0;
  cudaEvent_t e0, e1;
  NNPP_CUDA(cudaEventCreate(&e0));
  NNPP_CUDA(cudaEventCreate(&e1));
  for (int T : Ts) {
    const nnpp_status bs = build_lists(e, T);
    if (bs == NNPP_ERR_UNSUPPORTED) {
      clear_error();
      continue;
    }
    NNPP_TRY(bs);
    NNPP_TRY(refresh_params(e));
    for (int W : Ws) {
      e.W = W;
      if (prepare_kernels(e.halo_max, e.bond_max, W) != NNPP_OK) continue;
      EngineView v = make_view(e, 0, 0);
      NNPP_TRY(set_active(e, 1, 1));
      NNPP_TRY(launch_prep_b(e, v, prec, e.st, 0, nullptr));
      const bool win = prec == NNPP_MIXED && spmv_staged_fits(e);
      const int nvar = prec == NNPP_MIXED ? kSpmvVariants : 1;
      for (int var = 0; var < nvar; ++var) {
        if (!win && spmv_needs_windows(var)) continue;
        if (var == kSpmvHalo && !spmv_halo_fits(e)) continue;
        e.spmv_variant = var;
        NNPP_TRY(set_active(e, 1, 1));
        NNPP_TRY(launch_cg_spmv_b(e, v, prec, e.st));
        cudaEventRecord(e0, e.st);
        // the CG operator dominates; the FP64 tile kernels (residual, prep) follow the lanes
        for (int r = 0; r < 5; ++r) NNPP_TRY(launch_cg_spmv_b(e, v, prec, e.st));
        if (prec == NNPP_MIXED) NNPP_TRY(launch_cg_spmv_b(e, v, NNPP_FP64, e.st));
        cudaEventRecord(e1, e.st);
        NNPP_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
          best = ms;
          bT = T;
          bW = W;
          bS = e.spmv_variant;
        }
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  NNPP_CUDA(cudaStreamSynchronize(e.st));
  for (size_t i = 0; i < e.members.size(); ++i)
    NNPP_CUDA(cudaMemcpy(e.members[i]->dstate.get(), &saved[i], sizeof(DevState), cudaMemcpyHostToDevice));
  NNPP_TRY(build_lists(e, bT));
  e.W = bW;
  e.spmv_variant = bS;
  NNPP_TRY(prepare_kernels(e.halo_max, e.bond_max, bW));
  e.tuned = true;
  return NNPP_OK;
}

// ---------------------------------------------------------------- graph capture --------
nnpp_status add_while(cudaStream_t st, cudaGraphConditionalHandle hc, cudaGraph_t* body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  NNPP_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd));
  cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
  np.conditional.handle = hc;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  NNPP_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &np));
  *body = np.conditional.phGraph_out[0];
  NNPP_CUDA(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return NNPP_OK;
}

// warm start; prep; while(outer) { cg_init; while(inner) { spmv; update }; ir_update }
nnpp_status capture_solve(Engine& e, const EngineView& v, int prec) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  NNPP_CUDA(cudaStreamGetCaptureInfo(e.st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
  cudaGraphConditionalHandle hout;
  NNPP_CUDA(cudaGraphConditionalHandleCreate(&hout, g, 0, 0));
  NNPP_TRY(launch_warm_b(e, v, prec, e.st));
  NNPP_TRY(launch_prep_b(e, v, prec, e.st, hout, nullptr));
  cudaGraph_t body_out;
  NNPP_TRY(add_while(e.st, hout, &body_out));
  NNPP_CUDA(cudaStreamBeginCaptureToGraph(e.st_b1, body_out, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  cudaGraphConditionalHandle hin;
  NNPP_CUDA(cudaGraphConditionalHandleCreate(&hin, body_out, 0, 0));
  NNPP_TRY(launch_cg_init_b(e, v, prec, e.st_b1, hin));
  cudaGraph_t body_in;
  NNPP_TRY(add_while(e.st_b1, hin, &body_in));
  NNPP_CUDA(cudaStreamBeginCaptureToGraph(e.st_b2, body_in, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  NNPP_TRY(launch_cg_spmv_b(e, v, prec, e.st_b2));
  NNPP_TRY(launch_cg_update_b(e, v, prec, e.st_b2, hin));
  cudaGraph_t tmp;
  NNPP_CUDA(cudaStreamEndCapture(e.st_b2, &tmp));
  NNPP_TRY(launch_cg_final_b(e, v, prec, e.st_b1));
  NNPP_TRY(launch_ir_update_b(e, v, prec, e.st_b1, hout));
  NNPP_CUDA(cudaStreamEndCapture(e.st_b1, &tmp));
  return NNPP_OK;
}

// Eager form of capture_solve for profilers that cannot see into graphs with conditional
// nodes: the same kernels launched one at a time, the two loops driven by the host from the
// members' active flags.
nnpp_status any_active(Engine& e, int which, bool* any) {
  *any = false;
  std::vector<int> f(2 * e.members.size());
  for (size_t i = 0; i < e.members.size(); ++i)
    NNPP_CUDA(cudaMemcpyAsync(&f[2 * i], &e.members[i]->dstate.get()->outer_active, 2 * sizeof(int),
                              cudaMemcpyDeviceToHost, e.st));
  NNPP_CUDA(cudaStreamSynchronize(e.st));
  for (size_t i = 0; i < e.members.size(); ++i) *any = *any || f[2 * i + which] != 0;
  return NNPP_OK;
}

nnpp_status eager_solve(Engine& e, const EngineView& v, int prec) {
  NNPP_TRY(launch_warm_b(e, v, prec, e.st));
  NNPP_TRY(launch_prep_b(e, v, prec, e.st, 0, nullptr));
  bool go = false;
  for (int outer = 0; outer < (1 << 20); ++outer) {
    NNPP_TRY(any_active(e, 0, &go));
    if (!go) break;
    NNPP_TRY(launch_cg_init_b(e, v, prec, e.st, 0));
    for (int inner = 0; inner < (1 << 24); ++inner) {
      NNPP_TRY(any_active(e, 1, &go));
      if (!go) break;
      NNPP_TRY(launch_cg_spmv_b(e, v, prec, e.st));
      NNPP_TRY(launch_cg_update_b(e, v, prec, e.st, 0));
    }
    NNPP_TRY(launch_cg_final_b(e, v, prec, e.st));
    NNPP_TRY(launch_ir_update_b(e, v, prec, e.st, 0));
  }
  return NNPP_OK;
}

nnpp_status build_graph(Engine& e, int kind, int prec) {
  if (e.gexec[kind][prec][0]) return NNPP_OK;
  NNPP_CUDA(cudaStreamBeginCapture(e.st, cudaStreamCaptureModeThreadLocal));
  nnpp_status st = NNPP_OK;
  const int nsteps = kind == kGraphStep2 ? 2 : 1;
  for (int s = 0; s < nsteps && st == NNPP_OK; ++s) {
    EngineView v = make_view(e, s & 1, 1);
    st = capture_solve(e, v, prec);
    if (st == NNPP_OK && kind != kGraphSolve) st = launch_transport_b(e, v, prec, e.st, nullptr);
  }
  cudaGraph_t g = nullptr;
  cudaError_t err = cudaStreamEndCapture(e.st, &g);
  if (st != NNPP_OK) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return st;
  }
  if (err != cudaSuccess) return set_error(NNPP_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(err));
  cudaGraphExec_t ex = nullptr;
  err = cudaGraphInstantiate(&ex, g, 0);
  if (err != cudaSuccess) {
    cudaGraphDestroy(g);
    return set_error(NNPP_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(err));
  }
  e.graph[kind][prec][0] = g;
  e.gexec[kind][prec][0] = ex;
  return NNPP_OK;
}

nnpp_status prepare_run(Engine& e, int prec) {
  NNPP_TRY(sync_members(e));
  for (Handle* h : e.members) {
    NNPP_TRY(convert_state(*h, prec));
    NNPP_TRY(push_settings(*h));
  }
  if (!e.tuned || e.ntiles == 0) {
    NNPP_TRY(refresh_params(e));
    NNPP_TRY(tune(e, prec));
  } else {
    for (Handle* h : e.members)
      if (h->tiles_T != e.T) {
        NNPP_TRY(build_lists(e, e.T));
        NNPP_TRY(prepare_kernels(e.halo_max, e.bond_max, e.W));
        break;
      }
  }
  // two-level preconditioner of single-instance engines: recompute the coarse inverse when the
  // state was replaced; the captured graphs follow whether the coarse correction is applied
  for (Handle* hp : e.members) {
    Handle& h = *hp;
    if (h.coarse_enabled && h.coarse.n > 0 && (h.coarse.stale || !h.coarse.valid)) {
      NNPP_TRY(coarse_refresh(h));
      if (h.st != e.st) NNPP_CUDA(cudaStreamSynchronize(h.st));  // built on the member's stream
    }
  }
  const bool split = engine_coarse(e);
  if (split != e.coarse_graphs) {
    engine_destroy_graphs(e);
    e.coarse_graphs = split;
  }
  // the graphs hold the checked or the plain build of the kernels
  int checks = 0;
  for (Handle* h : e.members) checks |= h->checks;
  if (checks != e.checks) {
    engine_destroy_graphs(e);
    e.checks = checks;
  }
  NNPP_TRY(refresh_params(e));
  return NNPP_OK;
}

}  // namespace

Engine::~Engine() {
  engine_destroy_graphs(*this);
  if (st_b1) cudaStreamDestroy(st_b1);
  if (st_b2) cudaStreamDestroy(st_b2);
}

void engine_destroy_graphs(Engine& e) {
  for (int k = 0; k < kGraphKinds; ++k)
    for (int p = 0; p < 2; ++p)
      for (int c = 0; c < 2; ++c) {
        if (e.gexec[k][p][c]) cudaGraphExecDestroy(e.gexec[k][p][c]);
        if (e.graph[k][p][c]) cudaGraphDestroy(e.graph[k][p][c]);
        e.gexec[k][p][c] = nullptr;
        e.graph[k][p][c] = nullptr;
      }
}

EngineView make_view(Engine& e, int parity, int in_graph) {
  EngineView v;
  const int M = (int)e.members.size();
  v.inst = e.d_inst[parity].get();
  v.tiles = e.d_tiles.get();
  v.chunks = e.d_chunks.get();
  v.tile_first = e.d_meta.get();
  v.tile_count = e.d_meta.get() + M;
  v.chunk_first = e.d_meta.get() + 2 * M;
  v.chunk_count = e.d_meta.get() + 3 * M;
  v.slice_first = e.d_meta.get() + 4 * M;
  v.slice_count = e.d_meta.get() + 5 * M;
  v.slices = e.d_slices.get();
  v.htiles = e.d_htiles.get();
  v.cslices = e.d_cslices.get();
  v.cslice_first = e.d_meta.get() + 6 * M;
  v.cslice_count = e.d_meta.get() + 7 * M;
  v.ncslices = e.ncslices;
  v.hcode_max16 = e.hcode_max16;
  v.nslices = e.nslices;
  v.ticket = e.d_ticket.get();
  v.partials = e.d_partials.get();
  v.ntiles = e.ntiles;
  v.nchunks = e.nchunks;
  v.M = M;
  v.in_graph = in_graph;
  v.stride = std::max(std::max(e.ntiles, e.nchunks), std::max(e.nslices, e.ncslices));
  v.halo_max = e.halo_max;
  v.bond_max = e.bond_max;
  return v;
}

nnpp_status engine_build(Engine& e) {
  if (e.members.empty()) return set_error(NNPP_ERR_INVALID, "engine without members");
  e.device = e.members[0]->device;
  for (Handle* h : e.members) {
    if (!h->built) return set_error(NNPP_ERR_STATE, "engine member without neighbour lists");
    if (h->device != e.device) return set_error(NNPP_ERR_INVALID, "engine members on different devices");
  }
  if (!e.st_b1) NNPP_CUDA(cudaStreamCreateWithFlags(&e.st_b1, cudaStreamNonBlocking));
  if (!e.st_b2) NNPP_CUDA(cudaStreamCreateWithFlags(&e.st_b2, cudaStreamNonBlocking));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e.device);
  if (sms <= 0) sms = 152;
  e.sms = sms;
  e.grid = sms * 4;
  const char* eager = std::getenv("NNPP_EAGER");
  e.eager = eager && std::atoi(eager) != 0;
  NNPP_TRY(build_lists(e, e.T));
  NNPP_TRY(prepare_kernels(e.halo_max, e.bond_max, e.W));
  return NNPP_OK;
}

static nnpp_status run_steps(Engine& e, int n_steps, int prec) {
  if (e.eager) {
    for (int s = 0; s < n_steps; ++s) {
      EngineView v = make_view(e, 0, 0);
      NNPP_TRY(eager_solve(e, v, prec));
      NNPP_TRY(launch_transport_b(e, v, prec, e.st, nullptr));
      for (Handle* h : e.members) h->cur ^= 1;
      NNPP_TRY(refresh_params(e));
    }
    NNPP_CUDA(cudaStreamSynchronize(e.st));
    return NNPP_OK;
  }
  int done = 0;
  if (n_steps >= 2) NNPP_TRY(build_graph(e, kGraphStep2, prec));
  if (n_steps % 2) NNPP_TRY(build_graph(e, kGraphStep1, prec));
  while (n_steps - done >= 2) {
    NNPP_CUDA(cudaGraphLaunch(e.gexec[kGraphStep2][prec][0], e.st));
    done += 2;
  }
  if (n_steps - done == 1) {
    NNPP_CUDA(cudaGraphLaunch(e.gexec[kGraphStep1][prec][0], e.st));
    for (Handle* h : e.members) h->cur ^= 1;
    NNPP_TRY(refresh_params(e));
  }
  return NNPP_OK;
}

nnpp_status engine_run(Engine& e, int n_steps, int prec, bool prepared) {
  if (!prepared) NNPP_TRY(prepare_run(e, prec));
  // runs with the coarse correction stop at multiples of the first member's coarse_every
  // steps (counted since its state was replaced) to rebuild the coarse operators of members
  // whose phases changed
  Handle* h1 = e.members[0];
  const long long R = (engine_coarse(e) && !h1->coarse_replay) ? h1->coarse_every : 0;
  int done = 0;
  while (done < n_steps) {
    int seg = n_steps - done;
    if (R > 0) seg = (int)std::min<long long>(seg, R - h1->nstep % R);
    NNPP_TRY(run_steps(e, seg, prec));
    for (Handle* h : e.members) h->nstep += seg;
    done += seg;
    if (R > 0 && h1->nstep % R == 0) {
      // the checks and rebuilds run on the members' streams
      if (e.members.size() > 1 || h1->st != e.st) NNPP_CUDA(cudaStreamSynchronize(e.st));
      for (Handle* h : e.members) {
        NNPP_TRY(coarse_check(*h));
        if (h->st != e.st) NNPP_CUDA(cudaStreamSynchronize(h->st));
      }
      NNPP_TRY(refresh_params(e));  // a rebuilt operator may have another A P width
    }
  }
  if (e.members.size() > 1 || e.members[0]->st != e.st) NNPP_CUDA(cudaStreamSynchronize(e.st));
  return NNPP_OK;
}

nnpp_status engine_warm(Engine& e, int prec) {
  NNPP_TRY(prepare_run(e, prec));
  if (e.eager) return NNPP_OK;
  NNPP_TRY(build_graph(e, kGraphStep2, prec));
  NNPP_TRY(build_graph(e, kGraphStep1, prec));
  return NNPP_OK;
}

nnpp_status engine_params(Engine& e) { return refresh_params(e); }

nnpp_status engine_set_tiles(Engine& e, int T) { return build_lists(e, T); }

nnpp_status engine_solve(Engine& e, int prec) {
  NNPP_TRY(prepare_run(e, prec));
  if (e.eager) {
    NNPP_TRY(eager_solve(e, make_view(e, 0, 0), prec));
    NNPP_CUDA(cudaStreamSynchronize(e.st));
    return NNPP_OK;
  }
  NNPP_TRY(build_graph(e, kGraphSolve, prec));
  NNPP_CUDA(cudaGraphLaunch(e.gexec[kGraphSolve][prec][0], e.st));
  return NNPP_OK;
}

Handle::~Handle() {
  if (engine) {
    delete engine;
    engine = nullptr;
  }
}

}  // namespace nnpp
