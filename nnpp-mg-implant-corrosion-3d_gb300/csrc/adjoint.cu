// adjoint.cu -- forward/backward pair of the explicit step (checkpointed adjoint).
//
// nnpp_forward_ckpt runs the forward and samples the cumulative Mg mass loss.  When the FP64
// snapshots (c, phi, phase; 64 bytes per node) of every step fit the storage budget it keeps
// them all; otherwise it saves a full-state checkpoint every ck steps.  nnpp_backward runs
// the adjoint of each step backwards: the transposed bond sums (k_adj_transport), the adjoint
// potential solve A psi = nu through the same batched solver (right-hand side overridden) and
// the combination lambda^n = mu + (1/(K sigma)) F CSolid z_k psi.  With checkpoints it walks
// the segments from last to first, restoring a checkpoint and recomputing the segment's steps
// (the step kernels are deterministic, so the recomputed states are the forward's bit for
// bit) into (ck + 1) snapshots; a checkpoint holds the state and the warm-start history, so
// that the recomputed solves start from the same guesses.  Both modes give the same bits.
#include <algorithm>
#include <cstring>
#include <vector>

#include <cstddef>

#include "engine.cuh"

using namespace nnpp;

static_assert(offsetof(DevState, hist_head) == offsetof(DevState, hist_n) + sizeof(int),
              "hist_n and hist_head are written together");

struct nnpp_handle {
  Handle h;
};

namespace {

// Default relative tolerance of the mixed adjoint's potential solves.  The mixed gradient's
// own error (FP32 bond sums of the adjoint transport) is ~5e-7 relative to the FP64
// gradient on the 262k calibration workload; tightening these solves from 1e-8 to 1e-10
// moved its gradient by 2e-12 relative and cost 56% more inner iterations (15.7 -> 24.4 a
// solve over 2,000 steps), so 1e-8 keeps the solve's share of the error far below the floor.
constexpr double kAdjTolMixed = 1e-8;

nnpp_status save_ckpt(Handle& h, Handle::Ckpt& c) {
  const size_t N = h.N;
  if (!c.rec32.alloc(N) || !c.clo.alloc(N) || !c.rec64.alloc(N) || !c.phi.alloc(N) ||
      !c.phi_prev.alloc(N) || !c.flip.alloc(N))
    return set_error(NNPP_ERR_NOMEM, "checkpoint");
  const size_t HN = h.xh.get() ? (size_t)h.warm_hist * N : 0;
  if (HN && (!c.xh.alloc(HN) || !c.bh.alloc(HN))) return set_error(NNPP_ERR_NOMEM, "checkpoint history");
  c.cur = h.cur;
  c.prec = h.state_prec;
  if (HN) {
    NNPP_CUDA(cudaMemcpyAsync(c.xh.get(), h.xh.get(), sizeof(double) * HN, cudaMemcpyDeviceToDevice, h.st));
    NNPP_CUDA(cudaMemcpyAsync(c.bh.get(), h.bh.get(), sizeof(double) * HN, cudaMemcpyDeviceToDevice, h.st));
  }
  NNPP_CUDA(cudaMemcpyAsync(c.rec32.get(), h.rec32[h.cur].get(), sizeof(Rec32) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(c.clo.get(), h.clo.get(), sizeof(float4) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(c.rec64.get(), h.rec64[h.cur].get(), sizeof(Rec64) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(c.phi.get(), h.phi64.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(c.phi_prev.get(), h.phi_prev.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(c.flip.get(), h.flip_step.get(), sizeof(int) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(&c.ds, h.dstate.get(), sizeof(DevState), cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  return NNPP_OK;
}

nnpp_status load_ckpt(Handle& h, const Handle::Ckpt& c) {
  const size_t N = h.N;
  h.cur = c.cur;
  h.state_prec = c.prec;
  const size_t HN = h.xh.get() ? (size_t)h.warm_hist * N : 0;
  if (HN && c.xh.get()) {
    NNPP_CUDA(cudaMemcpyAsync(h.xh.get(), c.xh.get(), sizeof(double) * HN, cudaMemcpyDeviceToDevice, h.st));
    NNPP_CUDA(cudaMemcpyAsync(h.bh.get(), c.bh.get(), sizeof(double) * HN, cudaMemcpyDeviceToDevice, h.st));
  }
  NNPP_CUDA(cudaMemcpyAsync(h.rec32[h.cur].get(), c.rec32.get(), sizeof(Rec32) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.clo.get(), c.clo.get(), sizeof(float4) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.rec64[h.cur].get(), c.rec64.get(), sizeof(Rec64) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.phi64.get(), c.phi.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.phi_prev.get(), c.phi_prev.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, h.st));
  NNPP_CUDA(cudaMemcpyAsync(h.flip_step.get(), c.flip.get(), sizeof(int) * N, cudaMemcpyDeviceToDevice, h.st));
  DevState ds = c.ds;
  ds.op_valid = 0;  // the cached operator arrays are not part of a checkpoint
  NNPP_CUDA(cudaMemcpyAsync(h.dstate.get(), &ds, sizeof(DevState), cudaMemcpyHostToDevice, h.st));
  h.settings_pushed = false;
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  if (h.engine) NNPP_TRY(engine_params(*h.engine));
  return NNPP_OK;
}

// the inner iterations of the solve that just ended (one thread)
__global__ void k_adj_log(const DevState* ds, int* out) { *out = ds->solve_iters; }

nnpp_status read_ds(Handle& h, DevState* ds) {
  NNPP_CUDA(cudaMemcpyAsync(ds, h.dstate.get(), sizeof(DevState), cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  return NNPP_OK;
}

}  // namespace

extern "C" {

nnpp_status nnpp_forward_ckpt(nnpp_handle* hp, int n_steps, int precision, int ckpt_every,
                              int sample_every, double* mass_curve) {
  nnpp::TraceRange trace_("nnpp_forward_ckpt");
  clear_error();
  if (!hp) return set_error(NNPP_ERR_INVALID, "handle is NULL");
  Handle& h = hp->h;
  if (!h.built) return set_error(NNPP_ERR_STATE, "neighbour lists not built");
  if (n_steps < 1 || ckpt_every < 1 || sample_every < 1 || !mass_curve)
    return set_error(NNPP_ERR_INVALID, "forward_ckpt: bad argument");
  if (precision != NNPP_FP64 && precision != NNPP_MIXED) return set_error(NNPP_ERR_INVALID, "precision");
  if (h.p.vol_red != 0.0)
    return set_error(NNPP_ERR_UNSUPPORTED, "the adjoint needs vol_red = 0 (BV = 1 on mixed bonds)");
  NNPP_CUDA(cudaSetDevice(h.device));
  NNPP_TRY(engine_warm(*h.engine, precision));
  // coarse inverses used along the run: the current one from step 0, then each rebuild
  h.coarse_events.clear();
  h.coarse_event_cur = -1;
  h.coarse_record = false;
  if (engine_coarse(*h.engine)) {
    NNPP_TRY(coarse_record_event(h, 0));
    h.coarse_base = h.nstep;
    h.coarse_record = true;
  }
  struct RecordOff {
    Handle& h;
    ~RecordOff() {
      h.coarse_record = false;
      h.phi_keep[0] = h.phi_keep[1] = nullptr;
    }
  } record_off{h};
  h.fwd_steps = n_steps;
  h.ck_every = ckpt_every;
  h.sample_every = sample_every;
  h.fwd_prec = precision;
  h.ckpts.clear();
  h.snap_all_valid = false;
  const size_t N = h.N;
  bool store_all = h.adjoint_store == 2;
  if (h.adjoint_store == 0) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      free_b = 0;
    }
    const size_t need = (size_t)(n_steps + 1) * N * sizeof(Rec64);
    store_all = need <= free_b / 4 || (h.snap_all.get() && h.snap_all.size() >= (size_t)(n_steps + 1) * N);
  }
  if (store_all) {
    if (h.snap_all.size() < (size_t)(n_steps + 1) * N) {
      h.snap_all.reset();
      if (!h.snap_all.alloc((size_t)(n_steps + 1) * N))
        return set_error(NNPP_ERR_NOMEM, "adjoint snapshots of every step");
    }
  } else {
    h.snap_all.reset();
    h.ckpts.resize((n_steps + ckpt_every - 1) / ckpt_every);
  }
  // checkpoints: keep every step's solved potential as well (8 bytes per node and step) when
  // it fits a quarter of the free memory; backward then recomputes only the bond sums
  bool store_phi = false;
  h.phi_all_valid = false;
  if (!store_all && h.adjoint_store != 3) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      free_b = 0;
    }
    const size_t need = (size_t)n_steps * N;
    store_phi = h.phi_all.size() >= need || need * sizeof(double) <= free_b / 4;
    if (store_phi && h.phi_all.size() < need) {
      h.phi_all.reset();
      if (!h.phi_all.alloc(need)) {
        cudaGetLastError();
        store_phi = false;
      }
    }
    if (!store_phi) h.phi_all.reset();
  }
  double m0 = 0.0;
  NNPP_TRY(launch_sum_c0(h, h.scratch_d.get() + 8));
  NNPP_CUDA(cudaMemcpyAsync(&m0, h.scratch_d.get() + 8, sizeof(double), cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  h.curve.assign(n_steps / sample_every, 0.0);
  const double dV = h.p.dx * h.p.dy * h.p.dz;
  int s = 0;
  if (store_all) NNPP_TRY(launch_snap_state(h, h.snap_all.get()));
  while (s < n_steps) {
    int next;
    if (store_all) {
      // one step at a time: the potential it solved joins snapshot s, its result is s + 1
      NNPP_TRY(engine_run(*h.engine, 1, precision));
      NNPP_TRY(launch_snap_phi(h, h.snap_all.get() + (size_t)s * N));
      NNPP_TRY(launch_snap_state(h, h.snap_all.get() + (size_t)(s + 1) * N));
      next = s + 1;
    } else if (store_phi) {
      // up to two steps per graph launch, one per record parity: each step's transport also
      // writes the potential its solve left into phi_all (stops at checkpoints and samples)
      if (s % ckpt_every == 0) NNPP_TRY(save_ckpt(h, h.ckpts[s / ckpt_every]));
      next = std::min(n_steps, s + 2);
      next = std::min(next, (s / ckpt_every + 1) * ckpt_every);
      next = std::min(next, (s / sample_every + 1) * sample_every);
      h.phi_keep[h.cur & 1] = h.phi_all.get() + (size_t)s * N;
      h.phi_keep[(h.cur ^ 1) & 1] = next - s > 1 ? h.phi_all.get() + (size_t)(s + 1) * N : nullptr;
      NNPP_TRY(engine_run(*h.engine, next - s, precision));
    } else {
      if (s % ckpt_every == 0) NNPP_TRY(save_ckpt(h, h.ckpts[s / ckpt_every]));
      next = std::min(n_steps, (s / ckpt_every + 1) * ckpt_every);
      next = std::min(next, (s / sample_every + 1) * sample_every);
      NNPP_TRY(engine_run(*h.engine, next - s, precision));
    }
    s = next;
    if (s % sample_every == 0) {
      DevState ds;
      NNPP_TRY(read_ds(h, &ds));
      if (ds.wait_timeout) return set_error(NNPP_ERR_CUDA, "a bounded device wait timed out");
      if (ds.nonfinite) return set_error(NNPP_ERR_NONFINITE, "non-finite concentration in the state");
      h.curve[s / sample_every - 1] = dV * (m0 - ds.mg_mass_now);
    }
  }
  h.phi_keep[0] = h.phi_keep[1] = nullptr;
  NNPP_TRY(engine_params(*h.engine));
  NNPP_TRY(save_ckpt(h, h.fwd_end));
  h.snap_all_valid = store_all;
  h.phi_all_valid = store_phi;
  h.fwd_nstep_end = h.nstep;
  h.coarse_event_cur = (int)h.coarse_events.size() - 1;
  std::copy(h.curve.begin(), h.curve.end(), mass_curve);
  return NNPP_OK;
}

nnpp_status nnpp_get_adjoint_stats(nnpp_handle* hp, int64_t* cg_iterations, int64_t* solves,
                                   int64_t* sweeps, int* iterations_per_step) {
  clear_error();
  if (!hp) return set_error(NNPP_ERR_INVALID, "handle is NULL");
  Handle& h = hp->h;
  if (cg_iterations) *cg_iterations = h.adj_cg_iters;
  if (solves) *solves = h.adj_solves;
  if (sweeps) *sweeps = h.adj_sweeps;
  if (iterations_per_step) {
    if (h.fwd_steps < 1 || h.adj_log.size() < (size_t)h.fwd_steps)
      return set_error(NNPP_ERR_STATE, "adjoint stats: no backward run");
    NNPP_CUDA(cudaSetDevice(h.device));
    NNPP_CUDA(cudaMemcpyAsync(iterations_per_step, h.adj_log.get(), sizeof(int) * h.fwd_steps,
                              cudaMemcpyDeviceToHost, h.st));
    NNPP_CUDA(cudaStreamSynchronize(h.st));
  }
  return NNPP_OK;
}

nnpp_status nnpp_set_adjoint_solver(nnpp_handle* hp, double tol) {
  clear_error();
  if (!hp) return set_error(NNPP_ERR_INVALID, "handle is NULL");
  if (!(tol >= 0.0) || !(tol < 1.0)) return set_error(NNPP_ERR_INVALID, "adjoint tolerance must be in [0, 1)");
  hp->h.adj_tol = tol;
  return NNPP_OK;
}

nnpp_status nnpp_set_adjoint_store(nnpp_handle* hp, int mode) {
  clear_error();
  if (!hp) return set_error(NNPP_ERR_INVALID, "handle is NULL");
  if (mode < 0 || mode > 3)
    return set_error(NNPP_ERR_INVALID,
                     "adjoint store: 0 automatic, 1 checkpoints, 2 every step, 3 checkpoints without potentials");
  Handle& h = hp->h;
  h.adjoint_store = mode;
  h.fwd_steps = 0;
  h.ckpts.clear();
  h.snap_all_valid = false;
  h.phi_all_valid = false;
  if (mode == 1 || mode == 3) {
    NNPP_CUDA(cudaSetDevice(h.device));
    NNPP_CUDA(cudaStreamSynchronize(h.st));
    h.snap_all.reset();
    if (mode == 3) h.phi_all.reset();
  }
  return NNPP_OK;
}

nnpp_status nnpp_backward(nnpp_handle* hp, const double* dL_dmass, double* grad_D, double* grad_k) {
  nnpp::TraceRange trace_("nnpp_backward");
  clear_error();
  if (!hp) return set_error(NNPP_ERR_INVALID, "handle is NULL");
  Handle& h = hp->h;
  if (h.fwd_steps < 1 || (h.ckpts.empty() && !h.snap_all_valid))
    return set_error(NNPP_ERR_STATE, "backward without forward_ckpt");
  if (!dL_dmass || !grad_D || !grad_k) return set_error(NNPP_ERR_INVALID, "backward: NULL argument");
  NNPP_CUDA(cudaSetDevice(h.device));
  const int n_steps = h.fwd_steps, ck = h.ck_every, se = h.sample_every, prec = h.fwd_prec;
  const size_t N = h.N;
  const double dV = h.p.dx * h.p.dy * h.p.dz;
  DBuf<Rec64> snap;
  DBuf<double> lam, mu, nu, psi, acc, xa, ba;
  DBuf<float4> arec;  // FP32 adjoint records (mixed precision)
  if (prec == NNPP_MIXED && !arec.alloc(3 * N)) return set_error(NNPP_ERR_NOMEM, "adjoint records");
  // warm-start ring of the adjoint potential solves (host-tracked fill and head)
  const int hm = (h.extrapolate && h.warm_hist >= 3 && h.xh.get()) ? h.warm_hist : 0;
  int an = 0, ahead = hm ? hm - 1 : 0;
  if (hm && (!xa.alloc((size_t)hm * N) || !ba.alloc((size_t)hm * N)))
    return set_error(NNPP_ERR_NOMEM, "adjoint warm-start ring");
  const bool all = h.snap_all_valid;
  if ((!all && !snap.alloc((size_t)(ck + 1) * N)) || !lam.alloc(S * N) || !mu.alloc(S * N) || !nu.alloc(N) ||
      !psi.alloc(N) || !acc.alloc(8))
    return set_error(NNPP_ERR_NOMEM, "adjoint buffers");
  if (h.adj_log.size() < (size_t)n_steps) {
    h.adj_log.reset();
    if (!h.adj_log.alloc(n_steps)) return set_error(NNPP_ERR_NOMEM, "adjoint iteration log");
  }
  NNPP_CUDA(cudaMemsetAsync(h.adj_log.get(), 0, sizeof(int) * n_steps, h.st));
  if (!all) NNPP_CUDA(cudaMemsetAsync(snap.get(), 0, sizeof(Rec64) * (size_t)(ck + 1) * N, h.st));
  NNPP_CUDA(cudaMemsetAsync(lam.get(), 0, sizeof(double) * S * N, h.st));
  NNPP_CUDA(cudaMemsetAsync(psi.get(), 0, sizeof(double) * N, h.st));
  NNPP_CUDA(cudaMemsetAsync(acc.get(), 0, sizeof(double) * 8, h.st));
  nnpp_status st = NNPP_OK;
  // lambda^{n_steps}: the sample at the last step
  if (n_steps % se == 0) {
    NNPP_CUDA(cudaMemsetAsync(mu.get(), 0, sizeof(double) * S * N, h.st));
    h.b_override = nullptr;
    NNPP_TRY(engine_params(*h.engine));
    // freem / phi64 are irrelevant here: mu = 0, and psi is masked by freem; zero phi64
    NNPP_CUDA(cudaMemsetAsync(h.phi64.get(), 0, sizeof(double) * N, h.st));
    NNPP_TRY(launch_adj_combine(h, mu.get(), lam.get(), -dV * dL_dmass[n_steps / se - 1]));
  }
  Engine& e = *h.engine;
  // replay the recorded coarse inverses (no rebuilds while recomputing); afterwards the last
  // one and the step count of the end of the forward run are back
  h.coarse_replay = true;
  struct ReplayOff {
    Handle& h;
    ~ReplayOff() {
      coarse_select(h, h.fwd_steps);
      h.coarse_replay = false;
      h.nstep = h.fwd_nstep_end;
    }
  } replay_off{h};
  // the adjoint solves run to adj_tol when it is set, else mixed runs to max(tol, 1e-8) and
  // FP64 runs to tol; the recomputed forward steps always run to tol
  const double fwd_tol = h.tol;
  const double adj_tol = h.adj_tol > 0.0 ? h.adj_tol : (prec == NNPP_MIXED ? std::max(h.tol, kAdjTolMixed) : h.tol);
  struct TolBack {
    Handle& h;
    double tol;
    ~TolBack() {
      if (h.tol != tol) {
        h.tol = tol;
        h.settings_pushed = false;
      }
    }
  } tol_back{h, fwd_tol};
  auto use_tol = [&](double t) {
    if (h.tol != t) {
      h.tol = t;
      h.settings_pushed = false;
    }
  };
  h.adj_cg_iters = 0;
  h.adj_solves = 0;
  h.adj_sweeps = 0;
  // with every step's snapshot one segment covers the run and nothing is recomputed
  const int nseg = all ? 1 : (int)h.ckpts.size();
  const int seg_len = all ? n_steps : ck;
  for (int g = nseg - 1; g >= 0 && st == NNPP_OK; --g) {
    const int s0 = g * seg_len, s1 = std::min(n_steps, s0 + seg_len);
    const Rec64* base = all ? h.snap_all.get() : snap.get();
    if (!all) {
      use_tol(fwd_tol);
      NNPP_TRY(load_ckpt(h, h.ckpts[g]));
      NNPP_TRY(launch_snap_state(h, snap.get()));
      for (int n = s0; n < s1; ++n) {
        if (h.phi_all_valid) {
          // the step's potential as its solve left it, then its bond sums and update (the
          // transport reads nothing else the solve writes): the forward's state bit for bit
          NNPP_TRY(launch_load_phi(h, h.phi_all.get() + (size_t)n * N, snap.get() + (size_t)(n - s0) * N));
          NNPP_TRY(launch_transport_b(e, make_view(e, 0, 0), prec, h.st, nullptr));
          h.cur ^= 1;
          NNPP_TRY(engine_params(e));
        } else {
          NNPP_TRY(coarse_select(h, n, true));
          NNPP_TRY(engine_run(e, 1, prec));
          NNPP_TRY(launch_snap_phi(h, snap.get() + (size_t)(n - s0) * N));
        }
        NNPP_TRY(launch_snap_state(h, snap.get() + (size_t)(n - s0 + 1) * N));
      }
    }
    // the adjoint solves' inner iterations of this segment (the device counters come back
    // with each checkpoint)
    use_tol(adj_tol);
    DevState dseg;
    NNPP_TRY(read_ds(h, &dseg));
    for (int n = s1 - 1; n >= s0; --n) {
      const Rec64* sn = base + (size_t)(n - s0) * N;
      const Rec64* sn1 = base + (size_t)(n - s0 + 1) * N;
      NNPP_TRY(engine_params(e));
      EngineView v = make_view(e, 0, 0);
      if (prec == NNPP_MIXED)
        NNPP_TRY(launch_adj_transport32(e, v, h, sn, sn1, lam.get(), arec.get(), mu.get(), nu.get(), acc.get(), h.st));
      else
        NNPP_TRY(launch_adj_transport(e, v, sn, sn1, lam.get(), mu.get(), nu.get(), acc.get(), h.st));
      // adjoint potential solve on the unknowns of step n
      NNPP_TRY(coarse_select(h, n));
      NNPP_TRY(launch_adj_solve_setup(h, sn, psi.get()));
      h.b_override = nu.get();
      if (hm >= 3) {
        // the adjoint potentials form their own warm-start ring
        h.warm_x_alt = xa.get();
        h.warm_b_alt = ba.get();
        const int hs[2] = {an, ahead};
        NNPP_CUDA(cudaMemcpyAsync(&h.dstate.get()->hist_n, hs, sizeof(hs), cudaMemcpyHostToDevice, h.st));
      }
      st = engine_solve(e, prec);
      if (st == NNPP_OK) {
        k_adj_log<<<1, 1, 0, h.st>>>(h.dstate.get(), h.adj_log.get() + n);
        if (cudaGetLastError() != cudaSuccess) st = set_error(NNPP_ERR_CUDA, "adjoint iteration log");
      }
      if (st == NNPP_OK && hm >= 3) {
        ahead = (ahead + 1) % hm;
        an = an < hm ? an + 1 : hm;
        st = launch_record_solve(h, ahead);
      }
      h.b_override = nullptr;
      h.warm_x_alt = h.warm_b_alt = nullptr;
      if (st != NNPP_OK) break;
      NNPP_CUDA(cudaMemcpyAsync(psi.get(), h.phi64.get(), sizeof(double) * N, cudaMemcpyDeviceToDevice, h.st));
      const double inject = (n > 0 && n % se == 0) ? -dV * dL_dmass[n / se - 1] : 0.0;
      NNPP_TRY(launch_adj_combine(h, mu.get(), lam.get(), inject));
    }
    if (st != NNPP_OK) break;
    DevState dend;
    NNPP_TRY(read_ds(h, &dend));
    h.adj_cg_iters += dend.cg_iters - dseg.cg_iters;
    h.adj_solves += dend.cg_solves - dseg.cg_solves;
    h.adj_sweeps += dend.outer_total - dseg.outer_total;
  }
  double g5[8];
  NNPP_CUDA(cudaMemcpyAsync(g5, acc.get(), sizeof(double) * 8, cudaMemcpyDeviceToHost, h.st));
  NNPP_CUDA(cudaStreamSynchronize(h.st));
  use_tol(fwd_tol);
  nnpp_status st2 = load_ckpt(h, h.fwd_end);
  if (st != NNPP_OK) return st;
  for (int k = 0; k < S; ++k) grad_D[k] = g5[k];
  *grad_k = g5[4];
  return st2;
}

}  // extern "C"
