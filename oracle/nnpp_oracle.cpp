// nnpp_oracle.cpp -- FP64 CPU oracle of the nonlocal Nernst-Planck-Poisson hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: tests, the smoke check and the
// CPU-baseline leg of the benchmark call it; the product library never links or calls
// it.  It restates, in plain C++ with OpenMP, the reference's algorithm for the path:
//
//   neighbour build   grid.h:22-204          (build_clouds_hash, sphere_cube_intersects)
//   influence factor  utils.h:17-25          (Beta)
//   bond sums         utils.h:72-178 (Mg), utils.h:181-257 (generic species)
//   potential         utils.h:798-841 (F11), utils.h:1794-1848 (K11)
//   step / front      main.cpp:556-640, 676-712 (Dirichlet), 805-837 (clamp),
//                     914-922 (phase flip), 472-480 and 944-949 (volume)
//
// turned into the explicit step:  c^{n+1} = c^n - dt * (sum_KR1 + sum_KR2 - R)  with the
// potential phi^n solved from c^n (Jacobi-preconditioned CG, FP64) before the transport,
// and the Mg source R_0 = -k_diss * S(c_0 - CSat/CSolid) on solid interface nodes
// (the position of the reference's Mg rate terms, utils.h:162-167).
//
// Parity is pinned against the reference itself: ref_shim.cpp compiles grid.h and utils.h
// from the reference's sources and the tests compare this restatement with them (neighbour
// lists bit for bit, residuals and K11 to rounding); golden fixtures made from those runs
// are committed under tests/golden/.  Operation order inside each bond term follows the
// reference's expressions so that the FP64 residuals agree bit for bit.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <utility>
#include <vector>

#include <omp.h>

#include "../include/nnpp_gb300.h"

namespace {

const int S = NNPP_NSPECIES;

inline double sqr(double x) { return x * x; }

// grid.h:27-41
bool sphere_cube(double cx, double cy, double cz, double r, double bx, double by, double bz,
                 double w, double h, double d) {
  const double bmin[3] = {bx, by, bz};
  const double bmax[3] = {bx + w, by + h, bz + d};
  const double c[3] = {cx, cy, cz};
  const double r2 = sqr(r);
  double dmin = 0.0;
  for (int i = 0; i < 3; ++i) {
    if (c[i] < bmin[i])
      dmin += sqr(c[i] - bmin[i]);
    else if (c[i] > bmax[i])
      dmin += sqr(c[i] - bmax[i]);
  }
  return dmin <= r2;
}

// utils.h:17-25
double beta_fn(double xi, double delta, double dx) {
  if (xi <= delta - dx / 2.0) return 1.0;
  if ((xi > delta - dx / 2.0) && (xi <= delta + dx / 2.0)) return (delta + dx / 2.0 - xi) / (dx);
  return 0.0;
}

struct Oracle {
  nnpp_params p;
  int N = 0;
  std::vector<double> x, y, z;
  std::vector<int> bctypes;
  std::vector<double> bcv;  // (S+1)*N
  std::vector<unsigned char> dir;  // (S+1)*N Dirichlet flags
  // neighbour lists, reference format: row i = cols[row_ptr[i] .. row_ptr[i+1]), slot 0 self
  std::vector<int64_t> row_ptr;
  std::vector<int> cols;
  bool have_nb = false;
  // state
  std::vector<double> c;  // S*N
  std::vector<double> phi;  // N
  std::vector<int> phase;
  std::vector<int> flip_step;
  std::vector<double> c0_init;  // Mg at t = 0
  double vol0rel = 0.0, voln1rel = 0.0;
  int64_t steps_done = 0;
  int64_t solid_count = 0;
  double dissolved_total = 0.0;
  int64_t cg_iters_total = 0, cg_solves = 0, cg_nc = 0;
  double last_relres = 0.0;
  double tol = 1e-12;
  int max_iter = 20000;
  // potential operator cache (rebuilt when the phase changes)
  std::vector<double> wphi;  // per bond, w of the potential (K11 form), 0 if not LL
  std::vector<double> diag;
  std::vector<unsigned char> freev;
  bool op_valid = false;
  // adjoint checkpoints
  struct Ckpt {
    std::vector<double> c, phi;
    std::vector<int> phase;
    double voln1rel;
  };
  std::vector<Ckpt> ckpts;
  int ck_every = 0, sample_every = 0, fwd_steps = 0;
  std::vector<double> curve;
};

double mg_source_switch(const nnpp_params& p, double c0) {
  double cs = p.CSat / p.CSolid;
  if (p.switch_width > 0.0) return 1.0 / (1.0 + std::exp(-(c0 - cs) / p.switch_width));
  return c0 > cs ? 1.0 : 0.0;
}

double mg_source_switch_deriv(const nnpp_params& p, double c0) {
  if (p.switch_width <= 0.0) return 0.0;
  double cs = p.CSat / p.CSolid;
  double s = 1.0 / (1.0 + std::exp(-(c0 - cs) / p.switch_width));
  return s * (1.0 - s) / p.switch_width;
}

// ---------------------------------------------------------------- neighbour build --------
// grid.h:43-204.  Step 5 of the reference tests every cell against the sphere; here the
// scan is limited to the cells within one cell of the sphere's bounding box, which contains
// every cell the exact test can accept, and the accepted cells are visited in the same
// ascending-hash order, so the lists are identical.
int build_clouds(int max_node_no, double r, double cx, double cy, double cz, int N,
                 const double* X, const double* Y, const double* Z, std::vector<int64_t>& row_ptr,
                 std::vector<int>& cols, int* max_len) {
  if (N <= 0) return 1;
  double x0 = X[0], x1 = X[0], y0 = Y[0], y1 = Y[0], z0 = Z[0], z1 = Z[0];
  for (int i = 0; i < N; ++i) {
    x0 = std::min(x0, X[i]);
    x1 = std::max(x1, X[i]);
    y0 = std::min(y0, Y[i]);
    y1 = std::max(y1, Y[i]);
    z0 = std::min(z0, Z[i]);
    z1 = std::max(z1, Z[i]);
  }
  const int mx = static_cast<int>((x1 - x0) / cx) + 1;
  const int my = static_cast<int>((y1 - y0) / cy) + 1;
  std::vector<std::pair<int, int> > hashes(N);
#pragma omp parallel for
  for (int i = 0; i < N; ++i) {
    hashes[i].first = i;
    hashes[i].second = static_cast<int>((X[i] - x0) / cx) + mx * static_cast<int>((Y[i] - y0) / cy) +
                       mx * my * static_cast<int>((Z[i] - z0) / cz);
  }
  std::sort(hashes.begin(), hashes.end(),
            [](const std::pair<int, int>& a, const std::pair<int, int>& b) { return a.second < b.second; });
  const int max_hash = hashes[N - 1].second + 1;
  std::vector<int> start(max_hash + 1, 0), count(max_hash, 0);
  for (int k = 0; k < N; ++k) count[hashes[k].second]++;
  {
    int acc = 0;
    for (int h = 0; h < max_hash; ++h) {
      start[h] = acc;
      acc += count[h];
    }
    start[max_hash] = acc;
  }
  std::vector<int> len(N);
  std::vector<std::vector<int> > rows(N);
  int err = 0;
  const double r2 = sqr(r);
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < N; ++i) {
    const double px = X[i], py = Y[i], pz = Z[i];
    int lo[3], hi[3];
    const double o[3] = {x0, y0, z0}, w[3] = {cx, cy, cz}, q[3] = {px, py, pz};
    for (int d = 0; d < 3; ++d) {
      lo[d] = (int)std::floor((q[d] - r - o[d]) / w[d]) - 1;
      hi[d] = (int)std::floor((q[d] + r - o[d]) / w[d]) + 1;
      if (lo[d] < 0) lo[d] = 0;
    }
    if (hi[0] > mx - 1) hi[0] = mx - 1;
    if (hi[1] > my - 1) hi[1] = my - 1;
    std::vector<int>& row = rows[i];
    row.clear();
    row.push_back(i);
    int fill = 1;
    for (int kz = lo[2]; kz <= hi[2]; ++kz)
      for (int ky = lo[1]; ky <= hi[1]; ++ky)
        for (int kx = lo[0]; kx <= hi[0]; ++kx) {
          int m = kx + mx * ky + mx * my * kz;
          if (m >= max_hash) continue;
          // corner as grid.h:129-140
          int rr = (m % (mx * my)) % mx;
          int cc = (m % (mx * my)) / mx;
          int pp = m / (mx * my);
          double bx = x0 + rr * cx, by = y0 + cc * cy, bz = z0 + pp * cz;
          if (!sphere_cube(px, py, pz, r, bx, by, bz, cx, cy, cz)) continue;
          if (count[m] == 0) continue;
          for (int k = start[m]; k < start[m] + count[m]; ++k) {
            int cand = hashes[k].first;
            if (sqr(px - X[cand]) + sqr(py - Y[cand]) + sqr(pz - Z[cand]) <= r2 && cand != i) {
              if (fill == max_node_no) {
#pragma omp atomic write
                err = 1;
                break;
              }
              row.push_back(cand);
              fill++;
            }
          }
        }
    len[i] = fill;
  }
  if (err) return 2;
  row_ptr.assign(N + 1, 0);
  for (int i = 0; i < N; ++i) row_ptr[i + 1] = row_ptr[i] + len[i];
  cols.resize(row_ptr[N]);
  int ml = 0;
#pragma omp parallel for reduction(max : ml)
  for (int i = 0; i < N; ++i) {
    std::copy(rows[i].begin(), rows[i].end(), cols.begin() + row_ptr[i]);
    ml = std::max(ml, len[i]);
  }
  *max_len = ml;
  return 0;
}

// ---------------------------------------------------------------- bond sums --------------
// Residual F_k (utils.h:72-178 for k = 0, utils.h:181-257 for k >= 1) with U^{n+1} = U^n
// and the reference's operation order; R_k is the dissolution source of species 0.
// Optional outputs: transport part per species (sum_KR1 + sum_KR2) and the interface flag.
void residuals(const Oracle& o, const double* c, const double* phi, const int* phase,
               double voln1rel, double* F, double* transport, unsigned char* iface_out) {
  const nnpp_params& p = o.p;
  const int N = o.N;
  const double BVmix = std::pow(10., -p.vol_red * (1. - voln1rel));
  const double csat = p.CSat / p.CSolid;
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < N; ++i) {
    const int64_t b = o.row_ptr[i], e = o.row_ptr[i + 1];
    int iface = 0;
    if (phase[i] == 1)
      for (int64_t j = b + 1; j < e; ++j)
        if (phase[o.cols[j]] == 0) {
          iface = 1;
          break;
        }
    if (iface_out) iface_out[i] = (unsigned char)iface;
    for (int k = 0; k < S; ++k) {
      const double* ck = c + (int64_t)k * N;
      double s1 = 0.0, s2 = 0.0;
      for (int64_t j = b + 1; j < e; ++j) {
        const int n = o.cols[j];
        const double xix = o.x[n] - o.x[i], xiy = o.y[n] - o.y[i], xiz = o.z[n] - o.z[i];
        const double xi = std::sqrt(xix * xix + xiy * xiy + xiz * xiz);
        const int pi = phase[i], pn = phase[n];
        double a1, a2;  // K*D(*BV) prefixes, in the reference's multiplication order
        if (k == 0) {
          double BV = ((pi == 1 && pn == 0) || (pn == 1 && pi == 0)) ? BVmix : 1.0;
          if (pi == 0 && pn == 0) {
            a1 = p.K1[0] * p.D_liquid[0];
            a2 = p.K2[0] * p.D_liquid[0];
          } else {
            a1 = p.K1[0] * p.D_solid[0] * BV;
            a2 = p.K2[0] * p.D_solid[0] * BV;
          }
        } else {
          if (pi == 1 && pn == 1) continue;
          if (pi == 0 && pn == 0) {
            a1 = p.K1[k] * p.D_liquid[k];
            a2 = p.K2[k] * p.D_liquid[k];
          } else {
            a1 = p.K1[k] * p.D_solid[k];
            a2 = p.K2[k] * p.D_solid[k];
          }
        }
        const double bt = beta_fn(xi, p.delta, p.dx);
        s1 += -(a1 * (ck[n] - ck[i]) / std::pow(xi, 3.0 + 2.0 * p.s1[k])) * bt * p.dx * p.dy * p.dz;
        s2 += -(a2 * p.z[k] * p.F * ck[n] * (phi[n] - phi[i]) /
                (p.R * p.T * std::pow(xi, 3.0 + 2.0 * p.s2[k]))) *
              bt * p.dx * p.dy * p.dz;
      }
      double R = 0.0;
      if (k == 0 && iface == 1) R = -p.k_diss * mg_source_switch(p, ck[i]);
      if (transport) transport[(int64_t)k * N + i] = s1 + s2;
      F[(int64_t)k * N + i] = ((ck[i] - ck[i]) / p.dt) + s1 + s2 - R;
    }
    // potential residual utils.h:798-841
    double sp = 0.0;
    int flag = 0;
    for (int64_t j = b + 1; j < e; ++j) {
      const int n = o.cols[j];
      const double xix = o.x[n] - o.x[i], xiy = o.y[n] - o.y[i], xiz = o.z[n] - o.z[i];
      const double xi = std::sqrt(xix * xix + xiy * xiy + xiz * xiz);
      if (phase[i] == 0 && phase[n] == 0) {
        sp += -(p.K_phi * p.sigma * (phi[n] - phi[i]) / std::pow(xi, 3.0 + 2.0 * p.s_phi)) *
              beta_fn(xi, p.delta, p.dx) * p.dx * p.dy * p.dz;
        flag = 1;
      }
    }
    double f11 = 0.0;
    if (flag == 1) {
      double R11 = 0.0;
      for (int k = 0; k < S; ++k) R11 += p.z[k] * c[(int64_t)k * N + i];
      f11 = (1. / (p.K_phi * p.sigma)) * sp - (1. / (p.K_phi * p.sigma)) * p.F * p.CSolid * R11;
    }
    F[(int64_t)S * N + i] = f11;
  }
}

// ---------------------------------------------------------------- potential --------------
// K11 (utils.h:1797-1848): off-diagonal -(1/(K sigma)) (K sigma / xi^(3+2s)) beta dV on
// liquid-liquid bonds, diagonal the negated row sum (same expression), identity rows on
// Dirichlet nodes and on nodes without liquid-liquid bonds.
void build_operator(Oracle& o, const int* phase) {
  const nnpp_params& p = o.p;
  const int N = o.N;
  o.wphi.assign(o.cols.size(), 0.0);
  o.diag.assign(N, 1.0);
  o.freev.assign(N, 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < N; ++i) {
    const int64_t b = o.row_ptr[i], e = o.row_ptr[i + 1];
    if (o.dir[(int64_t)S * N + i]) continue;
    double sumK = 0.0;
    int flag = 0;
    for (int64_t j = b + 1; j < e; ++j) {
      const int n = o.cols[j];
      if (!(phase[i] == 0 && phase[n] == 0)) continue;
      const double xix = o.x[n] - o.x[i], xiy = o.y[n] - o.y[i], xiz = o.z[n] - o.z[i];
      const double xi = std::sqrt(xix * xix + xiy * xiy + xiz * xiz);
      const double bt = beta_fn(xi, p.delta, p.dx);
      sumK += -(p.K_phi * p.sigma / std::pow(xi, 3.0 + 2.0 * p.s_phi)) * bt * p.dx * p.dy * p.dz;
      double off = -(1. / (p.K_phi * p.sigma)) * (p.K_phi * p.sigma / std::pow(xi, 3.0 + 2.0 * p.s_phi)) *
                   bt * p.dx * p.dy * p.dz;
      o.wphi[j] = -off;  // store w >= 0; the matrix entry is -w
      flag = 1;
    }
    if (flag) {
      o.diag[i] = -(1. / (p.K_phi * p.sigma)) * sumK;
      o.freev[i] = 1;
    }
  }
  o.op_valid = true;
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  const int n = (int)a.size();
#pragma omp parallel for reduction(+ : s)
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

// y = A x on free rows (x must vanish off the free set except where couplings are wanted)
void apply_A(const Oracle& o, const std::vector<double>& xv, std::vector<double>& yv) {
  const int N = o.N;
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < N; ++i) {
    if (!o.freev[i]) {
      yv[i] = 0.0;
      continue;
    }
    double s = o.diag[i] * xv[i];
    for (int64_t j = o.row_ptr[i] + 1; j < o.row_ptr[i + 1]; ++j) s -= o.wphi[j] * xv[o.cols[j]];
    yv[i] = s;
  }
}

// Solve the potential for concentrations c and phase (phi: warm start in, solution out).
// Free rows: sum_LL w (phi_i - phi_n) = (1/(K sigma)) F CSolid sum_k z_k c_k  (F11 = 0);
// Dirichlet rows phi = bc (main.cpp:710-711); other rows keep their value.
int solve_potential(Oracle& o, const double* c, const int* phase, double* phi, int* iters,
                    double* relres) {
  const nnpp_params& p = o.p;
  const int N = o.N;
  build_operator(o, phase);
  std::vector<double> xv(phi, phi + N);
  for (int i = 0; i < N; ++i)
    if (o.dir[(int64_t)S * N + i]) xv[i] = o.bcv[(int64_t)S * N + i];
  const double lam = (1. / (p.K_phi * p.sigma)) * p.F * p.CSolid;
  std::vector<double> bvec(N, 0.0), beff(N, 0.0);
  for (int i = 0; i < N; ++i) {
    if (!o.freev[i]) continue;
    double R11 = 0.0;
    for (int k = 0; k < S; ++k) R11 += p.z[k] * c[(int64_t)k * N + i];
    bvec[i] = lam * R11;
    double cpl = 0.0;
    for (int64_t j = o.row_ptr[i] + 1; j < o.row_ptr[i + 1]; ++j) {
      int n = o.cols[j];
      if (o.wphi[j] != 0.0 && !o.freev[n]) cpl += o.wphi[j] * xv[n];
    }
    beff[i] = bvec[i] + cpl;
  }
  double bnorm = std::sqrt(dot(beff, beff));
  if (bnorm == 0.0) bnorm = 1.0;
  std::vector<double> r(N), zv(N), pv(N), q(N), tmp(N);
  int it_total = 0;
  double rel = 0.0;
  for (int restart = 0; restart < 20; ++restart) {
    // true residual with the full vector (fixed values included)
    {
      std::vector<double> xf(N);
      for (int i = 0; i < N; ++i) xf[i] = xv[i];
#pragma omp parallel for schedule(dynamic, 256)
      for (int i = 0; i < N; ++i) {
        if (!o.freev[i]) {
          r[i] = 0.0;
          continue;
        }
        double s = o.diag[i] * xf[i];
        for (int64_t j = o.row_ptr[i] + 1; j < o.row_ptr[i + 1]; ++j) s -= o.wphi[j] * xf[o.cols[j]];
        r[i] = bvec[i] - s;
      }
    }
    rel = std::sqrt(dot(r, r)) / bnorm;
    if (rel <= o.tol || it_total >= o.max_iter) break;
    for (int i = 0; i < N; ++i) zv[i] = o.freev[i] ? r[i] / o.diag[i] : 0.0;
    pv = zv;
    double rz = dot(r, zv);
    for (int it = 0; it < o.max_iter - it_total; ++it) {
      apply_A(o, pv, q);
      double pq = dot(pv, q);
      if (pq <= 0.0) break;
      double alpha = rz / pq;
      for (int i = 0; i < N; ++i) {
        if (!o.freev[i]) continue;
        xv[i] += alpha * pv[i];
        r[i] -= alpha * q[i];
      }
      ++it_total;
      double rn = std::sqrt(dot(r, r)) / bnorm;
      if (rn <= 0.5 * o.tol) break;
      for (int i = 0; i < N; ++i) zv[i] = o.freev[i] ? r[i] / o.diag[i] : 0.0;
      double rz2 = dot(r, zv);
      double bta = rz2 / rz;
      rz = rz2;
      for (int i = 0; i < N; ++i) pv[i] = zv[i] + bta * pv[i];
    }
  }
  for (int i = 0; i < N; ++i) phi[i] = xv[i];
  if (iters) *iters = it_total;
  if (relres) *relres = rel;
  return rel <= o.tol ? 0 : 4;
}

// ---------------------------------------------------------------- explicit step ----------
// One step with the reference's order of the per-step operations (main.cpp:547-1025):
// potential from c^n, transport with the Dirichlet override and the clamp, phase flip,
// volume every sub_step_no steps.  Optionally records what the adjoint needs.
struct StepRecord {
  std::vector<unsigned char> clamped;  // S*N
};

int step(Oracle& o, StepRecord* rec) {
  const nnpp_params& p = o.p;
  const int N = o.N;
  int it = 0;
  double rel = 0.0;
  int st = solve_potential(o, o.c.data(), o.phase.data(), o.phi.data(), &it, &rel);
  o.cg_iters_total += it;
  o.cg_solves += 1;
  o.last_relres = rel;
  if (st != 0) o.cg_nc += 1;
  std::vector<double> F((int64_t)(S + 1) * N);
  std::vector<unsigned char> iface(N);
  residuals(o, o.c.data(), o.phi.data(), o.phase.data(), o.voln1rel, F.data(), nullptr, iface.data());
  std::vector<double> cn((int64_t)S * N);
  double diss = 0.0;
  if (rec) rec->clamped.assign((int64_t)S * N, 0);
#pragma omp parallel for reduction(+ : diss)
  for (int i = 0; i < N; ++i) {
    for (int k = 0; k < S; ++k) {
      const int64_t a = (int64_t)k * N + i;
      double v;
      if (o.dir[a])
        v = o.bcv[a] / p.CSolid;
      else
        v = o.c[a] - p.dt * F[a];
      if (v < p.c_floor) {
        v = p.c_floor;
        if (rec) rec->clamped[a] = 1;
      }
      cn[a] = v;
    }
    if (iface[i] && !o.dir[i]) diss += p.k_diss * mg_source_switch(p, o.c[i]);
  }
  o.dissolved_total += diss * p.dt * p.dx * p.dy * p.dz;
  o.c.swap(cn);
  const double csat = p.CSat / p.CSolid;
  const int64_t s = o.steps_done + 1;
  int64_t flips = 0;
  for (int i = 0; i < N; ++i) {
    if (o.phase[i] == 1 && o.c[i] <= csat) {
      o.phase[i] = 0;
      o.flip_step[i] = (int)s;
      ++flips;
    }
  }
  o.solid_count -= flips;
  if (p.sub_step_no > 0 && s % p.sub_step_no == 0) {
    double v = 0.0;
    for (int i = 0; i < N; ++i)
      if (o.phase[i] == 1) v += (o.c[i] - csat);
    o.voln1rel = (o.vol0rel != 0.0) ? v / o.vol0rel : 0.0;
  }
  o.steps_done = s;
  return st;
}

// ---------------------------------------------------------------- adjoint ----------------
// Forward with every step recorded (small cases), then the exact adjoint of the explicit
// step: the transposed bond sums (the weights of the reference's tangent, utils.h:955-963),
// the adjoint potential solve (K11 is symmetric on the unknowns) and the smoothed
// dissolution switch.  Phase flips, interface flags and the unknown set are piecewise
// constant in the parameters; clamped and Dirichlet values have zero derivative.
struct Record {
  std::vector<std::vector<double> > c, phi;            // c^n (S*N), phi^n (N)
  std::vector<std::vector<int> > phase;                // phase^n
  std::vector<std::vector<unsigned char> > clamped;    // clamp of c^{n+1}
  std::vector<double> c0;                              // c_0 at t = 0
  int steps = 0, sample_every = 0;
};

Record g_rec;

// A psi = nu on the unknowns of `phase` (Dirichlet and frozen values 0), FP64 CG.
void adjoint_solve(Oracle& o, const int* phase, const std::vector<double>& nu, std::vector<double>& psi) {
  const int N = o.N;
  build_operator(o, phase);
  std::vector<double> b(N, 0.0);
  for (int i = 0; i < N; ++i) b[i] = o.freev[i] ? nu[i] : 0.0;
  double bn = std::sqrt(dot(b, b));
  psi.assign(N, 0.0);
  if (bn == 0.0) return;
  std::vector<double> r(b), z(N), p(N), q(N);
  for (int i = 0; i < N; ++i) z[i] = o.freev[i] ? r[i] / o.diag[i] : 0.0;
  p = z;
  double rz = dot(r, z);
  for (int it = 0; it < o.max_iter; ++it) {
    apply_A(o, p, q);
    const double pq = dot(p, q);
    if (pq <= 0.0) break;
    const double alpha = rz / pq;
    for (int i = 0; i < N; ++i) {
      psi[i] += alpha * p[i];
      r[i] -= alpha * q[i];
    }
    if (std::sqrt(dot(r, r)) <= 0.1 * o.tol * bn) break;
    for (int i = 0; i < N; ++i) z[i] = o.freev[i] ? r[i] / o.diag[i] : 0.0;
    const double rz2 = dot(r, z);
    const double bt = rz2 / rz;
    rz = rz2;
    for (int i = 0; i < N; ++i) p[i] = z[i] + bt * p[i];
  }
}

// bond weight beta dV / xi^(3+2s)
inline double bond_w(const Oracle& o, int i, int n) {
  const nnpp_params& p = o.p;
  const double xix = o.x[n] - o.x[i], xiy = o.y[n] - o.y[i], xiz = o.z[n] - o.z[i];
  const double xi = std::sqrt(xix * xix + xiy * xiy + xiz * xiz);
  return beta_fn(xi, p.delta, p.dx) * p.dx * p.dy * p.dz / std::pow(xi, 3.0 + 2.0 * p.s_phi);
}

// D of species k on a bond between phases pi, pn (with BV = 10^(-vol_red (1 - voln1rel)))
inline double pair_D(const nnpp_params& p, int k, int pi, int pn, double BVmix) {
  if (pi == 0 && pn == 0) return p.D_liquid[k];
  if (k == 0) return (pi == 1 && pn == 1) ? p.D_solid[0] : p.D_solid[0] * BVmix;
  if (pi == 1 && pn == 1) return 0.0;
  return p.D_solid[k];
}

void adjoint_step(Oracle& o, int n, std::vector<double>& lam, double* gD, double* gk) {
  const nnpp_params& p = o.p;
  const int N = o.N;
  const std::vector<double>& c = g_rec.c[n];
  const std::vector<double>& phi = g_rec.phi[n];
  const std::vector<int>& ph = g_rec.phase[n];
  const std::vector<unsigned char>& cl = g_rec.clamped[n];
  const double BV = std::pow(10., -p.vol_red * (1. - 0.0));
  const double csat = p.CSat / p.CSolid;
  std::vector<double> lh((int64_t)S * N);
  for (int k = 0; k < S; ++k)
    for (int i = 0; i < N; ++i) {
      const int64_t a = (int64_t)k * N + i;
      lh[a] = (o.dir[a] || cl[a]) ? 0.0 : lam[a];
    }
  std::vector<double> mu((int64_t)S * N, 0.0), nu(N, 0.0);
  double gDl[S] = {0, 0, 0, 0}, gkl = 0.0;
  for (int m = 0; m < N; ++m) {
    int iface = 0;
    if (ph[m] == 1)
      for (int64_t j = o.row_ptr[m] + 1; j < o.row_ptr[m + 1]; ++j)
        if (ph[o.cols[j]] == 0) {
          iface = 1;
          break;
        }
    double nul = 0.0;
    for (int k = 0; k < S; ++k) {
      const double* ck = c.data() + (int64_t)k * N;
      const double* lk = lh.data() + (int64_t)k * N;
      const double K2zF = p.K2[k] * p.z[k] * p.F / (p.R * p.T);
      double acc = lk[m], a1 = 0.0, a2 = 0.0, sl = 0.0, sc = 0.0;
      for (int64_t j = o.row_ptr[m] + 1; j < o.row_ptr[m + 1]; ++j) {
        const int i = o.cols[j];
        const double D = pair_D(p, k, ph[m], ph[i], BV);
        if (D == 0.0) continue;
        const double w = bond_w(o, m, i);
        acc += p.dt * p.K1[k] * D * w * (lk[i] - lk[m]);
        acc += lk[i] * p.dt * K2zF * D * w * (phi[m] - phi[i]);
        a1 += D * w * (ck[i] - ck[m]);
        a2 += D * w * ck[i] * (phi[i] - phi[m]);
        sl += D * w * lk[i];
        sc += D * w * ck[i];
      }
      const bool src = (k == 0) && iface && !o.dir[m];
      if (src) {
        acc += lk[m] * (-p.dt * p.k_diss * mg_source_switch_deriv(p, ck[m]));
        gkl += lk[m] * (-p.dt * mg_source_switch(p, ck[m]));
      }
      mu[(int64_t)k * N + m] = acc;
      nul += p.dt * K2zF * (ck[m] * sl - lk[m] * sc);
      gDl[k] += lk[m] * p.dt * (p.K1[k] * a1 + K2zF * a2) / p.D_liquid[k];
    }
    nu[m] = nul;
  }
  std::vector<double> psi;
  adjoint_solve(o, ph.data(), nu, psi);
  const double lamp = (1. / (p.K_phi * p.sigma)) * p.F * p.CSolid;
  for (int k = 0; k < S; ++k)
    for (int i = 0; i < N; ++i)
      if (o.freev[i]) mu[(int64_t)k * N + i] += lamp * p.z[k] * psi[i];
  lam.swap(mu);
  for (int k = 0; k < S; ++k) gD[k] += gDl[k];
  *gk += gkl;
}

double mg_mass_lost(const Oracle& o) {
  double m = 0.0;
  for (int i = 0; i < o.N; ++i) m += o.c0_init[i] - o.c[i];
  return m * o.p.dx * o.p.dy * o.p.dz;
}

// ---------------------------------------------------------------------------------------
// The reference's complete residual, utils::Residuals (utils.h:29-842): ten species, their
// reactions, the potential.  A restatement of its formulas in its operand order, each field's
// sums over the horizon in order, so that it reproduces the reference bit for bit (pinned
// against tests/golden/chemistry.npz).  Parameter arrays as the reference's data files hold
// them (utils.h:2343-2484): data2 (51), datac (10 x 7: z, D_solid, D_liquid, s_1, s_2,
// K_prop1, K_prop2), datac11 (sigma0, sigma1, s_11, K11prop1).  Clouds in the reference's
// format: row i's horizon cols[row_ptr[i] .. row_ptr[i+1]), the node itself first.
void residuals_full(int N, const double* x, const int64_t* rp, const int* cols, const double* Un1,
                    const double* Un, const int* phase, double voln1rel, const double* d2,
                    const double* dc, const double* d11, double* Fout) {
  const double dt = d2[2], dx = d2[3], dy = d2[4], dz = d2[5], delta = d2[6];
  const double CSolid = d2[7], CSat = d2[8];
  const double phim = d2[23], phimse = d2[24], alphaC = d2[27];
  const double k1b = d2[29], k2b = d2[31], k3b = d2[33], k4b = d2[35], k5b = d2[37], k6b = d2[39];
  const double k7b = d2[41], k8b = d2[43], k9b = d2[45];
  const double JHp = d2[46], T = d2[47], R = d2[48], Fc = d2[49], vol_red = d2[50];
  auto P = [&](int i) { return std::pow(10., -d2[i]) / CSolid; };  // 10^-pK / CSolid
  const double pMgOH2 = P(14), pMgCO3 = P(15), pMgHCO3 = P(16), pMgPO4 = P(17), pCaCO3 = P(18);
  const double pCa5 = P(19), pH2O = P(20), pHCO3 = P(21), pHPO4 = P(22);
  const double sigma1 = d11[1], s111 = d11[2], K11 = d11[3];
  auto U1 = [&](int k, int i) { return Un1[(int64_t)k * N + i]; };  // U_{k+1}^{n+1}
  auto U0 = [&](int k, int i) { return Un[(int64_t)k * N + i]; };   // U_{k+1}^n
  for (int k = 0; k <= 10; ++k)
    for (int i = 0; i < N; ++i) Fout[(int64_t)k * N + i] = 0.0;
  // species k (0-based): bond sums and the reaction term of node i
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < N; ++i) {
    int iface = 0;
    if (phase[i] == 1)
      for (int64_t j = rp[i] + 1; j < rp[i + 1]; ++j)
        if (phase[cols[j]] == 0) {
          iface = 1;
          break;
        }
    for (int k = 0; k < 10; ++k) {
      const double* c = dc + 7 * k;
      const double z = c[0], Ds = c[1], Dl = c[2], s1 = c[3], s2 = c[4], K1 = c[5], K2 = c[6];
      double sum1 = 0.0, sum2 = 0.0;
      for (int64_t j = rp[i] + 1; j < rp[i + 1]; ++j) {
        const int n = cols[j];
        const double xx = x[n] - x[i], yy = x[N + n] - x[N + i], zz = x[2 * N + n] - x[2 * N + i];
        const double xi = std::sqrt(xx * xx + yy * yy + zz * zz);
        const bool ss = phase[i] == 1 && phase[n] == 1, ll = phase[i] == 0 && phase[n] == 0;
        const double b = beta_fn(xi, delta, dx);
        const double du = U1(k, n) - U1(k, i), dphi = U0(10, n) - U0(10, i);
        if (k == 0) {
          // Mg (utils.h:100-160): BV on bonds touching the solid, solid-solid bonds kept
          if (!ll) {
            const double BV = ss ? 1.0 : std::pow(10., -vol_red * (1. - voln1rel));
            sum1 += -(K1 * Ds * BV * du / std::pow(xi, 3.0 + 2.0 * s1)) * b * dx * dy * dz;
            sum2 += -(K2 * Ds * BV * z * Fc * U1(k, n) * dphi / (R * T * std::pow(xi, 3.0 + 2.0 * s2))) * b * dx * dy * dz;
          } else {
            sum1 += -(K1 * Dl * du / std::pow(xi, 3.0 + 2.0 * s1)) * b * dx * dy * dz;
            sum2 += -(K2 * Dl * z * Fc * U1(k, n) * dphi / (R * T * std::pow(xi, 3.0 + 2.0 * s2))) * b * dx * dy * dz;
          }
        } else {
          // the other species (utils.h:205-239 and alike): solid-solid bonds skipped
          if (ss) continue;
          const double D = ll ? Dl : Ds;
          sum1 += -(K1 * D * du / std::pow(xi, 3.0 + 2.0 * s1)) * b * dx * dy * dz;
          sum2 += -(K2 * D * z * Fc * U1(k, n) * dphi / (R * T * std::pow(xi, 3.0 + 2.0 * s2))) * b * dx * dy * dz;
        }
      }
      const bool liq = phase[i] == 0, act = iface == 1 || liq;
      double Rk = 0.0;
      const double u8 = U0(7, i), u7 = U0(6, i);
      auto ca5 = [&](double a) { return a * u8 * u8 * u8 * u8 * u8 * u7 * u7 * u7; };
      switch (k) {
        case 0:  // utils.h:162-174
          if (act)
            Rk = -k1b * std::max((U1(0, i) * U0(2, i) * U0(2, i) - pMgOH2), 0.0) -
                 k2b * std::max((U1(0, i) * U0(4, i) - pMgCO3), 0.0) -
                 k3b * std::max((U1(0, i) * U0(4, i) - pMgHCO3), 0.0) -
                 k4b * std::max((U0(0, i) * U0(0, i) * U0(0, i) * U0(5, i) * U0(5, i) - pMgPO4), 0.0);
          break;
        case 1:  // utils.h:241-253
          if (iface == 1) {
            const double phic = (R * T / (Fc * dc[0])) * std::log(U0(0, i) / (CSat / CSolid));
            const double eta = phim + phimse - U0(10, i) - phic;
            Rk += (JHp / (z * Fc * CSolid)) * std::exp(-alphaC * Fc * eta / (R * T));
          } else if (liq) {
            Rk = k7b * (pH2O - U1(1, i) * U0(2, i)) + k8b * (pHCO3 - U1(1, i) * U0(4, i)) +
                 k9b * (pHPO4 - U1(1, i) * U0(6, i));
          }
          break;
        case 2:  // utils.h:321-330
          if (act) {
            Rk = -k1b * std::max((U0(2, i) * U0(2, i) * U0(0, i) - pMgOH2), 0.0) -
                 k6b * std::max((ca5(U1(2, i)) - pCa5), 0.0);
            if (liq) Rk += k7b * (pH2O - U1(2, i) * U0(1, i));
          }
          break;
        case 3:  // utils.h:396-401
          if (liq) Rk = k8b * (pHCO3 - U1(3, i) * U0(1, i));
          break;
        case 4:  // utils.h:466-476
          if (act) {
            Rk = -k2b * std::max((U1(4, i) * U0(0, i) - pMgCO3), 0.0) -
                 k3b * std::max((U1(4, i) * U0(0, i) - pMgHCO3), 0.0) -
                 k5b * std::max((U1(4, i) * U0(7, i) - pCaCO3), 0.0);
            if (liq) Rk += k8b * (pHCO3 - U0(1, i) * U1(4, i));
          }
          break;
        case 5:  // utils.h:541-547
          if (act) {
            Rk = -k4b * std::max((U0(0, i) * U0(0, i) * U0(0, i) * U0(5, i) * U0(5, i) - pMgPO4), 0.0);
            if (liq) Rk += k9b * (-pHPO4 + U0(6, i) * U0(1, i));
          }
          break;
        case 6:  // utils.h:612-618
          if (act) {
            Rk = -k6b * std::max((ca5(U0(2, i)) - pCa5), 0.0);
            if (liq) Rk += k9b * (pHPO4 - U1(6, i) * U0(1, i));
          }
          break;
        case 7:  // utils.h:683-690
          if (act)
            Rk = -k5b * std::max((U1(7, i) * U0(4, i) - pCaCO3), 0.0) -
                 k6b * std::max((ca5(U0(2, i)) - pCa5), 0.0);
          break;
        default:  // species 9, 10: no reaction (utils.h:744, 795)
          break;
      }
      Fout[(int64_t)k * N + i] = ((U1(k, i) - U0(k, i)) / dt) + sum1 + sum2 - Rk;
    }
    // potential (utils.h:801-841)
    double s11 = 0.0;
    int flag = 0;
    for (int64_t j = rp[i] + 1; j < rp[i + 1]; ++j) {
      const int n = cols[j];
      if (!(phase[i] == 0 && phase[n] == 0)) continue;
      const double xx = x[n] - x[i], yy = x[N + n] - x[N + i], zz = x[2 * N + n] - x[2 * N + i];
      const double xi = std::sqrt(xx * xx + yy * yy + zz * zz);
      s11 += -(K11 * sigma1 * (U1(10, n) - U1(10, i)) / std::pow(xi, 3.0 + 2.0 * s111)) *
             beta_fn(xi, delta, dx) * dx * dy * dz;
      flag = 1;
    }
    if (flag) {
      double r11 = 0.0;
      for (int k = 0; k < 10; ++k) r11 = (k == 0) ? dc[0] * U0(0, i) : r11 + dc[7 * k] * U0(k, i);
      Fout[(int64_t)10 * N + i] = (1. / (K11 * sigma1)) * s11 - (1. / (K11 * sigma1)) * Fc * CSolid * r11;
    }
  }
}

}  // namespace


// ================================================================ C interface =============
// ---------------------------------------------------------------- implicit step ----------
// The reference's production time step (main.cpp:640-922): backward Euler with one tangent
// per step (utils::NewtonMatrices, utils.h:844-1790), then Newton iterations of
//   F = Residuals(U^{n+1}, U^n)  (utils.h:29-842; Dirichlet rows F = U - bc, main.cpp:676-712)
//   K_f dU_f = -F_f for every field f separately (Eigen::GMRES, restart 30, diagonal
//   preconditioner, tolerance EPS, MAX_ITER iterations: main.cpp:714-779),
//   U += dU, the positivity clamp (main.cpp:805-837),
// until max_f | ||dU_f|| - ||dU_f|| of the previous iteration | < EPS (main.cpp:847-895), then
// the phase flip (main.cpp:914-922).  Here with four species and the potential: the migration
// terms use the lagged potential phi^n (U11n, utils.h:126), the potential's residual the
// new one.  EPS = 10E-6, MAX_ITER = 200 (main.cpp:33-36).
constexpr double kNewtonEps = 10E-6;
constexpr int kNewtonMaxIter = 200;

// Residual of the implicit step (utils.h:72-178, 181-257, 798-841 with U^{n+1} = c1, phi1 and
// U^n = c0, phi0): the time term (c1 - c0) / dt, the bond sums at c1 with the migration
// potential phi0, the dissolution source at c1; F11 from the potential phi1 and the charge
// of U^n (utils.h:829-831: R11 = z1 U1n + ... + z10 U10n).
void residuals_implicit(const Oracle& o, const double* c1, const double* phi1, const double* c0,
                        const double* phi0, const int* phase, double voln1rel, double* F) {
  residuals(o, c1, phi0, phase, voln1rel, F, nullptr, nullptr);
  const int N = o.N;
  std::vector<double> F11(F + (int64_t)S * N, F + (int64_t)(S + 1) * N);
  std::vector<double> tmp((int64_t)(S + 1) * N);
  residuals(o, c0, phi1, phase, voln1rel, tmp.data(), nullptr, nullptr);
#pragma omp parallel for
  for (int i = 0; i < N; ++i) {
    for (int k = 0; k < S; ++k) {
      const int64_t q = (int64_t)k * N + i;
      // residuals() adds (c - c) / dt = 0; the reference's (U^{n+1} - U^n) / dt first
      F[q] = ((c1[q] - c0[q]) / o.p.dt) + F[q];
    }
    F[(int64_t)S * N + i] = tmp[(int64_t)S * N + i];
  }
}

// Tangent of species k (utils.h:900-1010 for Mg, 1012-1102 for the generic species; the
// reaction terms of the diagonal vanish for this model): per bond (slot j of row i)
//   off[j] = -( K1 D(BV) / xi^(3+2s1) + K2 D(BV) z F / (R T) (phi_n - phi_i) / xi^(3+2s2) ) beta dV
// with the generic species' solid-solid bonds absent; diag[i] = 1/dt - sum_K,
// sum_K = sum -(K1 D(BV) / xi^(3+2s1)) beta dV; Dirichlet rows identity.
void species_tangent(const Oracle& o, int k, const double* phi0, const int* phase, double voln1rel,
                     std::vector<double>& diag, std::vector<double>& off) {
  const nnpp_params& p = o.p;
  const int N = o.N;
  const double BVmix = std::pow(10., -p.vol_red * (1. - voln1rel));
  diag.assign(N, 1.0);
  off.assign(o.cols.size(), 0.0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < N; ++i) {
    if (o.dir[(int64_t)k * N + i]) continue;
    double sumK = 0.0;
    for (int64_t j = o.row_ptr[i] + 1; j < o.row_ptr[i + 1]; ++j) {
      const int n = o.cols[j];
      const int pi = phase[i], pn = phase[n];
      double D, BV = 1.0;
      if (k == 0) {
        if ((pi == 1 && pn == 0) || (pn == 1 && pi == 0)) BV = BVmix;
        D = (pi == 0 && pn == 0) ? p.D_liquid[0] : p.D_solid[0];
      } else {
        if (pi == 1 && pn == 1) continue;
        D = (pi == 0 && pn == 0) ? p.D_liquid[k] : p.D_solid[k];
      }
      const double xix = o.x[n] - o.x[i], xiy = o.y[n] - o.y[i], xiz = o.z[n] - o.z[i];
      const double xi = std::sqrt(xix * xix + xiy * xiy + xiz * xiz);
      const double bt = beta_fn(xi, p.delta, p.dx);
      if (k == 0) {
        sumK += -(p.K1[0] * D * BV / std::pow(xi, 3.0 + 2.0 * p.s1[0])) * bt * p.dx * p.dy * p.dz;
        off[j] = -((p.K1[0] * D * BV / std::pow(xi, 3.0 + 2.0 * p.s1[0])) +
                   (p.K2[0] * D * BV * p.z[0] * p.F / (p.R * p.T) * (phi0[n] - phi0[i]) /
                    std::pow(xi, 3.0 + 2.0 * p.s2[0]))) *
                 bt * p.dx * p.dy * p.dz;
      } else {
        sumK += -(p.K1[k] * D / std::pow(xi, 3.0 + 2.0 * p.s1[k])) * bt * p.dx * p.dy * p.dz;
        off[j] = -((p.K1[k] * D / std::pow(xi, 3.0 + 2.0 * p.s1[k])) +
                   (p.K2[k] * D * p.z[k] * p.F / (p.R * p.T) * (phi0[n] - phi0[i]) /
                    std::pow(xi, 3.0 + 2.0 * p.s2[k]))) *
                 bt * p.dx * p.dy * p.dz;
      }
    }
    diag[i] = (1. / p.dt) - sumK - 0.0;
  }
}

// y = K x for a field's tangent: diag and per-bond off-diagonals (rows of the reference's
// neighbour lists, slot 0 the node itself)
void apply_tangent(const Oracle& o, const std::vector<double>& diag, const std::vector<double>& off,
                   const double* x, double* y) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < o.N; ++i) {
    double acc = diag[i] * x[i];
    for (int64_t j = o.row_ptr[i] + 1; j < o.row_ptr[i + 1]; ++j) acc += off[j] * x[o.cols[j]];
    y[i] = acc;
  }
}

double norm2(const double* a, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * a[i];
  return std::sqrt(s);
}

// Eigen::GMRES (GMRES.h:56-203) as the reference calls it: initial guess x = b
// (_solve_impl, GMRES.h:330-334; nothing to do for b = 0), the diagonal (Jacobi) preconditioner
// applied on the left, restarts of `restart` steps, iterations counted over restarts up to
// maxit, stop when |g_k| / ||M^-1 (b - A x_0)|| < tol (the initial preconditioned residual,
// kept across restarts).  The Arnoldi basis is built by modified Gram-Schmidt (the reference
// uses Householder reflections: the same Krylov space and least-squares problem).  Returns
// the iterations.
int gmres(const Oracle& o, const std::vector<double>& diag, const std::vector<double>& off, const double* b,
          double* x, double tol, int restart, int maxit) {
  const int n = o.N;
  bool zero = true;
  for (int i = 0; i < n && zero; ++i) zero = b[i] == 0.0;
  if (zero) {
    std::fill(x, x + n, 0.0);
    return 0;
  }
  std::copy(b, b + n, x);
  std::vector<double> r(n), t(n);
  auto presid = [&]() {
    apply_tangent(o, diag, off, x, t.data());
    for (int i = 0; i < n; ++i) r[i] = (b[i] - t[i]) / diag[i];
  };
  presid();
  const double r0norm = norm2(r.data(), n);
  if (r0norm == 0.0) return 0;
  int iters = 0;
  std::vector<std::vector<double> > V(restart + 1, std::vector<double>(n));
  std::vector<double> H((size_t)(restart + 1) * restart), cs(restart), sn(restart), g(restart + 1);
  for (;;) {
    const double beta = norm2(r.data(), n);
    for (int i = 0; i < n; ++i) V[0][i] = r[i] / beta;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;
    bool stop = false;
    for (k = 1; k <= restart; ++k) {
      ++iters;
      std::vector<double>& w = V[k];
      apply_tangent(o, diag, off, V[k - 1].data(), t.data());
      for (int i = 0; i < n; ++i) w[i] = t[i] / diag[i];
      for (int q = 0; q < k; ++q) {
        double h = 0.0;
        for (int i = 0; i < n; ++i) h += w[i] * V[q][i];
        H[(size_t)q * restart + (k - 1)] = h;
        for (int i = 0; i < n; ++i) w[i] -= h * V[q][i];
      }
      const double hk = norm2(w.data(), n);
      H[(size_t)k * restart + (k - 1)] = hk;
      if (hk != 0.0)
        for (int i = 0; i < n; ++i) w[i] /= hk;
      for (int q = 0; q < k - 1; ++q) {  // earlier rotations on the new column
        const double a = H[(size_t)q * restart + (k - 1)], c = H[(size_t)(q + 1) * restart + (k - 1)];
        H[(size_t)q * restart + (k - 1)] = cs[q] * a + sn[q] * c;
        H[(size_t)(q + 1) * restart + (k - 1)] = -sn[q] * a + cs[q] * c;
      }
      const double a = H[(size_t)(k - 1) * restart + (k - 1)], c = H[(size_t)k * restart + (k - 1)];
      const double den = std::hypot(a, c);
      cs[k - 1] = den == 0.0 ? 1.0 : a / den;
      sn[k - 1] = den == 0.0 ? 0.0 : c / den;
      H[(size_t)(k - 1) * restart + (k - 1)] = den;
      H[(size_t)k * restart + (k - 1)] = 0.0;
      g[k] = -sn[k - 1] * g[k - 1];
      g[k - 1] = cs[k - 1] * g[k - 1];
      const double err = std::abs(g[k]) / r0norm;
      stop = k == n || err < tol || iters == maxit;
      if (stop || k == restart) break;
    }
    if (k > restart) k = restart;
    // y = H^-1 g (upper triangular), x += V y
    std::vector<double> y(k);
    for (int q = k - 1; q >= 0; --q) {
      double sum = g[q];
      for (int u = q + 1; u < k; ++u) sum -= H[(size_t)q * restart + u] * y[u];
      y[q] = sum / H[(size_t)q * restart + q];
    }
    for (int q = 0; q < k; ++q)
      for (int i = 0; i < n; ++i) x[i] += y[q] * V[q][i];
    if (stop) return iters;
    presid();
  }
}

// K11 (the potential's tangent, utils.h:1797-1848) in the diag/off form of apply_tangent:
// off-diagonal -w on liquid-liquid bonds of free rows, identity rows elsewhere
void potential_tangent(Oracle& o, const int* phase, std::vector<double>& diag, std::vector<double>& off) {
  build_operator(o, phase);
  diag = o.diag;
  off.assign(o.cols.size(), 0.0);
  for (size_t j = 0; j < off.size(); ++j) off[j] = -o.wphi[j];
}

struct ImplicitStats {
  int newton = 0;
  int64_t krylov = 0;
};

// One implicit step of the reference's time loop from the oracle's state (c, phi = U^n).
int implicit_step(Oracle& o, ImplicitStats* st) {
  const nnpp_params& p = o.p;
  const int N = o.N;
  const int F1 = S + 1;
  std::vector<double> u0((int64_t)F1 * N), u1, F((int64_t)F1 * N), dU((int64_t)F1 * N), rhs(N);
  std::copy(o.c.begin(), o.c.end(), u0.begin());
  std::copy(o.phi.begin(), o.phi.end(), u0.begin() + (int64_t)S * N);
  u1 = u0;
  const double* phi0 = u0.data() + (int64_t)S * N;
  // the tangents once per step, at U^{n+1} = U^n (main.cpp:657-662)
  std::vector<double> diag[S + 1], off[S + 1];
  for (int k = 0; k < S; ++k) species_tangent(o, k, phi0, o.phase.data(), o.voln1rel, diag[k], off[k]);
  potential_tangent(o, o.phase.data(), diag[S], off[S]);
  double res_old[S + 1] = {0, 0, 0, 0, 0};
  const double floor_c = 1.0e-8 / p.CSolid;
  int it = 0;
  for (it = 0; it < kNewtonMaxIter; ++it) {
    residuals_implicit(o, u1.data(), u1.data() + (int64_t)S * N, u0.data(), phi0, o.phase.data(), o.voln1rel,
                       F.data());
    // main.cpp:676-712: species' boundary values divided by CSolid, the potential's not
    for (int f = 0; f <= S; ++f)
      for (int i = 0; i < N; ++i)
        if (o.dir[(int64_t)f * N + i])
          F[(int64_t)f * N + i] =
              u1[(int64_t)f * N + i] - (f < S ? o.bcv[(int64_t)f * N + i] / p.CSolid : o.bcv[(int64_t)f * N + i]);
    double res[S + 1];
    for (int f = 0; f <= S; ++f) {
      for (int i = 0; i < N; ++i) rhs[i] = -F[(int64_t)f * N + i];
      const int kit = gmres(o, diag[f], off[f], rhs.data(), dU.data() + (int64_t)f * N, kNewtonEps, 30,
                            kNewtonMaxIter);
      if (st) st->krylov += kit;
    }
    for (int f = 0; f <= S; ++f) {
      for (int i = 0; i < N; ++i) u1[(int64_t)f * N + i] += dU[(int64_t)f * N + i];
      res[f] = norm2(dU.data() + (int64_t)f * N, N);
    }
    for (int k = 0; k < S; ++k)
      for (int i = 0; i < N; ++i)
        if (u1[(int64_t)k * N + i] < floor_c) u1[(int64_t)k * N + i] = floor_c;
    double resMax = 0.0;
    for (int f = 0; f <= S; ++f) resMax = std::max(resMax, std::abs(res[f] - res_old[f]));
    if (resMax < kNewtonEps) {
      ++it;
      break;
    }
    for (int f = 0; f <= S; ++f) res_old[f] = res[f];
  }
  if (st) st->newton = it;
  std::copy(u1.begin(), u1.begin() + (int64_t)S * N, o.c.begin());
  std::copy(u1.begin() + (int64_t)S * N, u1.end(), o.phi.begin());
  // phase flip (main.cpp:914-922) and the volume (main.cpp:944-949) as in the explicit step
  const double csat = p.CSat / p.CSolid;
  for (int i = 0; i < N; ++i)
    if (o.phase[i] == 1 && o.c[i] <= csat) {
      o.phase[i] = 0;
      o.flip_step[i] = (int)(o.steps_done + 1);
      o.solid_count -= 1;
      o.op_valid = false;
    }
  o.steps_done += 1;
  if (p.sub_step_no > 0 && o.steps_done % p.sub_step_no == 0) {
    double v = 0.0;
    for (int i = 0; i < N; ++i)
      if (o.phase[i] == 1) v += o.c[i] - csat;
    o.voln1rel = o.vol0rel != 0.0 ? v / o.vol0rel : 0.0;
  }
  return 0;
}

// ------------------------------------------------ the complete model's implicit step -----
// The reference's time step with all eleven fields (main.cpp:640-922): the tangents of
// utils::NewtonMatrices (utils.h:846-1849) once at U^n, then Newton iterations on
// utils::Residuals (utils.h:29-842, residuals_full above) with the Dirichlet rows of
// main.cpp:676-712, eleven Eigen::GMRES corrections (gmres above), the update, the clamp of
// main.cpp:805-837 (U10 on liquid nodes only) and the update-norm test; then the flip of
// main.cpp:914-922.  Parameters as the reference's data files hold them (data2, datac rows
// z, D_solid, D_liquid, s_k1, s_k2, K_kprop1, K_kprop2, datac11).

// tangent of species k (Mg utils.h:900-1010; H+ 1012-1102; species 3-10 1104-1792): the
// off-diagonal and sum_K of species_tangent with the species' own constants; the diagonal
// 1/dt - sum_K - R_k with the linearised reaction terms at U^n (H+ on interface and liquid
// nodes, species 3, 4, 5 and 7 on liquid nodes, none for the others)
void chem_species_tangent(const Oracle& o, int k, const double* Un, const int* phase, const unsigned char* dir,
                          double voln1rel, const double* d2, const double* dc, std::vector<double>& diag,
                          std::vector<double>& off) {
  const int N = o.N;
  const double dt = d2[2], dx = d2[3], dy = d2[4], dz = d2[5], delta = d2[6];
  const double T = d2[47], R = d2[48], Fc = d2[49], vol_red = d2[50];
  const double k7b = d2[41], k8b = d2[43], k9b = d2[45];
  const double z = dc[7 * k], Ds = dc[7 * k + 1], Dl = dc[7 * k + 2], s1 = dc[7 * k + 3], s2 = dc[7 * k + 4];
  const double K1 = dc[7 * k + 5], K2 = dc[7 * k + 6];
  const double BVmix = std::pow(10., -vol_red * (1. - voln1rel));
  auto U = [&](int f, int i) { return Un[(int64_t)f * N + i]; };
  diag.assign(N, 1.0);
  off.assign(o.cols.size(), 0.0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < N; ++i) {
    if (dir[i]) continue;
    const int pi = phase[i];
    int iface = 0;
    if (pi == 1)
      for (int64_t j = o.row_ptr[i] + 1; j < o.row_ptr[i + 1]; ++j)
        if (phase[o.cols[j]] == 0) {
          iface = 1;
          break;
        }
    double sumK = 0.0;
    for (int64_t j = o.row_ptr[i] + 1; j < o.row_ptr[i + 1]; ++j) {
      const int n = o.cols[j];
      const int pn = phase[n];
      double D, BV = 1.0;
      if (k == 0) {
        if ((pi == 1 && pn == 0) || (pn == 1 && pi == 0)) BV = BVmix;
        D = (pi == 0 && pn == 0) ? Dl : Ds;
      } else {
        if (pi == 1 && pn == 1) continue;
        D = (pi == 0 && pn == 0) ? Dl : Ds;
      }
      const double xix = o.x[n] - o.x[i], xiy = o.y[n] - o.y[i], xiz = o.z[n] - o.z[i];
      const double xi = std::sqrt(xix * xix + xiy * xiy + xiz * xiz);
      const double bt = beta_fn(xi, delta, dx);
      const double dphi = U(10, n) - U(10, i);
      if (k == 0) {
        sumK += -(K1 * D * BV / std::pow(xi, 3.0 + 2.0 * s1)) * bt * dx * dy * dz;
        off[j] = -((K1 * D * BV / std::pow(xi, 3.0 + 2.0 * s1)) +
                   (K2 * D * BV * z * Fc / (R * T) * dphi / std::pow(xi, 3.0 + 2.0 * s2))) *
                 bt * dx * dy * dz;
      } else {
        sumK += -(K1 * D / std::pow(xi, 3.0 + 2.0 * s1)) * bt * dx * dy * dz;
        off[j] = -((K1 * D / std::pow(xi, 3.0 + 2.0 * s1)) +
                   (K2 * D * z * Fc / (R * T) * dphi / std::pow(xi, 3.0 + 2.0 * s2))) *
                 bt * dx * dy * dz;
      }
    }
    const bool liq = pi == 0;
    double Rk = 0.0;
    if (k == 1 && (iface || liq))
      Rk = k7b * (-U(2, i)) + k8b * (-U(4, i)) + k9b * (-U(6, i));
    else if (k == 2 && liq)
      Rk = k7b * (-U(1, i));
    else if ((k == 3 || k == 4) && liq)
      Rk = k8b * (-U(1, i));
    else if (k == 6 && liq)
      Rk = k9b * (-U(1, i));
    diag[i] = (1. / dt) - sumK - Rk;
  }
}

// K11 (utils.h:1794-1848) with datac11's constants: off-diagonal
// -(1/(K sigma)) (K sigma / xi^(3+2s)) beta dV on liquid-liquid bonds, diagonal
// -(1/(K sigma)) sum_K; identity rows on Dirichlet nodes and nodes without such bonds
void chem_potential_tangent(const Oracle& o, const int* phase, const unsigned char* dir, const double* d2,
                            const double* d11, std::vector<double>& diag, std::vector<double>& off) {
  const int N = o.N;
  const double dx = d2[3], dy = d2[4], dz = d2[5], delta = d2[6];
  const double sigma1 = d11[1], s111 = d11[2], K11 = d11[3];
  diag.assign(N, 1.0);
  off.assign(o.cols.size(), 0.0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < N; ++i) {
    if (dir[i]) continue;
    double sumK = 0.0;
    int flag = 0;
    for (int64_t j = o.row_ptr[i] + 1; j < o.row_ptr[i + 1]; ++j) {
      const int n = o.cols[j];
      if (!(phase[i] == 0 && phase[n] == 0)) continue;
      const double xix = o.x[n] - o.x[i], xiy = o.y[n] - o.y[i], xiz = o.z[n] - o.z[i];
      const double xi = std::sqrt(xix * xix + xiy * xiy + xiz * xiz);
      const double bt = beta_fn(xi, delta, dx);
      sumK += -(K11 * sigma1 / std::pow(xi, 3.0 + 2.0 * s111)) * bt * dx * dy * dz;
      off[j] = -(1. / (K11 * sigma1)) * (K11 * sigma1 / std::pow(xi, 3.0 + 2.0 * s111)) * bt * dx * dy * dz;
      flag = 1;
    }
    diag[i] = flag ? -(1. / (K11 * sigma1)) * sumK : 1.0;
  }
}

// One step from U (11 N, U^n in, U^{n+1} out) and phase (updated by the flip); dir (11 N)
// the Dirichlet flags, bcv (11 N) the raw boundary values.  Returns the Newton iterations.
int chem_implicit_step(const Oracle& o, double* U, int* phase, const unsigned char* dir, const double* bcv,
                       double voln1rel, const double* d2, const double* dc, const double* d11,
                       int64_t* krylov) {
  const int N = o.N;
  const int NF = 11;
  const double CSolid = d2[7], CSat = d2[8];
  std::vector<double> u0(U, U + (int64_t)NF * N), u1 = u0, F((int64_t)NF * N), dU((int64_t)NF * N), rhs(N);
  std::vector<double> xyz((int64_t)3 * N);
  std::copy(o.x.begin(), o.x.end(), xyz.begin());
  std::copy(o.y.begin(), o.y.end(), xyz.begin() + N);
  std::copy(o.z.begin(), o.z.end(), xyz.begin() + 2 * (int64_t)N);
  // the tangents once per step (main.cpp:657-662)
  std::vector<double> diag[11], off[11];
  for (int k = 0; k < 10; ++k)
    chem_species_tangent(o, k, u0.data(), phase, dir + (int64_t)k * N, voln1rel, d2, dc, diag[k], off[k]);
  chem_potential_tangent(o, phase, dir + (int64_t)10 * N, d2, d11, diag[10], off[10]);
  double res_old[11] = {0.0};
  const double floor_c = 1.0e-8 / CSolid;
  int it = 0;
  for (it = 0; it < kNewtonMaxIter; ++it) {
    residuals_full(N, xyz.data(), o.row_ptr.data(), o.cols.data(), u1.data(), u0.data(), phase, voln1rel, d2, dc,
                   d11, F.data());
    for (int f = 0; f < NF; ++f)
      for (int i = 0; i < N; ++i)
        if (dir[(int64_t)f * N + i])
          F[(int64_t)f * N + i] =
              u1[(int64_t)f * N + i] - (f < 10 ? bcv[(int64_t)f * N + i] / CSolid : bcv[(int64_t)f * N + i]);
    double res[11];
    for (int f = 0; f < NF; ++f) {
      for (int i = 0; i < N; ++i) rhs[i] = -F[(int64_t)f * N + i];
      const int kit = gmres(o, diag[f], off[f], rhs.data(), dU.data() + (int64_t)f * N, kNewtonEps, 30,
                            kNewtonMaxIter);
      if (krylov) *krylov += kit;
    }
    for (int f = 0; f < NF; ++f) {
      for (int i = 0; i < N; ++i) u1[(int64_t)f * N + i] += dU[(int64_t)f * N + i];
      res[f] = norm2(dU.data() + (int64_t)f * N, N);
    }
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < 10; ++k)
        if (u1[(int64_t)k * N + i] < floor_c && (k < 9 || phase[i] == 0)) u1[(int64_t)k * N + i] = floor_c;
    double resMax = 0.0;
    for (int f = 0; f < NF; ++f) resMax = std::max(resMax, std::abs(res[f] - res_old[f]));
    if (resMax < kNewtonEps) {
      ++it;
      break;
    }
    for (int f = 0; f < NF; ++f) res_old[f] = res[f];
  }
  std::copy(u1.begin(), u1.end(), U);
  const double csat = CSat / CSolid;
  for (int i = 0; i < N; ++i)
    if (phase[i] == 1 && U[i] <= csat) phase[i] = 0;
  return it;
}

extern "C" {

int orc_residuals_full(int N, const double* nodes, const int64_t* row_ptr, const int* cols, const double* Un1,
                       const double* Un, const int* phase, double voln1rel, const double* data2,
                       const double* datac, const double* datac11, double* F) {
  residuals_full(N, nodes, row_ptr, cols, Un1, Un, phase, voln1rel, data2, datac, datac11, F);
  return 0;
}

void* orc_create(const nnpp_params* p, int N, const double* xyz, const int* bctypes,
                 const double* bcvalues, const double* icvalues, const int* phase0) {
  Oracle* o = new Oracle();
  o->p = *p;
  o->N = N;
  o->x.assign(xyz, xyz + N);
  o->y.assign(xyz + N, xyz + 2 * N);
  o->z.assign(xyz + 2 * N, xyz + 3 * N);
  o->bctypes.assign(bctypes, bctypes + N);
  o->bcv.assign(bcvalues, bcvalues + (int64_t)(S + 1) * N);
  o->dir.assign((int64_t)(S + 1) * N, 0);
  for (int f = 0; f <= S; ++f)
    for (int i = 0; i < N; ++i)
      o->dir[(int64_t)f * N + i] = (bctypes[i] == 0 && bcvalues[(int64_t)f * N + i] != -1) ? 1 : 0;
  o->c.assign(icvalues, icvalues + (int64_t)S * N);
  o->phi.assign(icvalues + (int64_t)S * N, icvalues + (int64_t)(S + 1) * N);
  o->phase.resize(N);
  for (int i = 0; i < N; ++i) o->phase[i] = phase0 ? phase0[i] : (icvalues[i] > 0.0 + 10E-6 ? 1 : 0);
  o->flip_step.assign(N, -1);
  o->c0_init.assign(o->c.begin(), o->c.begin() + N);
  const double csat = p->CSat / p->CSolid;
  o->solid_count = 0;
  o->vol0rel = 0.0;
  for (int i = 0; i < N; ++i)
    if (o->phase[i] == 1) {
      o->solid_count++;
      o->vol0rel += (o->c[i] - csat);
    }
  o->voln1rel = 0.0;
  return o;
}

void orc_destroy(void* h) { delete static_cast<Oracle*>(h); }

void orc_set_solver(void* h, double tol, int max_iter) {
  Oracle* o = static_cast<Oracle*>(h);
  o->tol = tol;
  o->max_iter = max_iter;
}

int orc_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
}

// build_clouds_hash restated; lists kept in the handle
int orc_build_neighbours(void* h, int max_node_no, double r, double cx, double cy, double cz,
                         int* max_len) {
  Oracle* o = static_cast<Oracle*>(h);
  int st = build_clouds(max_node_no, r, cx, cy, cz, o->N, o->x.data(), o->y.data(), o->z.data(),
                        o->row_ptr, o->cols, max_len);
  o->have_nb = (st == 0);
  o->op_valid = false;
  return st;
}

int64_t orc_nnz(void* h) {
  Oracle* o = static_cast<Oracle*>(h);
  return o->have_nb ? o->row_ptr[o->N] : -1;
}

// reference-format lists: lengths (self included), row_ptr (N+1), cols (self first)
int orc_get_clouds(void* h, int* lengths, int64_t* row_ptr, int* cols) {
  Oracle* o = static_cast<Oracle*>(h);
  if (!o->have_nb) return 7;
  for (int i = 0; i < o->N; ++i) {
    if (lengths) lengths[i] = (int)(o->row_ptr[i + 1] - o->row_ptr[i]);
  }
  if (row_ptr) std::copy(o->row_ptr.begin(), o->row_ptr.end(), row_ptr);
  if (cols) std::copy(o->cols.begin(), o->cols.end(), cols);
  return 0;
}

int orc_set_clouds(void* h, const int64_t* row_ptr, const int* cols) {
  Oracle* o = static_cast<Oracle*>(h);
  o->row_ptr.assign(row_ptr, row_ptr + o->N + 1);
  o->cols.assign(cols, cols + row_ptr[o->N]);
  o->have_nb = true;
  o->op_valid = false;
  return 0;
}

int orc_residuals(void* h, const double* c, const double* phi, const int* phase, double voln1rel,
                  double* F) {
  Oracle* o = static_cast<Oracle*>(h);
  if (!o->have_nb) return 7;
  residuals(*o, c, phi, phase, voln1rel, F, nullptr, nullptr);
  return 0;
}

// K11 entries in CSR over the reference-format rows: diag[N], off[nnz] (-w, 0 if not LL),
// free[N].  Rows without liquid-liquid bonds and Dirichlet rows are identity.
int orc_poisson_matrix(void* h, const int* phase, double* diag, double* off, unsigned char* freev) {
  Oracle* o = static_cast<Oracle*>(h);
  if (!o->have_nb) return 7;
  build_operator(*o, phase);
  for (int i = 0; i < o->N; ++i) {
    diag[i] = o->diag[i];
    freev[i] = o->freev[i];
  }
  for (size_t j = 0; j < o->wphi.size(); ++j) off[j] = -o->wphi[j];
  return 0;
}

int orc_solve_potential(void* h, const double* c, const int* phase, double* phi, int* iters,
                        double* relres) {
  Oracle* o = static_cast<Oracle*>(h);
  if (!o->have_nb) return 7;
  return solve_potential(*o, c, phase, phi, iters, relres);
}

int orc_forward(void* h, int n_steps) {
  Oracle* o = static_cast<Oracle*>(h);
  if (!o->have_nb) return 7;
  int worst = 0;
  for (int s = 0; s < n_steps; ++s) {
    int st = step(*o, nullptr);
    if (st) worst = st;
  }
  return worst;
}

int orc_get_state(void* h, double* c, double* phi, int* phase, int* flip_step) {
  Oracle* o = static_cast<Oracle*>(h);
  if (c) std::copy(o->c.begin(), o->c.end(), c);
  if (phi) std::copy(o->phi.begin(), o->phi.end(), phi);
  if (phase) std::copy(o->phase.begin(), o->phase.end(), phase);
  if (flip_step) std::copy(o->flip_step.begin(), o->flip_step.end(), flip_step);
  return 0;
}

int orc_set_state(void* h, const double* c, const double* phi, const int* phase) {
  Oracle* o = static_cast<Oracle*>(h);
  if (c) o->c.assign(c, c + (int64_t)S * o->N);
  if (phi) o->phi.assign(phi, phi + o->N);
  if (phase) o->phase.assign(phase, phase + o->N);
  return 0;
}

// Forward n_steps recording every step; curve[m] = mass loss dV sum_i (c_0,i(0) - c_0,i(t))
// at t = (m+1) sample_every.  Needs vol_red == 0 (BV = 1) for the adjoint.
int orc_forward_record(void* h, int n_steps, int sample_every, double* curve) {
  Oracle* o = static_cast<Oracle*>(h);
  if (!o->have_nb || sample_every < 1) return 1;
  if (o->p.vol_red != 0.0) return 6;
  const int N = o->N;
  g_rec = Record();
  g_rec.steps = n_steps;
  g_rec.sample_every = sample_every;
  g_rec.c0.assign(o->c.begin(), o->c.begin() + N);
  const double dV = o->p.dx * o->p.dy * o->p.dz;
  int worst = 0;
  for (int s = 0; s < n_steps; ++s) {
    g_rec.c.push_back(o->c);
    g_rec.phase.push_back(o->phase);
    StepRecord rec;
    int st = step(*o, &rec);
    if (st) worst = st;
    g_rec.phi.push_back(o->phi);
    g_rec.clamped.push_back(rec.clamped);
    if ((s + 1) % sample_every == 0) {
      double m = 0.0;
      for (int i = 0; i < N; ++i) m += g_rec.c0[i] - o->c[i];
      curve[(s + 1) / sample_every - 1] = m * dV;
    }
  }
  return worst;
}

// dL/d(D_liquid[k]) and dL/dk_diss for dL/d(curve) given, by the adjoint of the recorded run.
int orc_backward(void* h, const double* dL_dcurve, double* grad_D, double* grad_k) {
  Oracle* o = static_cast<Oracle*>(h);
  const int N = o->N;
  const int se = g_rec.sample_every;
  if (g_rec.steps <= 0 || se < 1) return 7;
  const double dV = o->p.dx * o->p.dy * o->p.dz;
  std::vector<double> lam((int64_t)S * N, 0.0);
  for (int k = 0; k < S; ++k) grad_D[k] = 0.0;
  *grad_k = 0.0;
  for (int n = g_rec.steps - 1; n >= 0; --n) {
    if ((n + 1) % se == 0) {
      const double g = dL_dcurve[(n + 1) / se - 1];
      for (int i = 0; i < N; ++i) lam[i] += -dV * g;
    }
    adjoint_step(*o, n, lam, grad_D, grad_k);
  }
  return 0;
}

// diag layout: [steps, solid_count, voln1rel, vol0rel, mass0..3, mg_mass_lost,
//               dissolved_total, cg_iters, cg_solves, cg_nc, last_relres]
int orc_get_diag(void* h, double* out) {
  Oracle* o = static_cast<Oracle*>(h);
  const double dV = o->p.dx * o->p.dy * o->p.dz;
  out[0] = (double)o->steps_done;
  out[1] = (double)o->solid_count;
  out[2] = o->voln1rel;
  out[3] = o->vol0rel;
  for (int k = 0; k < S; ++k) {
    double m = 0.0;
    for (int i = 0; i < o->N; ++i) m += o->c[(int64_t)k * o->N + i];
    out[4 + k] = m * dV;
  }
  out[8] = mg_mass_lost(*o);
  out[9] = o->dissolved_total;
  out[10] = (double)o->cg_iters_total;
  out[11] = (double)o->cg_solves;
  out[12] = (double)o->cg_nc;
  out[13] = o->last_relres;
  return 0;
}

// The implant mask's counts (main.cpp:316-325 with kd_tree_interface.h:156-252): for each
// node the implant points inside the box node +- r (libkdtree++ region bounds c - r, c + r,
// region.hpp:50-51, inclusive as region.hpp:86-93 tests them) whose Euclidean distance
// sqrt(x*x + y*y + z*z) (kd_tree_interface.h:42-48, x = point - node) is <= r.  Every point
// is tested against every node (OpenMP over the nodes): the restatement needs no tree.
int orc_implant_counts(int N, const double* nodes, int M, const double* points, double r, int* counts) {
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < N; ++i) {
    const double c[3] = {nodes[i], nodes[(int64_t)N + i], nodes[2 * (int64_t)N + i]};
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      lo[d] = c[d] - r;
      hi[d] = c[d] + r;
    }
    int cnt = 0;
    for (int j = 0; j < M; ++j) {
      const double q[3] = {points[j], points[(int64_t)M + j], points[2 * (int64_t)M + j]};
      bool in = true;
      for (int d = 0; d < 3; ++d) in = in && !(q[d] < lo[d]) && !(hi[d] < q[d]);
      if (!in) continue;
      const double x = q[0] - c[0], y = q[1] - c[1], z = q[2] - c[2];
      if (std::sqrt(x * x + y * y + z * z) <= r) ++cnt;
    }
    counts[i] = cnt;
  }
  return 0;
}

// one step of the complete model (chem_implicit_step); dir flags from bct (N) and bcv (11 N):
// bct == 0 and bcv != -1.  Returns the Newton iterations (negative on a bad argument).
int orc_chem_implicit_step(void* h, double* U, int* phase, const int* bct, const double* bcv, double voln1rel,
                           const double* d2, const double* dc, const double* d11, int64_t* krylov) {
  if (!h || !U || !phase || !bct || !bcv || !d2 || !dc || !d11) return -1;
  const Oracle& o = *static_cast<Oracle*>(h);
  const int N = o.N;
  std::vector<unsigned char> dir((int64_t)11 * N, 0);
  for (int f = 0; f < 11; ++f)
    for (int i = 0; i < N; ++i) dir[(int64_t)f * N + i] = (bct[i] == 0 && bcv[(int64_t)f * N + i] != -1) ? 1 : 0;
  if (krylov) *krylov = 0;
  return chem_implicit_step(o, U, phase, dir.data(), bcv, voln1rel, d2, dc, d11, krylov);
}

// the tangent of field f (0..10) of the complete model as diag (N) and off (per bond slot)
int orc_chem_tangent(void* h, int f, const double* Un, const int* phase, const int* bct, const double* bcv,
                     double voln1rel, const double* d2, const double* dc, const double* d11, double* diag_out,
                     double* off_out) {
  if (!h || f < 0 || f > 10) return 1;
  const Oracle& o = *static_cast<Oracle*>(h);
  const int N = o.N;
  std::vector<unsigned char> dir(N);
  for (int i = 0; i < N; ++i) dir[i] = (bct[i] == 0 && bcv[(int64_t)f * N + i] != -1) ? 1 : 0;
  std::vector<double> d, q;
  if (f < 10)
    chem_species_tangent(o, f, Un, phase, dir.data(), voln1rel, d2, dc, d, q);
  else
    chem_potential_tangent(o, phase, dir.data(), d2, d11, d, q);
  std::copy(d.begin(), d.end(), diag_out);
  std::copy(q.begin(), q.end(), off_out);
  return 0;
}

// the implicit step's residual at (c1, phi1) from U^n = (c0, phi0) with the given phases
int orc_residuals_implicit(void* h, const double* c1, const double* phi1, const double* c0, const double* phi0,
                           const int* phase, double voln1rel, double* F) {
  if (!h || !c1 || !phi1 || !c0 || !phi0 || !phase || !F) return 1;
  residuals_implicit(*static_cast<Oracle*>(h), c1, phi1, c0, phi0, phase, voln1rel, F);
  return 0;
}

// n implicit steps (main.cpp:640-922); Newton iterations and GMRES iterations over them
int orc_implicit_forward(void* h, int n_steps, int64_t* newton, int64_t* krylov) {
  Oracle* o = static_cast<Oracle*>(h);
  if (!o->have_nb) return 7;
  int64_t nw = 0, kr = 0;
  for (int s = 0; s < n_steps; ++s) {
    ImplicitStats st;
    implicit_step(*o, &st);
    nw += st.newton;
    kr += st.krylov;
  }
  if (newton) *newton = nw;
  if (krylov) *krylov = kr;
  return 0;
}

// The tangent of field f (0..3 species, 4 potential) at the current state, in the layout of
// the neighbour lists (off[j] for slot j, slot 0 of a row unused)
int orc_tangent(void* h, int f, double* diag, double* off) {
  Oracle* o = static_cast<Oracle*>(h);
  if (!o->have_nb || f < 0 || f > S) return 1;
  std::vector<double> d, q;
  if (f < S)
    species_tangent(*o, f, o->phi.data(), o->phase.data(), o->voln1rel, d, q);
  else
    potential_tangent(*o, o->phase.data(), d, q);
  std::copy(d.begin(), d.end(), diag);
  std::copy(q.begin(), q.end(), off);
  return 0;
}

// x = GMRES(K_f, b) as the implicit step solves its corrections
int orc_tangent_gmres(void* h, int f, const double* b, double* x, double tol, int restart, int maxit) {
  Oracle* o = static_cast<Oracle*>(h);
  if (!o->have_nb || f < 0 || f > S) return -1;
  std::vector<double> d, q;
  if (f < S)
    species_tangent(*o, f, o->phi.data(), o->phase.data(), o->voln1rel, d, q);
  else
    potential_tangent(*o, o->phase.data(), d, q);
  return gmres(*o, d, q, b, x, tol, restart, maxit);
}

}  // extern "C"
