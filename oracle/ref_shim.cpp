// ref_shim.cpp -- C entry points around the reference's own hot-path code.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_oracle.py, in this container only,
// from the reference's headers where they lie (src/helpers/grid.h, src/helpers/utils.h,
// vendored Eigen); the output goes to oracle/_ref/, which is not committed.  It exists to
// pin the oracle restatement (nnpp_oracle.cpp) and to generate the golden fixtures under
// tests/golden/.  Nothing here is part of the product.
#include <cstdint>
#include <cstring>
#include <iostream>
#include <vector>

#include <Eigen/Dense>
#include <Eigen/Sparse>
#include <unsupported/Eigen/IterativeSolvers>

#include "grid.h"
#include "utils.h"
#include "kd_tree_interface.h"

namespace {

std::vector<int> g_len;
std::vector<int64_t> g_ptr;
std::vector<int> g_cols;

typedef Eigen::SparseMatrix<double> SpMat;

// Reference parameter object from the shim's flat inputs: data2 (51), datac (10 x 7),
// datac11 (4), laid out as utils::parameter::set_double expects (utils.h:2343-2484).
void make_params(utils::parameter& prm, int N, const double* data2, const double* datac,
                 const double* datac11) {
  Eigen::VectorXd d1(4), d2(51), c[10], c11(4);
  d1 << N, 1, 0, 0;
  for (int i = 0; i < 51; ++i) d2[i] = data2[i];
  for (int k = 0; k < 10; ++k) {
    c[k].resize(7);
    for (int j = 0; j < 7; ++j) c[k][j] = datac[k * 7 + j];
  }
  for (int j = 0; j < 4; ++j) c11[j] = datac11[j];
  prm.set_int(d1);
  prm.set_double(d2, c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], c[8], c[9], c11);
}

}  // namespace

extern "C" {

// build_clouds_hash (grid.h:43-204) as shipped; result kept for ref_get_clouds.
int ref_build_clouds_hash(int max_node_no, double r, double dx, double dy, double dz, int N,
                          const double* xyz, int* max_len, int64_t* nnz) {
  Eigen::MatrixXd nodes(N, 3);
  for (int i = 0; i < N; ++i) {
    nodes(i, 0) = xyz[i];
    nodes(i, 1) = xyz[N + i];
    nodes(i, 2) = xyz[2 * N + i];
  }
  Eigen::MatrixXi clouds;
  Eigen::VectorXi lengths;
  int ml = 0;
  try {
    build_clouds_hash(max_node_no, r, dx, dy, dz, nodes, clouds, lengths, ml);
  } catch (const std::runtime_error&) {
    return 2;
  }
  g_len.assign(lengths.data(), lengths.data() + N);
  g_ptr.assign(N + 1, 0);
  for (int i = 0; i < N; ++i) g_ptr[i + 1] = g_ptr[i] + g_len[i];
  g_cols.resize(g_ptr[N]);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < g_len[i]; ++j) g_cols[g_ptr[i] + j] = clouds(i, j);
  *max_len = ml;
  *nnz = g_ptr[N];
  return 0;
}

int ref_get_clouds(int* lengths, int64_t* row_ptr, int* cols) {
  std::copy(g_len.begin(), g_len.end(), lengths);
  std::copy(g_ptr.begin(), g_ptr.end(), row_ptr);
  std::copy(g_cols.begin(), g_cols.end(), cols);
  return 0;
}

// utils::Residuals (utils.h:29-842) with U^{n+1} = U^n.  U: 11*N (species 1..10, phi),
// clouds in the reference format (row_ptr/cols, self first), bctypes N, bcvalues 11*N.
// Writes F: 11*N.
int ref_residuals(int N, const double* xyz, const int64_t* row_ptr, const int* cols,
                  const double* U, const int* phase, const int* bctypes, const double* bcvalues,
                  double voln1rel, const double* data2, const double* datac,
                  const double* datac11, double* F) {
  utils::parameter prm;
  make_params(prm, N, data2, datac, datac11);
  Eigen::MatrixXd nodes(N, 3);
  int maxlen = 1;
  for (int i = 0; i < N; ++i) {
    nodes(i, 0) = xyz[i];
    nodes(i, 1) = xyz[N + i];
    nodes(i, 2) = xyz[2 * N + i];
    maxlen = std::max(maxlen, (int)(row_ptr[i + 1] - row_ptr[i]));
  }
  Eigen::MatrixXi hz(N, maxlen);
  hz.setConstant(-1);
  Eigen::VectorXi hl(N), ph(N), bt(N);
  for (int i = 0; i < N; ++i) {
    hl[i] = (int)(row_ptr[i + 1] - row_ptr[i]);
    for (int j = 0; j < hl[i]; ++j) hz(i, j) = cols[row_ptr[i] + j];
    ph[i] = phase[i];
    bt[i] = bctypes[i];
  }
  std::vector<Eigen::VectorXd> bc(11), u(11), u0(11), f(11);
  for (int k = 0; k < 11; ++k) {
    bc[k] = Eigen::Map<const Eigen::VectorXd>(bcvalues + (int64_t)k * N, N);
    u[k] = Eigen::Map<const Eigen::VectorXd>(U + (int64_t)k * N, N);
    u0[k] = Eigen::VectorXd::Zero(N);
    f[k] = Eigen::VectorXd::Zero(N);
  }
  std::vector<Eigen::VectorXd> un1(u);
  utils::Residuals(nodes, hz, bc[0], bc[1], bc[2], bc[3], bc[4], bc[5], bc[6], bc[7], bc[8],
                   bc[9], bc[10], un1[0], un1[1], un1[2], un1[3], un1[4], un1[5], un1[6], un1[7],
                   un1[8], un1[9], un1[10], u[0], u[1], u[2], u[3], u[4], u[5], u[6], u[7], u[8],
                   u[9], u[10], u0[0], u0[1], u0[2], u0[3], u0[4], u0[5], u0[6], u0[7], u0[8],
                   u0[9], u0[10], f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7], f[8], f[9],
                   f[10], ph, hl, bt, voln1rel, prm);
  for (int k = 0; k < 11; ++k) std::memcpy(F + (int64_t)k * N, f[k].data(), sizeof(double) * N);
  return 0;
}

// utils::Residuals (utils.h:29-842) with separate U^{n+1} (Un1) and U^n (Un), each 11*N,
// and the reference's parameter arrays as given (data2 51, datac 10 x 7, datac11 4): the
// complete ten-species residual with its reactions.  Writes F: 11*N.
int ref_residuals2(int N, const double* xyz, const int64_t* row_ptr, const int* cols,
                   const double* Un1, const double* Un, const int* phase, const int* bctypes,
                   const double* bcvalues, double voln1rel, const double* data2, const double* datac,
                   const double* datac11, double* F) {
  utils::parameter prm;
  make_params(prm, N, data2, datac, datac11);
  Eigen::MatrixXd nodes(N, 3);
  int maxlen = 1;
  for (int i = 0; i < N; ++i) {
    nodes(i, 0) = xyz[i];
    nodes(i, 1) = xyz[N + i];
    nodes(i, 2) = xyz[2 * N + i];
    maxlen = std::max(maxlen, (int)(row_ptr[i + 1] - row_ptr[i]));
  }
  Eigen::MatrixXi hz(N, maxlen);
  hz.setConstant(-1);
  Eigen::VectorXi hl(N), ph(N), bt(N);
  for (int i = 0; i < N; ++i) {
    hl[i] = (int)(row_ptr[i + 1] - row_ptr[i]);
    for (int j = 0; j < hl[i]; ++j) hz(i, j) = cols[row_ptr[i] + j];
    ph[i] = phase[i];
    bt[i] = bctypes[i];
  }
  std::vector<Eigen::VectorXd> bc(11), u1(11), u(11), u0(11), f(11);
  for (int k = 0; k < 11; ++k) {
    bc[k] = Eigen::Map<const Eigen::VectorXd>(bcvalues + (int64_t)k * N, N);
    u1[k] = Eigen::Map<const Eigen::VectorXd>(Un1 + (int64_t)k * N, N);
    u[k] = Eigen::Map<const Eigen::VectorXd>(Un + (int64_t)k * N, N);
    u0[k] = Eigen::VectorXd::Zero(N);
    f[k] = Eigen::VectorXd::Zero(N);
  }
  utils::Residuals(nodes, hz, bc[0], bc[1], bc[2], bc[3], bc[4], bc[5], bc[6], bc[7], bc[8],
                   bc[9], bc[10], u1[0], u1[1], u1[2], u1[3], u1[4], u1[5], u1[6], u1[7],
                   u1[8], u1[9], u1[10], u[0], u[1], u[2], u[3], u[4], u[5], u[6], u[7], u[8],
                   u[9], u[10], u0[0], u0[1], u0[2], u0[3], u0[4], u0[5], u0[6], u0[7], u0[8],
                   u0[9], u0[10], f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7], f[8], f[9],
                   f[10], ph, hl, bt, voln1rel, prm);
  for (int k = 0; k < 11; ++k) std::memcpy(F + (int64_t)k * N, f[k].data(), sizeof(double) * N);
  return 0;
}

// All eleven tangents of utils::NewtonMatrices (utils.h:844-1849) at the state U (used as
// both U^{n+1} and U^n), kept for the entry points below.
std::vector<SpMat> g_K;

void newton_matrices(int N, const double* xyz, const int64_t* row_ptr, const int* cols, const double* U,
                     const int* phase, const int* bctypes, const double* bcvalues, double voln1rel,
                     const double* data2, const double* datac, const double* datac11) {
  utils::parameter prm;
  make_params(prm, N, data2, datac, datac11);
  Eigen::MatrixXd nodes(N, 3);
  int maxlen = 1;
  for (int i = 0; i < N; ++i) {
    nodes(i, 0) = xyz[i];
    nodes(i, 1) = xyz[N + i];
    nodes(i, 2) = xyz[2 * N + i];
    maxlen = std::max(maxlen, (int)(row_ptr[i + 1] - row_ptr[i]));
  }
  Eigen::MatrixXi hz(N, maxlen);
  hz.setConstant(-1);
  Eigen::VectorXi hl(N), ph(N), bt(N);
  for (int i = 0; i < N; ++i) {
    hl[i] = (int)(row_ptr[i + 1] - row_ptr[i]);
    for (int j = 0; j < hl[i]; ++j) hz(i, j) = cols[row_ptr[i] + j];
    ph[i] = phase[i];
    bt[i] = bctypes[i];
  }
  std::vector<Eigen::VectorXd> bc(11), u(11);
  for (int k = 0; k < 11; ++k) {
    bc[k] = Eigen::Map<const Eigen::VectorXd>(bcvalues + (int64_t)k * N, N);
    u[k] = Eigen::Map<const Eigen::VectorXd>(U + (int64_t)k * N, N);
  }
  std::vector<Eigen::VectorXd> un1(u);
  g_K.assign(11, SpMat(N, N));
  std::vector<SpMat>& K = g_K;
  utils::NewtonMatrices(K[0], K[1], K[2], K[3], K[4], K[5], K[6], K[7], K[8], K[9], K[10], nodes,
                        hz, bc[0], bc[1], bc[2], bc[3], bc[4], bc[5], bc[6], bc[7], bc[8], bc[9],
                        bc[10], un1[0], un1[1], un1[2], un1[3], un1[4], un1[5], un1[6], un1[7],
                        un1[8], un1[9], un1[10], u[0], u[1], u[2], u[3], u[4], u[5], u[6], u[7],
                        u[8], u[9], u[10], ph, hl, bt, voln1rel, prm);
}

// K_(which+1) of utils::NewtonMatrices (which 0..10; 10 is K11, utils.h:1794-1848) as COO;
// call with ri == NULL for nnz.
int ref_newton_k(int which, int N, const double* xyz, const int64_t* row_ptr, const int* cols,
                 const double* U, const int* phase, const int* bctypes, const double* bcvalues,
                 double voln1rel, const double* data2, const double* datac, const double* datac11,
                 int64_t* nnz, int* ri, int* ci, double* val) {
  if (which < 0 || which > 10) return 1;
  newton_matrices(N, xyz, row_ptr, cols, U, phase, bctypes, bcvalues, voln1rel, data2, datac, datac11);
  const SpMat& A = g_K[which];
  *nnz = A.nonZeros();
  if (!ri) return 0;
  int64_t t = 0;
  for (int col = 0; col < A.outerSize(); ++col)
    for (SpMat::InnerIterator it(A, col); it; ++it) {
      ri[t] = (int)it.row();
      ci[t] = (int)it.col();
      val[t] = it.value();
      ++t;
    }
  return 0;
}

int ref_newton_k11(int N, const double* xyz, const int64_t* row_ptr, const int* cols,
                   const double* U, const int* phase, const int* bctypes, const double* bcvalues,
                   double voln1rel, const double* data2, const double* datac,
                   const double* datac11, int64_t* nnz, int* ri, int* ci, double* val) {
  return ref_newton_k(10, N, xyz, row_ptr, cols, U, phase, bctypes, bcvalues, voln1rel, data2, datac,
                      datac11, nnz, ri, ci, val);
}

// x = GMRES(K_(which+1)) b as main.cpp:714-779 solves the Newton corrections: Eigen::GMRES
// with the diagonal preconditioner, tolerance EPS = 10E-6, MAX_ITER = 200 iterations.
// Returns the iterations.
int ref_gmres(int which, int N, const double* xyz, const int64_t* row_ptr, const int* cols,
              const double* U, const int* phase, const int* bctypes, const double* bcvalues,
              double voln1rel, const double* data2, const double* datac, const double* datac11,
              const double* b, double* x) {
  if (which < 0 || which > 10) return -1;
  newton_matrices(N, xyz, row_ptr, cols, U, phase, bctypes, bcvalues, voln1rel, data2, datac, datac11);
  Eigen::GMRES<SpMat, Eigen::DiagonalPreconditioner<double> > solver(g_K[which]);
  solver.setTolerance(10E-6);
  solver.setMaxIterations(200);
  Eigen::VectorXd bb = Eigen::Map<const Eigen::VectorXd>(b, N);
  Eigen::VectorXd xx = solver.solve(bb);
  for (int i = 0; i < N; ++i) x[i] = xx[i];
  return (int)solver.iterations();
}

// The implant mask's point counts as main.cpp:316-325 computes them: build_clouds(0,
// max_node_no, r, 0, nodes, implant points, ...) of kd_tree_interface.h:156-252 (libkdtree++
// range query, Euclidean filter); the cloud lengths are the counts.  2 where it throws.
int ref_implant_counts(int N, const double* xyz, int M, const double* pts, double r, int max_node_no,
                       int* counts) {
  Eigen::MatrixXd nodes(N, 3), implant(M, 3);
  for (int i = 0; i < N; ++i)
    for (int d = 0; d < 3; ++d) nodes(i, d) = xyz[(int64_t)d * N + i];
  for (int j = 0; j < M; ++j)
    for (int d = 0; d < 3; ++d) implant(j, d) = pts[(int64_t)d * M + j];
  Eigen::MatrixXi clouds;
  Eigen::VectorXi lengths;
  int ml = 0;
  double mean = 0.0;
  try {
    build_clouds(0, max_node_no, r, 0.0, nodes, implant, clouds, lengths, ml, mean);
  } catch (const std::runtime_error&) {
    return 2;
  }
  for (int i = 0; i < N; ++i) counts[i] = lengths[i];
  return 0;
}

}  // extern "C"
