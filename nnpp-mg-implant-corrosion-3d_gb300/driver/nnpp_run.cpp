// nnpp_run -- C++ host driver over the C ABI, in the reference's job-file layout.
//
//   nnpp_run <prefix> <jobname> [<startfileNo>] [--steps N] [--every K]
//            [--precision mixed|fp64] [--k-diss K] [--switch-width W] [--tol T] [--device D]
//            [--no-output] [--restart S0] [--model four|full]
//   nnpp_run --write-synth <kind> <n_side> <seed> <jobname> [--steps N]
//
// Run mode mirrors the reference executable's start-up and time loop (main.cpp:153-1025):
// it reads <jobname>.data1 (4 ints), .data2 (51), .datac1..datac11, .nodes (N rows x y z),
// .bctypes and .bcvalues1..11 / .icvalues1..11 (utils.h:1852-1887 read them as whitespace-
// separated text), builds the neighbourhoods with the reference's call convention
// (r = delta (1 + 1e-5), hash cells 10 dx, 1024 slots: main.cpp:304-305), and advances
// data1[1] explicit steps.  Every K steps (default sub_step_no = 8, main.cpp:39,935) it
// appends voln1rel to <jobname><prefix>.volume and the energy sum of U1^2 dV to .energy, and
// writes <jobname><prefix>-<s>.output.csv with the reference's 15 columns (utils.h:2054-2100,
// 16 significant digits).  The default model transports species 1-4 and the potential;
// columns 5-10 hold the initial values of those species (read from .icvalues5..10 when
// present).  --model full advances all eleven fields (run_full below).
//
// The initial phase is read from <jobname>.phase0 (N ints) when that file exists; otherwise
// a node is solid when icvalues1 > 10E-6 (main.cpp:413-421, BunnyConditions = 0).  When
// data1[3] > 0 and <jobname>.bunnyNodes holds that many points, the implant comes from that
// point cloud instead (BunnyConditions = 1, main.cpp:316-325, 422-457; nnpp_implant_mask).
//
// Restart (main.cpp:507-542): with a start file number s0 (the reference's third argument,
// or --restart s0) the state is read by column name from <jobname><prefix>-<s0>.output.csv
// and the run continues from step s0.
//
// Text input, the output CSV and the restart file are parsed and formatted by all host
// threads (at millions of nodes the reference's serial streams dominate the run's I/O).
//
// --model full runs the reference's complete model instead (ten species and the potential)
// with its own implicit time loop (run_full below).
//
// --write-synth writes one of the library's seeded synthetic workloads in that layout (plus
// .phase0, since those workloads hold Mg in the electrolyte too).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "nnpp_gb300.h"

namespace {

constexpr int kMaxHorizon = 1024;  // MAX_HORIZON_LENGTH, main.cpp:34
constexpr int kSpecies = 4;
constexpr int kFields = 11;

bool slurp(const std::string& path, std::string& out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out.resize(n > 0 ? (size_t)n : 0);
  const size_t got = n > 0 ? std::fread(&out[0], 1, (size_t)n, f) : 0;
  std::fclose(f);
  return got == out.size();
}

// Host threads of the parallel text passes.
int host_threads() {
  const unsigned n = std::thread::hardware_concurrency();
  return n == 0 ? 1 : (int)std::min(n, 64u);
}

// Run f(t) for t in [0, n) on n threads.
template <class F>
void parallel(int n, F f) {
  std::vector<std::thread> th;
  for (int t = 1; t < n; ++t) th.emplace_back(f, t);
  f(0);
  for (auto& x : th) x.join();
}

bool is_space(char c) { return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// Whitespace-separated numbers, the first `count` of them (operator>> semantics of
// read_vector_from_file / read_matrix_from_file, utils.h:1852-1887).  Returns false when
// the file is missing or holds fewer numbers.  The buffer is cut at whitespace into one
// piece per thread; each piece's tokens are counted, then parsed with strtod into their
// places, so the values are those of a serial pass.
bool read_doubles(const std::string& path, size_t count, std::vector<double>& v) {
  std::string buf;
  if (!slurp(path, buf)) return false;
  v.resize(count);
  const size_t L = buf.size();
  const int T = L < (1u << 20) ? 1 : host_threads();
  std::vector<size_t> cut(T + 1, L);
  cut[0] = 0;
  for (int t = 1; t < T; ++t) {
    size_t c = std::max(cut[t - 1], L * t / T);
    while (c < L && !is_space(buf[c])) ++c;
    cut[t] = c;
  }
  std::vector<size_t> ntok(T, 0);
  parallel(T, [&](int t) {
    size_t n = 0;
    bool in = false;
    for (size_t i = cut[t]; i < cut[t + 1]; ++i) {
      const bool sp = is_space(buf[i]);
      if (!sp && !in) ++n;
      in = !sp;
    }
    ntok[t] = n;
  });
  std::vector<size_t> first(T + 1, 0);
  for (int t = 0; t < T; ++t) first[t + 1] = first[t] + ntok[t];
  if (first[T] < count) return false;
  std::vector<char> bad(T, 0);
  parallel(T, [&](int t) {
    const char* p = buf.c_str() + cut[t];
    const char* e = buf.c_str() + cut[t + 1];
    for (size_t k = first[t]; k < first[t + 1] && k < count; ++k) {
      while (p < e && is_space(*p)) ++p;
      char* end = nullptr;
      const double x = std::strtod(p, &end);
      if (end == p) {
        bad[t] = 1;
        return;
      }
      v[k] = x;
      p = end;
    }
  });
  for (int t = 0; t < T; ++t)
    if (bad[t]) return false;
  return true;
}

bool read_ints(const std::string& path, size_t count, std::vector<int>& v) {
  std::vector<double> d;
  if (!read_doubles(path, count, d)) return false;
  v.resize(count);
  for (size_t i = 0; i < count; ++i) v[i] = (int)d[i];
  return true;
}

struct Out {
  FILE* f = nullptr;
  std::vector<char> buf;
  explicit Out(const std::string& path, const char* mode = "wb") {
    f = std::fopen(path.c_str(), mode);
    if (f) {
      buf.resize(1 << 22);
      std::setvbuf(f, buf.data(), _IOFBF, buf.size());
    }
  }
  ~Out() {
    if (f) std::fclose(f);
  }
  bool ok() const { return f != nullptr; }
};

// %.16g is the text the reference's streams write with precision(16) (default float field);
// input files written here use %.17g, which reads back to the same double.
void put(FILE* f, double x) { std::fprintf(f, "%.16g", x); }
void put_exact(FILE* f, double x) { std::fprintf(f, "%.17g", x); }

// The 15-column output CSV of main.cpp:935-999 (utils.h:2054-2100) with its rows formatted
// by all host threads into per-thread buffers, written in order.
bool write_output_csv(const std::string& path, size_t N, const std::vector<double>& rows,
                      const std::vector<double>& c, const std::vector<double>& passive,
                      const std::vector<double>& phi, const std::vector<int>& phase, int species) {
  const int T = N < 4096 ? 1 : host_threads();
  std::vector<std::string> out(T);
  parallel(T, [&](int t) {
    const size_t i0 = N * t / T, i1 = N * (t + 1) / T;
    std::string& o = out[t];
    o.reserve((i1 - i0) * 300);
    char tmp[40];
    for (size_t i = i0; i < i1; ++i) {
      for (int d = 0; d < 3; ++d) o.append(tmp, std::snprintf(tmp, sizeof tmp, "%.16g,", rows[3 * i + d]));
      for (int k = 0; k < species; ++k) o.append(tmp, std::snprintf(tmp, sizeof tmp, "%.16g,", c[(size_t)k * N + i]));
      for (int k = 0; k < 6; ++k) o.append(tmp, std::snprintf(tmp, sizeof tmp, "%.16g,", passive[(size_t)k * N + i]));
      o.append(tmp, std::snprintf(tmp, sizeof tmp, "%.16g,%d\n", phi[i], phase[i]));
    }
  });
  Out f(path);
  if (!f.ok()) return false;
  std::fputs("X,Y,Z,Mg++,H+,OH-,HCO3-,CO32-,HPO42-,PO43-,Ca++,Na+,Cl-,Phi,Phase\n", f.f);
  for (const std::string& o : out) std::fwrite(o.data(), 1, o.size(), f.f);
  return true;
}

// Restart file (utils.h:1929-2027, read_vector_from_startfile as main.cpp:507-542 calls it):
// the header names the columns (a repeated name keeps its last position); every named column
// that is present fills its vector row by row (std::stod / std::stoi), rows beyond num_nodes
// are ignored and missing ones stay zero.  Lines are parsed by all host threads.
bool read_start_csv(const std::string& path, size_t N, const std::vector<std::string>& names,
                    std::vector<std::vector<double> >& cols, std::vector<int>& phase) {
  std::string buf;
  if (!slurp(path, buf)) return false;
  std::vector<size_t> line;  // starts of the data lines
  size_t e = buf.find('\n');
  const std::string header = buf.substr(0, e == std::string::npos ? buf.size() : e);
  std::map<std::string, size_t> pos;
  {
    size_t i = 0, k = 0;
    while (i <= header.size()) {
      size_t j = header.find(',', i);
      if (j == std::string::npos) j = header.size();
      pos[header.substr(i, j - i)] = k++;
      i = j + 1;
    }
  }
  for (size_t p = e == std::string::npos ? buf.size() : e + 1; p < buf.size() && line.size() < N;) {
    line.push_back(p);
    const size_t q = buf.find('\n', p);
    p = q == std::string::npos ? buf.size() : q + 1;
  }
  std::vector<long> want(names.size() + 1, -1);  // column of each name, phase last
  for (size_t n = 0; n < names.size(); ++n) {
    auto it = pos.find(names[n]);
    if (it != pos.end()) want[n] = (long)it->second;
  }
  {
    auto it = pos.find("Phase");
    if (it != pos.end()) want[names.size()] = (long)it->second;
  }
  cols.assign(names.size(), std::vector<double>(N, 0.0));
  phase.assign(N, 0);
  const int T = line.size() < 4096 ? 1 : host_threads();
  parallel(T, [&](int t) {
    std::vector<const char*> field;
    for (size_t r = line.size() * t / T; r < line.size() * (t + 1) / T; ++r) {
      const char* p = buf.c_str() + line[r];
      const char* end = buf.c_str() + (r + 1 < line.size() ? line[r + 1] : buf.size());
      field.clear();
      field.push_back(p);
      for (const char* q = p; q < end && *q != '\n'; ++q)
        if (*q == ',') field.push_back(q + 1);
      for (size_t n = 0; n <= names.size(); ++n) {
        if (want[n] < 0 || (size_t)want[n] >= field.size()) continue;
        if (n < names.size())
          cols[n][r] = std::strtod(field[want[n]], nullptr);
        else
          phase[r] = (int)std::strtol(field[want[n]], nullptr, 10);
      }
    }
  });
  return true;
}

int fail_status(const char* what, nnpp_status st) {
  std::fprintf(stderr, "nnpp_run: %s failed (status %d): %s\n", what, (int)st, nnpp_last_error());
  return 2;
}

#define CALL(what, expr)                          \
  do {                                            \
    const nnpp_status st_ = (expr);               \
    if (st_ != NNPP_OK) return fail_status(what, st_); \
  } while (0)

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------- --write-synth ---------
int write_synth(int kind, int n_side, uint64_t seed, const std::string& job, int steps) {
  const int64_t N64 = nnpp_synth_count(kind, n_side);
  if (N64 <= 0) {
    std::fprintf(stderr, "nnpp_run: bad synthetic kind/n_side\n");
    return 1;
  }
  const size_t N = (size_t)N64;
  std::vector<double> xyz(3 * N), bcv((kSpecies + 1) * N), ic((kSpecies + 1) * N);
  std::vector<int> bct(N), ph(N);
  nnpp_params p;
  CALL("nnpp_synth_fill", nnpp_synth_fill(kind, n_side, seed, xyz.data(), bct.data(), bcv.data(),
                                          ic.data(), ph.data(), &p));
  int bc_nodes = 0;
  for (size_t i = 0; i < N; ++i) bc_nodes += bct[i] == 0 ? 1 : 0;
  {
    Out o(job + ".data1");
    if (!o.ok()) return 1;
    std::fprintf(o.f, "%zu\n%d\n%d\n0\n", N, steps, bc_nodes);
  }
  {
    // utils.h:2348-2398: t0, t1, dt, dx, dy, dz, delta, CSolid, CSat, 38 chemistry
    // constants (zero: out of the modelled path), T, R, F, vol_red
    double d2[51] = {0};
    d2[0] = 0.0;
    d2[1] = steps * p.dt;
    d2[2] = p.dt;
    d2[3] = p.dx;
    d2[4] = p.dy;
    d2[5] = p.dz;
    d2[6] = p.delta;
    d2[7] = p.CSolid;
    d2[8] = p.CSat;
    d2[47] = p.T;
    d2[48] = p.R;
    d2[49] = p.F;
    d2[50] = p.vol_red;
    Out o(job + ".data2");
    for (double x : d2) put_exact(o.f, x), std::fputc('\n', o.f);
  }
  for (int c = 1; c <= 10; ++c) {
    Out o(job + ".datac" + std::to_string(c));
    double row[7] = {0, 0, 0, 0, 0, 0, 0};
    if (c <= kSpecies) {
      const int s = c - 1;
      const double r[7] = {p.z[s], p.D_solid[s], p.D_liquid[s], p.s1[s], p.s2[s], p.K1[s], p.K2[s]};
      std::memcpy(row, r, sizeof(row));
    } else {
      row[3] = row[4] = p.s_phi;
    }
    for (double x : row) put_exact(o.f, x), std::fputc('\n', o.f);
  }
  {
    Out o(job + ".datac11");
    const double r[4] = {p.sigma, p.sigma, p.s_phi, p.K_phi};
    for (double x : r) put_exact(o.f, x), std::fputc('\n', o.f);
  }
  {
    Out o(job + ".nodes");
    for (size_t i = 0; i < N; ++i) {
      put_exact(o.f, xyz[i]);
      std::fputc(' ', o.f);
      put_exact(o.f, xyz[N + i]);
      std::fputc(' ', o.f);
      put_exact(o.f, xyz[2 * N + i]);
      std::fputc('\n', o.f);
    }
  }
  {
    Out o(job + ".bctypes");
    for (size_t i = 0; i < N; ++i) std::fprintf(o.f, "%d\n", bct[i]);
  }
  {
    Out o(job + ".phase0");
    for (size_t i = 0; i < N; ++i) std::fprintf(o.f, "%d\n", ph[i]);
  }
  for (int f = 1; f <= kFields; ++f) {
    // fields 1-4: species, 11: potential; 5-10 free (-1) with zero initial values
    const int src = f <= kSpecies ? f - 1 : (f == kFields ? kSpecies : -1);
    Out ob(job + ".bcvalues" + std::to_string(f));
    Out oi(job + ".icvalues" + std::to_string(f));
    for (size_t i = 0; i < N; ++i) {
      put_exact(ob.f, src >= 0 ? bcv[(size_t)src * N + i] : -1.0);
      std::fputc('\n', ob.f);
      put_exact(oi.f, src >= 0 ? ic[(size_t)src * N + i] : 0.0);
      std::fputc('\n', oi.f);
    }
  }
  std::printf("wrote %s.* : %zu nodes, %d Dirichlet-shell nodes, %d steps\n", job.c_str(), N,
              bc_nodes, steps);
  return 0;
}

// ---------------------------------------------------------------- run -------------------
struct Options {
  int steps = -1;
  int every = -1;
  int precision = NNPP_MIXED;
  double k_diss = 0.05;
  double switch_width = 0.0;
  double tol = 1e-10;
  int device = 0;
  bool output = true;
  int restart = -1;  // start file number (main.cpp's third argument), -1: start from t = 0
  bool full = false;  // --model full: the reference's complete model and implicit time loop
};

int run_full(const std::string& prefix, const std::string& job, const Options& opt);

int run(const std::string& prefix, const std::string& job, const Options& opt) {
  if (opt.full) return run_full(prefix, job, opt);
  std::vector<int> d1;
  std::vector<double> d2, dc[11];
  if (!read_ints(job + ".data1", 4, d1)) return std::fprintf(stderr, "nnpp_run: cannot read %s.data1\n", job.c_str()), 1;
  if (!read_doubles(job + ".data2", 51, d2)) return std::fprintf(stderr, "nnpp_run: cannot read %s.data2\n", job.c_str()), 1;
  for (int c = 1; c <= 4; ++c)
    if (!read_doubles(job + ".datac" + std::to_string(c), 7, dc[c - 1]))
      return std::fprintf(stderr, "nnpp_run: cannot read %s.datac%d\n", job.c_str(), c), 1;
  if (!read_doubles(job + ".datac11", 4, dc[10])) return std::fprintf(stderr, "nnpp_run: cannot read %s.datac11\n", job.c_str()), 1;
  const int N = d1[0];
  const int steps = opt.steps >= 0 ? opt.steps : d1[1];
  if (N <= 0) return std::fprintf(stderr, "nnpp_run: data1 holds no nodes\n"), 1;
  nnpp_params p;
  CALL("nnpp_params_from_reference",
       nnpp_params_from_reference(d2.data(), dc[0].data(), dc[1].data(), dc[2].data(), dc[3].data(),
                                  dc[10].data(), opt.k_diss, opt.switch_width, &p));
  const int every = opt.every > 0 ? opt.every : (p.sub_step_no > 0 ? p.sub_step_no : 8);

  std::vector<double> rows, xyz(3 * (size_t)N);
  if (!read_doubles(job + ".nodes", 3 * (size_t)N, rows)) return std::fprintf(stderr, "nnpp_run: cannot read %s.nodes\n", job.c_str()), 1;
  double energy_bound = -INFINITY;  // nodes.maxCoeff(), main.cpp:245
  for (size_t i = 0; i < (size_t)N; ++i)
    for (int d = 0; d < 3; ++d) {
      xyz[(size_t)d * N + i] = rows[3 * i + d];
      energy_bound = std::fmax(energy_bound, rows[3 * i + d]);
    }
  std::vector<int> bct;
  if (!read_ints(job + ".bctypes", N, bct)) return std::fprintf(stderr, "nnpp_run: cannot read %s.bctypes\n", job.c_str()), 1;
  std::vector<double> bcv((kSpecies + 1) * (size_t)N), ic((kSpecies + 1) * (size_t)N), tmp;
  for (int f = 0; f <= kSpecies; ++f) {
    const int file = f < kSpecies ? f + 1 : kFields;
    if (!read_doubles(job + ".bcvalues" + std::to_string(file), N, tmp)) return std::fprintf(stderr, "nnpp_run: cannot read bcvalues%d\n", file), 1;
    std::copy(tmp.begin(), tmp.end(), bcv.begin() + (size_t)f * N);
    if (!read_doubles(job + ".icvalues" + std::to_string(file), N, tmp)) return std::fprintf(stderr, "nnpp_run: cannot read icvalues%d\n", file), 1;
    std::copy(tmp.begin(), tmp.end(), ic.begin() + (size_t)f * N);
  }
  std::vector<double> passive(6 * (size_t)N, 0.0);  // columns 5-10 of the output
  for (int f = 5; f <= 10; ++f)
    if (read_doubles(job + ".icvalues" + std::to_string(f), N, tmp))
      std::copy(tmp.begin(), tmp.end(), passive.begin() + (size_t)(f - 5) * N);

  std::vector<int> phase0;
  bool have_phase = read_ints(job + ".phase0", N, phase0);
  // implant from its point cloud (BunnyConditions = 1, main.cpp:236-240, 316-325, 422-457):
  // data1[3] points in <job>.bunnyNodes; a node within 3 * 0.4 dx (1 + 1e-5) of one is solid
  // (Mg2+ at CSolid / CSolid, the other species 0), the others liquid with the reference's
  // electrolyte (Mg2+ 0, H+ and OH- 1e-4 / CSolid, HCO3- C0HCO3 / CSolid = data2[11] / CSolid),
  // the potential 0
  std::vector<double> bunny;
  if (d1[3] > 0 && read_doubles(job + ".bunnyNodes", 3 * (size_t)d1[3], bunny)) {
    const size_t M = d1[3];
    std::vector<double> pts(3 * M);
    for (size_t j = 0; j < M; ++j)
      for (int d = 0; d < 3; ++d) pts[d * M + j] = bunny[3 * j + d];
    phase0.assign(N, 0);
    const double t0 = now_s();
    CALL("nnpp_implant_mask", nnpp_implant_mask(N, xyz.data(), (int)M, pts.data(), 3. * 0.4 * p.dx * (1.00 + 1e-5),
                                               kMaxHorizon, nullptr, phase0.data()));
    long long solid = 0;
    const double liquid[kSpecies] = {0.0, 1e-4 / p.CSolid, 1e-4 / p.CSolid, d2[11] / p.CSolid};
    for (size_t i = 0; i < (size_t)N; ++i) {
      solid += phase0[i];
      for (int k = 0; k < kSpecies; ++k)
        ic[(size_t)k * N + i] = phase0[i] ? (k == 0 ? p.CSolid / p.CSolid : 0.0) : liquid[k];
      ic[(size_t)kSpecies * N + i] = 0.0;
    }
    have_phase = true;
    std::printf("Building bunnyNodes took %g seconds (%zu implant points, %lld solid nodes)\n", now_s() - t0, M,
                solid);
  }

  CALL("nnpp_set_device", nnpp_set_device(opt.device));
  nnpp_handle* h = nullptr;
  CALL("nnpp_create", nnpp_create(&h, &p, N, xyz.data(), bct.data(), bcv.data(), ic.data(),
                                  have_phase ? phase0.data() : nullptr));
  int max_len = 0;
  double t0 = now_s();
  CALL("nnpp_build_neighbours",
       nnpp_build_neighbours(h, kMaxHorizon, p.delta * (1.00 + 1e-5), p.dx * 10., p.dy * 10., p.dz * 10.,
                             NNPP_ORDER_REFERENCE, nullptr, nullptr, &max_len));
  std::printf("Building horizons took %g seconds. Max. horizon length: %d\n", now_s() - t0, max_len);
  std::printf("%d nodes; horizon radius: %.16g\n", N, p.delta);
  CALL("nnpp_set_solver", nnpp_set_solver(h, opt.tol, 2000, 0));
  int s = 0;
  if (opt.restart >= 0) {
    // main.cpp:507-542: the state of <job><prefix>-<s0>.output.csv, read by column name
    const std::string path = job + prefix + "-" + std::to_string(opt.restart) + ".output.csv";
    const std::vector<std::string> names = {"Mg++", "H+", "OH-", "HCO3-", "CO32-", "HPO42-",
                                            "PO43-", "Ca++", "Na+", "Cl-", "Phi"};
    std::vector<std::vector<double> > cols;
    std::vector<int> ph;
    const double tr = now_s();
    if (!read_start_csv(path, N, names, cols, ph)) return std::fprintf(stderr, "No start file found!\n"), 1;
    std::vector<double> c0((size_t)kSpecies * N);
    for (int k = 0; k < kSpecies; ++k) std::copy(cols[k].begin(), cols[k].end(), c0.begin() + (size_t)k * N);
    for (int k = 0; k < 6; ++k) std::copy(cols[4 + k].begin(), cols[4 + k].end(), passive.begin() + (size_t)k * N);
    CALL("nnpp_set_state", nnpp_set_state(h, c0.data(), cols[10].data(), ph.data()));
    s = opt.restart;
    std::printf("Restart from %s (%.3f s)\n", path.c_str(), now_s() - tr);
  }

  const double dV = p.dx * p.dy * p.dz;
  std::vector<double> c((size_t)kSpecies * N), phi(N);
  std::vector<int> phase(N);
  if (opt.output) {
    Out v(job + prefix + ".volume");  // truncate the append-only files of a previous run
    Out e(job + prefix + ".energy");
  }
  std::printf("Time Marching started:\n");
  t0 = now_s();
  while (s < steps) {
    const int n = std::min(every - s % every, steps - s);
    CALL("nnpp_forward", nnpp_forward(h, n, opt.precision));
    s += n;
    if (s % every != 0 && s != steps) continue;
    nnpp_diag dg;
    CALL("nnpp_get_diagnostics", nnpp_get_diagnostics(h, &dg));
    std::printf("step %d  t: %.6g  solid nodes: %lld  Volume rel: %.16g  Mg lost: %.6g  (%.3f ms/step)\n", s,
                s * p.dt, (long long)dg.solid_count, dg.voln1rel, dg.mg_mass_lost,
                1e3 * (now_s() - t0) / n);
    t0 = now_s();
    if (!opt.output) continue;
    CALL("nnpp_get_state", nnpp_get_state(h, c.data(), phi.data(), phase.data()));
    {
      Out v(job + prefix + ".volume", "ab");
      put(v.f, dg.voln1rel);
      std::fputs(",\n", v.f);
    }
    double energy = 0.0;  // main.cpp:962-969
    for (size_t i = 0; i < (size_t)N; ++i)
      if (std::fabs(rows[3 * i]) < energy_bound || std::fabs(rows[3 * i + 1]) < energy_bound)
        energy += c[i] * c[i] * dV;
    {
      Out e(job + prefix + ".energy", "ab");
      put(e.f, energy);
      std::fputc('\n', e.f);
    }
    if (!write_output_csv(job + prefix + "-" + std::to_string(s) + ".output.csv", N, rows, c, passive, phi, phase,
                          kSpecies))
      return std::fprintf(stderr, "nnpp_run: cannot write output\n"), 1;
  }
  nnpp_destroy(h);
  return 0;
}

// --model full: the reference's complete model (ten species and the potential) with its own
// time integration (main.cpp:640-922, backward Euler with Newton/GMRES: nnpp_chem_*), from the
// same job files (all of .datac1..10, .bcvalues1..11, .icvalues1..11); the phase from .phase0
// or icvalues1 > 10E-6 (main.cpp:413-421); the relative volume 0 until the first update
// (main.cpp:474-475), vol0rel from the initial state; restart by column name as above.
int run_full(const std::string& prefix, const std::string& job, const Options& opt) {
  std::vector<int> d1;
  std::vector<double> d2, d11, datac(70), tmp;
  if (!read_ints(job + ".data1", 4, d1)) return std::fprintf(stderr, "nnpp_run: cannot read %s.data1\n", job.c_str()), 1;
  if (!read_doubles(job + ".data2", 51, d2)) return std::fprintf(stderr, "nnpp_run: cannot read %s.data2\n", job.c_str()), 1;
  for (int c = 1; c <= 10; ++c) {
    if (!read_doubles(job + ".datac" + std::to_string(c), 7, tmp))
      return std::fprintf(stderr, "nnpp_run: cannot read %s.datac%d\n", job.c_str(), c), 1;
    std::copy(tmp.begin(), tmp.end(), datac.begin() + 7 * (c - 1));
  }
  if (!read_doubles(job + ".datac11", 4, d11)) return std::fprintf(stderr, "nnpp_run: cannot read %s.datac11\n", job.c_str()), 1;
  if (d1[3] > 0) return std::fprintf(stderr, "nnpp_run: --model full starts from the initial-value files only\n"), 1;
  const int N = d1[0];
  const int steps = opt.steps >= 0 ? opt.steps : d1[1];
  if (N <= 0) return std::fprintf(stderr, "nnpp_run: data1 holds no nodes\n"), 1;
  const int every = opt.every > 0 ? opt.every : 8;
  const double dx = d2[3], dy = d2[4], dz = d2[5], delta = d2[6], CSolid = d2[7], CSat = d2[8];
  std::vector<double> rows, xyz(3 * (size_t)N);
  if (!read_doubles(job + ".nodes", 3 * (size_t)N, rows)) return std::fprintf(stderr, "nnpp_run: cannot read %s.nodes\n", job.c_str()), 1;
  double energy_bound = -INFINITY;  // nodes.maxCoeff(), main.cpp:245
  for (size_t i = 0; i < (size_t)N; ++i)
    for (int d = 0; d < 3; ++d) {
      xyz[(size_t)d * N + i] = rows[3 * i + d];
      energy_bound = std::fmax(energy_bound, rows[3 * i + d]);
    }
  std::vector<int> bct;
  if (!read_ints(job + ".bctypes", N, bct)) return std::fprintf(stderr, "nnpp_run: cannot read %s.bctypes\n", job.c_str()), 1;
  std::vector<double> bcv((size_t)kFields * N), U((size_t)kFields * N);
  for (int f = 1; f <= kFields; ++f) {
    if (!read_doubles(job + ".bcvalues" + std::to_string(f), N, tmp)) return std::fprintf(stderr, "nnpp_run: cannot read bcvalues%d\n", f), 1;
    std::copy(tmp.begin(), tmp.end(), bcv.begin() + (size_t)(f - 1) * N);
    if (!read_doubles(job + ".icvalues" + std::to_string(f), N, tmp)) return std::fprintf(stderr, "nnpp_run: cannot read icvalues%d\n", f), 1;
    std::copy(tmp.begin(), tmp.end(), U.begin() + (size_t)(f - 1) * N);
  }
  std::vector<int> phase;
  if (!read_ints(job + ".phase0", N, phase)) {
    phase.assign(N, 0);
    for (int i = 0; i < N; ++i) phase[i] = U[i] > 0.0 + 10E-6 ? 1 : 0;
  }
  CALL("nnpp_set_device", nnpp_set_device(opt.device));
  // the reference's neighbourhoods (main.cpp:304-305), compacted to the longest horizon
  std::vector<int> clouds((size_t)N * kMaxHorizon), lengths(N);
  int ml = 0;
  double t0 = now_s();
  CALL("nnpp_build_clouds_hash",
       nnpp_build_clouds_hash(kMaxHorizon, delta * (1.00 + 1e-5), dx * 10., dy * 10., dz * 10., N, xyz.data(),
                              NNPP_ORDER_REFERENCE, clouds.data(), lengths.data(), &ml));
  clouds.resize((size_t)N * ml);
  std::printf("Building horizons took %g seconds. Max. horizon length: %d\n", now_s() - t0, ml);
  nnpp_chem* ch = nullptr;
  CALL("nnpp_chem_create", nnpp_chem_create(&ch, N, xyz.data(), clouds.data(), ml, lengths.data(), bct.data(),
                                            bcv.data(), d2.data(), datac.data(), d11.data()));
  const double csat = CSat / CSolid;
  double vol0rel = 0.0;  // main.cpp:474-480, from the initial state
  for (int i = 0; i < N; ++i)
    if (phase[i] == 1) vol0rel += U[i] - csat;
  double voln1rel = 0.0;
  int s = 0;
  if (opt.restart >= 0) {
    const std::string path = job + prefix + "-" + std::to_string(opt.restart) + ".output.csv";
    const std::vector<std::string> names = {"Mg++", "H+", "OH-", "HCO3-", "CO32-", "HPO42-",
                                            "PO43-", "Ca++", "Na+", "Cl-", "Phi"};
    std::vector<std::vector<double> > cols;
    if (!read_start_csv(path, N, names, cols, phase)) return std::fprintf(stderr, "No start file found!\n"), 1;
    for (int f = 0; f < kFields; ++f) std::copy(cols[f].begin(), cols[f].end(), U.begin() + (size_t)f * N);
    voln1rel = 0.0;  // main.cpp:530-536
    for (int i = 0; i < N; ++i)
      if (phase[i] == 1) voln1rel += U[i] - csat;
    voln1rel /= vol0rel;
    s = opt.restart;
    std::printf("Restart from %s\n", path.c_str());
  }
  CALL("nnpp_chem_set_state", nnpp_chem_set_state(ch, U.data(), phase.data(), voln1rel, vol0rel));
  const double dV = dx * dy * dz;
  std::vector<double> c((size_t)kSpecies * N), passive(6 * (size_t)N), phi(N);
  if (opt.output) {
    Out v(job + prefix + ".volume");
    Out e(job + prefix + ".energy");
  }
  std::printf("Time Marching started (complete model, implicit):\n");
  t0 = now_s();
  while (s < steps) {
    const int n = std::min(every - s % every, steps - s);
    int64_t newton = 0, krylov = 0;
    CALL("nnpp_chem_step", nnpp_chem_step(ch, n, &newton, &krylov));
    s += n;
    if (s % every != 0 && s != steps) continue;
    CALL("nnpp_chem_get_state", nnpp_chem_get_state(ch, U.data(), phase.data(), &voln1rel));
    long long solid = 0;
    for (int i = 0; i < N; ++i) solid += phase[i];
    std::printf("step %d  t: %.6g  solid nodes: %lld  Volume rel: %.16g  Newton: %lld  GMRES: %lld  (%.3f ms/step)\n",
                s, s * d2[2], solid, voln1rel, (long long)newton, (long long)krylov, 1e3 * (now_s() - t0) / n);
    t0 = now_s();
    if (!opt.output) continue;
    {
      Out v(job + prefix + ".volume", "ab");
      put(v.f, voln1rel);
      std::fputs(",\n", v.f);
    }
    double energy = 0.0;  // main.cpp:962-969
    for (size_t i = 0; i < (size_t)N; ++i)
      if (std::fabs(rows[3 * i]) < energy_bound || std::fabs(rows[3 * i + 1]) < energy_bound)
        energy += U[i] * U[i] * dV;
    {
      Out e(job + prefix + ".energy", "ab");
      put(e.f, energy);
      std::fputc('\n', e.f);
    }
    std::copy(U.begin(), U.begin() + (size_t)kSpecies * N, c.begin());
    std::copy(U.begin() + (size_t)kSpecies * N, U.begin() + (size_t)10 * N, passive.begin());
    std::copy(U.begin() + (size_t)10 * N, U.end(), phi.begin());
    if (!write_output_csv(job + prefix + "-" + std::to_string(s) + ".output.csv", N, rows, c, passive, phi, phase,
                          kSpecies))
      return std::fprintf(stderr, "nnpp_run: cannot write output\n"), 1;
  }
  nnpp_chem_destroy(ch);
  return 0;
}

int usage() {
  std::fprintf(stderr,
               "usage: nnpp_run <prefix> <jobname> [<startfileNo>] [--steps N] [--every K]\n"
               "                [--precision mixed|fp64] [--k-diss K] [--switch-width W] [--tol T]\n"
               "                [--device D] [--no-output] [--restart S0] [--model four|full]\n"
               "       nnpp_run --write-synth <kind> <n_side> <seed> <jobname> [--steps N]\n");
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc >= 6 && std::strcmp(argv[1], "--write-synth") == 0) {
    int steps = 1000;
    for (int i = 6; i + 1 < argc; i += 2)
      if (std::strcmp(argv[i], "--steps") == 0) steps = std::atoi(argv[i + 1]);
    return write_synth(std::atoi(argv[2]), std::atoi(argv[3]), std::strtoull(argv[4], nullptr, 10),
                       argv[5], steps);
  }
  if (argc < 3) return usage();
  Options opt;
  for (int i = 3; i < argc; ++i) {
    const std::string a = argv[i];
    const bool has = i + 1 < argc;
    if (a == "--no-output") opt.output = false;
    else if (a == "--steps" && has) opt.steps = std::atoi(argv[++i]);
    else if (a == "--every" && has) opt.every = std::atoi(argv[++i]);
    else if (a == "--k-diss" && has) opt.k_diss = std::atof(argv[++i]);
    else if (a == "--switch-width" && has) opt.switch_width = std::atof(argv[++i]);
    else if (a == "--tol" && has) opt.tol = std::atof(argv[++i]);
    else if (a == "--device" && has) opt.device = std::atoi(argv[++i]);
    else if (a == "--restart" && has) opt.restart = std::atoi(argv[++i]);
    else if (a == "--model" && has) {
      const std::string v = argv[++i];
      if (v == "full") opt.full = true;
      else if (v != "four") return usage();
    }
    else if (i == 3 && a.size() && a[0] != '-') opt.restart = std::atoi(argv[i]);  // main.cpp's 3rd argument
    else if (a == "--precision" && has) {
      const std::string v = argv[++i];
      if (v == "fp64") opt.precision = NNPP_FP64;
      else if (v == "mixed") opt.precision = NNPP_MIXED;
      else return usage();
    } else return usage();
  }
  return run(argv[1], argv[2], opt);
}
