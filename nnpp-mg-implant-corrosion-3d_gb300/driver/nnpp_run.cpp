// nnpp_run -- C++ host driver over the C ABI, in the reference's job-file layout.
//
//   nnpp_run <prefix> <jobname> [--steps N] [--every K] [--precision mixed|fp64]
//            [--k-diss K] [--switch-width W] [--tol T] [--device D] [--no-output]
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
// 16 significant digits).  The model transports species 1-4 and the potential; columns 5-10
// hold the initial values of those species (read from .icvalues5..10 when present).
//
// The initial phase is read from <jobname>.phase0 (N ints) when that file exists; otherwise
// a node is solid when icvalues1 > 10E-6 (main.cpp:413-421, BunnyConditions = 0).
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
#include <string>
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

// Whitespace-separated numbers, the first `count` of them (operator>> semantics of
// read_vector_from_file / read_matrix_from_file).  Returns false when the file is missing
// or holds fewer numbers.
bool read_doubles(const std::string& path, size_t count, std::vector<double>& v) {
  std::string buf;
  if (!slurp(path, buf)) return false;
  v.resize(count);
  const char* p = buf.c_str();
  for (size_t i = 0; i < count; ++i) {
    char* end = nullptr;
    const double x = std::strtod(p, &end);
    if (end == p) return false;
    v[i] = x;
    p = end;
  }
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
};

int run(const std::string& prefix, const std::string& job, const Options& opt) {
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
  const bool have_phase = read_ints(job + ".phase0", N, phase0);

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

  const double dV = p.dx * p.dy * p.dz;
  std::vector<double> c((size_t)kSpecies * N), phi(N);
  std::vector<int> phase(N);
  if (opt.output) {
    Out v(job + prefix + ".volume");  // truncate the append-only files of a previous run
    Out e(job + prefix + ".energy");
  }
  std::printf("Time Marching started:\n");
  int s = 0;
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
    Out o(job + prefix + "-" + std::to_string(s) + ".output.csv");
    if (!o.ok()) return std::fprintf(stderr, "nnpp_run: cannot write output\n"), 1;
    std::fputs("X,Y,Z,Mg++,H+,OH-,HCO3-,CO32-,HPO42-,PO43-,Ca++,Na+,Cl-,Phi,Phase\n", o.f);
    for (size_t i = 0; i < (size_t)N; ++i) {
      for (int d = 0; d < 3; ++d) put(o.f, rows[3 * i + d]), std::fputc(',', o.f);
      for (int k = 0; k < kSpecies; ++k) put(o.f, c[(size_t)k * N + i]), std::fputc(',', o.f);
      for (int k = 0; k < 6; ++k) put(o.f, passive[(size_t)k * N + i]), std::fputc(',', o.f);
      put(o.f, phi[i]);
      std::fprintf(o.f, ",%d\n", phase[i]);
    }
  }
  nnpp_destroy(h);
  return 0;
}

int usage() {
  std::fprintf(stderr,
               "usage: nnpp_run <prefix> <jobname> [--steps N] [--every K] [--precision mixed|fp64]\n"
               "                [--k-diss K] [--switch-width W] [--tol T] [--device D] [--no-output]\n"
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
    else if (a == "--precision" && has) {
      const std::string v = argv[++i];
      if (v == "fp64") opt.precision = NNPP_FP64;
      else if (v == "mixed") opt.precision = NNPP_MIXED;
      else return usage();
    } else return usage();
  }
  return run(argv[1], argv[2], opt);
}
