// synth.cpp -- deterministic synthetic workloads in the reference's input layout.
//
// The reference reads its geometry, boundary and initial values from text files
// (main.cpp:234-289, utils.h:1852-1887); the paper's files are not available, so every
// workload here is generated from a seed.  The generator uses only IEEE +, -, *, / and
// sqrt (compiled with -ffp-contract=off) and its own sine/cosine, so the same seed gives
// bit-identical node coordinates on x86-64 and aarch64 hosts.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "nnpp_gb300.h"
#include "nnpp_internal.h"

namespace {

struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() {  // splitmix64
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double u01() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double uni(double a, double b) { return a + (b - a) * u01(); }
};

const double kPi = 3.14159265358979323846;

// sin and cos of a in [-pi, pi] from their Taylor series (terms to x^27), no libm.
void sincos_series(double a, double* s, double* c) {
  double a2 = a * a;
  double ts = a, tc = 1.0, ss = a, cc = 1.0;
  for (int k = 1; k <= 13; ++k) {
    ts = -ts * a2 / (double)((2 * k) * (2 * k + 1));
    tc = -tc * a2 / (double)((2 * k - 1) * (2 * k));
    ss += ts;
    cc += tc;
  }
  *s = ss;
  *c = cc;
}

// Real spherical harmonics of degree 1..4 in Cartesian form on the unit vector (x,y,z),
// with the usual orthonormalisation constants.  Index 0..23.
double real_sh(int idx, double x, double y, double z) {
  const double c1 = std::sqrt(3.0 / (4.0 * kPi));
  const double c2a = 0.5 * std::sqrt(15.0 / kPi), c2b = 0.25 * std::sqrt(5.0 / kPi),
               c2c = 0.25 * std::sqrt(15.0 / kPi);
  const double c3a = 0.25 * std::sqrt(35.0 / (2.0 * kPi)), c3b = 0.5 * std::sqrt(105.0 / kPi),
               c3c = 0.25 * std::sqrt(21.0 / (2.0 * kPi)), c3d = 0.25 * std::sqrt(7.0 / kPi),
               c3e = 0.25 * std::sqrt(105.0 / kPi);
  const double c4a = 0.75 * std::sqrt(35.0 / kPi), c4b = 0.75 * std::sqrt(35.0 / (2.0 * kPi)),
               c4c = 0.75 * std::sqrt(5.0 / kPi), c4d = 0.75 * std::sqrt(5.0 / (2.0 * kPi)),
               c4e = (3.0 / 16.0) * std::sqrt(1.0 / kPi), c4f = (3.0 / 8.0) * std::sqrt(5.0 / kPi),
               c4g = (3.0 / 16.0) * std::sqrt(35.0 / kPi);
  double x2 = x * x, y2 = y * y, z2 = z * z;
  switch (idx) {
    case 0: return c1 * y;
    case 1: return c1 * z;
    case 2: return c1 * x;
    case 3: return c2a * x * y;
    case 4: return c2a * y * z;
    case 5: return c2b * (3.0 * z2 - 1.0);
    case 6: return c2a * x * z;
    case 7: return c2c * (x2 - y2);
    case 8: return c3a * y * (3.0 * x2 - y2);
    case 9: return c3b * x * y * z;
    case 10: return c3c * y * (5.0 * z2 - 1.0);
    case 11: return c3d * z * (5.0 * z2 - 3.0);
    case 12: return c3c * x * (5.0 * z2 - 1.0);
    case 13: return c3e * z * (x2 - y2);
    case 14: return c3a * x * (x2 - 3.0 * y2);
    case 15: return c4a * x * y * (x2 - y2);
    case 16: return c4b * y * z * (3.0 * x2 - y2);
    case 17: return c4c * x * y * (7.0 * z2 - 1.0);
    case 18: return c4d * y * z * (7.0 * z2 - 3.0);
    case 19: return c4e * (35.0 * z2 * z2 - 30.0 * z2 + 3.0);
    case 20: return c4d * x * z * (7.0 * z2 - 3.0);
    case 21: return c4f * (x2 - y2) * (7.0 * z2 - 1.0);
    case 22: return c4b * x * z * (x2 - 3.0 * y2);
    default: return c4g * (x2 * (x2 - 3.0 * y2) - y2 * (3.0 * x2 - y2));
  }
}

bool in_shell(int ix, int iy, int iz, int n, int width) {
  int m = ix;
  if (iy < m) m = iy;
  if (iz < m) m = iz;
  if (n - 1 - ix < m) m = n - 1 - ix;
  if (n - 1 - iy < m) m = n - 1 - iy;
  if (n - 1 - iz < m) m = n - 1 - iz;
  return m < width;
}

}  // namespace

namespace nnpp {

// Model parameters of the synthetic workloads: four species with charges (+2,-1,-1,+1)
// and liquid diffusivities (0.7, 2.0, 5.3, 1.3)e-3, solid diffusivities 1e-3 times the
// liquid ones (the ratio of the reference's datac2..datac4), kernel exponents s = 0,
// K_prop1 = K11prop1 = 3/(pi delta^2), K_prop2 = 1/(pi delta^2) (the constants of
// data/NNPP.datac1..11 for delta), CSat/CSolid = 0.035 (data/NNPP.data2: 2312.884/66082.4),
// F = R = T = 1 (potential in units of RT/F), sigma = 0.01, dt = 0.2 dx^2 / max(D).
void synth_default_params(int n_side, nnpp_params* p) {
  std::memset(p, 0, sizeof(*p));
  double dx = 1.0 / (double)n_side;
  p->dx = p->dy = p->dz = dx;
  p->delta = 3.015 * dx;
  p->CSolid = 1.0;
  p->CSat = 0.035;
  p->F = 1.0;
  p->R = 1.0;
  p->T = 1.0;
  p->vol_red = 0.0;
  const double z[4] = {2.0, -1.0, -1.0, 1.0};
  const double D[4] = {0.7e-3, 2.0e-3, 5.3e-3, 1.3e-3};
  double K1 = 3.0 / (kPi * p->delta * p->delta);
  double K2 = 1.0 / (kPi * p->delta * p->delta);
  double dmax = 0.0;
  for (int k = 0; k < 4; ++k) {
    p->z[k] = z[k];
    p->D_liquid[k] = D[k];
    p->D_solid[k] = 1e-3 * D[k];
    p->s1[k] = 0.0;
    p->s2[k] = 0.0;
    p->K1[k] = K1;
    p->K2[k] = K2;
    if (D[k] > dmax) dmax = D[k];
  }
  p->sigma = 0.01;
  p->s_phi = 0.0;
  p->K_phi = K1;
  p->k_diss = 0.05;
  p->switch_width = 0.0;
  p->c_floor = 1e-8 / p->CSolid;
  p->sub_step_no = 8;
  p->dt = 0.2 * dx * dx / dmax;
}

}  // namespace nnpp

extern "C" int64_t nnpp_synth_count(int kind, int n_side) {
  if (kind < 0 || kind > 4 || n_side < 2 || n_side > 2000) return -1;
  return (int64_t)n_side * n_side * n_side;
}

extern "C" nnpp_status nnpp_synth_fill(int kind, int n_side, uint64_t seed, double* nodes,
                                       int* bctypes, double* bcvalues, double* icvalues,
                                       int* phase0, nnpp_params* params) {
  using namespace nnpp;
  int64_t N64 = nnpp_synth_count(kind, n_side);
  if (N64 <= 0 || N64 > 0x7fffffff) return set_error(NNPP_ERR_INVALID, "synth: bad kind/n_side");
  if (!nodes || !bctypes || !bcvalues || !icvalues || !phase0 || !params)
    return set_error(NNPP_ERR_INVALID, "synth: null output");
  const int N = (int)N64;
  const int n = n_side;
  const int S = NNPP_NSPECIES;
  synth_default_params(n, params);
  const double dx = params->dx;
  Rng rng(seed * 0x2545F4914F6CDD1Dull + (uint64_t)kind * 0x9E3779B97F4A7C15ull + 12345u);

  // Instance-level draws first (shape, modes, parameters), then per-node draws.
  double sh_coef[8];
  int sh_idx[8];
  int shape = 0;
  double semi[3] = {0.3, 0.3, 0.3};
  if (kind == 1) {
    double norm = 0.0;
    for (int m = 0; m < 8; ++m) {
      sh_idx[m] = (int)(rng.next() % 24u);
      sh_coef[m] = rng.uni(-1.0, 1.0);
      norm += sh_coef[m] * sh_coef[m];
    }
    norm = std::sqrt(norm);
    for (int m = 0; m < 8; ++m) sh_coef[m] /= norm;
  }
  if (kind == 4) {
    shape = (int)(rng.next() % 3u);  // 0 sphere, 1 cylinder (z), 2 ellipsoid
    for (int d = 0; d < 3; ++d) semi[d] = rng.uni(0.15, 0.35);
    if (shape == 0) semi[1] = semi[2] = semi[0];
    if (shape == 1) semi[1] = semi[0];
    double dmax = 0.0;
    for (int k = 0; k < S; ++k) {
      double f = rng.uni(0.5, 2.0);
      params->D_liquid[k] *= f;
      params->D_solid[k] *= f;
      if (params->D_liquid[k] > dmax) dmax = params->D_liquid[k];
    }
    params->dt = 0.2 * dx * dx / dmax;
    params->k_diss = rng.uni(0.02, 0.08);
  }
  if (kind == 3) params->switch_width = 0.01;

  const bool jitter = (kind != 0);
  const int shell = (kind == 3) ? 8 : 3;
  std::vector<int> perm;
  if (kind == 2) {
    perm.resize(N);
    for (int i = 0; i < N; ++i) perm[i] = i;
    for (int i = N - 1; i > 0; --i) {
      int j = (int)(rng.next() % (uint64_t)(i + 1));
      int t = perm[i];
      perm[i] = perm[j];
      perm[j] = t;
    }
  }

  for (int iz = 0; iz < n; ++iz)
    for (int iy = 0; iy < n; ++iy)
      for (int ix = 0; ix < n; ++ix) {
        int lat = ix + n * (iy + n * iz);
        int i = (kind == 2) ? perm[lat] : lat;
        double jx = 0.0, jy = 0.0, jz = 0.0;
        if (jitter) {
          jx = (rng.u01() - 0.5) * 0.5;
          jy = (rng.u01() - 0.5) * 0.5;
          jz = (rng.u01() - 0.5) * 0.5;
        }
        double x = ((double)ix + 0.5 + jx) * dx;
        double y = ((double)iy + 0.5 + jy) * dx;
        double z = ((double)iz + 0.5 + jz) * dx;
        nodes[i] = x;
        nodes[N + i] = y;
        nodes[2 * N + i] = z;

        bool dir = in_shell(ix, iy, iz, n, shell);
        bool solid = false;
        if (kind == 0) {
          int lo = n / 4, hi = n / 4 + n / 2;
          solid = ix >= lo && ix < hi && iy >= lo && iy < hi && iz >= lo && iz < hi;
        } else if (kind == 1) {
          double ux = x - 0.5, uy = y - 0.5, uz = z - 0.5;
          double rr = std::sqrt(ux * ux + uy * uy + uz * uz);
          if (rr == 0.0) {
            solid = true;
          } else {
            double vx = ux / rr, vy = uy / rr, vz = uz / rr;
            double pert = 0.0;
            for (int m = 0; m < 8; ++m) pert += sh_coef[m] * real_sh(sh_idx[m], vx, vy, vz);
            solid = rr < 0.3 + 0.02 * pert;
          }
        } else if (kind == 2) {
          // Screw along z: core radius 0.12, sinusoidal helical thread of depth 0.03 and
          // pitch 0.1 (outer radius 0.15), length 0.8 centred in the unit box.
          double ux = x - 0.5, uy = y - 0.5;
          if (z >= 0.1 && z <= 0.9) {
            double rho = std::sqrt(ux * ux + uy * uy);
            if (rho <= 0.12) {
              solid = true;
            } else if (rho <= 0.15) {
              double t = z / 0.1;
              double fr = t - (double)(int64_t)t;        // in [0,1)
              double a = 2.0 * kPi * fr - kPi;           // in [-pi, pi)
              double sa, ca;
              sincos_series(a, &sa, &ca);
              // cos(theta - psi) with psi = a + pi: cos(psi) = -ca, sin(psi) = -sa
              double cth = (ux * (-ca) + uy * (-sa)) / rho;
              solid = rho <= 0.135 + 0.015 * cth;
            }
          }
        } else if (kind == 3) {
          double ux = x - 0.5, uy = y - 0.5;
          solid = (ux * ux + uy * uy) < 0.25 * 0.25;
        } else {
          double ux = x - 0.5, uy = y - 0.5, uz = z - 0.5;
          double qx = ux / semi[0], qy = uy / semi[1], qz = uz / semi[2];
          if (shape == 1)
            solid = (qx * qx + qy * qy) < 1.0 && uz > -0.35 && uz < 0.35;
          else
            solid = (qx * qx + qy * qy + qz * qz) < 1.0;
        }
        if (dir) solid = false;

        phase0[i] = solid ? 1 : 0;
        bctypes[i] = dir ? 0 : 1;
        for (int k = 0; k < S; ++k) {
          double ic;
          if (dir) {
            ic = 0.1;
          } else if (solid) {
            ic = (k == 0) ? 1.0 : 0.0;
          } else {
            ic = 0.1 + 0.01 * rng.u01();
          }
          icvalues[(int64_t)k * N + i] = ic;
          bcvalues[(int64_t)k * N + i] = dir ? 0.1 * params->CSolid : -1.0;
        }
        icvalues[(int64_t)S * N + i] = 0.0;
        bcvalues[(int64_t)S * N + i] = dir ? 0.0 : -1.0;
      }
  return NNPP_OK;
}
