// chem.cu -- the reference's complete residual: ten species with their reactions and the
// potential (utils::Residuals, utils.h:29-842), in FP64 on the GPU.
//
// The explicit step of this library transports four species with one dissolution source;
// the reference's model has ten species coupled by nine solubility-limited reactions (MgOH2,
// MgCO3, MgHCO3, Mg3(PO4)2, CaCO3, Ca5OH(PO4)3, water, HCO3, HPO4) and, on the implant's
// interface nodes, a cathodic H+ source of Butler-Volmer form.  This entry point evaluates
// all eleven fields as the reference does at the states U^{n+1}, U^n:
//   F_k = (U_k^{n+1} - U_k^n) / dt + sum_KRk1 + sum_KRk2 - R_k              (k = 1..10)
//   F11 = (sum_KR111 - F CSolid sum_k z_k U_k^n) / (K11prop1 sigma1)       (nodes with a
//                                                                           liquid-liquid bond)
// with the bond sums over each node's horizon (diffusion of U^{n+1}, migration in the
// potential of U^n), each species' phase rule (Mg keeps solid-solid bonds and scales bonds
// touching the solid by BV = 10^(-vol_red (1 - voln1rel)); the others skip solid-solid bonds
// and use D_solid on mixed ones) and the reaction terms of utils.h:162-174, 241-253,
// 321-330, 396-401, 466-476, 541-547, 612-618, 683-690.
//
// A thread per node walks its horizon once and carries the 21 bond sums together; each sum
// still runs over the horizon in the reference's order.  The reference forms every term as
// K D (U_n - U_i) / xi^(3+2s) beta dx dy dz with a pow and divisions per term.  Here a bond
// forms 1 / xi from one reciprocal square root and 1 / xi^e by products when all exponents
// agree and e is whole (s = 0 in the reference's data), else through pow; the constant
// factors of a term (K_k1 D, K_k2 D z_k F, K11prop1 sigma1, dx dy dz, 1 / (R T)) are formed on
// the host, and each species' sums run in units of its liquid-liquid factor, which multiplies
// them once per node (bonds of the other classes carry their factor's ratio to it).  A
// species then costs a liquid-liquid bond a subtraction, a product and two fused
// multiply-adds on the FP64 pipe, which bounds the kernel.  Reordering the products moves
// each term by a few ulps: the fields agree with the reference to ~1e-15 of their scale.
// The powers of ten of the solubility constants and BV are formed on the host with the C
// library's pow, as the reference forms them; exp and log at the interface are CUDA's.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "dbuf.cuh"

namespace nnpp {
namespace {

constexpr int kSp = 10;  // species; field kSp is the potential

// The reference's parameter object from its data arrays (utils.h:2343-2484): data2 (51
// values), per species k the datac_k array (z, D_solid, D_liquid, s_k1, s_k2, K_kprop1,
// K_kprop2), datac11 (sigma0, sigma1, s111, K11prop1); derived constants formed on the host.
struct ChemParams {
  double dt, dx, dy, dz, delta, CSolid, CSat;
  double phim, phimse, alphaC, JHp, T, R, F;
  double k1b, k2b, k3b, k4b, k5b, k6b, k7b, k8b, k9b;
  // 10^(-pK) / CSolid of MgOH2, MgCO3, MgHCO3, MgPO4, CaCO3, Ca5OHPO4, H2O, HCO3, HPO4
  double pMgOH2, pMgCO3, pMgHCO3, pMgPO4, pCaCO3, pCa5OHPO4, pH2O, pHCO3, pHPO4;
  double z[kSp], Ds[kSp], Dl[kSp], e1[kSp], e2[kSp];  // e = 3 + 2 s
  double K1[kSp], K2[kSp];
  double sigma1, e11, K11;
  double BV;  // 10^(-vol_red (1 - voln1rel))
  // formed from the above for the bond sums: dx dy dz; per bond class (0 liquid-liquid,
  // 1 liquid-solid, 2 solid-solid) and species K_k1 D and K_k2 D z_k F (Mg: times BV on
  // liquid-solid bonds); K11prop1 sigma1; the common exponent as a whole number (0 if the
  // exponents differ or are not whole)
  double dxyz, a1[3][kSp], a2[3][kSp], KS11;
  int ie, one_exp;
  // the bond sums' factors: sg = the liquid-liquid factor (1 where it is zero), on = it is
  // not zero, q[0] / q[1] = the liquid-solid / solid-solid factor over sg
  double sg1[kSp], sg2[kSp], q1[2][kSp], q2[2][kSp];
  int on1[kSp], on2[kSp];
};

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double pos(double a) { return fmax(a, 0.0); }  // std::max(a, 0.0)

// U8 U8 U8 U8 U8 U7 U7 U7 after a leading factor a, left to right
__device__ __forceinline__ double ca5ohpo4(double a, double u8, double u7) {
  double t = a;
  for (int q = 0; q < 5; ++q) t = mul(t, u8);
  for (int q = 0; q < 3; ++q) t = mul(t, u7);
  return t;
}

// 1 / xi^e from rs = 1 / xi: by repeated products when e is a small whole number (ie > 0),
// else through pow
__device__ __forceinline__ double rpow(double rs, double xi, double e, int ie) {
  if (ie > 0) {
    double p = rs;
    for (int q = 1; q < ie; ++q) p = mul(p, rs);
    return p;
  }
  return dvd(1.0, pow(xi, e));
}

template <bool kOneExp, bool kAllOn>
__global__ void k_residuals_full(ChemParams c, int N, const double* __restrict__ xyz, const int* __restrict__ hz,
                                 const int* __restrict__ hl, const double* __restrict__ Un1,
                                 const double* __restrict__ Un, const int* __restrict__ phase,
                                 double* __restrict__ F) {
  const double rRT = dvd(1.0, mul(c.R, c.T));
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const int pi = phase[i];
    const int len = hl[i];
    const double xi0 = xyz[i], yi0 = xyz[N + i], zi0 = xyz[2 * N + i];
    int iface = 0;
    if (pi == 1)
      for (int j = 1; j < len; ++j)
        if (phase[hz[(size_t)j * N + i]] == 0) {
          iface = 1;
          break;
        }
    // S1, S2: the bond sums in units of the species' liquid-liquid factors (sg1, sg2): a
    // liquid-liquid bond adds w (U_n - U_i) and v U_n dphi, other bonds the same scaled by
    // their class's factor over the liquid-liquid one
    double S1[kSp], S2[kSp], ui[kSp], S11 = 0.0;
#pragma unroll
    for (int k = 0; k < kSp; ++k) {
      S1[k] = S2[k] = 0.0;
      ui[k] = Un1[(size_t)k * N + i];
    }
    int flag = 0;
    const double phi_i = Un[(size_t)kSp * N + i];
    const double phi1_i = Un1[(size_t)kSp * N + i];
    for (int j = 1; j < len; ++j) {
      const int n = hz[(size_t)j * N + i];
      const double ex = sub(xyz[n], xi0), ey = sub(xyz[N + n], yi0), ez = sub(xyz[2 * N + n], zi0);
      const double x2 = fma(ex, ex, fma(ey, ey, mul(ez, ez)));
      const double rs = rsqrt(x2);  // 1 / xi
      const double xi = mul(x2, rs);
      const double beta = beta_fn<double>(xi, c.delta, c.dx);
      const int pn = phase[n];
      const bool ss = pi == 1 && pn == 1, ll = pi == 0 && pn == 0;
      const int cls = ss ? 1 : 0;  // the factors of a bond that is not liquid-liquid
      const double dphi = sub(Un[(size_t)kSp * N + n], phi_i);
      // the bond's beta dx dy dz, and 1 / (R T) for the migration terms
      const double bd = mul(beta, c.dxyz);
      double w1 = 0.0, v2 = 0.0;
      if (kOneExp) {
        w1 = mul(rpow(rs, xi, c.e1[0], c.ie), bd);
        v2 = mul(w1, rRT);
      }
      if (ll) {
        // liquid-liquid: the sums' own units (ON: a species whose liquid-liquid factor is
        // zero takes nothing here)
#pragma unroll
        for (int k = 0; k < kSp; ++k) {
          if (!kOneExp) {
            w1 = mul(rpow(rs, xi, c.e1[k], 0), bd);
            v2 = mul(mul(rpow(rs, xi, c.e2[k], 0), bd), rRT);
          }
          const double un = Un1[(size_t)k * N + n];
          if (kAllOn || c.on1[k]) S1[k] = fma(w1, sub(un, ui[k]), S1[k]);
          if (kAllOn || c.on2[k]) S2[k] = fma(v2, mul(un, dphi), S2[k]);
        }
      } else {
#pragma unroll
        for (int k = 0; k < kSp; ++k) {
          if (k > 0 && ss) continue;  // solid-solid bonds carry only Mg
          if (!kOneExp) {
            w1 = mul(rpow(rs, xi, c.e1[k], 0), bd);
            v2 = mul(mul(rpow(rs, xi, c.e2[k], 0), bd), rRT);
          }
          const double un = Un1[(size_t)k * N + n];
          S1[k] = fma(mul(w1, c.q1[cls][k]), sub(un, ui[k]), S1[k]);
          S2[k] = fma(mul(v2, c.q2[cls][k]), mul(un, dphi), S2[k]);
        }
      }
      if (ll) {
        const double w11 = kOneExp ? w1 : mul(rpow(rs, xi, c.e11, 0), bd);
        S11 = fma(w11, sub(Un1[(size_t)kSp * N + n], phi1_i), S11);
        flag = 1;
      }
    }
    double s1[kSp], s2[kSp];
#pragma unroll
    for (int k = 0; k < kSp; ++k) {
      s1[k] = -mul(c.sg1[k], S1[k]);
      s2[k] = -mul(c.sg2[k], S2[k]);
    }
    const double s11 = -mul(c.KS11, S11);
    // the fields' values at the node
    double u1[kSp], u0[kSp];
#pragma unroll
    for (int k = 0; k < kSp; ++k) {
      u1[k] = ui[k];
      u0[k] = Un[(size_t)k * N + i];
    }
    const bool liq = pi == 0;
    const bool act = iface || liq;  // solid nodes with a liquid neighbour, liquid nodes
    double R[kSp];
#pragma unroll
    for (int k = 0; k < kSp; ++k) R[k] = 0.0;
    // Mg (utils.h:162-174)
    if (act) {
      double t = mul(-c.k1b, pos(sub(mul(mul(u1[0], u0[2]), u0[2]), c.pMgOH2)));
      t = sub(t, mul(c.k2b, pos(sub(mul(u1[0], u0[4]), c.pMgCO3))));
      t = sub(t, mul(c.k3b, pos(sub(mul(u1[0], u0[4]), c.pMgHCO3))));
      t = sub(t, mul(c.k4b, pos(sub(mul(mul(mul(mul(u0[0], u0[0]), u0[0]), u0[5]), u0[5]), c.pMgPO4))));
      R[0] = t;
    }
    // H+ (utils.h:241-253): the interface's Butler-Volmer source, the liquid's equilibria
    if (iface) {
      const double phic = mul(dvd(mul(c.R, c.T), mul(c.F, c.z[0])), log(dvd(u0[0], dvd(c.CSat, c.CSolid))));
      const double eta = sub(sub(add(c.phim, c.phimse), phi_i), phic);
      R[1] = add(0.0, mul(dvd(c.JHp, mul(mul(c.z[1], c.F), c.CSolid)),
                          exp(dvd(mul(mul(-c.alphaC, c.F), eta), mul(c.R, c.T)))));
    } else if (liq) {
      double t = mul(c.k7b, sub(c.pH2O, mul(u1[1], u0[2])));
      t = add(t, mul(c.k8b, sub(c.pHCO3, mul(u1[1], u0[4]))));
      t = add(t, mul(c.k9b, sub(c.pHPO4, mul(u1[1], u0[6]))));
      R[1] = t;
    }
    // OH- (utils.h:321-330)
    if (act) {
      double t = mul(-c.k1b, pos(sub(mul(mul(u0[2], u0[2]), u0[0]), c.pMgOH2)));
      t = sub(t, mul(c.k6b, pos(sub(ca5ohpo4(u1[2], u0[7], u0[6]), c.pCa5OHPO4))));
      if (liq) t = add(t, mul(c.k7b, sub(c.pH2O, mul(u1[2], u0[1]))));
      R[2] = t;
    }
    // species 4 (utils.h:396-401): the liquid's HCO3 equilibrium
    if (liq) R[3] = mul(c.k8b, sub(c.pHCO3, mul(u1[3], u0[1])));
    // species 5 (utils.h:466-476)
    if (act) {
      double t = mul(-c.k2b, pos(sub(mul(u1[4], u0[0]), c.pMgCO3)));
      t = sub(t, mul(c.k3b, pos(sub(mul(u1[4], u0[0]), c.pMgHCO3))));
      t = sub(t, mul(c.k5b, pos(sub(mul(u1[4], u0[7]), c.pCaCO3))));
      if (liq) t = add(t, mul(c.k8b, sub(c.pHCO3, mul(u0[1], u1[4]))));
      R[4] = t;
    }
    // species 6 (utils.h:541-547)
    if (act) {
      double t = mul(-c.k4b, pos(sub(mul(mul(mul(mul(u0[0], u0[0]), u0[0]), u0[5]), u0[5]), c.pMgPO4)));
      if (liq) t = add(t, mul(c.k9b, add(-c.pHPO4, mul(u0[6], u0[1]))));
      R[5] = t;
    }
    // species 7 (utils.h:612-618)
    if (act) {
      double t = mul(-c.k6b, pos(sub(ca5ohpo4(u0[2], u0[7], u0[6]), c.pCa5OHPO4)));
      if (liq) t = add(t, mul(c.k9b, sub(c.pHPO4, mul(u1[6], u0[1]))));
      R[6] = t;
    }
    // species 8 (utils.h:683-690)
    if (act) {
      double t = mul(-c.k5b, pos(sub(mul(u1[7], u0[4]), c.pCaCO3)));
      t = sub(t, mul(c.k6b, pos(sub(ca5ohpo4(u0[2], u0[7], u0[6]), c.pCa5OHPO4))));
      R[7] = t;
    }
#pragma unroll
    for (int k = 0; k < kSp; ++k)
      F[(size_t)k * N + i] = sub(add(add(dvd(sub(u1[k], u0[k]), c.dt), s1[k]), s2[k]), R[k]);
    // potential (utils.h:801-841)
    double f11 = 0.0;
    if (flag) {
      double r11 = mul(c.z[0], u0[0]);
#pragma unroll
      for (int k = 1; k < kSp; ++k) r11 = add(r11, mul(c.z[k], u0[k]));
      const double inv = dvd(1.0, mul(c.K11, c.sigma1));
      f11 = sub(mul(inv, s11), mul(mul(mul(inv, c.F), c.CSolid), r11));
    }
    F[(size_t)kSp * N + i] = f11;
  }
}

// every neighbour index of the first len[i] cloud columns names a node (flag set otherwise)
__global__ void k_check_clouds(int N, const int* __restrict__ hz, const int* __restrict__ hl, int* flag) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const int len = hl[i];
    bool bad = false;
    for (int j = 0; j < len; ++j) {
      const int n = hz[(size_t)j * N + i];
      bad = bad || n < 0 || n >= N;
    }
    if (bad) atomicExch(flag, 1);
  }
}

ChemParams make_chem_params(const double* d2, const double* dc, const double* d11, double voln1rel) {
  ChemParams c;
  c.dt = d2[2];
  c.dx = d2[3];
  c.dy = d2[4];
  c.dz = d2[5];
  c.delta = d2[6];
  c.CSolid = d2[7];
  c.CSat = d2[8];
  const double* pk = d2 + 14;  // MgOH2, MgCO3, MgHCO3, MgPO4, CaCO3, Ca5OHPO4, H2O, HCO3, HPO4
  c.pMgOH2 = std::pow(10., -pk[0]) / c.CSolid;
  c.pMgCO3 = std::pow(10., -pk[1]) / c.CSolid;
  c.pMgHCO3 = std::pow(10., -pk[2]) / c.CSolid;
  c.pMgPO4 = std::pow(10., -pk[3]) / c.CSolid;
  c.pCaCO3 = std::pow(10., -pk[4]) / c.CSolid;
  c.pCa5OHPO4 = std::pow(10., -pk[5]) / c.CSolid;
  c.pH2O = std::pow(10., -pk[6]) / c.CSolid;
  c.pHCO3 = std::pow(10., -pk[7]) / c.CSolid;
  c.pHPO4 = std::pow(10., -pk[8]) / c.CSolid;
  c.phim = d2[23];
  c.phimse = d2[24];
  c.alphaC = d2[27];
  c.k1b = d2[29];
  c.k2b = d2[31];
  c.k3b = d2[33];
  c.k4b = d2[35];
  c.k5b = d2[37];
  c.k6b = d2[39];
  c.k7b = d2[41];
  c.k8b = d2[43];
  c.k9b = d2[45];
  c.JHp = d2[46];
  c.T = d2[47];
  c.R = d2[48];
  c.F = d2[49];
  const double vol_red = d2[50];
  c.BV = std::pow(10., -vol_red * (1. - voln1rel));
  for (int k = 0; k < kSp; ++k) {
    const double* s = dc + 7 * k;
    c.z[k] = s[0];
    c.Ds[k] = s[1];
    c.Dl[k] = s[2];
    c.e1[k] = 3.0 + 2.0 * s[3];
    c.e2[k] = 3.0 + 2.0 * s[4];
    c.K1[k] = s[5];
    c.K2[k] = s[6];
  }
  c.sigma1 = d11[1];
  c.e11 = 3.0 + 2.0 * d11[2];
  c.K11 = d11[3];
  c.dxyz = c.dx * c.dy * c.dz;
  for (int k = 0; k < kSp; ++k) {
    const double bv = k == 0 ? c.BV : 1.0;
    c.a1[0][k] = c.K1[k] * c.Dl[k];
    c.a1[1][k] = c.K1[k] * c.Ds[k] * bv;
    c.a1[2][k] = k == 0 ? c.K1[k] * c.Ds[k] : 0.0;
    c.a2[0][k] = c.K2[k] * c.Dl[k] * c.z[k] * c.F;
    c.a2[1][k] = c.K2[k] * c.Ds[k] * bv * c.z[k] * c.F;
    c.a2[2][k] = k == 0 ? c.K2[k] * c.Ds[k] * c.z[k] * c.F : 0.0;
  }
  c.KS11 = c.K11 * c.sigma1;
  for (int k = 0; k < kSp; ++k) {
    c.on1[k] = c.a1[0][k] != 0.0;
    c.on2[k] = c.a2[0][k] != 0.0;
    c.sg1[k] = c.on1[k] ? c.a1[0][k] : 1.0;
    c.sg2[k] = c.on2[k] ? c.a2[0][k] : 1.0;
    for (int q = 0; q < 2; ++q) {
      c.q1[q][k] = c.a1[q + 1][k] / c.sg1[k];
      c.q2[q][k] = c.a2[q + 1][k] / c.sg2[k];
    }
  }
  c.one_exp = c.e11 == c.e1[0];
  for (int k = 0; k < kSp; ++k) c.one_exp = c.one_exp && c.e1[k] == c.e1[0] && c.e2[k] == c.e1[0];
  c.ie = 0;
  if (c.one_exp && c.e1[0] >= 1.0 && c.e1[0] <= 8.0 && c.e1[0] == std::floor(c.e1[0])) c.ie = (int)c.e1[0];
  return c;
}

}  // namespace
}  // namespace nnpp

using namespace nnpp;

extern "C" {

nnpp_status nnpp_residuals_full_device(int n_nodes, const double* d_nodes, const int* d_clouds,
                                       const int* d_lengths, const double* d_U_n1, const double* d_U_n,
                                       const int* d_phase, double voln1rel, const double* data2,
                                       const double* datac, const double* datac11, double* d_F,
                                       void* stream) {
  nnpp::TraceRange trace_("nnpp_residuals_full_device");
  clear_error();
  if (n_nodes <= 0 || !d_nodes || !d_clouds || !d_lengths || !d_U_n1 || !d_U_n || !d_phase || !data2 ||
      !datac || !datac11 || !d_F)
    return set_error(NNPP_ERR_INVALID, "residuals_full: NULL argument");
  const ChemParams c = make_chem_params(data2, datac, datac11, voln1rel);
  if (!(c.dt != 0.0) || !(c.dx > 0.0) || !(c.K11 * c.sigma1 != 0.0))
    return set_error(NNPP_ERR_INVALID, "residuals_full: dt, dx or K11prop1 sigma1 is zero");
  const int blocks = std::max(1, std::min((n_nodes + 127) / 128, 152 * 16));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  bool all_on = true;
  for (int k = 0; k < kSp; ++k) all_on = all_on && c.on1[k] && c.on2[k];
  auto go = [&](auto kern) {
    kern<<<blocks, 128, 0, st>>>(c, n_nodes, d_nodes, d_clouds, d_lengths, d_U_n1, d_U_n, d_phase, d_F);
  };
  if (c.one_exp)
    all_on ? go(k_residuals_full<true, true>) : go(k_residuals_full<true, false>);
  else
    all_on ? go(k_residuals_full<false, true>) : go(k_residuals_full<false, false>);
  NNPP_CUDA(cudaGetLastError());
  return NNPP_OK;
}

nnpp_status nnpp_residuals_full(int n_nodes, const double* nodes_colmajor, const int* clouds_colmajor,
                                int max_node_no, const int* cloud_lengths, const double* U_n1,
                                const double* U_n, const int* phase, double voln1rel, const double* data2,
                                const double* datac, const double* datac11, double* F) {
  nnpp::TraceRange trace_("nnpp_residuals_full");
  clear_error();
  if (n_nodes <= 0 || max_node_no < 1 || !nodes_colmajor || !clouds_colmajor || !cloud_lengths || !U_n1 ||
      !U_n || !phase || !F)
    return set_error(NNPP_ERR_INVALID, "residuals_full: bad argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return set_error(NNPP_ERR_CUDA, "residuals_full: no CUDA device");
  }
  const size_t N = (size_t)n_nodes;
  int ml = 1;
  for (size_t i = 0; i < N; ++i) {
    const int l = cloud_lengths[i];
    if (l < 1 || l > max_node_no) return set_error(NNPP_ERR_INVALID, "residuals_full: cloud length out of range");
    ml = std::max(ml, l);
  }
  // only the first ml columns of the clouds matter; every index must name a node (checked on
  // the device after the copy, before the residual runs)
  DBuf<double> dx, du1, du0, df;
  DBuf<int> dhz, dhl, dph, dflag;
  if (!dx.alloc(3 * N) || !du1.alloc((kSp + 1) * N) || !du0.alloc((kSp + 1) * N) || !df.alloc((kSp + 1) * N) ||
      !dhz.alloc((size_t)ml * N) || !dhl.alloc(N) || !dph.alloc(N) || !dflag.alloc(1))
    return set_error(NNPP_ERR_NOMEM, "residuals_full buffers");
  cudaStream_t st = nullptr;
  NNPP_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } guard{st};
  NNPP_CUDA(cudaMemcpyAsync(dx.get(), nodes_colmajor, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, st));
  NNPP_CUDA(cudaMemcpyAsync(du1.get(), U_n1, sizeof(double) * (kSp + 1) * N, cudaMemcpyHostToDevice, st));
  NNPP_CUDA(cudaMemcpyAsync(du0.get(), U_n, sizeof(double) * (kSp + 1) * N, cudaMemcpyHostToDevice, st));
  NNPP_CUDA(cudaMemcpyAsync(dhz.get(), clouds_colmajor, sizeof(int) * (size_t)ml * N, cudaMemcpyHostToDevice, st));
  NNPP_CUDA(cudaMemcpyAsync(dhl.get(), cloud_lengths, sizeof(int) * N, cudaMemcpyHostToDevice, st));
  NNPP_CUDA(cudaMemcpyAsync(dph.get(), phase, sizeof(int) * N, cudaMemcpyHostToDevice, st));
  NNPP_CUDA(cudaMemsetAsync(dflag.get(), 0, sizeof(int), st));
  k_check_clouds<<<std::max(1, std::min((n_nodes + 255) / 256, 152 * 16)), 256, 0, st>>>(n_nodes, dhz.get(), dhl.get(),
                                                                                      dflag.get());
  NNPP_CUDA(cudaGetLastError());
  int bad = 0;
  NNPP_CUDA(cudaMemcpyAsync(&bad, dflag.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  if (bad) return set_error(NNPP_ERR_INVALID, "residuals_full: cloud index out of range");
  NNPP_TRY(nnpp_residuals_full_device(n_nodes, dx.get(), dhz.get(), dhl.get(), du1.get(), du0.get(), dph.get(),
                                      voln1rel, data2, datac, datac11, df.get(), st));
  NNPP_CUDA(cudaMemcpyAsync(F, df.get(), sizeof(double) * (kSp + 1) * N, cudaMemcpyDeviceToHost, st));
  NNPP_CUDA(cudaStreamSynchronize(st));
  return NNPP_OK;
}

}  // extern "C"
