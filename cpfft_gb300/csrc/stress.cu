// stress.cu -- per-voxel stress update and consistent tangent, FP64 (sm_103a).
//
// One thread per voxel.  Each thread runs the material-point sequence of
// do_nleps_block (src/drive_eps_sig.f:200-325): polar decompositions, the unrotated
// strain increment, the mm10 Voce/FCC crystal update (src/mm10_a.f, src/mm10_b.f), the
// Cauchy -> first Piola-Kirchhoff pull-back and the exact dP/dF of cep2A
// (src/cep2A.f:86-284).  The arithmetic is reorganised for a GPU whose FP64 pipe is
// the bound: integer powers by binary powering when the rate exponent is integral,
// reciprocals hoisted out of the 12-slip loops, and cep2A's 81-term loops contracted
// through 3x3 intermediates (about 1.6 kflop instead of ~20 kflop).  Every local loop
// is bounded by miter and the line-search cap, so no thread can spin.
#include <algorithm>

#include "common.cuh"

// Slip systems of the crystals this translation unit serves: 12 here (fcc, bcc, roters,
// bcc12: the slip table is the grid's, in the crystal records);
// stress48.cu compiles this file again with CPFFT_NSLIP 48 (BCC {110},{112},{123}<111>),
// stress6.cu with 6 (hcp6, hcp18) and stress1.cu with 1 (single).
#ifndef CPFFT_NSLIP
#define CPFFT_NSLIP 12
#define CPFFT_STRESS_LAUNCH launch_stress
#endif
// Hardening law: Voce (1) here; stress_mts.cu compiles this file again with CPFFT_LAW 2
// (MTS), stress_mrr.cu with CPFFT_LAW 7 (Ma-Roters-Raabe, mrr.cuh) and stress_ornl.cu with
// CPFFT_LAW 4 (ORNL, mrr.cuh).  The kernels that serve every grid (mm01, the voxel queue)
// live in the first unit.
#ifndef CPFFT_LAW
#define CPFFT_LAW 1
#endif
#define CPFFT_FIRST_UNIT (CPFFT_NSLIP == 12 && CPFFT_LAW == 1)
#include "mlp.cuh"

namespace {

constexpr int NS = CPFFT_NSLIP;  // slip systems
constexpr bool MTS = CPFFT_LAW == 2;
constexpr bool MRR = CPFFT_LAW == 7 || CPFFT_LAW == 4;  // the dislocation-density laws
// the temperature of the reference's FFT path (drive_10_update, src/rstgp1.f:832)
constexpr double TEMP = 297.0;

__device__ __forceinline__ double sgn1(double x) { return x < 0.0 ? -1.0 : 1.0; }

// |x|^e for a non-negative integer e by binary powering
__device__ __forceinline__ double ipow(double x, int e) {
  double r = 1.0, b = x;
  while (e) {
    if (e & 1) r *= b;
    b *= b;
    e >>= 1;
  }
  return r;
}
__device__ __forceinline__ double powabs(double x, int n_int, double e) {
  return n_int >= 0 ? ipow(fabs(x), n_int) : pow(fabs(x), e);
}

// ---- 3x3 helpers (row-major [9]; FP64, or FP32 for the fast form's tangent) ------------
template <typename R>
__device__ __forceinline__ void mm3(const R* a, const R* b, R* c) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      c[3 * i + j] = a[3 * i] * b[j] + a[3 * i + 1] * b[3 + j] + a[3 * i + 2] * b[6 + j];
}
template <typename R>
__device__ __forceinline__ void mtm3(const R* a, const R* b, R* c) {  // a^T b
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      c[3 * i + j] = a[i] * b[j] + a[3 + i] * b[3 + j] + a[6 + i] * b[6 + j];
}
template <typename R>
__device__ __forceinline__ void mmt3(const R* a, const R* b, R* c) {  // a b^T
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++)
      c[3 * i + j] = a[3 * i] * b[3 * j] + a[3 * i + 1] * b[3 * j + 1] + a[3 * i + 2] * b[3 * j + 2];
}
template <typename R>
__device__ __forceinline__ R det3(const R* a) {
  return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
         a[2] * (a[3] * a[7] - a[4] * a[6]);
}
// inverse by cofactors (inv33, src/drive_eps_sig.f:1017-1100); returns the determinant
__device__ __forceinline__ double inv3(const double* a, double* g) {
  double j1 = a[4] * a[8] - a[5] * a[7];
  double j2 = a[3] * a[8] - a[5] * a[6];
  double j3 = a[3] * a[7] - a[4] * a[6];
  double dj = a[0] * j1 - a[1] * j2 + a[2] * j3;
  double r = 1.0 / dj;
  g[0] = j1 * r;
  g[3] = -j2 * r;
  g[6] = j3 * r;
  g[1] = (a[7] * a[2] - a[1] * a[8]) * r;
  g[4] = (a[0] * a[8] - a[6] * a[2]) * r;
  g[7] = (a[1] * a[6] - a[0] * a[7]) * r;
  g[2] = (a[1] * a[5] - a[2] * a[4]) * r;
  g[5] = (a[2] * a[3] - a[0] * a[5]) * r;
  g[8] = (a[0] * a[4] - a[1] * a[3]) * r;
  return dj;
}

// Polar decomposition R = F U^-1 with U^-1 from the invariants of U (rtcmp1/irscp1,
// src/polar.f:18-120); eigenvalues of C = F^T F from the trigonometric solution of
// the characteristic cubic.
__device__ void polar_R(const double* f, double* r) {
  double c0 = f[0] * f[0] + f[3] * f[3] + f[6] * f[6];   // C11
  double c1 = f[0] * f[1] + f[3] * f[4] + f[6] * f[7];   // C12
  double c2 = f[1] * f[1] + f[4] * f[4] + f[7] * f[7];   // C22
  double c3 = f[0] * f[2] + f[3] * f[5] + f[6] * f[8];   // C13
  double c4 = f[1] * f[2] + f[4] * f[5] + f[7] * f[8];   // C23
  double c5 = f[2] * f[2] + f[5] * f[5] + f[8] * f[8];   // C33
  double cc0 = c0 * c0 + c1 * c1 + c3 * c3;
  double cc1 = c0 * c1 + c1 * c2 + c3 * c4;
  double cc2 = c1 * c1 + c2 * c2 + c4 * c4;
  double cc3 = c0 * c3 + c1 * c4 + c3 * c5;
  double cc4 = c1 * c3 + c2 * c4 + c4 * c5;
  double cc5 = c3 * c3 + c4 * c4 + c5 * c5;
  double q = (c0 + c2 + c5) * (1.0 / 3.0);
  double s0 = c0 - q, s2 = c2 - q, s5 = c5 - q;
  double p1 = c1 * c1 + c3 * c3 + c4 * c4;
  double p2 = s0 * s0 + s2 * s2 + s5 * s5 + 2.0 * p1;
  double e1, e2, e3;
  if (p2 <= 0.0) {
    e1 = e2 = e3 = q;
  } else {
    double p = sqrt(p2 * (1.0 / 6.0));
    double ip = 1.0 / p;
    double B0 = s0 * ip, B2 = s2 * ip, B5 = s5 * ip, B1 = c1 * ip, B3 = c3 * ip, B4 = c4 * ip;
    double rr = 0.5 * (B0 * (B2 * B5 - B4 * B4) - B1 * (B1 * B5 - B4 * B3) + B3 * (B1 * B4 - B2 * B3));
    double phi = rr <= -1.0 ? (M_PI / 3.0) : (rr >= 1.0 ? 0.0 : acos(rr) * (1.0 / 3.0));
    e1 = q + 2.0 * p * cos(phi);
    e3 = q + 2.0 * p * cos(phi + 2.0 * M_PI / 3.0);
    e2 = 3.0 * q - e1 - e3;
  }
  e1 = sqrt(e1);
  e2 = sqrt(e2);
  e3 = sqrt(e3);
  double iu = e1 + e2 + e3;
  double iiu = e1 * e2 + e2 * e3 + e1 * e3;
  double iiiu = e1 * e2 * e3;
  double a2 = 1.0 / (iiiu * (iu * iiu - iiiu));
  double b2 = iu * iiu * iiu - iiiu * (iu * iu + iiu);
  double cq = -iiiu - iu * (iu * iu - 2.0 * iiu);
  double d2 = iu;
  double u0 = a2 * (b2 + cq * c0 + d2 * cc0), u1 = a2 * (cq * c1 + d2 * cc1);
  double u2 = a2 * (b2 + cq * c2 + d2 * cc2), u3 = a2 * (cq * c3 + d2 * cc3);
  double u4 = a2 * (cq * c4 + d2 * cc4), u5 = a2 * (b2 + cq * c5 + d2 * cc5);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    r[3 * i + 0] = f[3 * i] * u0 + f[3 * i + 1] * u1 + f[3 * i + 2] * u3;
    r[3 * i + 1] = f[3 * i] * u1 + f[3 * i + 1] * u2 + f[3 * i + 2] * u4;
    r[3 * i + 2] = f[3 * i] * u3 + f[3 * i + 1] * u4 + f[3 * i + 2] * u5;
  }
}

// Voigt pairs xx,yy,zz,xy,yz,xz
__constant__ int c_vi[6] = {0, 1, 2, 0, 1, 0};
__constant__ int c_vj[6] = {0, 1, 2, 1, 2, 2};

// 6x6 rotation of a tensor-shear Voigt vector, rv = R (.) R^T (mm10_rt2rve)
__device__ void rt2rve(const double* r, double* rv) {
  for (int a = 0; a < 6; a++) {
    int ia = c_vi[a], ja = c_vj[a];
    for (int b = 0; b < 6; b++) {
      int kb = c_vi[b], lb = c_vj[b];
      rv[6 * a + b] = b < 3 ? r[3 * ia + kb] * r[3 * ja + kb]
                            : r[3 * ia + kb] * r[3 * ja + lb] + r[3 * ia + lb] * r[3 * ja + kb];
    }
  }
}
// unsigned minors: the reference's rotation of (w23,w13,w12) skew vectors (mm10_rt2rvw)
__device__ __forceinline__ void rt2rvw(const double* t, double* rv) {
  rv[0] = t[4] * t[8] - t[5] * t[7];
  rv[1] = t[3] * t[8] - t[5] * t[6];
  rv[2] = t[3] * t[7] - t[4] * t[6];
  rv[3] = t[1] * t[8] - t[2] * t[7];
  rv[4] = t[0] * t[8] - t[2] * t[6];
  rv[5] = t[0] * t[7] - t[1] * t[6];
  rv[6] = t[1] * t[5] - t[2] * t[4];
  rv[7] = t[0] * t[5] - t[2] * t[3];
  rv[8] = t[0] * t[4] - t[1] * t[3];
}

// symmetric part of S*W in the reference's vector forms (mm10_symsw, src/mm10_b.f:1505)
__device__ __forceinline__ void symsw(const double* s, const double* w, double* sw) {
  sw[0] = s[3] * w[2] - s[5] * w[1];
  sw[1] = s[3] * w[2] - s[4] * w[0];
  sw[2] = s[5] * w[1] + s[4] * w[0];
  sw[3] = 0.5 * (w[2] * (s[0] - s[1]) + w[0] * s[5] - w[1] * s[4]);
  sw[4] = 0.5 * (w[0] * (s[1] - s[2]) + w[1] * s[3] + w[2] * s[5]);
  sw[5] = 0.5 * (w[1] * (s[0] - s[2]) + w[0] * s[3] - w[2] * s[4]);
}

// LU with partial pivoting, in place, n <= 7, one right-hand side
template <int n>
__device__ bool lu_solve1(double* a, double* b) {
  for (int k = 0; k < n; k++) {
    int p = k;
    double best = fabs(a[k * n + k]);
    for (int i = k + 1; i < n; i++) {
      double v = fabs(a[i * n + k]);
      if (v > best) { best = v; p = i; }
    }
    if (best == 0.0) return false;
    if (p != k) {
      for (int j = 0; j < n; j++) { double t = a[k * n + j]; a[k * n + j] = a[p * n + j]; a[p * n + j] = t; }
      double t = b[k]; b[k] = b[p]; b[p] = t;
    }
    double inv = 1.0 / a[k * n + k];
    for (int i = k + 1; i < n; i++) {
      double l = a[i * n + k] * inv;
      a[i * n + k] = l;
      for (int j = k + 1; j < n; j++) a[i * n + j] -= l * a[k * n + j];
      b[i] -= l * b[k];
    }
  }
  for (int i = n - 1; i >= 0; i--) {
    double s = b[i];
    for (int k = i + 1; k < n; k++) s -= a[i * n + k] * b[k];
    b[i] = s / a[i * n + i];
  }
  return true;
}

// ---- mm10 Voce crystal (one crystal per voxel) ---------------------------------------
struct Crystal {
  const CrysRec* cr;
  const double* C;       // global 6x6 (orientation record)
  const double* nsig;    // sigma_n
  double ntt, nttr;
  double nD[6];
  // np1 / curr pieces
  double D[6];
  double tinc, dg;
  double ms[NS][6];
  double qc[NS][3];
  double Cms[NS][6];  // C ms_i, constant while ms is (the reference forms it per call)
  // MTS: shear modulus and thresholds of this (sub)step, the n-state values of the history's
  // u words (nu1, nu2 < 0: first step), and the temperature of the (sub)step
  double mu, tau_y, tau_v, ntau_y, nmu, nu1, nu2, temp;
};

__device__ __forceinline__ double Cv(const double* C, int a, int b) { return __ldg(C + 6 * a + b); }

// mm10_setup (src/mm10_a.f:830-975) + Voce setup (:2058-2080): rotate the slip tensors
// of the orientation record by the plastic rotation and the current rotation.
__device__ void setup_np1(Crystal& s, const OriRec* rec, const double* D, double tinc,
                          const double* R, const double* nRp) {
  for (int i = 0; i < 6; i++) s.D[i] = D[i];
  s.tinc = tinc;
  if (s.cr->alter_mode && !MTS) {  // mm10_setup_voche only (src/mm10_a.f:2073)
    s.dg = s.cr->gamma_bar * tinc;
  } else {
    double t1 = D[0] * D[0] + D[1] * D[1] + D[2] * D[2];
    double t2 = D[3] * D[3] + D[4] * D[4] + D[5] * D[5];
    s.dg = sqrt((2.0 / 3.0) * (t1 + 0.5 * t2));
  }
  double tr[9], work[9], RWC[9], RE[36];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) tr[3 * i + j] = nRp[3 * j + i];
  rt2rve(tr, RE);
  mm3(R, tr, work);
  rt2rvw(work, RWC);
  for (int i = 0; i < NS; i++) {
    double m0[6], q0[3];
    for (int a = 0; a < 6; a++) m0[a] = __ldg(rec->ms + 6 * i + a);
    for (int a = 0; a < 3; a++) q0[a] = __ldg(rec->qs + 3 * i + a);
    for (int a = 0; a < 6; a++) {
      double v = RE[6 * a] * m0[0];
      for (int j = 1; j < 6; j++) v = v + RE[6 * a + j] * m0[j];
      s.ms[i][a] = v;
    }
    for (int a = 0; a < 3; a++)
      s.qc[i][a] = RWC[3 * a] * q0[0] + RWC[3 * a + 1] * q0[1] + RWC[3 * a + 2] * q0[2];
    for (int a = 0; a < 6; a++) {
      double v = 0.0;
      for (int j = 0; j < 6; j++) v += Cv(s.C, a, j) * s.ms[i][j];
      s.Cms[i][a] = v;
    }
  }
}

// resolved shear and slip increment of every system (mm10_rs, mm10_slipinc):
//   si = dg/tt |rs/tt|^(n-1) rs = dg |rs|^(n-1) rs / tt^n,
// keeping pw = |rs|^(n-1), which the Jacobian reuses (d si / d rs, d si / d tt)
__device__ __forceinline__ void slips(const Crystal& s, const double* st, double tt, double* rs,
                                      double* si, double* pw) {
  const CrysRec& c = *s.cr;
  double itt = 1.0 / tt;
  double dgn = s.dg * (c.n_int >= 0 ? ipow(itt, c.n_int + 1) : pow(itt, c.rate_n));
  for (int i = 0; i < NS; i++) {
    double r = st[0] * s.ms[i][0] + st[1] * s.ms[i][1] + st[2] * s.ms[i][2] +
               st[3] * s.ms[i][3] + st[4] * s.ms[i][4] + st[5] * s.ms[i][5];
    rs[i] = r;
    double p = powabs(r, c.n_int, c.rate_n - 1.0);
    pw[i] = p;
    si[i] = dgn * p * r;
  }
}

// mm10_setup_mts (src/mm10_a.f:2109-2166): mu(T), the thermal thresholds from the
// continuum rate dg / tinc, and tau_y, mu at n (the history's u, or this step's values)
__device__ void mts_setup(Crystal& s, double T) {
  const CrysRec& c = *s.cr;
  s.temp = T;
  s.mu = T == 0.0 ? c.mu_0 : c.mu_0 - c.D_0 / (exp(c.T_0 / T) - 1.0);
  const double dgc = s.dg / s.tinc;
  if (dgc == 0.0) {
    s.tau_v = c.tau_hat_v;
    s.tau_y = c.tau_hat_y;
  } else {
    const double b3 = pow(c.burgers, 3.0);
    s.tau_v = c.tau_hat_v * pow(1.0 - pow(c.boltzman * T / (s.mu * b3 * c.G_0_v) *
                                              log(c.eps_dot_0_v / dgc), 1.0 / c.q_v), 1.0 / c.p_v);
    s.tau_y = c.tau_hat_y * pow(1.0 - pow(c.boltzman * T / (s.mu * b3 * c.G_0_y) *
                                              log(c.gamma_bar / dgc), 1.0 / c.q_y), 1.0 / c.p_y);
  }
  s.ntau_y = s.nu1 < 0.0 ? s.tau_y : s.nu1;
  s.nmu = s.nu2 < 0.0 ? s.mu : s.nu2;
}

// MTS's (ct + tau_l / cta)^m with tau_l = 0, cta = (mu_0/mu)(tt - tau_a) - tau_y
// (mm10_h_mts, src/mm10_b.f:2093-2100); 0/cta keeps the reference's NaN at cta = 0
__device__ __forceinline__ double mts_cta(const Crystal& s, double tt) {
  const CrysRec& c = *s.cr;
  return (c.mu_0 / s.mu) * tt - (c.mu_0 / s.mu) * c.tau_a - s.tau_y;
}
__device__ __forceinline__ double mts_base(const Crystal& s, double cta) {
  return 1.0 - cta / s.tau_v + 0.0 / cta;
}

__device__ __forceinline__ double hterm(const CrysRec& c, double tt) {
  // tau_l = 0 (the lattice-curvature gradients are zeroed by the reference)
  double h = 1.0 - (tt - c.tau_y) * c.inv_tau_v;
  if (tt == c.tau_y) h = __longlong_as_double(0x7ff8000000000000ULL);  // 0/0 of the reference
  return h;
}
__device__ __forceinline__ double hpow(const CrysRec& c, double h) {
  return c.m_is_one ? fabs(h) : pow(fabs(h), c.voce_m);
}

// R1 (mm10_formR1, src/mm10_b.f:1061-1101) from precomputed rs / slip increments
__device__ void formR1(const Crystal& s, const double* st, const double* rs, const double* si,
                       double* R1) {
  const CrysRec& c = *s.cr;
  double dbar[6] = {0, 0, 0, 0, 0, 0}, w[3] = {0, 0, 0};
  double tid = s.tinc * c.iD_v;
  for (int i = 0; i < NS; i++) {
    double f = rs[i] * tid + si[i];
    for (int a = 0; a < 6; a++) dbar[a] += f * s.ms[i][a];
    for (int a = 0; a < 3; a++) w[a] += f * s.qc[i][a];
  }
  double sw[6], wv[6];
  symsw(st, w, sw);
  for (int a = 0; a < 6; a++) wv[a] = s.D[a] - dbar[a];
  for (int a = 0; a < 6; a++) {
    double v = 0.0;
    for (int j = 0; j < 6; j++) v += Cv(s.C, a, j) * wv[j];
    R1[a] = st[a] - s.nsig[a] - v + 2.0 * sw[a];
  }
}

// full residual (mm10_formR + mm10_formR2 / mm10_h_voche); returns tau_tilde rate
__device__ double formR(const Crystal& s, const double* x, double* R, double* rs, double* si,
                        double* pw) {
  const CrysRec& c = *s.cr;
  slips(s, x, x[6], rs, si, pw);
  formR1(s, x, rs, si, R);
  double h = 0.0;
  if constexpr (MTS) {  // mm10_h_mts (src/mm10_b.f:2080-2108)
    const double hp = pow(mts_base(s, mts_cta(s, x[6])), c.voce_m);
    for (int i = 0; i < NS; i++) h += hp * fabs(si[i]);
    h = c.tau_a * (1.0 - s.mu / s.nmu) + (s.mu / c.mu_0) * (s.tau_y - s.ntau_y) +
        (s.mu / s.nmu) * s.ntt + c.theta_0 * (s.mu / c.mu_0) * h;
  } else {
    double ht = hterm(c, x[6]);
    double hp = hpow(c, ht) * sgn1(ht);
    for (int i = 0; i < NS; i++) h += hp * fabs(si[i]);
    h = s.ntt + c.theta_0 * h;
  }
  R[6] = x[6] - h;
  return (h - s.ntt) / s.tinc;
}

// J11 (mm10_formJ11, src/mm10_b.f:177-257); J is 6x6 row-major inside a 7x7 when ld=7
template <int ld, bool WITH12>
__device__ void formJ11(const Crystal& s, const double* st, double tt, const double* rs,
                        const double* si, const double* pw, double* J, double* J12,
                        double itt) {
  const CrysRec& c = *s.cr;
  for (int a = 0; a < 6; a++)
    for (int b = 0; b < 6; b++) J[ld * a + b] = 0.0;
  // d si / d rs = dg n |rs|^(n-1) / tt^n (mm10_dgdt_voche)
  double fac = s.dg * c.rate_n / (c.n_int >= 0 ? ipow(tt, c.n_int + 1) : pow(tt, c.rate_n));
  double tid = s.tinc * c.iD_v;
  double w[3] = {0, 0, 0};
  for (int i = 0; i < NS; i++) {
    double dgdt = fac * pw[i] + tid;
    double sq[6], wv[6];
    symsw(st, s.qc[i], sq);
    for (int a = 0; a < 6; a++) wv[a] = s.Cms[i][a] + 2.0 * sq[a];
    for (int b = 0; b < 6; b++) {
      double t = dgdt * s.ms[i][b];
      for (int a = 0; a < 6; a++) J[ld * a + b] += wv[a] * t;
    }
    if (WITH12) {  // the same (C ms + 2 symTW) vector drives J12 (mm10_formJ12)
      double dgdtt = -c.rate_n * itt * si[i];  // mm10_dgdh_voche
      for (int a = 0; a < 6; a++) J12[a] += wv[a] * dgdtt;
    }
    double f = rs[i] * tid + si[i];
    for (int a = 0; a < 3; a++) w[a] += f * s.qc[i][a];
  }
  // mm10_iw (src/mm10_b.f:1590-1634) and the identity
  J[ld * 0 + 3] += 2.0 * w[2];  J[ld * 0 + 5] -= 2.0 * w[1];
  J[ld * 1 + 3] += 2.0 * w[2];  J[ld * 1 + 4] -= 2.0 * w[0];
  J[ld * 2 + 4] += 2.0 * w[0];  J[ld * 2 + 5] += 2.0 * w[1];
  J[ld * 3 + 0] += w[2];  J[ld * 3 + 1] -= w[2];  J[ld * 3 + 4] -= w[1];  J[ld * 3 + 5] += w[0];
  J[ld * 4 + 1] += w[0];  J[ld * 4 + 2] -= w[0];  J[ld * 4 + 3] += w[1];  J[ld * 4 + 5] += w[2];
  J[ld * 5 + 0] += w[1];  J[ld * 5 + 2] -= w[1];  J[ld * 5 + 3] += w[0];  J[ld * 5 + 4] -= w[2];
  for (int a = 0; a < 6; a++) J[ld * a + a] += 1.0;
}

// full 7x7 Jacobian (mm10_formJ, src/mm10_b.f:901-954)
__device__ void formJ(const Crystal& s, const double* x, const double* rs, const double* si,
                      const double* pw, double* J) {
  const CrysRec& c = *s.cr;
  double tt = x[6];
  double itt = 1.0 / tt;
  double J12[6] = {0, 0, 0, 0, 0, 0}, et[6] = {0, 0, 0, 0, 0, 0};
  formJ11<7, true>(s, x, tt, rs, si, pw, J, J12, itt);
  if constexpr (MTS) {
    // mm10_estress_mts / mm10_ehard_mts (src/mm10_b.f:2110-2187)
    const double cta = mts_cta(s, tt);
    const double b = mts_base(s, cta);
    const double bm = pow(b, c.voce_m);
    const double ur = s.mu / c.mu_0;
    double sum = 0.0;
    for (int i = 0; i < NS; i++) {
      double r2 = c.n_int >= 0 ? (rs[i] < 0.0 ? -pw[i] : (rs[i] > 0.0 ? pw[i] : 0.0))
                               : pow(fabs(rs[i]), c.rate_n - 2.0) * rs[i];
      for (int a = 0; a < 6; a++) et[a] += bm * r2 * s.ms[i][a];
      sum += (c.voce_m * (1.0 / s.tau_v + 0.0 / (cta * cta)) * pow(b, -1.0) +
              ur * c.rate_n / tt) * bm * fabs(si[i]);
    }
    const double fac = c.theta_0 * ur * c.rate_n * s.dg /
                       (c.n_int >= 0 ? ipow(tt, c.n_int + 1) : pow(tt, c.rate_n));
    for (int a = 0; a < 6; a++) {
      J[7 * a + 6] = J12[a];
      J[7 * 6 + a] = -(fac * et[a]);
    }
    J[48] = 1.0 + c.theta_0 * sum;
    return;
  }
  double ht = hterm(c, tt);
  double hp = hpow(c, ht);
  double sh = sgn1(ht);
  double etau = 0.0;
  for (int i = 0; i < NS; i++) {
    // mm10_estress_voche: |rs|^(n-2) rs = |rs|^(n-1) sign(rs)
    double r2 = c.n_int >= 0 ? (rs[i] < 0.0 ? -pw[i] : (rs[i] > 0.0 ? pw[i] : 0.0))
                             : pow(fabs(rs[i]), c.rate_n - 2.0) * rs[i];
    double f = hp * sh * r2;
    for (int a = 0; a < 6; a++) et[a] += f * s.ms[i][a];
    double asi = fabs(si[i]);                          // mm10_ehard_voche
    double ta = c.voce_m * (-c.inv_tau_v) * asi / fabs(ht);
    double tb = asi * c.rate_n * itt * sh;
    if (!c.exact_j22) tb *= sgn1(si[i]);
    etau += (ta - tb) * hp;
  }
  double fac = c.theta_0 * s.dg * c.rate_n / (c.n_int >= 0 ? ipow(tt, c.n_int + 1) : pow(tt, c.rate_n));
  for (int a = 0; a < 6; a++) {
    J[7 * a + 6] = J12[a];
    J[7 * 6 + a] = -(fac * et[a]);
  }
  J[48] = 1.0 - c.theta_0 * etau;
}

// mm10_tangent's JA and JB for MTS (src/mm10_a.f:658-815 with mm10_ed_mts and
// mm10_dgdd_mts, src/mm10_b.f:2189-2378) at the converged (sigma, tau) of the full step:
// JR -= JA + JB, JA = sum_i (C ms_i + 2 symtq) (x) dgamma_i/dD, JB = J12 (x) ed / J22.
// The reference passes the whole symtqmat where a column is meant, so every system's JA
// term takes system 1's column (mm10_a_mult_type_4 reads its first six words).
__device__ void mts_tangent_rhs(const Crystal& s, const double* st, double tt, const double* J,
                                double* JR) {
  const CrysRec& c = *s.cr;
  double rs[NS], si[NS], pw[NS];
  slips(s, st, tt, rs, si, pw);
  const double dm[6] = {s.D[0], s.D[1], s.D[2], 0.5 * s.D[3], 0.5 * s.D[4], 0.5 * s.D[5]};
  const double alpha = 2.0 / (3.0 * s.dg * s.dg);
  double sq1[6];
  symsw(st, s.qc[0], sq1);
  // JA: sum_i wv_i (x) (alpha si_i d_mod)
  for (int i = 0; i < NS; i++) {
    double wv[6];
    for (int a = 0; a < 6; a++) wv[a] = s.Cms[i][a] + 2.0 * sq1[a];
    const double g = alpha * si[i];
    for (int a = 0; a < 6; a++)
      for (int b = 0; b < 6; b++) JR[6 * a + b] -= wv[a] * (g * dm[b]);
  }
  // ed (mm10_ed_mts)
  const double dgc = s.dg / s.tinc;
  const double b3 = pow(c.burgers, 3.0);
  const double lny = log(c.gamma_bar / dgc);
  const double ty = c.boltzman * s.temp / (s.mu * b3 * c.G_0_y) * lny;
  const double fy = 2.0 * c.tau_hat_y / (3.0 * s.dg * s.dg * c.q_y * c.p_y * lny) *
                    pow(1.0 - pow(ty, 1.0 / c.q_y), 1.0 / c.p_y - 1.0) * pow(ty, 1.0 / c.q_y);
  const double lnv = log(c.eps_dot_0_v / dgc);
  const double tv = c.boltzman * s.temp / (s.mu * b3 * c.G_0_v) * lnv;
  const double fv = 2.0 * c.tau_hat_v / (3.0 * s.dg * s.dg * c.q_v * c.p_v * lnv) *
                    pow(1.0 - pow(tv, 1.0 / c.q_v), 1.0 / c.p_v - 1.0) * pow(tv, 1.0 / c.q_v);
  const double mnp0 = s.mu / c.mu_0;
  const double sc = tt / mnp0 - c.tau_a / mnp0 - s.tau_y;
  const double base = 1.0 - sc / s.tau_v + 0.0 / sc;
  const double bm1 = pow(base, c.voce_m - 1.0), bm = pow(base, c.voce_m);
  double ky = 0.0, kv = 0.0, kd = 0.0;
  for (int i = 0; i < NS; i++) {
    const double asi = fabs(si[i]);
    ky += c.voce_m * (1.0 / s.tau_v + 0.0 / (sc * sc)) * bm1 * asi;
    kv += c.voce_m / (s.tau_v * s.tau_v) * sc * bm1 * asi;
    kd += 2.0 / (3.0 * s.dg * s.dg) * bm * asi;
  }
  double ed[6];
  for (int b = 0; b < 6; b++)
    ed[b] = c.theta_0 * mnp0 * (ky * fy * dm[b] + kv * fv * dm[b] + kd * dm[b]) + mnp0 * fy * dm[b];
  // JB = J12 (J22^-1 ed)
  const double i22 = 1.0 / J[48];
  for (int a = 0; a < 6; a++)
    for (int b = 0; b < 6; b++) JR[6 * a + b] -= J[7 * a + 6] * (ed[b] * i22);
}

__device__ __forceinline__ bool anynan(const double* x, int n) {
  bool r = false;
  for (int i = 0; i < n; i++) r |= isnan(x[i]);
  return r;
}

__device__ bool newton_update(Crystal& cu, double* x, double inR_alt, double* Jlast, bool& haveJ,
                              int& iters, double& ttrate, bool fixed_scale = false,
                              int cap = 1 << 30);

// tau_tilde extrapolated along the previous step's rate (mm10_solve, src/mm10_a.f:2900-2935):
// tau_n + max(cos(dev D, dev D_n), 0) * tau_rate_n * dt
__device__ double tau_extrapolated(const Crystal& cu, double tt, double dtinc) {
  double d1[6], d2[6];
  for (int i = 0; i < 6; i++) { d1[i] = cu.D[i]; d2[i] = cu.nD[i]; }
  for (int k = 0; k < 2; k++) {
    double* d = k ? d2 : d1;
    double dtr = (d[0] + d[1] + d[2]) / 3.0;
    d[0] -= dtr; d[1] -= dtr; d[2] -= dtr;
    double t = d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + d[3] * d[3] + d[4] * d[4] + d[5] * d[5];
    double sc = t == 0.0 ? 0.0 : 1.0 / sqrt(t);
    for (int i = 0; i < 6; i++) d[i] = t == 0.0 ? 0.0 : d[i] * sc;
  }
  double cs = d1[0] * d2[0] + d1[1] * d2[1] + d1[2] * d2[2] + d1[3] * d2[3] + d1[4] * d2[4] + d1[5] * d2[5];
  cs = fmax(cs, 0.0);
  return tt + cs * cu.nttr * dtinc;
}

// mm10_solve (src/mm10_a.f:2860-3295): predict on R1 with tau_tilde extrapolated, then
// the coupled Newton; Armijo line search c = 1e-4, halving, at most 11 trials.
__device__ bool solve(Crystal& cu, double dtinc, double* stress, double& tt, double* Jlast,
                      bool& haveJ, int& iters, int& piters, double& ttrate) {
  const CrysRec& c = *cu.cr;
  const double cls = 1.0e-4;
  double x[7], rs[NS], si[NS], pw[NS];
  for (int i = 0; i < 6; i++) x[i] = stress[i];
  x[6] = tt;
  double inR1;
  {  // ---- predict
    double x2 = tau_extrapolated(cu, x[6], dtinc);
    double x1[6], R1[6];
    for (int i = 0; i < 6; i++) x1[i] = x[i];
    slips(cu, x1, x2, rs, si, pw);
    formR1(cu, x1, rs, si, R1);
    double dot = 0;
    for (int a = 0; a < 6; a++) dot += R1[a] * R1[a];
    double nR1 = sqrt(dot);
    inR1 = nR1;
    int it = 0;
    while (nR1 > c.atol1 && nR1 / inR1 > c.rtol1) {
      double J[36], mJ[36], dx[6];
      formJ11<6, false>(cu, x1, x2, rs, si, pw, J, nullptr, 0.0);
      for (int a = 0; a < 36; a++) mJ[a] = -J[a];
      for (int a = 0; a < 6; a++) dx[a] = R1[a];
      lu_solve1<6>(mJ, dx);
      double ls1 = 0.5 * dot, ls2 = 0.0;
      for (int a = 0; a < 6; a++) {
        double wv = 0.0;
        for (int b = 0; b < 6; b++) wv += J[6 * b + a] * R1[b];
        ls2 += dx[a] * wv;
      }
      ls2 *= cls;
      double alpha = 1.0;
      for (int ls = 0;; ls++) {
        double xn[6];
        for (int a = 0; a < 6; a++) xn[a] = x1[a] + alpha * dx[a];
        slips(cu, xn, x2, rs, si, pw);
        formR1(cu, xn, rs, si, R1);
        dot = 0;
        for (int a = 0; a < 6; a++) dot += R1[a] * R1[a];
        nR1 = sqrt(dot);
        if (0.5 * dot <= ls1 + ls2 * alpha || ls > 10) {
          for (int a = 0; a < 6; a++) x1[a] = xn[a];
          break;
        }
        alpha *= 0.5;
      }
      it++;
      if (it > c.miter || anynan(x1, 6)) { piters += it; return false; }
    }
    piters += it;
    for (int i = 0; i < 6; i++) x[i] = x1[i];
    x[6] = x2;
  }
  // ---- update
  if (!newton_update(cu, x, inR1, Jlast, haveJ, iters, ttrate)) return false;
  for (int i = 0; i < 6; i++) stress[i] = x[i];
  tt = x[6];
  return true;
}

// Pull a start (sigma, tau) back along the segment from sigma_n until no slip system's
// resolved shear exceeds frac * tau: the power-law Newton converges from inside the rate
// surface and diverges from far outside it.
__device__ void pull_inside(const Crystal& cu, const double* nsig, double* x, double frac) {
  double smax = 1.0;
  const double lim = frac * x[6];
  for (int i = 0; i < NS; i++) {
    double r0 = 0.0, dr = 0.0;
    for (int k = 0; k < 6; k++) {
      r0 += nsig[k] * cu.ms[i][k];
      dr += (x[k] - nsig[k]) * cu.ms[i][k];
    }
    if (dr > 0.0 && r0 + dr > lim) smax = fmin(smax, fmax(0.0, (lim - r0) / dr));
    if (dr < 0.0 && r0 + dr < -lim) smax = fmin(smax, fmax(0.0, (-lim - r0) / dr));
  }
  for (int k = 0; k < 6; k++) x[k] = nsig[k] + smax * (x[k] - nsig[k]);
}

// The full step's coupled Newton started at x0 = (sigma, tau) -- the previous global
// iteration's converged local state, the return-mapped elastic trial or the learned
// guess -- in place of the predictor's result: no predictor.  The stop test is the coupled Newton's, scaled by the residual of
// the reference's start (sigma_n, extrapolated tau), so both starts iterate to the same
// tolerance; at most `cap` iterations, after which the caller runs the plain solve.
__device__ bool solve_from(Crystal& cu, double dtinc, const double* x0, double* stress,
                           double& tt, double* Jlast, bool& haveJ, int& iters, double& ttrate,
                           int cap) {
  double x[7], R[7], rs[NS], si[NS], pw[NS];
  for (int i = 0; i < 6; i++) x[i] = stress[i];
  x[6] = tau_extrapolated(cu, tt, dtinc);
  formR(cu, x, R, rs, si, pw);
  double dot = 0;
  for (int a = 0; a < 7; a++) dot += R[a] * R[a];
  const double scale = sqrt(dot);
  for (int i = 0; i < 7; i++) x[i] = x0[i];
  if (!(x[6] > 0.0) || anynan(x, 7)) return false;
  if (!newton_update(cu, x, scale, Jlast, haveJ, iters, ttrate, true, cap)) return false;
  for (int i = 0; i < 6; i++) stress[i] = x[i];
  tt = x[6];
  return true;
}

// The coupled 7x7 Newton of mm10_solve (src/mm10_a.f:3105-3295) from x = (sigma, tau):
// Armijo line search, converged when ||R|| <= atol or ||R|| / ||R_0|| <= rtol after at
// least one iteration; inR_alt replaces ||R_0|| when the start is an exact root.
// fixed_scale: inR_alt is the relative test's scale (a start other than the predictor's);
// cap: an iteration limit below miter (that start is then abandoned)
__device__ bool newton_update(Crystal& cu, double* x, double inR_alt, double* Jlast, bool& haveJ,
                              int& iters, double& ttrate, bool fixed_scale, int cap) {
  const CrysRec& c = *cu.cr;
  const double cls = 1.0e-4;
  double rs[NS], si[NS], pw[NS];
  int it = 0;
  double R[7];
  ttrate = formR(cu, x, R, rs, si, pw);
  double dot = 0;
  for (int a = 0; a < 7; a++) dot += R[a] * R[a];
  double nR = sqrt(dot), inR = nR;
  if (inR == 0.0 || fixed_scale) inR = inR_alt;
  const int mit = min(c.miter, cap);
  while ((nR > c.atol && nR / inR > c.rtol) || it < 1) {
    formJ(cu, x, rs, si, pw, Jlast);
    haveJ = true;
    double mJ[49], dx[7];
    for (int a = 0; a < 49; a++) mJ[a] = -Jlast[a];
    for (int a = 0; a < 7; a++) dx[a] = R[a];
    lu_solve1<7>(mJ, dx);
    double ls1 = 0.5 * dot, ls2 = 0.0;
    for (int a = 0; a < 7; a++) {
      double wv = 0.0;
      for (int b = 0; b < 7; b++) wv += Jlast[7 * b + a] * R[b];
      ls2 += dx[a] * wv;
    }
    ls2 *= cls;
    double alpha = 1.0;
    for (int ls = 0;; ls++) {
      double xn[7];
      for (int a = 0; a < 7; a++) xn[a] = x[a] + alpha * dx[a];
      ttrate = formR(cu, xn, R, rs, si, pw);
      dot = 0;
      for (int a = 0; a < 7; a++) dot += R[a] * R[a];
      nR = sqrt(dot);
      if (0.5 * dot <= ls1 + ls2 * alpha || ls > 10) {
        for (int a = 0; a < 7; a++) x[a] = xn[a];
        break;
      }
      alpha *= 0.5;
    }
    it++;
    if (it > mit || anynan(x, 7)) { iters += it; return false; }
  }
  iters += it;
  return true;
}

// cep2A (src/cep2A.f:86-284), contracted through 3x3 intermediates.  T = double (the
// reference's arithmetic) or float (the fast form: the tangent only steers the global
// Newton iteration, whose residual and stresses stay FP64).
//   Fn, Fn1, Rh, R, fnhinv, finv: row-major 3x3;  t: unrotated Cauchy stress 3x3;
//   C: 6x6 tangent (row-major, local);  J = det Fn1.  Writes A[81] (ij)(kl).
template <typename T>
__device__ void cep2A(const T* Fn, const T* Fn1, const T* t, const T* C, const T* Rh, const T* R,
                      const T* fnhinv, const T* finv, T J, T* A) {
  T U[9], Y[9], tmp[9], sigma[9], Uinv[9], tU[9], Rt[9], RY[9], RYR[9], RtRF[9];
  mtm3(R, Fn1, U);
  T trU = U[0] + U[4] + U[8];
  for (int i = 0; i < 9; i++) Y[i] = -U[i];
  Y[0] += trU; Y[4] += trU; Y[8] += trU;
  mm3(R, t, Rt);
  mmt3(Rt, R, sigma);
  mm3(finv, R, Uinv);
  mm3(t, Uinv, tU);
  mm3(R, Y, RY);
  mmt3(RY, R, RYR);
  T dY = T(1) / det3(Y);
  mm3(Rt, Uinv, RtRF);
  T Fnh[9], Uh[9], Yh[9], RYh[9], RYRh[9], Fp[9], L[9], D2[9];
  for (int i = 0; i < 9; i++) { Fnh[i] = T(0.5) * (Fn1[i] + Fn[i]); Fp[i] = T(0.5) * fnhinv[i]; tmp[i] = Fn1[i] - Fn[i]; }
  mtm3(Rh, Fnh, Uh);
  T trUh = Uh[0] + Uh[4] + Uh[8];
  for (int i = 0; i < 9; i++) Yh[i] = -Uh[i];
  Yh[0] += trUh; Yh[4] += trUh; Yh[8] += trUh;
  mm3(Rh, Yh, RYh);
  mmt3(RYh, Rh, RYRh);
  T hY = T(0.5) / det3(Yh);
  mm3(tmp, Fp, L);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) D2[3 * i + j] = L[3 * i + j] + L[3 * j + i];
  // dt/dF pieces: E = D2 Rh, A1 = RYRh^T E, B1 = RYh^T E, a = Rh^T (I - L), b = Fp Rh
  T E[9], A1[9], B1[9], M[9], am[9], bm[9];
  mm3(D2, Rh, E);
  mtm3(RYRh, E, A1);
  mtm3(RYh, E, B1);
  for (int i = 0; i < 9; i++) M[i] = -L[i];
  M[0] += T(1); M[4] += T(1); M[8] += T(1);
  mtm3(Rh, M, am);
  mm3(Fp, Rh, bm);
  // dt1[(i,j),(p,q)] is symmetric in (i,j); keep its 6 Voigt rows, shear rows doubled
  T w[6][9];
  for (int v = 0; v < 6; v++) {
    int i = c_vi[v], j = c_vj[v];
    for (int p = 0; p < 3; p++)
      for (int q = 0; q < 3; q++) {
        T d13 = hY * (A1[3 * p + j] * Yh[3 * q + i] - B1[3 * q + j] * RYh[3 * p + i]) +
                     hY * (A1[3 * p + i] * Yh[3 * q + j] - B1[3 * q + i] * RYh[3 * p + j]);
        T d2 = am[3 * i + p] * bm[3 * q + j] + bm[3 * q + i] * am[3 * j + p];
        T s = d13 + d2;
        w[v][3 * p + q] = v < 3 ? s : T(2) * s;
      }
  }
  // T_pq[m][n] = sum_v C[v][vm(mn)] w[v][pq] (cep2A_ddot44 with the row index summed)
  // P-terms: P0 + P1 + P2 + P4 from 3x3 products, P3 = J R T_kl Uinv
  T S1[9], YtU[9], RYtU[9], RtYt[9], fRYR[9], RtRYt[9], fRY[9], dJ[9];
  mmt3(sigma, finv, S1);
  mm3(Y, tU, YtU);
  mm3(RY, tU, RYtU);
  mmt3(Rt, Y, RtYt);
  mm3(finv, RYR, fRYR);
  mmt3(Rt, RY, RtRYt);
  mm3(finv, RY, fRY);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) dJ[3 * i + j] = finv[3 * j + i] * J;
  const T JdY = J * dY;
  for (int k = 0; k < 3; k++)
    for (int l = 0; l < 3; l++) {
      int pq = 3 * k + l;
      T Tk[9];
      for (int u = 0; u < 6; u++) {  // distinct (m,n) Voigt column u
        T s = T(0);
        for (int v = 0; v < 6; v++) s += C[6 * v + u] * w[v][pq];
        int m = c_vi[u], n = c_vj[u];
        Tk[3 * m + n] = s;
        Tk[3 * n + m] = s;
      }
      T RT[9], RTU[9];
      mm3(R, Tk, RT);
      mm3(RT, Uinv, RTU);
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          T P0 = RtRF[3 * i + j] * dJ[3 * k + l];
          T P1 = -J * S1[3 * i + l] * finv[3 * j + k];
          T P2 = JdY * (RYR[3 * i + k] * YtU[3 * l + j] - RY[3 * i + l] * RYtU[3 * k + j]);
          T P3 = J * RTU[3 * i + j];
          T P4 = JdY * (RtYt[3 * i + l] * fRYR[3 * j + k] - RtRYt[3 * i + k] * fRY[3 * j + l]);
          T a = P0 + P1 + P2 + P3 + P4;
          long long col = 9 * (3 * i + j) + pq;
          A[col] = a;
        }
    }
}

// margin of the returned starts below the rate surface: |tau_i| <= START_SURFACE tau
constexpr double START_SURFACE = 0.98;

// block state of the learned initial guess inside the stress kernel
struct GuessBlock {
  unsigned char* smem;  // mlp::FWD_SMEM bytes
  uint32_t tmem;        // 256 TMEM columns
  uint64_t* bar;
  uint32_t phase;
};

// Features of the learned initial guess (mlp::NIN, raw units): the quaternion of the
// lattice rotation the local solve sees (Rp_n^T g; sign with w >= 0), the unrotated strain
// increment D (6), the return-mapped elastic trial stress (6), tau_n, the extrapolated tau,
// cos(dev D, dev D_n) (the extrapolation factor) and |D|.  The network's outputs correct
// the return-mapped trial (stress and tau).  FP32: only an initial guess depends on them.
__device__ void guess_features(const double* g, const double* nRp, const double* D,
                               const double* nsig, double ntt, double nttr, const double* nD,
                               float* f) {
  float M[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      M[3 * i + j] = (float)(nRp[i] * g[j] + nRp[3 + i] * g[3 + j] + nRp[6 + i] * g[6 + j]);
  float w, x, y, z;  // Shepperd's branch choice keeps the square root away from zero
  const float t = M[0] + M[4] + M[8];
  if (t > 0.0f) {
    float q = 2.0f * sqrtf(1.0f + t);
    w = 0.25f * q; x = (M[7] - M[5]) / q; y = (M[2] - M[6]) / q; z = (M[3] - M[1]) / q;
  } else if (M[0] > M[4] && M[0] > M[8]) {
    float q = 2.0f * sqrtf(fmaxf(1.0f + M[0] - M[4] - M[8], 1e-20f));
    w = (M[7] - M[5]) / q; x = 0.25f * q; y = (M[1] + M[3]) / q; z = (M[2] + M[6]) / q;
  } else if (M[4] > M[8]) {
    float q = 2.0f * sqrtf(fmaxf(1.0f + M[4] - M[0] - M[8], 1e-20f));
    w = (M[2] - M[6]) / q; x = (M[1] + M[3]) / q; y = 0.25f * q; z = (M[5] + M[7]) / q;
  } else {
    float q = 2.0f * sqrtf(fmaxf(1.0f + M[8] - M[0] - M[4], 1e-20f));
    w = (M[3] - M[1]) / q; x = (M[2] + M[6]) / q; y = (M[5] + M[7]) / q; z = 0.25f * q;
  }
  const float sg = w < 0.0f ? -1.0f : 1.0f;
  f[0] = sg * w; f[1] = sg * x; f[2] = sg * y; f[3] = sg * z;
  for (int i = 0; i < 6; i++) { f[4 + i] = (float)D[i]; f[10 + i] = (float)nsig[i]; }
  f[16] = (float)ntt;
  f[17] = (float)nttr;
  float d1[6], d2[6], n1 = 0.0f, n2 = 0.0f, dd = 0.0f;
  const float tr1 = (float)(D[0] + D[1] + D[2]) / 3.0f, tr2 = (float)(nD[0] + nD[1] + nD[2]) / 3.0f;
  for (int i = 0; i < 6; i++) {
    d1[i] = (float)D[i] - (i < 3 ? tr1 : 0.0f);
    d2[i] = (float)nD[i] - (i < 3 ? tr2 : 0.0f);
    n1 += d1[i] * d1[i];
    n2 += d2[i] * d2[i];
    dd += d1[i] * d2[i];
  }
  f[18] = (n1 > 0.0f && n2 > 0.0f) ? dd * rsqrtf(n1 * n2) : 0.0f;
  float dn = 0.0f;
  for (int i = 0; i < 6; i++) dn += (float)(D[i] * D[i]);
  f[19] = sqrtf(dn);
}

template <bool WARM>
__device__ void voxel_update(const StressArgs& a, long long v, bool valid, int& iters,
                             int& piters, bool& ok, int& rejected, GuessBlock* gb);
__device__ void kinematics(const double* Fn, const double* Fn1, double* rnh, double* rn1,
                           double* fnhinv, double* uddt);
__device__ void store_P_K4(const StressArgs& a, long long v, const double* Fn, const double* Fn1,
                           const double* stress, const double* cep, const double* rnh,
                           const double* rn1, const double* fnhinv);

#if CPFFT_LAW == 7 || CPFFT_LAW == 4
#include "mrr.cuh"
#endif

// WARM: the learned initial guess starts each local Newton solve (launches with iter > 0
// only); every thread of the block takes part in the block-level network evaluation, so
// the tail chunk's surplus threads evaluate a copy of the last voxel and store nothing.
//
// Voxel order: one block per 128 consecutive voxels, or (a.perm != null) the voxel work
// queue: persistent blocks take 128-voxel chunks of a.perm -- voxels sorted by the local
// cost of their previous pass, heaviest first -- from the atomic head a.queue, so a warp
// holds voxels of similar iteration counts and the SMs even out at the tail.
template <bool WARM>
__global__ void __launch_bounds__(128) stress_kernel(StressArgs a) {
  int iters = 0, piters = 0, rej = 0, fails = 0;
  GuessBlock gb{nullptr, 0u, nullptr, 0u};
  if (WARM) {
    extern __shared__ __align__(128) unsigned char guess_smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tslot;
    if (threadIdx.x == 0) {
      tc::mbar_init(&bar, 1);
      tc::fence_mbar_init();
    }
    gb = GuessBlock{guess_smem, mlp::tmem_block_alloc(&tslot, 256), &bar, 0u};
  }
  __shared__ long long chunk;
  // queue: a block takes a.qchunk voxels at a time and works through them 128 at a time
  const int sub_n = a.perm ? a.qchunk / 128 : 1;
  for (long long round = 0, sub = 0;; round++) {
    long long base;
    if (a.perm) {
      if (sub == 0) {
        if (threadIdx.x == 0) chunk = (long long)atomicAdd(a.queue, (unsigned)a.qchunk);
        __syncthreads();
      }
      base = chunk + 128 * sub;
      if (++sub == sub_n) {
        sub = 0;
        __syncthreads();  // every thread has read `chunk` before the next take
      }
    } else {
      base = (long long)blockIdx.x * 128;
    }
    if (base >= a.N3 || (!a.perm && round > 0)) break;
    const long long idx = base + threadIdx.x;
    const bool valid = idx < a.N3;
    const long long last = a.N3 - 1;
    const long long v = a.perm ? (long long)a.perm[valid ? idx : last] : (valid ? idx : last);
    // mm01 voxels belong to launch_mises: here they only fill the network's tile
    const bool mine = valid && (!a.mises || __ldg(a.mises + v) < 0);
    int it = 0, pit = 0, rj = 0;
    bool ok = true;
#if CPFFT_LAW == 7 || CPFFT_LAW == 4
    if (mine) voxel_update_mrr(a, v, it, pit, ok);  // no learned guess for these grids
#else
    if (WARM) {
      voxel_update<true>(a, v, mine, it, pit, ok, rj, &gb);
    } else if (mine) {
      voxel_update<false>(a, v, true, it, pit, ok, rj, nullptr);
    }
#endif
    if (mine) {
      iters += it;
      piters += pit;
      rej += rj;
      fails += ok ? 0 : 1;
      if (a.cost) a.cost[v] = (unsigned char)min(it + pit, 255);
    }
  }
  if (WARM) mlp::tmem_block_free(gb.tmem, 256);
  // statistics, warp-aggregated (every lane of the warp reaches this point)
  unsigned long long li = iters, pi = piters, fl = fails, rj = rej;
  for (int o = 16; o > 0; o >>= 1) {
    li += __shfl_down_sync(0xffffffffu, li, o);
    pi += __shfl_down_sync(0xffffffffu, pi, o);
    fl += __shfl_down_sync(0xffffffffu, fl, o);
    rj += __shfl_down_sync(0xffffffffu, rj, o);
  }
  if ((threadIdx.x & 31) == 0 && a.stats) {
    atomicAdd(a.stats + 0, li);
    atomicAdd(a.stats + 1, fl);
    atomicAdd(a.stats + 2, pi);
    atomicAdd(a.stats + 3, rj);
  }
}

#if CPFFT_FIRST_UNIT
// ---- the voxel work queue: voxels sorted by the cost of their previous pass -----------
constexpr int QBINS = 64;  // costs 0 .. 62 and >= 63 (iterations of the local solve)

// per-bin voxel counts (hist zeroed before)
__global__ void __launch_bounds__(256) k_cost_hist(const unsigned char* __restrict__ cost,
                                                   long long N3, unsigned int* __restrict__ hist) {
  __shared__ unsigned int h[QBINS];
  for (int b = threadIdx.x; b < QBINS; b += blockDim.x) h[b] = 0;
  __syncthreads();
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < N3;
       v += (long long)gridDim.x * blockDim.x)
    atomicAdd(&h[min((int)cost[v], QBINS - 1)], 1u);
  __syncthreads();
  for (int b = threadIdx.x; b < QBINS; b += blockDim.x)
    if (h[b]) atomicAdd(&hist[b], h[b]);
}

// first queue slot of every bin, heaviest bin first (one block of QBINS threads); also
// resets the queue head
__global__ void k_cost_offsets(const unsigned int* __restrict__ hist, unsigned int* __restrict__ offs,
                               unsigned int* __restrict__ queue) {
  __shared__ unsigned int h[QBINS];
  h[threadIdx.x] = hist[threadIdx.x];
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int run = 0;
    for (int b = QBINS - 1; b >= 0; b--) {
      offs[b] = run;
      run += h[b];
    }
    *queue = 0u;
  }
}

// scatter voxel ids into their bins' ranges: each block reserves its bins' slots with one
// atomic per bin, then fills them (order inside a bin is arbitrary)
__global__ void __launch_bounds__(256) k_cost_scatter(const unsigned char* __restrict__ cost,
                                                      long long N3, long long per_block,
                                                      unsigned int* __restrict__ offs,
                                                      int* __restrict__ perm) {
  __shared__ unsigned int cnt[QBINS], start[QBINS];
  for (int b = threadIdx.x; b < QBINS; b += blockDim.x) cnt[b] = 0;
  __syncthreads();
  const long long v0 = (long long)blockIdx.x * per_block;
  const long long v1 = min(v0 + per_block, N3);
  for (long long v = v0 + threadIdx.x; v < v1; v += blockDim.x)
    atomicAdd(&cnt[min((int)cost[v], QBINS - 1)], 1u);
  __syncthreads();
  for (int b = threadIdx.x; b < QBINS; b += blockDim.x) {
    start[b] = cnt[b] ? atomicAdd(&offs[b], cnt[b]) : 0u;
    cnt[b] = 0;
  }
  __syncthreads();
  for (long long v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
    const int b = min((int)cost[v], QBINS - 1);
    perm[start[b] + atomicAdd(&cnt[b], 1u)] = (int)v;
  }
}

#endif

template <bool WARM>
__device__ void voxel_update(const StressArgs& a, long long v, bool valid, int& iters,
                             int& piters, bool& ok, int& rejected, GuessBlock* gb) {
  const long long N3 = a.N3;
  double Fn[9], Fn1[9];
  for (int i = 0; i < 9; i++) {
    Fn[i] = __ldg(a.Fn + i * N3 + v);
    Fn1[i] = __ldg(a.Fn1 + i * N3 + v);
  }
  const OriRec* rec = a.oris + __ldg(a.ori + v);
  const CrysRec* cr = a.cryss + __ldg(a.crys + v);
  // history at n (step 1 re-initialises it, src/mm10_a.f:78-83 and :473-571; MTS:
  // mm10_init_mts's -1 flags, src/mm10_a.f:2090-2107)
  double nsig[6], ntt, nttr, nRp[9], nD[6], nu1 = -1.0, nu2 = -1.0;
  if (a.step == 1) {
    for (int i = 0; i < 6; i++) { nsig[i] = 0.0; nD[i] = 0.0; }
    ntt = MTS ? -1.0 : cr->tau_y + 1.0e-5;
    nttr = 0.0;
    for (int i = 0; i < 9; i++) nRp[i] = (i % 4 == 0) ? 1.0 : 0.0;
  } else {
    if constexpr (MTS) {
      nu1 = a.hist_n[H_U * N3 + v];
      nu2 = a.hist_n[(H_U + 1) * N3 + v];
    }
    for (int i = 0; i < 6; i++) nsig[i] = a.hist_n[(H_SIG + i) * N3 + v];
    ntt = a.hist_n[H_TT * N3 + v];
    // stored column-major; keep row-major locally
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) nRp[3 * i + j] = a.hist_n[(H_RP + 3 * j + i) * N3 + v];
    for (int i = 0; i < 6; i++) nD[i] = a.hist_n[(H_D + i) * N3 + v];
    nttr = a.hist_n[H_TTR * N3 + v];
  }
  double rnh[9], rn1[9], fnhinv[9], uddt[6];
  kinematics(Fn, Fn1, rnh, rn1, fnhinv, uddt);
  // ---- mm10 (src/mm10_a.f:2628-2845, 1080-1157)
  Crystal s;
  s.cr = cr;
  s.C = rec->C;
  s.nsig = nsig;
  s.nttr = nttr;
  s.nu1 = nu1;
  s.nu2 = nu2;
  for (int i = 0; i < 6; i++) s.nD[i] = nD[i];
  setup_np1(s, rec, uddt, a.dt, rn1, nRp);
  if constexpr (MTS) {  // the full step's setup sets tau_tilde at n on the first step
    mts_setup(s, TEMP);
    if (ntt < 0.0) ntt = cr->tau_a + (s.mu / cr->mu_0) * s.tau_y + 0.1;
  }
  s.ntt = ntt;
  double stress[6], tt = ntt, ttrate = 0.0;
  for (int i = 0; i < 6; i++) stress[i] = nsig[i];
  double t1 = 0, t2 = 0;
  for (int i = 0; i < 6; i++) { t1 += uddt[i] * uddt[i]; t2 += stress[i] * stress[i]; }
  bool no_load = t1 == 0.0 && t2 == 0.0;
  bool iter0 = a.iter == 0;
  double cep[36];
  double Jl[49];
  bool haveJ = false;
  ok = true;
  // ---- the return-mapped elastic trial: sigma_n + C D with tau extrapolated, returned
  //      inside the rate surface -- the trial start, and the base the learned guess corrects
  const bool implicit_load = !iter0 && !no_load;
  const bool logit = !WARM && a.log_X && valid && implicit_load &&
                     (v % a.log_stride) == a.log_phase;
  double trial[7];
  for (int i = 0; i < 6; i++) trial[i] = nsig[i];
  trial[6] = ntt;
  if (implicit_load && (WARM || logit || a.start_trial)) {
    for (int i = 0; i < 6; i++) {
      double t = 0.0;
      for (int j = 0; j < 6; j++) t += Cv(s.C, i, j) * uddt[j];
      trial[i] = nsig[i] + t;
    }
    trial[6] = tau_extrapolated(s, ntt, a.dt);
    pull_inside(s, nsig, trial, START_SURFACE);
  }
  // ---- learned initial guess / logging features
  float feat[mlp::NIN];
  if (WARM || logit) guess_features(rec->g, nRp, uddt, trial, ntt, trial[6], nD, feat);
  double guess[7];
  bool have_guess = false;
  if (WARM) {
    float out[mlp::NOUT];
    const mlp::Weights w{reinterpret_cast<const __nv_bfloat16*>(a.mlp_packed), a.mlp_params,
                         a.mlp_norm};
    const bool mok = mlp::forward_tile(w, gb->smem, gb->tmem, gb->bar, &gb->phase, feat, out);
    if (!mok && threadIdx.x == 0) atomicExch(a.mlp_err, 1);
    if (mok) {  // the network's correction of the return-mapped trial
      for (int i = 0; i < 7; i++) guess[i] = trial[i] + (double)out[i];
      have_guess = !anynan(guess, 7) && guess[6] > 0.0 && implicit_load;
    }
    if (have_guess) pull_inside(s, nsig, guess, START_SURFACE);
  } else if (a.start_iterate && !iter0 && !no_load && valid) {
    // the previous global iteration's converged local state of this step (history n+1)
    for (int i = 0; i < 6; i++) guess[i] = a.hist_np1[(H_SIG + i) * N3 + v];
    guess[6] = a.hist_np1[H_TT * N3 + v];
    have_guess = !anynan(guess, 7) && guess[6] > 0.0;
  } else if (a.start_trial && implicit_load) {
    for (int i = 0; i < 7; i++) guess[i] = trial[i];
    have_guess = !anynan(guess, 7) && guess[6] > 0.0;
  }
  if (iter0 || no_load) {
    for (int i = 0; i < 36; i++) cep[i] = __ldg(rec->C + i);
    if (!no_load) {
      double rs[NS], si[NS], pw[NS], R1[6];
      slips(s, stress, tt, rs, si, pw);
      formR1(s, stress, rs, si, R1);
      for (int i = 0; i < 6; i++) stress[i] -= R1[i];
    }
    ttrate = 0.0;
  } else {
    // adaptive sub-stepping: at most 4 halvings (mm10_solve_strup_iterate)
    double ostress[6], ott = ntt, frac = 0.0, stp = 1.0;
    for (int i = 0; i < 6; i++) ostress[i] = stress[i];
    int cuts = 0;
    bool fail = false;
    if (have_guess) {
      // the full step's coupled Newton from the start (learned guess or previous
      // iterate); a solve that fails from there is dropped and the plain path below runs
      double st[6], ttw = ntt, trw = 0.0;
      for (int i = 0; i < 6; i++) st[i] = stress[i];
      const bool okg = solve_from(s, a.dt, guess, st, ttw, Jl, haveJ, iters, trw, a.start_cap);
      if (okg && !anynan(st, 6) && !isnan(ttw)) {
        for (int i = 0; i < 6; i++) stress[i] = st[i];
        tt = ttw;
        ttrate = trw;
        frac = 1.0;
      } else {
        rejected = 1;
        haveJ = false;
      }
    }
    while (frac < 1.0) {
      double Dw[6];
      for (int i = 0; i < 6; i++) Dw[i] = uddt[i] * (stp + frac);
      // the sub-step state differs from np1 only in D, tinc and dg
      s.tinc = a.dt * (stp + frac);
      for (int i = 0; i < 6; i++) s.D[i] = Dw[i];
      if (cr->alter_mode && !MTS) {
        s.dg = cr->gamma_bar * s.tinc;
      } else {
        double q1 = Dw[0] * Dw[0] + Dw[1] * Dw[1] + Dw[2] * Dw[2];
        double q2 = Dw[3] * Dw[3] + Dw[4] * Dw[4] + Dw[5] * Dw[5];
        s.dg = sqrt((2.0 / 3.0) * (q1 + 0.5 * q2));
      }
      // the sub-step's temperature: n's is zero, so it scales with the sub-step
      // (mm10_solve_strup_iterate, src/mm10_a.f:2769)
      if constexpr (MTS) mts_setup(s, TEMP * (stp + frac));
      tt = ntt;
      double tr_sub = 0.0;
      fail = !solve(s, a.dt * stp, stress, tt, Jl, haveJ, iters, piters, tr_sub);
      if (fail) {
        for (int i = 0; i < 6; i++) stress[i] = ostress[i];
        tt = ott;
        stp *= 0.5;
        if (++cuts > 4) break;
        fail = false;
      } else {
        for (int i = 0; i < 6; i++) ostress[i] = stress[i];
        ott = tt;
        frac += stp;
        ttrate = tr_sub;
      }
    }
    if (cuts && a.stats) atomicAdd(a.stats + 4, 1ull);  // a sub-stepped solve (rare)
    // restore the full-step np1 (used by the rotation update below)
    s.tinc = a.dt;
    for (int i = 0; i < 6; i++) s.D[i] = uddt[i];
    if (cr->alter_mode && !MTS) {
      s.dg = cr->gamma_bar * a.dt;
    } else {
      double q1 = uddt[0] * uddt[0] + uddt[1] * uddt[1] + uddt[2] * uddt[2];
      double q2 = uddt[3] * uddt[3] + uddt[4] * uddt[4] + uddt[5] * uddt[5];
      s.dg = sqrt((2.0 / 3.0) * (q1 + 0.5 * q2));
    }
    if constexpr (MTS) mts_setup(s, TEMP);
    ok = !(fail || isnan(tt) || anynan(stress, 6));
    if (ok) {
      // mm10_tangent for Voce (JA = JB = 0): T = (J11 - J12 J21 / J22)^-1 C, symmetrised
      double JJ[36];
      for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) JJ[6 * i + j] = Jl[7 * i + j] - Jl[7 * i + 6] * (Jl[42 + j] / Jl[48]);
      // LU of JJ once, 6 right-hand sides (columns of C)
      int piv[6];
      for (int k = 0; k < 6; k++) {
        int p = k;
        double best = fabs(JJ[6 * k + k]);
        for (int i = k + 1; i < 6; i++)
          if (fabs(JJ[6 * i + k]) > best) { best = fabs(JJ[6 * i + k]); p = i; }
        piv[k] = p;
        if (p != k)
          for (int j = 0; j < 6; j++) { double t = JJ[6 * k + j]; JJ[6 * k + j] = JJ[6 * p + j]; JJ[6 * p + j] = t; }
        double inv = 1.0 / JJ[6 * k + k];
        for (int i = k + 1; i < 6; i++) {
          double l = JJ[6 * i + k] * inv;
          JJ[6 * i + k] = l;
          for (int j = k + 1; j < 6; j++) JJ[6 * i + j] -= l * JJ[6 * k + j];
        }
      }
      // right-hand side C - JA - JB (JA = JB = 0 for Voce)
      double JR[36];
      for (int i = 0; i < 36; i++) JR[i] = __ldg(rec->C + i);
      if constexpr (MTS) mts_tangent_rhs(s, stress, tt, Jl, JR);
      double T[36];
      for (int c = 0; c < 6; c++) {
        double b[6];
        for (int i = 0; i < 6; i++) b[i] = JR[6 * i + c];
        for (int k = 0; k < 6; k++)
          if (piv[k] != k) { double t = b[k]; b[k] = b[piv[k]]; b[piv[k]] = t; }
        for (int i = 1; i < 6; i++)
          for (int k = 0; k < i; k++) b[i] -= JJ[6 * i + k] * b[k];
        for (int i = 5; i >= 0; i--) {
          double sacc = b[i];
          for (int k = i + 1; k < 6; k++) sacc -= JJ[6 * i + k] * b[k];
          b[i] = sacc / JJ[6 * i + i];
        }
        for (int i = 0; i < 6; i++) T[6 * i + c] = b[i];
      }
      for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) cep[6 * i + j] = (T[6 * i + j] + T[6 * j + i]) * 0.5;
    } else {
      for (int i = 0; i < 6; i++) stress[i] = nsig[i];
      tt = ntt;
      ttrate = 0.0;
      for (int i = 0; i < 36; i++) cep[i] = __ldg(rec->C + i);
    }
    if (logit && ok) {  // (features, converged increments) for training the guess
      const unsigned long long slot = atomicAdd(a.log_n, 1ull);
      if ((long long)slot < a.log_cap) {
        for (int i = 0; i < mlp::NIN; i++) a.log_X[slot * mlp::NIN + i] = feat[i];
        for (int i = 0; i < 6; i++) a.log_T[slot * mlp::NOUT + i] = (float)(stress[i] - trial[i]);
        a.log_T[slot * mlp::NOUT + 6] = (float)(tt - trial[6]);
      }
    }
  }
  // ---- plastic rotation (mm10_update_rotation, src/mm10_a.f:3310-3327)
  double Rp[9];
  if (!ok) {
    for (int i = 0; i < 9; i++) Rp[i] = nRp[i];
  } else if (iter0 || no_load) {
    for (int i = 0; i < 9; i++) Rp[i] = 0.0;  // mm10_setup_np1 zero kept by the early return
  } else {
    double tr[9], RW[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) tr[3 * i + j] = nRp[3 * j + i];
    rt2rvw(tr, RW);
    double rs[NS], si[NS], pw[NS], wb[3] = {0, 0, 0};
    slips(s, stress, tt, rs, si, pw);
    double tid = s.tinc * cr->iD_v;
    for (int i = 0; i < NS; i++) {
      double q0[3], qs[3];
      for (int k = 0; k < 3; k++) q0[k] = __ldg(rec->qs + 3 * i + k);
      for (int k = 0; k < 3; k++) qs[k] = RW[3 * k] * q0[0] + RW[3 * k + 1] * q0[1] + RW[3 * k + 2] * q0[2];
      double f = si[i] + rs[i] * tid;
      for (int k = 0; k < 3; k++) wb[k] += f * qs[k];
    }
    double W[9] = {0.0, wb[2], wb[1], -wb[2], 0.0, wb[0], -wb[1], -wb[0], 0.0};
    double al = sqrt(W[5] * W[5] + W[2] * W[2] + W[1] * W[1]);
    double ex[9];
    if (al < 1.0e-16) {
      for (int i = 0; i < 9; i++) ex[i] = 0.0;
    } else {
      double WW[9];
      mm3(W, W, WW);
      double ca = (1.0 - cos(al)) / (al * al), sa = sin(al) / al;
      for (int i = 0; i < 9; i++) ex[i] = ca * WW[i] + sa * W[i];
    }
    ex[0] += 1.0; ex[4] += 1.0; ex[8] += 1.0;
    mm3(ex, nRp, Rp);
  }
  if (!valid) return;
  // ---- store history n+1
  for (int i = 0; i < 6; i++) a.hist_np1[(H_SIG + i) * N3 + v] = stress[i];
  a.hist_np1[H_TT * N3 + v] = tt;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a.hist_np1[(H_RP + 3 * j + i) * N3 + v] = Rp[3 * i + j];
  for (int i = 0; i < 6; i++) a.hist_np1[(H_D + i) * N3 + v] = uddt[i];
  a.hist_np1[H_TTR * N3 + v] = ttrate;
  a.hist_np1[H_U * N3 + v] = MTS ? s.tau_y : 0.0;  // mm10_setup_mts's u(1:2)
  a.hist_np1[(H_U + 1) * N3 + v] = MTS ? s.mu : 0.0;
  // strains at n+1 = strains at n + the unrotated increment (rstgp1_update_strains,
  // src/drive_eps_sig.f:264-265, src/rstgp1.f:1378-1394); zero at n for step 1
  for (int i = 0; i < 6; i++)
    a.hist_np1[(H_EPS + i) * N3 + v] = (a.step == 1 ? 0.0 : a.hist_n[(H_EPS + i) * N3 + v]) + uddt[i];
  store_P_K4(a, v, Fn, Fn1, stress, cep, rnh, rn1, fnhinv);
}

// kinematics of the material point (src/drive_eps_sig.f:227-265): the rotations of F at
// the half step and at n+1, (F_n+1/2)^-1, and the unrotated strain increment uddt
// (engineering shear)
__device__ void kinematics(const double* Fn, const double* Fn1, double* rnh, double* rn1,
                           double* fnhinv, double* uddt) {
  double fnh[9], dfn[9];
  for (int i = 0; i < 9; i++) { fnh[i] = 0.5 * (Fn[i] + Fn1[i]); dfn[i] = Fn1[i] - Fn[i]; }
  polar_R(fnh, rnh);
  polar_R(Fn1, rn1);
  inv3(fnh, fnhinv);
  double ddt[6];
  {
    double L[9];
    mm3(dfn, fnhinv, L);
    ddt[0] = L[0]; ddt[1] = L[4]; ddt[2] = L[8];
    ddt[3] = L[3] + L[1]; ddt[4] = L[7] + L[5]; ddt[5] = L[6] + L[2];
  }
  {  // getrm1 option 1 + qmply1: d = R^T D R in engineering-shear Voigt form
    double Dm[9] = {ddt[0], 0.5 * ddt[3], 0.5 * ddt[5], 0.5 * ddt[3], ddt[1], 0.5 * ddt[4],
                    0.5 * ddt[5], 0.5 * ddt[4], ddt[2]};
    double t1[9], dm[9];
    mtm3(rnh, Dm, t1);
    mm3(t1, rnh, dm);
    uddt[0] = dm[0]; uddt[1] = dm[4]; uddt[2] = dm[8];
    uddt[3] = 2.0 * dm[1]; uddt[4] = 2.0 * dm[5]; uddt[5] = 2.0 * dm[2];
  }
}

// P = J T F^-T from the unrotated stress (getrm1 option 2 + cs2p, src/drive_eps_sig.f:
// 285-296, 1182-1224) and dP/dF from the 6x6 tangent (cep2A, src/cep2A.f:86-284), into
// P, K4 and the FP32 copies the mixed-precision operator reads
__device__ void store_P_K4(const StressArgs& a, long long v, const double* Fn, const double* Fn1,
                           const double* stress, const double* cep, const double* rnh,
                           const double* rn1, const double* fnhinv) {
  const long long N3 = a.N3;
  double fn1inv[9];
  double tm[9] = {stress[0], stress[3], stress[5], stress[3], stress[1], stress[4],
                  stress[5], stress[4], stress[2]};
  double detF = inv3(Fn1, fn1inv);
  {
    double Rt[9], T[9], P[9];
    mm3(rn1, tm, Rt);
    mmt3(Rt, rn1, T);
    mmt3(T, fn1inv, P);  // T F^-T
    for (int i = 0; i < 9; i++) a.P[i * N3 + v] = detF * P[i];
  }
  if (a.tangent_f32) {
    // the fast form's tangent in FP32 (K4 = K4f exactly, K4lo = 0)
    float f[9], f1[9], tf[9], rh[9], r1[9], fhi[9], f1i[9], cf[36], Af[81];
    for (int i = 0; i < 9; i++) {
      f[i] = (float)Fn[i]; f1[i] = (float)Fn1[i]; tf[i] = (float)tm[i]; rh[i] = (float)rnh[i];
      r1[i] = (float)rn1[i]; fhi[i] = (float)fnhinv[i]; f1i[i] = (float)fn1inv[i];
    }
    for (int i = 0; i < 36; i++) cf[i] = (float)cep[i];
    cep2A<float>(f, f1, tf, cf, rh, r1, fhi, f1i, (float)detF, Af);
    for (int m = 0; m < 81; m++) a.K4[m * N3 + v] = (double)Af[m];
    if (a.K4f)
      for (int m = 0; m < 81; m++) a.K4f[m * N3 + v] = Af[m];
    if (a.K4lo)
      for (int m = 0; m < 81; m++) a.K4lo[m * N3 + v] = 0.0f;
    return;
  }
  double A[81];
  cep2A<double>(Fn, Fn1, tm, cep, rnh, rn1, fnhinv, fn1inv, detF, A);
  for (int m = 0; m < 81; m++) a.K4[m * N3 + v] = A[m];
  if (a.K4f)
    for (int m = 0; m < 81; m++) a.K4f[m * N3 + v] = (float)A[m];
  if (a.K4lo)
    for (int m = 0; m < 81; m++) {
      const float h = (float)A[m];
      a.K4lo[m * N3 + v] = (float)(A[m] - (double)h);
    }
}

#if CPFFT_FIRST_UNIT
// ---- mm01: rate-independent Mises plasticity, bilinear uniaxial curve, mixed isotropic /
// kinematic hardening (src/mm01.f), one voxel ---------------------------------------------
// The isothermal update: mm01_init (:328-535), mm01_simple1 (:704-785), mm01_sig_final
// (:626-690), mm01_plastic_work (:546-615), and the consistent tangent cnst1
// (:1222-1374); the reference's decimal constants are kept as it writes them.  Inputs:
// deps = uddt (engineering shear), the H_WORDS history words at n (step 1: the state of
// mm01_set_history, :240-310, with zero stresses).  Outputs: those words at n+1 except
// H_EPS, and the 6x6 tangent (row-major).
__device__ void mises_update(const MisesRec& m, int step, const double* hn, const double* deps,
                             double* hn1, double* cep) {
  const double one = 1.0, two = 2.0, three = 3.0, half = 0.5;
  const double root2 = 1.414213562373095, root3 = 1.7320508075688;
  const double twthrd = 0.666666666666667, root23 = 0.816496580927;
  const double yld_tol = 1.0e-7, htol = 1.0e-6;
  double cgn[9], hist[12];  // stress vector at n (6 stresses, U, Wp, eps_p bar); hist[1..11]
  if (step == 1) {
    for (int i = 0; i < 9; i++) cgn[i] = 0.0;
    for (int i = 0; i < 12; i++) hist[i] = 0.0;
    hist[2] = m.yld / 1.73205080756888;
    hist[4] = 3.0;
    hist[5] = m.h;
  } else {
    for (int i = 0; i < 6; i++) cgn[i] = hn[H_SIG + i];
    cgn[6] = hn[M1_U];
    cgn[7] = hn[M1_WP];
    cgn[8] = hn[M1_EBP];
    hist[0] = 0.0;
    for (int i = 1; i <= 11; i++) hist[i] = hn[M1_LDT + i - 1];
  }
  // ---- mm01_init: trial elastic state with the moduli at n and n+1 (both the deck's)
  const double e = m.e, nu = m.nu, beta = m.beta, hp = m.h;
  const double deps_vol = deps[0] + deps[1] + deps[2];
  const double eps_mean = deps_vol / three;
  const double g_n = e / two / (one + nu);
  const double een1 = (cgn[0] - nu * (cgn[1] + cgn[2])) / e;
  const double een2 = (cgn[1] - nu * (cgn[0] + cgn[2])) / e;
  const double een3 = (cgn[2] - nu * (cgn[0] + cgn[1])) / e;
  const double een4 = cgn[3] / g_n, een5 = cgn[4] / g_n, een6 = cgn[5] / g_n;
  const double eps_vol_n1 = een1 + een2 + een3 + deps_vol;
  const double eps_mean_n = (een1 + een2 + een3) / three;
  const double ee[6] = {(een1 - eps_mean_n) + (deps[0] - eps_mean),
                        (een2 - eps_mean_n) + (deps[1] - eps_mean),
                        (een3 - eps_mean_n) + (deps[2] - eps_mean),
                        een4 + deps[3], een5 + deps[4], een6 + deps[5]};
  const double G = e / (two * (one + nu));
  double dev_el[6], alpha[6], rtse[6];
  for (int i = 0; i < 3; i++) dev_el[i] = two * G * ee[i];
  for (int i = 3; i < 6; i++) dev_el[i] = G * ee[i];
  for (int i = 0; i < 6; i++) alpha[i] = hist[6 + i];
  const double hbari_np1 = beta * hp, hbark_np1 = (one - beta) * hp;
  const double hbark_n = (one - beta) * hist[5];
  const double kbar = (m.yld + hbari_np1 * hist[3]) / root3;
  double lk = one;
  if (fabs(hbark_n) > htol) lk = hbark_np1 / hbark_n;
  for (int i = 0; i < 6; i++) rtse[i] = dev_el[i] - alpha[i] * lk;
  double mrts = sqrt(rtse[0] * rtse[0] + rtse[1] * rtse[1] + rtse[2] * rtse[2] +
                     two * (rtse[3] * rtse[3] + rtse[4] * rtse[4] + rtse[5] * rtse[5]));
  const double yf = mrts - root2 * kbar;
  for (int i = 0; i < 6; i++) rtse[i] = dev_el[i] - alpha[i];
  mrts = sqrt(rtse[0] * rtse[0] + rtse[1] * rtse[1] + rtse[2] * rtse[2] +
              two * (rtse[3] * rtse[3] + rtse[4] * rtse[4] + rtse[5] * rtse[5]));
  const bool yield = yf >= yld_tol * root2 * kbar;
  // ---- mm01_simple1 (yielding) or the elastic update of mm01
  double h1[12], dev[6];
  if (yield) {
    const double ldt = (mrts - root2 * kbar) / (twthrd * (three * G + hp));
    const double k_np1 = kbar + (root2 / three) * hbari_np1 * ldt;
    h1[1] = ldt;
    h1[2] = k_np1;
    h1[3] = hist[3] + ldt * root23;
    h1[5] = hp;
    const double const1 = twthrd * hbark_np1 * ldt / mrts;
    const double const2 = root2 * k_np1 / mrts;
    for (int i = 0; i < 6; i++) {
      h1[6 + i] = hist[6 + i] + const1 * rtse[i];
      dev[i] = h1[6 + i] + const2 * rtse[i];
    }
  } else {
    h1[1] = 0.0;
    h1[2] = kbar;
    h1[3] = hist[3];
    h1[5] = hp;
    for (int i = 0; i < 6; i++) {
      h1[6 + i] = alpha[i] * lk;
      dev[i] = rtse[i] + alpha[i];
    }
  }
  h1[4] = yield ? 1.0 : 3.0;
  // ---- mm01_sig_final: mean stress, energy density
  double cgn1[9];
  const double sig_mean =
      eps_vol_n1 * (three * e * nu / ((one + nu) * (one - two * nu)) + two * G) / three;
  for (int i = 0; i < 3; i++) cgn1[i] = dev[i] + sig_mean;
  for (int i = 3; i < 6; i++) cgn1[i] = dev[i];
  {
    double w = 0.0;
    for (int i = 0; i < 6; i++) w += deps[i] * (cgn1[i] + cgn[i]);
    cgn1[6] = cgn[6] + half * w;
  }
  // ---- mm01_plastic_work
  cgn1[7] = cgn[7];
  cgn1[8] = cgn[8];
  if (yield) {
    double ds[6], dp[6];
    for (int i = 0; i < 6; i++) ds[i] = cgn1[i] - cgn[i];
    dp[0] = deps[0] - (ds[0] - nu * (ds[1] + ds[2])) / e;
    dp[1] = deps[1] - (ds[1] - nu * (ds[0] + ds[2])) / e;
    dp[2] = deps[2] - (ds[2] - nu * (ds[0] + ds[1])) / e;
    for (int i = 3; i < 6; i++) dp[i] = deps[i] - ds[i] / G;
    double w = 0.0;
    for (int i = 0; i < 6; i++) w += dp[i] * (cgn1[i] + cgn[i]);
    cgn1[7] = cgn[7] + half * w;
    const double f1 = (dp[0] - dp[1]) * (dp[0] - dp[1]) + (dp[1] - dp[2]) * (dp[1] - dp[2]) +
                      (dp[0] - dp[2]) * (dp[0] - dp[2]);
    const double f2 = dp[3] * dp[3] + dp[4] * dp[4] + dp[5] * dp[5];
    cgn1[8] = cgn[8] + (root2 / three) * sqrt(f1 + (three / two) * f2);
  }
  // ---- cnst1: consistent tangent (rtsg = rtse, kn1 = k_n+1, ldt = lambda dt)
  for (int i = 0; i < 36; i++) cep[i] = 0.0;
  if (!yield) {
    const double c1 = e / ((one + nu) * (one - two * nu));
    const double c2 = (one - nu) * c1, c3 = ((one - two * nu) / two) * c1, c4 = nu * c1;
    for (int i = 0; i < 3; i++) {
      for (int j = 0; j < 3; j++) cep[6 * i + j] = i == j ? c2 : c4;
      cep[6 * (i + 3) + i + 3] = c3;
    }
  } else {
    const double root2c = 1.414213562;  // cnst1's own sqrt(2)
    const double g = e / (two * (one + nu));
    const double l = (e * nu) / ((one + nu) * (one - two * nu));
    const double k = (three * l + two * g) / three;
    const double mrtsq = rtse[0] * rtse[0] + rtse[1] * rtse[1] + rtse[2] * rtse[2] +
                         two * (rtse[3] * rtse[3] + rtse[4] * rtse[4] + rtse[5] * rtse[5]);
    const double bb = (root2c * h1[2] + (two / three) * (one - beta) * h1[5] * h1[1]) / sqrt(mrtsq);
    const double gamma = one / (one + h1[5] / (three * g));
    const double gambar = gamma - one + bb;
    const double gbar = g * bb;
    const double albar = k - two * gbar / three;
    const double thbar = two * g * gambar;
    for (int i = 0; i < 6; i++)
      for (int j = 0; j <= i; j++) {
        double c = -(thbar * rtse[j] * rtse[i] / mrtsq);
        if (i < 3 && j < 3) c += albar;
        if (i == j) c += i < 3 ? two * gbar : gbar;
        cep[6 * i + j] = c;
        cep[6 * j + i] = c;
      }
  }
  for (int i = 0; i < 6; i++) hn1[H_SIG + i] = cgn1[i];
  for (int i = 1; i <= 11; i++) hn1[M1_LDT + i - 1] = h1[i];
  hn1[M1_U] = cgn1[6];
  hn1[M1_WP] = cgn1[7];
  hn1[M1_EBP] = cgn1[8];
  for (int w = M1_EBP + 1; w < H_EPS; w++) hn1[w] = 0.0;
  for (int w = H_U; w < H_WORDS; w++) hn1[w] = 0.0;
}

__global__ void __launch_bounds__(128) mises_kernel(StressArgs a) {
  const long long N3 = a.N3;
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < N3;
       v += (long long)gridDim.x * blockDim.x) {
    const int mi = __ldg(a.mises + v);
    if (mi < 0) continue;
    const MisesRec m = a.misess[mi];
    double Fn[9], Fn1[9], hn[H_WORDS], hn1[H_WORDS], cep[36];
    for (int i = 0; i < 9; i++) {
      Fn[i] = __ldg(a.Fn + i * N3 + v);
      Fn1[i] = __ldg(a.Fn1 + i * N3 + v);
    }
    for (int w = 0; w < H_WORDS; w++) hn[w] = a.step == 1 ? 0.0 : a.hist_n[w * N3 + v];
    double rnh[9], rn1[9], fnhinv[9], uddt[6];
    kinematics(Fn, Fn1, rnh, rn1, fnhinv, uddt);
    mises_update(m, a.step, hn, uddt, hn1, cep);
    for (int i = 0; i < 6; i++) hn1[H_EPS + i] = hn[H_EPS + i] + uddt[i];
    for (int w = 0; w < H_WORDS; w++) a.hist_np1[w * N3 + v] = hn1[w];
    store_P_K4(a, v, Fn, Fn1, hn1 + H_SIG, cep, rnh, rn1, fnhinv);
  }
}
#endif

}  // namespace

#if CPFFT_FIRST_UNIT
cudaError_t launch_mises(const StressArgs& a, cudaStream_t s) {
  if (a.N3 <= 0 || !a.mises) return cudaSuccess;
  const unsigned blocks = (unsigned)std::min<long long>((a.N3 + 127) / 128, 152LL * 16);
  mises_kernel<<<blocks, 128, 0, s>>>(a);
  g_kernel_launches += 1;
  return cudaGetLastError();
}
#endif

cudaError_t CPFFT_STRESS_LAUNCH(const StressArgs& a, bool warm_in, cudaStream_t s) {
  if (a.N3 <= 0) return cudaSuccess;
  const bool warm = warm_in && !MRR;  // the MRR solve has no learned guess
  if (warm) {  // set on every call: the attribute belongs to the current device
    cudaError_t e = cudaFuncSetAttribute(stress_kernel<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         mlp::FWD_SMEM);
    if (e != cudaSuccess) return e;
  }
  unsigned blocks = (unsigned)((a.N3 + 127) / 128);
  if (a.perm) {
    // persistent: as many blocks as fit on the GPU at once, or a.qbps per SM
    int dev = 0, sms = 0, per = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    e = warm ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, stress_kernel<true>, 128, mlp::FWD_SMEM)
             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, stress_kernel<false>, 128, 0);
    if (e != cudaSuccess) return e;
    if (per < 1) per = 1;
    if (a.qbps > 0 && a.qbps < per) per = a.qbps;
    blocks = (unsigned)std::min<long long>((long long)sms * per, (long long)blocks);
  }
  if (warm) stress_kernel<true><<<blocks, 128, mlp::FWD_SMEM, s>>>(a);
  else stress_kernel<false><<<blocks, 128, 0, s>>>(a);
  g_kernel_launches += 1;
  return cudaGetLastError();
}

#if CPFFT_FIRST_UNIT
cudaError_t launch_voxel_queue(const unsigned char* cost, long long N3, unsigned int* scratch,
                               int* perm, unsigned int* queue, cudaStream_t s) {
  unsigned int* hist = scratch;
  unsigned int* offs = scratch + QBINS;
  cudaError_t e = cudaMemsetAsync(hist, 0, QBINS * sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  const int hb = (int)std::min<long long>((N3 + 255) / 256, 1024);
  k_cost_hist<<<hb, 256, 0, s>>>(cost, N3, hist);
  k_cost_offsets<<<1, QBINS, 0, s>>>(hist, offs, queue);
  const long long per_block = 8192;
  k_cost_scatter<<<(unsigned)((N3 + per_block - 1) / per_block), 256, 0, s>>>(cost, N3, per_block,
                                                                             offs, perm);
  g_kernel_launches += 3;
  return cudaGetLastError();
}
#endif
