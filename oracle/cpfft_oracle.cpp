// cpfft_oracle.cpp -- CPU restatement of the CPFFT finite-strain FFT crystal-plasticity
// hot path (TEST INFRASTRUCTURE ONLY; the product never links it).
//
// Each routine cites the reference routine (path:line, relative to the reference
// project) it restates.  Parity is unpinned: the reference has no tests or golden
// data and cannot be built here; the oracle is checked against analytic known answers
// (tests/test_oracle_*.py).  Third-party arithmetic the reference takes from Intel MKL
// (no version pinned, src/makefile:9-13) is restated from the published algorithms:
// DFTI -> an exact mixed-radix DFT, RCI dcg -> textbook Hestenes-Stiefel CG,
// dgesv -> LU with partial pivoting, dsytrf/dsytri -> Gauss-Jordan inverse.
// The eigenvalues of C = F^T F use the trigonometric closed form of the cubic
// (O. K. Smith, Comm. ACM 4(4) 168, 1961).
#include "cpfft_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef double M3[3][3];
typedef double M6[6][6];
const double PI = 3.141592653589793;  // mm10_constants pi (src/mod_crystals.f:121)

inline double sgn1(double x) { return x < 0.0 ? -1.0 : 1.0; }  // Fortran sign(1,x)

// Voigt pairs in the reference order xx,yy,zz,xy,yz,xz
const int VI[6] = {0, 1, 2, 0, 1, 0};
const int VJ[6] = {0, 1, 2, 1, 2, 2};

void mm33(const M3 a, const M3 b, M3 c) {  // c = a b
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      c[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j];
}
void tr33(const M3 a, M3 b) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) b[i][j] = a[j][i];
}
double det33(const M3 a) {  // cep2A_det33 order (src/cep2A.f:341-360)
  double d = a[0][0] * a[1][1] * a[2][2];
  d = d + a[0][1] * a[1][2] * a[2][0];
  d = d + a[0][2] * a[1][0] * a[2][1];
  d = d - a[0][0] * a[1][2] * a[2][1];
  d = d - a[0][1] * a[1][0] * a[2][2];
  d = d - a[0][2] * a[1][1] * a[2][0];
  return d;
}

// inv33 (src/drive_eps_sig.f:1017-1100): cofactor inverse and determinant
double inv33(const M3 a, M3 g) {
  double j1 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
  double j2 = a[1][0] * a[2][2] - a[1][2] * a[2][0];
  double j3 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
  double dj = a[0][0] * j1 - a[0][1] * j2 + a[0][2] * j3;
  g[0][0] = j1 / dj;
  g[1][0] = -j2 / dj;
  g[2][0] = j3 / dj;
  g[0][1] = (a[2][1] * a[0][2] - a[0][1] * a[2][2]) / dj;
  g[1][1] = (a[0][0] * a[2][2] - a[2][0] * a[0][2]) / dj;
  g[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / dj;
  g[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / dj;
  g[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / dj;
  g[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / dj;
  return dj;
}

// LU with partial pivoting, solve a x = b for nrhs right-hand sides (dgesv).
// a is n x n row-major (destroyed), b is n x nrhs row-major.  Returns 0 or k+1 for a
// zero pivot at step k (LAPACK's info convention).
int lu_solve(int n, double* a, int nrhs, double* b) {
  int info = 0;
  for (int k = 0; k < n; k++) {
    int p = k;
    double best = std::fabs(a[k * n + k]);
    for (int i = k + 1; i < n; i++) {
      double v = std::fabs(a[i * n + k]);
      if (v > best) { best = v; p = i; }
    }
    if (a[p * n + k] == 0.0) { if (!info) info = k + 1; continue; }
    if (p != k) {
      for (int j = 0; j < n; j++) std::swap(a[k * n + j], a[p * n + j]);
      for (int j = 0; j < nrhs; j++) std::swap(b[k * nrhs + j], b[p * nrhs + j]);
    }
    double inv = 1.0 / a[k * n + k];
    for (int i = k + 1; i < n; i++) {
      double l = a[i * n + k] * inv;
      a[i * n + k] = l;
      for (int j = k + 1; j < n; j++) a[i * n + j] -= l * a[k * n + j];
      for (int j = 0; j < nrhs; j++) b[i * nrhs + j] -= l * b[k * nrhs + j];
    }
  }
  if (info) return info;
  for (int j = 0; j < nrhs; j++)
    for (int i = n - 1; i >= 0; i--) {
      double s = b[i * nrhs + j];
      for (int k = i + 1; k < n; k++) s -= a[i * n + k] * b[k * nrhs + j];
      b[i * nrhs + j] = s / a[i * n + i];
    }
  return 0;
}

// Gauss-Jordan inverse of a 6x6 (mm10_invsym's role, src/mm10_a.f:1370-1395)
void inv66(const M6 a, M6 out) {
  double m[6][12];
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 12; j++) m[i][j] = j < 6 ? a[i][j] : (j - 6 == i ? 1.0 : 0.0);
  for (int k = 0; k < 6; k++) {
    int p = k;
    for (int i = k + 1; i < 6; i++)
      if (std::fabs(m[i][k]) > std::fabs(m[p][k])) p = i;
    for (int j = 0; j < 12; j++) std::swap(m[k][j], m[p][j]);
    double inv = 1.0 / m[k][k];
    for (int j = 0; j < 12; j++) m[k][j] *= inv;
    for (int i = 0; i < 6; i++)
      if (i != k) {
        double f = m[i][k];
        for (int j = 0; j < 12; j++) m[i][j] -= f * m[k][j];
      }
  }
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) out[i][j] = m[i][j + 6];
}

// ---- rotation helpers (src/mm10_a.f:1287-1520) -------------------------------------
// Kocks angles in degrees -> crystal rotation g (mm10_rotation_matrix, :1287-1345)
void kocks_g(const double ang[3], M3 r) {
  double psi = ang[0] * PI / 180.0, th = ang[1] * PI / 180.0, phi = ang[2] * PI / 180.0;
  r[0][0] = -std::sin(psi) * std::sin(phi) - std::cos(psi) * std::cos(phi) * std::cos(th);
  r[0][1] = std::cos(psi) * std::sin(phi) - std::sin(psi) * std::cos(phi) * std::cos(th);
  r[0][2] = std::cos(phi) * std::sin(th);
  r[1][0] = std::sin(psi) * std::cos(phi) - std::cos(psi) * std::sin(phi) * std::cos(th);
  r[1][1] = -std::cos(psi) * std::cos(phi) - std::sin(psi) * std::sin(phi) * std::cos(th);
  r[1][2] = std::sin(phi) * std::sin(th);
  r[2][0] = std::cos(psi) * std::sin(th);
  r[2][1] = std::sin(psi) * std::sin(th);
  r[2][2] = std::cos(th);
}
// 6x6 rotation of a tensor-shear Voigt vector: rv = R (.) R^T (mm10_rt2rve :1400-1447,
// also getrm1 option 2, src/polar.f:729-780)
void rt2rve(const M3 r, M6 rv) {
  for (int a = 0; a < 6; a++)
    for (int b = 0; b < 6; b++) {
      int ia = VI[a], ja = VJ[a], kb = VI[b], lb = VJ[b];
      rv[a][b] = b < 3 ? r[ia][kb] * r[ja][kb]
                       : r[ia][kb] * r[ja][lb] + r[ia][lb] * r[ja][kb];
    }
}
// unsigned minors, the reference's 3x3 rotation of its (w23,w13,w12) skew vectors
// (mm10_rt2rvw :1460-1475)
void rt2rvw(const M3 t, M3 rv) {
  rv[0][0] = t[1][1] * t[2][2] - t[1][2] * t[2][1];
  rv[0][1] = t[1][0] * t[2][2] - t[1][2] * t[2][0];
  rv[0][2] = t[1][0] * t[2][1] - t[1][1] * t[2][0];
  rv[1][0] = t[0][1] * t[2][2] - t[0][2] * t[2][1];
  rv[1][1] = t[0][0] * t[2][2] - t[0][2] * t[2][0];
  rv[1][2] = t[0][0] * t[2][1] - t[0][1] * t[2][0];
  rv[2][0] = t[0][1] * t[1][2] - t[0][2] * t[1][1];
  rv[2][1] = t[0][0] * t[1][2] - t[0][2] * t[1][0];
  rv[2][2] = t[0][0] * t[1][1] - t[0][1] * t[1][0];
}
// rotation of an engineering-shear Voigt strain: d = R^T D R (getrm1 option 1,
// src/polar.f:680-728)
void getrm1_opt1(const M3 r, M6 q) {
  for (int a = 0; a < 6; a++)
    for (int b = 0; b < 6; b++) {
      int ia = VI[a], ja = VJ[a], kb = VI[b], lb = VJ[b];
      double v = b < 3 ? r[kb][ia] * r[kb][ja]
                       : 0.5 * (r[kb][ia] * r[lb][ja] + r[lb][ia] * r[kb][ja]);
      q[a][b] = a < 3 ? v : 2.0 * v;
    }
}
void mv6(const M6 a, const double* x, double* y) {  // mm10_a_mult_type_2 order
  for (int i = 0; i < 6; i++) y[i] = a[i][0] * x[0];
  for (int j = 1; j < 6; j++)
    for (int i = 0; i < 6; i++) y[i] = y[i] + a[i][j] * x[j];
}

// ---- polar decomposition (rtcmp1/irscp1/ivcmp1, src/polar.f:18-224) ----------------
void sym3_eigs(const double c[6], double ev[3]) {
  // c in the reference's packed order c11,c12,c22,c13,c23,c33
  double a11 = c[0], a12 = c[1], a22 = c[2], a13 = c[3], a23 = c[4], a33 = c[5];
  double p1 = a12 * a12 + a13 * a13 + a23 * a23;
  double q = (a11 + a22 + a33) / 3.0;
  double b11 = a11 - q, b22 = a22 - q, b33 = a33 - q;
  double p2 = b11 * b11 + b22 * b22 + b33 * b33 + 2.0 * p1;
  if (p2 <= 0.0) { ev[0] = ev[1] = ev[2] = q; return; }
  double p = std::sqrt(p2 / 6.0);
  double ip = 1.0 / p;
  double B11 = b11 * ip, B22 = b22 * ip, B33 = b33 * ip;
  double B12 = a12 * ip, B13 = a13 * ip, B23 = a23 * ip;
  double detB = B11 * (B22 * B33 - B23 * B23) - B12 * (B12 * B33 - B23 * B13) +
                B13 * (B12 * B23 - B22 * B13);
  double r = 0.5 * detB;
  double phi = r <= -1.0 ? PI / 3.0 : (r >= 1.0 ? 0.0 : std::acos(r) / 3.0);
  double e1 = q + 2.0 * p * std::cos(phi);
  double e3 = q + 2.0 * p * std::cos(phi + 2.0 * PI / 3.0);
  double e2 = 3.0 * q - e1 - e3;
  ev[0] = e3; ev[1] = e2; ev[2] = e1;
}
void polar_R(const M3 f, M3 r) {
  double c[6], cc[6];
  c[0] = f[0][0] * f[0][0] + f[1][0] * f[1][0] + f[2][0] * f[2][0];
  c[1] = f[0][0] * f[0][1] + f[1][0] * f[1][1] + f[2][0] * f[2][1];
  c[2] = f[0][1] * f[0][1] + f[1][1] * f[1][1] + f[2][1] * f[2][1];
  c[3] = f[0][0] * f[0][2] + f[1][0] * f[1][2] + f[2][0] * f[2][2];
  c[4] = f[0][1] * f[0][2] + f[1][1] * f[1][2] + f[2][1] * f[2][2];
  c[5] = f[0][2] * f[0][2] + f[1][2] * f[1][2] + f[2][2] * f[2][2];
  cc[0] = c[0] * c[0] + c[1] * c[1] + c[3] * c[3];
  cc[1] = c[0] * c[1] + c[1] * c[2] + c[3] * c[4];
  cc[2] = c[1] * c[1] + c[2] * c[2] + c[4] * c[4];
  cc[3] = c[0] * c[3] + c[1] * c[4] + c[3] * c[5];
  cc[4] = c[1] * c[3] + c[2] * c[4] + c[4] * c[5];
  cc[5] = c[3] * c[3] + c[4] * c[4] + c[5] * c[5];
  double ev[3];
  sym3_eigs(c, ev);
  for (int i = 0; i < 3; i++) ev[i] = std::sqrt(ev[i]);
  double iu = ev[0] + ev[1] + ev[2];
  double iiu = ev[0] * ev[1] + ev[1] * ev[2] + ev[0] * ev[2];
  double iiiu = ev[0] * ev[1] * ev[2];
  // inverse right stretch from the invariants (Hoger & Carlson closed form)
  double a2 = 1.0 / (iiiu * (iu * iiu - iiiu));
  double b2 = iu * iiu * iiu - iiiu * (iu * iu + iiu);
  double c2 = -iiiu - iu * (iu * iu - 2.0 * iiu);
  double d2 = iu;
  double ui[6];
  ui[0] = a2 * (b2 + c2 * c[0] + d2 * cc[0]);
  ui[1] = a2 * (c2 * c[1] + d2 * cc[1]);
  ui[2] = a2 * (b2 + c2 * c[2] + d2 * cc[2]);
  ui[3] = a2 * (c2 * c[3] + d2 * cc[3]);
  ui[4] = a2 * (c2 * c[4] + d2 * cc[4]);
  ui[5] = a2 * (b2 + c2 * c[5] + d2 * cc[5]);
  for (int i = 0; i < 3; i++) {
    r[i][0] = f[i][0] * ui[0] + f[i][1] * ui[1] + f[i][2] * ui[3];
    r[i][1] = f[i][0] * ui[1] + f[i][1] * ui[2] + f[i][2] * ui[4];
    r[i][2] = f[i][0] * ui[3] + f[i][1] * ui[4] + f[i][2] * ui[5];
  }
}

// ---- crystal data (src/mod_crystals.f:438-515, 1796-1880) --------------------------
struct Crys {
  cpfft_crystal p;
  M6 C0;                 // stiffness in the crystal frame
  int ns;                // slip systems
  double b[48][3], n[48][3];
  // Ma-Roters-Raabe interaction matrices (h_type 7): rho_F = Gm rho, rho_P = Hm rho
  double Gm[12][12], Hm[12][12];
};
void fcc_systems(double b[12][3], double n[12][3]) {
  // FCC {111}<110>: slip directions and plane normals, in the reference's order.
  const double f = 1.0 / std::sqrt(2.0), g = 1.0 / std::sqrt(3.0);
  const double B[12][3] = {{0, -f, f}, {f, 0, -f}, {-f, f, 0}, {0, f, f},
                           {f, 0, f},  {f, -f, 0}, {0, -f, f}, {-f, 0, -f},
                           {f, f, 0},  {0, f, f},  {f, 0, -f}, {-f, -f, 0}};
  const double Nn[12][3] = {{g, g, g},  {g, g, g},  {g, g, g},  {-g, -g, g},
                            {-g, -g, g}, {-g, -g, g}, {-g, g, g}, {-g, g, g},
                            {-g, g, g}, {g, -g, g},  {g, -g, g}, {g, -g, g}};
  for (int s = 0; s < 12; s++)
    for (int k = 0; k < 3; k++) { b[s][k] = B[s][k]; n[s][k] = Nn[s][k]; }
}
// BCC {110}, {112}, {123} <111> (slip_type 8, src/mod_crystals.f:812-1207), in the
// reference's order and signs: directions (+-1,+-1,+-1)/sqrt(3), plane normals as integer
// Miller triples normalised by their lengths.
void bcc48_systems(double b[48][3], double n[48][3]) {
  static const int B[48][3] = {
      {-1, 1, 1}, {1, -1, 1}, {1, 1, 1}, {1, 1, -1},
      {1, 1, -1}, {-1, 1, 1}, {1, 1, 1}, {1, -1, 1},
      {1, 1, -1}, {1, -1, 1}, {1, 1, 1}, {-1, 1, 1},
      {1, 1, -1}, {1, -1, 1}, {-1, 1, 1}, {1, 1, 1},
      {1, -1, 1}, {1, 1, -1}, {1, 1, 1}, {-1, 1, 1},
      {-1, 1, 1}, {1, 1, 1}, {1, 1, -1}, {1, -1, 1},
      {1, 1, -1}, {1, -1, 1}, {-1, 1, 1}, {1, 1, 1},
      {1, -1, 1}, {1, 1, -1}, {1, 1, 1}, {-1, 1, 1},
      {1, 1, -1}, {1, -1, 1}, {-1, 1, 1}, {1, 1, 1},
      {1, -1, 1}, {1, 1, -1}, {1, 1, 1}, {-1, 1, 1},
      {-1, 1, 1}, {1, 1, 1}, {1, 1, -1}, {1, -1, 1},
      {-1, 1, 1}, {1, 1, 1}, {1, 1, -1}, {1, -1, 1}};
  static const int Nn[48][3] = {
      {1, 1, 0}, {1, 1, 0}, {1, -1, 0}, {1, -1, 0},
      {1, 0, 1}, {1, 0, 1}, {1, 0, -1}, {1, 0, -1},
      {0, 1, 1}, {0, 1, 1}, {0, 1, -1}, {0, 1, -1},
      {1, 1, 2}, {-1, 1, 2}, {1, -1, 2}, {1, 1, -2},
      {1, 2, 1}, {-1, 2, 1}, {1, -2, 1}, {1, 2, -1},
      {2, 1, 1}, {-2, 1, 1}, {2, -1, 1}, {2, 1, -1},
      {1, 2, 3}, {-1, 2, 3}, {1, -2, 3}, {1, 2, -3},
      {1, 3, 2}, {-1, 3, 2}, {1, -3, 2}, {1, 3, -2},
      {2, 1, 3}, {-2, 1, 3}, {2, -1, 3}, {2, 1, -3},
      {2, 3, 1}, {-2, 3, 1}, {2, -3, 1}, {2, 3, -1},
      {3, 1, 2}, {-3, 1, 2}, {3, -1, 2}, {3, 1, -2},
      {3, 2, 1}, {-3, 2, 1}, {3, -2, 1}, {3, 2, -1}};
  for (int s = 0; s < 48; s++) {
    const double len = std::sqrt((double)(Nn[s][0] * Nn[s][0] + Nn[s][1] * Nn[s][1] + Nn[s][2] * Nn[s][2]));
    for (int k = 0; k < 3; k++) {
      b[s][k] = B[s][k] * (1.0 / std::sqrt(3.0));
      n[s][k] = (double)Nn[s][k] / len;
    }
  }
}
// BCC {110}<111> (slip_type 2, src/mod_crystals.f:516-593), in the reference's order and
// signs: directions +-1/sqrt(3), normals 0 or +-1/sqrt(2) per component.
void bcc_systems(double b[12][3], double n[12][3]) {
  const double f = 1.0 / std::sqrt(2.0), g = 1.0 / std::sqrt(3.0);
  const double B[12][3] = {{g, g, g},   {g, g, g},   {g, g, g},   {-g, -g, g},
                           {-g, -g, g}, {-g, -g, g}, {-g, g, g},  {-g, g, g},
                           {-g, g, g},  {g, -g, g},  {g, -g, g},  {g, -g, g}};
  const double Nn[12][3] = {{0, -f, f}, {f, 0, -f}, {-f, f, 0}, {0, f, f},
                            {f, 0, f},  {f, -f, 0}, {0, -f, f}, {-f, 0, -f},
                            {f, f, 0},  {0, f, f},  {f, 0, -f}, {-f, -f, 0}};
  for (int s = 0; s < 12; s++)
    for (int k = 0; k < 3; k++) { b[s][k] = B[s][k]; n[s][k] = Nn[s][k]; }
}
// FCC {111}<110> in Roters' order (slip_type 6 "roters", src/mod_crystals.f:604-704):
// directions 0 or +-1/sqrt(2), normals +-1/sqrt(3).
void roters_systems(double b[12][3], double n[12][3]) {
  const double f = 1.0 / std::sqrt(2.0), g = 1.0 / std::sqrt(3.0);
  const double B[12][3] = {{f, -f, 0}, {f, 0, -f}, {0, f, -f}, {f, f, 0},
                           {f, 0, f},  {0, f, -f}, {f, f, 0},  {f, 0, -f},
                           {0, f, f},  {f, -f, 0}, {f, 0, f},  {0, f, f}};
  const double Nn[12][3] = {{g, g, g},   {-g, -g, -g}, {g, g, g},   {g, -g, -g},
                            {-g, g, g},  {g, -g, -g},  {g, -g, g},  {g, -g, g},
                            {-g, g, -g}, {-g, -g, g},  {-g, -g, g}, {g, g, -g}};
  for (int s = 0; s < 12; s++)
    for (int k = 0; k < 3; k++) { b[s][k] = B[s][k]; n[s][k] = Nn[s][k]; }
}
// HCP (slip_type 9 "hcp6", src/mod_crystals.f:1208-1476): basal {0001}<11-20> systems 1-3
// and prismatic {10-10}<11-20> systems 4-6 in the reference's Cartesian frame (a1 along x,
// c along z), entries 0, +-0.5, +-1 and +-sqrt(3)/2.  slip_type 10 "hcp18" (:1477-1759)
// assigns the same six and leaves systems 7-18 (its commented-out pyramidal ones) at the
// zero of the crystal record: kept here as eighteen systems, twelve of them zero vectors.
void hcp_systems(double b[][3], double n[][3]) {
  const double r = std::sqrt(3.0) / 2.0;
  const double B[6][3] = {{0.5, -r, 0.0}, {0.5, r, 0.0}, {-1.0, 0.0, 0.0},
                          {1.0, 0.0, 0.0}, {0.5, r, 0.0}, {-0.5, r, 0.0}};
  const double Nn[6][3] = {{0.0, 0.0, 1.0}, {0.0, 0.0, 1.0}, {0.0, 0.0, 1.0},
                           {0.0, 1.0, 0.0}, {-r, 0.5, 0.0}, {-r, -0.5, 0.0}};
  for (int s = 0; s < 6; s++)
    for (int k = 0; k < 3; k++) { b[s][k] = B[s][k]; n[s][k] = Nn[s][k]; }
}
void crystal_finalize(const cpfft_crystal& p, Crys& c) {
  c.p = p;
  double b[12][3], n[12][3];
  c.ns = 12;
  std::memset(c.b, 0, sizeof(c.b));
  std::memset(c.n, 0, sizeof(c.n));
  switch (p.slip_type) {
    case 8: c.ns = 48; bcc48_systems(c.b, c.n); break;
    case 7: bcc48_systems(c.b, c.n); break;  // bcc12: bcc48's first twelve (:705-811)
    case 3:  // single (:594-603): direction x on the plane normal to y
      c.ns = 1;
      c.b[0][0] = 1.0;
      c.n[0][1] = 1.0;
      break;
    case 9: c.ns = 6; hcp_systems(c.b, c.n); break;
    case 10: c.ns = 18; hcp_systems(c.b, c.n); break;
    default:  // the 12-system tables
      if (p.slip_type == 2) bcc_systems(b, n);
      else if (p.slip_type == 6) roters_systems(b, n);
      else fcc_systems(b, n);
      std::memcpy(c.b, b, sizeof(b));
      std::memcpy(c.n, n, sizeof(n));
      break;
  }
  // the forest and parallel projections of mm10_mrr_GH's tables (mm10_mrr_GHfcc, GHbcc,
  // GHfcc12, GHbcc12, src/mm10_e.f:16-1424):
  // Gm(a,b) = |n_a . t_b|, Hm(a,b) = |n_a x t_b|, t_b = n_b x b_b the edge line direction
  for (int a = 0; a < 12; a++)
    for (int q = 0; q < 12; q++) {
      double t[3] = {c.n[q][1] * c.b[q][2] - c.n[q][2] * c.b[q][1],
                     c.n[q][2] * c.b[q][0] - c.n[q][0] * c.b[q][2],
                     c.n[q][0] * c.b[q][1] - c.n[q][1] * c.b[q][0]};
      double tl = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
      for (int k = 0; k < 3; k++) t[k] /= tl;
      const double* na = c.n[a];
      double x[3] = {na[1] * t[2] - na[2] * t[1], na[2] * t[0] - na[0] * t[2],
                     na[0] * t[1] - na[1] * t[0]};
      c.Gm[a][q] = std::fabs(na[0] * t[0] + na[1] * t[1] + na[2] * t[2]);
      c.Hm[a][q] = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    }
  std::memset(c.C0, 0, sizeof(c.C0));
  if (p.elastic_type == 3) {
    double C22 = p.C11, C23 = p.C13, C66 = p.C55;
    c.C0[0][0] = p.C11; c.C0[0][1] = p.C12; c.C0[0][2] = p.C13;
    c.C0[1][0] = p.C12; c.C0[1][1] = C22;   c.C0[1][2] = C23;
    c.C0[2][0] = p.C13; c.C0[2][1] = C23;   c.C0[2][2] = p.C33;
    c.C0[3][3] = p.C44; c.C0[4][4] = p.C55; c.C0[5][5] = C66;
  } else {
    M6 flex;
    std::memset(flex, 0, sizeof(flex));
    double e = p.e, v = p.nu;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) flex[i][j] = i == j ? 1.0 / e : -v / e;
    double sh = p.elastic_type == 1 ? 2.0 * (1.0 + v) / e : 1.0 / p.mu;
    for (int i = 3; i < 6; i++) flex[i][i] = sh;
    inv66(flex, c.C0);
  }
}

// Per-voxel orientation data: setup_mm10_rknstr (src/drive_eps_sig.f:537-1002)
struct VoxProps {
  M6 C;            // stiffness rotated to the sample frame
  int ns;          // slip systems
  double ms[48][6], qs[48][3];
  M3 g;
};
void voxel_props(const Crys& cr, const double ang[3], VoxProps& vp) {
  kocks_g(ang, vp.g);
  M3 tr;
  tr33(vp.g, tr);  // trans_rot
  vp.ns = cr.ns;
  for (int s = 0; s < cr.ns; s++) {
    double bs[3], ns[3];
    for (int i = 0; i < 3; i++) {
      bs[i] = tr[i][0] * cr.b[s][0] + tr[i][1] * cr.b[s][1] + tr[i][2] * cr.b[s][2];
      ns[i] = tr[i][0] * cr.n[s][0] + tr[i][1] * cr.n[s][1] + tr[i][2] * cr.n[s][2];
    }
    M3 A, As, Aa;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) A[i][j] = bs[i] * ns[j];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        As[i][j] = 0.5 * (A[i][j] + A[j][i]);
        Aa[i][j] = 0.5 * (A[i][j] - A[j][i]);
      }
    // mm10_et2ev / mm10_wt2wv (src/mm10_a.f:1487-1520)
    vp.ms[s][0] = As[0][0]; vp.ms[s][1] = As[1][1]; vp.ms[s][2] = As[2][2];
    vp.ms[s][3] = 2.0 * As[0][1]; vp.ms[s][4] = 2.0 * As[1][2]; vp.ms[s][5] = 2.0 * As[0][2];
    vp.qs[s][0] = Aa[1][2]; vp.qs[s][1] = Aa[0][2]; vp.qs[s][2] = Aa[0][1];
  }
  M6 Rs, tmp;
  rt2rve(tr, Rs);
  for (int i = 0; i < 6; i++)       // temp66 = C0 * Rs^T
    for (int j = 0; j < 6; j++) {
      double s = 0;
      for (int k = 0; k < 6; k++) s += cr.C0[i][k] * Rs[j][k];
      tmp[i][j] = s;
    }
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) {
      double s = 0;
      for (int k = 0; k < 6; k++) s += Rs[i][k] * tmp[k][j];
      vp.C[i][j] = s;
    }
}

// ---- mm10 (Voce, one crystal) -------------------------------------------------------
struct State {          // compact history (CPFFT_HIST_WORDS order)
  double sig[6];
  double tt;
  M3 Rp;
  double D[6];
  double tt_rate;
  double eps[6];        // unrotated strain (rstgp1_update_strains, src/rstgp1.f:1378-1394)
  // mm01 voxels (m01 set): the history vector (1-based as the reference's, [1..11]) and
  // the extra stress-vector words cgn(7:9); tt, Rp, D and tt_rate are not used
  bool m01;
  double h01[12];
  double cgx[3];
  double u[2];          // MTS: tau_y and mu of the step (mm10's u(1:2)); -1 = not yet set
  // Ma-Roters-Raabe crystals (mrr set): the twelve dislocation densities (tau_tilde(1:12))
  // and their rates, history words 31..42 and 43..54; tt and tt_rate are not used
  bool mrr;
  double rho[12], rho_rate[12];
};
void state_init(const Crys& cr, State& s) {  // mm10_init_cc_hist0 (src/mm10_a.f:473-571)
  std::memset(&s, 0, sizeof(s));
  for (int i = 0; i < 3; i++) s.Rp[i][i] = 1.0;
  s.tt = cr.p.tau_y + 1.0e-5;                // mm10_init_voche (:2046-2056)
  if (cr.p.h_type == 2) {                    // mm10_init_mts (:2090-2107): flags
    s.tt = -1.0;
    s.u[0] = s.u[1] = -1.0;
  }
  if (cr.p.h_type == 7 || cr.p.h_type == 4) {  // mm10_init_mrr / _ornl (:2205-2223, 2286-2304)
    s.mrr = true;
    s.tt = 0.0;
    for (int i = 0; i < 12; i++) s.rho[i] = cr.p.theta_0 == 0.0 ? 1.0e8 : cr.p.theta_0;
  }
}
void state_pack(const State& s, double* h) {
  if (s.m01) {  // words 6..16 history, 17..19 cgn(7:9), 20..22 zero
    for (int i = 0; i < ORC_HIST; i++) h[i] = 0.0;
    for (int i = 0; i < 6; i++) h[i] = s.sig[i];
    for (int k = 1; k <= 11; k++) h[5 + k] = s.h01[k];
    for (int k = 0; k < 3; k++) h[17 + k] = s.cgx[k];
    for (int i = 0; i < 6; i++) h[23 + i] = s.eps[i];
    return;
  }
  for (int i = 0; i < 6; i++) h[i] = s.sig[i];
  h[6] = s.tt;
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) h[7 + 3 * j + i] = s.Rp[i][j];  // column-major
  for (int i = 0; i < 6; i++) h[16 + i] = s.D[i];
  h[22] = s.tt_rate;
  for (int i = 0; i < 6; i++) h[23 + i] = s.eps[i];
  h[29] = s.u[0];
  h[30] = s.u[1];
  if (s.mrr)
    for (int i = 0; i < 12; i++) {
      h[ORC_HIST + i] = s.rho[i];
      h[ORC_HIST + 12 + i] = s.rho_rate[i];
    }
}
void state_unpack(const double* h, State& s) {
  if (s.m01) {
    for (int i = 0; i < 6; i++) s.sig[i] = h[i];
    s.h01[0] = 0.0;
    for (int k = 1; k <= 11; k++) s.h01[k] = h[5 + k];
    for (int k = 0; k < 3; k++) s.cgx[k] = h[17 + k];
    for (int i = 0; i < 6; i++) s.eps[i] = h[23 + i];
    return;
  }
  for (int i = 0; i < 6; i++) s.sig[i] = h[i];
  s.tt = h[6];
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) s.Rp[i][j] = h[7 + 3 * j + i];
  for (int i = 0; i < 6; i++) s.D[i] = h[16 + i];
  s.tt_rate = h[22];
  for (int i = 0; i < 6; i++) s.eps[i] = h[23 + i];
  s.u[0] = h[29];
  s.u[1] = h[30];
  if (s.mrr)
    for (int i = 0; i < 12; i++) {
      s.rho[i] = h[ORC_HIST + i];
      s.rho_rate[i] = h[ORC_HIST + 12 + i];
    }
}

// the np1 / curr "crystal_state" pieces the Voce routines read
struct Np1 {
  double D[6];
  double tinc, dg;
  double ms[48][6], qs[48][3], qc[48][3];
  double tt_rate;
  double temp, mu, tau_y, tau_v, ntau_y, nmu;  // MTS
  double rho_rate[12];                          // MRR: rates of the twelve densities
};

// mm10_setup_mts's shear modulus and thresholds (src/mm10_a.f:2109-2150) at rate dgc, T
void mts_thresholds(const cpfft_crystal& p, double dgc, double T, double& mu, double& tau_v,
                    double& tau_y) {
  if (T == 0.0) mu = p.mu_0;
  else mu = p.mu_0 - p.D_0 / (std::exp(p.T_0 / T) - 1.0);
  if (dgc == 0.0) {
    tau_v = p.tau_hat_v;
    tau_y = p.tau_hat_y;
  } else {
    tau_v = p.tau_hat_v * std::pow(1.0 - std::pow(p.boltzman * T / (mu * std::pow(p.burgers, 3.0) *
                                   p.G_0_v) * std::log(p.eps_dot_0_v / dgc), 1.0 / p.q_v), 1.0 / p.p_v);
    tau_y = p.tau_hat_y * std::pow(1.0 - std::pow(p.boltzman * T / (mu * std::pow(p.burgers, 3.0) *
                                   p.G_0_y) * std::log(p.gamma_bar / dgc), 1.0 / p.q_y), 1.0 / p.p_y);
  }
}
const double TEMP = 297.0;  // gp_temps of drive_10_update (src/rstgp1.f:832)

struct Mm10 {
  const cpfft_crystal* p;
  const VoxProps* vp;
  const State* n;

  // mm10_setup (src/mm10_a.f:830-975) + mm10_setup_voche (:2058-2080)
  bool mts() const { return p->h_type == 2; }
  double iDv() const { return mts() ? 0.0 : p->iD_v; }  // MTS has no diffusion term
  void setup(Np1& s, const double D[6], double tinc, const M3 R, double T = TEMP) const {
    for (int i = 0; i < 6; i++) s.D[i] = D[i];
    s.tinc = tinc;
    double t1 = D[0] * D[0] + D[1] * D[1] + D[2] * D[2];
    double t2 = D[3] * D[3] + D[4] * D[4] + D[5] * D[5];
    s.dg = std::sqrt((2.0 / 3.0) * (t1 + 0.5 * t2));
    M3 tnRp, RW, work, RWC;
    tr33(n->Rp, tnRp);
    M6 RE;
    rt2rve(tnRp, RE);
    rt2rvw(tnRp, RW);
    mm33(R, tnRp, work);
    rt2rvw(work, RWC);
    for (int i = 0; i < vp->ns; i++) {
      mv6(RE, vp->ms[i], s.ms[i]);
      for (int a = 0; a < 3; a++) {
        s.qs[i][a] = RW[a][0] * vp->qs[i][0] + RW[a][1] * vp->qs[i][1] + RW[a][2] * vp->qs[i][2];
        s.qc[i][a] = RWC[a][0] * vp->qs[i][0] + RWC[a][1] * vp->qs[i][1] + RWC[a][2] * vp->qs[i][2];
      }
    }
    if (p->alter_mode && !mts()) s.dg = p->gamma_bar * s.tinc;  // mm10_setup_voche only
    s.tt_rate = 0.0;
    s.temp = T;
    if (mts()) {  // mm10_setup_mts: n's tau_y and mu from the history's u, else this step's
      mts_thresholds(*p, s.dg / s.tinc, T, s.mu, s.tau_v, s.tau_y);
      s.ntau_y = n->u[0] < 0.0 ? s.tau_y : n->u[0];
      s.nmu = n->u[1] < 0.0 ? s.mu : n->u[1];
    }
  }
  double rs(const Np1& s, const double* st, int i) const {  // mm10_rs (src/mm10_b.f:1831)
    return st[0] * s.ms[i][0] + st[1] * s.ms[i][1] + st[2] * s.ms[i][2] +
           st[3] * s.ms[i][3] + st[4] * s.ms[i][4] + st[5] * s.ms[i][5];
  }
  double slipinc(const Np1& s, const double* st, double tt, int i) const {  // :1805-1820
    double r = rs(s, st, i);
    return s.dg / tt * std::pow(std::fabs(r / tt), p->harden_n - 1.0) * r;
  }
  double hterm(double tt) const {  // Voce h_term with tau_l = 0 (gradFeinv is zeroed)
    return 1.0 - (tt - p->tau_y) / p->tau_v + 0.0 / (tt - p->tau_y);
  }
  // symmetric part of S*W in the reference's vector forms (mm10_symsw :1505-1525)
  static void symsw(const double* s, const double* w, double* sw) {
    sw[0] = s[3] * w[2] - s[5] * w[1];
    sw[1] = s[3] * w[2] - s[4] * w[0];
    sw[2] = s[5] * w[1] + s[4] * w[0];
    sw[3] = 0.5 * (w[2] * (s[0] - s[1]) + w[0] * s[5] - w[1] * s[4]);
    sw[4] = 0.5 * (w[0] * (s[1] - s[2]) + w[1] * s[3] + w[2] * s[5]);
    sw[5] = 0.5 * (w[1] * (s[0] - s[2]) + w[0] * s[3] - w[2] * s[4]);
  }
  void form_wp(const Np1& s, const double* st, double tt, double w[3]) const {
    w[0] = w[1] = w[2] = 0.0;
    for (int i = 0; i < vp->ns; i++) {  // mm10_form_wp (src/mm10_b.f:1304-1381)
      double si = slipinc(s, st, tt, i);
      for (int a = 0; a < 3; a++) w[a] = w[a] + si * s.qc[i][a];
      double r = rs(s, st, i);
      for (int a = 0; a < 3; a++) w[a] = w[a] + r * s.tinc * iDv() * s.qc[i][a];
    }
  }
  // mm10_formR1 (src/mm10_b.f:1061-1101)
  void formR1(const Np1& s, const double* st, double tt, double R1[6]) const {
    double dbar[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < vp->ns; i++) {  // mm10_form_dbarp voce (:1161-1190)
      double si = slipinc(s, st, tt, i);
      double r = rs(s, st, i);
      double f = r * s.tinc * iDv() + si;
      for (int a = 0; a < 6; a++) dbar[a] = dbar[a] + f * s.ms[i][a];
    }
    double w[3], sw[6], wv1[6], wv2[6];
    form_wp(s, st, tt, w);
    symsw(st, w, sw);
    for (int a = 0; a < 6; a++) wv1[a] = s.D[a] - dbar[a];
    mv6(vp->C, wv1, wv2);
    for (int a = 0; a < 6; a++) R1[a] = st[a] - n->sig[a] - wv2[a] + 2.0 * sw[a];
  }
  // mm10_h_voche (src/mm10_b.f:1888-1912)
  double h_voce(const Np1& s, const double* st, double tt) const {
    double h = 0.0;
    for (int i = 0; i < vp->ns; i++) {
      double si = slipinc(s, st, tt, i);
      double ht = hterm(tt);
      h = h + std::pow(std::fabs(ht), p->voce_m) * sgn1(ht) * std::fabs(si);
    }
    return n->tt + p->theta_0 * h;
  }
  // mm10_h_mts (src/mm10_b.f:2080-2108), tau_l = 0
  double h_mts(const Np1& s, const double* st, double tt) const {
    double cta = (p->mu_0 / s.mu) * tt - (p->mu_0 / s.mu) * p->tau_a - s.tau_y;
    double ct = 1.0 - cta / s.tau_v;
    double h = 0.0;
    for (int i = 0; i < vp->ns; i++)
      h = h + std::pow(ct + 0.0 / cta, p->voce_m) * std::fabs(slipinc(s, st, tt, i));
    return p->tau_a * (1.0 - s.mu / s.nmu) + (s.mu / p->mu_0) * (s.tau_y - s.ntau_y) +
           (s.mu / s.nmu) * n->tt + p->theta_0 * (s.mu / p->mu_0) * h;
  }
  // mm10_formR (src/mm10_b.f:1029-1047) with mm10_formR2 (:63-113)
  void formR(Np1& s, const double* x, double R[7]) const {
    formR1(s, x, x[6], R);
    double h = mts() ? h_mts(s, x, x[6]) : h_voce(s, x, x[6]);
    R[6] = x[6] - h;
    s.tt_rate = (h - n->tt) / s.tinc;
  }
  // mm10_formJ11 (src/mm10_b.f:177-257)
  void formJ11(const Np1& s, const double* st, double tt, double J[6][6]) const {
    double sq[48][6];
    for (int i = 0; i < vp->ns; i++) symsw(st, s.qc[i], sq[i]);
    std::memset(J, 0, 36 * sizeof(double));
    for (int i = 0; i < vp->ns; i++) {
      double r = rs(s, st, i);
      double dgdt = std::pow(std::fabs(r), p->harden_n - 1.0);
      dgdt = s.dg * p->harden_n / std::pow(tt, p->harden_n) * dgdt;
      dgdt = dgdt + s.tinc * iDv();
      double wv[6];
      for (int a = 0; a < 6; a++) wv[a] = 2.0 * sq[i][a];
      for (int j = 0; j < 6; j++)
        for (int a = 0; a < 6; a++) wv[a] = wv[a] + vp->C[a][j] * s.ms[i][j];
      for (int c = 0; c < 6; c++) {
        double t = dgdt * s.ms[i][c];
        for (int a = 0; a < 6; a++) J[a][c] += wv[a] * t;
      }
    }
    double w[3];
    form_wp(s, st, tt, w);
    double iw[6][6];
    std::memset(iw, 0, sizeof(iw));  // mm10_iw (src/mm10_b.f:1590-1634)
    iw[0][3] = 2.0 * w[2];  iw[0][5] = -2.0 * w[1];
    iw[1][3] = 2.0 * w[2];  iw[1][4] = -2.0 * w[0];
    iw[2][4] = 2.0 * w[0];  iw[2][5] = 2.0 * w[1];
    iw[3][0] = w[2];  iw[3][1] = -w[2]; iw[3][4] = -w[1]; iw[3][5] = w[0];
    iw[4][1] = w[0];  iw[4][2] = -w[0]; iw[4][3] = w[1];  iw[4][5] = w[2];
    iw[5][0] = w[1];  iw[5][2] = -w[1]; iw[5][3] = w[0];  iw[5][4] = -w[2];
    for (int a = 0; a < 6; a++)
      for (int c = 0; c < 6; c++) J[a][c] = J[a][c] + iw[a][c];
    for (int a = 0; a < 6; a++) J[a][a] = J[a][a] + 1.0;
  }
  // mm10_formJ (src/mm10_b.f:901-954): J11 | J12 ; J21 | J22
  void formJ(const Np1& s, const double* x, double J[7][7]) const {
    const double* st = x;
    double tt = x[6];
    double J11[6][6];
    formJ11(s, st, tt, J11);
    double sq[48][6];
    for (int i = 0; i < vp->ns; i++) symsw(st, s.qc[i], sq[i]);
    double J12[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < vp->ns; i++) {  // mm10_formJ12 + mm10_dgdh_voche (:271-353, 2012-2030)
      double dgam = slipinc(s, st, tt, i);
      double dgdtt = -p->harden_n / tt * dgam;
      double tm[6];
      for (int a = 0; a < 6; a++) tm[a] = 2.0 * sq[i][a];
      for (int j = 0; j < 6; j++)
        for (int a = 0; a < 6; a++) tm[a] = tm[a] + vp->C[a][j] * s.ms[i][j];
      for (int a = 0; a < 6; a++) J12[a] += tm[a] * dgdtt;
    }
    if (mts()) {  // mm10_estress_mts / mm10_ehard_mts (:2110-2187)
      double cta = (p->mu_0 / s.mu) * tt - (p->mu_0 / s.mu) * p->tau_a - s.tau_y;
      double ct = 1.0 - cta / s.tau_v;
      double et[6] = {0, 0, 0, 0, 0, 0};
      for (int i = 0; i < vp->ns; i++) {
        double r = rs(s, st, i);
        double f = std::pow(ct + 0.0 / cta, p->voce_m) * std::pow(std::fabs(r), p->harden_n - 2.0) * r;
        for (int a = 0; a < 6; a++) et[a] = et[a] + f * s.ms[i][a];
      }
      for (int a = 0; a < 6; a++)
        et[a] = p->theta_0 * (s.mu / p->mu_0) * et[a] * p->harden_n * s.dg / std::pow(tt, p->harden_n);
      double ur = s.mu / p->mu_0, etau = 0.0;
      for (int i = 0; i < vp->ns; i++) {
        double si = slipinc(s, st, tt, i);
        etau = etau + (p->voce_m * (1.0 / s.tau_v + 0.0 / (cta * cta)) *
                       std::pow(ct + 0.0 / cta, -1.0) + ur * p->harden_n / tt) *
                      std::pow(ct + 0.0 / cta, p->voce_m) * std::fabs(si);
      }
      etau = -p->theta_0 * etau;
      etau = 1.0 - etau;
      for (int a = 0; a < 6; a++) {
        for (int c = 0; c < 6; c++) J[a][c] = J11[a][c];
        J[a][6] = J12[a];
        J[6][a] = -et[a];
      }
      J[6][6] = etau;
      return;
    }
    double et[6] = {0, 0, 0, 0, 0, 0};  // mm10_estress_voche (:1914-1940)
    for (int i = 0; i < vp->ns; i++) {
      double r = rs(s, st, i);
      double ht = hterm(tt);
      double f = std::pow(std::fabs(ht), p->voce_m) * sgn1(ht) *
                 std::pow(std::fabs(r), p->harden_n - 2.0) * r;
      for (int a = 0; a < 6; a++) et[a] = et[a] + f * s.ms[i][a];
    }
    double fac = p->theta_0 * s.dg * p->harden_n / std::pow(tt, p->harden_n);
    double etau = 0.0;  // mm10_ehard_voche (:1942-1968)
    for (int i = 0; i < vp->ns; i++) {
      double si = slipinc(s, st, tt, i);
      double ht = hterm(tt);
      double a = p->voce_m * (-1.0 / p->tau_v - 0.0 / ((tt - p->tau_y) * (tt - p->tau_y))) *
                 std::fabs(si) / std::fabs(ht);
      double b = std::fabs(si) * p->harden_n / tt * sgn1(ht);
      if (!p->exact_j22) b = b * sgn1(si);  // the reference's extra factor
      etau = etau + (a - b) * std::pow(std::fabs(ht), p->voce_m);
    }
    etau = p->theta_0 * etau;
    etau = 1.0 - etau;
    for (int a = 0; a < 6; a++) {
      for (int c = 0; c < 6; c++) J[a][c] = J11[a][c];
      J[a][6] = J12[a];
      J[6][a] = -(fac * et[a]);
    }
    J[6][6] = etau;
  }

  // mm10_tangent's JA + JB for MTS (src/mm10_a.f:711-800; mm10_ed_mts, mm10_dgdd_mts,
  // src/mm10_b.f:2189-2378), subtracted from JR = C.  mm10_a_mult_type_4 is handed the
  // whole symtqmat array, so every system's term reads system 1's column.
  void mts_tangent_rhs(const Np1& s, const double* st, double tt, const double J[7][7],
                       double* JR) const {
    double d_mod[6] = {s.D[0], s.D[1], s.D[2], 0.5 * s.D[3], 0.5 * s.D[4], 0.5 * s.D[5]};
    double symtq1[6];
    symsw(st, s.qc[0], symtq1);
    double alpha = 2.0 / (3.0 * s.dg * s.dg);
    double JA[6][6];
    std::memset(JA, 0, sizeof(JA));
    for (int i = 0; i < vp->ns; i++) {
      double dgam = slipinc(s, st, tt, i);
      double work[6];
      for (int a = 0; a < 6; a++) {
        work[a] = 2.0 * symtq1[a];
        for (int j = 0; j < 6; j++) work[a] = work[a] + vp->C[a][j] * s.ms[i][j];
      }
      for (int a = 0; a < 6; a++)
        for (int b = 0; b < 6; b++) JA[a][b] = JA[a][b] + work[a] * (alpha * dgam * d_mod[b]);
    }
    // mm10_ed_mts
    double dgc = s.dg / s.tinc;
    double lny = std::log(p->gamma_bar / dgc);
    double ty = p->boltzman * s.temp / (s.mu * std::pow(p->burgers, 3.0) * p->G_0_y) * lny;
    double dydd[6], dvdd[6];
    double fy = 2.0 * p->tau_hat_y / (3.0 * s.dg * s.dg * p->q_y * p->p_y * lny) *
                std::pow(1.0 - std::pow(ty, 1.0 / p->q_y), 1.0 / p->p_y - 1.0) *
                std::pow(ty, 1.0 / p->q_y);
    double lnv = std::log(p->eps_dot_0_v / dgc);
    double tv = p->boltzman * s.temp / (s.mu * std::pow(p->burgers, 3.0) * p->G_0_v) * lnv;
    double fv = 2.0 * p->tau_hat_v / (3.0 * s.dg * s.dg * p->q_v * p->p_v * lnv) *
                std::pow(1.0 - std::pow(tv, 1.0 / p->q_v), 1.0 / p->p_v - 1.0) *
                std::pow(tv, 1.0 / p->q_v);
    for (int a = 0; a < 6; a++) { dydd[a] = fy * d_mod[a]; dvdd[a] = fv * d_mod[a]; }
    double mnp0 = s.mu / p->mu_0;
    double sc = tt / mnp0 - p->tau_a / mnp0 - s.tau_y;
    double ed[6] = {0, 0, 0, 0, 0, 0};
    for (int i = 0; i < vp->ns; i++) {
      double asi = std::fabs(slipinc(s, st, tt, i));
      double base = 1.0 - sc / s.tau_v + 0.0 / sc;
      for (int a = 0; a < 6; a++)
        ed[a] = ed[a] + (p->voce_m * (1.0 / s.tau_v + 0.0 / (sc * sc)) *
                             std::pow(base, p->voce_m - 1.0) * dydd[a] +
                         p->voce_m / (s.tau_v * s.tau_v) * sc * std::pow(base, p->voce_m - 1.0) * dvdd[a] +
                         2.0 / (3.0 * s.dg * s.dg) * std::pow(base, p->voce_m) * d_mod[a]) * asi;
    }
    for (int a = 0; a < 6; a++) ed[a] = p->theta_0 * mnp0 * ed[a] + mnp0 * dydd[a];
    // JB = J12 (J22^-1 ed)
    for (int a = 0; a < 6; a++)
      for (int b = 0; b < 6; b++)
        JR[a * 6 + b] = JR[a * 6 + b] - JA[a][b] - J[a][6] * (ed[b] / J[6][6]);
  }

  struct Result {
    double sig[6], tt, tt_rate;
    double J[7][7];   // last Jacobian formed by the update phase
    bool have_J;
    int iters;        // update-phase Newton iterations (summed over sub-steps)
  };

  // mm10_solve (src/mm10_a.f:2860-3295); returns false on failure
  bool solve(Np1& cu, double dtinc, double stress[6], double& tt, Result& res) const {
    const double c = 1.0e-4, red = 0.5;
    const int mls = 10, mmin = 1;
    double x[7];
    for (int i = 0; i < 6; i++) x[i] = stress[i];
    x[6] = tt;
    // ---- predict (:2975-3156)
    double inR1;
    {
      int iter = 0;
      double x1[6], x2;
      for (int i = 0; i < 6; i++) x1[i] = x[i];
      double d1[6], d2[6];
      for (int i = 0; i < 6; i++) { d1[i] = cu.D[i]; d2[i] = n->D[i]; }
      for (double* d : {d1, d2}) {
        double dtr = (d[0] + d[1] + d[2]) / 3.0;
        d[0] -= dtr; d[1] -= dtr; d[2] -= dtr;
        double t1 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        double t2 = d[3] * d[3] + d[4] * d[4] + d[5] * d[5];
        if (t1 + t2 == 0.0) for (int i = 0; i < 6; i++) d[i] = 0.0;
        else { double nn = std::sqrt(t1 + t2); for (int i = 0; i < 6; i++) d[i] = d[i] / nn; }
      }
      double t1 = d1[0] * d2[0] + d1[1] * d2[1] + d1[2] * d2[2];
      double t2 = d1[3] * d2[3] + d1[4] * d2[4] + d1[5] * d2[5];
      double cos_ang = std::max(t1 + t2, 0.0);
      x2 = x[6] + cos_ang * n->tt_rate * dtinc;
      double R1[6];
      formR1(cu, x1, x2, R1);
      double nR1 = std::sqrt(R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2] + R1[3] * R1[3] +
                             R1[4] * R1[4] + R1[5] * R1[5]);
      inR1 = nR1;
#ifdef ORC_DEBUG
      fprintf(stderr, "  predict start nR1 %.3e x2 %.6f\n", nR1, x2);
#endif
      while (nR1 > p->atol1 && nR1 / inR1 > p->rtol1) {
        double J11[6][6];
        formJ11(cu, x1, x2, J11);
        double mJ[36], dx1[6];
        for (int a = 0; a < 6; a++)
          for (int b = 0; b < 6; b++) mJ[a * 6 + b] = -J11[a][b];
        for (int a = 0; a < 6; a++) dx1[a] = R1[a];
        lu_solve(6, mJ, 1, dx1);
        double alpha = 1.0;
        double dotR1 = R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2] + R1[3] * R1[3] +
                       R1[4] * R1[4] + R1[5] * R1[5];
        double ls1 = 0.5 * dotR1;
        double wv[6];
        for (int a = 0; a < 6; a++) {
          wv[a] = 0.0;
          for (int b = 0; b < 6; b++) wv[a] += J11[b][a] * R1[b];
        }
        double ls2 = c * (dx1[0] * wv[0] + dx1[1] * wv[1] + dx1[2] * wv[2] + dx1[3] * wv[3] +
                          dx1[4] * wv[4] + dx1[5] * wv[5]);
        int ls = 0;
        for (;;) {
          double nlsx = ls1 + ls2 * alpha;
          double xn[6];
          for (int a = 0; a < 6; a++) xn[a] = x1[a] + alpha * dx1[a];
          formR1(cu, xn, x2, R1);
          dotR1 = R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2] + R1[3] * R1[3] +
                  R1[4] * R1[4] + R1[5] * R1[5];
          nR1 = std::sqrt(dotR1);
          double nRs = 0.5 * dotR1;
          if (nRs <= nlsx || ls > mls) {
            for (int a = 0; a < 6; a++) x1[a] = xn[a];
            break;
          }
          alpha = red * alpha;
          ls++;
        }
        iter++;
#ifdef ORC_DEBUG
        fprintf(stderr, "  predict it %d nR1 %.3e ls %d\n", iter, nR1, ls);
#endif
        bool nan = false;
        for (int a = 0; a < 6; a++) nan |= std::isnan(x1[a]);
        if (iter > p->miter || nan) return false;
      }
      for (int i = 0; i < 6; i++) x[i] = x1[i];
      x[6] = x2;
    }
    // ---- update (:3162-3293)
    int iter = 0;
    double R[7];
    formR(cu, x, R);
    double dotR = 0;
    for (int a = 0; a < 7; a++) dotR += R[a] * R[a];
    double nR = std::sqrt(dotR), inR = nR;
    if (inR == 0.0) inR = inR1;
    while ((nR > p->atol && nR / inR > p->rtol) || iter < mmin) {
      formJ(cu, x, res.J);
      res.have_J = true;
      double mJ[49], dx[7];
      for (int a = 0; a < 7; a++)
        for (int b = 0; b < 7; b++) mJ[a * 7 + b] = -res.J[a][b];
      for (int a = 0; a < 7; a++) dx[a] = R[a];
      lu_solve(7, mJ, 1, dx);
      double alpha = 1.0;
      dotR = 0;
      for (int a = 0; a < 7; a++) dotR += R[a] * R[a];
      double ls1 = 0.5 * dotR;
      double wv[7];
      for (int a = 0; a < 7; a++) {
        wv[a] = 0.0;
        for (int b = 0; b < 7; b++) wv[a] += res.J[b][a] * R[b];
      }
      double ls2 = 0;
      for (int a = 0; a < 7; a++) ls2 += dx[a] * wv[a];
      ls2 = c * ls2;
      int ls = 0;
      for (;;) {
        double nlsx = ls1 + ls2 * alpha;
        double xn[7];
        for (int a = 0; a < 7; a++) xn[a] = x[a] + alpha * dx[a];
        formR(cu, xn, R);
        dotR = 0;
        for (int a = 0; a < 7; a++) dotR += R[a] * R[a];
        nR = std::sqrt(dotR);
        double nRs = 0.5 * dotR;
        if (nRs <= nlsx || ls > mls) {
          for (int a = 0; a < 7; a++) x[a] = xn[a];
          break;
        }
        alpha = red * alpha;
        ls++;
      }
      iter++;
#ifdef ORC_DEBUG
      fprintf(stderr, "  update it %d nR %.3e inR %.3e ls %d tt %.6f\n", iter, nR, inR, ls, x[6]);
#endif
      bool nan = false;
      for (int a = 0; a < 7; a++) nan |= std::isnan(x[a]);
      if (iter > p->miter || nan) { res.iters += iter; return false; }
    }
    res.iters += iter;
    for (int i = 0; i < 6; i++) stress[i] = x[i];
    tt = x[6];
    return true;
  }

  // mm10_solve_strup + mm10_solve_crystal (src/mm10_a.f:2628-2845, 1080-1157).
  // Returns false when the local solve failed (the reference then keeps sigma_n).
  bool update(const double D[6], double dt, const M3 R, bool iter0, State& out,
              double cep[6][6], int* local_iters) const {
    Np1 np1;
    setup(np1, D, dt, R);
    out.u[0] = mts() ? np1.tau_y : 0.0;  // the history's u(1:2) (mm10_setup_mts)
    out.u[1] = mts() ? np1.mu : 0.0;
    double stress[6], ostress[6], tt = n->tt, ott = n->tt;
    for (int i = 0; i < 6; i++) stress[i] = ostress[i] = n->sig[i];
    double temp1 = 0, temp2 = 0;
    for (int i = 0; i < 6; i++) { temp1 += D[i] * D[i]; temp2 += stress[i] * stress[i]; }
    bool no_load = temp2 == 0.0 && temp1 == 0.0;
    Result res;
    res.have_J = false;
    res.iters = 0;
    double tt_rate_out = 0.0;
    bool ok = true;
    if (iter0 || no_load) {  // mm10_solve_strup_a (:2721-2743)
      for (int a = 0; a < 6; a++)
        for (int b = 0; b < 6; b++) cep[a][b] = vp->C[a][b];
      if (!no_load) {
        double R1[6];
        formR1(np1, stress, tt, R1);
        for (int a = 0; a < 6; a++) stress[a] = stress[a] - R1[a];
      }
      tt_rate_out = 0.0;
    } else {  // mm10_solve_strup_iterate (:2747-2843)
      double frac = 0.0, step = 1.0;
      int cuts = 0;
      const int mcuts = 4;
      Np1 curr;
      bool fail = false;
      while (frac < 1.0) {
        double Dw[6];
        for (int i = 0; i < 6; i++) Dw[i] = np1.D[i] * (step + frac);
        // n's temperature is zero: the sub-step's scales with it (:2769)
        setup(curr, Dw, np1.tinc * (step + frac), R, TEMP * (step + frac));
        tt = n->tt;
        fail = !solve(curr, np1.tinc * step, stress, tt, res);
        if (fail) {
          for (int i = 0; i < 6; i++) stress[i] = ostress[i];
          tt = ott;
          step = step * 0.5;
          cuts++;
          if (cuts > mcuts) break;
          fail = false;
        } else {
          for (int i = 0; i < 6; i++) ostress[i] = stress[i];
          ott = tt;
          frac = frac + step;
        }
      }
      bool nan = std::isnan(tt);
      for (int i = 0; i < 6; i++) nan |= std::isnan(stress[i]);
      if (fail || nan) ok = false;
      tt_rate_out = curr.tt_rate;
    }
    if (local_iters) *local_iters = res.iters;
    if (!ok) {
      // Reference: material_cut_step is raised and never checked by the FFT driver
      // (src/mm10_a.f:2806-2841).  Keep sigma_n / tau_n and the elastic tangent.
      for (int i = 0; i < 6; i++) out.sig[i] = n->sig[i];
      out.tt = n->tt;
      out.tt_rate = 0.0;
      for (int i = 0; i < 6; i++) out.D[i] = D[i];
      std::memcpy(out.Rp, n->Rp, sizeof(M3));
      for (int a = 0; a < 6; a++)
        for (int b = 0; b < 6; b++) cep[a][b] = vp->C[a][b];
      return false;
    }
    for (int i = 0; i < 6; i++) out.sig[i] = stress[i];
    out.tt = tt;
    out.tt_rate = tt_rate_out;
    for (int i = 0; i < 6; i++) out.D[i] = D[i];
    if (iter0 || no_load) {
      // early return of mm10_solve_crystal: np1%Rp keeps the zero of mm10_setup_np1
      std::memset(out.Rp, 0, sizeof(M3));
      return true;
    }
    // mm10_tangent (src/mm10_a.f:658-815) for Voce: JA = JB = 0, JR = C
    {
      double J22 = res.J[6][6];
      double JJ[36], JR[36];
      for (int a = 0; a < 6; a++)
        for (int b = 0; b < 6; b++) {
          double beta = res.J[6][b] / J22;
          JJ[a * 6 + b] = res.J[a][b] - res.J[a][6] * beta;
          JR[a * 6 + b] = vp->C[a][b];
        }
      if (mts()) mts_tangent_rhs(np1, out.sig, out.tt, res.J, JR);
      lu_solve(6, JJ, 6, JR);
      for (int a = 0; a < 6; a++)  // mm10_a_make_symm_1
        for (int b = 0; b < 6; b++) cep[a][b] = (JR[a * 6 + b] + JR[b * 6 + a]) * 0.5;
    }
    // mm10_update_rotation (src/mm10_a.f:3310-3327) with np1 at the converged x
    {
      double wb[3] = {0, 0, 0};
      for (int i = 0; i < vp->ns; i++) {  // mm10_form_wbarp (src/mm10_b.f:1231-1290)
        double si = slipinc(np1, out.sig, out.tt, i);
        for (int a = 0; a < 3; a++) wb[a] = wb[a] + si * np1.qs[i][a];
        double r = rs(np1, out.sig, i);
        for (int a = 0; a < 3; a++) wb[a] = wb[a] + r * np1.tinc * p->iD_v * np1.qs[i][a];
      }
      M3 W = {{0.0, wb[2], wb[1]}, {-wb[2], 0.0, wb[0]}, {-wb[1], -wb[0], 0.0}};
      M3 ex;  // mm10_expmw3x3 (:3360-3385)
      double alpha = std::sqrt(W[1][2] * W[1][2] + W[0][2] * W[0][2] + W[0][1] * W[0][1]);
      if (alpha < 1.0e-16) {
        std::memset(ex, 0, sizeof(ex));
      } else {
        M3 WW;
        mm33(W, W, WW);
        double ca = (1.0 - std::cos(alpha)) / (alpha * alpha), sa = std::sin(alpha) / alpha;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) ex[i][j] = ca * WW[i][j] + sa * W[i][j];
      }
      for (int i = 0; i < 3; i++) ex[i][i] += 1.0;
      mm33(ex, n->Rp, out.Rp);
    }
    return true;
  }
};

// ---- Ma-Roters-Raabe hardening (h_type 7), FCC, one density per slip system --------
// mm10_slipinc_mrr .. mm10_dgdd_mrr (src/mm10_b.f:2343-3325), the (6 + 12)-unknown
// mm10_solve (src/mm10_a.f:2860-3295) and mm10_tangent (:658-815) with ed = dgammadd = 0
// (mm10_ed_mrr, mm10_dgdd_mrr).  exact_j22 = 0 forms the local Jacobian with the
// reference's formulas, which do not all differentiate its residual: estress / ehard use
// sqrt(rho_F) where mm10_h_mrr has sqrt(rho_P) (src/mm10_b.f:2635, 2952, 3075), the
// estress "badterm" lacks the sign of tau, and the extrapolated branch of dgdt / dgdh
// (fract > 1) drops terms.  exact_j22 = 1 differentiates the residual exactly.
const int MRR_NH = 12;
struct Mrr {
  const cpfft_crystal* p;
  const VoxProps* vp;
  const State* n;
  const double (*Gm)[12];   // rho_F = Gm rho  (mm10_mrr_GH)
  const double (*Hm)[12];   // rho_P = Hm rho

  // mm10_setup (src/mm10_a.f:830-975) with mm10_setup_mrr (:2225-2240: time only)
  void setup(Np1& s, const double D[6], double tinc, const M3 R, double T) const {
    for (int i = 0; i < 6; i++) s.D[i] = D[i];
    s.tinc = tinc;
    s.dg = 0.0;
    M3 tnRp, RW, work, RWC;
    tr33(n->Rp, tnRp);
    M6 RE;
    rt2rve(tnRp, RE);
    rt2rvw(tnRp, RW);
    mm33(R, tnRp, work);
    rt2rvw(work, RWC);
    for (int i = 0; i < vp->ns; i++) {
      mv6(RE, vp->ms[i], s.ms[i]);
      for (int a = 0; a < 3; a++) {
        s.qs[i][a] = RW[a][0] * vp->qs[i][0] + RW[a][1] * vp->qs[i][1] + RW[a][2] * vp->qs[i][2];
        s.qc[i][a] = RWC[a][0] * vp->qs[i][0] + RWC[a][1] * vp->qs[i][1] + RWC[a][2] * vp->qs[i][2];
      }
    }
    s.temp = T;
  }
  double rs(const Np1& s, const double* st, int i) const {
    return st[0] * s.ms[i][0] + st[1] * s.ms[i][1] + st[2] * s.ms[i][2] +
           st[3] * s.ms[i][3] + st[4] * s.ms[i][4] + st[5] * s.ms[i][5];
  }
  // the quantities of system a at (st, tt) that every MRR routine forms
  struct Sys {
    double rs, rhoF, rhoP, g0, tpass, tcut, fract, slip;
  };
  bool ornl() const { return p->h_type == 4; }
  // shear modulus: MRR's constant mu_0; ORNL's mu(T) = mu_0 - D_0 / (exp(T_0 / T) - 1)
  double shear(const Np1& s) const {
    return ornl() ? p->mu_0 - p->D_0 / (std::exp(p->T_0 / s.temp) - 1.0) : p->mu_0;
  }
  // ORNL's attack frequency (G_0_y; exp(-G_0_y) when negative)
  double vs() const { return p->G_0_y < 0.0 ? std::exp(-p->G_0_y) : p->G_0_y; }
  // the slip-law exponent p: ORNL takes 1 below the passing stress (fract < 0)
  double pexp(double fract) const { return ornl() && fract < 0.0 ? 1.0 : p->p_v; }
  void sys(const Np1& s, const double* st, const double* tt, int a, Sys& y) const {
    const double k = p->boltzman, th = s.temp, G = shear(s), b = p->burgers;
    y.rs = rs(s, st, a);
    y.rhoF = 0.0;
    y.rhoP = 0.0;
    for (int q = 0; q < MRR_NH; q++) {
      y.rhoF += Gm[a][q] * tt[q];
      y.rhoP += Hm[a][q] * tt[q];
    }
    if (ornl()) {  // mm10_slipinc_ornl (src/mm10_b.f:3457-3540): mobile density 0.1 rho_a
      y.g0 = 0.1 * tt[a] * b * vs() / b * (p->u2 * b);
      y.tpass = p->u1 * G * b * std::sqrt(y.rhoP);
      y.tcut = p->u3 * G / p->mu_0;
    } else {
      y.g0 = p->G_0_y * k * th / (p->u1 * p->u3 * G * b * b) * std::sqrt(y.rhoP);   // (15)
      y.tpass = p->u1 * G * b * std::sqrt(y.rhoP);                                 // (16)
      y.tcut = p->G_0_v / (p->u2 * p->u3 * b * b) * std::sqrt(y.rhoF);             // (17)
    }
    y.fract = (std::fabs(y.rs) - y.tpass) / y.tcut;
    // mm10_slipinc_mrr (src/mm10_b.f:2477-2546)
    const double Qk = p->G_0_v / k / th;
    if (y.fract > 1.0) {  // linear extrapolation past fract = 1
      double m = y.g0 * (-p->q_v * Qk) * (-p->p_v) * sgn1(y.rs) / y.tcut;
      y.slip = s.tinc * (m * y.fract + y.g0);
    } else if (std::fabs(y.rs) > 0.0) {
      y.slip = s.tinc * y.g0 * sgn1(y.rs) *
               std::exp(-Qk * std::pow(1.0 - std::pow(y.fract, pexp(y.fract)), p->q_v));  // (14)
    } else {
      y.slip = 0.0;
    }
  }
  // d slip / d rs (mm10_dgdt_mrr, src/mm10_b.f:3111-3198)
  double dgdt(const Np1& s, const Sys& y) const {
    const double Qk = p->G_0_v / p->boltzman / s.temp;
    const double dfract = sgn1(y.rs) / y.tcut;
    if (y.fract > 1.0) {
      double m = y.g0 * (-p->q_v * Qk) * (-p->p_v) * sgn1(y.rs) / y.tcut;
      return p->exact_j22 ? s.tinc * m * dfract : s.tinc * m;
    }
    if (std::fabs(y.rs) > 0.0) {
      const double pe = pexp(y.fract);
      double slipexp = std::exp(-Qk * std::pow(1.0 - std::pow(y.fract, pe), p->q_v)) * sgn1(y.rs);
      return s.tinc * (-y.g0 * slipexp * Qk * p->q_v *
                       std::pow(1.0 - std::pow(y.fract, pe), p->q_v - 1.0) * (-1.0) * pe *
                       std::pow(y.fract, pe - 1.0) * dfract);
    }
    return 0.0;
  }
  // d slip_a / d rho_c (mm10_dgdh_mrr, src/mm10_b.f:3201-3306)
  // (ORNL: mm10_dgdh_ornl, :4224-4347: the rate prefactor depends on rho_a alone, the
  // cutting stress on no density)
  double dgdh(const Np1& s, const Sys& y, int a, int c) const {
    const double k = p->boltzman, th = s.temp, G = shear(s), b = p->burgers;
    const double Qk = p->G_0_v / k / th;
    const double drhoF = Gm[a][c], drhoP = Hm[a][c];
    const double dg0 = ornl() ? (a == c ? 0.1 : 0.0) * b * vs() / b * (p->u2 * b)
                              : 0.5 * p->G_0_y * k * th / (p->u1 * p->u3 * G * b * b) /
                                    std::sqrt(y.rhoP) * drhoP;
    const double dtpass = 0.5 * p->u1 * G * b / std::sqrt(y.rhoP) * drhoP;
    const double dtcut = ornl() ? 0.0 : 0.5 * p->G_0_v / (p->u2 * p->u3 * b * b) / std::sqrt(y.rhoF) * drhoF;
    const double dfract = ((-dtpass) * y.tcut - (std::fabs(y.rs) - y.tpass) * dtcut) / (y.tcut * y.tcut);
    if (y.fract > 1.0) {
      double K = (-p->q_v * Qk) * (-p->p_v) * sgn1(y.rs);
      double dm = K * (dg0 / y.tcut - y.g0 * dtcut / (y.tcut * y.tcut));
      if (!p->exact_j22) return s.tinc * dm;
      double m = y.g0 * K / y.tcut;
      return s.tinc * (dm * y.fract + m * dfract + dg0);
    }
    if (std::fabs(y.rs) > 0.0) {
      const double pe = pexp(y.fract);
      double slipexp = std::exp(-Qk * std::pow(1.0 - std::pow(y.fract, pe), p->q_v));
      return s.tinc * (dg0 * slipexp * sgn1(y.rs) +
                       y.g0 * sgn1(y.rs) * slipexp * (-1.0) * Qk * p->q_v *
                           std::pow(1.0 - std::pow(y.fract, pe), p->q_v - 1.0) * (-1.0) *
                           pe * std::pow(y.fract, pe - 1.0) * dfract);
    }
    return 0.0;
  }
  // R1 (mm10_formR1, src/mm10_b.f:1061-1101) with dbarp / wp of the MRR slips
  void formR1(const Np1& s, const double* st, const double* tt, double R1[6]) const {
    double dbar[6] = {0, 0, 0, 0, 0, 0}, w[3] = {0, 0, 0};
    for (int i = 0; i < vp->ns; i++) {
      Sys y;
      sys(s, st, tt, i, y);
      for (int a = 0; a < 6; a++) dbar[a] = dbar[a] + y.slip * s.ms[i][a];
      for (int a = 0; a < 3; a++) w[a] = w[a] + y.slip * s.qc[i][a];
    }
    double sw[6], wv1[6], wv2[6];
    Mm10::symsw(st, w, sw);
    for (int a = 0; a < 6; a++) wv1[a] = s.D[a] - dbar[a];
    mv6(vp->C, wv1, wv2);
    for (int a = 0; a < 6; a++) R1[a] = st[a] - n->sig[a] - wv2[a] + 2.0 * sw[a];
  }
  // mm10_h_mrr (src/mm10_b.f:2549-2646) and R2 = tt - h (mm10_formR2, :63-113)
  void formR2(Np1& s, const double* st, const double* tt, double* R2) const {
    const double k = p->boltzman, th = s.temp, G = shear(s), b = p->burgers, v = 0.3;
    for (int a = 0; a < MRR_NH; a++) {
      Sys y;
      sys(s, st, tt, a, y);
      const double rho = tt[a], rho_n = n->rho[a];
      const double ddip = std::sqrt(3.0) * G * b / (16.0 * PI * (1.0 - v)) / std::fabs(y.rs);  // (42)
      const double rhoM = (2.0 * k / (p->u1 * p->u2 * p->u3 * G * b * b * b)) * th *
                          std::sqrt(y.rhoF * y.rhoP);                                       // (13)
      const double gd = std::fabs(y.slip / s.tinc);
      const double tem1 = p->u4 / b * std::sqrt(y.rhoP) * gd;
      const double tem2 = p->u6 * ddip / b * rhoM * gd;
      const double tem3 = p->u5 * rho * gd;
      const double tem4 = p->tau_hat_y * std::exp(-p->tau_a / k / th) * std::fabs(y.rs) / (k * th) *
                          rho * rho * std::pow(gd, p->tau_hat_v);
      const double h = rho_n + s.tinc * (tem1 + tem2 - tem3 - tem4);                       // (18)
      R2[a] = tt[a] - h;
      s.rho_rate[a] = (h - rho_n) / s.tinc;
    }
  }
  void formR(Np1& s, const double* x, double* R) const {
    formR1(s, x, x + 6, R);
    formR2(s, x, x + 6, R + 6);
  }
  // J11 (mm10_formJ11, src/mm10_b.f:177-257) with mm10_dgdt_mrr
  void formJ11(const Np1& s, const double* st, const double* tt, double J[6][6]) const {
    std::memset(J, 0, 36 * sizeof(double));
    double w[3] = {0, 0, 0};
    for (int i = 0; i < vp->ns; i++) {
      Sys y;
      sys(s, st, tt, i, y);
      const double dg = dgdt(s, y);
      double sq[6], wv[6];
      Mm10::symsw(st, s.qc[i], sq);
      for (int a = 0; a < 6; a++) wv[a] = 2.0 * sq[a];
      for (int j = 0; j < 6; j++)
        for (int a = 0; a < 6; a++) wv[a] = wv[a] + vp->C[a][j] * s.ms[i][j];
      for (int c = 0; c < 6; c++) {
        double t = dg * s.ms[i][c];
        for (int a = 0; a < 6; a++) J[a][c] += wv[a] * t;
      }
      for (int a = 0; a < 3; a++) w[a] = w[a] + y.slip * s.qc[i][a];  // mm10_form_wp
    }
    double iw[6][6];
    std::memset(iw, 0, sizeof(iw));  // mm10_iw (src/mm10_b.f:1590-1634)
    iw[0][3] = 2.0 * w[2];  iw[0][5] = -2.0 * w[1];
    iw[1][3] = 2.0 * w[2];  iw[1][4] = -2.0 * w[0];
    iw[2][4] = 2.0 * w[0];  iw[2][5] = 2.0 * w[1];
    iw[3][0] = w[2];  iw[3][1] = -w[2]; iw[3][4] = -w[1]; iw[3][5] = w[0];
    iw[4][1] = w[0];  iw[4][2] = -w[0]; iw[4][3] = w[1];  iw[4][5] = w[2];
    iw[5][0] = w[1];  iw[5][2] = -w[1]; iw[5][3] = w[0];  iw[5][4] = -w[2];
    for (int a = 0; a < 6; a++)
      for (int c = 0; c < 6; c++) J[a][c] = J[a][c] + iw[a][c];
    for (int a = 0; a < 6; a++) J[a][a] = J[a][a] + 1.0;
  }
  // the (6 + 12)^2 Jacobian (mm10_formJ, src/mm10_b.f:901-954), row-major J[18*r + c]:
  // J12 (mm10_formJ12 with mm10_dgdh_mrr), J21 = -estress (mm10_estress_mrr,
  // src/mm10_b.f:2859-2963), J22 = ehard (mm10_ehard_mrr, :2966-3092)
  void formJ(const Np1& s, const double* x, double* J) const {
    const int L = 6 + MRR_NH;
    const double* st = x;
    const double* tt = x + 6;
    double J11[6][6];
    formJ11(s, st, tt, J11);
    for (int a = 0; a < 6; a++)
      for (int c = 0; c < 6; c++) J[L * a + c] = J11[a][c];
    Sys ys[MRR_NH];
    double dgt[MRR_NH];
    for (int a = 0; a < MRR_NH; a++) {
      sys(s, st, tt, a, ys[a]);
      dgt[a] = dgdt(s, ys[a]);
    }
    // J12
    for (int a = 0; a < 6; a++)
      for (int c = 0; c < MRR_NH; c++) J[L * a + 6 + c] = 0.0;
    for (int i = 0; i < vp->ns; i++) {
      double sq[6], tm[6];
      Mm10::symsw(st, s.qc[i], sq);
      for (int a = 0; a < 6; a++) tm[a] = 2.0 * sq[a];
      for (int j = 0; j < 6; j++)
        for (int a = 0; a < 6; a++) tm[a] = tm[a] + vp->C[a][j] * s.ms[i][j];
      for (int c = 0; c < MRR_NH; c++) {
        double d = dgdh(s, ys[i], i, c);
        for (int a = 0; a < 6; a++) J[L * a + 6 + c] += tm[a] * d;
      }
    }
    // J21, J22
    const double k = p->boltzman, th = s.temp, G = shear(s), b = p->burgers, v = 0.3;
    const double dt = s.tinc;
    const double cdip = std::sqrt(3.0) * G * b / (16.0 * PI * (1.0 - v));
    const double cM = 2.0 * k / (p->u1 * p->u2 * p->u3 * G * b * b * b) * th;
    const double E = p->tau_hat_y * std::exp(-p->tau_a / k / th) / (k * th);
    const double c8 = p->tau_hat_v;
    for (int a = 0; a < MRR_NH; a++) {
      const Sys& y = ys[a];
      const double rho = tt[a], sg = sgn1(y.rs), ars = std::fabs(y.rs);
      const double ddip = cdip / ars;
      const double dddip = -cdip / (ars * ars) * sg;
      const double rhoM = cM * std::sqrt(y.rhoF * y.rhoP);
      const double gd = std::fabs(y.slip / dt);
      const double dsl = dgt[a] / dt;
      double et;
      if (!p->exact_j22) {
        double bad = gd == 0.0 ? 0.0 : c8 * ars * std::pow(gd, c8 - 1.0) * dsl;
        et = dt * (p->u4 / b * std::sqrt(y.rhoF) * sg * dsl +
                   p->u6 / b * rhoM * (ddip * sg * dsl + dddip * gd) - p->u5 * rho * sg * dsl -
                   E * rho * rho * (bad + sg * std::pow(gd, c8)));
      } else {
        const double sgd = sgn1(y.slip);  // d|slip| = sign(slip) d slip
        const double dgd = sgd * dsl;     // d gd / d rs
        double bad = gd == 0.0 ? 0.0 : c8 * ars * std::pow(gd, c8 - 1.0) * dgd;
        et = dt * (p->u4 / b * std::sqrt(y.rhoP) * dgd +
                   p->u6 / b * rhoM * (ddip * dgd + dddip * gd) - p->u5 * rho * dgd -
                   E * rho * rho * (bad + sg * std::pow(gd, c8)));
      }
      for (int c = 0; c < 6; c++) J[L * (6 + a) + c] = -et * s.ms[a][c];
      for (int c = 0; c < MRR_NH; c++) {
        const double drhoF = Gm[a][c], drhoP = Hm[a][c];
        const double drhoM = 0.5 * cM / std::sqrt(y.rhoF * y.rhoP) * (drhoF * y.rhoP + y.rhoF * drhoP);
        const double d = a == c ? 1.0 : 0.0;
        const double dsh = dgdh(s, y, a, c) / dt;
        double e;
        if (!p->exact_j22) {
          double bad = gd == 0.0 ? 0.0 : c8 * std::pow(gd, c8 - 1.0) * dsh;
          e = d - dt * (p->u4 / b * (0.5 * drhoF / std::sqrt(y.rhoF) * gd * sg + std::sqrt(y.rhoF) * dsh) +
                        p->u6 / b * (rhoM * ddip * dsh + drhoM * ddip * gd * sg) -
                        p->u5 * (rho * dsh + d * gd * sg) -
                        E * ars * (rho * rho * bad + 2.0 * rho * sg * d * std::pow(gd, c8))) * sg;
        } else {
          const double dgd = sgn1(y.slip) * dsh;
          double bad = gd == 0.0 ? 0.0 : c8 * std::pow(gd, c8 - 1.0) * dgd;
          e = d - dt * (p->u4 / b * (0.5 * drhoP / std::sqrt(y.rhoP) * gd + std::sqrt(y.rhoP) * dgd) +
                        p->u6 / b * ddip * (rhoM * dgd + drhoM * gd) - p->u5 * (rho * dgd + d * gd) -
                        E * ars * (rho * rho * bad + 2.0 * rho * d * std::pow(gd, c8)));
        }
        J[L * (6 + a) + 6 + c] = e;
      }
    }
  }

  // mm10_solve (src/mm10_a.f:2860-3295) for 6 + 12 unknowns; Jl: the last Jacobian
  bool solve(Np1& cu, double dtinc, double stress[6], double* tt, double* Jl, bool& haveJ,
             int& iters) const {
    const int L = 6 + MRR_NH;
    const double c = 1.0e-4, red = 0.5;
    const int mls = 10, mmin = 1;
    double x[6 + MRR_NH];
    for (int i = 0; i < 6; i++) x[i] = stress[i];
    for (int i = 0; i < MRR_NH; i++) x[6 + i] = tt[i];
    double inR1;
    {  // predict (:2975-3156): R1 Newton with the densities extrapolated
      int iter = 0;
      double x1[6], x2[MRR_NH];
      for (int i = 0; i < 6; i++) x1[i] = x[i];
      double d1[6], d2[6];
      for (int i = 0; i < 6; i++) { d1[i] = cu.D[i]; d2[i] = n->D[i]; }
      for (double* d : {d1, d2}) {
        double dtr = (d[0] + d[1] + d[2]) / 3.0;
        d[0] -= dtr; d[1] -= dtr; d[2] -= dtr;
        double t1 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        double t2 = d[3] * d[3] + d[4] * d[4] + d[5] * d[5];
        if (t1 + t2 == 0.0) for (int i = 0; i < 6; i++) d[i] = 0.0;
        else { double nn = std::sqrt(t1 + t2); for (int i = 0; i < 6; i++) d[i] = d[i] / nn; }
      }
      double t1 = d1[0] * d2[0] + d1[1] * d2[1] + d1[2] * d2[2];
      double t2 = d1[3] * d2[3] + d1[4] * d2[4] + d1[5] * d2[5];
      double cos_ang = std::max(t1 + t2, 0.0);
      for (int i = 0; i < MRR_NH; i++) x2[i] = x[6 + i] + cos_ang * n->rho_rate[i] * dtinc;
      double R1[6];
      formR1(cu, x1, x2, R1);
      double nR1 = std::sqrt(R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2] + R1[3] * R1[3] +
                             R1[4] * R1[4] + R1[5] * R1[5]);
      inR1 = nR1;
      while (nR1 > p->atol1 && nR1 / inR1 > p->rtol1) {
        double J11[6][6];
        formJ11(cu, x1, x2, J11);
        double mJ[36], dx1[6];
        for (int a = 0; a < 6; a++)
          for (int b = 0; b < 6; b++) mJ[a * 6 + b] = -J11[a][b];
        for (int a = 0; a < 6; a++) dx1[a] = R1[a];
        lu_solve(6, mJ, 1, dx1);
        double alpha = 1.0;
        double dotR1 = 0;
        for (int a = 0; a < 6; a++) dotR1 += R1[a] * R1[a];
        double ls1 = 0.5 * dotR1, wv[6], ls2 = 0;
        for (int a = 0; a < 6; a++) {
          wv[a] = 0.0;
          for (int b = 0; b < 6; b++) wv[a] += J11[b][a] * R1[b];
        }
        for (int a = 0; a < 6; a++) ls2 += dx1[a] * wv[a];
        ls2 = c * ls2;
        int ls = 0;
        for (;;) {
          double nlsx = ls1 + ls2 * alpha;
          double xn[6];
          for (int a = 0; a < 6; a++) xn[a] = x1[a] + alpha * dx1[a];
          formR1(cu, xn, x2, R1);
          dotR1 = 0;
          for (int a = 0; a < 6; a++) dotR1 += R1[a] * R1[a];
          nR1 = std::sqrt(dotR1);
          if (0.5 * dotR1 <= nlsx || ls > mls) {
            for (int a = 0; a < 6; a++) x1[a] = xn[a];
            break;
          }
          alpha = red * alpha;
          ls++;
        }
        iter++;
        bool nan = false;
        for (int a = 0; a < 6; a++) nan |= std::isnan(x1[a]);
        if (iter > p->miter || nan) return false;
      }
      for (int i = 0; i < 6; i++) x[i] = x1[i];
      for (int i = 0; i < MRR_NH; i++) x[6 + i] = x2[i];
    }
    // update (:3162-3293)
    int iter = 0;
    double R[6 + MRR_NH];
    formR(cu, x, R);
    double dotR = 0;
    for (int a = 0; a < L; a++) dotR += R[a] * R[a];
    double nR = std::sqrt(dotR), inR = nR;
    if (inR == 0.0) inR = inR1;
    while ((nR > p->atol && nR / inR > p->rtol) || iter < mmin) {
      formJ(cu, x, Jl);
      haveJ = true;
      double mJ[L * L], dx[L];
      for (int a = 0; a < L * L; a++) mJ[a] = -Jl[a];
      for (int a = 0; a < L; a++) dx[a] = R[a];
      lu_solve(L, mJ, 1, dx);
      double alpha = 1.0;
      dotR = 0;
      for (int a = 0; a < L; a++) dotR += R[a] * R[a];
      double ls1 = 0.5 * dotR, ls2 = 0;
      for (int a = 0; a < L; a++) {
        double w = 0.0;
        for (int b = 0; b < L; b++) w += Jl[L * b + a] * R[b];
        ls2 += dx[a] * w;
      }
      ls2 = c * ls2;
      int ls = 0;
      for (;;) {
        double nlsx = ls1 + ls2 * alpha;
        double xn[L];
        for (int a = 0; a < L; a++) xn[a] = x[a] + alpha * dx[a];
        formR(cu, xn, R);
        dotR = 0;
        for (int a = 0; a < L; a++) dotR += R[a] * R[a];
        nR = std::sqrt(dotR);
        if (0.5 * dotR <= nlsx || ls > mls) {
          for (int a = 0; a < L; a++) x[a] = xn[a];
          break;
        }
        alpha = red * alpha;
        ls++;
      }
      iter++;
      bool nan = false;
      for (int a = 0; a < L; a++) nan |= std::isnan(x[a]);
      if (iter > p->miter || nan) { iters += iter; return false; }
    }
    iters += iter;
    for (int i = 0; i < 6; i++) stress[i] = x[i];
    for (int i = 0; i < MRR_NH; i++) tt[i] = x[6 + i];
    return true;
  }

  // mm10_solve_strup + mm10_solve_crystal (src/mm10_a.f:2628-2845, 1080-1157)
  bool update(const double D[6], double dt, const M3 R, bool iter0, State& out,
              double cep[6][6], int* local_iters) const {
    const int L = 6 + MRR_NH;
    Np1 np1;
    setup(np1, D, dt, R, TEMP);
    double stress[6], ostress[6], tt[MRR_NH], ott[MRR_NH], rate[MRR_NH];
    for (int i = 0; i < 6; i++) stress[i] = ostress[i] = n->sig[i];
    for (int i = 0; i < MRR_NH; i++) { tt[i] = ott[i] = n->rho[i]; rate[i] = 0.0; }
    double temp1 = 0, temp2 = 0;
    for (int i = 0; i < 6; i++) { temp1 += D[i] * D[i]; temp2 += stress[i] * stress[i]; }
    const bool no_load = temp2 == 0.0 && temp1 == 0.0;
    double Jl[L * L];
    bool haveJ = false;
    int iters = 0;
    bool ok = true;
    if (iter0 || no_load) {  // mm10_solve_strup_a (:2721-2743)
      for (int a = 0; a < 6; a++)
        for (int b = 0; b < 6; b++) cep[a][b] = vp->C[a][b];
      if (!no_load) {
        double R1[6];
        formR1(np1, stress, tt, R1);
        for (int a = 0; a < 6; a++) stress[a] = stress[a] - R1[a];
      }
    } else {  // mm10_solve_strup_iterate (:2747-2843)
      double frac = 0.0, step = 1.0;
      int cuts = 0;
      Np1 curr;
      bool fail = false;
      while (frac < 1.0) {
        double Dw[6];
        for (int i = 0; i < 6; i++) Dw[i] = np1.D[i] * (step + frac);
        setup(curr, Dw, np1.tinc * (step + frac), R, TEMP * (step + frac));
        for (int i = 0; i < MRR_NH; i++) tt[i] = n->rho[i];
        fail = !solve(curr, np1.tinc * step, stress, tt, Jl, haveJ, iters);
        if (fail) {
          for (int i = 0; i < 6; i++) stress[i] = ostress[i];
          for (int i = 0; i < MRR_NH; i++) tt[i] = ott[i];
          step = step * 0.5;
          if (++cuts > 4) break;
          fail = false;
        } else {
          for (int i = 0; i < 6; i++) ostress[i] = stress[i];
          for (int i = 0; i < MRR_NH; i++) ott[i] = tt[i];
          frac = frac + step;
          for (int i = 0; i < MRR_NH; i++) rate[i] = curr.rho_rate[i];
        }
      }
      bool nan = false;
      for (int i = 0; i < 6; i++) nan |= std::isnan(stress[i]);
      for (int i = 0; i < MRR_NH; i++) nan |= std::isnan(tt[i]);
      if (fail || nan) ok = false;
    }
    if (local_iters) *local_iters = iters;
    for (int i = 0; i < 6; i++) out.D[i] = D[i];
    out.tt = 0.0;
    out.tt_rate = 0.0;
    out.u[0] = out.u[1] = 0.0;
    if (!ok) {  // keep sigma_n / rho_n and the elastic tangent (see Mm10::update)
      for (int i = 0; i < 6; i++) out.sig[i] = n->sig[i];
      for (int i = 0; i < MRR_NH; i++) { out.rho[i] = n->rho[i]; out.rho_rate[i] = 0.0; }
      std::memcpy(out.Rp, n->Rp, sizeof(M3));
      for (int a = 0; a < 6; a++)
        for (int b = 0; b < 6; b++) cep[a][b] = vp->C[a][b];
      return false;
    }
    for (int i = 0; i < 6; i++) out.sig[i] = stress[i];
    for (int i = 0; i < MRR_NH; i++) { out.rho[i] = tt[i]; out.rho_rate[i] = rate[i]; }
    if (iter0 || no_load) {
      std::memset(out.Rp, 0, sizeof(M3));
      return true;
    }
    // mm10_tangent (:658-815): T = (J11 - J12 J22^-1 J21)^-1 C (ed = dgammadd = 0)
    {
      double A22[MRR_NH * MRR_NH], B[MRR_NH * 6];
      for (int a = 0; a < MRR_NH; a++) {
        for (int c = 0; c < MRR_NH; c++) A22[MRR_NH * a + c] = Jl[L * (6 + a) + 6 + c];
        for (int c = 0; c < 6; c++) B[6 * a + c] = Jl[L * (6 + a) + c];
      }
      lu_solve(MRR_NH, A22, 6, B);  // beta = J22^-1 J21
      double JJ[36], JR[36];
      for (int a = 0; a < 6; a++)
        for (int c = 0; c < 6; c++) {
          double s = Jl[L * a + c];
          for (int q = 0; q < MRR_NH; q++) s -= Jl[L * a + 6 + q] * B[6 * q + c];
          JJ[6 * a + c] = s;
          JR[6 * a + c] = vp->C[a][c];
        }
      lu_solve(6, JJ, 6, JR);
      for (int a = 0; a < 6; a++)
        for (int b = 0; b < 6; b++) cep[a][b] = (JR[a * 6 + b] + JR[b * 6 + a]) * 0.5;
    }
    // mm10_update_rotation (:3310-3327): wbarp of the full step's slips at the solution
    {
      double wb[3] = {0, 0, 0};
      for (int i = 0; i < vp->ns; i++) {
        Sys y;
        sys(np1, out.sig, out.rho, i, y);
        for (int a = 0; a < 3; a++) wb[a] = wb[a] + y.slip * np1.qs[i][a];
      }
      M3 W = {{0.0, wb[2], wb[1]}, {-wb[2], 0.0, wb[0]}, {-wb[1], -wb[0], 0.0}};
      M3 ex;
      double al = std::sqrt(W[1][2] * W[1][2] + W[0][2] * W[0][2] + W[0][1] * W[0][1]);
      if (al < 1.0e-16) {
        std::memset(ex, 0, sizeof(ex));
      } else {
        M3 WW;
        mm33(W, W, WW);
        double ca = (1.0 - std::cos(al)) / (al * al), sa = std::sin(al) / al;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) ex[i][j] = ca * WW[i][j] + sa * W[i][j];
      }
      for (int i = 0; i < 3; i++) ex[i][i] += 1.0;
      mm33(ex, n->Rp, out.Rp);
    }
    return true;
  }
};

// ---- cep2A (src/cep2A.f:86-284) ------------------------------------------------------
inline int I4(int i, int j, int k, int l) { return i * 27 + j * 9 + k * 3 + l; }
void cep2A(const M3 Fn, const M3 t, const double C[6][6], const M3 Rh, const M3 fnhinv,
           const M3 R, const M3 Fn1, const M3 finv, double detFn1, double dPdF[81]) {
  M3 transR, U, Y, temp, sigma, Uinv, t_Uinv, R_t, RY, RYR, RtRF, dJdF;
  tr33(R, transR);
  mm33(transR, Fn1, U);
  double trU = U[0][0] + U[1][1] + U[2][2];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Y[i][j] = (i == j ? trU : 0.0) - U[i][j];
  mm33(R, t, temp);
  mm33(temp, transR, sigma);
  mm33(finv, R, Uinv);
  mm33(t, Uinv, t_Uinv);
  mm33(R, t, R_t);
  mm33(R, Y, RY);
  mm33(RY, transR, RYR);
  double detY_1 = 1.0 / det33(Y);
  mm33(R_t, Uinv, RtRF);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) dJdF[i][j] = finv[j][i] * detFn1;
  M3 dFn, Fnh, transRh, Uh, Yh, RYRh, RYh, FpFinv, L33, D2;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      dFn[i][j] = Fn1[i][j] - Fn[i][j];
      Fnh[i][j] = 0.5 * (Fn1[i][j] + Fn[i][j]);
    }
  tr33(Rh, transRh);
  mm33(transRh, Fnh, Uh);
  double trUh = Uh[0][0] + Uh[1][1] + Uh[2][2];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Yh[i][j] = (i == j ? trUh : 0.0) - Uh[i][j];
  mm33(Rh, Yh, temp);
  mm33(temp, transRh, RYRh);
  double detYh_1 = 1.0 / det33(Yh);
  mm33(Rh, Yh, RYh);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) FpFinv[i][j] = 0.5 * fnhinv[i][j];
  mm33(dFn, FpFinv, L33);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) D2[i][j] = L33[i][j] + L33[j][i];
  const int iv[9] = {0, 3, 5, 3, 1, 4, 5, 4, 2};
  double cep99[9][9];
  for (int a = 0; a < 9; a++)
    for (int b = 0; b < 9; b++) cep99[a][b] = C[iv[a]][iv[b]];
  double dRdF[81], dRhdF[81], dLdF[81];
  for (int m = 0; m < 81; m++) {
    int i = m / 27, j = (m / 9) % 3, k = (m / 3) % 3, l = m % 3;
    dRdF[m] = detY_1 * (RYR[i][k] * Y[l][j] - RY[i][l] * RY[k][j]);
    dRhdF[m] = detYh_1 * (RYRh[i][k] * Yh[l][j] - RYh[i][l] * RYh[k][j]);
    dRhdF[m] = dRhdF[m] * 0.5;
    dLdF[m] = -L33[i][k] * FpFinv[l][j];
    if (i == k) dLdF[m] = dLdF[m] + FpFinv[l][j];
  }
  double dtdF[81], d1[81], d2[81], d3[81];
  for (int a = 0; a < 81; a++) {
    int i = a / 27, j = (a / 9) % 3, p = (a / 3) % 3, q = a % 3;
    double s1 = 0, s2 = 0, s3 = 0;
    for (int m = 0; m < 3; m++)
      for (int n = 0; n < 3; n++) {
        s1 = s1 + dRhdF[I4(m, i, p, q)] * D2[m][n] * Rh[n][j];
        s2 = s2 + Rh[m][i] * dLdF[I4(m, n, p, q)] * Rh[n][j];
        s2 = s2 + Rh[m][i] * dLdF[I4(n, m, p, q)] * Rh[n][j];
        s3 = s3 + Rh[m][i] * D2[m][n] * dRhdF[I4(n, j, p, q)];
      }
    d1[a] = s1; d2[a] = s2; d3[a] = s3;
  }
  double dt1[81];
  for (int a = 0; a < 81; a++) dt1[a] = d1[a] + d2[a] + d3[a];
  // cep2A_ddot44 (src/cep2A.f:319-339): column-major walk of the 9x9 cep99
  const int off[9] = {0, 27, 54, 9, 36, 63, 18, 45, 72};
  for (int ii = 0; ii < 9; ii++)
    for (int jj = 0; jj < 9; jj++) {
      double s = 0;
      for (int r = 0; r < 9; r++) s += cep99[r][ii] * dt1[off[r] + jj];
      dtdF[ii * 9 + jj] = s;
    }
  for (int pp = 0; pp < 81; pp++) {
    int i = pp / 27, j = (pp / 9) % 3, k = (pp / 3) % 3, l = pp % 3;
    double P0 = RtRF[i][j] * dJdF[k][l], P1 = 0, P2 = 0, P3 = 0, P4 = 0;
    for (int m = 0; m < 3; m++) {
      P1 = P1 - detFn1 * sigma[i][m] * finv[j][k] * finv[l][m];
      P2 = P2 + detFn1 * dRdF[I4(i, m, k, l)] * t_Uinv[m][j];
      for (int n = 0; n < 3; n++) {
        P3 = P3 + detFn1 * R[i][m] * dtdF[I4(m, n, k, l)] * Uinv[n][j];
        P4 = P4 + detFn1 * R_t[i][m] * dRdF[I4(n, m, k, l)] * finv[j][n];
      }
    }
    dPdF[pp] = P0 + P1 + P2 + P3 + P4;
  }
}

// ---- one material point: do_nleps_block body (src/drive_eps_sig.f:200-325) ----------
struct PointOut {
  double P[9], A[81], sig[6], cep[6][6];
  int iters;
  bool ok;
};
struct Kin {
  M3 rnh, rn1, fnhinv;
  double uddt[6];
};
void kinematics(const M3 Fn, const M3 Fn1, Kin& k) {
  M3 fnh, dfn;
  M3& rnh = k.rnh;
  M3& rn1 = k.rn1;
  M3& fnhinv = k.fnhinv;
  double* uddt = k.uddt;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      fnh[i][j] = 0.5 * (Fn[i][j] + Fn1[i][j]);
      dfn[i][j] = Fn1[i][j] - Fn[i][j];
    }
  polar_R(fnh, rnh);
  polar_R(Fn1, rn1);
  inv33(fnh, fnhinv);
  // mul33 (src/drive_eps_sig.f:1110-1170): ddt = sym(dfn * fnhinv), engineering shear
  double ddt[6];
  {
    const M3& A = dfn;
    const M3& B = fnhinv;
    ddt[0] = A[0][0] * B[0][0] + A[0][1] * B[1][0] + A[0][2] * B[2][0];
    ddt[3] = A[1][0] * B[0][0] + A[1][1] * B[1][0] + A[1][2] * B[2][0] + A[0][0] * B[0][1] +
             A[0][1] * B[1][1] + A[0][2] * B[2][1];
    ddt[5] = A[2][0] * B[0][0] + A[2][1] * B[1][0] + A[2][2] * B[2][0] + A[0][0] * B[0][2] +
             A[0][1] * B[1][2] + A[0][2] * B[2][2];
    ddt[1] = A[1][0] * B[0][1] + A[1][1] * B[1][1] + A[1][2] * B[2][1];
    ddt[4] = A[2][0] * B[0][1] + A[2][1] * B[1][1] + A[2][2] * B[2][1] + A[1][0] * B[0][2] +
             A[1][1] * B[1][2] + A[1][2] * B[2][2];
    ddt[2] = A[2][0] * B[0][2] + A[2][1] * B[1][2] + A[2][2] * B[2][2];
  }
  M6 qnh;
  getrm1_opt1(rnh, qnh);
  for (int j = 0; j < 6; j++)  // qmply1 (src/qmply1.f:15-49)
    uddt[j] = qnh[j][0] * ddt[0] + qnh[j][1] * ddt[1] + qnh[j][2] * ddt[2] +
              qnh[j][3] * ddt[3] + qnh[j][4] * ddt[4] + qnh[j][5] * ddt[5];
}

void pull_back(const M3 Fn, const M3 Fn1, const Kin& k, const State& np1, PointOut& o);

void material_point(const Crys& cr, const VoxProps& vp, double dt, int step, int iter,
                    const M3 Fn, const M3 Fn1, const State& n_in, State& np1, PointOut& o) {
  State n = n_in;
  if (step == 1) state_init(cr, n);  // mm10 re-initialises history at step 1 (:78-83)
  Kin k;
  kinematics(Fn, Fn1, k);
  if (cr.p.h_type == 2 && n.tt < 0.0) {
    // mm10_setup_mts with the full step sets tau_tilde at n on the first step (:2167-2171)
    const double* d = k.uddt;
    double dg = std::sqrt((2.0 / 3.0) * (d[0] * d[0] + d[1] * d[1] + d[2] * d[2] +
                                         0.5 * (d[3] * d[3] + d[4] * d[4] + d[5] * d[5])));
    double mu, tv, ty;
    mts_thresholds(cr.p, dg / dt, TEMP, mu, tv, ty);
    n.tt = cr.p.tau_a + (mu / cr.p.mu_0) * ty + 0.1;
  }
  int it = 0;
  if (cr.p.h_type == 7 || cr.p.h_type == 4) {
    Mrr mm{&cr.p, &vp, &n, cr.Gm, cr.Hm};
    o.ok = mm.update(k.uddt, dt, k.rn1, iter == 0, np1, o.cep, &it);
    np1.mrr = true;
  } else {
    Mm10 mm{&cr.p, &vp, &n};
    o.ok = mm.update(k.uddt, dt, k.rn1, iter == 0, np1, o.cep, &it);
    np1.mrr = false;
  }
  np1.m01 = false;
  o.iters = it;
  // strains at n+1 = strains at n + uddt (src/drive_eps_sig.f:264-265)
  for (int i = 0; i < 6; i++) np1.eps[i] = n.eps[i] + k.uddt[i];
  pull_back(Fn, Fn1, k, np1, o);
}

void pull_back(const M3 Fn, const M3 Fn1, const Kin& k, const State& np1, PointOut& o) {
  const M3& rnh = k.rnh;
  const M3& rn1 = k.rn1;
  const M3& fnhinv = k.fnhinv;
  M3 fn1inv;
  for (int i = 0; i < 6; i++) o.sig[i] = np1.sig[i];
  // Cauchy stress T = R t R^T (getrm1 opt 2 + qmply1), P = J T F^-T (cs2p :1182-1224)
  M6 qt;
  rt2rve(rn1, qt);
  double cs[6];
  for (int j = 0; j < 6; j++)
    cs[j] = qt[j][0] * np1.sig[0] + qt[j][1] * np1.sig[1] + qt[j][2] * np1.sig[2] +
            qt[j][3] * np1.sig[3] + qt[j][4] * np1.sig[4] + qt[j][5] * np1.sig[5];
  double detF = inv33(Fn1, fn1inv);
  const M3& fi = fn1inv;
  o.P[0] = detF * (cs[0] * fi[0][0] + cs[3] * fi[0][1] + cs[5] * fi[0][2]);
  o.P[1] = detF * (cs[0] * fi[1][0] + cs[3] * fi[1][1] + cs[5] * fi[1][2]);
  o.P[2] = detF * (cs[0] * fi[2][0] + cs[3] * fi[2][1] + cs[5] * fi[2][2]);
  o.P[3] = detF * (cs[3] * fi[0][0] + cs[1] * fi[0][1] + cs[4] * fi[0][2]);
  o.P[4] = detF * (cs[3] * fi[1][0] + cs[1] * fi[1][1] + cs[4] * fi[1][2]);
  o.P[5] = detF * (cs[3] * fi[2][0] + cs[1] * fi[2][1] + cs[4] * fi[2][2]);
  o.P[6] = detF * (cs[5] * fi[0][0] + cs[4] * fi[0][1] + cs[2] * fi[0][2]);
  o.P[7] = detF * (cs[5] * fi[1][0] + cs[4] * fi[1][1] + cs[2] * fi[1][2]);
  o.P[8] = detF * (cs[5] * fi[2][0] + cs[4] * fi[2][1] + cs[2] * fi[2][2]);
  M3 t33 = {{np1.sig[0], np1.sig[3], np1.sig[5]},
            {np1.sig[3], np1.sig[1], np1.sig[4]},
            {np1.sig[5], np1.sig[4], np1.sig[2]}};
  cep2A(Fn, t33, o.cep, rnh, fnhinv, rn1, Fn1, fn1inv, detF, o.A);
}

// ---- mm01: bilinear Mises, mixed hardening (src/mm01.f) -------------------------------
// One material point of the isothermal path, in the reference's own sequence and with
// 1-based vectors: cgn/cgn1 are the 9-word stress vectors (6 stresses, energy density,
// plastic work, equivalent plastic strain), history/history1 the 11-word history.
struct MisesP {
  double e, nu, beta, yld, h;  // setup_mm01_rknstr (src/drive_eps_sig.f:486-520)
};
MisesP mises_props(const cpfft_mises& p) {
  return MisesP{p.e, p.nu, p.beta, p.yld_pt, p.tan_e * p.e / (p.e - p.tan_e)};
}
void mises_state_init(const MisesP& m, State& s) {  // mm01_set_history (src/mm01.f:240-310)
  std::memset(&s, 0, sizeof(s));
  s.m01 = true;
  s.h01[2] = m.yld / 1.73205080756888;
  s.h01[4] = 3.0;  // state: not yielding
  s.h01[5] = m.h;
}
// mm01 + cnst1 for one point; deps = uddt.  Returns the 6x6 tangent in cep.
void mm01_point(const MisesP& m, const double deps1[6], const State& n, State& np1,
                double cep[6][6]) {
  const double root2 = 1.414213562373095, root3 = 1.7320508075688;
  double deps[7], cgn[10], cgn1[10], history[12], history1[12];
  for (int i = 1; i <= 6; i++) deps[i] = deps1[i - 1];
  for (int i = 1; i <= 6; i++) cgn[i] = n.sig[i - 1];
  for (int i = 7; i <= 9; i++) cgn[i] = n.cgx[i - 7];
  for (int i = 1; i <= 11; i++) history[i] = n.h01[i];
  for (int i = 1; i <= 11; i++) history1[i] = 0.0;
  const double ym = m.e, nu = m.nu;
  // mm01_init (src/mm01.f:328-535)
  double deps_vol = deps[1] + deps[2] + deps[3];
  double eps_mean = deps_vol / 3.0;
  double de[7];
  for (int i = 1; i <= 3; i++) de[i] = deps[i] - eps_mean;
  for (int i = 4; i <= 6; i++) de[i] = deps[i];
  double g_n = ym / 2.0 / (1.0 + nu);
  double een[7];
  een[1] = (cgn[1] - nu * (cgn[2] + cgn[3])) / ym;
  een[2] = (cgn[2] - nu * (cgn[1] + cgn[3])) / ym;
  een[3] = (cgn[3] - nu * (cgn[1] + cgn[2])) / ym;
  for (int i = 4; i <= 6; i++) een[i] = cgn[i] / g_n;
  double eps_vol_n1 = een[1] + een[2] + een[3] + deps_vol;
  double eps_mean_n = (een[1] + een[2] + een[3]) / 3.0;
  double ev[7];
  for (int i = 1; i <= 3; i++) ev[i] = (een[i] - eps_mean_n) + de[i];
  for (int i = 4; i <= 6; i++) ev[i] = een[i] + de[i];
  double shear_mod = ym / (2.0 * (1.0 + nu));
  double devel[7], alpha_n[7], rtse[7];
  for (int i = 1; i <= 3; i++) devel[i] = 2.0 * shear_mod * ev[i];
  for (int i = 4; i <= 6; i++) devel[i] = shear_mod * ev[i];
  for (int i = 1; i <= 6; i++) alpha_n[i] = history[5 + i];
  double hbari_np1 = m.beta * m.h, hbark_np1 = (1.0 - m.beta) * m.h;
  double hbark_n = (1.0 - m.beta) * history[5];
  double kbar = (m.yld + hbari_np1 * history[3]) / root3;
  double lk = 1.0;
  if (std::fabs(hbark_n) > 0.000001) lk = hbark_np1 / hbark_n;
  auto norm = [&](const double* r) {
    return std::sqrt(r[1] * r[1] + r[2] * r[2] + r[3] * r[3] +
                     2.0 * (r[4] * r[4] + r[5] * r[5] + r[6] * r[6]));
  };
  for (int i = 1; i <= 6; i++) rtse[i] = devel[i] - alpha_n[i] * lk;
  double yf = norm(rtse) - root2 * kbar;
  for (int i = 1; i <= 6; i++) rtse[i] = devel[i] - alpha_n[i];
  double mrts = norm(rtse);
  int instat = 3;
  bool yield = false;
  if (yf >= 0.0000001 * root2 * kbar) { yield = true; instat = 1; }
  // mm01_simple1 (src/mm01.f:704-785) or the elastic branch of mm01 (:190-199)
  double devstr[7];
  if (yield) {
    const double twthrd = 0.666666666666667, root23 = 0.816496580927;
    double ldt = (mrts - root2 * kbar) / (twthrd * (3.0 * shear_mod + m.h));
    double k_np1 = kbar + (root2 / 3.0) * hbari_np1 * ldt;
    history1[1] = ldt;
    history1[2] = k_np1;
    history1[3] = history[3] + ldt * root23;
    history1[5] = m.h;
    double const1 = twthrd * hbark_np1 * ldt / mrts;
    double const2 = root2 * k_np1 / mrts;
    for (int i = 1; i <= 6; i++) history1[5 + i] = history[5 + i] + const1 * rtse[i];
    for (int i = 1; i <= 6; i++) devstr[i] = history1[5 + i] + const2 * rtse[i];
  } else {
    history1[1] = 0.0;
    history1[2] = kbar;
    history1[3] = history[3];
    history1[5] = m.h;
    for (int i = 1; i <= 6; i++) history1[5 + i] = alpha_n[i] * lk;
    for (int i = 1; i <= 6; i++) devstr[i] = rtse[i] + alpha_n[i];
  }
  // mm01_sig_final (src/mm01.f:626-690)
  double sig_mean = eps_vol_n1 * (3.0 * ym * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)) +
                                  2.0 * shear_mod) / 3.0;
  for (int i = 1; i <= 3; i++) cgn1[i] = devstr[i] + sig_mean;
  for (int i = 4; i <= 6; i++) cgn1[i] = devstr[i];
  double w = 0.0;
  for (int i = 1; i <= 6; i++) w += deps[i] * (cgn1[i] + cgn[i]);
  cgn1[7] = cgn[7] + 0.5 * w;
  history1[4] = instat;
  // mm01_plastic_work (src/mm01.f:546-615)
  cgn1[8] = cgn[8];
  cgn1[9] = cgn[9];
  if (yield) {
    double dsig[7], dp[7];
    for (int i = 1; i <= 6; i++) dsig[i] = cgn1[i] - cgn[i];
    dp[1] = deps[1] - (dsig[1] - nu * (dsig[2] + dsig[3])) / ym;
    dp[2] = deps[2] - (dsig[2] - nu * (dsig[1] + dsig[3])) / ym;
    dp[3] = deps[3] - (dsig[3] - nu * (dsig[1] + dsig[2])) / ym;
    for (int i = 4; i <= 6; i++) dp[i] = deps[i] - dsig[i] / shear_mod;
    double wp = 0.0;
    for (int i = 1; i <= 6; i++) wp += dp[i] * (cgn1[i] + cgn[i]);
    cgn1[8] = cgn[8] + 0.5 * wp;
    double f1 = std::pow(dp[1] - dp[2], 2) + std::pow(dp[2] - dp[3], 2) + std::pow(dp[1] - dp[3], 2);
    double f2 = dp[4] * dp[4] + dp[5] * dp[5] + dp[6] * dp[6];
    cgn1[9] = cgn[9] + (root2 / 3.0) * std::sqrt(f1 + 1.5 * f2);
  }
  // cnst1 (src/mm01.f:1222-1374), with the reference's 10-digit sqrt(2)
  for (int a = 0; a < 6; a++)
    for (int b = 0; b < 6; b++) cep[a][b] = 0.0;
  if (!yield) {
    double c1 = ym / ((1.0 + nu) * (1.0 - 2.0 * nu));
    double c2 = (1.0 - nu) * c1, c3 = ((1.0 - 2.0 * nu) / 2.0) * c1, c4 = nu * c1;
    for (int a = 0; a < 3; a++) {
      for (int b = 0; b < 3; b++) cep[a][b] = a == b ? c2 : c4;
      cep[a + 3][a + 3] = c3;
    }
  } else {
    const double r2 = 1.414213562;
    const double* r = rtse;
    double g = ym / (2.0 * (1.0 + nu));
    double l = (ym * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu));
    double k = (3.0 * l + 2.0 * g) / 3.0;
    double mrtsq = r[1] * r[1] + r[2] * r[2] + r[3] * r[3] + 2.0 * (r[4] * r[4] + r[5] * r[5] + r[6] * r[6]);
    double bb = (r2 * history1[2] + (2.0 / 3.0) * (1.0 - m.beta) * history1[5] * history1[1]) /
                std::sqrt(mrtsq);
    double gamma = 1.0 / (1.0 + history1[5] / (3.0 * g));
    double gambar = gamma - 1.0 + bb;
    double gbar = g * bb;
    double albar = k - 2.0 * gbar / 3.0;
    double thbar = 2.0 * g * gambar;
    for (int a = 1; a <= 6; a++)
      for (int b = 1; b <= 6; b++) {
        double t = -(thbar * r[a] * r[b] / mrtsq);
        if (a <= 3 && b <= 3) t += albar;
        if (a == b) t += (a <= 3) ? 2.0 * gbar : gbar;
        cep[a - 1][b - 1] = t;
      }
  }
  np1 = n;
  np1.m01 = true;
  for (int i = 1; i <= 6; i++) np1.sig[i - 1] = cgn1[i];
  for (int i = 7; i <= 9; i++) np1.cgx[i - 7] = cgn1[i];
  np1.h01[0] = 0.0;
  for (int i = 1; i <= 11; i++) np1.h01[i] = history1[i];
}

void mises_point(const MisesP& m, int step, const M3 Fn, const M3 Fn1, const State& n_in,
                 State& np1, PointOut& o) {
  State n = n_in;
  if (step == 1) mises_state_init(m, n);  // mm01 calls mm01_set_history at step 1 (:160)
  Kin k;
  kinematics(Fn, Fn1, k);
  mm01_point(m, k.uddt, n, np1, o.cep);
  for (int i = 0; i < 6; i++) np1.eps[i] = n.eps[i] + k.uddt[i];
  o.ok = true;
  o.iters = 0;
  pull_back(Fn, Fn1, k, np1, o);
}

// ---- mm00: the FFT program's original St-Venant-Kirchhoff material ------------------
// constitutive (src/mm00.f:13-60): E = (F^T F - I) / 2, S = K tr(E) I + 2 mu dev(E),
// P = F S and A_iJkL = dP_iJ / dF_kL = delta_ik S_LJ + F_iM C_MJNL F_kN with the isotropic
// C of bulk modulus K and shear modulus mu.  A known-answer material for the global loop:
// homogeneous grids and laminates have closed-form solutions.
void svk_point(double K, double mu, const M3 F, double P[9], double A[81]) {
  M3 E, S;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double c = 0.0;
      for (int k = 0; k < 3; k++) c += F[k][i] * F[k][j];
      E[i][j] = 0.5 * (c - (i == j ? 1.0 : 0.0));
    }
  const double tr = E[0][0] + E[1][1] + E[2][2];
  const double lam = K - 2.0 * mu / 3.0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) S[i][j] = 2.0 * mu * E[i][j] + (i == j ? lam * tr : 0.0);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double c = 0.0;
      for (int k = 0; k < 3; k++) c += F[i][k] * S[k][j];
      P[3 * i + j] = c;
    }
  auto C = [&](int a, int b, int c, int d) {
    return lam * (a == b) * (c == d) + mu * ((a == c) * (b == d) + (a == d) * (b == c));
  };
  for (int i = 0; i < 3; i++)
    for (int J = 0; J < 3; J++)
      for (int k = 0; k < 3; k++)
        for (int L = 0; L < 3; L++) {
          double a = (i == k) ? S[L][J] : 0.0;
          for (int m = 0; m < 3; m++)
            for (int n = 0; n < 3; n++) a += F[i][m] * C(m, J, n, L) * F[k][n];
          A[I4(i, J, k, L)] = a;
        }
}

// ---- FFT (restated DFTI role: exact complex DFT) --------------------------------------
struct FFT1 {
  int n;
  std::vector<int> fac;
  std::vector<std::complex<double>> tw;  // exp(-2 pi i k / n)
  explicit FFT1(int n_) : n(n_) {
    int m = n;
    for (int f : {4, 2, 3, 5, 7})
      while (m % f == 0) { fac.push_back(f); m /= f; }
    for (int f = 11; m > 1; f += 2)
      while (m % f == 0) { fac.push_back(f); m /= f; }
    tw.resize(n);
    for (int k = 0; k < n; k++)
      tw[k] = std::complex<double>(std::cos(2.0 * PI * k / n), -std::sin(2.0 * PI * k / n));
  }
  // recursive mixed-radix decimation in time; sign -1 forward, +1 backward (unscaled)
  void rec(const std::complex<double>* in, std::complex<double>* out, int len, int stride,
           int fi, int sign, std::complex<double>* scratch) const {
    if (len == 1) { out[0] = in[0]; return; }
    int r = fac[fi], m = len / r;
    for (int q = 0; q < r; q++) rec(in + q * stride, out + q * m, m, stride * r, fi + 1, sign, scratch);
    int step = n / len;
    for (int k = 0; k < m; k++) {
      std::complex<double> v[16];
      std::complex<double>* vv = r <= 16 ? v : scratch;
      for (int q = 0; q < r; q++) {
        std::complex<double> w = tw[(q * k * step) % n];
        if (sign > 0) w = std::conj(w);
        vv[q] = out[q * m + k] * w;
      }
      for (int s = 0; s < r; s++) {
        std::complex<double> acc = 0.0;
        for (int q = 0; q < r; q++) {
          std::complex<double> w = tw[((q * s) % r) * (n / r)];
          if (sign > 0) w = std::conj(w);
          acc += vv[q] * w;
        }
        scratch[r + s] = acc;
      }
      for (int s = 0; s < r; s++) out[s * m + k] = scratch[r + s];
    }
  }
  void run(std::complex<double>* data, int sign, std::vector<std::complex<double>>& buf) const {
    if ((int)buf.size() < 2 * n + 64) buf.resize(2 * n + 64);
    std::complex<double>* in = buf.data();
    std::complex<double>* scratch = buf.data() + n;
    for (int i = 0; i < n; i++) in[i] = data[i];
    rec(in, data, n, 1, 0, sign, scratch);
  }
};

void fft3(const FFT1& f, double* re, double* im, int sign) {
  int N = f.n;
  std::vector<std::complex<double>> line(N), buf;
  for (int axis = 0; axis < 3; axis++) {
    long s = axis == 0 ? 1 : (axis == 1 ? N : (long)N * N);
    for (int u = 0; u < N; u++)
      for (int w = 0; w < N; w++) {
        long base;
        if (axis == 0) base = (long)u * N + (long)w * N * N;
        else if (axis == 1) base = u + (long)w * N * N;
        else base = u + (long)w * N;
        for (int k = 0; k < N; k++) line[k] = std::complex<double>(re[base + k * s], im[base + k * s]);
        f.run(line.data(), sign, buf);
        for (int k = 0; k < N; k++) { re[base + k * s] = line[k].real(); im[base + k * s] = line[k].imag(); }
      }
  }
  if (sign > 0) {
    double sc = 1.0 / ((double)N * N * N);
    long N3 = (long)N * N * N;
    for (long v = 0; v < N3; v++) { re[v] *= sc; im[v] *= sc; }
  }
}

}  // namespace

// ======================================================================================
struct orc_ctx {
  int N;
  long N3;
  double dt;
  int gmap, nthreads;
  std::vector<Crys> crys;
  std::vector<int> kind;           // per material: 0 crystal, 1 mm01, 2 not yet defined
  std::vector<MisesP> mp;          // per material (mm01)
  std::vector<double> svk;         // per material (mm00, kind 3): K, mu
  std::vector<int> mat;            // 0-based material per voxel
  std::vector<VoxProps> vprops;
  std::vector<State> hn, hn1;
  std::vector<double> Fn, Fn1, Pn, Pn1, K4, b, dFm;
  // G_K_dF tables: Ghat "centered" q per axis and the fftshift phase
  std::vector<double> qax;         // per axis value of q for memory index k
  std::vector<char> nyq;           // per axis: memory index k holds the Nyquist frequency
  std::vector<double> coef_c, coef_s;
  FFT1* fft;
  // FFT_nr3 persistent locals (Fortran DATA => SAVE'd, src/FFT_nr3.f:29-34)
  double barF_t[9], P_bar[9], C_homo[81];
  double eq_tol = 0.0;  // equilibrium stop test of the Newton loop (0: the reference's loop)
  int coupled_bc = 0;  // the P_bar update inside the Newton iteration (2: implicit first pass)
  int hist_words = ORC_HIST;  // ORC_HIST_MRR on grids of Ma-Roters-Raabe crystals
};

static void ghat_apply(const orc_ctx* c, long v, const double* in9, double* out9,
                       const double q[3]) {
  (void)c; (void)v;
  double qq = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
  if (std::fabs(qq) <= 1.0e-10) { for (int i = 0; i < 9; i++) out9[i] = 0.0; return; }
  // (G:A)_ij = sum_kl delta_ik q_j q_l / |q|^2 A_kl  (formG, src/FFT_init.f:272-340)
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0;
      for (int l = 0; l < 3; l++) s += (q[j] * q[l] / qq) * in9[3 * i + l];
      out9[3 * i + j] = s;
    }
}

extern "C" {

orc_ctx* orc_create(int N, const int* matList, const double* kocks_deg,
                    const cpfft_crystal* props, int ncrystals, double tstep, int g_mapping,
                    int nthreads) {
  orc_ctx* c = new orc_ctx;
  c->N = N;
  c->N3 = (long)N * N * N;
  c->dt = tstep;
  c->gmap = g_mapping;
  c->nthreads = nthreads > 0 ? nthreads : 1;
  c->crys.resize(ncrystals);
  c->kind.assign(ncrystals, 0);
  c->mp.resize(ncrystals);
  c->svk.assign(2 * ncrystals, 0.0);
  for (int i = 0; i < ncrystals; i++) {
    if (props[i].slip_type == CPFFT_NOT_A_CRYSTAL) { c->kind[i] = 2; continue; }
    crystal_finalize(props[i], c->crys[i]);
    if (props[i].h_type == 7 || props[i].h_type == 4) c->hist_words = ORC_HIST_MRR;
  }
  long N3 = c->N3;
  c->mat.resize(N3);
  c->vprops.resize(N3);
  for (long v = 0; v < N3; v++) {
    c->mat[v] = matList[v] - 1;
    if (c->kind[c->mat[v]] != 0) continue;
    double ang[3] = {kocks_deg[v], kocks_deg[N3 + v], kocks_deg[2 * N3 + v]};
    voxel_props(c->crys[c->mat[v]], ang, c->vprops[v]);
  }
  c->hn.resize(N3);
  c->hn1.resize(N3);
  for (long v = 0; v < N3; v++) {
    if (c->kind[c->mat[v]] == 0) state_init(c->crys[c->mat[v]], c->hn[v]);
    else std::memset(&c->hn[v], 0, sizeof(State));
    c->hn1[v] = c->hn[v];
  }
  c->Fn.assign(9 * N3, 0.0);
  for (int d : {0, 4, 8})
    for (long v = 0; v < N3; v++) c->Fn[d * N3 + v] = 1.0;
  c->Fn1 = c->Fn;
  c->Pn.assign(9 * N3, 0.0);
  c->Pn1.assign(9 * N3, 0.0);
  c->K4.assign(81 * N3, 0.0);
  c->b.assign(9 * N3, 0.0);
  c->dFm.assign(9 * N3, 0.0);
  int Nhalf = (N % 2 == 1) ? (N + 1) / 2 : N / 2 + 1;  // src/FFT_init.f:146-147
  c->qax.resize(N);
  c->nyq.assign(N, 0);
  for (int k = 0; k < N; k++) {
    // memory index k of the phase-shifted transform holds true frequency (k+Nhalf) mod N
    int f = (k + Nhalf) % N;
    if (g_mapping == CPFFT_G_REF_SHIFT) {
      c->qax[k] = (double)(k + 1 - Nhalf);
    } else {
      c->qax[k] = (double)(f <= (N - 1) / 2 ? f : f - N);  // signed wavenumber
      // even N: the Nyquist frequency has no signed partner; its Green operator is zero
      c->nyq[k] = (N % 2 == 0 && 2 * f == N) ? 1 : 0;
    }
  }
  c->coef_c.resize(N3);
  c->coef_s.resize(N3);
  double NhN = (double)Nhalf * 2.0 * PI / (double)N;  // formfftshift (:354-385)
  for (int k = 0; k < N; k++)
    for (int j = 0; j < N; j++)
      for (int i = 0; i < N; i++) {
        double temp = NhN * (double)(i + j + k);
        long v = i + (long)N * j + (long)N * N * k;
        c->coef_c[v] = std::cos(temp);
        c->coef_s[v] = -std::sin(temp);
      }
  c->fft = new FFT1(N);
  for (int i = 0; i < 9; i++) c->barF_t[i] = (i % 4 == 0) ? 1.0 : 0.0;
  for (int i = 0; i < 9; i++) c->P_bar[i] = 0.0;
  for (int i = 0; i < 81; i++) c->C_homo[i] = 0.0;
  return c;
}

void orc_destroy(orc_ctx* c) {
  if (!c) return;
  delete c->fft;
  delete c;
}

static void load33(const double* f, long N3, long v, M3 m) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) m[i][j] = f[(3 * i + j) * N3 + v];
}

// the material point of voxel v with its material's model
static void voxel_point(orc_ctx* c, long v, int step, int iter, const M3 fn, const M3 fn1,
                        PointOut& o) {
  const int m = c->mat[v];
  if (c->kind[m] == 0) {
    material_point(c->crys[m], c->vprops[v], c->dt, step, iter, fn, fn1, c->hn[v], c->hn1[v], o);
  } else if (c->kind[m] == 1) {
    mises_point(c->mp[m], step, fn, fn1, c->hn[v], c->hn1[v], o);
  } else if (c->kind[m] == 3) {  // hyperelastic: no history
    (void)fn;
    svk_point(c->svk[2 * m], c->svk[2 * m + 1], fn1, o.P, o.A);
    c->hn1[v] = c->hn[v];
    o.ok = true;
    o.iters = 0;
  } else {  // undefined material
    std::memset(&o, 0, sizeof(o));
    o.ok = false;
  }
}

void orc_set_mises(orc_ctx* c, int material, const cpfft_mises* props) {
  const int m = material - 1;
  c->kind[m] = 1;
  c->mp[m] = mises_props(*props);
  for (long v = 0; v < c->N3; v++)
    if (c->mat[v] == m) {
      mises_state_init(c->mp[m], c->hn[v]);
      c->hn1[v] = c->hn[v];
    }
}

void orc_set_svk(orc_ctx* c, int material, double K, double mu) {
  const int m = material - 1;
  c->kind[m] = 3;
  c->svk[2 * m] = K;
  c->svk[2 * m + 1] = mu;
  for (long v = 0; v < c->N3; v++)
    if (c->mat[v] == m) {
      std::memset(&c->hn[v], 0, sizeof(State));
      c->hn1[v] = c->hn[v];
    }
}

void orc_svk_point(double K, double mu, const double F[9], double P[9], double A[81]) {
  M3 f;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) f[i][j] = F[3 * i + j];
  svk_point(K, mu, f, P, A);
}

int orc_stress_update(orc_ctx* c, int step, int iter, const double* Fn, const double* Fn1,
                      double* Pn1, double* K4, long long* local_iters) {
  long N3 = c->N3;
  if (Fn) std::copy(Fn, Fn + 9 * N3, c->Fn.begin());
  if (Fn1) std::copy(Fn1, Fn1 + 9 * N3, c->Fn1.begin());
  int fails = 0;
  long long its = 0;
#pragma omp parallel for schedule(dynamic, 128) reduction(+ : fails, its) num_threads(c->nthreads)
  for (long v = 0; v < N3; v++) {
    M3 fn, fn1;
    load33(c->Fn.data(), N3, v, fn);
    load33(c->Fn1.data(), N3, v, fn1);
    PointOut o;
    voxel_point(c, v, step, iter, fn, fn1, o);
    if (!o.ok) fails++;
    its += o.iters;
    for (int i = 0; i < 9; i++) c->Pn1[i * N3 + v] = o.P[i];
    for (int m = 0; m < 81; m++) c->K4[m * N3 + v] = o.A[m];
  }
  if (Pn1) std::copy(c->Pn1.begin(), c->Pn1.end(), Pn1);
  if (K4) std::copy(c->K4.begin(), c->K4.end(), K4);
  if (local_iters) *local_iters = its;
  return fails;
}

// stress update of voxels [v0, v1) only (bounded CPU-baseline samples); no outputs
int orc_stress_sample(orc_ctx* c, int step, int iter, long v0, long v1) {
  long N3 = c->N3;
  int fails = 0;
#pragma omp parallel for schedule(dynamic, 128) reduction(+ : fails) num_threads(c->nthreads)
  for (long v = v0; v < v1; v++) {
    M3 fn, fn1;
    load33(c->Fn.data(), N3, v, fn);
    load33(c->Fn1.data(), N3, v, fn1);
    PointOut o;
    voxel_point(c, v, step, iter, fn, fn1, o);
    if (!o.ok) fails++;
    for (int i = 0; i < 9; i++) c->Pn1[i * N3 + v] = o.P[i];
    for (int m = 0; m < 81; m++) c->K4[m * N3 + v] = o.A[m];
  }
  return fails;
}

void orc_commit(orc_ctx* c) {  // update (src/update.f) + FFT_nr3.f:173-179
  c->hn = c->hn1;
  c->Fn = c->Fn1;
  c->Pn = c->Pn1;
}

// G_K_dF (src/G_K_dF.f:11-87), restated with an explicit complex DFT
void orc_green_apply(orc_ctx* c, const double* x, double* y, int flgK, const double* K4) {
  long N3 = c->N3;
  int N = c->N;
  const double* K = K4 ? K4 : c->K4.data();
  std::vector<double> r1(9 * N3), r2(9 * N3), r3(9 * N3);
  if (flgK) {
    // ddot42n (src/G_K_dF.f:241-268), its summation order kept
#pragma omp parallel for num_threads(c->nthreads)
    for (long v = 0; v < N3; v++)
      for (int i = 0; i < 9; i++) {
        double t[9];
        for (int j = 0; j < 9; j++) t[j] = K[(9 * i + j) * N3 + v] * x[j * N3 + v];
        double s1 = t[1] + t[5], s2 = t[2] + t[6], s3 = t[3] + t[7], s4 = t[4] + t[8];
        s1 = s1 + s3; s2 = s2 + s4;
        s1 = s1 + s2;
        r1[i * N3 + v] = t[0] + s1;
      }
  } else {
    std::copy(x, x + 9 * N3, r1.begin());
  }
#pragma omp parallel for num_threads(std::min(c->nthreads, 9))
  for (int i = 0; i < 9; i++) {  // fftfem3d (:101-157)
    double* re = &r2[i * N3];
    double* im = &r3[i * N3];
    for (long v = 0; v < N3; v++) {
      re[v] = r1[i * N3 + v] * c->coef_c[v];
      im[v] = r1[i * N3 + v] * c->coef_s[v];
    }
    fft3(*c->fft, re, im, -1);
  }
  // Ghat multiply of the real and imaginary parts (:64-65); memory index (a,b,cc)
  // with a fastest carries q = (q[cc], q[b], q[a]) (formG, src/FFT_init.f:310-318)
#pragma omp parallel for num_threads(c->nthreads)
  for (long v = 0; v < N3; v++) {
    int a = (int)(v % N), bb = (int)((v / N) % N), cc = (int)(v / ((long)N * N));
    double q[3] = {c->qax[cc], c->qax[bb], c->qax[a]};
    double in_re[9], in_im[9], o_re[9], o_im[9];
    for (int i = 0; i < 9; i++) { in_re[i] = r2[i * N3 + v]; in_im[i] = r3[i * N3 + v]; }
    if (c->nyq[cc] || c->nyq[bb] || c->nyq[a]) q[0] = q[1] = q[2] = 0.0;
    ghat_apply(c, v, in_re, o_re, q);
    ghat_apply(c, v, in_im, o_im, q);
    for (int i = 0; i < 9; i++) { r1[i * N3 + v] = o_re[i]; r2[i * N3 + v] = o_im[i]; }
  }
#pragma omp parallel for num_threads(std::min(c->nthreads, 9))
  for (int i = 0; i < 9; i++) {  // ifftfem3d (:171-227)
    double* re = &r1[i * N3];
    double* im = &r2[i * N3];
    fft3(*c->fft, re, im, +1);
    for (long v = 0; v < N3; v++) y[i * N3 + v] = re[v] * c->coef_c[v] + im[v] * c->coef_s[v];
  }
}

static double nrm2(const double* x, long n) {
  double s = 0;
  for (long i = 0; i < n; i++) s += x[i] * x[i];
  return std::sqrt(s);
}
static double dotp(const double* x, const double* y, long n) {
  double s = 0;
  for (long i = 0; i < n; i++) s += x[i] * y[i];
  return s;
}

// fftPcg (src/FFT_nr3.f:214-360): unpreconditioned CG from x = 0 with the reference's
// stop test ||r|| <= tol*||b|| .or. ||r|| <= tol, maxIter 1000
int orc_cg(orc_ctx* c, const double* b, double* x, double tol, int* iters) {
  long n = 9 * c->N3;
  const int maxIter = 1000;
  std::fill(x, x + n, 0.0);
  *iters = 0;
  double n2b = nrm2(b, n);
  double tolb = tol * n2b;
  if (tol <= 2.220446049250313e-16 || tol >= 1.0) return CPFFT_ERR_CG_TOL;
  if (n2b <= 2.220446049250313e-16) return 0;
  std::vector<double> r(b, b + n), p(b, b + n), Ap(n);
  double rr = dotp(r.data(), r.data(), n);
  int it = 0;
  while (true) {
    orc_green_apply(c, p.data(), Ap.data(), 1, nullptr);
    double pAp = dotp(p.data(), Ap.data(), n);
    double alpha = rr / pAp;
    for (long i = 0; i < n; i++) { x[i] += alpha * p[i]; r[i] -= alpha * Ap[i]; }
    it++;
    double rn = nrm2(r.data(), n);
    if (rn <= tolb || rn <= tol) break;
    if (it >= maxIter) break;
    double rr_new = rn * rn;
    double beta = rr_new / rr;
    rr = rr_new;
    for (long i = 0; i < n; i++) p[i] = r[i] + beta * p[i];
  }
  *iters = it;
  return it >= maxIter ? CPFFT_ERR_CG_MAXIT : 0;  // src/FFT_nr3.f:335-339
}

// tangent_homo (src/tangent_homo.f:11-73)
int orc_tangent_homo(orc_ctx* c, double tolPCG, double* C_homo) {
  long N3 = c->N3;
  std::vector<double> Cij(9 * N3);
  int total = 0;
  for (int i = 0; i < 9; i++) {
    for (int j = 0; j < 9; j++)
      std::copy(&c->K4[(9 * j + i) * N3], &c->K4[(9 * j + i) * N3] + N3, &Cij[j * N3]);
    orc_green_apply(c, Cij.data(), c->b.data(), 0, nullptr);
    for (long k = 0; k < 9 * N3; k++) c->b[k] = -c->b[k];
    int its = 0;
    int rc = orc_cg(c, c->b.data(), Cij.data(), tolPCG, &its);
    total += its;
    if (rc) return rc;
    for (long v = 0; v < N3; v++) Cij[i * N3 + v] += 1.0;
    for (int j = 0; j < 9; j++) {
      double s = dotp(&c->K4[(9 * j) * N3], Cij.data(), 9 * N3);
      C_homo[9 * j + i] = s / (double)N3;
    }
  }
  return total;
}

// NBC_update (src/FFT_nr3.f:375-433)
static int nbc_update(const double* C_homo, double* DbarF, const double* P_bar,
                      const double* PBC, const int* isNBC) {
  double A[81], bb[9];
  for (int i = 0; i < 9; i++) {
    if (isNBC[i]) {
      for (int k = 0; k < 9; k++) A[i * 9 + k] = C_homo[k + 9 * i];  // C_homo(1:9, i)
      bb[i] = PBC[i] - P_bar[i];
    } else {
      for (int k = 0; k < 9; k++) A[i * 9 + k] = 0.0;
      A[i * 9 + i] = 1.0;
      bb[i] = DbarF[i];
    }
  }
  int info = lu_solve(9, A, 1, bb);
  if (info) return CPFFT_ERR_NBC_SINGULAR;
  for (int i = 0; i < 9; i++) DbarF[i] = bb[i];
  return 0;
}

// ||g|| / (sqrt(N3) ||mean of Pn1||), g = G(Pn1)
static double equil_residual(const orc_ctx* c, const double* g) {
  const long N3 = c->N3;
  double pb = 0;
  for (int i = 0; i < 9; i++) {
    double s = 0;
    for (long v = 0; v < N3; v++) s += c->Pn1[i * N3 + v];
    pb += (s / (double)N3) * (s / (double)N3);
  }
  return nrm2(g, 9 * N3) / (std::sqrt((double)N3) * std::sqrt(pb));
}

void orc_set_equilibrium_tol(orc_ctx* c, double tol) { c->eq_tol = tol; }
void orc_set_coupled_bc(orc_ctx* c, int on) { c->coupled_bc = on; }

// The library's coupled P_bar update (cpfft_set_coupled_bc, an extension restated here
// for its parity tests; mode 2 makes the first stress pass implicit): after each stress
// pass, DbarF from NBC_update's system with the current C_homo (recomputed after the
// first implicit pass), then the fluctuation
// solves G(K : dF) = -G(P) - G(K : DbarF); increments that raise the equilibrium residual
// are halved (at most 4 times in a row); the step ends when P_bar, the equilibrium
// residual and the last increment all meet their tolerances.
static int coupled_step(orc_ctx* c, int step, const double* PBC, const int* isNBC,
                        double* barF, double Fnorm, double tolNR, double tolPCG, int maxIter,
                        cpfft_stats& S) {
  const long N3 = c->N3, n = 9 * N3;
  double resfft = 1.0;
  int tangents = 0, rc = 0;
  std::vector<double> g(n), w(n);
  double eq_prev = HUGE_VAL, frac = 1.0, lastD[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int halvings = 0;
  for (int k = 0;; k++) {
    long long li = 0;
    const int iter = c->coupled_bc == 2 ? k + 1 : k;  // mode 2: no explicit opening pass
    S.local_fallbacks += orc_stress_update(c, step, iter, nullptr, nullptr, nullptr, nullptr, &li);
    S.local_iters += li;
    S.stress_updates++;
    orc_green_apply(c, c->Pn1.data(), g.data(), 0, nullptr);
    const double e = equil_residual(c, g.data());
    S.res_equil = e;
    double res1 = 0, res2 = 0;
    for (int i = 0; i < 9; i++) {
      double s = 0;
      for (long v = 0; v < N3; v++) s += c->Pn1[i * N3 + v];
      c->P_bar[i] = s / (double)N3;
      res2 += c->P_bar[i] * c->P_bar[i];
      if (isNBC[i]) res1 += (c->P_bar[i] - PBC[i]) * (c->P_bar[i] - PBC[i]);
    }
    const double res3 = res2 < 1.0e-8 ? std::sqrt(res1) : std::sqrt(res1 / res2);
    S.res_pbar = res3;
    if (res3 <= tolNR && e <= c->eq_tol && resfft <= tolNR) break;
    if (k == maxIter) return CPFFT_ERR_NEWTON_MAXIT;
    if (k >= 2 && e > eq_prev && halvings < 4) {  // halve the last increment
      frac *= 0.5;
      for (int i = 0; i < 9; i++) barF[i] -= frac * lastD[i];
      for (int i = 0; i < 9; i++)
        for (long v = 0; v < N3; v++) c->Fn1[i * N3 + v] -= frac * (c->dFm[i * N3 + v] + lastD[i]);
      halvings++;
      resfft *= 0.5;
      continue;
    }
    eq_prev = e;
    halvings = 0;
    frac = 1.0;
    if (k >= (c->coupled_bc == 2 ? 0 : 1) && tangents < 1) {
      int th = orc_tangent_homo(c, tolPCG, c->C_homo);
      if (th < 0) return th;
      S.cg_solves += 9; S.cg_iters += th;
      tangents++;
    }
    double DbarF[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if ((rc = nbc_update(c->C_homo, DbarF, c->P_bar, PBC, isNBC))) return rc;
    for (int i = 0; i < 9; i++)
      for (long v = 0; v < N3; v++) c->dFm[i * N3 + v] = DbarF[i];
    orc_green_apply(c, c->dFm.data(), w.data(), 1, nullptr);
    for (long q = 0; q < n; q++) {
      c->b[q] = -g[q] - w[q];
      c->Fn1[q] += c->dFm[q];
    }
    for (int i = 0; i < 9; i++) {
      barF[i] += DbarF[i];
      lastD[i] = DbarF[i];
    }
    int its = 0;
    rc = orc_cg(c, c->b.data(), c->dFm.data(), tolPCG, &its);
    S.cg_solves++; S.cg_iters += its;
    if (rc) return rc;
    for (long q = 0; q < n; q++) c->Fn1[q] += c->dFm[q];
    double db = 0;
    for (int i = 0; i < 9; i++) db += DbarF[i] * DbarF[i];
    const double dn = nrm2(c->dFm.data(), n);
    resfft = std::sqrt(dn * dn + (double)N3 * db) / Fnorm;
    S.newton_iters++;
    S.res_fft = resfft;
  }
  S.nbc_iters = 1;
  return 0;
}

int orc_nr3_begin(orc_ctx* c, double tolPCG) {
  orc_stress_update(c, 1, 0, nullptr, nullptr, nullptr, nullptr, nullptr);
  int rc = orc_tangent_homo(c, tolPCG, c->C_homo);
  return rc < 0 ? rc : 0;
}

// one load step of FFT_nr3 (src/FFT_nr3.f:51-185)
int orc_nr3_step(orc_ctx* c, int step, const double* BC, const int* isNBC, double tolNR,
                 double tolPCG, int maxIter, double* Pbar, cpfft_stats* st) {
  using clk = std::chrono::steady_clock;
  auto t0 = clk::now();
  cpfft_stats S;
  std::memset(&S, 0, sizeof(S));
  long N3 = c->N3, n = 9 * N3;
  bool existNBC = false;
  for (int i = 0; i < 9; i++) existNBC |= isNBC[i] != 0;
  double PBC[9], FBC[9], DbarF[9], barF[9];
  for (int i = 0; i < 9; i++) {
    PBC[i] = FBC[i] = DbarF[i] = 0.0;
    if (isNBC[i]) PBC[i] = BC[i];
    else { FBC[i] = BC[i]; DbarF[i] = FBC[i] - c->barF_t[i]; }
  }
  int rc = 0;
  if (existNBC && (rc = nbc_update(c->C_homo, DbarF, c->P_bar, PBC, isNBC))) return rc;
  for (int i = 0; i < 9; i++) barF[i] = c->barF_t[i] + DbarF[i];
  int iiter_NBC = 0;
  double tp = 0, ts = 0;
  auto tic = [] { return clk::now(); };
  auto sec = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
  while (true) {
    for (int i = 0; i < 9; i++)
      for (long v = 0; v < N3; v++) c->dFm[i * N3 + v] = DbarF[i];
    double Fnorm = nrm2(c->Fn1.data(), n);
    for (long k = 0; k < n; k++) c->Fn1[k] += c->dFm[k];
    orc_green_apply(c, c->dFm.data(), c->b.data(), 1, nullptr);
    for (long k = 0; k < n; k++) c->b[k] = -c->b[k];
    int its = 0;
    auto a = tic();
    rc = orc_cg(c, c->b.data(), c->dFm.data(), tolPCG, &its);
    tp += sec(a);
    S.cg_solves++; S.cg_iters += its;
    if (rc) return rc;
    for (long k = 0; k < n; k++) c->Fn1[k] += c->dFm[k];
    if (c->eq_tol > 0.0 && existNBC && c->coupled_bc) {
      if ((rc = coupled_step(c, step, PBC, isNBC, barF, Fnorm, tolNR, tolPCG, maxIter, S)))
        return rc;
      break;
    }
    double resfft = 1.0;
    int iiter_EBC = 0;
    // equilibrium test (an extension of the library, restated here for its parity tests):
    // the loop body starts with the stress update, which also closes the loop when
    // ||dF||/||F|| <= tolNR and ||G(P)|| / (sqrt(N3) ||P_bar||) <= eq_tol; an increment
    // after which that residual has grown is halved (at most 4 times) before the next solve
    const bool eq_mode = c->eq_tol > 0.0;
    bool closed = false;
    double eq_prev = HUGE_VAL, frac = 1.0;
    int halvings = 0;
    while (eq_mode || resfft > tolNR) {
      a = tic();
      long long li = 0;
      S.local_fallbacks += orc_stress_update(c, step, iiter_EBC, nullptr, nullptr, nullptr, nullptr, &li);
      ts += sec(a);
      S.local_iters += li;
      S.stress_updates++;
      orc_green_apply(c, c->Pn1.data(), c->b.data(), 0, nullptr);
      if (eq_mode) {
        S.res_equil = equil_residual(c, c->b.data());
        if (resfft <= tolNR && S.res_equil <= c->eq_tol) { closed = true; break; }
        if (iiter_EBC >= 2 && S.res_equil > eq_prev && halvings < 4) {
          frac *= 0.5;
          for (long k = 0; k < n; k++) c->Fn1[k] -= frac * c->dFm[k];
          halvings++;
          resfft *= 0.5;
          continue;
        }
        eq_prev = S.res_equil;
        halvings = 0;
        frac = 1.0;
      }
      for (long k = 0; k < n; k++) c->b[k] = -c->b[k];
      a = tic();
      rc = orc_cg(c, c->b.data(), c->dFm.data(), tolPCG, &its);
      tp += sec(a);
      S.cg_solves++; S.cg_iters += its;
      if (rc) return rc;
      for (long k = 0; k < n; k++) c->Fn1[k] += c->dFm[k];
      resfft = nrm2(c->dFm.data(), n) / Fnorm;
      S.newton_iters++;
      S.res_fft = resfft;
      if (getenv("ORC_LOG"))
        fprintf(stderr, "  nbc %d newton %d resfft %.3e cg %d\n", iiter_NBC, iiter_EBC, resfft, its);
      if (iiter_EBC == maxIter) return CPFFT_ERR_NEWTON_MAXIT;
      iiter_EBC++;
    }
    if (!closed) {
      a = tic();
      long long li = 0;
      S.local_fallbacks += orc_stress_update(c, step, iiter_EBC, nullptr, nullptr, nullptr, nullptr, &li);
      ts += sec(a);
      S.local_iters += li;
      S.stress_updates++;
    }
    double res1 = 0, res2 = 0;
    for (int i = 0; i < 9; i++) {
      double s = 0;
      for (long v = 0; v < N3; v++) s += c->Pn1[i * N3 + v];
      c->P_bar[i] = s / (double)N3;
      res2 += c->P_bar[i] * c->P_bar[i];
      if (isNBC[i]) res1 += (c->P_bar[i] - PBC[i]) * (c->P_bar[i] - PBC[i]);
    }
    double res3 = res2 < 1.0e-8 ? std::sqrt(res1) : std::sqrt(res1 / res2);
    S.res_pbar = res3;
    S.nbc_iters = iiter_NBC + 1;
    if (res3 <= tolNR) break;
    if (iiter_NBC > maxIter) return CPFFT_ERR_NBC_MAXIT;
    a = tic();
    int th = orc_tangent_homo(c, tolPCG, c->C_homo);
    tp += sec(a);
    if (th < 0) return th;
    S.cg_solves += 9; S.cg_iters += th;
    for (int i = 0; i < 9; i++) DbarF[i] = 0.0;
    if ((rc = nbc_update(c->C_homo, DbarF, c->P_bar, PBC, isNBC))) return rc;
    for (int i = 0; i < 9; i++) barF[i] += DbarF[i];
    iiter_NBC++;
  }
  for (int i = 0; i < 9; i++) c->barF_t[i] = barF[i];
  orc_commit(c);
  if (Pbar) for (int i = 0; i < 9; i++) Pbar[i] = c->P_bar[i];
  // equilibrium residual ||G(P)|| / (sqrt(N3) ||P_bar||) of the committed state (already
  // evaluated on it by the equilibrium test)
  if (!c->eq_tol) {
    orc_green_apply(c, c->Pn1.data(), c->b.data(), 0, nullptr);
    S.res_equil = equil_residual(c, c->b.data());
  }
  S.t_pcg = tp;
  S.t_sigeps = ts;
  S.t_total = sec(t0);
  if (st) *st = S;
  return S.local_fallbacks ? CPFFT_WARN_LOCAL_FALLBACK : 0;
}

void orc_get_fields(orc_ctx* c, double* Fn, double* Fn1, double* Pn, double* Pn1, double* K4) {
  if (Fn) std::copy(c->Fn.begin(), c->Fn.end(), Fn);
  if (Fn1) std::copy(c->Fn1.begin(), c->Fn1.end(), Fn1);
  if (Pn) std::copy(c->Pn.begin(), c->Pn.end(), Pn);
  if (Pn1) std::copy(c->Pn1.begin(), c->Pn1.end(), Pn1);
  if (K4) std::copy(c->K4.begin(), c->K4.end(), K4);
}
void orc_set_fields(orc_ctx* c, const double* Fn, const double* Fn1) {
  if (Fn) std::copy(Fn, Fn + 9 * c->N3, c->Fn.begin());
  if (Fn1) std::copy(Fn1, Fn1 + 9 * c->N3, c->Fn1.begin());
}
int orc_hist_words(orc_ctx* c) { return c->hist_words; }
void orc_get_history(orc_ctx* c, double* hist_n, double* hist_np1) {
  long N3 = c->N3;
  const int W = c->hist_words;
  double h[ORC_HIST_MRR];
  for (long v = 0; v < N3; v++) {
    std::fill(h, h + ORC_HIST_MRR, 0.0);
    if (hist_n) { state_pack(c->hn[v], h); for (int w = 0; w < W; w++) hist_n[w * N3 + v] = h[w]; }
    std::fill(h, h + ORC_HIST_MRR, 0.0);
    if (hist_np1) { state_pack(c->hn1[v], h); for (int w = 0; w < W; w++) hist_np1[w * N3 + v] = h[w]; }
  }
}
void orc_set_history_n(orc_ctx* c, const double* hist_n) {
  long N3 = c->N3;
  const int W = c->hist_words;
  double h[ORC_HIST_MRR];
  for (long v = 0; v < N3; v++) {
    for (int w = 0; w < W; w++) h[w] = hist_n[w * N3 + v];
    std::memset(&c->hn[v], 0, sizeof(State));
    const int m = c->mat[v];
    c->hn[v].m01 = c->kind[m] == 1;
    c->hn[v].mrr = c->kind[m] == 0 && (c->crys[m].p.h_type == 7 || c->crys[m].p.h_type == 4);
    state_unpack(h, c->hn[v]);
  }
}

int orc_voxel_update(const cpfft_crystal* props, const double kocks_deg[3], double tstep,
                     int step, int iter, const double Fn[9], const double Fn1[9],
                     const double* hist_n, double* hist_np1, double P[9], double A[81],
                     double out_sig6[6], double out_cep36[36]) {
  Crys cr;
  crystal_finalize(*props, cr);
  VoxProps vp;
  voxel_props(cr, kocks_deg, vp);
  State n, np1;
  std::memset(&n, 0, sizeof(n));
  std::memset(&np1, 0, sizeof(np1));
  n.mrr = props->h_type == 7 || props->h_type == 4;
  if (hist_n) state_unpack(hist_n, n);
  else state_init(cr, n);
  M3 fn, fn1;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) { fn[i][j] = Fn[3 * i + j]; fn1[i][j] = Fn1[3 * i + j]; }
  PointOut o;
  material_point(cr, vp, tstep, step, iter, fn, fn1, n, np1, o);
  if (hist_np1) state_pack(np1, hist_np1);
  if (P) for (int i = 0; i < 9; i++) P[i] = o.P[i];
  if (A) for (int i = 0; i < 81; i++) A[i] = o.A[i];
  if (out_sig6) for (int i = 0; i < 6; i++) out_sig6[i] = o.sig[i];
  if (out_cep36) for (int a = 0; a < 6; a++) for (int b = 0; b < 6; b++) out_cep36[a * 6 + b] = o.cep[a][b];
  return o.ok ? o.iters : -1;
}

int orc_mises_update(const cpfft_mises* props, int step, const double Fn[9], const double Fn1[9],
                     const double* hist_n, double* hist_np1, double P[9], double A[81],
                     double out_sig6[6], double out_cep36[36]) {
  const MisesP m = mises_props(*props);
  State n, np1;
  std::memset(&n, 0, sizeof(n));
  n.m01 = true;
  if (hist_n) state_unpack(hist_n, n);
  else mises_state_init(m, n);
  M3 fn, fn1;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) { fn[i][j] = Fn[3 * i + j]; fn1[i][j] = Fn1[3 * i + j]; }
  PointOut o;
  mises_point(m, step, fn, fn1, n, np1, o);
  if (hist_np1) state_pack(np1, hist_np1);
  if (P) for (int i = 0; i < 9; i++) P[i] = o.P[i];
  if (A) for (int i = 0; i < 81; i++) A[i] = o.A[i];
  if (out_sig6) for (int i = 0; i < 6; i++) out_sig6[i] = o.sig[i];
  if (out_cep36) for (int a = 0; a < 6; a++) for (int b = 0; b < 6; b++) out_cep36[a * 6 + b] = o.cep[a][b];
  return 0;
}

void orc_mrr_interaction(int slip_type, double G[144], double H[144]) {
  cpfft_crystal p;
  std::memset(&p, 0, sizeof(p));
  p.slip_type = slip_type;
  p.elastic_type = 1;
  p.e = 1.0;
  p.nu = 0.3;
  Crys cr;
  crystal_finalize(p, cr);
  for (int a = 0; a < 12; a++)
    for (int q = 0; q < 12; q++) {
      G[12 * a + q] = cr.Gm[a][q];
      H[12 * a + q] = cr.Hm[a][q];
    }
}

int orc_mrr_residual(const cpfft_crystal* props, const double kocks_deg[3], const double D[6],
                     double tinc, const double* hist_n, const double x[18], double R[18],
                     double J[324]) {
  if (props->h_type != 7 && props->h_type != 4) return -1;
  Crys cr;
  crystal_finalize(*props, cr);
  VoxProps vp;
  voxel_props(cr, kocks_deg, vp);
  State n;
  std::memset(&n, 0, sizeof(n));
  n.mrr = true;
  if (hist_n) state_unpack(hist_n, n);
  else state_init(cr, n);
  Mrr mm{&cr.p, &vp, &n, cr.Gm, cr.Hm};
  Np1 s;
  M3 I = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  mm.setup(s, D, tinc, I, TEMP);
  if (R) mm.formR(s, x, R);
  if (J) mm.formJ(s, x, J);
  return 0;
}

void orc_polar(const double F[9], double R[9]) {
  M3 f, r;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) f[i][j] = F[3 * i + j];
  polar_R(f, r);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) R[3 * i + j] = r[i][j];
}

void orc_crystal_setup(const cpfft_crystal* props, const double kocks_deg[3], double C66[36],
                       double* ms, double* qs) {
  Crys cr;
  crystal_finalize(*props, cr);
  VoxProps vp;
  voxel_props(cr, kocks_deg, vp);
  for (int a = 0; a < 6; a++)
    for (int b = 0; b < 6; b++) C66[a * 6 + b] = vp.C[a][b];
  for (int s = 0; s < vp.ns; s++) {
    for (int a = 0; a < 6; a++) ms[s * 6 + a] = vp.ms[s][a];
    for (int a = 0; a < 3; a++) qs[s * 3 + a] = vp.qs[s][a];
  }
}

void orc_fft3(int N, double* re, double* im, int sign) {
  FFT1 f(N);
  fft3(f, re, im, sign);
}

}  // extern "C"
