// api.cu -- the C-ABI of include/cpfft_gpu.h: device context, material set-up, and the
// host-side control of the resident Newton-Krylov loop (FFT_nr3 / fftPcg /
// tangent_homo / NBC_update of src/FFT_nr3.f and src/tangent_homo.f).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <ctime>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "fft_green.cuh"
#include "mlp.cuh"

// element result text (results.cu)
void host_e15(double v, char* out);
cudaError_t launch_format_flat(const double* hist, long long N3, int word0, int nvals, char* text,
                               unsigned char* flags, cudaStream_t st);
cudaError_t launch_format_values(const double* x, long long n, char* out, unsigned char* flags,
                                 cudaStream_t st);

// nodal displacements (disp.cu)
cudaError_t f2disp_device(const double* F, int N, double lx, double ly, double lz,
                          const double* ctab, double* work, double* u, cudaStream_t st);

// the learned initial guess's device weights and error check (mlp.cu)
bool mlp_device_weights(mlp::Weights* w, int** err);
int mlp_check_error();
#include "krylov.cuh"

// per host thread: a thread drives one context (cpfft_batch_solve runs several at once)
static thread_local char g_err[512] = "";
thread_local long long g_kernel_launches = 0;
void cpfft_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

// cudaFuncSetAttribute acts on the current device, so the raised limit is kept per
// (device, kernel)
cudaError_t raise_max_dynamic_smem(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void*>, size_t> set;
  int dev = 0;
  cudaError_t ge = cudaGetDevice(&dev);
  if (ge != cudaSuccess) return ge;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = set[std::make_pair(dev, func)];
  if (bytes <= cur) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

namespace {

// ---- host-side material set-up (setup_mm10_rknstr, src/drive_eps_sig.f:537-1002;
//      finalize_new_crystal, src/mod_crystals.f:414-1931) --------------------------
const int VI[6] = {0, 1, 2, 0, 1, 0};
const int VJ[6] = {0, 1, 2, 1, 2, 2};

void fcc_geometry(double b[12][3], double n[12][3]) {
  const double f = 1.0 / std::sqrt(2.0), g = 1.0 / std::sqrt(3.0);
  // {111}<110>: direction and normal of each system, in the reference's order
  const double B[12][3] = {{0, -f, f}, {f, 0, -f}, {-f, f, 0}, {0, f, f}, {f, 0, f}, {f, -f, 0},
                           {0, -f, f}, {-f, 0, -f}, {f, f, 0}, {0, f, f}, {f, 0, -f}, {-f, -f, 0}};
  const double Nn[12][3] = {{g, g, g},  {g, g, g},  {g, g, g},  {-g, -g, g}, {-g, -g, g}, {-g, -g, g},
                            {-g, g, g}, {-g, g, g}, {-g, g, g}, {g, -g, g},  {g, -g, g},  {g, -g, g}};
  memcpy(b, B, sizeof(B));
  memcpy(n, Nn, sizeof(Nn));
}

// BCC {110}, {112}, {123} <111>, 48 systems in the reference's order and signs
// (slip_type 8, src/mod_crystals.f:812-1207): directions (+-1,+-1,+-1)/sqrt(3) and plane
// normals as integer Miller triples, each normalised by its length as the reference's
// constants are (1/sqrt(2), 1/sqrt(6), 2/sqrt(6), 1/sqrt(14), 2/sqrt(14), 3/sqrt(14)).
void bcc48_geometry(double b[48][3], double n[48][3]) {
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
  const double f3 = 1.0 / std::sqrt(3.0);
  for (int s = 0; s < 48; s++) {
    const double len = std::sqrt((double)(Nn[s][0] * Nn[s][0] + Nn[s][1] * Nn[s][1] + Nn[s][2] * Nn[s][2]));
    for (int i = 0; i < 3; i++) {
      b[s][i] = B[s][i] * f3;
      n[s][i] = (double)Nn[s][i] / len;
    }
  }
}

// The other 12-system cubic sets, directions and plane normals as integer Miller triples
// in the reference's order and signs, each normalised by its length (the reference's
// constants are 1/sqrt(2) and 1/sqrt(3)):
//   slip_type 2, bcc:     {110}<111> (src/mod_crystals.f:516-593)
//   slip_type 6, roters:  {111}<110>, the FCC systems in Roters' order (:604-704)
// slip_type 7 (bcc12, :705-811) is the first twelve systems of bcc48.
void miller_systems(const int B[12][3], const int Nn[12][3], double b[][3], double n[][3]) {
  for (int s = 0; s < 12; s++) {
    const double lb = std::sqrt((double)(B[s][0] * B[s][0] + B[s][1] * B[s][1] + B[s][2] * B[s][2]));
    const double ln = std::sqrt((double)(Nn[s][0] * Nn[s][0] + Nn[s][1] * Nn[s][1] + Nn[s][2] * Nn[s][2]));
    for (int i = 0; i < 3; i++) {
      b[s][i] = (double)B[s][i] / lb;
      n[s][i] = (double)Nn[s][i] / ln;
    }
  }
}

void bcc_geometry(double b[][3], double n[][3]) {
  static const int B[12][3] = {{1, 1, 1},   {1, 1, 1},   {1, 1, 1},   {-1, -1, 1},
                               {-1, -1, 1}, {-1, -1, 1}, {-1, 1, 1},  {-1, 1, 1},
                               {-1, 1, 1},  {1, -1, 1},  {1, -1, 1},  {1, -1, 1}};
  static const int Nn[12][3] = {{0, -1, 1}, {1, 0, -1}, {-1, 1, 0}, {0, 1, 1},
                                {1, 0, 1},  {1, -1, 0}, {0, -1, 1}, {-1, 0, -1},
                                {1, 1, 0},  {0, 1, 1},  {1, 0, -1}, {-1, -1, 0}};
  miller_systems(B, Nn, b, n);
}

void roters_geometry(double b[][3], double n[][3]) {
  static const int B[12][3] = {{1, -1, 0}, {1, 0, -1}, {0, 1, -1}, {1, 1, 0},
                               {1, 0, 1},  {0, 1, -1}, {1, 1, 0},  {1, 0, -1},
                               {0, 1, 1},  {1, -1, 0}, {1, 0, 1},  {0, 1, 1}};
  static const int Nn[12][3] = {{1, 1, 1},   {-1, -1, -1}, {1, 1, 1},   {1, -1, -1},
                                {-1, 1, 1},  {1, -1, -1},  {1, -1, 1},  {1, -1, 1},
                                {-1, 1, -1}, {-1, -1, 1},  {-1, -1, 1}, {1, 1, -1}};
  miller_systems(B, Nn, b, n);
}

// One system, direction x on the plane normal to y (slip_type 3 "single",
// src/mod_crystals.f:594-603).
void single_geometry(double b[][3], double n[][3]) {
  const double B[3] = {1.0, 0.0, 0.0}, Nn[3] = {0.0, 1.0, 0.0};
  for (int i = 0; i < 3; i++) { b[0][i] = B[i]; n[0][i] = Nn[i]; }
}

// HCP basal {0001}<11-20> (systems 1-3) and prismatic {10-10}<11-20> (4-6) systems in
// the reference's Cartesian frame, a1 along x and c along z (slip_type 9 "hcp6",
// src/mod_crystals.f:1208-1476), written with h = sqrt(3)/2 as the reference does.
// slip_type 10 "hcp18" declares 18 systems but assigns only these six (its pyramidal
// <c+a> systems are commented out, :1477-1759), so its other twelve keep zero vectors:
// they never slip and add exact zeros to every sum, and an hcp18 grid runs the same
// arithmetic on these six.
void hcp6_geometry(double b[][3], double n[][3]) {
  const double h = std::sqrt(3.0) / 2.0;
  const double B[6][3] = {{0.5, -h, 0.0}, {0.5, h, 0.0}, {-1.0, 0.0, 0.0},
                          {1.0, 0.0, 0.0}, {0.5, h, 0.0}, {-0.5, h, 0.0}};
  const double Nn[6][3] = {{0.0, 0.0, 1.0}, {0.0, 0.0, 1.0}, {0.0, 0.0, 1.0},
                           {0.0, 1.0, 0.0}, {-h, 0.5, 0.0}, {-h, -0.5, 0.0}};
  for (int s = 0; s < 6; s++)
    for (int i = 0; i < 3; i++) { b[s][i] = B[s][i]; n[s][i] = Nn[s][i]; }
}

// slip systems of a slip_type as the stress kernels see them: 1 (single), 6 (hcp6,
// hcp18), 12 (fcc, bcc, roters, bcc12) or 48 (bcc48); 0 when not supported
int slip_geometry(int slip_type, double b[48][3], double n[48][3]) {
  if (slip_type == 3) {
    single_geometry(b, n);
    return 1;
  }
  if (slip_type == 9 || slip_type == 10) {
    hcp6_geometry(b, n);
    return 6;
  }
  if (slip_type == 1) {
    double bf[12][3], nf[12][3];
    fcc_geometry(bf, nf);
    memcpy(b, bf, sizeof(bf));
    memcpy(n, nf, sizeof(nf));
    return 12;
  }
  if (slip_type == 2) {
    bcc_geometry(b, n);
    return 12;
  }
  if (slip_type == 6) {
    roters_geometry(b, n);
    return 12;
  }
  if (slip_type == 7) {
    bcc48_geometry(b, n);
    return 12;
  }
  if (slip_type == 8) {
    bcc48_geometry(b, n);
    return 48;
  }
  return 0;
}

bool invert6(const double a[36], double out[36]) {
  double m[6][12];
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 12; j++) m[i][j] = j < 6 ? a[6 * i + j] : (j - 6 == i ? 1.0 : 0.0);
  for (int k = 0; k < 6; k++) {
    int p = k;
    for (int i = k + 1; i < 6; i++)
      if (std::fabs(m[i][k]) > std::fabs(m[p][k])) p = i;
    if (m[p][k] == 0.0) return false;
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
    for (int j = 0; j < 6; j++) out[6 * i + j] = m[i][j + 6];
  return true;
}

// stiffness in the crystal frame (src/mod_crystals.f:1796-1880)
bool crystal_stiffness(const cpfft_crystal& p, double C0[36]) {
  memset(C0, 0, 36 * sizeof(double));
  if (p.elastic_type == 3) {
    C0[0] = p.C11; C0[1] = p.C12; C0[2] = p.C13;
    C0[6] = p.C12; C0[7] = p.C11; C0[8] = p.C13;
    C0[12] = p.C13; C0[13] = p.C13; C0[14] = p.C33;
    C0[21] = p.C44; C0[28] = p.C55; C0[35] = p.C55;
    return true;
  }
  if (p.elastic_type != 1 && p.elastic_type != 2) return false;
  double flex[36] = {0};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) flex[6 * i + j] = i == j ? 1.0 / p.e : -p.nu / p.e;
  double sh = p.elastic_type == 1 ? 2.0 * (1.0 + p.nu) / p.e : 1.0 / p.mu;
  for (int i = 3; i < 6; i++) flex[6 * i + i] = sh;
  return invert6(flex, C0);
}

void kocks_rotation(const double ang[3], double r[9]) {  // src/mm10_a.f:1287-1345
  const double pi = 3.141592653589793;
  double psi = ang[0] * pi / 180.0, th = ang[1] * pi / 180.0, phi = ang[2] * pi / 180.0;
  r[0] = -sin(psi) * sin(phi) - cos(psi) * cos(phi) * cos(th);
  r[1] = cos(psi) * sin(phi) - sin(psi) * cos(phi) * cos(th);
  r[2] = cos(phi) * sin(th);
  r[3] = sin(psi) * cos(phi) - cos(psi) * sin(phi) * cos(th);
  r[4] = -cos(psi) * cos(phi) - sin(psi) * sin(phi) * cos(th);
  r[5] = sin(phi) * sin(th);
  r[6] = cos(psi) * sin(th);
  r[7] = sin(psi) * sin(th);
  r[8] = cos(th);
}

void orientation_record(const double C0[36], const double bb[48][3], const double nn[48][3],
                        int nslip, const double ang[3], OriRec& o) {
  double g[9], tr[9];
  kocks_rotation(ang, g);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) tr[3 * i + j] = g[3 * j + i];
  for (int s = 0; s < nslip; s++) {
    double bs[3], ns[3];
    for (int i = 0; i < 3; i++) {
      bs[i] = tr[3 * i] * bb[s][0] + tr[3 * i + 1] * bb[s][1] + tr[3 * i + 2] * bb[s][2];
      ns[i] = tr[3 * i] * nn[s][0] + tr[3 * i + 1] * nn[s][1] + tr[3 * i + 2] * nn[s][2];
    }
    double A[3][3];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) A[i][j] = bs[i] * ns[j];
    for (int a = 0; a < 6; a++) {
      double sym = 0.5 * (A[VI[a]][VJ[a]] + A[VJ[a]][VI[a]]);
      o.ms[6 * s + a] = a < 3 ? sym : 2.0 * sym;
    }
    o.qs[3 * s + 0] = 0.5 * (A[1][2] - A[2][1]);
    o.qs[3 * s + 1] = 0.5 * (A[0][2] - A[2][0]);
    o.qs[3 * s + 2] = 0.5 * (A[0][1] - A[1][0]);
  }
  for (int i = 0; i < 9; i++) o.g[i] = tr[i];
  double Rs[36], tmp[36];
  for (int a = 0; a < 6; a++)
    for (int b = 0; b < 6; b++) {
      int ia = VI[a], ja = VJ[a], kb = VI[b], lb = VJ[b];
      Rs[6 * a + b] = b < 3 ? tr[3 * ia + kb] * tr[3 * ja + kb]
                            : tr[3 * ia + kb] * tr[3 * ja + lb] + tr[3 * ia + lb] * tr[3 * ja + kb];
    }
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) {
      double s = 0;
      for (int k = 0; k < 6; k++) s += C0[6 * i + k] * Rs[6 * j + k];
      tmp[6 * i + j] = s;
    }
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) {
      double s = 0;
      for (int k = 0; k < 6; k++) s += Rs[6 * i + k] * tmp[6 * k + j];
      o.C[6 * i + j] = s;
    }
}

// Ma-Roters-Raabe interaction matrices of a 12-system slip type (mm10_mrr_GH's tables
// mm10_mrr_GHfcc / GHbcc / GHfcc12 / GHbcc12, src/mm10_e.f:16-1424, formed here from the
// geometry): Gm(a,q) = |n_a . t_q| (forest projection), Hm(a,q) = |n_a x t_q| (parallel),
// t_q = n_q x b_q the edge dislocation line of system q
void mrr_interaction(int slip_type, double Gm[144], double Hm[144]) {
  double b[48][3], n[48][3];
  slip_geometry(slip_type, b, n);
  for (int a = 0; a < 12; a++)
    for (int q = 0; q < 12; q++) {
      double t[3] = {n[q][1] * b[q][2] - n[q][2] * b[q][1], n[q][2] * b[q][0] - n[q][0] * b[q][2],
                     n[q][0] * b[q][1] - n[q][1] * b[q][0]};
      const double tl = std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
      for (int k = 0; k < 3; k++) t[k] /= tl;
      const double x[3] = {n[a][1] * t[2] - n[a][2] * t[1], n[a][2] * t[0] - n[a][0] * t[2],
                           n[a][0] * t[1] - n[a][1] * t[0]};
      Gm[12 * a + q] = std::fabs(n[a][0] * t[0] + n[a][1] * t[1] + n[a][2] * t[2]);
      Hm[12 * a + q] = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    }
}

CrysRec crystal_record(const cpfft_crystal& p) {
  CrysRec c;
  std::memset(&c, 0, sizeof(c));
  c.rate_n = p.harden_n;
  c.tau_y = p.tau_y;
  c.tau_v = p.tau_v;
  c.inv_tau_v = 1.0 / p.tau_v;
  c.theta_0 = p.theta_0;
  c.voce_m = p.voce_m;
  c.gamma_bar = p.gamma_bar;
  c.iD_v = p.h_type == 2 ? 0.0 : p.iD_v;  // MTS has no diffusion slip term (src/mm10_b.f:1191-1197)
  c.atol = p.atol;
  c.atol1 = p.atol1;
  c.rtol = p.rtol;
  c.rtol1 = p.rtol1;
  c.tau_a = p.tau_a;
  c.tau_hat_y = p.tau_hat_y;
  c.G_0_y = p.G_0_y;
  c.p_y = p.p_y;
  c.q_y = p.q_y;
  c.tau_hat_v = p.tau_hat_v;
  c.G_0_v = p.G_0_v;
  c.p_v = p.p_v;
  c.q_v = p.q_v;
  c.eps_dot_0_v = p.eps_dot_0_v;
  c.burgers = p.burgers;
  c.boltzman = p.boltzman;
  c.mu_0 = p.mu_0;
  c.D_0 = p.D_0;
  c.T_0 = p.T_0;
  c.u1 = p.u1;
  c.u2 = p.u2;
  c.u3 = p.u3;
  c.u4 = p.u4;
  c.u5 = p.u5;
  c.u6 = p.u6;
  if (p.h_type == 7 || p.h_type == 4) mrr_interaction(p.slip_type, c.Gm, c.Hm);
  c.h_type = p.h_type;
  c.miter = p.miter;
  c.alter_mode = p.alter_mode;
  c.exact_j22 = p.exact_j22;
  double r = std::round(p.harden_n);
  c.n_int = (r == p.harden_n && r >= 2.0 && r <= 64.0) ? (int)r - 1 : -1;
  c.m_is_one = p.voce_m == 1.0;
  return c;
}

// ---- device context -------------------------------------------------------------
struct Ctx {
  int N = 0;
  long long N3 = 0;
  double dt = 0;
  int prec = CPFFT_PREC_FP64, warm = 0;
  int nslip = 12;  // slip systems of the grid's stress kernel (1, 6, 12 or 48)
  int h_type = 1;  // hardening law of the grid's crystals (1 voce, 2 mts, 7 mrr)
  int hist_words = H_WORDS;  // H_WORDS_MRR on dislocation-density grids (MRR, ORNL)
  int pass_step = 0, pass_iter = -1;  // the last stress pass (its state is in history n+1)
  // voxel work queue of the implicit stress passes (cpfft_set_schedule)
  int sched = CPFFT_SCHED_BLOCKS;
  int tangent_f32 = 0;  // mixed precision: the consistent tangent in FP32 (CPFFT_TANGENT_F32)
  unsigned char* vcost = nullptr;  // (N3) local iterations of each voxel's last implicit pass
  int* vperm = nullptr;            // (N3) queue order
  unsigned int* vq = nullptr;      // 2 x 64 bin counters / offsets + the queue head
  int qchunk = 128;                // voxels a block takes from the queue at a time
  int qbps = 0;                    // persistent blocks per SM (0: as many as fit)
  bool qtuned = false;             // the chunk has been autotuned (first implicit queue pass)
  // tuning times: chunks 128 / 256 / 512 with as many blocks per SM as fit, then with one
  float qchunk_ms[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  cudaStream_t st = nullptr;
  GridDesc g;
  double *Fn = nullptr, *Fn1 = nullptr, *P = nullptr, *K4 = nullptr, *b = nullptr, *dFm = nullptr;
  double *r = nullptr, *p = nullptr, *Ap = nullptr, *w = nullptr, *io = nullptr;
  double* w2 = nullptr;  // mixed precision: FP64 copy of an inner correction
  float* th_x = nullptr;  // mixed precision: tangent_homo's 9 solutions of the last call
                          // (FP32: they only start the next call's solves)
  bool th_valid = false;
  // logging of (features, converged increments) pairs for the learned initial guess
  float *log_X = nullptr, *log_T = nullptr;
  unsigned long long* log_n = nullptr;
  long long log_cap = 0;
  int log_stride = 1, log_phase = 0;
  bool log = false;      // CPFFT_LOG=1: the reference's residual reports on stderr
  double* hist[2] = {nullptr, nullptr};
  int hn = 0;  // index of the history at n
  float *K4f = nullptr, *xf = nullptr, *rf = nullptr, *pf = nullptr, *Apf = nullptr;
  // mixed precision: FP64-accurate operator in double-float (power-of-two N 32..256):
  // K4 = K4f + K4lo to 48 bits, double-float twiddles
  float* K4lo = nullptr;
  dfl2* twdf = nullptr;
  bool df_ok = false;
  GridDesc gdf;            // the double-float operator's tile shapes (autotuned)
  float tune_ms[2] = {0.f, 0.f};  // autotuned time per apply: FP32, double-float
  int *ori = nullptr, *crys = nullptr;
  OriRec* oris = nullptr;
  CrysRec* cryss = nullptr;
  // materials: 0-based material of every voxel; per material 0 = crystal, 1 = mm01
  // (cpfft_set_mises), 2 = declared non-crystal and not yet defined
  std::vector<int> mat;
  std::vector<int> mat_kind;
  long long n_crys_vox = 0, n_mises_vox = 0, n_undef_vox = 0;
  std::vector<MisesRec> h_mises;  // per material (index = material)
  int* mises = nullptr;           // (N3) material of an mm01 voxel, -1 for a crystal voxel
  MisesRec* misess = nullptr;     // per material
  double2* S = nullptr;
  float2* Sf = nullptr;
  double2* tw = nullptr;
  float2* twf = nullptr;
  double *part = nullptr, *sc = nullptr, *h_sc = nullptr;
  unsigned long long* stats = nullptr;
  unsigned long long* h_stats = nullptr;
  bool K4f_valid = false;
  // the preconditioned FP32 CG iteration as a graph: a WHILE node around one iteration
  // (p update, G0(K:p) with alpha, x/r update with beta, stop test)
  cudaGraph_t cg_graph = nullptr;
  cudaGraphExec_t cg_exec = nullptr;
  cudaGraphConditionalHandle cg_handle = 0;
  int cg_graph_state = 0;         // 0 not built, 1 built, -1 unavailable (eager iterations)
  long long cg_body_launches = 0; // kernels of one iteration
  // reference-medium preconditioner of the FP32 inner iterations (cpfft_set_precond)
  int precond = 0;
  bool pre_ok = false;     // the current reference medium is usable
  double* k0sum = nullptr; // (81) component sums of K4f
  double* h_k0 = nullptr;  // pinned (81) copy
  float* h_pre = nullptr;  // pinned: 36 acoustic coefficients + 81 entries of K0
  float* pre_dev = nullptr;  // the same on the device (read by the preconditioned kernels)
  // FFT_nr3 locals that persist across steps (Fortran DATA => SAVE, src/FFT_nr3.f:29-34)
  double barF_t[9], P_bar[9], C_homo[81];
  // equilibrium stop test of the Newton loop (cpfft_set_equilibrium_tol; 0 = the reference's)
  double eq_tol = 0.0;
  // inexact Newton (cpfft_set_inexact_newton; 0 = every Krylov solve to tolPCG): the
  // largest relative tolerance of a Newton system's solve
  double eta_max = 0.0;
  // relative tolerance of tangent_homo's solves under inexact Newton (cpfft_set_tangent_tol)
  double th_tol = 1.0e-2;
  // the P_bar update inside the Newton iteration (cpfft_set_coupled_bc: 0 off, 1 on,
  // 2 on with an implicit first stress pass)
  int coupled_bc = 0;
  bool cg_rel_only = false;  // the current solve stops on ||r|| <= tol ||b|| alone
  // counters of the last stress pass: local iterations, fallbacks, predictor iterations,
  // starts dropped, sub-stepped solves (cpfft_pass_counts)
  long long last_pass[5] = {0, 0, 0, 0, 0};
  // counters of the current step
  long long cg_iters = 0, cg_solves = 0, f64_matvecs = 0, f32_matvecs = 0;
  long long syncs = 0;  // host waits on the stream
  // CUDA-event timing of every stress / Green launch on the library stream
  static const int KT_CAP = 512;
  cudaEvent_t kt_ev[2 * KT_CAP];
  int kt_kind[KT_CAP];
  int kt_used = 0;
  bool kt_ready = false;
  double kt_acc[4] = {0, 0, 0, 0};
  long long kt_cnt[4] = {0, 0, 0, 0};
  cudaEvent_t step_ev[2];
};

enum { KT_STRESS = 0, KT_G64 = 1, KT_G32 = 2, KT_CGGRAPH = 3 };

int kt_drain(Ctx* c) {
  if (!c->kt_used) return 0;
  if (cudaStreamSynchronize(c->st) != cudaSuccess) {
    cpfft_set_error("stream synchronize failed");
    return CPFFT_ERR_CUDA;
  }
  for (int i = 0; i < c->kt_used; i++) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->kt_ev[2 * i], c->kt_ev[2 * i + 1]);
    c->kt_acc[c->kt_kind[i]] += 1e-3 * ms;
    c->kt_cnt[c->kt_kind[i]]++;
  }
  c->kt_used = 0;
  return 0;
}
void kt_start(Ctx* c, int kind) {
  if (!c->kt_ready) return;
  c->kt_kind[c->kt_used] = kind;
  cudaEventRecord(c->kt_ev[2 * c->kt_used], c->st);
}
int kt_stop(Ctx* c) {
  if (!c->kt_ready) return 0;
  cudaEventRecord(c->kt_ev[2 * c->kt_used + 1], c->st);
  if (++c->kt_used == Ctx::KT_CAP) return kt_drain(c);
  return 0;
}
void kt_reset(Ctx* c) {
  for (int k = 0; k < 4; k++) { c->kt_acc[k] = 0; c->kt_cnt[k] = 0; }
}
thread_local Ctx* g_ctx = nullptr;

#define TRY(expr)                 \
  do {                            \
    int _rc = (expr);             \
    if (_rc) return _rc;          \
  } while (0)

template <typename Ptr>
int dalloc(Ptr& p, size_t bytes) {
  cudaError_t e = cudaMalloc((void**)&p, bytes);
  if (e != cudaSuccess) {
    cpfft_set_error("cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    p = nullptr;
    return CPFFT_ERR_NO_MEMORY;
  }
  return 0;
}

void free_ctx(Ctx* c) {
  if (!c) return;
  void* ptrs[] = {c->log_X, c->log_T, c->log_n,
                  c->Fn, c->Fn1, c->P, c->K4, c->b, c->dFm, c->r, c->p, c->Ap, c->w, c->io, c->w2, c->th_x,
                  c->hist[0], c->hist[1], c->K4f, c->xf, c->rf, c->pf, c->Apf, c->ori, c->crys,
                  c->oris, c->cryss, c->S, c->Sf, c->tw, c->twf, c->part, c->sc, c->stats,
                  c->k0sum, c->K4lo, c->twdf, c->vcost, c->vperm, c->vq, c->pre_dev,
                  c->mises, c->misess};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (c->h_sc) cudaFreeHost(c->h_sc);
  if (c->h_stats) cudaFreeHost(c->h_stats);
  if (c->h_k0) cudaFreeHost(c->h_k0);
  if (c->h_pre) cudaFreeHost(c->h_pre);
  if (c->kt_ready) {
    for (int i = 0; i < 2 * Ctx::KT_CAP; i++) cudaEventDestroy(c->kt_ev[i]);
    cudaEventDestroy(c->step_ev[0]);
    cudaEventDestroy(c->step_ev[1]);
  }
  if (c->cg_exec) cudaGraphExecDestroy(c->cg_exec);
  if (c->cg_graph) cudaGraphDestroy(c->cg_graph);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

int cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    cpfft_set_error("%s: %s", what, cudaGetErrorString(e));
    return CPFFT_ERR_CUDA;
  }
  return 0;
}
#define CK(expr) TRY(cuda_check((expr), #expr))

int sync(Ctx* c) {
  c->syncs++;
  return cuda_check(cudaStreamSynchronize(c->st), "stream synchronize");
}

int read_scalar(Ctx* c, int slot, double* out) {
  CK(cudaMemcpyAsync(c->h_sc + slot, c->sc + slot, sizeof(double), cudaMemcpyDeviceToHost, c->st));
  TRY(sync(c));
  *out = c->h_sc[slot];
  return 0;
}

int dnrm2(Ctx* c, const double* x, double* out) {
  CK(dev_dot(x, x, 9 * c->N3, c->part, c->sc, SC_TMP, OP_STORE, c->st));
  double v;
  TRY(read_scalar(c, SC_TMP, &v));
  *out = std::sqrt(v);
  return 0;
}

// ||g|| / (sqrt(N3) ||mean of P||) with g = G(P): the equilibrium residual of the current
// state (one synchronisation)
int equil_residual(Ctx* c, const double* g, double* out) {
  CK(dev_dot(g, g, 9 * c->N3, c->part, c->sc, SC_TMP, OP_STORE, c->st));
  CK(dev_sum9(c->P, c->N3, c->part, c->sc, SC_SUM9, c->st));
  CK(cudaMemcpyAsync(c->h_sc + SC_TMP, c->sc + SC_TMP, (SC_SUM9 + 9 - SC_TMP) * sizeof(double),
                     cudaMemcpyDeviceToHost, c->st));
  TRY(sync(c));
  double pb = 0;
  for (int i = 0; i < 9; i++) {
    const double m = c->h_sc[SC_SUM9 + i] / (double)c->N3;
    pb += m * m;
  }
  *out = std::sqrt(c->h_sc[SC_TMP]) / (std::sqrt((double)c->N3) * std::sqrt(pb));
  return 0;
}

// FP64 matvec y = G(K4:x) or G(x)
int matvec64(Ctx* c, const double* x, double* y, int flgK) {
  c->f64_matvecs++;
  kt_start(c, KT_G64);
  TRY(cuda_check(green_apply<double>(x, c->K4, flgK, y, c->S, c->tw, c->g, c->st), "green_apply fp64"));
  return kt_stop(c);
}

// The FP64-accurate operator of the solver: mixed precision evaluates it in double-float
// on the FP32 pipes where the grid allows (about 1e-13 relative to the FP64 operator, far
// inside the 1e-10 CG tolerance it serves), the plain form in native FP64.
int matvec_acc(Ctx* c, const double* x, double* y, int flgK) {
  if (!(c->prec == CPFFT_PREC_MIXED && c->df_ok && (c->K4f_valid || !flgK)))
    return matvec64(c, x, y, flgK);
  c->f64_matvecs++;
  kt_start(c, KT_G64);
  TRY(cuda_check(green_apply_df(x, c->K4f, c->K4lo, flgK, y, reinterpret_cast<dfl2*>(c->S),
                                c->twdf, c->gdf, c->st),
                 "green_apply double-float"));
  return kt_stop(c);
}
// y = G(K4f : x) and sc[SC_PAP] = x . y with alpha = rr / (x . y): the product is summed
// inside the last FFT pass where that pass supports it, else by a separate reduction
int matvec32_alpha(Ctx* c, const float* x, float* y) {
  c->f32_matvecs++;
  kt_start(c, KT_G32);
  int np = 0;
  TRY(cuda_check(green_apply_dot<float>(x, c->K4f, 1, y, c->Sf, c->twf, c->g, c->st, c->part, &np),
                 "green_apply fp32"));
  TRY(kt_stop(c));
  if (np) CK(dev_final(c->part, np, c->sc, SC_PAP, OP_ALPHA, c->st));
  else CK(dev_dot_f(x, y, 9 * c->N3, c->part, c->sc, SC_PAP, OP_ALPHA, c->st));
  return 0;
}

// ---- reference-medium preconditioning of the FP32 inner iterations -------------------
// The inner system G(K : x) = b is solved as G0(K : x) = G0(b), G0 the Green operator of a
// homogeneous reference medium K0 (the symmetrised volume average of the current tangent).
// Both have the same solutions on compatible fields (G0 o G = G0, and G0 annihilates
// exactly the divergence-free fields), and G0(K : .) is self-adjoint in the inner product
// <a, b>_K0 on compatible fields, where CG on it is CG preconditioned by G(K0 : .).  Its
// iteration count follows the contrast of K against K0 instead of against the identity.

// Sums of K4f (after a stress update or an uploaded tangent), read back with the stream's
// next synchronisation; reference_build then forms the medium.
int reference_reduce(Ctx* c) {
  if (!c->k0sum) {
    TRY(dalloc(c->k0sum, 81 * sizeof(double)));
    TRY(dalloc(c->pre_dev, (36 + 81) * sizeof(float)));
    c->g.acoef = c->pre_dev;
    if (cudaMallocHost((void**)&c->h_k0, 81 * sizeof(double)) != cudaSuccess ||
        cudaMallocHost((void**)&c->h_pre, (36 + 81) * sizeof(float)) != cudaSuccess) {
      cpfft_set_error("cudaMallocHost failed");
      return CPFFT_ERR_NO_MEMORY;
    }
  }
  CK(dev_mean81(c->K4f, c->N3, c->part, c->k0sum, c->st));
  CK(cudaMemcpyAsync(c->h_k0, c->k0sum, 81 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  return 0;
}

// K0 = sym(mean K4) / its largest entry; usable when the acoustic tensor
// A0(n)_ik = K0_ijkl n_j n_l is positive definite on a dense set of directions n.
int reference_build(Ctx* c) {
  double K0[81], mx = 0.0;
  for (int I = 0; I < 9; I++)
    for (int J = 0; J < 9; J++) {
      K0[9 * I + J] = 0.5 * (c->h_k0[9 * I + J] + c->h_k0[9 * J + I]) / (double)c->N3;
      mx = std::max(mx, std::fabs(K0[9 * I + J]));
    }
  c->pre_ok = false;
  if (!(mx > 0.0) || !std::isfinite(mx)) return 0;
  for (double& k : K0) k /= mx;
  static const int RI[6] = {0, 1, 2, 0, 1, 0}, RK[6] = {0, 1, 2, 1, 2, 2};
  static const int PJ[6] = {0, 1, 2, 0, 1, 0}, PL[6] = {0, 1, 2, 1, 2, 2};
  double coef[36];
  for (int r = 0; r < 6; r++)
    for (int m = 0; m < 6; m++) {
      const int i = RI[r], k = RK[r], j = PJ[m], l = PL[m];
      double v = K0[9 * (3 * i + j) + 3 * k + l];
      if (j != l) v += K0[9 * (3 * i + l) + 3 * k + j];
      coef[6 * r + m] = v;
    }
  // positive definiteness (Sylvester) with a margin, on 64 x 128 directions of the sphere
  const double pi = 3.14159265358979323846;
  double lo = 1e300, hi = 0.0;
  for (int it = 0; it <= 64; it++)
    for (int ip = 0; ip < 128; ip++) {
      const double th = pi * it / 64.0, ph = 2.0 * pi * ip / 128.0;
      const double n[3] = {std::sin(th) * std::cos(ph), std::sin(th) * std::sin(ph), std::cos(th)};
      const double pr[6] = {n[0] * n[0], n[1] * n[1], n[2] * n[2], n[0] * n[1], n[1] * n[2], n[0] * n[2]};
      double a[6];
      for (int r = 0; r < 6; r++) {
        a[r] = 0.0;
        for (int m = 0; m < 6; m++) a[r] += coef[6 * r + m] * pr[m];
      }
      const double m2 = a[0] * a[1] - a[3] * a[3];
      const double det = a[0] * (a[1] * a[2] - a[4] * a[4]) - a[3] * (a[3] * a[2] - a[4] * a[5]) +
                         a[5] * (a[3] * a[4] - a[1] * a[5]);
      const double tr = a[0] + a[1] + a[2];
      if (!(a[0] > 0.0 && m2 > 0.0 && det > 0.0 && tr > 0.0)) return 0;
      // det / tr^3 bounds the smallest eigenvalue's share from below
      lo = std::min(lo, det / (tr * tr * tr));
      hi = std::max(hi, tr);
    }
  if (c->log)
    fprintf(stderr, "         reference medium: min det/tr^3 of the acoustic tensor %.3e%s\n", lo,
            lo > 1.0e-9 ? "" : " (not used)");
  if (!(lo > 1.0e-9)) return 0;
  for (int k = 0; k < 36; k++) c->h_pre[k] = (float)coef[k];
  for (int k = 0; k < 81; k++) c->h_pre[36 + k] = (float)K0[k];
  CK(cudaMemcpyAsync(c->pre_dev, c->h_pre, (36 + 81) * sizeof(float), cudaMemcpyHostToDevice,
                     c->st));
  c->pre_ok = true;
  return 0;
}

// the preconditioned operator is a projection for odd N or the centered mapping
bool pre_applies(const Ctx* c) {
  return c->precond && c->prec == CPFFT_PREC_MIXED &&
         (c->g.gmap == CPFFT_G_CENTERED || (c->N & 1));
}

// y = G0(K4f : x) (flgK = 1) or G0(x); with want_alpha also sc[SC_PAP] = <K4f : x, x>
// (= <x, y>_K0) and alpha = rr / pAp
int matvec32_pre(Ctx* c, const float* x, float* y, int flgK, bool want_alpha) {
  c->f32_matvecs++;
  GridDesc g = c->g;
  g.pre = 1;
  int np = 0;
  kt_start(c, KT_G32);
  TRY(cuda_check(green_apply_dot<float>(x, c->K4f, flgK, y, c->Sf, c->twf, g, c->st,
                                        want_alpha ? c->part : nullptr, &np),
                 "green_apply fp32 (reference medium)"));
  TRY(kt_stop(c));
  if (want_alpha) {
    if (!np) {
      cpfft_set_error("internal: the preconditioned product was not fused");
      return CPFFT_ERR_CUDA;
    }
    CK(dev_final(c->part, np, c->sc, SC_PAP, OP_ALPHA, c->st));
  }
  return 0;
}

// fftPcg (src/FFT_nr3.f:214-360), plain FP64: CG from x = 0 with the stop test
// ||r|| <= tol*||b|| .or. ||r|| <= tol and at most 1000 iterations
int cg64(Ctx* c, const double* b, double* x, double tol, int* iters) {
  const long long n = 9 * c->N3;
  const int maxIter = 1000;
  *iters = 0;
  CK(cudaMemsetAsync(x, 0, n * sizeof(double), c->st));
  double n2b;
  TRY(dnrm2(c, b, &n2b));
  if (!(tol > 2.220446049250313e-16 && tol < 1.0)) return CPFFT_ERR_CG_TOL;
  if (!std::isfinite(n2b)) { cpfft_set_error("non-finite CG right-hand side"); return CPFFT_ERR_NONFINITE; }
  if (n2b <= 2.220446049250313e-16) return 0;
  const double tolb = tol * n2b;
  CK(cudaMemcpyAsync(c->r, b, n * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
  CK(cudaMemcpyAsync(c->p, b, n * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
  CK(dev_dot(c->r, c->r, n, c->part, c->sc, SC_RR, OP_STORE, c->st));
  int it = 0;
  for (;;) {
    TRY(matvec64(c, c->p, c->Ap, 1));
    CK(dev_dot(c->p, c->Ap, n, c->part, c->sc, SC_PAP, OP_ALPHA, c->st));
    CK(dev_cg_xr<double>(x, c->r, c->p, c->Ap, n, c->part, c->sc, c->st));
    it++;
    double rr;
    TRY(read_scalar(c, SC_RRNEW, &rr));
    double rn = std::sqrt(rr);
    if (!std::isfinite(rn)) { *iters = it; cpfft_set_error("CG residual is not finite"); return CPFFT_ERR_NONFINITE; }
    if (rn <= tolb || rn <= tol || it >= maxIter) break;
    CK(dev_cg_p<double>(c->p, c->r, n, c->sc, c->st));
  }
  *iters = it;
  c->cg_iters += it;
  c->cg_solves++;
  return it >= maxIter ? CPFFT_ERR_CG_MAXIT : 0;
}

// Mixed precision: FP32 Green/FFT/CG inner solves corrected by an FP64 outer residual
// (iterative refinement).  Same stop test on the FP64 residual as cg64.
// Reduction of the residual norm per segment of FP32 iterations before a reliable
// update.  Tight solves take 1e-2 (1e-3 lets the FP32 recursion drift until the solve
// stagnates, measured at 128^3); a solve to tol >= 1e-4 runs in one segment to its
// tolerance, where the recursion's drift (about 1e-7 of the starting residual) stays
// far below what the solve asks.
double reliable_delta(double tol) { return tol >= 1.0e-4 ? std::min(1.0e-2, 0.5 * tol) : 1.0e-2; }

int cg_mixed(Ctx* c, const double* b, double* x, double tol, int* iters, bool use_x0) {
  const long long n = 9 * c->N3;
  const int maxIter = 2000;     // FP32 iterations (the FP64 path's cap is 1000)
  const double delta = reliable_delta(tol);  // reliable-update threshold
  *iters = 0;
  if (!use_x0) CK(cudaMemsetAsync(x, 0, n * sizeof(double), c->st));
  double n2b;
  TRY(dnrm2(c, b, &n2b));
  if (!(tol > 2.220446049250313e-16 && tol < 1.0)) return CPFFT_ERR_CG_TOL;
  if (!std::isfinite(n2b)) { cpfft_set_error("non-finite CG right-hand side"); return CPFFT_ERR_NONFINITE; }
  if (n2b <= 2.220446049250313e-16) return 0;
  if (!c->K4f_valid) {
    cpfft_set_error("mixed precision CG needs the FP32 tangent of a stress update");
    return CPFFT_ERR_BAD_ARG;
  }
  const double tolb = tol * n2b;
  // the reference's absolute test ||r|| <= tol, off for the inexact Newton solves
  const double tola = c->cg_rel_only ? 0.0 : tol;
  // FP32 CG on scaled vectors (rf = r / ||r_true||) with reliable updates: whenever the
  // recursive FP32 residual has dropped by `delta` since the last true residual, the
  // FP32 increment is projected and added to x in FP64, the true residual
  // b - G(K4 : x) is recomputed in FP64, and the recursion continues from it with the
  // same search direction (rescaled).  The stop test is the reference's, on the FP64
  // residual.  The FP64 projection G keeps x in the range of G (compatible, zero-mean
  // fields) where every FP64 CG iterate lives: FP32 rounding leaks into the kernel of G,
  // which the residual cannot see.
  double rn = n2b;
  if (use_x0) {
    // start from the caller's x (kept in the range of G): r = b - G(K4 : x) in FP64
    TRY(matvec_acc(c, x, c->Ap, 1));
    CK(dev_sub(c->w, b, c->Ap, n, c->st));
    TRY(dnrm2(c, c->w, &rn));
    if (!std::isfinite(rn)) { cpfft_set_error("FP64 residual is not finite"); return CPFFT_ERR_NONFINITE; }
    if (rn <= tolb || rn <= tola) {
      c->cg_solves++;
      return 0;
    }
  } else {
    CK(cudaMemcpyAsync(c->w, b, n * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
  }
  double scale = 1.0 / rn, maxr = rn;
  CK(dev_to_f32(c->rf, c->w, scale, n, c->st));
  CK(cudaMemsetAsync(c->xf, 0, n * sizeof(float), c->st));
  CK(cudaMemcpyAsync(c->pf, c->rf, n * sizeof(float), cudaMemcpyDeviceToDevice, c->st));
  CK(dev_dot_f(c->rf, c->rf, n, c->part, c->sc, SC_RR, OP_STORE, c->st));
  double rr_prev;
  TRY(read_scalar(c, SC_RR, &rr_prev));
  int it = 0;
  bool converged = false;
  int restarts = 0;
  for (;;) {
    TRY(matvec32_alpha(c, c->pf, c->Apf));
    CK(dev_cg_xr<float>(c->xf, c->rf, c->pf, c->Apf, n, c->part, c->sc, c->st));
    it++;
    double rr;
    TRY(read_scalar(c, SC_RRNEW, &rr));
    if (!std::isfinite(rr)) { cpfft_set_error("FP32 CG residual is not finite"); return CPFFT_ERR_NONFINITE; }
    const double rest = std::sqrt(rr) / scale;
    if (rest < delta * maxr || rest <= tolb || rest <= tola || it >= maxIter) {
      // reliable update
      restarts++;
      CK(cudaMemsetAsync(c->w2, 0, n * sizeof(double), c->st));
      CK(dev_add_f32(c->w2, c->xf, 1.0 / scale, n, c->st));
      TRY(matvec_acc(c, c->w2, c->Ap, 0));
      CK(dev_axpy(x, c->Ap, 1.0, n, c->st));
      TRY(matvec_acc(c, x, c->Ap, 1));
      CK(dev_sub(c->w, b, c->Ap, n, c->st));
      TRY(dnrm2(c, c->w, &rn));
      if (!std::isfinite(rn)) { cpfft_set_error("FP64 residual is not finite"); return CPFFT_ERR_NONFINITE; }
      if (rn <= tolb || rn <= tola) { converged = true; break; }
      if (it >= maxIter) break;
      const double nscale = 1.0 / rn, k = nscale / scale;
      CK(dev_to_f32(c->rf, c->w, nscale, n, c->st));
      CK(cudaMemsetAsync(c->xf, 0, n * sizeof(float), c->st));
      CK(dev_scale_f(c->pf, (float)k, n, c->st));
      CK(dev_dot_f(c->rf, c->rf, n, c->part, c->sc, SC_RRNEW, OP_STORE, c->st));
      TRY(read_scalar(c, SC_RRNEW, &rr));
      // beta = |r_true|^2 / |r_prev|^2 with both in the new scaling
      c->h_sc[SC_BETA] = rr / (rr_prev * k * k);
      CK(cudaMemcpyAsync(c->sc + SC_BETA, c->h_sc + SC_BETA, sizeof(double),
                         cudaMemcpyHostToDevice, c->st));
      scale = nscale;
      maxr = rn;
    }
    CK(dev_cg_p<float>(c->pf, c->rf, n, c->sc, c->st));
    rr_prev = rr;
  }
  *iters = it;
  c->cg_iters += it;
  c->cg_solves++;
  if (c->log)
    fprintf(stderr, "         cg (mixed): %d iterations, %d restarts, |r|/|b| %.2e\n", it, restarts,
            rn / n2b);
  if (!converged) { cpfft_set_error("mixed-precision CG did not converge"); return CPFFT_ERR_CG_MAXIT; }
  return 0;
}

// One preconditioned FP32 CG iteration on the device: p = r + beta p (and rr <- rr_new),
// Ap = G0(K4f : p) with pAp = <K4f : p, p> and alpha = rr / pAp, x += alpha p, r -= alpha Ap
// with rr_new = <r, r>_K0 and beta, then the stop test (k_cg_cond).  `timed` brackets the
// Green apply with the per-launch CUDA events (never inside a capture).
int cg_pre_body(Ctx* c, bool use_handle, bool timed) {
  const long long n = 9 * c->N3;
  GridDesc g = c->g;
  g.pre = 1;
  int np = 0;
  if (green_df_supported(c->N)) {
    // the register-FFT grids run the whole iteration in the five transform passes: p is
    // updated in the first, x, r and the partials of <r, r>_K0 in the last
    if (timed) kt_start(c, KT_G32);
    CK(green_cg_iteration(c->xf, c->rf, c->pf, c->K4f, c->Sf, c->twf, g, c->st, c->part,
                          c->part, c->pre_dev + 36, c->sc));
    if (timed) TRY(kt_stop(c));
    CK(dev_final(c->part, (c->N / 2) * c->N, c->sc, SC_RRNEW, OP_BETA, c->st));
    CK(dev_cg_cond(c->sc, c->cg_handle, use_handle, c->st));
    return 0;
  }
  CK(dev_cg_p<float>(c->pf, c->rf, n, c->sc, c->st));
  if (timed) kt_start(c, KT_G32);
  CK(green_apply_dot<float>(c->pf, c->K4f, 1, c->Apf, c->Sf, c->twf, g, c->st, c->part, &np));
  if (timed) TRY(kt_stop(c));
  if (!np) {
    cpfft_set_error("internal: the preconditioned product was not fused");
    return CPFFT_ERR_CUDA;
  }
  CK(dev_final(c->part, np, c->sc, SC_PAP, OP_ALPHA, c->st));
  CK(dev_cg_xr_k0(c->xf, c->rf, c->pf, c->Apf, c->N3, c->pre_dev + 36, c->part, c->sc, c->st));
  CK(dev_cg_cond(c->sc, c->cg_handle, use_handle, c->st));
  return 0;
}

// Capture the iteration once into a graph whose WHILE node repeats it while k_cg_cond
// says so (the node's default value runs the body at least once per launch).  Every
// buffer and launch shape is fixed for the context; alpha, beta and the stop test's
// inputs live in device memory.  If anything fails, the iterations run eagerly instead.
void build_cg_graph(Ctx* c) {
  if (c->cg_graph_state) return;
  c->cg_graph_state = -1;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ex = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) { cudaGetLastError(); return; }
  cudaGraphConditionalHandle h;
  cudaGraphNodeParams prm = {};
  cudaGraphNode_t node, gate = nullptr;
  bool ok = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  // the gate kernel, then the WHILE node after it
  if (ok) {
    ok = cudaStreamBeginCaptureToGraph(c->st, g, nullptr, nullptr, 0,
                                       cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      const cudaError_t e1 = dev_cg_gate(c->sc, h, c->st);
      g_kernel_launches -= 1;
      cudaGraph_t out = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(c->st, &out);
      size_t nn = 1;
      ok = e1 == cudaSuccess && e2 == cudaSuccess &&
           cudaGraphGetNodes(g, &gate, &nn) == cudaSuccess && nn == 1;
    }
  }
  if (ok) {
    prm.type = cudaGraphNodeTypeConditional;
    prm.conditional.handle = h;
    prm.conditional.type = cudaGraphCondTypeWhile;
    prm.conditional.size = 1;
    ok = cudaGraphAddNode(&node, g, &gate, nullptr, 1, &prm) == cudaSuccess;
  }
  if (ok) {
    cudaGraph_t body = prm.conditional.phGraph_out[0];
    ok = cudaStreamBeginCaptureToGraph(c->st, body, nullptr, nullptr, 0,
                                       cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      const long long l0 = g_kernel_launches;
      c->cg_handle = h;
      const int rc = cg_pre_body(c, true, false);
      cudaGraph_t out = nullptr;
      const cudaError_t e = cudaStreamEndCapture(c->st, &out);
      c->cg_body_launches = g_kernel_launches - l0;
      g_kernel_launches = l0;
      ok = rc == 0 && e == cudaSuccess;
    }
  }
  if (ok) ok = cudaGraphInstantiate(&ex, g, 0) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    if (g) cudaGraphDestroy(g);
    c->cg_handle = 0;
    return;
  }
  c->cg_graph = g;
  c->cg_exec = ex;
  c->cg_graph_state = 1;
}

// Run iterations from the current (rf, pf, xf) until k_cg_cond stops them: the first one
// eagerly with the Green apply timed (the per-launch figure of the FP32 operator), the
// rest as one launch of the iteration graph.  rr (in) is <r,r>_K0 now; *rr_out the value
// at the end; *it_out the iteration count after the segment; *stop the reason.
int cg_segment(Ctx* c, double rr, double rn, double tolb, double tol, double delta, int it,
               int maxIter, double beta, double* rr_out, double* rr_prev_out, int* it_out,
               int* stop) {
  double* h = c->h_sc;
  h[SC_BETA] = beta;
  h[SC_RRNEW] = rr;
  CK(cudaMemcpyAsync(c->sc + SC_BETA, h + SC_BETA, sizeof(double), cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->sc + SC_RRNEW, h + SC_RRNEW, sizeof(double), cudaMemcpyHostToDevice, c->st));
  h[SC_RR0] = rr; h[SC_RN] = rn; h[SC_TOLB] = tolb; h[SC_TOL] = tol; h[SC_DELTA] = delta;
  h[SC_CNT] = (double)it; h[SC_MAXIT] = (double)maxIter; h[SC_STOP] = 0.0;
  CK(cudaMemcpyAsync(c->sc + SC_RR0, h + SC_RR0, (SC_STOP - SC_RR0 + 1) * sizeof(double),
                     cudaMemcpyHostToDevice, c->st));
  build_cg_graph(c);
  int done = 0;
  for (;;) {
    TRY(cg_pre_body(c, false, done == 0));
    done++;
    if (c->cg_graph_state == 1) {  // the graph's gate skips its loop if already stopped
      kt_start(c, KT_CGGRAPH);
      CK(cudaGraphLaunch(c->cg_exec, c->st));
      TRY(kt_stop(c));
      g_kernel_launches += 1;
      break;
    }
    double st;
    TRY(read_scalar(c, SC_STOP, &st));
    if (st != 0.0) break;
  }
  CK(cudaMemcpyAsync(h + SC_CNT, c->sc + SC_CNT, (SC_STOP - SC_CNT + 1) * sizeof(double),
                     cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(h + SC_RR, c->sc + SC_RR, sizeof(double), cudaMemcpyDeviceToHost, c->st));
  TRY(read_scalar(c, SC_RRNEW, rr_out));
  *rr_prev_out = h[SC_RR];  // <r,r>_K0 before the last iteration (its beta's denominator)
  const int it_end = (int)h[SC_CNT];
  const long long its = it_end - it;
  c->f32_matvecs += its;
  if (c->cg_graph_state == 1) g_kernel_launches += (its - done) * c->cg_body_launches;
  *it_out = it_end;
  *stop = (int)h[SC_STOP];
  return 0;
}

// Mixed precision with the reference-medium preconditioner: FP32 CG on G0(K : x) = G0(r)
// in the K0 inner product, with the same reliable updates, FP64 residual b - G(K4 : x),
// FP64 projection of each correction and the reference's stop test as cg_mixed.  After a
// reliable update the recursion restarts from G0 of the true residual.
int cg_mixed_pre(Ctx* c, const double* b, double* x, double tol, int* iters, bool use_x0) {
  const long long n = 9 * c->N3;
  const int maxIter = 2000;
  // reduction of <r,r>_K0 per segment before a reliable update (reliable_delta)
  const double delta = reliable_delta(tol);
  *iters = 0;
  if (!use_x0) CK(cudaMemsetAsync(x, 0, n * sizeof(double), c->st));
  double n2b;
  TRY(dnrm2(c, b, &n2b));
  if (!(tol > 2.220446049250313e-16 && tol < 1.0)) return CPFFT_ERR_CG_TOL;
  if (!std::isfinite(n2b)) { cpfft_set_error("non-finite CG right-hand side"); return CPFFT_ERR_NONFINITE; }
  if (n2b <= 2.220446049250313e-16) return 0;
  if (!c->K4f_valid) {
    cpfft_set_error("mixed precision CG needs the FP32 tangent of a stress update");
    return CPFFT_ERR_BAD_ARG;
  }
  const double tolb = tol * n2b;
  // the reference's absolute test ||r|| <= tol, off for the inexact Newton solves
  const double tola = c->cg_rel_only ? 0.0 : tol;
  double rn = n2b;
  if (use_x0) {
    TRY(matvec_acc(c, x, c->Ap, 1));
    CK(dev_sub(c->w, b, c->Ap, n, c->st));
    TRY(dnrm2(c, c->w, &rn));
    if (!std::isfinite(rn)) { cpfft_set_error("FP64 residual is not finite"); return CPFFT_ERR_NONFINITE; }
    if (rn <= tolb || rn <= tola) {
      c->cg_solves++;
      return 0;
    }
  } else {
    CK(cudaMemcpyAsync(c->w, b, n * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
  }
  // preconditioned residual rf = G0(w / ||w||)
  double scale = 1.0 / rn;
  CK(dev_to_f32(c->Apf, c->w, scale, n, c->st));
  TRY(matvec32_pre(c, c->Apf, c->rf, 0, false));
  CK(cudaMemsetAsync(c->xf, 0, n * sizeof(float), c->st));
  CK(cudaMemcpyAsync(c->pf, c->rf, n * sizeof(float), cudaMemcpyDeviceToDevice, c->st));
  CK(dev_dot_k0(c->rf, c->rf, c->N3, c->pre_dev + 36, c->part, c->sc, SC_RRNEW, OP_STORE, c->st));
  double rr;
  TRY(read_scalar(c, SC_RRNEW, &rr));
  double beta = 0.0;  // the first iteration's p = r + 0 p = r
  int it = 0, restarts = 0;
  bool converged = false;
  for (;;) {
    // one segment of iterations on the device: until <r,r>_K0 has dropped by delta, the
    // true residual it predicts meets the stop test, or maxIter
    int stop = 0;
    double rr_prev = rr;
    TRY(cg_segment(c, rr, rn, tolb, tola, delta, it, maxIter, beta, &rr, &rr_prev, &it, &stop));
    if (stop == STOP_NONFINITE) { cpfft_set_error("FP32 CG residual is not finite"); return CPFFT_ERR_NONFINITE; }
    // reliable update: x += G(xf / scale) in FP64-accurate arithmetic, true residual
    restarts++;
    CK(cudaMemsetAsync(c->w2, 0, n * sizeof(double), c->st));
    CK(dev_add_f32(c->w2, c->xf, 1.0 / scale, n, c->st));
    TRY(matvec_acc(c, c->w2, c->Ap, 0));
    CK(dev_axpy(x, c->Ap, 1.0, n, c->st));
    TRY(matvec_acc(c, x, c->Ap, 1));
    CK(dev_sub(c->w, b, c->Ap, n, c->st));
    TRY(dnrm2(c, c->w, &rn));
    if (!std::isfinite(rn)) { cpfft_set_error("FP64 residual is not finite"); return CPFFT_ERR_NONFINITE; }
    if (rn <= tolb || rn <= tola) { converged = true; break; }
    if (it >= maxIter) break;
    // restart from G0 of the true residual, keeping the search direction (rescaled)
    const double nscale = 1.0 / rn, k = nscale / scale;
    CK(dev_to_f32(c->Apf, c->w, nscale, n, c->st));
    TRY(matvec32_pre(c, c->Apf, c->rf, 0, false));
    CK(cudaMemsetAsync(c->xf, 0, n * sizeof(float), c->st));
    CK(dev_scale_f(c->pf, (float)k, n, c->st));
    CK(dev_dot_k0(c->rf, c->rf, c->N3, c->pre_dev + 36, c->part, c->sc, SC_RRNEW, OP_STORE, c->st));
    double rr_new;
    TRY(read_scalar(c, SC_RRNEW, &rr_new));
    // beta = |r_true|^2 / |r_prev|^2 with both in the new scaling (the iteration's beta
    // with the recomputed residual in place of the recursive one)
    beta = rr_new / (rr_prev * k * k);
    rr = rr_new;
    scale = nscale;
  }
  *iters = it;
  c->cg_iters += it;
  c->cg_solves++;
  if (c->log)
    fprintf(stderr, "         cg (mixed, reference medium): %d iterations, %d restarts, |r|/|b| %.2e%s\n",
            it, restarts, rn / n2b, c->cg_graph_state == 1 ? " (graph)" : "");
  if (!converged) { cpfft_set_error("mixed-precision CG did not converge"); return CPFFT_ERR_CG_MAXIT; }
  return 0;
}

int cg_mixed_any(Ctx* c, const double* b, double* x, double tol, int* iters, bool use_x0) {
  if (pre_applies(c) && c->pre_ok) return cg_mixed_pre(c, b, x, tol, iters, use_x0);
  return cg_mixed(c, b, x, tol, iters, use_x0);
}

int cg(Ctx* c, const double* b, double* x, double tol, int* iters) {
  return c->prec == CPFFT_PREC_MIXED ? cg_mixed_any(c, b, x, tol, iters, false)
                                     : cg64(c, b, x, tol, iters);
}

// Queue autotuner: on the context's first implicit queue pass, the pass runs once per
// candidate -- chunk (voxels a block takes from the work queue at a time) 128 / 256 / 512,
// with as many persistent blocks per SM as fit or with one (half the threads in flight:
// their local-memory spill working set then stays closer to the L2's size) -- timed with
// CUDA events, and the fastest is kept.  The runs give identical results (no local solve
// of this pass starts from an earlier pass's state); their statistics and logged pairs
// are not kept.
// the stress kernel compiled for the grid's slip systems and hardening law
cudaError_t launch_crystals(Ctx* c, const StressArgs& a, bool warm) {
  if (c->h_type == 2) return launch_stress_mts(a, warm, c->st);
  if (c->h_type == 7) return launch_stress_mrr(a, false, c->st);
  if (c->h_type == 4) return launch_stress_ornl(a, false, c->st);
  switch (c->nslip) {
    case 48: return launch_stress48(a, warm, c->st);
    case 6: return launch_stress6(a, warm, c->st);
    case 1: return launch_stress1(a, warm, c->st);
    default: return launch_stress(a, warm, c->st);
  }
}

int tune_queue_chunk(Ctx* c, StressArgs a, bool warm) {
  c->qtuned = true;
  a.log_X = nullptr;
  a.log_cap = 0;
  const long long l0 = g_kernel_launches;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  int bestq = 128, bestb = 0, k = 0;
  for (int bps : {0, 1})
  for (int q : {128, 256, 512}) {
    a.qchunk = q;
    a.qbps = bps;
    CK(launch_voxel_queue(c->vcost, c->N3, c->vq, c->vperm, c->vq + 128, c->st));
    CK(cudaEventRecord(e0, c->st));
    CK(launch_crystals(c, a, warm));
    CK(cudaEventRecord(e1, c->st));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    c->qchunk_ms[k++] = ms;
    if (ms < best) { best = ms; bestq = q; bestb = bps; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  g_kernel_launches = l0;  // tuning launches are not the caller's work
  c->qchunk = bestq;
  c->qbps = bestb;
  if (c->log)
    fprintf(stderr, "       queue: chunk %d voxels, %s blocks per SM (%.2f / %.2f / %.2f ms for "
            "128 / 256 / 512; %.2f / %.2f / %.2f ms with one block per SM)\n", bestq,
            bestb ? "1" : "all", c->qchunk_ms[0], c->qchunk_ms[1], c->qchunk_ms[2],
            c->qchunk_ms[3], c->qchunk_ms[4], c->qchunk_ms[5]);
  return 0;
}

int stress(Ctx* c, int step, int iter, long long* local_iters, int* fails,
           long long* predict_iters = nullptr, long long* rejected = nullptr) {
  StressArgs a;
  a.Fn = c->Fn;
  a.Fn1 = c->Fn1;
  a.hist_n = c->hist[c->hn];
  a.hist_np1 = c->hist[1 - c->hn];
  a.P = c->P;
  a.K4 = c->K4;
  a.K4f = c->prec == CPFFT_PREC_MIXED ? c->K4f : nullptr;
  a.K4lo = c->prec == CPFFT_PREC_MIXED && c->df_ok ? c->K4lo : nullptr;
  a.tangent_f32 = c->prec == CPFFT_PREC_MIXED && c->tangent_f32;
  a.ori = c->ori;
  a.crys = c->crys;
  a.oris = c->oris;
  a.cryss = c->cryss;
  a.mises = c->n_mises_vox ? c->mises : nullptr;
  a.misess = c->misess;
  a.stats = c->stats;
  if (c->n_undef_vox) {
    cpfft_set_error("stress update: %lld voxels of a material declared CPFFT_NOT_A_CRYSTAL "
                    "that cpfft_set_mises has not defined", c->n_undef_vox);
    return CPFFT_ERR_NOT_INIT;
  }
  a.N3 = c->N3;
  a.dt = c->dt;
  a.step = step;
  a.iter = iter;
  a.mlp_packed = nullptr;
  a.mlp_params = a.mlp_norm = nullptr;
  a.mlp_err = nullptr;
  // start of the local solves.  Plain: the reference's (predictor from sigma_n).
  // CPFFT_START_ITERATE: a pass that follows an implicit pass of the same step starts the
  // coupled Newton from that pass's converged state.  On the other implicit passes,
  // CPFFT_START_LEARNED starts it from the network's guess and CPFFT_START_TRIAL from the
  // elastic trial, both returned inside the rate surface.
  // (iter == pass_iter: the same Newton iteration re-evaluated at a shortened increment)
  const bool have_iterate = c->pass_step == step && c->pass_iter >= 1 &&
                            (iter == c->pass_iter + 1 || iter == c->pass_iter);
  a.start_iterate = (c->warm & CPFFT_START_ITERATE) && iter >= 2 && have_iterate;
  a.start_trial = (c->warm & CPFFT_START_TRIAL) && !(c->warm & CPFFT_START_LEARNED) &&
                  !a.start_iterate;
  a.start_cap = 8;
  bool warm = false;
  if ((c->warm & CPFFT_START_LEARNED) && iter > 0 && !a.start_iterate) {
    mlp::Weights w;
    if (!mlp_device_weights(&w, &a.mlp_err)) {
      cpfft_set_error("learned initial guess selected but the network is not initialised");
      return CPFFT_ERR_NOT_INIT;
    }
    a.mlp_packed = w.packed;
    a.mlp_params = w.params;
    a.mlp_norm = w.norm;
    warm = true;
  }
  a.log_X = c->log_cap > 0 ? c->log_X : nullptr;
  a.log_T = c->log_T;
  a.log_n = c->log_n;
  a.log_cap = c->log_cap;
  a.log_stride = c->log_stride;
  a.log_phase = c->log_phase;
  a.perm = nullptr;
  a.queue = nullptr;
  a.cost = nullptr;
  a.qchunk = c->qchunk;
  a.qbps = c->qbps;
  if (c->sched == CPFFT_SCHED_QUEUE && iter > 0 && c->n_crys_vox) {
    a.perm = c->vperm;
    a.queue = c->vq + 128;
    a.cost = c->vcost;
    if (!c->qtuned && !a.start_iterate) TRY(tune_queue_chunk(c, a, warm));
    CK(launch_voxel_queue(c->vcost, c->N3, c->vq, c->vperm, c->vq + 128, c->st));
  }
  CK(cudaMemsetAsync(c->stats, 0, 5 * sizeof(unsigned long long), c->st));
  kt_start(c, KT_STRESS);
  if (c->n_crys_vox) CK(launch_crystals(c, a, warm));
  if (c->n_mises_vox) CK(launch_mises(a, c->st));
  TRY(kt_stop(c));
  c->pass_step = step;
  c->pass_iter = iter;
  c->K4f_valid = a.K4f != nullptr;
  const bool reduce = c->K4f_valid && pre_applies(c);
  if (reduce) TRY(reference_reduce(c));
  CK(cudaMemcpyAsync(c->h_stats, c->stats, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->st));
  TRY(sync(c));
  if (reduce) TRY(reference_build(c));
  for (int k = 0; k < 5; k++) c->last_pass[k] = (long long)c->h_stats[k];
  if (local_iters) *local_iters = (long long)c->h_stats[0];
  if (fails) *fails = (int)c->h_stats[1];
  if (predict_iters) *predict_iters = (long long)c->h_stats[2];
  if (rejected) *rejected = (long long)c->h_stats[3];
  if (c->log)  // per-pass local work (CPFFT_LOG=1)
    fprintf(stderr, "       stress pass step %d iter %d: update %.4f predictor %.4f per voxel%s, "
            "%.4f starts dropped, %llu sub-stepped\n", step, iter,
            (double)c->h_stats[0] / (double)c->N3, (double)c->h_stats[2] / (double)c->N3,
            warm ? " (learned start)" : a.start_iterate ? " (iterate start)" :
            a.start_trial && iter > 0 ? " (trial start)" : "",
            (double)c->h_stats[3] / (double)c->N3, c->h_stats[4]);
  if (warm) TRY(mlp_check_error());
  return 0;
}

// One of tangent_homo's solves in FP32 alone, for a loose tolerance (>= 1e-4, the fast
// form's inexact mode): G(K : (E_i + x)) = 0 for the fluctuation x, started from the
// previous call's x (th_x), with the reference-medium preconditioned iteration and no
// reliable updates -- the FP32 recursion's drift (about 1e-7 of the starting residual)
// stays far below the tolerance, and C_homo only steers the P_bar update.  The stop test
// is ||r|| <= tol ||G(K : E_i)|| on the recursion's estimate.  On return io = E_i + x
// (FP64) and th_x holds x.
int tangent_solve_f32(Ctx* c, int i, double tol, int* its) {
  const long long N3 = c->N3, n = 9 * N3;
  float* x0 = c->th_x + i * n;
  auto apply = [&](const float* in, float* out) -> int {
    int np = 0;
    c->f32_matvecs++;
    kt_start(c, KT_G32);
    TRY(cuda_check(green_apply_dot<float>(in, c->K4f, 1, out, c->Sf, c->twf, c->g, c->st,
                                          nullptr, &np), "green_apply fp32"));
    return kt_stop(c);
  };
  // b = G(K : E_i), the start's residual w = -G(K : (E_i + x0)), their squared norms, the
  // preconditioned residual rf = G0(w) and <rf, rf>_K0, read back in one transfer (the
  // recursion needs no normalisation: its stop test uses ratios)
  CK(cudaMemsetAsync(c->io, 0, n * sizeof(double), c->st));
  CK(dev_add_const(c->io + i * N3, 1.0, N3, c->st));
  CK(dev_to_f32(c->pf, c->io, 1.0, n, c->st));
  TRY(apply(c->pf, c->rf));
  CK(dev_dot_f(c->rf, c->rf, n, c->part, c->sc, SC_T1, OP_STORE, c->st));
  if (c->th_valid) {
    CK(dev_add_f32(c->io, x0, 1.0, n, c->st));
    CK(dev_to_f32(c->pf, c->io, 1.0, n, c->st));
    TRY(apply(c->pf, c->Apf));
  } else {
    CK(cudaMemcpyAsync(c->Apf, c->rf, n * sizeof(float), cudaMemcpyDeviceToDevice, c->st));
  }
  CK(dev_scale_f(c->Apf, -1.0f, n, c->st));
  CK(dev_dot_f(c->Apf, c->Apf, n, c->part, c->sc, SC_T2, OP_STORE, c->st));
  TRY(matvec32_pre(c, c->Apf, c->rf, 0, false));
  CK(cudaMemsetAsync(c->xf, 0, n * sizeof(float), c->st));
  CK(cudaMemcpyAsync(c->pf, c->rf, n * sizeof(float), cudaMemcpyDeviceToDevice, c->st));
  CK(dev_dot_k0(c->rf, c->rf, c->N3, c->pre_dev + 36, c->part, c->sc, SC_RRNEW, OP_STORE, c->st));
  CK(cudaMemcpyAsync(c->h_sc + SC_RRNEW, c->sc + SC_RRNEW, (SC_T2 - SC_RRNEW + 1) * sizeof(double),
                     cudaMemcpyDeviceToHost, c->st));
  TRY(sync(c));
  const double nb = std::sqrt(c->h_sc[SC_T1]), rn = std::sqrt(c->h_sc[SC_T2]);
  const double rr = c->h_sc[SC_RRNEW];
  *its = 0;
  if (!std::isfinite(rn) || !std::isfinite(nb) || !std::isfinite(rr)) {
    cpfft_set_error("non-finite tangent right-hand side");
    return CPFFT_ERR_NONFINITE;
  }
  if (rn > tol * nb && rr > 0.0) {
    double rr_out, rr_prev;
    int it = 0, stop = 0;
    TRY(cg_segment(c, rr, rn, tol * nb, 0.0, 0.0, 0, 2000, 0.0, &rr_out, &rr_prev, &it, &stop));
    if (stop == STOP_NONFINITE) { cpfft_set_error("FP32 CG residual is not finite"); return CPFFT_ERR_NONFINITE; }
    if (stop == STOP_MAXIT) { cpfft_set_error("tangent_homo: FP32 CG did not converge"); return CPFFT_ERR_CG_MAXIT; }
    *its = it;
    c->cg_iters += it;
    CK(dev_add_f32(c->io, c->xf, 1.0, n, c->st));  // io = E_i + x0 + correction
  }
  c->cg_solves++;
  // th_x = x = io - E_i
  CK(dev_add_const(c->io + i * N3, -1.0, N3, c->st));
  CK(dev_to_f32(x0, c->io, 1.0, n, c->st));
  CK(dev_add_const(c->io + i * N3, 1.0, N3, c->st));
  if (c->log)
    fprintf(stderr, "         cg (FP32 tangent): %d iterations, |r0|/|b| %.2e\n", *its, rn / nb);
  return 0;
}

// Column i of C_homo from io = E_i + x: C_homo(j, i) = mean of K : (E_i + x) over the
// grid, component j (src/tangent_homo.f:60-68); the nine sums read back at once.
int homo_column(Ctx* c, int i, double* C_homo) {
  const long long N3 = c->N3, n = 9 * N3;
  for (int j = 0; j < 9; j++)
    CK(dev_dot(c->K4 + 9 * j * N3, c->io, n, c->part, c->sc, SC_SUM9 + j, OP_STORE, c->st));
  CK(cudaMemcpyAsync(c->h_sc + SC_SUM9, c->sc + SC_SUM9, 9 * sizeof(double),
                     cudaMemcpyDeviceToHost, c->st));
  TRY(sync(c));
  for (int j = 0; j < 9; j++) C_homo[9 * j + i] = c->h_sc[SC_SUM9 + j] / (double)N3;
  return 0;
}

// tangent_homo (src/tangent_homo.f:11-73): 9 CG solves, C_homo(i,j) stored at 9*j+i.
// In mixed precision each solve starts from the fluctuation field the same column
// converged to in the previous call (the tangent changes little between calls), kept in
// FP32; the stop test, ||r|| <= tol ||b||, is unchanged.  The plain FP64 path starts from zero as
// the reference does.
int tangent_homo(Ctx* c, double tolPCG, double* C_homo, int* its_total) {
  const long long N3 = c->N3, n = 9 * N3;
  *its_total = 0;
  const bool warm = c->prec == CPFFT_PREC_MIXED;
  if (warm && !c->th_x) TRY(dalloc(c->th_x, 9 * n * sizeof(float)));
  // loose tolerances (the fast form's inexact mode) on a preconditioned grid: FP32 alone
  const bool f32 = warm && tolPCG >= 1.0e-4 && pre_applies(c) && c->pre_ok;
  for (int i = 0; i < 9; i++) {
    if (f32) {
      int its = 0;
      TRY(tangent_solve_f32(c, i, tolPCG, &its));
      *its_total += its;
      TRY(homo_column(c, i, C_homo));
      continue;
    }
    for (int j = 0; j < 9; j++)
      CK(cudaMemcpyAsync(c->io + j * N3, c->K4 + (9 * j + i) * N3, N3 * sizeof(double),
                         cudaMemcpyDeviceToDevice, c->st));
    TRY(matvec_acc(c, c->io, c->b, 0));
    CK(dev_scale(c->b, -1.0, n, c->st));
    int its = 0;
    if (warm) {
      if (c->th_valid) {
        CK(cudaMemsetAsync(c->io, 0, n * sizeof(double), c->st));
        CK(dev_add_f32(c->io, c->th_x + i * n, 1.0, n, c->st));
      }
      TRY(cg_mixed_any(c, c->b, c->io, tolPCG, &its, c->th_valid));
      CK(dev_to_f32(c->th_x + i * n, c->io, 1.0, n, c->st));
    } else {
      TRY(cg(c, c->b, c->io, tolPCG, &its));
    }
    *its_total += its;
    CK(dev_add_const(c->io + i * N3, 1.0, N3, c->st));
    TRY(homo_column(c, i, C_homo));
  }
  if (warm) c->th_valid = true;
  return 0;
}

// NBC_update (src/FFT_nr3.f:375-433): 9x9 LU with partial pivoting
int nbc_update(const double* C_homo, double* DbarF, const double* P_bar, const double* PBC,
               const int* isNBC) {
  double A[81], bb[9];
  for (int i = 0; i < 9; i++) {
    if (isNBC[i]) {
      for (int k = 0; k < 9; k++) A[9 * i + k] = C_homo[k + 9 * i];
      bb[i] = PBC[i] - P_bar[i];
    } else {
      for (int k = 0; k < 9; k++) A[9 * i + k] = 0.0;
      A[9 * i + i] = 1.0;
      bb[i] = DbarF[i];
    }
  }
  for (int k = 0; k < 9; k++) {
    int p = k;
    for (int i = k + 1; i < 9; i++)
      if (std::fabs(A[9 * i + k]) > std::fabs(A[9 * p + k])) p = i;
    if (A[9 * p + k] == 0.0 || !std::isfinite(A[9 * p + k])) {
      cpfft_set_error("P_bar update failed: singular mixed-BC system");
      return CPFFT_ERR_NBC_SINGULAR;
    }
    if (p != k) {
      for (int j = 0; j < 9; j++) std::swap(A[9 * k + j], A[9 * p + j]);
      std::swap(bb[k], bb[p]);
    }
    for (int i = k + 1; i < 9; i++) {
      double l = A[9 * i + k] / A[9 * k + k];
      for (int j = k; j < 9; j++) A[9 * i + j] -= l * A[9 * k + j];
      bb[i] -= l * bb[k];
    }
  }
  for (int i = 8; i >= 0; i--) {
    double s = bb[i];
    for (int k = i + 1; k < 9; k++) s -= A[9 * i + k] * bb[k];
    bb[i] = s / A[9 * i + i];
  }
  for (int i = 0; i < 9; i++) DbarF[i] = bb[i];
  return 0;
}

int need_ctx() {
  if (!g_ctx) {
    cpfft_set_error("cpfft_init has not been called");
    return CPFFT_ERR_NOT_INIT;
  }
  return 0;
}

int alloc_mixed(Ctx* c) {
  const long long n = 9 * c->N3;
  if (c->K4f) return 0;
  const long long launches0 = g_kernel_launches;
  TRY(dalloc(c->w2, n * sizeof(double)));
  TRY(dalloc(c->K4f, 81 * c->N3 * sizeof(float)));
  TRY(dalloc(c->xf, n * sizeof(float)));
  TRY(dalloc(c->rf, n * sizeof(float)));
  TRY(dalloc(c->pf, n * sizeof(float)));
  TRY(dalloc(c->Apf, n * sizeof(float)));
  TRY(dalloc(c->Sf, (size_t)9 * c->N * c->N * c->g.H * sizeof(float2)));
  TRY(dalloc(c->twf, c->N * sizeof(float2)));
  std::vector<float2> twf(c->N);
  for (int k = 0; k < c->N; k++) {
    long double a = -2.0L * 3.14159265358979323846264338327950288L * k / c->N;
    twf[k] = make_float2((float)cosl(a), (float)sinl(a));
  }
  CK(cudaMemcpy(c->twf, twf.data(), c->N * sizeof(float2), cudaMemcpyHostToDevice));
  CK(green_setup<float>(c->N));
  if (green_df_supported(c->N)) {
    TRY(dalloc(c->K4lo, 81 * c->N3 * sizeof(float)));
    TRY(dalloc(c->twdf, c->N * sizeof(dfl2)));
    std::vector<dfl2> tw(c->N);
    for (int k = 0; k < c->N; k++) {
      long double a = -2.0L * 3.14159265358979323846264338327950288L * k / c->N;
      long double cr = cosl(a), ci = sinl(a);
      const float hr = (float)cr, hi = (float)ci;
      tw[k].x = dfl(hr, (float)(cr - (long double)hr));
      tw[k].y = dfl(hi, (float)(ci - (long double)hi));
    }
    CK(cudaMemcpy(c->twdf, tw.data(), c->N * sizeof(dfl2), cudaMemcpyHostToDevice));
    CK(green_setup_df(c->N));
    c->df_ok = true;
    // tile shapes of both operators, timed on this GPU with this grid's buffers
    CK(cudaMemsetAsync(c->K4f, 0, 81 * c->N3 * sizeof(float), c->st));
    CK(cudaMemsetAsync(c->K4lo, 0, 81 * c->N3 * sizeof(float), c->st));
    CK(cudaMemsetAsync(c->xf, 0, n * sizeof(float), c->st));
    CK(cudaMemsetAsync(c->io, 0, n * sizeof(double), c->st));
    CK(green_autotune_f32(c->xf, c->K4f, c->Apf, c->Sf, c->twf, &c->g, c->st, &c->tune_ms[0]));
    c->gdf = c->g;
    c->gdf.wtc = 0;
    c->gdf.wc2 = 0;
    CK(green_autotune_df(c->io, c->K4f, c->K4lo, c->b, reinterpret_cast<dfl2*>(c->S), c->twdf,
                         &c->gdf, c->st, &c->tune_ms[1]));
    g_kernel_launches = launches0;  // tuning launches are not the caller's work
    if (c->log)
      fprintf(stderr, "       autotuned tiles: FP32 B/D %d C %d (%.3f ms), double-float B/D %d C %d "
              "(%.3f ms)\n", c->g.wtb, c->g.wtc, c->tune_ms[0], c->gdf.wtb, c->gdf.wtc,
              c->tune_ms[1]);
  }
  return 0;
}

}  // namespace

// =====================================================================================
extern "C" {

const char* cpfft_last_error(void) { return g_err; }

void cpfft_finalize(void) {
  free_ctx(g_ctx);
  g_ctx = nullptr;
}

int cpfft_init(int N, const int* matList, const double* kocks_deg, const cpfft_crystal* props,
               int ncrystals, double tstep, int g_mapping) {
  cpfft_finalize();
  if (N < 2 || N > 256 || !matList || !kocks_deg || !props || ncrystals < 1 || !(tstep > 0) ||
      (g_mapping != CPFFT_G_REF_SHIFT && g_mapping != CPFFT_G_CENTERED)) {
    cpfft_set_error("cpfft_init: invalid argument (N in [2,256], tstep > 0, mapping 0/1)");
    return CPFFT_ERR_BAD_ARG;
  }
  const long long N3 = (long long)N * N * N;
  std::vector<CrysRec> cr(ncrystals);
  std::vector<std::vector<double>> C0(ncrystals, std::vector<double>(36));
  double bb[48][3], nn[48][3];
  int nslip = 0, h_type = 0;
  int first_crystal = -1;
  for (int k = 0; k < ncrystals; k++) {
    const cpfft_crystal& p = props[k];
    if (p.slip_type == CPFFT_NOT_A_CRYSTAL) continue;  // defined by cpfft_set_mises
    if (first_crystal < 0) first_crystal = k;
    const int ns = slip_geometry(p.slip_type, bb, nn);
    // Voce needs tau_v != 0; MTS (12-system types) positive thermal-barrier parameters
    const bool voce_ok = p.h_type == 1 && p.tau_v != 0;
    const bool mts_ok = p.h_type == 2 && ns == 12 && p.mu_0 > 0 && p.burgers > 0 &&
                        p.boltzman > 0 && p.G_0_y > 0 && p.G_0_v > 0 && p.p_y > 0 &&
                        p.q_y > 0 && p.p_v > 0 && p.q_v > 0 && p.gamma_bar > 0 &&
                        p.eps_dot_0_v > 0;
    // MRR: positive constants (mm10_h_mrr stops on a non-positive temperature; the
    // densities enter square roots and the rates divide by c1 c2 c3)
    const bool mrr_ok = p.h_type == 7 && ns == 12 && p.mu_0 > 0 && p.burgers > 0 &&
                        p.boltzman > 0 && p.G_0_y > 0 && p.G_0_v > 0 && p.p_v > 0 &&
                        p.q_v > 0 && p.u1 > 0 && p.u2 > 0 && p.u3 > 0 && p.theta_0 >= 0;
    // ORNL: the same, with a negative G_0_y read as exp(-G_0_y) (mm10_slipinc_ornl)
    const bool ornl_ok = p.h_type == 4 && ns == 12 && p.mu_0 > 0 && p.burgers > 0 &&
                         p.boltzman > 0 && p.G_0_v > 0 && p.p_v > 0 && p.q_v > 0 &&
                         p.u1 > 0 && p.u2 > 0 && p.u3 > 0 && p.theta_0 >= 0;
    const bool n_ok = p.h_type == 7 || p.h_type == 4 || p.harden_n > 0;
    if (!ns || !(voce_ok || mts_ok || mrr_ok || ornl_ok) || !n_ok ||
        p.miter < 0 || p.miter > 1000 || !crystal_stiffness(p, C0[k].data())) {
      cpfft_set_error("cpfft_init: crystal %d unsupported (fcc, bcc, roters, bcc12, bcc48, "
                      "single, hcp6 or hcp18 slip with voce hardening, the 12-system types with "
                      "mts, roters or ornl hardening, valid elasticity)", k + 1);
      return CPFFT_ERR_BAD_ARG;
    }
    // one slip table per grid: the Schmid tensors are formed from the first crystal's
    if ((nslip && p.slip_type != props[first_crystal].slip_type) || (h_type && p.h_type != h_type)) {
      cpfft_set_error("cpfft_init: the crystals of one grid must share the slip type and the "
                      "hardening law");
      return CPFFT_ERR_BAD_ARG;
    }
    nslip = ns;
    h_type = p.h_type;
    cr[k] = crystal_record(p);
  }
  if (first_crystal >= 0) slip_geometry(props[first_crystal].slip_type, bb, nn);
  if (!nslip) nslip = 12;
  // distinct (crystal, orientation) records; a voxel of another material points at the
  // first crystal's first record (the crystal kernel reads but never stores it)
  std::vector<int> ori(N3), crys(N3), mat(N3);
  std::map<std::tuple<int, double, double, double>, int> seen;
  std::vector<OriRec> oris;
  long long n_crys_vox = 0;
  for (long long v = 0; v < N3; v++) {
    int m = matList[v] - 1;
    if (m < 0 || m >= ncrystals) {
      cpfft_set_error("cpfft_init: matList[%lld] = %d out of range", v, matList[v]);
      return CPFFT_ERR_BAD_ARG;
    }
    mat[v] = m;
    if (props[m].slip_type == CPFFT_NOT_A_CRYSTAL) continue;
    n_crys_vox++;
    double ang[3] = {kocks_deg[v], kocks_deg[N3 + v], kocks_deg[2 * N3 + v]};
    auto key = std::make_tuple(m, ang[0], ang[1], ang[2]);
    auto it = seen.find(key);
    int id;
    if (it == seen.end()) {
      id = (int)oris.size();
      oris.emplace_back();
      orientation_record(C0[m].data(), bb, nn, nslip, ang, oris.back());
      seen.emplace(key, id);
    } else {
      id = it->second;
    }
    ori[v] = id;
    crys[v] = m;
  }
  if (oris.empty()) oris.emplace_back(OriRec{});  // no crystal voxel: never read
  for (long long v = 0; v < N3; v++)
    if (props[mat[v]].slip_type == CPFFT_NOT_A_CRYSTAL) {
      ori[v] = 0;
      crys[v] = first_crystal >= 0 ? first_crystal : 0;
    }
  Ctx* c = new Ctx;
  c->nslip = nslip;
  c->h_type = h_type;
  c->hist_words = (h_type == 7 || h_type == 4) ? H_WORDS_MRR : H_WORDS;
  const int HW = c->hist_words;
  c->mat = mat;
  c->mat_kind.assign(ncrystals, 0);
  for (int k = 0; k < ncrystals; k++)
    if (props[k].slip_type == CPFFT_NOT_A_CRYSTAL) c->mat_kind[k] = 2;
  c->h_mises.assign(ncrystals, MisesRec{});
  c->n_crys_vox = n_crys_vox;
  c->n_undef_vox = N3 - n_crys_vox;
  c->N = N;
  c->N3 = N3;
  c->dt = tstep;
  c->g.N = N;
  c->g.H = N / 2 + 1;
  c->g.N3 = N3;
  c->g.Nhalf = (N % 2 == 1) ? (N + 1) / 2 : N / 2 + 1;
  c->g.gmap = g_mapping;
  c->g.inv_n3 = 1.0 / (double)N3;
  c->g.tkb = 16;
  c->g.tkc = 2;
  c->g.plan = make_plan(N);
  {
    const char* lg = getenv("CPFFT_LOG");
    c->log = lg && lg[0] == '1';
  }
  auto fail = [&](int rc) { free_ctx(c); return rc; };
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
    cpfft_set_error("cudaStreamCreate failed");
    return fail(CPFFT_ERR_CUDA);
  }
  {
    bool ok = true;
    for (int i = 0; i < 2 * Ctx::KT_CAP; i++) ok &= cudaEventCreate(&c->kt_ev[i]) == cudaSuccess;
    ok &= cudaEventCreate(&c->step_ev[0]) == cudaSuccess;
    ok &= cudaEventCreate(&c->step_ev[1]) == cudaSuccess;
    if (!ok) {
      cpfft_set_error("cudaEventCreate failed");
      return fail(CPFFT_ERR_CUDA);
    }
    c->kt_ready = true;
  }
  const size_t f9 = 9 * N3 * sizeof(double);
  int rc = 0;
  if ((rc = dalloc(c->Fn, f9)) || (rc = dalloc(c->Fn1, f9)) || (rc = dalloc(c->P, f9)) ||
      (rc = dalloc(c->K4, 81 * N3 * sizeof(double))) || (rc = dalloc(c->b, f9)) ||
      (rc = dalloc(c->dFm, f9)) || (rc = dalloc(c->r, f9)) || (rc = dalloc(c->p, f9)) ||
      (rc = dalloc(c->Ap, f9)) || (rc = dalloc(c->w, f9)) || (rc = dalloc(c->io, f9)) ||
      (rc = dalloc(c->hist[0], HW * N3 * sizeof(double))) ||
      (rc = dalloc(c->hist[1], HW * N3 * sizeof(double))) ||
      (rc = dalloc(c->ori, N3 * sizeof(int))) || (rc = dalloc(c->crys, N3 * sizeof(int))) ||
      (rc = dalloc(c->oris, oris.size() * sizeof(OriRec))) ||
      (rc = dalloc(c->cryss, ncrystals * sizeof(CrysRec))) ||
      (rc = dalloc(c->S, (size_t)9 * N * N * c->g.H * sizeof(double2))) ||
      (rc = dalloc(c->tw, N * sizeof(double2))) || (rc = dalloc(c->part, (size_t)std::max<long long>(9 * NPART, (long long)N * N) * sizeof(double))) ||
      (rc = dalloc(c->sc, SC_COUNT * sizeof(double))) ||
      (rc = dalloc(c->stats, 8 * sizeof(unsigned long long))))
    return fail(rc);
  if (cudaMallocHost((void**)&c->h_sc, SC_COUNT * sizeof(double)) != cudaSuccess ||
      cudaMallocHost((void**)&c->h_stats, 8 * sizeof(unsigned long long)) != cudaSuccess) {
    cpfft_set_error("cudaMallocHost failed");
    return fail(CPFFT_ERR_NO_MEMORY);
  }
  std::vector<double2> tw(N);
  for (int k = 0; k < N; k++) {
    long double a = -2.0L * 3.14159265358979323846264338327950288L * k / N;
    tw[k] = make_double2((double)cosl(a), (double)sinl(a));
  }
  std::vector<double> F(9 * N3, 0.0);
  for (int d : {0, 4, 8})
    for (long long v = 0; v < N3; v++) F[d * N3 + v] = 1.0;
  // history at n = the state of mm10_init_cc_hist0 (sigma 0, tau_y + 1e-5, Rp = I)
  std::vector<double> h(HW * N3, 0.0);
  for (long long v = 0; v < N3; v++) {
    if (props[mat[v]].slip_type == CPFFT_NOT_A_CRYSTAL) continue;
    if (props[crys[v]].h_type == 2) {  // mm10_init_mts: flags, set by the first update
      h[H_TT * N3 + v] = -1.0;
      h[H_U * N3 + v] = -1.0;
      h[(H_U + 1) * N3 + v] = -1.0;
    } else if (props[crys[v]].h_type == 7 || props[crys[v]].h_type == 4) {
      // mm10_init_mrr / mm10_init_ornl (src/mm10_a.f:2205-2223, 2286-2304)
      const double r0 = props[crys[v]].theta_0 == 0.0 ? 1.0e8 : props[crys[v]].theta_0;
      for (int i = 0; i < 12; i++) h[(H_RHO + i) * N3 + v] = r0;
    } else {
      h[H_TT * N3 + v] = props[crys[v]].tau_y + 1.0e-5;
    }
    for (int d : {0, 4, 8}) h[(H_RP + d) * N3 + v] = 1.0;
  }
  cudaError_t e;
  if ((e = cudaMemcpy(c->tw, tw.data(), N * sizeof(double2), cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(c->Fn, F.data(), f9, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(c->Fn1, F.data(), f9, cudaMemcpyHostToDevice)) ||
      (e = cudaMemset(c->P, 0, f9)) || (e = cudaMemset(c->K4, 0, 81 * N3 * sizeof(double))) ||
      (e = cudaMemcpy(c->hist[0], h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(c->hist[1], h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(c->ori, ori.data(), N3 * sizeof(int), cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(c->crys, crys.data(), N3 * sizeof(int), cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(c->oris, oris.data(), oris.size() * sizeof(OriRec), cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(c->cryss, cr.data(), ncrystals * sizeof(CrysRec), cudaMemcpyHostToDevice)) ||
      (e = green_setup<double>(N))) {
    cpfft_set_error("cpfft_init: %s", cudaGetErrorString(e));
    return fail(CPFFT_ERR_CUDA);
  }
  for (int i = 0; i < 9; i++) {
    c->barF_t[i] = (i % 4 == 0) ? 1.0 : 0.0;
    c->P_bar[i] = 0.0;
  }
  for (int i = 0; i < 81; i++) c->C_homo[i] = 0.0;
  g_ctx = c;
  return 0;
}

int cpfft_set_mises(int material, const cpfft_mises* props) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (material < 1 || material > (int)c->mat_kind.size() || !props) {
    cpfft_set_error("cpfft_set_mises: material %d out of range", material);
    return CPFFT_ERR_BAD_ARG;
  }
  const int m = material - 1;
  const cpfft_mises& p = *props;
  if (c->mat_kind[m] == 0) {
    cpfft_set_error("cpfft_set_mises: material %d is a crystal (declare it with slip_type "
                    "CPFFT_NOT_A_CRYSTAL in cpfft_init)", material);
    return CPFFT_ERR_BAD_ARG;
  }
  if (!(p.e > 0) || !(p.nu > -1.0 && p.nu < 0.5) || !(p.yld_pt > 0) || !(p.tan_e >= 0) ||
      !(p.tan_e < p.e) || !(p.beta >= 0 && p.beta <= 1)) {
    cpfft_set_error("cpfft_set_mises: material %d: need e > 0, -1 < nu < 0.5, yld_pt > 0, "
                    "0 <= tan_e < e, 0 <= beta <= 1", material);
    return CPFFT_ERR_BAD_ARG;
  }
  // the copies below use the default stream: the context's (non-blocking) stream drains first
  TRY(sync(c));
  // setup_mm01_rknstr (src/drive_eps_sig.f:486-520): h = tan_e e / (e - tan_e)
  c->h_mises[m] = MisesRec{p.e, p.nu, p.yld_pt, p.tan_e * p.e / (p.e - p.tan_e), p.beta};
  const long long N3 = c->N3;
  if (!c->mises) TRY(dalloc(c->mises, N3 * sizeof(int)));
  if (!c->misess) TRY(dalloc(c->misess, c->mat_kind.size() * sizeof(MisesRec)));
  c->mat_kind[m] = 1;
  std::vector<int> idx(N3);
  long long nm = 0, nu = 0;
  for (long long v = 0; v < N3; v++) {
    const int k = c->mat_kind[c->mat[v]];
    idx[v] = k == 1 ? c->mat[v] : -1;
    nm += k == 1;
    nu += k == 2;
  }
  // the voxels' state at n and n+1: mm01_set_history's (src/mm01.f:240-310)
  std::vector<double> h((size_t)c->hist_words * N3);
  cudaError_t e;
  for (int t = 0; t < 2; t++) {
    if ((e = cudaMemcpy(h.data(), c->hist[t], h.size() * sizeof(double), cudaMemcpyDeviceToHost))) {
      cpfft_set_error("cpfft_set_mises: %s", cudaGetErrorString(e));
      return CPFFT_ERR_CUDA;
    }
    for (long long v = 0; v < N3; v++) {
      if (c->mat[v] != m) continue;
      for (int w = 0; w < c->hist_words; w++) h[w * N3 + v] = 0.0;
      h[M1_K * N3 + v] = p.yld_pt / 1.73205080756888;
      h[M1_STATE * N3 + v] = 3.0;
      h[M1_HP * N3 + v] = c->h_mises[m].h;
    }
    if ((e = cudaMemcpy(c->hist[t], h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice))) {
      cpfft_set_error("cpfft_set_mises: %s", cudaGetErrorString(e));
      return CPFFT_ERR_CUDA;
    }
  }
  if ((e = cudaMemcpy(c->mises, idx.data(), N3 * sizeof(int), cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(c->misess, c->h_mises.data(), c->h_mises.size() * sizeof(MisesRec),
                      cudaMemcpyHostToDevice))) {
    cpfft_set_error("cpfft_set_mises: %s", cudaGetErrorString(e));
    return CPFFT_ERR_CUDA;
  }
  c->n_mises_vox = nm;
  c->n_undef_vox = nu;
  return 0;
}

int cpfft_set_mode(int precision, int warm_start) {
  TRY(need_ctx());
  if (precision != CPFFT_PREC_FP64 && precision != CPFFT_PREC_MIXED) {
    cpfft_set_error("cpfft_set_mode: unknown precision %d", precision);
    return CPFFT_ERR_BAD_ARG;
  }
  if (warm_start & ~(CPFFT_START_LEARNED | CPFFT_START_ITERATE | CPFFT_START_TRIAL |
                     CPFFT_TANGENT_F32)) {
    cpfft_set_error("cpfft_set_mode: unknown start flags %d", warm_start);
    return CPFFT_ERR_BAD_ARG;
  }
  if (warm_start & CPFFT_START_LEARNED) {
    mlp::Weights w;
    int* err;
    if (!mlp_device_weights(&w, &err)) {
      cpfft_set_error("cpfft_set_mode: the learned initial guess needs cpfft_mlp_init (and "
                      "trained parameters)");
      return CPFFT_ERR_NOT_INIT;
    }
  }
  if (precision == CPFFT_PREC_MIXED) TRY(alloc_mixed(g_ctx));
  if (precision != g_ctx->prec) g_ctx->K4f_valid = false;
  g_ctx->prec = precision;
  g_ctx->warm = warm_start & (CPFFT_START_LEARNED | CPFFT_START_ITERATE | CPFFT_START_TRIAL);
  g_ctx->tangent_f32 = (warm_start & CPFFT_TANGENT_F32) != 0;
  return 0;
}

int cpfft_set_precond(int precond) {
  TRY(need_ctx());
  if (precond != CPFFT_PRECOND_NONE && precond != CPFFT_PRECOND_REFERENCE) {
    cpfft_set_error("cpfft_set_precond: unknown preconditioner %d", precond);
    return CPFFT_ERR_BAD_ARG;
  }
  Ctx* c = g_ctx;
  c->precond = precond;
  c->pre_ok = false;
  // the medium of the current FP32 tangent, if there is one
  if (c->K4f_valid && pre_applies(c)) {
    TRY(reference_reduce(c));
    TRY(sync(c));
    TRY(reference_build(c));
  }
  return 0;
}

int cpfft_set_inexact_newton(double eta_max) {
  TRY(need_ctx());
  if (!(eta_max >= 0.0 && eta_max < 1.0)) {
    cpfft_set_error("cpfft_set_inexact_newton: eta_max must lie in [0, 1)");
    return CPFFT_ERR_BAD_ARG;
  }
  g_ctx->eta_max = eta_max;
  return 0;
}

int cpfft_set_coupled_bc(int on) {
  TRY(need_ctx());
  if (on < 0 || on > 2) {
    cpfft_set_error("cpfft_set_coupled_bc: mode must be 0, 1 or 2");
    return CPFFT_ERR_BAD_ARG;
  }
  g_ctx->coupled_bc = on;
  return 0;
}

int cpfft_set_tangent_tol(double tol) {
  TRY(need_ctx());
  if (!(tol > 0.0 && tol < 1.0)) {
    cpfft_set_error("cpfft_set_tangent_tol: tolerance must lie in (0, 1)");
    return CPFFT_ERR_BAD_ARG;
  }
  g_ctx->th_tol = tol;
  return 0;
}

int cpfft_set_equilibrium_tol(double tol) {
  TRY(need_ctx());
  if (!(tol >= 0.0) || !std::isfinite(tol)) {
    cpfft_set_error("cpfft_set_equilibrium_tol: tolerance must be finite and >= 0");
    return CPFFT_ERR_BAD_ARG;
  }
  g_ctx->eq_tol = tol;
  return 0;
}

int cpfft_tuning(int* tiles, double* ms) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (tiles) {
    tiles[0] = c->g.wtb;
    tiles[1] = c->g.wc2 ? -c->g.wc2 : c->g.wtc;
    tiles[2] = c->gdf.wtb;
    tiles[3] = c->gdf.wtc;
  }
  if (ms) {
    ms[0] = c->tune_ms[0];
    ms[1] = c->tune_ms[1];
  }
  return 0;
}

int cpfft_queue_chunk(int* voxels, int* blocks_per_sm, double* ms) {
  TRY(need_ctx());
  if (voxels) *voxels = g_ctx->qtuned ? g_ctx->qchunk : 0;
  if (blocks_per_sm) *blocks_per_sm = g_ctx->qbps;
  if (ms)
    for (int k = 0; k < 6; k++) ms[k] = g_ctx->qchunk_ms[k];
  return 0;
}

int cpfft_set_tiles(const int* tiles) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (!tiles) {
    cpfft_set_error("cpfft_set_tiles: null pointer");
    return CPFFT_ERR_BAD_ARG;
  }
  if (!c->df_ok) {
    cpfft_set_error("cpfft_set_tiles: no register-FFT passes for this grid (or the mixed "
                    "form was not selected)");
    return CPFFT_ERR_BAD_ARG;
  }
  const int tb = tiles[0], tc = tiles[1], db = tiles[2], dc = tiles[3];
  const bool ok = (tb == 8 || tb == 16 || tb == 32) && (tc == 2 || tc == 4 || tc == -2 || tc == -4) &&
                  (db == 16 || db == 32) && dc == 2;
  if (!ok) {
    cpfft_set_error("cpfft_set_tiles: unsupported tile shapes {%d, %d, %d, %d}", tb, tc, db, dc);
    return CPFFT_ERR_BAD_ARG;
  }
  c->g.wtb = tb;
  c->g.wtc = tc > 0 ? tc : 2;
  c->g.wc2 = tc < 0 ? -tc : 0;
  c->gdf.wtb = db;
  c->gdf.wtc = dc;
  c->gdf.wc2 = 0;
  if (c->cg_exec) {  // the captured CG iteration bakes in the launch shapes
    cudaGraphExecDestroy(c->cg_exec);
    c->cg_exec = nullptr;
  }
  if (c->cg_graph) {
    cudaGraphDestroy(c->cg_graph);
    c->cg_graph = nullptr;
  }
  c->cg_graph_state = 0;
  return 0;
}

int cpfft_set_schedule(int schedule) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (schedule != CPFFT_SCHED_BLOCKS && schedule != CPFFT_SCHED_QUEUE) {
    cpfft_set_error("cpfft_set_schedule: unknown schedule %d", schedule);
    return CPFFT_ERR_BAD_ARG;
  }
  if (schedule == CPFFT_SCHED_QUEUE && !c->vcost) {
    TRY(dalloc(c->vcost, c->N3));
    TRY(dalloc(c->vperm, c->N3 * sizeof(int)));
    TRY(dalloc(c->vq, 129 * sizeof(unsigned int)));
    CK(cudaMemset(c->vcost, 0, c->N3));
  }
  c->sched = schedule;
  return 0;
}

int cpfft_learn_log(long long capacity, int stride, int phase) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (capacity < 0 || stride < 1 || phase < 0 || phase >= stride) {
    cpfft_set_error("cpfft_learn_log: bad arguments");
    return CPFFT_ERR_BAD_ARG;
  }
  for (void* q : {(void*)c->log_X, (void*)c->log_T, (void*)c->log_n})
    if (q) cudaFree(q);
  c->log_X = c->log_T = nullptr;
  c->log_n = nullptr;
  c->log_cap = 0;
  if (capacity == 0) return 0;
  TRY(dalloc(c->log_X, (size_t)capacity * mlp::NIN * sizeof(float)));
  TRY(dalloc(c->log_T, (size_t)capacity * mlp::NOUT * sizeof(float)));
  TRY(dalloc(c->log_n, sizeof(unsigned long long)));
  CK(cudaMemset(c->log_n, 0, sizeof(unsigned long long)));
  c->log_cap = capacity;
  c->log_stride = stride;
  c->log_phase = phase;
  return 0;
}

int cpfft_learn_fetch(float* X, float* T, long long* n) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (!n) {
    cpfft_set_error("cpfft_learn_fetch: n is NULL");
    return CPFFT_ERR_BAD_ARG;
  }
  *n = 0;
  if (!c->log_cap) return 0;
  unsigned long long cnt = 0;
  CK(cudaMemcpyAsync(&cnt, c->log_n, sizeof(cnt), cudaMemcpyDeviceToHost, c->st));
  TRY(sync(c));
  const long long m = std::min<long long>((long long)cnt, c->log_cap);
  if (X) CK(cudaMemcpyAsync(X, c->log_X, (size_t)m * mlp::NIN * sizeof(float), cudaMemcpyDeviceToHost, c->st));
  if (T) CK(cudaMemcpyAsync(T, c->log_T, (size_t)m * mlp::NOUT * sizeof(float), cudaMemcpyDeviceToHost, c->st));
  TRY(sync(c));
  *n = m;
  return 0;
}

int cpfft_set_F(const double* Fn, const double* Fn1) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  const size_t f9 = 9 * c->N3 * sizeof(double);
  if (Fn) CK(cudaMemcpyAsync(c->Fn, Fn, f9, cudaMemcpyHostToDevice, c->st));
  if (Fn1) CK(cudaMemcpyAsync(c->Fn1, Fn1, f9, cudaMemcpyHostToDevice, c->st));
  return sync(c);
}

int cpfft_stress_update(int step, int iter, const double* Fn, const double* Fn1, double* Pn1,
                        double* K4) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (step < 1 || iter < 0) {
    cpfft_set_error("cpfft_stress_update: step >= 1 and iter >= 0 required");
    return CPFFT_ERR_BAD_ARG;
  }
  TRY(cpfft_set_F(Fn, Fn1));
  long long li;
  int fails;
  TRY(stress(c, step, iter, &li, &fails));
  if (Pn1) CK(cudaMemcpyAsync(Pn1, c->P, 9 * c->N3 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  if (K4) CK(cudaMemcpyAsync(K4, c->K4, 81 * c->N3 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  TRY(sync(c));
  return fails ? CPFFT_WARN_LOCAL_FALLBACK : 0;
}

int cpfft_pass_counts(long long* counts) {
  TRY(need_ctx());
  if (!counts) {
    cpfft_set_error("cpfft_pass_counts: null pointer");
    return CPFFT_ERR_BAD_ARG;
  }
  for (int k = 0; k < 5; k++) counts[k] = g_ctx->last_pass[k];
  return 0;
}

int cpfft_set_K4(const double* K4) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  CK(cudaMemcpyAsync(c->K4, K4, 81 * c->N3 * sizeof(double), cudaMemcpyHostToDevice, c->st));
  if (c->prec == CPFFT_PREC_MIXED) {
    // FP32 copy for the inner solves (and its FP32 remainder for the double-float operator)
    std::vector<float> kf(81 * c->N3);
    for (long long i = 0; i < 81 * c->N3; i++) kf[i] = (float)K4[i];
    CK(cudaMemcpyAsync(c->K4f, kf.data(), kf.size() * sizeof(float), cudaMemcpyHostToDevice, c->st));
    TRY(sync(c));
    if (c->df_ok) {
      for (long long i = 0; i < 81 * c->N3; i++) kf[i] = (float)(K4[i] - (double)(float)K4[i]);
      CK(cudaMemcpyAsync(c->K4lo, kf.data(), kf.size() * sizeof(float), cudaMemcpyHostToDevice, c->st));
      TRY(sync(c));
    }
    c->K4f_valid = true;
    if (pre_applies(c)) {
      TRY(reference_reduce(c));
      TRY(sync(c));
      TRY(reference_build(c));
    }
  }
  return sync(c);
}

int cpfft_green_apply(const double* x, double* y, int flgK) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  const size_t f9 = 9 * c->N3 * sizeof(double);
  CK(cudaMemcpyAsync(c->io, x, f9, cudaMemcpyHostToDevice, c->st));
  TRY(matvec64(c, c->io, c->b, flgK ? 1 : 0));
  CK(cudaMemcpyAsync(y, c->b, f9, cudaMemcpyDeviceToHost, c->st));
  return sync(c);
}

int cpfft_green_apply_f32(const float* x, float* y, int flgK) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (c->prec != CPFFT_PREC_MIXED || (flgK && !c->K4f_valid)) {
    cpfft_set_error("cpfft_green_apply_f32: needs mixed precision and, with K, the FP32 "
                    "tangent of a stress update");
    return CPFFT_ERR_BAD_ARG;
  }
  const size_t f9 = 9 * c->N3 * sizeof(float);
  CK(cudaMemcpyAsync(c->rf, x, f9, cudaMemcpyHostToDevice, c->st));
  c->f32_matvecs++;
  TRY(cuda_check(green_apply<float>(c->rf, c->K4f, flgK ? 1 : 0, c->Apf, c->Sf, c->twf, c->g, c->st),
                 "green_apply fp32"));
  CK(cudaMemcpyAsync(y, c->Apf, f9, cudaMemcpyDeviceToHost, c->st));
  return sync(c);
}

int cpfft_green_apply_df(const double* x, double* y, int flgK) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (c->prec != CPFFT_PREC_MIXED || !c->df_ok || (flgK && !c->K4f_valid)) {
    cpfft_set_error("cpfft_green_apply_df: needs mixed precision, N in {32, 64, 128, 256} "
                    "and, with K, the tangent of a stress update");
    return CPFFT_ERR_BAD_ARG;
  }
  const size_t f9 = 9 * c->N3 * sizeof(double);
  CK(cudaMemcpyAsync(c->io, x, f9, cudaMemcpyHostToDevice, c->st));
  TRY(matvec_acc(c, c->io, c->b, flgK ? 1 : 0));
  CK(cudaMemcpyAsync(y, c->b, f9, cudaMemcpyDeviceToHost, c->st));
  return sync(c);
}

int cpfft_cg(const double* b, double* x, double tol, int* iters) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  c->cg_rel_only = false;
  const size_t f9 = 9 * c->N3 * sizeof(double);
  int its = 0;
  CK(cudaMemcpyAsync(c->b, b, f9, cudaMemcpyHostToDevice, c->st));
  int rc = cg(c, c->b, c->io, tol, &its);
  if (iters) *iters = its;
  if (rc < 0 && rc != CPFFT_ERR_CG_MAXIT) return rc;
  CK(cudaMemcpyAsync(x, c->io, f9, cudaMemcpyDeviceToHost, c->st));
  TRY(sync(c));
  return rc;
}

int cpfft_tangent_homo(double tolPCG, double* C_homo) {
  TRY(need_ctx());
  int its;
  double C[81];
  TRY(tangent_homo(g_ctx, tolPCG, C, &its));
  if (C_homo) memcpy(C_homo, C, sizeof(C));
  return 0;
}

int cpfft_nr3_begin(double tolPCG) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  long long li;
  int fails, its;
  TRY(stress(c, 1, 0, &li, &fails));
  TRY(tangent_homo(c, tolPCG, c->C_homo, &its));
  return 0;
}

// One load step with the mixed boundary conditions inside the Newton iteration
// (cpfft_set_coupled_bc; needs the equilibrium test).  FFT_nr3 nests
// a Newton loop at fixed macroscopic F inside a loop over P_bar updates
// (src/FFT_nr3.f:75-171), and each P_bar pass starts again with an explicit stress pass.
// Here each Newton iteration updates the prescribed-stress components of F_bar as well:
// after the stress pass, DbarF solves C_homo DbarF = PBC - P_bar on those components
// (NBC_update, src/FFT_nr3.f:375-433), and the fluctuation solves
// G(K : dF) = -G(P) - G(K : DbarF), so that F_bar and the fluctuation take one
// Newton step on the coupled system (C_homo is that system's Schur complement).  C_homo
// is recomputed after the first implicit stress pass (a second recomputation after the
// next pass left the stress-pass count unchanged); increments that raise the equilibrium
// residual are halved as in the nested loops.  The step ends when P_bar
// meets tolNR, the equilibrium residual eq_tol and the last increment tolNR, the same
// tests as the nested loops' last pass.  On entry barF holds F_bar with the step's
// predicted DbarF applied and Fn1 the predictor's field.
int coupled_step(Ctx* c, int step, const double* PBC, const int* isNBC, double* barF,
                 double Fnorm, double tolNR, double tolPCG, int maxIter, cpfft_stats& S,
                 double& tp, double& ts) {
  using clk = std::chrono::steady_clock;
  auto sec = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
  const long long N3 = c->N3, n = 9 * N3;
  const bool inexact = c->eta_max > 0.0;
  double resfft = 1.0, eta = c->eta_max, eq_last = HUGE_VAL;
  int tangents = 0;
  // backtracking as in the nested loops: an increment after which the equilibrium
  // residual has grown is halved, at most 4 times in a row (lastD: its F_bar part)
  double eq_prev = HUGE_VAL, frac = 1.0, lastD[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int halvings = 0;
  // ||dF||^2 of the last solve is summed into SC_T1 on the device and read back with the
  // next equilibrium residual (one host wait fewer per iteration)
  bool pending_dn = false;
  double pending_db = 0.0;
  int pending_its = 0, pending_fails = 0;
  for (int k = 0;; k++) {
    auto a = clk::now();
    long long li, pi = 0, rj = 0;
    int fails;
    // mode 2: no explicit opening pass (the stress kernel's iteration 0)
    TRY(stress(c, step, c->coupled_bc == 2 ? k + 1 : k, &li, &fails, &pi, &rj));
    ts += sec(a);
    S.predict_iters += pi;
    S.guess_rejected += rj;
    S.local_iters += li;
    S.local_fallbacks += fails;
    S.stress_updates++;
    TRY(matvec_acc(c, c->P, c->b, 0));
    double e;
    TRY(equil_residual(c, c->b, &e));  // also leaves sum(P) and SC_T1 in h_sc
    S.res_equil = e;
    if (pending_dn) {
      resfft = std::sqrt(c->h_sc[SC_T1] + (double)N3 * pending_db) / Fnorm;
      pending_dn = false;
      if (!std::isfinite(resfft)) { cpfft_set_error("Newton residual is not finite"); return CPFFT_ERR_NONFINITE; }
      S.newton_iters++;
      S.res_fft = resfft;
      if (c->log)
        fprintf(stderr, "       Iteration %5d  residual %10.3e  (cg %d, local fallbacks %d)\n", k - 1,
                resfft, pending_its, pending_fails);
    }
    double res1 = 0, res2 = 0;
    for (int i = 0; i < 9; i++) {
      c->P_bar[i] = c->h_sc[SC_SUM9 + i] / (double)N3;
      res2 += c->P_bar[i] * c->P_bar[i];
      if (isNBC[i]) res1 += (c->P_bar[i] - PBC[i]) * (c->P_bar[i] - PBC[i]);
    }
    const double res3 = res2 < 1.0e-8 ? std::sqrt(res1) : std::sqrt(res1 / res2);
    S.res_pbar = res3;
    if (c->log)
      fprintf(stderr, "       coupled iteration %d: equilibrium %10.3e  P_bar %10.3e\n", k, e, res3);
    if (res3 <= tolNR && e <= c->eq_tol && resfft <= tolNR) break;
    if (k == maxIter) {
      cpfft_set_error("coupled Newton loop does not converge (step %d)", step);
      return CPFFT_ERR_NEWTON_MAXIT;
    }
    if (k >= 2 && e > eq_prev && halvings < 4) {
      frac *= 0.5;
      double h[9];
      for (int i = 0; i < 9; i++) {
        h[i] = -frac * lastD[i];
        barF[i] += h[i];
      }
      CK(dev_axpy(c->Fn1, c->dFm, -frac, n, c->st));
      CK(dev_fill9(c->w, N3, h, c->st));
      CK(dev_axpy(c->Fn1, c->w, 1.0, n, c->st));
      halvings++;
      resfft *= 0.5;
      if (c->log) fprintf(stderr, "       increment halved (%d)\n", halvings);
      continue;
    }
    eq_prev = e;
    halvings = 0;
    frac = 1.0;
    // the Schur complement at the first implicit state (tangent_homo's solves use the b
    // buffer: G(P) is formed again after it)
    if (k >= (c->coupled_bc == 2 ? 0 : 1) && tangents < 1) {
      a = clk::now();
      int th;
      TRY(tangent_homo(c, inexact ? std::max(tolPCG, c->th_tol) : tolPCG, c->C_homo, &th));
      tp += sec(a);
      tangents++;
      TRY(matvec_acc(c, c->P, c->b, 0));
    }
    double DbarF[9];
    for (int i = 0; i < 9; i++) DbarF[i] = 0.0;
    TRY(nbc_update(c->C_homo, DbarF, c->P_bar, PBC, isNBC));
    // right-hand side -G(P) - G(K : DbarF)
    CK(dev_fill9(c->dFm, N3, DbarF, c->st));
    CK(dev_scale(c->b, -1.0, n, c->st));
    TRY(matvec_acc(c, c->dFm, c->w, 1));
    CK(dev_axpy(c->b, c->w, -1.0, n, c->st));
    CK(dev_axpy(c->Fn1, c->dFm, 1.0, n, c->st));  // F_bar += DbarF
    for (int i = 0; i < 9; i++) {
      barF[i] += DbarF[i];
      lastD[i] = DbarF[i];
    }
    double tol_k = tolPCG;
    if (inexact) {  // Eisenstat-Walker forcing as in the nested loops
      double eta_k = eq_last < HUGE_VAL ? 0.9 * (e / eq_last) * (e / eq_last) : c->eta_max;
      const double sg = 0.9 * eta * eta;
      if (sg > 0.1) eta_k = std::max(eta_k, sg);
      eta_k = std::max(eta_k, 0.5 * c->eq_tol / e);
      eta = std::min(c->eta_max, eta_k);
      eq_last = e;
      tol_k = std::max(tolPCG, eta);
    }
    a = clk::now();
    int its;
    c->cg_rel_only = inexact;
    TRY(cg(c, c->b, c->dFm, tol_k, &its));
    c->cg_rel_only = false;
    tp += sec(a);
    CK(dev_axpy(c->Fn1, c->dFm, 1.0, n, c->st));
    CK(dev_dot(c->dFm, c->dFm, n, c->part, c->sc, SC_T1, OP_STORE, c->st));
    pending_db = 0.0;
    for (int i = 0; i < 9; i++) pending_db += DbarF[i] * DbarF[i];
    pending_dn = true;
    pending_its = its;
    pending_fails = fails;
  }
  S.nbc_iters = 1;
  return 0;
}

int cpfft_nr3_step(int step, const double* BC, const int* isNBC, double tolNR, double tolPCG,
                   int maxIter, double* Pbar, cpfft_stats* st) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (!BC || !isNBC || step < 1) {
    cpfft_set_error("cpfft_nr3_step: invalid argument");
    return CPFFT_ERR_BAD_ARG;
  }
  using clk = std::chrono::steady_clock;
  auto sec = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
  auto t0 = clk::now();
  cpfft_stats S;
  memset(&S, 0, sizeof(S));
  c->cg_iters = c->cg_solves = c->f64_matvecs = c->f32_matvecs = 0;
  c->syncs = 0;
  c->cg_rel_only = false;
  TRY(kt_drain(c));
  kt_reset(c);
  const long long launches0 = g_kernel_launches;
  CK(cudaEventRecord(c->step_ev[0], c->st));
  const long long N3 = c->N3, n = 9 * N3;
  bool existNBC = false;
  for (int i = 0; i < 9; i++) existNBC |= isNBC[i] != 0;
  double PBC[9], FBC[9], DbarF[9], barF[9];
  for (int i = 0; i < 9; i++) {
    PBC[i] = FBC[i] = DbarF[i] = 0.0;
    if (isNBC[i]) PBC[i] = BC[i];
    else { FBC[i] = BC[i]; DbarF[i] = FBC[i] - c->barF_t[i]; }
  }
  if (existNBC) TRY(nbc_update(c->C_homo, DbarF, c->P_bar, PBC, isNBC));
  for (int i = 0; i < 9; i++) barF[i] = c->barF_t[i] + DbarF[i];
  int iiter_NBC = 0;
  double tp = 0, ts = 0;
  for (;;) {
    CK(dev_fill9(c->dFm, N3, DbarF, c->st));
    double Fnorm;
    TRY(dnrm2(c, c->Fn1, &Fnorm));
    CK(dev_axpy(c->Fn1, c->dFm, 1.0, n, c->st));
    TRY(matvec_acc(c, c->dFm, c->b, 1));
    CK(dev_scale(c->b, -1.0, n, c->st));
    int its;
    auto a = clk::now();
    // inexact Newton: the predictor's system only starts the iteration
    const bool inexact = c->eta_max > 0.0 && c->eq_tol > 0.0;
    c->cg_rel_only = inexact;
    TRY(cg(c, c->b, c->dFm, inexact ? std::max(tolPCG, c->eta_max) : tolPCG, &its));
    c->cg_rel_only = false;
    tp += sec(a);
    CK(dev_axpy(c->Fn1, c->dFm, 1.0, n, c->st));
    if (c->eq_tol > 0.0 && existNBC && c->coupled_bc) {
      TRY(coupled_step(c, step, PBC, isNBC, barF, Fnorm, tolNR, tolPCG, maxIter, S, tp, ts));
      break;
    }
    double resfft = 1.0;
    double eta = c->eta_max, eq_last = HUGE_VAL;
    int iiter_EBC = 0;
    // With the equilibrium test the loop body starts with the stress update, so the
    // update that follows the last accepted increment (the reference's closing
    // drive_eps_sig) also evaluates the test: the loop ends there when both tests pass.
    bool closed = false;  // the state's P is current (the closing update has run)
    const bool eq_mode = c->eq_tol > 0.0;
    // backtracking on the equilibrium residual (equilibrium test only): an increment
    // after which the residual has grown is halved, at most 4 times, before the next solve
    double eq_prev = HUGE_VAL, frac = 1.0;
    int halvings = 0;
    while (eq_mode || resfft > tolNR) {
      a = clk::now();
      long long li;
      int fails;
      long long pi = 0, rj = 0;
      TRY(stress(c, step, iiter_EBC, &li, &fails, &pi, &rj));
      ts += sec(a);
      S.predict_iters += pi;
      S.guess_rejected += rj;
      S.local_iters += li;
      S.local_fallbacks += fails;
      S.stress_updates++;
      TRY(matvec_acc(c, c->P, c->b, 0));
      if (eq_mode || c->log) {
        double eq;
        TRY(equil_residual(c, c->b, &eq));
        S.res_equil = eq;
        if (c->log)
          fprintf(stderr, "       equilibrium residual %10.3e (iteration %d)\n", eq, iiter_EBC);
        if (eq_mode && resfft <= tolNR && eq <= c->eq_tol) {
          closed = true;
          break;
        }
        if (eq_mode && iiter_EBC >= 2 && eq > eq_prev && halvings < 4) {
          frac *= 0.5;
          CK(dev_axpy(c->Fn1, c->dFm, -frac, n, c->st));
          halvings++;
          resfft *= 0.5;
          if (c->log) fprintf(stderr, "       increment halved (%d)\n", halvings);
          continue;
        }
        eq_prev = eq;
        halvings = 0;
        frac = 1.0;
      }
      CK(dev_scale(c->b, -1.0, n, c->st));
      double tol_k = tolPCG;
      if (inexact) {
        // Eisenstat-Walker forcing (choice 2, gamma 0.9, exponent 2) with its safeguard,
        // no tighter than the equilibrium tolerance needs, never below tolPCG
        const double e = S.res_equil;
        double eta_k = eq_last < HUGE_VAL ? 0.9 * (e / eq_last) * (e / eq_last) : c->eta_max;
        const double sg = 0.9 * eta * eta;
        if (sg > 0.1) eta_k = std::max(eta_k, sg);
        eta_k = std::max(eta_k, 0.5 * c->eq_tol / e);
        eta = std::min(c->eta_max, eta_k);
        eq_last = e;
        tol_k = std::max(tolPCG, eta);
      }
      a = clk::now();
      c->cg_rel_only = inexact;
      TRY(cg(c, c->b, c->dFm, tol_k, &its));
      c->cg_rel_only = false;
      tp += sec(a);
      CK(dev_axpy(c->Fn1, c->dFm, 1.0, n, c->st));
      double dn;
      TRY(dnrm2(c, c->dFm, &dn));
      resfft = dn / Fnorm;
      if (!std::isfinite(resfft)) { cpfft_set_error("Newton residual is not finite"); return CPFFT_ERR_NONFINITE; }
      S.newton_iters++;
      S.res_fft = resfft;
      if (c->log)  // the reference's per-iteration report (src/FFT_nr3.f:115, format 1001)
        fprintf(stderr, "       Iteration %5d  residual %10.3e  (cg %d, local fallbacks %d)\n",
                iiter_EBC, resfft, its, fails);
      if (iiter_EBC == maxIter) {
        cpfft_set_error("Newton loop does not converge (step %d)", step);
        return CPFFT_ERR_NEWTON_MAXIT;
      }
      iiter_EBC++;
    }
    if (!closed) {
      a = clk::now();
      long long li;
      int fails;
      long long pi = 0, rj = 0;
      TRY(stress(c, step, iiter_EBC, &li, &fails, &pi, &rj));
      ts += sec(a);
      S.predict_iters += pi;
      S.guess_rejected += rj;
      S.local_iters += li;
      S.local_fallbacks += fails;
      S.stress_updates++;
    }
    CK(dev_sum9(c->P, N3, c->part, c->sc, SC_SUM9, c->st));
    CK(cudaMemcpyAsync(c->h_sc + SC_SUM9, c->sc + SC_SUM9, 9 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    TRY(sync(c));
    double res1 = 0, res2 = 0;
    for (int i = 0; i < 9; i++) {
      c->P_bar[i] = c->h_sc[SC_SUM9 + i] / (double)N3;
      res2 += c->P_bar[i] * c->P_bar[i];
      if (isNBC[i]) res1 += (c->P_bar[i] - PBC[i]) * (c->P_bar[i] - PBC[i]);
    }
    double res3 = res2 < 1.0e-8 ? std::sqrt(res1) : std::sqrt(res1 / res2);
    S.res_pbar = res3;
    if (c->log)  // src/FFT_nr3.f:148, format 1002
      fprintf(stderr, "       Stress iteration %5d  residual %10.3e\n", iiter_NBC, res3);
    S.nbc_iters = iiter_NBC + 1;
    if (res3 <= tolNR) break;
    if (iiter_NBC > maxIter) {
      cpfft_set_error("prescribed stress cannot be reached (step %d)", step);
      return CPFFT_ERR_NBC_MAXIT;
    }
    a = clk::now();
    int th;
    // the homogenised tangent only steers the P_bar update (its loop tests P_bar itself)
    TRY(tangent_homo(c, inexact ? std::max(tolPCG, c->th_tol) : tolPCG, c->C_homo, &th));
    tp += sec(a);
    for (int i = 0; i < 9; i++) DbarF[i] = 0.0;
    TRY(nbc_update(c->C_homo, DbarF, c->P_bar, PBC, isNBC));
    for (int i = 0; i < 9; i++) barF[i] += DbarF[i];
    iiter_NBC++;
  }
  // roll-over: Fn <- Fn1, history n <- n+1 (src/FFT_nr3.f:173-179, src/update.f)
  for (int i = 0; i < 9; i++) c->barF_t[i] = barF[i];
  CK(cudaMemcpyAsync(c->Fn, c->Fn1, n * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
  c->hn = 1 - c->hn;
  c->pass_step = 0;
  if (Pbar)
    for (int i = 0; i < 9; i++) Pbar[i] = c->P_bar[i];
  // equilibrium residual ||G(P)|| / (sqrt(N3) ||P_bar||) of the committed state (the
  // equilibrium test has evaluated it on that state already)
  if (!c->eq_tol) {
    TRY(matvec_acc(c, c->P, c->b, 0));
    TRY(equil_residual(c, c->b, &S.res_equil));
  }
  S.cg_solves = (int)c->cg_solves;
  S.cg_iters = (int)c->cg_iters;
  S.t_pcg = tp;
  S.t_sigeps = ts;
  CK(cudaEventRecord(c->step_ev[1], c->st));
  TRY(kt_drain(c));
  CK(cudaEventSynchronize(c->step_ev[1]));
  {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->step_ev[0], c->step_ev[1]));
    S.t_device = 1e-3 * ms;
  }
  S.t_stress_kernel = c->kt_acc[KT_STRESS];
  S.t_green64 = c->kt_acc[KT_G64];
  S.t_green32 = c->kt_acc[KT_G32];
  S.n_green64 = c->kt_cnt[KT_G64];
  S.n_green32 = c->f32_matvecs;
  S.n_green32_timed = c->kt_cnt[KT_G32];
  S.t_cg_graph = c->kt_acc[KT_CGGRAPH];
  S.kernel_launches = g_kernel_launches - launches0;
  if (c->log)
    fprintf(stderr, "       step %d: %lld host synchronisations, %lld kernel launches\n", step,
            c->syncs, S.kernel_launches);
  S.t_total = sec(t0);
  if (st) *st = S;
  return S.local_fallbacks ? CPFFT_WARN_LOCAL_FALLBACK : 0;
}

int cpfft_sync_to_host(double* Fn1, double* Pn1, double* history) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  const size_t f9 = 9 * c->N3 * sizeof(double);
  if (Fn1) CK(cudaMemcpyAsync(Fn1, c->Fn1, f9, cudaMemcpyDeviceToHost, c->st));
  if (Pn1) CK(cudaMemcpyAsync(Pn1, c->P, f9, cudaMemcpyDeviceToHost, c->st));
  if (history)
    CK(cudaMemcpyAsync(history, c->hist[c->hn], c->hist_words * c->N3 * sizeof(double),
                       cudaMemcpyDeviceToHost, c->st));
  return sync(c);
}

int cpfft_hist_words(void) {
  TRY(need_ctx());
  return g_ctx->hist_words;
}

int cpfft_slip_systems(int slip_type, double* b, double* n) {
  double bb[48][3], nn[48][3];
  const int ns = slip_geometry(slip_type, bb, nn);
  if (!ns) {
    cpfft_set_error("cpfft_slip_systems: slip_type %d has no slip table here", slip_type);
    return CPFFT_ERR_BAD_ARG;
  }
  for (int s = 0; s < ns; s++)
    for (int i = 0; i < 3; i++) {
      if (b) b[3 * s + i] = bb[s][i];
      if (n) n[3 * s + i] = nn[s][i];
    }
  return ns;
}

int cpfft_commit_step(void) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  CK(cudaMemcpyAsync(c->Fn, c->Fn1, 9 * c->N3 * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
  c->hn = 1 - c->hn;
  c->pass_step = 0;
  return sync(c);
}

// ---- many RVEs: one context per RVE, worker threads over a largest-first queue --------
static void batch_one(cpfft_rve& r, int precision, int options, int precond, int schedule,
                      const cpfft_newton* nt, double tolNR, double tolPCG, int maxIter) {
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  r.status = 0;
  r.steps_done = 0;
  r.voxel_updates = 0;
  r.cg_iters = 0;
  r.error[0] = 0;
  auto fail = [&](int rc) {
    r.status = rc;
    snprintf(r.error, sizeof(r.error), "%s", cpfft_last_error());
  };
  int rc = cpfft_init(r.N, r.matList, r.kocks_deg, r.props, r.ncrystals, r.tstep, r.g_mapping);
  for (int m = 0; rc >= 0 && r.mises && m < r.ncrystals; m++)
    if (r.props[m].slip_type == CPFFT_NOT_A_CRYSTAL) rc = cpfft_set_mises(m + 1, &r.mises[m]);
  if (rc < 0) { fail(rc); r.seconds = std::chrono::duration<double>(clk::now() - t0).count(); return; }
  if ((rc = cpfft_set_mode(precision, options)) < 0 ||
      (precision == CPFFT_PREC_MIXED && (rc = cpfft_set_precond(precond)) < 0) ||
      (precision == CPFFT_PREC_MIXED && (rc = cpfft_set_schedule(schedule)) < 0) ||
      (nt && ((rc = cpfft_set_equilibrium_tol(nt->equilibrium_tol)) < 0 ||
              (rc = cpfft_set_inexact_newton(nt->eta_max)) < 0 ||
              (nt->tangent_tol > 0.0 && (rc = cpfft_set_tangent_tol(nt->tangent_tol)) < 0) ||
              (rc = cpfft_set_coupled_bc(nt->coupled_bc)) < 0)) ||
      (rc = cpfft_nr3_begin(tolPCG)) < 0) {
    fail(rc);
  } else {
    const long long N3 = (long long)r.N * r.N * r.N;
    for (int s = 1; s <= r.nsteps; s++) {
      cpfft_stats st;
      double pb[9];
      rc = cpfft_nr3_step(s, r.BC_all + 9 * (s - 1), r.isNBC, tolNR, tolPCG, maxIter, pb, &st);
      if (rc < 0) { fail(rc); break; }
      if (rc > r.status) r.status = rc;
      if (r.Pbar) memcpy(r.Pbar + 9 * (s - 1), pb, sizeof(pb));
      r.steps_done = s;
      r.voxel_updates += N3 * st.stress_updates;
      r.cg_iters += st.cg_iters;
    }
    if (r.status >= 0 && (r.Fn1 || r.Pn1) && (rc = cpfft_sync_to_host(r.Fn1, r.Pn1, nullptr)) < 0)
      fail(rc);
  }
  cpfft_finalize();
  r.seconds = std::chrono::duration<double>(clk::now() - t0).count();
}

int cpfft_batch_solve(cpfft_rve* rves, int nrve, int precision, int options, int precond,
                      int schedule, double tolNR, double tolPCG, int maxIter, int nthreads) {
  return cpfft_batch_solve_newton(rves, nrve, precision, options, precond, schedule, nullptr,
                                  tolNR, tolPCG, maxIter, nthreads);
}

int cpfft_batch_solve_newton(cpfft_rve* rves, int nrve, int precision, int options,
                             int precond, int schedule, const cpfft_newton* nt,
                             double tolNR, double tolPCG, int maxIter, int nthreads) {
  if (nrve < 0 || (nrve > 0 && !rves) || nthreads < 1) {
    cpfft_set_error("cpfft_batch_solve: invalid argument");
    return CPFFT_ERR_BAD_ARG;
  }
  // the setters' own ranges, checked here so that no RVE starts with options it refuses
  if (nt && (!(nt->equilibrium_tol >= 0.0) || !std::isfinite(nt->equilibrium_tol) ||
             !(nt->eta_max >= 0.0 && nt->eta_max < 1.0) ||
             !(nt->tangent_tol >= 0.0 && nt->tangent_tol < 1.0) || nt->coupled_bc < 0 ||
             nt->coupled_bc > 2)) {
    cpfft_set_error("cpfft_batch_solve_newton: Newton option out of range");
    return CPFFT_ERR_BAD_ARG;
  }
  for (int k = 0; k < nrve; k++)
    if (rves[k].nsteps < 0 || (rves[k].nsteps > 0 && (!rves[k].BC_all || !rves[k].isNBC))) {
      cpfft_set_error("cpfft_batch_solve: RVE %d has no loading", k);
      return CPFFT_ERR_BAD_ARG;
    }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cpfft_set_error("cpfft_batch_solve: no CUDA device");
    return CPFFT_ERR_CUDA;
  }
  std::vector<int> order(nrve);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return rves[a].N > rves[b].N; });
  std::atomic<int> next{0};
  auto worker = [&]() {
    cudaSetDevice(dev);
    for (;;) {
      const int k = next.fetch_add(1);
      if (k >= nrve) break;
      batch_one(rves[order[k]], precision, options, precond, schedule, nt, tolNR, tolPCG,
                maxIter);
    }
  };
  std::vector<std::thread> pool;
  for (int i = 0; i < std::min(nthreads, nrve); i++) pool.emplace_back(worker);
  for (auto& t : pool) t.join();
  for (int k = 0; k < nrve; k++)
    if (rves[k].status < 0) {
      cpfft_set_error("RVE %d: %s", k, rves[k].error);
      return rves[k].status;
    }
  return 0;
}

// ---- element result files (ouelestr / oupestr / ouddpa_flat_header) -----------------
int cpfft_format_e15(const double* x, long long n, char* out) {
  if (n < 0 || (n > 0 && (!x || !out))) {
    cpfft_set_error("cpfft_format_e15: invalid argument");
    return CPFFT_ERR_BAD_ARG;
  }
  if (n == 0) return 0;
  double* dx = nullptr;
  char* dout = nullptr;
  unsigned char* dfl = nullptr;
  int rc = 0;
  if ((rc = dalloc(dx, n * sizeof(double))) || (rc = dalloc(dout, n * 15)) ||
      (rc = dalloc(dfl, n))) {
    cudaFree(dx); cudaFree(dout); cudaFree(dfl);
    return rc;
  }
  std::vector<unsigned char> fl(n);
  cudaError_t e;
  if ((e = cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice)) ||
      (e = launch_format_values(dx, n, dout, dfl, 0)) ||
      (e = cudaMemcpy(out, dout, n * 15, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(fl.data(), dfl, n, cudaMemcpyDeviceToHost)))
    rc = cuda_check(e, "cpfft_format_e15");
  cudaFree(dx); cudaFree(dout); cudaFree(dfl);
  if (rc) return rc;
  for (long long i = 0; i < n; i++)
    if (fl[i]) host_e15(x[i], out + 15 * i);
  return 0;
}

int cpfft_format_flat(int quantity, char* text, long long capacity, long long* length) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (quantity != 1 && quantity != 2) {
    cpfft_set_error("cpfft_format_flat: quantity must be 1 (strains) or 2 (stresses)");
    return CPFFT_ERR_BAD_ARG;
  }
  const int nvals = quantity == 2 ? 26 : 22;  // num_short_stress / num_short_strain + 15
  const int word0 = quantity == 2 ? H_SIG : H_EPS;
  const long long L = nvals * 15LL + 1, total = c->N3 * L;
  if (length) *length = total;
  if (!text || capacity < total) {
    cpfft_set_error("cpfft_format_flat: buffer of %lld bytes needed", total);
    return CPFFT_ERR_BAD_ARG;
  }
  char* dt = nullptr;
  unsigned char* dfl = nullptr;
  int rc = 0;
  if ((rc = dalloc(dt, total)) || (rc = dalloc(dfl, 6 * c->N3))) {
    cudaFree(dt);
    cudaFree(dfl);
    return rc;
  }
  std::vector<unsigned char> fl(6 * c->N3);
  cudaError_t e;
  if ((e = launch_format_flat(c->hist[c->hn], c->N3, word0, nvals, dt, dfl, c->st)) ||
      (e = cudaMemcpyAsync(text, dt, total, cudaMemcpyDeviceToHost, c->st)) ||
      (e = cudaMemcpyAsync(fl.data(), dfl, 6 * c->N3, cudaMemcpyDeviceToHost, c->st)) ||
      (e = cudaStreamSynchronize(c->st)))
    rc = cuda_check(e, "cpfft_format_flat");
  cudaFree(dt);
  cudaFree(dfl);
  if (rc) return rc;
  // the fields the device could not round exactly: formatted here from the same values
  std::vector<double> hv;
  for (long long v = 0; v < c->N3; v++)
    for (int j = 0; j < 6; j++)
      if (fl[6 * v + j]) {
        if (hv.empty()) {
          hv.resize(6 * c->N3);
          std::vector<double> w(c->N3);
          for (int jj = 0; jj < 6; jj++) {
            CK(cudaMemcpy(w.data(), c->hist[c->hn] + (word0 + jj) * c->N3, c->N3 * sizeof(double),
                          cudaMemcpyDeviceToHost));
            for (long long u = 0; u < c->N3; u++) hv[6 * u + jj] = w[u];
          }
        }
        double x = hv[6 * v + j];
        if (std::fabs(x) < 1.0e-30) x = 0.0;
        host_e15(x, text + v * L + 15 * j);
      }
  return 0;
}

int cpfft_write_flat(int quantity, int step, const char* structure_name, const char* directory) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  long long total = 0;
  cpfft_format_flat(quantity, nullptr, 0, &total);
  if (quantity != 1 && quantity != 2) return CPFFT_ERR_BAD_ARG;
  std::vector<char> text(total);
  TRY(cpfft_format_flat(quantity, text.data(), total, &total));
  // wes / wee + step (i5.5) + _text (ouocst_elem, src/ouresult.f:700-712)
  int stepno = step > 99999 ? step - 99999 : step;
  char name[64];
  snprintf(name, sizeof(name), "%s%05d_text", quantity == 2 ? "wes" : "wee", stepno);
  std::string path = directory && directory[0] ? std::string(directory) + "/" + name : name;
  FILE* f = fopen(path.c_str(), "w");
  if (!f) {
    cpfft_set_error("cpfft_write_flat: cannot open %s", path.c_str());
    return CPFFT_ERR_BAD_ARG;
  }
  // header (ouddpa_flat_header, src/ouresult.f:335-396)
  char sname[9];
  snprintf(sname, sizeof(sname), "%-8.8s", structure_name ? structure_name : "");
  time_t now = time(nullptr);
  char date[32];
  strftime(date, sizeof(date), "%a %b %e %H:%M:%S %Y", localtime(&now));  // fdate's layout
  const long long nonode = (long long)(c->N + 1) * (c->N + 1) * (c->N + 1);
  fprintf(f, "#\n#  WARP3D element results: %-15s\n#  Structure name: %s\n"
             "#  Model nodes, elements: %8lld%8lld\n#  %-24s\n#  Load(time) step: %8d\n#\n",
          quantity == 2 ? "stresses" : "strains", sname, nonode, c->N3, date, step);
  const size_t w = fwrite(text.data(), 1, text.size(), f);
  fclose(f);
  if (w != text.size()) {
    cpfft_set_error("cpfft_write_flat: short write to %s", path.c_str());
    return CPFFT_ERR_BAD_ARG;
  }
  return 0;
}

// ---- nodal displacements (f2disp) -----------------------------------------------------
int cpfft_f2disp(double lx, double ly, double lz, double* u) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  if (!u || !(lx > 0) || !(ly > 0) || !(lz > 0)) {
    cpfft_set_error("cpfft_f2disp: invalid argument");
    return CPFFT_ERR_BAD_ARG;
  }
  const int N = c->N;
  const long long N1 = N + 1, nodes = N1 * N1 * N1;
  // cos(pi k i / N) with the angle reduced to [0, 2 pi) in integers first
  std::vector<double> ctab(N1 * N1);
  for (long long k = 0; k < N1; k++)
    for (long long i = 0; i < N1; i++) {
      const long long m = (k * i) % (2LL * N);
      ctab[k * N1 + i] = (double)cosl(3.14159265358979323846264338327950288L * m / N);
    }
  double *dtab = nullptr, *work = nullptr, *du = nullptr;
  int rc = 0;
  if ((rc = dalloc(dtab, ctab.size() * sizeof(double))) ||
      (rc = dalloc(work, 6 * nodes * sizeof(double))) || (rc = dalloc(du, 3 * nodes * sizeof(double)))) {
    cudaFree(dtab); cudaFree(work); cudaFree(du);
    return rc;
  }
  cudaError_t e;
  if ((e = cudaMemcpyAsync(dtab, ctab.data(), ctab.size() * sizeof(double), cudaMemcpyHostToDevice, c->st)) ||
      (e = f2disp_device(c->Fn1, N, lx, ly, lz, dtab, work, du, c->st)) ||
      (e = cudaMemcpyAsync(u, du, 3 * nodes * sizeof(double), cudaMemcpyDeviceToHost, c->st)) ||
      (e = cudaStreamSynchronize(c->st)))
    rc = cuda_check(e, "cpfft_f2disp");
  cudaFree(dtab);
  cudaFree(work);
  cudaFree(du);
  return rc;
}

int cpfft_write_disp_flat(int step, double lx, double ly, double lz, const char* structure_name,
                          const char* directory) {
  TRY(need_ctx());
  Ctx* c = g_ctx;
  const long long N1 = c->N + 1, nodes = N1 * N1 * N1;
  std::vector<double> u(3 * nodes);
  TRY(cpfft_f2disp(lx, ly, lz, u.data()));
  for (double& x : u)
    if (std::fabs(x) < 1.0e-30) x = 0.0;  // oudisp's small_tol (src/ouresult.f:71,107)
  std::vector<char> fields(15 * 3 * nodes);
  TRY(cpfft_format_e15(u.data(), 3 * nodes, fields.data()));
  // wnd + step (i5.5) + _text (ouocdd, src/ouresult.f:419-540); header of
  // ouddpa_flat_header with type 1, quantity 1 (src/ouresult.f:335-396)
  int stepno = step > 99999 ? step - 99999 : step;
  char name[64];
  snprintf(name, sizeof(name), "wnd%05d_text", stepno);
  std::string path = directory && directory[0] ? std::string(directory) + "/" + name : name;
  FILE* f = fopen(path.c_str(), "w");
  if (!f) {
    cpfft_set_error("cpfft_write_disp_flat: cannot open %s", path.c_str());
    return CPFFT_ERR_BAD_ARG;
  }
  char sname[9];
  snprintf(sname, sizeof(sname), "%-8.8s", structure_name ? structure_name : "");
  time_t now = time(nullptr);
  char date[32];
  strftime(date, sizeof(date), "%a %b %e %H:%M:%S %Y", localtime(&now));
  fprintf(f, "#\n#  WARP3D nodal results: %-15s\n#  Structure name: %s\n"
             "#  Model nodes, elements: %8lld%8lld\n#  %-24s\n#  Load(time) step: %8d\n#\n",
          "displacements", sname, nodes, c->N3, date, step);
  bool ok = true;
  for (long long n = 0; n < nodes && ok; n++) {  // format (3e15.6), one node a line
    ok = fwrite(fields.data() + 45 * n, 1, 45, f) == 45 && fputc('\n', f) != EOF;
  }
  fclose(f);
  if (!ok) {
    cpfft_set_error("cpfft_write_disp_flat: short write to %s", path.c_str());
    return CPFFT_ERR_BAD_ARG;
  }
  return 0;
}

// ouresult (src/ouresult.f:12-42, called from src/FFT_nr3.f:183): the nodal displacement
// file, then the element strain and stress files of the step (oustates writes nothing)
int cpfft_ouresult(int step, double lx, double ly, double lz, const char* structure_name,
                   const char* directory) {
  TRY(cpfft_write_disp_flat(step, lx, ly, lz, structure_name, directory));
  TRY(cpfft_write_flat(1, step, structure_name, directory));
  TRY(cpfft_write_flat(2, step, structure_name, directory));
  return 0;
}

}  // extern "C"
