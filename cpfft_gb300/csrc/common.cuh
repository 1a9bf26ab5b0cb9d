// common.cuh -- shared device/host helpers of the GB300 CPFFT hot path.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "../../include/cpfft_gpu.h"

#define CPFFT_CUDA_TRY(expr)                                                       \
  do {                                                                             \
    cudaError_t _e = (expr);                                                       \
    if (_e != cudaSuccess) {                                                       \
      cpfft_set_error("%s:%d %s: %s", __FILE__, __LINE__, #expr,                   \
                      cudaGetErrorString(_e));                                     \
      return CPFFT_ERR_CUDA;                                                       \
    }                                                                              \
  } while (0)

void cpfft_set_error(const char* fmt, ...);

// Raise a kernel's maximum dynamic shared memory to at least `bytes` (never lowers it;
// thread-safe), for kernels whose launches need different sizes per grid.
cudaError_t raise_max_dynamic_smem(const void* func, size_t bytes);

// Kernels launched by the calling host thread through this library (each thread drives
// its own context); every launch wrapper adds its launches here.
extern thread_local long long g_kernel_launches;

// ---- per-orientation material data (computed once at init, see api.cu) ------------
// One record per distinct (crystal, orientation): the rotated stiffness and the slip
// tensors of setup_mm10_rknstr (src/drive_eps_sig.f:537-1002), which the reference
// recomputes on every call for every voxel.
struct OriRec {
  double C[36];    // stiffness in the sample frame, row-major 6x6
  double ms[48 * 6];  // nslip x 6 sym(b (x) n) Voigt, engineering shear
  double qs[48 * 3];  // nslip x 3 skew(b (x) n) as (w23, w13, w12)
  double g[9];     // lattice -> sample rotation applied to b and n, row-major
};

// Scalars of one crystal definition that the Voce path reads.
struct CrysRec {
  double rate_n, tau_y, tau_v, inv_tau_v, theta_0, voce_m, gamma_bar, iD_v;
  double atol, atol1, rtol, rtol1;
  // MTS (h_type 2)
  double tau_a, tau_hat_y, G_0_y, p_y, q_y, tau_hat_v, G_0_v, p_v, q_v, eps_dot_0_v;
  double burgers, boltzman, mu_0, D_0, T_0;
  // Ma-Roters-Raabe (h_type 7): c1..c6 and the interaction matrices (row-major 12 x 12),
  // rho_F = Gm rho, rho_P = Hm rho
  double u1, u2, u3, u4, u5, u6;
  double Gm[144], Hm[144];
  int h_type;
  int miter, alter_mode, exact_j22;
  int n_int;       // rate_n - 1 when rate_n is integer-valued in [2, 64], else -1
  int m_is_one;    // voce_m == 1
};

// One bilinear Mises material (mm01, src/mm01.f; properties of setup_mm01_rknstr,
// src/drive_eps_sig.f:486-520): e, nu, uniaxial yield stress, plastic modulus
// h = tan_e e / (e - tan_e) and the isotropic fraction beta of the hardening.
struct MisesRec {
  double e, nu, yld, h, beta;
};

// Words of the compact per-voxel history (CPFFT_HIST_WORDS)
enum {
  H_SIG = 0,      // 6  unrotated Cauchy stress
  H_TT = 6,       // 1  slip resistance tau_tilde
  H_RP = 7,       // 9  plastic rotation Rp, column-major
  H_D = 16,       // 6  unrotated strain increment of the step
  H_TTR = 22,     // 1  tau_tilde rate
  H_EPS = 23,     // 6  unrotated strain (sum of the step increments, rstgp1_update_strains)
  H_U = 29,       // 2  MTS: tau_y and mu of the step (mm10's u(1:2)); -1 = not yet set
  H_WORDS = 31,
  // grids of Ma-Roters-Raabe crystals (CPFFT_HIST_WORDS_MRR): the twelve dislocation
  // densities, then their rates; H_TT and H_TTR are zero there
  H_RHO = 31,     // 12 + 12
  H_WORDS_MRR = 55
};

// The same words for an mm01 voxel: H_SIG and H_EPS as above, and in words 6..19 the
// mm01 history vector (mm01_set_history, src/mm01.f:240-310) followed by the three extra
// stress-vector words of oupestr's cgn(7:9) (src/mm01.f:95-100)
enum {
  M1_LDT = 6,     // 1  lambda * dt of the step (plastic multiplier)
  M1_K = 7,       // 1  radius k of the yield surface (shear yield stress)
  M1_EPSP = 8,    // 1  accumulated uniaxial plastic strain
  M1_STATE = 9,   // 1  1 = actively yielding, 3 = not
  M1_HP = 10,     // 1  plastic modulus at n+1
  M1_ALPHA = 11,  // 6  back stress
  M1_U = 17,      // 1  strain energy density
  M1_WP = 18,     // 1  plastic work density
  M1_EBP = 19     // 1  accumulated equivalent plastic strain (of the plastic work update)
};

// Stress kernel launch arguments
struct StressArgs {
  const double* Fn;      // (9, N3)
  const double* Fn1;     // (9, N3)
  const double* hist_n;  // (H_WORDS, N3)
  double* hist_np1;      // (H_WORDS, N3): written; read as the previous iterate's local state
  double* P;             // (9, N3)
  double* K4;            // (81, N3)
  float* K4f;            // (81, N3) optional FP32 copy (mixed precision), may be null
  float* K4lo;           // (81, N3) optional FP32 remainder K4 - K4f (double-float operator)
  const int* ori;        // (N3) orientation record id
  const int* crys;       // (N3) crystal id, 0-based
  const OriRec* oris;
  const CrysRec* cryss;
  // mm01 voxels: mises[v] = index into misess, -1 for a crystal voxel (null: none)
  const int* mises;
  const MisesRec* misess;
  unsigned long long* stats;  // [0] local iters, [1] failures, [2] predict iters,
                              // [3] learned guesses the Newton solve rejected
  long long N3;
  double dt;
  int step, iter;
  // learned initial guess (mlp.cuh): BF16 operand copies, FP32 parameters, normalisation
  const void* mlp_packed;
  const float* mlp_params;
  const float* mlp_norm;
  int* mlp_err;               // set when a tensor-core wait gave up
  // start of the local solves (fast modes), each in place of the reference's predictor:
  // start_iterate = 1: the coupled Newton starts from the state left in hist_np1 by the
  // previous global iteration of this step; start_trial = 1: from the elastic trial
  // returned inside the rate surface; warm launches: from the learned guess returned
  // inside the surface.  start_cap bounds the iterations from such a start before the
  // plain solve takes over.
  int start_iterate;
  int start_trial;
  int start_cap;
  // voxel work queue (null perm: one block per 128 consecutive voxels)
  const int* perm;            // (N3) voxel ids, heaviest previous-pass cost first
  unsigned int* queue;        // next queue slot (zeroed by launch_voxel_queue)
  unsigned char* cost;        // (N3) out: local iterations of this pass (null: not kept)
  int qchunk;                 // voxels a block takes from the queue at a time (multiple of 128)
  int qbps;                   // persistent blocks per SM (0: as many as fit)
  int tangent_f32;            // 1: dP/dF (cep2A) in FP32 (the fast form; it steers Newton only)
  // logging of (features, converged increments) pairs from the plain solve
  float* log_X;               // [cap][20], null: no logging
  float* log_T;               // [cap][7]
  unsigned long long* log_n;  // pairs written (may exceed cap: extra pairs are dropped)
  long long log_cap;
  int log_stride, log_phase;  // voxels v with v % stride == phase are logged
};

// warm = true: the learned initial guess starts the local Newton solve.  launch_stress
// serves crystals with 12 slip systems, launch_stress48 those with 48 (BCC48).
cudaError_t launch_stress(const StressArgs& a, bool warm, cudaStream_t s);
cudaError_t launch_stress48(const StressArgs& a, bool warm, cudaStream_t s);
// the 6-system (hcp6, hcp18) and 1-system (single) crystals (stress6.cu, stress1.cu)
cudaError_t launch_stress6(const StressArgs& a, bool warm, cudaStream_t s);
cudaError_t launch_stress1(const StressArgs& a, bool warm, cudaStream_t s);
// MTS-hardened 12-system crystals (stress_mts.cu)
cudaError_t launch_stress_mts(const StressArgs& a, bool warm, cudaStream_t s);
// Ma-Roters-Raabe / ORNL 12-system crystals (stress_mrr.cu / stress_ornl.cu; warm is ignored: no
// learned guess)
cudaError_t launch_stress_mrr(const StressArgs& a, bool warm, cudaStream_t s);
cudaError_t launch_stress_ornl(const StressArgs& a, bool warm, cudaStream_t s);
// the mm01 voxels (a.mises[v] >= 0) of the grid; the crystal launches skip them
cudaError_t launch_mises(const StressArgs& a, cudaStream_t s);
// Build the voxel work queue from the per-voxel costs: perm = voxel ids by descending cost
// bin, queue head zeroed.  scratch: 128 unsigned ints.
cudaError_t launch_voxel_queue(const unsigned char* cost, long long N3, unsigned int* scratch,
                               int* perm, unsigned int* queue, cudaStream_t s);
