/*
 * cpfft_oracle.h -- CPU restatement of the CPFFT hot path.  TEST INFRASTRUCTURE ONLY:
 * used by tests/, by __graft_entry__.smoke() and by bench.py's CPU baseline as the
 * checker and the timed CPU stand-in.  Nothing in the product links it.
 *
 * Parity unpinned: the reference ships no tests or golden outputs, and it cannot be
 * built here (Fortran + Intel MKL only, src/makefile:9-25).  The oracle is pinned to
 * analytic known answers instead (see tests/).
 */
#ifndef CPFFT_ORACLE_H
#define CPFFT_ORACLE_H
#include "../include/cpfft_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_ctx orc_ctx;

/* Per-voxel compact state, same words and order as CPFFT_HIST_WORDS; grids of
 * Ma-Roters-Raabe crystals (h_type 7) carry ORC_HIST_MRR words (CPFFT_HIST_WORDS_MRR). */
#define ORC_HIST 31
#define ORC_HIST_MRR 55

orc_ctx* orc_create(int N, const int* matList, const double* kocks_deg,
                    const cpfft_crystal* props, int ncrystals, double tstep,
                    int g_mapping, int nthreads);
void     orc_destroy(orc_ctx* c);

/* make a material declared with slip_type CPFFT_NOT_A_CRYSTAL an mm01 bilinear Mises
 * material (resets its voxels' state) */
void orc_set_mises(orc_ctx* c, int material, const cpfft_mises* props);

/* make a material declared with slip_type CPFFT_NOT_A_CRYSTAL the FFT program's original
 * St-Venant-Kirchhoff material (constitutive, src/mm00.f:13-60) of bulk modulus K and shear
 * modulus mu: a known-answer material for the global loop (not a product model) */
void orc_set_svk(orc_ctx* c, int material, double K, double mu);
/* P and dP/dF (row-major, (ij)(kl)) of that material at F (row-major) */
void orc_svk_point(double K, double mu, const double F[9], double P[9], double A[81]);

/* drive_eps_sig on every voxel; Fn/Fn1 NULL -> use the context's fields.
 * Pn1/K4 NULL -> keep in the context.  Returns number of local failures. */
int orc_stress_update(orc_ctx* c, int step, int iter, const double* Fn,
                      const double* Fn1, double* Pn1, double* K4,
                      long long* local_iters);
/* the same on voxels [v0, v1) only (bounded CPU-baseline samples) */
int orc_stress_sample(orc_ctx* c, int step, int iter, long v0, long v1);
/* update(): history n <- n+1, Fn <- Fn1, Pn <- Pn1 */
void orc_commit(orc_ctx* c);

/* G_K_dF with the context's K4 (or K4 given, may be NULL). */
void orc_green_apply(orc_ctx* c, const double* x, double* y, int flgK,
                     const double* K4);
/* fftPcg; returns 0 / CPFFT_ERR_*; *iters = iterations */
int  orc_cg(orc_ctx* c, const double* b, double* x, double tol, int* iters);
/* tangent_homo */
int  orc_tangent_homo(orc_ctx* c, double tolPCG, double* C_homo);
/* FFT_nr3 start (drive_eps_sig(1,0) + tangent_homo) */
int  orc_nr3_begin(orc_ctx* c, double tolPCG);
/* the library's equilibrium stop test of the Newton loop (cpfft_set_equilibrium_tol) */
void orc_set_equilibrium_tol(orc_ctx* c, double tol);
/* the library's P_bar update inside the Newton iteration (cpfft_set_coupled_bc: 0 off,
 * 1 on, 2 on with an implicit first stress pass) */
void orc_set_coupled_bc(orc_ctx* c, int on);
/* one load step of FFT_nr3 */
int  orc_nr3_step(orc_ctx* c, int step, const double* BC, const int* isNBC,
                  double tolNR, double tolPCG, int maxIter, double* Pbar,
                  cpfft_stats* st);

/* access to fields (N3,9) / (N3,81) / history (N3, ORC_HIST) */
void orc_get_fields(orc_ctx* c, double* Fn, double* Fn1, double* Pn, double* Pn1,
                    double* K4);
void orc_set_fields(orc_ctx* c, const double* Fn, const double* Fn1);
int  orc_hist_words(orc_ctx* c);   /* ORC_HIST or ORC_HIST_MRR */
void orc_get_history(orc_ctx* c, double* hist_n, double* hist_np1);
void orc_set_history_n(orc_ctx* c, const double* hist_n);

/* ---- single-voxel entry points used by the unit tests ---------------------------- */
/* Full material-point update of one voxel (kinematics + mm10 + cep2A).
 * hist_n (ORC_HIST words, ORC_HIST_MRR for h_type 7) is read unless step == 1 (then
 * initialised); hist_np1 written.
 * out_sig6 = unrotated Cauchy stress, out_cep36 = 6x6 tangent (row-major).
 * Returns local Newton iterations (update phase), or -1 on failure. */
int orc_voxel_update(const cpfft_crystal* props, const double kocks_deg[3],
                     double tstep, int step, int iter, const double Fn[9],
                     const double Fn1[9], const double* hist_n, double* hist_np1,
                     double P[9], double A[81], double out_sig6[6],
                     double out_cep36[36]);
/* The same for an mm01 voxel (kinematics + mm01 + cnst1 + cep2A); hist_n NULL or
 * step 1: mm01_set_history's state. */
int orc_mises_update(const cpfft_mises* props, int step, const double Fn[9],
                     const double Fn1[9], const double* hist_n, double* hist_np1,
                     double P[9], double A[81], double out_sig6[6], double out_cep36[36]);
/* Ma-Roters-Raabe interaction matrices of a 12-system slip type (1 fcc, 2 bcc, 6 roters,
 * 7 bcc12; row-major 12 x 12): rho_F = G rho, rho_P = H rho */
void orc_mrr_interaction(int slip_type, double G[144], double H[144]);
/* Ma-Roters-Raabe local residual R (18) and Jacobian J (18 x 18, row-major) at
 * x = (sigma 6, densities 12) for the strain increment D over tinc at 297 K, the current
 * rotation the identity; hist_n NULL: the initial state.  Returns -1 unless h_type 7. */
int orc_mrr_residual(const cpfft_crystal* props, const double kocks_deg[3], const double D[6],
                     double tinc, const double* hist_n, const double x[18], double R[18],
                     double J[324]);
/* polar decomposition F = R U (rtcmp1), F and R row-major 3x3 */
void orc_polar(const double F[9], double R[9]);
/* crystal stiffness in the sample frame (row-major 6x6) and slip tensors (12x6) */
void orc_crystal_setup(const cpfft_crystal* props, const double kocks_deg[3],
                       double C66[36], double* ms /*nslip x 6*/, double* qs /*nslip x 3*/);
/* 3-D complex DFT of an N^3 array (split re/im), sign -1 forward, +1 backward
 * (backward scaled by 1/N^3), first index fastest. */
void orc_fft3(int N, double* re, double* im, int sign);

#ifdef __cplusplus
}
#endif
#endif
