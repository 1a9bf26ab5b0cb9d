/*
 * cpfft_gpu.h -- C-ABI of the GB300 finite-strain FFT crystal-plasticity hot path.
 *
 * This is the drop-in boundary for the Fortran driver of CPFFT (maranGit/CPFFT).  The
 * host keeps its .in parser, material/crystal blocks and result writers; the bodies of
 * the routines listed below become thin ISO_C_BINDING calls into this library.  All
 * arguments are plain pointers and sizes; fields use the reference's column-major
 * layouts:
 *   - a 9-component field is (N3, 9), component order 11,12,13,21,22,23,31,32,33
 *     (src/drive_eps_sig.f:205-226), voxel index v = a + N*b + N*N*c with `a` the
 *     fastest memory axis (src/FFT_init.f:310-318);
 *   - a 4th-order field is (N3, 81), column (ij)(kl) = 9*(3*(i-1)+j-1) + 3*(k-1)+l
 *     (src/G_K_dF.f:258-264, src/cep2A.f:133-154).
 * Everything is FP64 at the boundary.
 *
 * Threading: a context (one RVE, one CUDA stream; the reference keeps this state in module
 * arrays, src/mod_fft.f) belongs to the host thread that called cpfft_init, and every
 * call acts on the calling thread's context; cpfft_batch_solve runs several contexts at
 * once from its own threads.  Calls on one context are not re-entrant.
 *
 * Return codes: 0 = success, > 0 = warning, < 0 = error (see CPFFT_* below).  The
 * reference aborts (`die_abort`, src/mpi_code.f:35-53) on every error; a Fortran caller
 * maps negative codes to `die_abort` to keep that behaviour.
 */
#ifndef CPFFT_GPU_H
#define CPFFT_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define CPFFT_OK                     0
#define CPFFT_WARN_LOCAL_FALLBACK    1   /* >= 1 voxel's local mm10 solve failed        */
#define CPFFT_ERR_CG_MAXIT          -1   /* fftPcg hit maxIter (src/FFT_nr3.f:335-339)   */
#define CPFFT_ERR_NEWTON_MAXIT      -2   /* Newton loop (src/FFT_nr3.f:116-119)          */
#define CPFFT_ERR_NBC_MAXIT         -3   /* P_bar loop (src/FFT_nr3.f:153-156)           */
#define CPFFT_ERR_NBC_SINGULAR      -4   /* dgesv info /= 0 (src/FFT_nr3.f:417-421)      */
#define CPFFT_ERR_BAD_ARG           -5
#define CPFFT_ERR_CUDA              -6
#define CPFFT_ERR_NOT_INIT          -7
#define CPFFT_ERR_CG_TOL            -8   /* improper CG tolerance (src/FFT_nr3.f:248-251)*/
#define CPFFT_ERR_NO_MEMORY         -9
#define CPFFT_ERR_NONFINITE        -10   /* NaN/Inf reached a global residual            */

/* Green-operator frequency mapping (src/FFT_init.f:146-147, 310-318, 354-385). */
#define CPFFT_G_REF_SHIFT  0   /* bit-faithful to the reference: q = ((k-Nhalf) mod N)+1-Nhalf */
#define CPFFT_G_CENTERED   1   /* signed wavenumber (identical to REF_SHIFT for odd N)         */

/* Krylov / Green precision: plain FP64, or FP32 inner iterations under an FP64 residual. */
#define CPFFT_PREC_FP64    0   /* plain: every operator in FP64                                */
#define CPFFT_PREC_MIXED   1   /* FP32 Green/FFT/CG inner iterations, FP64 outer refinement    */

/*
 * One crystal definition: the fields of the reference's `crystal` block that the
 * crystal path reads (src/mod_crystals.f:231-410 defaults, 1796-1880 elasticity;
 * keyword parser src/incrystal.f).  Units are the deck's (MPa, s).
 */
typedef struct cpfft_crystal {
    int    slip_type;      /* 12 systems: 1 = fcc {111}<110>, 2 = bcc {110}<111>,
                              6 = roters ({111}<110> in Roters' order), 7 = bcc12 ({110}<111>,
                              bcc48's first twelve); with Voce only: 8 = bcc48 {110},{112},
                              {123}<111> (48 systems), 3 = single (one system), 9 = hcp6
                              (basal and prismatic <a>), 10 = hcp18 (the reference assigns
                              hcp6's six systems and leaves twelve zero vectors, which never
                              slip: run as hcp6) (src/mod_crystals.f:438-1759); the crystals
                              of one grid share the slip type; CPFFT_NOT_A_CRYSTAL (0):
                              another material model (cpfft_set_mises)                       */
    int    elastic_type;   /* 1 isotropic (e,nu), 2 cubic (e,nu,mu), 3 anisotropic (Cij)  */
    double e, nu, mu;
    double C11, C12, C13, C33, C44, C55;
    int    h_type;         /* 1 = voce, 2 = mts, 7 = roters (Ma-Roters-Raabe dislocation
                              densities, one per slip system), 4 = ornl (the same densities,
                              ORNL's slip law); mts, roters and ornl with the 12-system slip
                              types; the crystals of one grid share the hardening law      */
    double harden_n;       /* rate exponent                                               */
    double tau_y, tau_v, theta_0, voce_m;
    double gamma_bar;      /* eps_dot_0_y                                                 */
    double iD_v;           /* diffusion slip term                                         */
    int    alter_mode;     /* 1: dg = gamma_bar * dt (src/mm10_a.f:2075-2076)             */
    double atol, atol1, rtol, rtol1;   /* local Newton tolerances                          */
    int    miter;          /* local Newton iteration cap                                  */
    int    exact_j22;      /* 0: the reference's d(R2)/d(tau_tilde) (src/mm10_b.f:1942-1968),
                              which carries an extra sign(1,slip increment) factor and so
                              converges only linearly once slip reverses on any system;
                              1: the exact derivative (no such factor). Not a deck keyword. */
    /* MTS hardening (h_type 2: mm10_h_mts .. mm10_dgdd_mts, src/mm10_b.f:2080-2380; setup
       and initial state mm10_setup_mts / mm10_init_mts, src/mm10_a.f:2090-2173), at the
       297 K of the reference's FFT path (src/rstgp1.f:832).  Not read by Voce.           */
    double tau_a;                       /* athermal slip resistance                       */
    double tau_hat_y, G_0_y, p_y, q_y;  /* thermal barrier of the yield part              */
    double tau_hat_v, G_0_v, p_v, q_v;  /* thermal barrier of the saturation part         */
    double eps_dot_0_v;                 /* reference rate of the saturation part (the yield
                                           part's is gamma_bar, eps_dot_0_y)               */
    double burgers, boltzman;
    double mu_0, D_0, T_0;              /* mu(T) = mu_0 - D_0 / (exp(T_0 / T) - 1)       */
    /* Ma-Roters-Raabe hardening (h_type 7: mm10_slipinc_mrr .. mm10_dgdd_mrr,
       src/mm10_b.f:2343-3325; initial densities mm10_init_mrr, src/mm10_a.f:2205-2223):
       twelve dislocation densities, the slip resistance variables of the twelve systems.
       It reads tau_a (Q_bulk), G_0_v (Q_slip), G_0_y (attack frequency), p_v, q_v,
       tau_hat_y (c7), tau_hat_v (c8), burgers, boltzman, mu_0 (shear modulus),
       theta_0 (initial density; 0 gives 1e8) and c1..c6 below.  exact_j22 = 1 takes
       the exact derivatives of the residual in the local Jacobian (the reference's use
       sqrt(rho_F) where the residual has sqrt(rho_P), src/mm10_b.f:2635 against :2952
       and :3075).                                                                    */
    /* ORNL hardening (h_type 4: mm10_slipinc_ornl .. mm10_dgdd_ornl,
       src/mm10_b.f:3330-4370): MRR's hardening law with mu(T) = mu_0 - D_0 /
       (exp(T_0 / T) - 1); slip rate 0.1 rho_a v_s (c2 b) exp(-Q_slip / kT
       (1 - fract^p)^q) with v_s = G_0_y (exp(-G_0_y) when negative), the cutting stress
       c3 mu(T) / mu_0 and p = 1 below the passing stress.                          */
    double u1, u2, u3, u4, u5, u6;      /* c1 .. c6                                      */
} cpfft_crystal;

/* slip_type of a material that is not a crystal: its cpfft_crystal entry is not read, and
 * cpfft_set_mises defines it before the first stress update. */
#define CPFFT_NOT_A_CRYSTAL 0

/*
 * One bilinear Mises material: the `properties bilinear` keywords the mm01 path reads
 * (src/inmat.f:96-126 into matprp(1:5), read by setup_mm01_rknstr,
 * src/drive_eps_sig.f:486-520).  The reference stores them in single precision (matprp is
 * `real`, src/mod_fft.f:20): pass those values widened to double for the same numbers.
 */
typedef struct cpfft_mises {
    double e;        /* Young's modulus (matprp 1, default 30000)                      */
    double nu;       /* Poisson's ratio (matprp 2, default 0.3)                        */
    double yld_pt;   /* uniaxial yield stress (matprp 5)                               */
    double tan_e;    /* tangent modulus of the bilinear curve (matprp 4)               */
    double beta;     /* isotropic fraction of the hardening, 1 = isotropic (matprp 3,
                        default 1)                                                     */
} cpfft_mises;

/* Per load-step statistics (mirrors the thyme buckets of src/thyme.f:15-47). */
typedef struct cpfft_stats {
    int       newton_iters;     /* global Newton iterations, summed over P_bar passes      */
    int       nbc_iters;        /* P_bar (natural BC) passes                               */
    int       cg_solves;        /* fftPcg calls                                            */
    int       cg_iters;         /* total CG iterations                                     */
    int       stress_updates;   /* full-grid drive_eps_sig passes                          */
    int       local_fallbacks;  /* voxel updates whose local solve failed                  */
    long long local_iters;      /* sum over voxel updates of local Newton iterations       */
    double    res_fft;          /* last ||dF|| / ||F|| (src/FFT_nr3.f:114)                 */
    double    res_pbar;         /* last relative P_bar residual (src/FFT_nr3.f:143-147)    */
    double    res_equil;        /* ||G(P)|| / (sqrt(N3) * ||P_bar||) after the step        */
    double    t_pcg;            /* seconds in CG (bucket 1)                                */
    double    t_sigeps;         /* seconds in stress updates (bucket 2)                    */
    double    t_total;          /* seconds in the whole call (host clock)                  */
    double    t_device;         /* seconds between CUDA events at the call's start and end */
    double    t_stress_kernel;  /* summed CUDA-event time of the stress-update kernel      */
    double    t_green64;        /* summed CUDA-event time of FP64-accurate Green applies   */
    double    t_green32;        /* summed CUDA-event time of the timed FP32 Green applies  */
    long long n_green64;        /* FP64-accurate Green applies (FP64 or double-float)      */
    long long n_green32;        /* FP32 Green applies                                      */
    long long kernel_launches;  /* kernels this call launched                              */
    long long predict_iters;    /* local predictor (6x6) Newton iterations, summed         */
    long long guess_rejected;   /* learned initial guesses the Newton solve dropped        */
    double    t_cg_graph;       /* CUDA-event time of the graph-launched CG iterations     */
    long long n_green32_timed;  /* FP32 Green applies timed one by one (t_green32 covers
                                   these; the others run inside the iteration graph)       */
} cpfft_stats;

/*
 * Set up the grid, the material point data and the device state.
 * Replaces FFT_init (src/FFT_init.f:16-177: Ghat4/coeffs tables are not stored, the
 * Green operator is evaluated from q on the fly), fftAllocate(1/3) (:191-234) and the
 * per-call orientation setup of setup_mm10_rknstr (src/drive_eps_sig.f:537-1002),
 * which is done once here.
 *   N          grid points per axis (N3 = N^3 voxels)
 *   matList    (N3) 1-based crystal number per voxel (src/mod_fft.f:550)
 *   kocks_deg  (N3, 3) column-major Kocks angles in degrees (psi, theta, phi)
 *   props      (ncrystals) crystal definitions
 *   tstep      time step of every load step (src/indypm.f: "time step")
 *   g_mapping  CPFFT_G_REF_SHIFT or CPFFT_G_CENTERED
 * Fn = Fn1 = I, Pn = Pn1 = 0 afterwards (src/FFT_init.f:157-161).
 */
int cpfft_init(int N, const int* matList, const double* kocks_deg,
               const cpfft_crystal* props, int ncrystals, double tstep, int g_mapping);

/* Make `material` (1-based, a matList value whose cpfft_init entry has slip_type
 * CPFFT_NOT_A_CRYSTAL) an mm01 bilinear Mises material (src/mm01.f, model 1 of
 * rknstr_set_up_materials, src/drive_eps_sig.f:355-420): its voxels are updated by mm01
 * and its consistent tangent cnst1, then the same P and dP/dF pull-back as the crystals.
 * Resets those voxels' state to mm01_set_history's.  Call before the first load step;
 * stress updates fail with CPFFT_ERR_NOT_INIT while a declared material is undefined. */
int cpfft_set_mises(int material, const cpfft_mises* props);

/* Select the Krylov precision (CPFFT_PREC_*) and the start of the local mm10 solves
 * (warm_start: 0 = the reference's predictor from sigma_n, or an OR of the flags below).
 * Extensions with no counterpart in the reference.  A start replaces the predictor: the
 * coupled Newton of mm10_solve runs from it to the reference's local tolerance (its test
 * scaled by the residual of the reference's start), and a start that has not converged
 * within 8 iterations falls back to the reference's solve; only the number of local
 * iterations changes.
 *   CPFFT_START_LEARNED  the return-mapped elastic trial (below) corrected by the learned
 *                        network, returned along the segment from sigma_n to 98 % of the
 *                        rate surface (needs cpfft_mlp_init and trained parameters)
 *   CPFFT_START_ITERATE  on a stress pass that follows an implicit pass of the same
 *                        load step: that pass's converged local state (precedence over
 *                        the other two on those passes)
 *   CPFFT_START_TRIAL    the elastic trial sigma_n + C D, tau extrapolated, returned to
 *                        98 % of the rate surface (ignored with CPFFT_START_LEARNED)
 * and, with CPFFT_PREC_MIXED,
 *   CPFFT_TANGENT_F32    the consistent tangent dP/dF (cep2A) evaluated in FP32: it only
 *                        steers the global Newton iteration (stresses, local solves and
 *                        every residual stay FP64); K4 then holds the FP32 values */
#define CPFFT_START_LEARNED  1
#define CPFFT_START_ITERATE  2
#define CPFFT_START_TRIAL    4
#define CPFFT_TANGENT_F32    8
int cpfft_set_mode(int precision, int warm_start);

/* Preconditioner of the FP32 inner iterations of CPFFT_PREC_MIXED (extension; the
 * reference's fftPcg, src/FFT_nr3.f:214-360, is unpreconditioned, and so is the FP64
 * path here).  CPFFT_PRECOND_REFERENCE solves G0(K : x) = G0(b) instead of
 * G(K : x) = b, G0 the Green operator of a homogeneous reference medium K0 = the
 * symmetrised volume average of the current tangent, recomputed after every stress
 * update.  Same solutions (both equations say K : x - b' is divergence free), the same
 * FP64 residual b - G(K : x) and stop test; fewer iterations.  It applies to odd N and to
 * CPFFT_G_CENTERED (where the Green operator is a projection); elsewhere, or when the
 * averaged tangent is not strongly elliptic, the plain inner iteration runs. */
#define CPFFT_PRECOND_NONE       0
#define CPFFT_PRECOND_REFERENCE  1
int cpfft_set_precond(int precond);

/* Voxel order of the implicit stress passes (extension; the reference runs OpenMP over
 * 128-voxel blocks in order, src/drive_eps_sig.f:31-39).  CPFFT_SCHED_BLOCKS: one thread
 * block per 128 consecutive voxels.  CPFFT_SCHED_QUEUE: a persistent kernel whose blocks
 * take 128-voxel chunks from a device work queue ordered by each voxel's local iteration
 * count in its previous implicit pass, heaviest first, so the threads of a warp iterate
 * alike and the SMs finish together.  Results are identical; only the timing changes. */
#define CPFFT_SCHED_BLOCKS  0
#define CPFFT_SCHED_QUEUE   1
int cpfft_set_schedule(int schedule);
/* The work-queue shape the autotuner chose (extension): on a context's first implicit
 * CPFFT_SCHED_QUEUE pass the pass runs once per candidate -- 128, 256 or 512 voxels taken
 * from the queue by a block at a time, with as many persistent blocks per SM as fit or
 * with one -- timed with CUDA events, and the fastest is kept (identical results).
 * *voxels = the chosen chunk (0 before that pass); *blocks_per_sm = 0 (as many as fit) or
 * 1; ms (6, may be NULL) = the pass times of the candidates, chunks 128 / 256 / 512 with
 * all blocks, then with one block per SM. */
int cpfft_queue_chunk(int* voxels, int* blocks_per_sm, double* ms);

/* Tile shapes the autotuner chose for this grid when CPFFT_PREC_MIXED was first selected
 * (extension): columns per block of the transform passes along the middle axis (both
 * directions) and along the slowest axis (with the Green contraction), for the FP32
 * operator (tiles[0], tiles[1]) and the double-float operator (tiles[2], tiles[3]); a
 * negative tiles[1] means the FP32 slowest-axis pass holding each column's rows in
 * registers, with -tiles[1] columns per block; ms: the measured time per apply of each.  Zeros before the mixed form is selected or for
 * grids the register passes do not cover (N other than 32, 64, 128, 256). */
int cpfft_tuning(int* tiles, double* ms);
/* Override the autotuner's choice (same encoding as cpfft_tuning: FP32 {8,16,32},
 * {2,4,-2,-4}; double-float {16,32}, 2).  For callers that pin launch shapes, and for
 * tests of every shape. */
int cpfft_set_tiles(const int* tiles);

/*
 * Stress update of every voxel: replaces drive_eps_sig(step, iter)
 * (src/drive_eps_sig.f:16-45, do_nleps_block :57-340, rstgp1/mm10 below it).
 * Fn, Fn1 (N3,9) host arrays; writes Pn1 (N3,9) and K4 (N3,81) host arrays (either
 * may be NULL to leave the result on the device only).  Uses and advances the
 * device-resident history at n+1; the history at n changes only in cpfft_commit_step.
 * iter == 0 selects the explicit predictor with the elastic tangent
 * (src/rstgp1.f:870-877).  Returns CPFFT_WARN_LOCAL_FALLBACK if a local solve failed.
 */
int cpfft_stress_update(int step, int iter, const double* Fn, const double* Fn1,
                        double* Pn1, double* K4);

/* Counters of the last stress pass (diagnostic, no counterpart in the reference):
 * counts[0] local Newton iterations summed over the voxels, [1] voxels whose local solve
 * failed, [2] predictor iterations summed, [3] starts the solve dropped, [4] voxels whose
 * solve was sub-stepped (mm10_solve_strup's cuts, src/mm10_a.f:2765-2802). */
int cpfft_pass_counts(long long* counts);

/*
 * y = G(K4 : x) (flgK = 1) or y = G(x) (flgK = 0): replaces G_K_dF (src/G_K_dF.f:11-87).
 * K4 is the device copy written by the last cpfft_stress_update (or cpfft_set_K4).
 * x, y (N3,9) host arrays.
 */
int cpfft_green_apply(const double* x, double* y, int flgK);

/* The FP32 form of the same operator (the mixed-precision inner Krylov matvec) on FP32
 * host arrays; needs CPFFT_PREC_MIXED and, for flgK = 1, a stress update since. */
int cpfft_green_apply_f32(const float* x, float* y, int flgK);

/* The FP64-accurate operator of CPFFT_PREC_MIXED in double-float arithmetic (each value
 * a pair of floats, about 48 bits, on the FP32 pipes): the outer residuals and
 * projections of the mixed-precision CG use it where N is 32, 64, 128 or 256, in place of
 * the native FP64 G_K_dF.  x, y (N3,9) FP64 host arrays. */
int cpfft_green_apply_df(const double* x, double* y, int flgK);

/*
 * y = G(K4 : x) (flgK = 1) or y = G(x) without any device allocation.  No counterpart in
 * the reference: it is for callers that cannot call cudaMalloc (host programs that give
 * all device memory to their own pool allocator at start-up or run under a fixed
 * device-memory budget).  x, K4, y are the CALLER's device buffers ((N3,9), (N3,81),
 * (N3,9); K4 may be NULL when flgK = 0); no cpfft_init is needed.  The scratch is one
 * static device array sized for N <= 32 (2.5 MB, kept by every GPU that loads the
 * library until exit); larger N returns CPFFT_ERR_BAD_ARG.  The first call on a device
 * looks up that array's address with the device current -- make it before any stream
 * capture.  All calls share the array: calls that overlap on the GPU race.  `stream` is
 * a cudaStream_t (NULL = the legacy default stream); the call returns after enqueueing.
 */
int cpfft_green_apply_noalloc(int N, int g_mapping, const double* x, const double* K4,
                              int flgK, double* y, void* stream);

/* Upload a tangent field K4 (N3,81) from the host (for callers that own K4). */
int cpfft_set_K4(const double* K4);

/*
 * Unpreconditioned CG on G(K4 : x) = b from x = 0: replaces fftPcg
 * (src/FFT_nr3.f:214-360; MKL RCI dcg with the user stop test ||r|| <= tol*||b||
 * or ||r|| <= tol, at most 1000 iterations).  b, x (N3,9) host arrays.
 * *iters receives the iteration count.
 */
int cpfft_cg(const double* b, double* x, double tol, int* iters);

/*
 * Homogenised tangent C_homo (81, column-major (9,9)): replaces tangent_homo
 * (src/tangent_homo.f:11-73), 9 CG solves with the device K4.
 */
int cpfft_tangent_homo(double tolPCG, double* C_homo);

/*
 * One whole load step resident on the device: replaces the body of the step loop of
 * FFT_nr3 (src/FFT_nr3.f:51-185) up to and including the state roll-over
 * (Fn <- Fn1, Pn <- Pn1, update).  The homogenised tangent used by the first
 * NBC_update of the step is the one left by the previous step (or by
 * cpfft_nr3_begin for step 1), exactly as the reference keeps C_homo across steps.
 *   BC      (9) this step's column of BC_all (src/inlod.f:57-63)
 *   isNBC   (9) 1 where P is prescribed, 0 where F is prescribed
 *   Pbar    (9) out: volume-averaged P after the step
 *   st      out: statistics (may be NULL)
 */
int cpfft_nr3_step(int step, const double* BC, const int* isNBC, double tolNR,
                   double tolPCG, int maxIter, double* Pbar, cpfft_stats* st);

/*
 * Equilibrium stop test of the global Newton loop (extension; the reference stops on
 * ||dF|| / ||F|| <= tolNR alone, src/FFT_nr3.f:107-122).  With tol > 0, cpfft_nr3_step
 * ends a Newton loop only when that test holds AND the equilibrium residual of the state
 * reached, ||G(P)|| / (sqrt(N3) ||P_bar||) with G(P) evaluated by the FP64-accurate
 * operator, is <= tol; while it is not, the loop continues with further Newton iterations
 * (counted against maxIter).  The stress update that evaluates the test is the
 * reference's closing drive_eps_sig (src/FFT_nr3.f:123), so a step whose first test
 * passes costs what the reference's does.  The loop is globalised by backtracking on the
 * same residual: from the third Newton iteration on, an increment after which the
 * residual has grown is halved (at most 4 times in a row, each costing one stress update)
 * before the next Krylov solve.  Without it the reference's undamped iteration can
 * settle into a cycle (128^3 plane-strain compression, load step 2: ||dF||/||F|| stays
 * at 6.7e-6, the equilibrium residual near 6e-4).  tol = 0 (the default) restores the
 * reference's loop.  cpfft_stats.res_equil reports the value of the last test.
 */
int cpfft_set_equilibrium_tol(double tol);

/*
 * Inexact Newton (extension; the reference solves every Newton system to the CG
 * tolerance, src/FFT_nr3.f:95, 112).  With eta_max > 0 and the equilibrium test on
 * (cpfft_set_equilibrium_tol), cpfft_nr3_step solves each Newton system to the relative
 * tolerance eta_k = min(eta_max, 0.9 (e_k / e_{k-1})^2) (Eisenstat-Walker's second
 * choice with its safeguard max(eta_k, 0.9 eta_{k-1}^2) when that exceeds 0.1, and no
 * tighter than 0.5 tol / e_k), e_k the equilibrium residual of iterate k; the predictor's
 * system to eta_max and the homogenised tangent's to 1e-2 (cpfft_set_tangent_tol; it
 * only steers the P_bar update), never below tolPCG.  The loop still ends on the equilibrium test, so the
 * converged state meets the same tolerance with fewer Krylov iterations.  eta_max = 0
 * (the default) solves every system to tolPCG.
 */
int cpfft_set_inexact_newton(double eta_max);

/*
 * Relative tolerance of tangent_homo's 9 solves under inexact Newton (extension; default
 * 1e-2, never below tolPCG).  C_homo only steers the P_bar update of the mixed boundary
 * conditions (src/FFT_nr3.f:150-170), whose loop tests P_bar itself, so a looser
 * tangent can cost P_bar iterations but does not change what the step converges to
 * (128^3 plane-strain compression: the same P_bar and Newton counts from 1e-6 to 1e-2,
 * P_bar within 5e-9 of the 1e-6 solves).  Without inexact Newton the solves use tolPCG
 * as the reference does.
 */
int cpfft_set_tangent_tol(double tol);

/*
 * The P_bar update inside the Newton iteration (extension; on != 0; applies with the
 * equilibrium test and prescribed-stress components).  The reference nests a
 * Newton loop at fixed macroscopic F inside a loop of P_bar updates, each pass opening
 * with an explicit stress pass (src/FFT_nr3.f:75-171).  Here every Newton iteration also
 * updates the prescribed-stress components of F_bar with NBC_update's system and solves
 * the fluctuation for both changes, one Newton step on the coupled system (C_homo, its
 * Schur complement, recomputed after the first implicit stress pass).  The step ends
 * on the nested loops' final tests: P_bar within tolNR, the equilibrium residual within
 * its tolerance, the last increment within tolNR.  on = 2 also makes the step's first
 * stress pass implicit (the reference's iteration 0 is an explicit elastic predictor).
 * Default off.
 */
int cpfft_set_coupled_bc(int on);

/*
 * Start of FFT_nr3 (src/FFT_nr3.f:36-47): the initial drive_eps_sig(1,0) of the
 * `compute` command (src/FFT_finite_3d.f:145) and the first tangent_homo.
 */
int cpfft_nr3_begin(double tolPCG);

/*
 * Many RVEs at once (extension; the reference solves one RVE per run).  Each RVE runs the
 * whole `compute` sequence -- cpfft_init, the selected mode, cpfft_nr3_begin, nsteps x
 * cpfft_nr3_step -- in its own library context and CUDA stream, driven by one of
 * `nthreads` host threads that take RVEs from a shared queue, largest grid first; the
 * RVEs' kernels therefore run concurrently on the GPU.  Per-RVE results are identical to
 * solving the RVEs one after another.  The calling thread's own context is untouched.
 */
typedef struct cpfft_rve {
    /* in */
    int N;                        /* grid points per axis                                  */
    const int* matList;           /* (N3) as cpfft_init                                    */
    const double* kocks_deg;      /* (N3, 3)                                               */
    const cpfft_crystal* props;
    int ncrystals;
    double tstep;
    int g_mapping;
    int nsteps;
    const double* BC_all;         /* (9, nsteps): column s-1 = the BC of load step s       */
    const int* isNBC;             /* (9)                                                   */
    /* out */
    double* Pbar;                 /* (9, nsteps) volume-averaged P after each step         */
    double* Fn1;                  /* (N3, 9) final F, or NULL                              */
    double* Pn1;                  /* (N3, 9) final P, or NULL                              */
    int status;                   /* first error, else the largest warning, else 0         */
    int steps_done;
    long long voxel_updates;      /* N3 x stress-update passes                             */
    long long cg_iters;
    double seconds;               /* host wall time of this RVE                            */
    char error[160];              /* cpfft_last_error() of the failing call                */
    /* in, optional */
    const cpfft_mises* mises;     /* (ncrystals) or NULL: entry m defines material m+1 as a
                                     bilinear Mises material when props[m].slip_type is
                                     CPFFT_NOT_A_CRYSTAL (cpfft_set_mises)                 */
} cpfft_rve;

/* precision / options / precond / schedule as cpfft_set_mode, cpfft_set_precond and
 * cpfft_set_schedule (precond and schedule apply to CPFFT_PREC_MIXED); tolerances as
 * cpfft_nr3_step.  Returns 0, or the first RVE error in queue order. */
int cpfft_batch_solve(cpfft_rve* rves, int nrve, int precision, int options, int precond,
                      int schedule, double tolNR, double tolPCG, int maxIter, int nthreads);

/* The Newton options of the fast form for every RVE of a batch (extension). */
typedef struct cpfft_newton {
    double equilibrium_tol;       /* cpfft_set_equilibrium_tol; 0: the reference's loop    */
    double eta_max;               /* cpfft_set_inexact_newton; 0: every system to tolPCG   */
    double tangent_tol;           /* cpfft_set_tangent_tol; 0 keeps its default (1e-2)     */
    int coupled_bc;               /* cpfft_set_coupled_bc: 0, 1 or 2                       */
} cpfft_newton;

/* cpfft_batch_solve with `newton` applied in each RVE's context after its mode
 * (newton == NULL: cpfft_batch_solve).  Options out of their setters' ranges return
 * CPFFT_ERR_BAD_ARG before any RVE starts. */
int cpfft_batch_solve_newton(cpfft_rve* rves, int nrve, int precision, int options,
                             int precond, int schedule, const cpfft_newton* newton,
                             double tolNR, double tolPCG, int maxIter, int nthreads);

/* Copy device fields to the host (any pointer may be NULL): Fn1, Pn1 (N3,9) and the
 * compact history at n (N3, cpfft_hist_words()) used by the result writers. */
#define CPFFT_HIST_WORDS 31   /* sigma(6) tau_tilde(1) Rp(9) D(6) tau_tilde_rate(1) eps(6)
                                 u(2): MTS tau_y and mu at the step's end (mm10's u(1:2)) */
#define CPFFT_HIST_WORDS_MRR 55  /* grids of dislocation-density crystals (h_type 7, 4): the words
                                    above (tau_tilde, its rate and u zero), then the twelve
                                    dislocation densities (mm10's tau_tilde(1:12)) and their
                                    rates (tt_rate(1:12))                                  */
int cpfft_sync_to_host(double* Fn1, double* Pn1, double* history);
/* Words per voxel of the current context's history: CPFFT_HIST_WORDS, or
 * CPFFT_HIST_WORDS_MRR on a grid of Ma-Roters-Raabe crystals; negative on error. */
int cpfft_hist_words(void);
/* The slip systems the stress kernels use for a slip_type (host only, no context):
 * returns their number (1, 6, 12 or 48; hcp18 gives hcp6's six, its other twelve being
 * zero vectors in the reference) and fills the unit directions b and plane normals n
 * (systems x 3, row-major, crystal frame) when not NULL; CPFFT_ERR_BAD_ARG for a type
 * without a table. */
int cpfft_slip_systems(int slip_type, double* b, double* n);

/* ---- element result files (ouelestr, src/ouresult.f:140-300) --------------------------
 * The per-voxel lines of the flat text files wesNNNNN_text (quantity 2: the unrotated
 * Cauchy stress, 26 values a line) and weeNNNNN_text (quantity 1: the unrotated strain,
 * 22 values a line), from the history after the last roll-over (where ouresult is
 * called, src/FFT_nr3.f:173-183).  Every value is written as the Fortran E15.6 of
 * oupestr's `(30e15.6)`, rounded to nearest (ties to even), values below 1e-30 as zero,
 * the columns past the six components zero as in the reference; formatted on the GPU.
 * cpfft_format_flat fills `text` (capacity >= *length = N3 x (values x 15 + 1) bytes; with
 * text NULL it only reports the size).  cpfft_write_flat writes the whole file, header
 * included (ouddpa_flat_header: structure name, node and element counts, date, step),
 * named as ouocst_elem names it, into `directory` (NULL or "" = the working directory). */
int cpfft_format_flat(int quantity, char* text, long long capacity, long long* length);
int cpfft_write_flat(int quantity, int step, const char* structure_name, const char* directory);
/* E15.6 of n values (15 characters each, no separators) into out: the formatter above. */
int cpfft_format_e15(const double* x, long long n, char* out);

/* Nodal displacements of the current F field: replaces f2disp (src/f2disp.f:16-135) with
 * form_BTB and its PARDISO solve.  The mesh is blkgen's (N+1)^3 nodes over the box lx x
 * ly x lz (`sizes of x_direction ..`, src/oumodel.f:178-330), node n = i + (N+1) j +
 * (N+1)^2 k, i along x; u (3 (N+1)^3) is the reference's u array: u[3 n + r], node 1 held
 * at the origin.  The same least-squares system (B^T B with 2x2x2 Gauss points, B^T F with
 * one point) is solved exactly by separable DCT-I transforms on the GPU: on the regular grid
 * the operator is a tensor product of 1-D linear-element stiffness and mass matrices. */
int cpfft_f2disp(double lx, double ly, double lz, double* u);
/* The nodal displacement file wndNNNNN_text of oudisp (src/ouresult.f:56-128): header,
 * then one line of (3e15.6) per node, values below 1e-30 as zero, formatted on the GPU. */
int cpfft_write_disp_flat(int step, double lx, double ly, double lz, const char* structure_name,
                          const char* directory);
/* ouresult(step) (src/ouresult.f:12-42; called from src/FFT_nr3.f:183 on output steps): the
 * three flat text files of the step -- wndNNNNN_text, weeNNNNN_text, wesNNNNN_text -- from
 * the device state of the committed step: after cpfft_nr3_step, which ends with the
 * update, or after cpfft_commit_step in mirror mode. */
int cpfft_ouresult(int step, double lx, double ly, double lz, const char* structure_name,
                   const char* directory);

/* State roll-over Fn <- Fn1, Pn <- Pn1, history n <- n+1: replaces update
 * (src/update.f:16-193) and FFT_nr3.f:173-179 in mirror mode. */
int cpfft_commit_step(void);

/* Overwrite the device Fn / Fn1 fields (N3,9) from the host (mirror mode). */
int cpfft_set_F(const double* Fn, const double* Fn1);

/* Release every device allocation. */
void cpfft_finalize(void);

/* Human-readable text of the last error (static storage). */
const char* cpfft_last_error(void);

/* Diagnostic, no counterpart in the reference: measured FP64 FMA rate of the current
 * GPU in TFLOP/s (the roofline denominator of the FP64-bound kernels). */
int cpfft_measure_fp64_peak(double* tflops);

/* ---- Learned initial guess of the local mm10 solve (extension; no reference
 * counterpart).  A 20-128-128-7 SiLU network (BF16 weights, FP32 accumulation, tcgen05
 * tensor cores) maps a voxel's features -- lattice quaternion (4), rotated strain
 * increment D (6), the return-mapped elastic trial stress (6), tau_n, the extrapolated
 * tau, cos(D, D_n), |D| -- to the converged state's offset from the return-mapped trial:
 * sigma - sigma_trial (6) and tau - tau_extrapolated.  Parameters: CPFFT_MLP_PARAMS floats
 * (W1 [128][32], b1, W2 [128][128], b2, W3 [16][128], b3; padded rows and columns zero);
 * normalisation: CPFFT_MLP_NORM floats (feature means, inverse deviations, target means,
 * target deviations).  X is (n, 20) and Y, T are (n, 7), row-major FP32 host arrays. */
#define CPFFT_MLP_NIN 20
#define CPFFT_MLP_NOUT 7
#define CPFFT_MLP_PARAMS 22800
#define CPFFT_MLP_NORM 54

int cpfft_mlp_init(int seed);                                  /* Glorot init, identity norm */
int cpfft_mlp_set_params(const float* params, const float* norm);  /* either may be NULL */
int cpfft_mlp_get_params(float* params, float* norm);
int cpfft_mlp_forward(const float* X, long long n, float* Y);
/* mean squared error (normalised outputs) of one batch and its gradient, no update */
int cpfft_mlp_loss_grad(const float* X, const float* T, long long n, float* grad, float* loss);
/* Adam over (X, T): `epochs` shuffled passes, minibatches of batch_tiles x 128 samples;
 * sets the normalisation from the data; *loss = mean loss of the last epoch */
int cpfft_mlp_train(const float* X, const float* T, long long n, int epochs, int batch_tiles,
                    float lr, int seed, float* loss);
/* Log (features, converged offsets) pairs of the plain local solves of voxels with
 * v % stride == phase into device buffers of `capacity` pairs (0 stops logging). */
int cpfft_learn_log(long long capacity, int stride, int phase);
/* Copy the logged pairs to host arrays X (n, 20) and T (n, 7); *n = pairs copied. */
int cpfft_learn_fetch(float* X, float* T, long long* n);

#ifdef __cplusplus
}
#endif
#endif /* CPFFT_GPU_H */
