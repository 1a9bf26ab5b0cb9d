"""GB300 finite-strain FFT crystal-plasticity hot path (CPFFT drop-in).

The product is the C-ABI shared library ``_build/libcpfft_gb300.so`` (declared in
include/cpfft_gpu.h).  This module is a thin ctypes mirror of the reference's routines
for Python callers and tests: :class:`Solver` exposes ``drive_eps_sig``, ``G_K_dF``,
``fftPcg``, ``tangent_homo`` and one ``FFT_nr3`` load step with the reference's
argument meaning and error behaviour (a negative status raises :class:`CpfftError`).
There is no CPU fallback: loading fails loudly when the library is missing.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcpfft_gb300.so")
HIST_WORDS = 31
HIST_WORDS_MRR = 55  # grids of dislocation-density crystals (h_type 7, 4)
NOT_A_CRYSTAL = 0  # slip_type of a material defined by Solver.set_mises

G_REF_SHIFT, G_CENTERED = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
PRECOND_NONE, PRECOND_REFERENCE = 0, 1
START_PLAIN, START_LEARNED, START_ITERATE, START_TRIAL = 0, 1, 2, 4
SCHED_BLOCKS, SCHED_QUEUE = 0, 1
TANGENT_F32 = 8  # set_mode option of the mixed form

STATUS = {
    0: "ok", 1: "local mm10 fallback", -1: "CG reached maxIter", -2: "Newton maxIter",
    -3: "stress BC maxIter", -4: "singular mixed-BC system", -5: "bad argument",
    -6: "CUDA error", -7: "not initialised", -8: "improper CG tolerance",
    -9: "out of device memory", -10: "non-finite residual",
}


class CpfftError(RuntimeError):
    def __init__(self, code, where, detail):
        super().__init__(f"{where}: {STATUS.get(code, code)} ({code}): {detail}")
        self.code = code


class Crystal(ctypes.Structure):
    """``cpfft_crystal`` of include/cpfft_gpu.h."""

    _fields_ = [
        ("slip_type", ctypes.c_int), ("elastic_type", ctypes.c_int),
        ("e", ctypes.c_double), ("nu", ctypes.c_double), ("mu", ctypes.c_double),
        ("C11", ctypes.c_double), ("C12", ctypes.c_double), ("C13", ctypes.c_double),
        ("C33", ctypes.c_double), ("C44", ctypes.c_double), ("C55", ctypes.c_double),
        ("h_type", ctypes.c_int), ("harden_n", ctypes.c_double),
        ("tau_y", ctypes.c_double), ("tau_v", ctypes.c_double),
        ("theta_0", ctypes.c_double), ("voce_m", ctypes.c_double),
        ("gamma_bar", ctypes.c_double), ("iD_v", ctypes.c_double),
        ("alter_mode", ctypes.c_int),
        ("atol", ctypes.c_double), ("atol1", ctypes.c_double),
        ("rtol", ctypes.c_double), ("rtol1", ctypes.c_double),
        ("miter", ctypes.c_int), ("exact_j22", ctypes.c_int),
        ("tau_a", ctypes.c_double),
        ("tau_hat_y", ctypes.c_double), ("G_0_y", ctypes.c_double),
        ("p_y", ctypes.c_double), ("q_y", ctypes.c_double),
        ("tau_hat_v", ctypes.c_double), ("G_0_v", ctypes.c_double),
        ("p_v", ctypes.c_double), ("q_v", ctypes.c_double),
        ("eps_dot_0_v", ctypes.c_double),
        ("burgers", ctypes.c_double), ("boltzman", ctypes.c_double),
        ("mu_0", ctypes.c_double), ("D_0", ctypes.c_double), ("T_0", ctypes.c_double),
        ("u1", ctypes.c_double), ("u2", ctypes.c_double), ("u3", ctypes.c_double),
        ("u4", ctypes.c_double), ("u5", ctypes.c_double), ("u6", ctypes.c_double),
    ]


class Stats(ctypes.Structure):
    """``cpfft_stats`` of include/cpfft_gpu.h."""

    _fields_ = [
        ("newton_iters", ctypes.c_int), ("nbc_iters", ctypes.c_int),
        ("cg_solves", ctypes.c_int), ("cg_iters", ctypes.c_int),
        ("stress_updates", ctypes.c_int), ("local_fallbacks", ctypes.c_int),
        ("local_iters", ctypes.c_longlong),
        ("res_fft", ctypes.c_double), ("res_pbar", ctypes.c_double),
        ("res_equil", ctypes.c_double),
        ("t_pcg", ctypes.c_double), ("t_sigeps", ctypes.c_double),
        ("t_total", ctypes.c_double), ("t_device", ctypes.c_double),
        ("t_stress_kernel", ctypes.c_double), ("t_green64", ctypes.c_double),
        ("t_green32", ctypes.c_double), ("n_green64", ctypes.c_longlong),
        ("n_green32", ctypes.c_longlong), ("kernel_launches", ctypes.c_longlong),
        ("predict_iters", ctypes.c_longlong), ("guess_rejected", ctypes.c_longlong),
        ("t_cg_graph", ctypes.c_double), ("n_green32_timed", ctypes.c_longlong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Mises(ctypes.Structure):
    """``cpfft_mises`` of include/cpfft_gpu.h (bilinear Mises, mm01)."""

    _fields_ = [("e", ctypes.c_double), ("nu", ctypes.c_double), ("yld_pt", ctypes.c_double),
                ("tan_e", ctypes.c_double), ("beta", ctypes.c_double)]


class Rve(ctypes.Structure):
    """``cpfft_rve`` of include/cpfft_gpu.h (one RVE of cpfft_batch_solve)."""

    _fields_ = [
        ("N", ctypes.c_int), ("matList", ctypes.POINTER(ctypes.c_int)),
        ("kocks_deg", ctypes.POINTER(ctypes.c_double)), ("props", ctypes.POINTER(Crystal)),
        ("ncrystals", ctypes.c_int), ("tstep", ctypes.c_double), ("g_mapping", ctypes.c_int),
        ("nsteps", ctypes.c_int), ("BC_all", ctypes.POINTER(ctypes.c_double)),
        ("isNBC", ctypes.POINTER(ctypes.c_int)),
        ("Pbar", ctypes.POINTER(ctypes.c_double)), ("Fn1", ctypes.POINTER(ctypes.c_double)),
        ("Pn1", ctypes.POINTER(ctypes.c_double)), ("status", ctypes.c_int),
        ("steps_done", ctypes.c_int), ("voxel_updates", ctypes.c_longlong),
        ("cg_iters", ctypes.c_longlong), ("seconds", ctypes.c_double),
        ("error", ctypes.c_char * 160),
        ("mises", ctypes.POINTER(Mises)),
    ]


class Newton(ctypes.Structure):
    """``cpfft_newton`` of include/cpfft_gpu.h (the fast form's Newton options of a batch)."""

    _fields_ = [("equilibrium_tol", ctypes.c_double), ("eta_max", ctypes.c_double),
                ("tangent_tol", ctypes.c_double), ("coupled_bc", ctypes.c_int)]


# every exported symbol and its signature
_D, _I, _P = ctypes.c_double, ctypes.c_int, ctypes.POINTER
_DP, _IP = _P(_D), _P(_I)
_FP, _LL = _P(ctypes.c_float), ctypes.c_longlong
SIGNATURES = {
    "cpfft_init": (_I, [_I, _IP, _DP, _P(Crystal), _I, _D, _I]),
    "cpfft_set_mode": (_I, [_I, _I]),
    "cpfft_set_precond": (_I, [_I]),
    "cpfft_set_equilibrium_tol": (_I, [_D]),
    "cpfft_set_inexact_newton": (_I, [_D]),
    "cpfft_set_tangent_tol": (_I, [_D]),
    "cpfft_set_coupled_bc": (_I, [_I]),
    "cpfft_set_mises": (_I, [_I, ctypes.POINTER(Mises)]),
    "cpfft_set_schedule": (_I, [_I]),
    "cpfft_tuning": (_I, [_IP, _DP]),
    "cpfft_set_tiles": (_I, [_IP]),
    "cpfft_queue_chunk": (_I, [_IP, _IP, _DP]),
    "cpfft_format_flat": (_I, [_I, ctypes.c_char_p, _LL, _P(_LL)]),
    "cpfft_write_flat": (_I, [_I, _I, ctypes.c_char_p, ctypes.c_char_p]),
    "cpfft_format_e15": (_I, [_DP, _LL, ctypes.c_char_p]),
    "cpfft_f2disp": (_I, [_D, _D, _D, _DP]),
    "cpfft_write_disp_flat": (_I, [_I, _D, _D, _D, ctypes.c_char_p, ctypes.c_char_p]),
    "cpfft_ouresult": (_I, [_I, _D, _D, _D, ctypes.c_char_p, ctypes.c_char_p]),
    "cpfft_batch_solve": (_I, [ctypes.POINTER(Rve), _I, _I, _I, _I, _I, _D, _D, _I, _I]),
    "cpfft_slip_systems": (_I, [_I, _DP, _DP]),
    "cpfft_batch_solve_newton": (_I, [ctypes.POINTER(Rve), _I, _I, _I, _I, _I,
                                      ctypes.POINTER(Newton), _D, _D, _I, _I]),
    "cpfft_stress_update": (_I, [_I, _I, _DP, _DP, _DP, _DP]),
    "cpfft_green_apply": (_I, [_DP, _DP, _I]),
    "cpfft_green_apply_f32": (_I, [_FP, _FP, _I]),
    "cpfft_green_apply_df": (_I, [_DP, _DP, _I]),
    "cpfft_set_K4": (_I, [_DP]),
    "cpfft_pass_counts": (_I, [_P(_LL)]),
    "cpfft_cg": (_I, [_DP, _DP, _D, _IP]),
    "cpfft_tangent_homo": (_I, [_D, _DP]),
    "cpfft_nr3_step": (_I, [_I, _DP, _IP, _D, _D, _I, _DP, _P(Stats)]),
    "cpfft_nr3_begin": (_I, [_D]),
    "cpfft_sync_to_host": (_I, [_DP, _DP, _DP]),
    "cpfft_hist_words": (_I, []),
    "cpfft_commit_step": (_I, []),
    "cpfft_set_F": (_I, [_DP, _DP]),
    "cpfft_finalize": (None, []),
    "cpfft_last_error": (ctypes.c_char_p, []),
    "cpfft_measure_fp64_peak": (_I, [_DP]),
    "cpfft_green_apply_noalloc": (_I, [_I, _I, ctypes.c_void_p, ctypes.c_void_p, _I,
                                       ctypes.c_void_p, ctypes.c_void_p]),
    "cpfft_mlp_init": (_I, [_I]),
    "cpfft_mlp_set_params": (_I, [_FP, _FP]),
    "cpfft_mlp_get_params": (_I, [_FP, _FP]),
    "cpfft_mlp_forward": (_I, [_FP, _LL, _FP]),
    "cpfft_mlp_loss_grad": (_I, [_FP, _FP, _LL, _FP, _FP]),
    "cpfft_mlp_train": (_I, [_FP, _FP, _LL, _I, _I, ctypes.c_float, _I, _FP]),
    "cpfft_learn_log": (_I, [_LL, _I, _I]),
    "cpfft_learn_fetch": (_I, [_FP, _FP, _P(_LL)]),
}

MLP_NIN, MLP_NOUT, MLP_PARAMS, MLP_NORM = 20, 7, 22800, 54


def _fp(a):
    if a is None:
        return None
    if a.dtype != np.float32 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("expected a C-contiguous float32 array")
    return a.ctypes.data_as(_FP)


class Mlp:
    """The learned initial guess's network on the GPU (one per process)."""

    def __init__(self, seed=0):
        _check(load_library().cpfft_mlp_init(int(seed)), "mlp_init")

    def params(self):
        p = np.zeros(MLP_PARAMS, np.float32)
        n = np.zeros(MLP_NORM, np.float32)
        _check(load_library().cpfft_mlp_get_params(_fp(p), _fp(n)), "mlp_get_params")
        return p, n

    def set_params(self, params=None, norm=None):
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, np.float32)
        _check(load_library().cpfft_mlp_set_params(_fp(p), _fp(n)), "mlp_set_params")

    def forward(self, X):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((X.shape[0], MLP_NOUT), np.float32)
        _check(load_library().cpfft_mlp_forward(_fp(X), X.shape[0], _fp(Y)), "mlp_forward")
        return Y

    def loss_grad(self, X, T):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = ctypes.c_float(0.0)
        _check(load_library().cpfft_mlp_loss_grad(_fp(X), _fp(T), X.shape[0], _fp(g),
                                                   ctypes.byref(loss)), "mlp_loss_grad")
        return loss.value, g

    def train(self, X, T, epochs, batch_tiles=16, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        loss = ctypes.c_float(0.0)
        _check(load_library().cpfft_mlp_train(_fp(X), _fp(T), X.shape[0], int(epochs),
                                               int(batch_tiles), float(lr), int(seed),
                                               ctypes.byref(loss)), "mlp_train")
        return loss.value


def measure_fp64_peak():
    """FP64 FMA rate of the current GPU in TFLOP/s."""
    v = ctypes.c_double(0.0)
    _check(load_library().cpfft_measure_fp64_peak(ctypes.byref(v)), "fp64 peak")
    return v.value

_lib = None


def load_library(path=LIB_PATH):
    """Load the C-ABI library (never a CPU substitute)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; "
                "g.build()'` (the GPU path has no fallback)")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _dp(a):
    if a is None:
        return None
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(_DP)


def _check(code, where):
    if code < 0:
        raise CpfftError(code, where, load_library().cpfft_last_error().decode())
    return code


def crystal_struct(crystals):
    arr = (Crystal * len(crystals))()
    for k, c in enumerate(crystals):
        for name, _ in Crystal._fields_:
            setattr(arr[k], name, c[name])
    return arr


class Solver:
    """Device-resident RVE.  Fields are numpy arrays shaped (9, N3) / (81, N3), i.e. the
    memory of the reference's column-major (N3, 9) / (N3, 81) module arrays."""

    def __init__(self, N, mat_list, kocks_deg, crystals, tstep, g_mapping=G_REF_SHIFT,
                 precision=PREC_FP64):
        L = load_library()
        self.N, self.N3 = N, N ** 3
        self._crys = crystal_struct(crystals)
        ml = np.ascontiguousarray(mat_list, dtype=np.int32)
        ka = np.ascontiguousarray(np.asarray(kocks_deg, dtype=np.float64).reshape(3, self.N3))
        _check(L.cpfft_init(N, ml.ctypes.data_as(_IP), _dp(ka), self._crys, len(crystals),
                            tstep, g_mapping), "cpfft_init")
        if precision != PREC_FP64:
            self.set_mode(precision)

    def close(self):
        load_library().cpfft_finalize()

    def set_mode(self, precision, warm_start=START_PLAIN):
        """warm_start: START_PLAIN or an OR of START_LEARNED / START_ITERATE / START_TRIAL,
        and TANGENT_F32 (mixed precision)."""
        _check(load_library().cpfft_set_mode(precision, int(warm_start)), "cpfft_set_mode")

    def set_schedule(self, schedule=SCHED_QUEUE):
        """Voxel order of the implicit stress passes: blocks in order, or the work queue."""
        _check(load_library().cpfft_set_schedule(int(schedule)), "cpfft_set_schedule")

    def tuning(self):
        """Autotuned tile shapes {fp32: (B/D, C), double_float: (B/D, C)} and ms/apply."""
        t = np.zeros(4, np.int32)
        ms = np.zeros(2)
        _check(load_library().cpfft_tuning(t.ctypes.data_as(_IP), _dp(ms)), "cpfft_tuning")
        return {"fp32_tiles": t[:2].tolist(), "double_float_tiles": t[2:].tolist(),
                "fp32_ms": float(ms[0]), "double_float_ms": float(ms[1])}

    def queue_chunk(self):
        """The autotuned voxel-queue chunk and the candidates' pass times (ms)."""
        v, b = ctypes.c_int(0), ctypes.c_int(0)
        ms = np.zeros(6)
        _check(load_library().cpfft_queue_chunk(ctypes.byref(v), ctypes.byref(b), _dp(ms)),
               "cpfft_queue_chunk")
        return {"chunk": v.value, "blocks_per_sm": b.value or "all",
                "ms_128_256_512": ms[:3].tolist(), "ms_one_block_per_sm": ms[3:].tolist()}

    def set_tiles(self, fp32_bd, fp32_c, df_bd=16, df_c=2):
        """Pin the register passes' tile shapes (fp32_c < 0: the register-resident
        slowest-axis pass with -fp32_c columns per block)."""
        t = np.array([fp32_bd, fp32_c, df_bd, df_c], np.int32)
        _check(load_library().cpfft_set_tiles(t.ctypes.data_as(_IP)), "cpfft_set_tiles")

    def set_mises(self, material, e, nu, yld_pt, tan_e, beta=1.0):
        """Make the 1-based ``material`` (declared with slip_type NOT_A_CRYSTAL) a bilinear
        Mises material (mm01)."""
        m = Mises(float(e), float(nu), float(yld_pt), float(tan_e), float(beta))
        _check(load_library().cpfft_set_mises(int(material), ctypes.byref(m)),
               "cpfft_set_mises")

    def set_precond(self, precond=PRECOND_REFERENCE):
        """Reference-medium preconditioner of the mixed-precision inner iterations."""
        _check(load_library().cpfft_set_precond(int(precond)), "cpfft_set_precond")

    def set_inexact_newton(self, eta_max):
        """Solve each Newton system of nr3_step only as far as the equilibrium residual
        needs (Eisenstat-Walker forcing, at most eta_max; needs set_equilibrium_tol)."""
        _check(load_library().cpfft_set_inexact_newton(float(eta_max)), "cpfft_set_inexact_newton")

    def set_coupled_bc(self, on=True):
        """Update the prescribed-stress components of F_bar inside the Newton iteration
        (with set_equilibrium_tol); on = 2 also makes the step's first stress pass
        implicit."""
        _check(load_library().cpfft_set_coupled_bc(int(on)), "cpfft_set_coupled_bc")

    def set_tangent_tol(self, tol):
        """Relative tolerance of tangent_homo's solves under inexact Newton (default 1e-2)."""
        _check(load_library().cpfft_set_tangent_tol(float(tol)), "cpfft_set_tangent_tol")

    def set_equilibrium_tol(self, tol):
        """Also require ||G(P)|| / (sqrt(N3) ||P_bar||) <= tol to end a Newton loop of
        nr3_step (0: the reference's ||dF|| / ||F|| test alone)."""
        _check(load_library().cpfft_set_equilibrium_tol(float(tol)), "cpfft_set_equilibrium_tol")

    # --- learned initial guess of the local solve --------------------------------------
    def learn_log(self, capacity, stride=1, phase=0):
        """Log (features, converged increments) of the plain local solves of every
        stride-th voxel into device buffers of `capacity` pairs (0 stops logging)."""
        _check(load_library().cpfft_learn_log(int(capacity), int(stride), int(phase)),
               "cpfft_learn_log")
        self._log_cap = int(capacity)

    def learn_fetch(self):
        cap = getattr(self, "_log_cap", 0)
        X = np.zeros((cap, MLP_NIN), np.float32)
        T = np.zeros((cap, MLP_NOUT), np.float32)
        n = ctypes.c_longlong(0)
        _check(load_library().cpfft_learn_fetch(_fp(X), _fp(T), ctypes.byref(n)),
               "cpfft_learn_fetch")
        return X[:n.value], T[:n.value]

    # --- mirror of the reference routines ------------------------------------------
    def drive_eps_sig(self, step, it, Fn=None, Fn1=None, want_P=True, want_K4=False):
        P = np.zeros((9, self.N3)) if want_P else None
        K = np.zeros((81, self.N3)) if want_K4 else None
        rc = _check(load_library().cpfft_stress_update(step, it, _dp(Fn), _dp(Fn1), _dp(P),
                                                       _dp(K)), "drive_eps_sig")
        return P, K, rc

    def pass_counts(self):
        """Counters of the last stress pass: local iterations (summed over voxels),
        failed local solves, predictor iterations, dropped starts, sub-stepped solves."""
        c = (ctypes.c_longlong * 5)()
        _check(load_library().cpfft_pass_counts(c), "cpfft_pass_counts")
        return {"local_iters": c[0], "fallbacks": c[1], "predict_iters": c[2],
                "starts_dropped": c[3], "substepped": c[4]}

    def G_K_dF(self, x, flgK=True):
        y = np.zeros((9, self.N3))
        _check(load_library().cpfft_green_apply(_dp(np.ascontiguousarray(x)), _dp(y),
                                                int(flgK)), "G_K_dF")
        return y

    def G_K_dF_f32(self, x, flgK=True):
        """The FP32 operator of the mixed-precision Krylov iterations."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((9, self.N3), np.float32)
        _check(load_library().cpfft_green_apply_f32(_fp(x), _fp(y), int(flgK)), "G_K_dF_f32")
        return y

    def G_K_dF_df(self, x, flgK=True):
        """The double-float FP64-accurate operator of the mixed-precision solver."""
        y = np.zeros((9, self.N3))
        _check(load_library().cpfft_green_apply_df(_dp(np.ascontiguousarray(x)), _dp(y),
                                                   int(flgK)), "G_K_dF_df")
        return y

    def set_K4(self, K4):
        _check(load_library().cpfft_set_K4(_dp(np.ascontiguousarray(K4))), "set_K4")

    def fftPcg(self, b, tol):
        x = np.zeros((9, self.N3))
        its = ctypes.c_int(0)
        rc = load_library().cpfft_cg(_dp(np.ascontiguousarray(b)), _dp(x), tol,
                                     ctypes.byref(its))
        _check(rc, "fftPcg")
        return x, its.value

    def tangent_homo(self, tol):
        C = np.zeros(81)
        _check(load_library().cpfft_tangent_homo(tol, _dp(C)), "tangent_homo")
        return C.reshape(9, 9).T.copy()  # C[i, j] = C_homo(i, j) of the reference

    def nr3_begin(self, tolPCG):
        _check(load_library().cpfft_nr3_begin(tolPCG), "FFT_nr3 start")

    def nr3_step(self, step, BC, isNBC, tolNR, tolPCG, maxIter):
        Pbar = np.zeros(9)
        st = Stats()
        bc = np.ascontiguousarray(BC, dtype=np.float64)
        nb = np.ascontiguousarray(isNBC, dtype=np.int32)
        rc = _check(load_library().cpfft_nr3_step(step, _dp(bc), nb.ctypes.data_as(_IP), tolNR,
                                                  tolPCG, maxIter, _dp(Pbar),
                                                  ctypes.byref(st)), "FFT_nr3 step")
        return rc, Pbar, st.as_dict()

    def fields(self, history=False):
        F = np.zeros((9, self.N3))
        P = np.zeros((9, self.N3))
        H = np.zeros((_check(load_library().cpfft_hist_words(), "cpfft_hist_words"), self.N3)) \
            if history else None
        _check(load_library().cpfft_sync_to_host(_dp(F), _dp(P), _dp(H)), "sync_to_host")
        return (F, P, H) if history else (F, P)

    # --- element result files (ouelestr) ---------------------------------------------
    def format_flat(self, quantity):
        """The data lines of wesNNNNN_text (quantity 2) / weeNNNNN_text (1) as bytes."""
        L = load_library()
        n = ctypes.c_longlong(0)
        L.cpfft_format_flat(int(quantity), None, 0, ctypes.byref(n))
        buf = ctypes.create_string_buffer(n.value)
        _check(L.cpfft_format_flat(int(quantity), buf, n.value, ctypes.byref(n)), "format_flat")
        return buf.raw[:n.value]

    def write_flat(self, quantity, step, structure_name="cpfft", directory=""):
        _check(load_library().cpfft_write_flat(int(quantity), int(step),
                                               structure_name.encode(), directory.encode()),
               "write_flat")

    def f2disp(self, lengths=(100.0, 100.0, 100.0)):
        """Nodal displacements (the reference's u array as ((N+1)^3, 3))."""
        u = np.zeros(3 * (self.N + 1) ** 3)
        _check(load_library().cpfft_f2disp(float(lengths[0]), float(lengths[1]),
                                           float(lengths[2]), _dp(u)), "f2disp")
        return u.reshape(-1, 3)

    def write_disp_flat(self, step, lengths=(100.0, 100.0, 100.0), structure_name="cpfft",
                        directory=""):
        _check(load_library().cpfft_write_disp_flat(int(step), float(lengths[0]),
                                                    float(lengths[1]), float(lengths[2]),
                                                    structure_name.encode(),
                                                    directory.encode()), "write_disp_flat")

    def ouresult(self, step, lengths=(100.0, 100.0, 100.0), structure_name="cpfft",
                 directory=""):
        """ouresult(step): the wnd, wee and wes flat files of the step."""
        _check(load_library().cpfft_ouresult(int(step), float(lengths[0]), float(lengths[1]),
                                             float(lengths[2]), structure_name.encode(),
                                             directory.encode()), "ouresult")

    def commit(self):
        _check(load_library().cpfft_commit_step(), "commit_step")

    def set_F(self, Fn=None, Fn1=None):
        _check(load_library().cpfft_set_F(_dp(Fn), _dp(Fn1)), "set_F")


def batch_solve(rves, precision=PREC_MIXED, options=0, precond=PRECOND_REFERENCE,
                schedule=SCHED_QUEUE, tolNR=1e-5, tolPCG=1e-10, maxIter=20, nthreads=4,
                want_fields=False, newton=None):
    """Solve many RVEs at once (cpfft_batch_solve).  rves: dicts with N, mat_list, kocks,
    crystals, tstep, g_mapping and a loading (rve.Loading: BC_all, isNBC, nsteps used), and
    optionally mises: {material (1-based): dict(e, nu, yld_pt, tan_e, beta)} for materials
    declared NOT_A_CRYSTAL.  newton: None, or a dict of cpfft_newton's fields
    (equilibrium_tol, eta_max, tangent_tol, coupled_bc; absent ones 0) applied to every RVE
    (cpfft_batch_solve_newton).  Returns one dict per RVE: Pbar (nsteps, 9), status,
    voxel_updates, cg_iters, seconds, and (want_fields) F, P (9, N3)."""
    L = load_library()
    arr = (Rve * len(rves))()
    keep, out = [], []
    for k, d in enumerate(rves):
        N, N3 = d["N"], d["N"] ** 3
        ml = np.ascontiguousarray(d["mat_list"], dtype=np.int32)
        ka = np.ascontiguousarray(np.asarray(d["kocks"], dtype=np.float64).reshape(3, N3))
        cr = crystal_struct(d["crystals"])
        nsteps = int(d["nsteps"])
        bc = np.ascontiguousarray(np.asarray(d["BC_all"], dtype=np.float64)[:nsteps])
        nb = np.ascontiguousarray(d["isNBC"], dtype=np.int32)
        pb = np.zeros((nsteps, 9))
        F = np.zeros((9, N3)) if want_fields else None
        P = np.zeros((9, N3)) if want_fields else None
        keep += [ml, ka, cr, bc, nb, pb, F, P]
        r = arr[k]
        r.N, r.ncrystals, r.tstep, r.g_mapping, r.nsteps = N, len(d["crystals"]), d["tstep"], \
            d.get("g_mapping", G_CENTERED), nsteps
        r.matList = ml.ctypes.data_as(_IP)
        r.kocks_deg, r.BC_all, r.Pbar = _dp(ka), _dp(bc), _dp(pb)
        r.props = ctypes.cast(cr, ctypes.POINTER(Crystal))
        r.isNBC = nb.ctypes.data_as(_IP)
        r.Fn1, r.Pn1 = _dp(F), _dp(P)
        if d.get("mises"):
            ms = (Mises * len(d["crystals"]))()
            for m, p in d["mises"].items():
                ms[m - 1] = Mises(p["e"], p["nu"], p["yld_pt"], p["tan_e"], p.get("beta", 1.0))
            keep.append(ms)
            r.mises = ctypes.cast(ms, ctypes.POINTER(Mises))
        out.append({"Pbar": pb, "F": F, "P": P})
    if newton is None:
        rc = L.cpfft_batch_solve(arr, len(rves), precision, options, precond, schedule, tolNR,
                                 tolPCG, maxIter, nthreads)
    else:
        unknown = set(newton) - {f for f, _ in Newton._fields_}
        if unknown:
            raise ValueError("batch_solve: unknown Newton options %s" % sorted(unknown))
        nt = Newton(**newton)
        rc = L.cpfft_batch_solve_newton(arr, len(rves), precision, options, precond, schedule,
                                        ctypes.byref(nt), tolNR, tolPCG, maxIter, nthreads)
    for k, o in enumerate(out):
        r = arr[k]
        o.update(status=r.status, steps_done=r.steps_done, voxel_updates=r.voxel_updates,
                 cg_iters=r.cg_iters, seconds=r.seconds, error=r.error.decode())
    _check(rc, "cpfft_batch_solve")
    return out


def slip_systems(slip_type):
    """The slip directions and plane normals (systems x 3, crystal frame) the stress
    kernels use for a slip_type (cpfft_slip_systems; host only)."""
    L = load_library()
    ns = _check(L.cpfft_slip_systems(int(slip_type), None, None), "slip_systems")
    b, n = np.zeros((ns, 3)), np.zeros((ns, 3))
    _check(L.cpfft_slip_systems(int(slip_type), _dp(b), _dp(n)), "slip_systems")
    return b, n


def format_e15(values):
    """Fortran E15.6 of each value (the GPU formatter of the result files)."""
    x = np.ascontiguousarray(values, dtype=np.float64).ravel()
    buf = ctypes.create_string_buffer(15 * len(x) + 1)
    _check(load_library().cpfft_format_e15(_dp(x), len(x), buf), "format_e15")
    raw = buf.raw[:15 * len(x)].decode()
    return [raw[15 * i:15 * i + 15] for i in range(len(x))]
