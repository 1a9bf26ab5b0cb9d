"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module, and only as the parity reference or the timed CPU stand-in.  The product path never
touches it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcpfft_oracle.so")
HIST_WORDS = 31
HIST_WORDS_MRR = 55  # grids of dislocation-density crystals (h_type 7, 4)

_lib = None


class Crystal(ctypes.Structure):
    """Mirror of ``cpfft_crystal`` in include/cpfft_gpu.h."""

    _fields_ = [
        ("slip_type", ctypes.c_int),
        ("elastic_type", ctypes.c_int),
        ("e", ctypes.c_double), ("nu", ctypes.c_double), ("mu", ctypes.c_double),
        ("C11", ctypes.c_double), ("C12", ctypes.c_double), ("C13", ctypes.c_double),
        ("C33", ctypes.c_double), ("C44", ctypes.c_double), ("C55", ctypes.c_double),
        ("h_type", ctypes.c_int),
        ("harden_n", ctypes.c_double),
        ("tau_y", ctypes.c_double), ("tau_v", ctypes.c_double),
        ("theta_0", ctypes.c_double), ("voce_m", ctypes.c_double),
        ("gamma_bar", ctypes.c_double),
        ("iD_v", ctypes.c_double),
        ("alter_mode", ctypes.c_int),
        ("atol", ctypes.c_double), ("atol1", ctypes.c_double),
        ("rtol", ctypes.c_double), ("rtol1", ctypes.c_double),
        ("miter", ctypes.c_int),
        ("exact_j22", ctypes.c_int),
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


class Mises(ctypes.Structure):
    """cpfft_mises of include/cpfft_gpu.h."""

    _fields_ = [("e", ctypes.c_double), ("nu", ctypes.c_double), ("yld_pt", ctypes.c_double),
                ("tan_e", ctypes.c_double), ("beta", ctypes.c_double)]


def _mises(m):
    return Mises(m["e"], m["nu"], m["yld_pt"], m["tan_e"], m.get("beta", 1.0))


class Stats(ctypes.Structure):
    """Mirror of ``cpfft_stats``."""

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


def build():
    """Compile the oracle with its Makefile (portable flags, both host arches)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        d, i, vp = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
        dp = P(d)
        ip = P(i)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [i, ip, dp, P(Crystal), i, d, i, i]
        L.orc_destroy.argtypes = [vp]
        L.orc_stress_update.restype = i
        L.orc_stress_update.argtypes = [vp, i, i, dp, dp, dp, dp, P(ctypes.c_longlong)]
        L.orc_commit.argtypes = [vp]
        L.orc_stress_sample.restype = i
        L.orc_stress_sample.argtypes = [vp, i, i, ctypes.c_long, ctypes.c_long]
        L.orc_green_apply.argtypes = [vp, dp, dp, i, dp]
        L.orc_cg.restype = i
        L.orc_cg.argtypes = [vp, dp, dp, d, ip]
        L.orc_tangent_homo.restype = i
        L.orc_tangent_homo.argtypes = [vp, d, dp]
        L.orc_nr3_begin.restype = i
        L.orc_nr3_begin.argtypes = [vp, d]
        L.orc_set_equilibrium_tol.argtypes = [vp, d]
        L.orc_set_coupled_bc.argtypes = [vp, i]
        L.orc_nr3_step.restype = i
        L.orc_nr3_step.argtypes = [vp, i, dp, ip, d, d, i, dp, P(Stats)]
        L.orc_get_fields.argtypes = [vp, dp, dp, dp, dp, dp]
        L.orc_set_fields.argtypes = [vp, dp, dp]
        L.orc_get_history.argtypes = [vp, dp, dp]
        L.orc_hist_words.restype = i
        L.orc_hist_words.argtypes = [vp]
        L.orc_set_history_n.argtypes = [vp, dp]
        L.orc_voxel_update.restype = i
        L.orc_voxel_update.argtypes = [P(Crystal), dp, d, i, i, dp, dp, dp, dp, dp, dp,
                                       dp, dp]
        L.orc_set_mises.argtypes = [vp, i, P(Mises)]
        L.orc_set_svk.argtypes = [vp, i, d, d]
        L.orc_svk_point.argtypes = [d, d, dp, dp, dp]
        L.orc_mises_update.restype = i
        L.orc_mises_update.argtypes = [P(Mises), i, dp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_polar.argtypes = [dp, dp]
        L.orc_mrr_interaction.argtypes = [ctypes.c_int, dp, dp]
        L.orc_mrr_residual.restype = i
        L.orc_mrr_residual.argtypes = [P(Crystal), dp, dp, d, dp, dp, dp, dp]
        L.orc_crystal_setup.argtypes = [P(Crystal), dp, dp, dp, dp]
        L.orc_fft3.argtypes = [i, dp, dp, i]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def crystal_array(crystals):
    arr = (Crystal * len(crystals))()
    for k, c in enumerate(crystals):
        for name, _ in Crystal._fields_:
            setattr(arr[k], name, c[name])
    return arr


class Oracle:
    """One RVE on the CPU oracle.  Fields are numpy arrays shaped (9, N3) /
    (81, N3), i.e. the reference's column-major (N3, 9) / (N3, 81) memory."""

    def __init__(self, N, mat_list, kocks_deg, crystals, tstep, g_mapping=0,
                 nthreads=None):
        self.N = N
        self.N3 = N ** 3
        self._crys = crystal_array(crystals)
        ml = np.ascontiguousarray(mat_list, dtype=np.int32)
        ka = np.ascontiguousarray(np.asarray(kocks_deg, dtype=np.float64).reshape(3, self.N3))
        nthreads = nthreads or os.cpu_count()
        self.h = lib().orc_create(N, _ip(ml), _p(ka), self._crys, len(crystals), tstep,
                                  g_mapping, nthreads)

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    __del__ = close

    def stress_update(self, step, it, Fn=None, Fn1=None):
        P = np.zeros((9, self.N3))
        K = np.zeros((81, self.N3))
        li = ctypes.c_longlong(0)
        fails = lib().orc_stress_update(self.h, step, it, _p(Fn), _p(Fn1), _p(P), _p(K),
                                        ctypes.byref(li))
        return P, K, fails, li.value

    def stress_sample(self, step, it, v0, v1):
        return lib().orc_stress_sample(self.h, step, it, v0, v1)

    def commit(self):
        lib().orc_commit(self.h)

    def green(self, x, flgK=True, K4=None):
        y = np.zeros((9, self.N3))
        lib().orc_green_apply(self.h, _p(np.ascontiguousarray(x)), _p(y), int(flgK),
                              _p(K4) if K4 is not None else None)
        return y

    def cg(self, b, tol):
        x = np.zeros((9, self.N3))
        its = ctypes.c_int(0)
        rc = lib().orc_cg(self.h, _p(np.ascontiguousarray(b)), _p(x), tol, ctypes.byref(its))
        return x, its.value, rc

    def tangent_homo(self, tol):
        C = np.zeros(81)
        rc = lib().orc_tangent_homo(self.h, tol, _p(C))
        return C.reshape(9, 9).T.copy(), rc  # C[i, j] = C_homo(i, j) (Fortran)

    def set_equilibrium_tol(self, tol):
        lib().orc_set_equilibrium_tol(self.h, float(tol))

    def set_coupled_bc(self, on=True):
        lib().orc_set_coupled_bc(self.h, int(on))

    def nr3_begin(self, tolPCG):
        return lib().orc_nr3_begin(self.h, tolPCG)

    def nr3_step(self, step, BC, isNBC, tolNR, tolPCG, maxIter):
        Pbar = np.zeros(9)
        st = Stats()
        bc = np.ascontiguousarray(BC, dtype=np.float64)
        nb = np.ascontiguousarray(isNBC, dtype=np.int32)
        rc = lib().orc_nr3_step(self.h, step, _p(bc), _ip(nb), tolNR, tolPCG, maxIter,
                                _p(Pbar), ctypes.byref(st))
        return rc, Pbar, st.as_dict()

    def fields(self):
        out = [np.zeros((9, self.N3)) for _ in range(4)] + [np.zeros((81, self.N3))]
        lib().orc_get_fields(self.h, *[_p(a) for a in out])
        return dict(zip(["Fn", "Fn1", "Pn", "Pn1", "K4"], out))

    def set_fields(self, Fn=None, Fn1=None):
        lib().orc_set_fields(self.h, _p(Fn), _p(Fn1))

    def history(self):
        W = lib().orc_hist_words(self.h)
        hn = np.zeros((W, self.N3))
        hn1 = np.zeros((W, self.N3))
        lib().orc_get_history(self.h, _p(hn), _p(hn1))
        return hn, hn1

    def set_history_n(self, hn):
        lib().orc_set_history_n(self.h, _p(np.ascontiguousarray(hn)))

    def set_svk(self, material, K, mu):
        """A St-Venant-Kirchhoff material (the FFT program's original mm00)."""
        lib().orc_set_svk(self.h, int(material), float(K), float(mu))

    def set_mises(self, material, props):
        """props: dict e, nu, yld_pt, tan_e, beta (a bilinear Mises material, mm01)."""
        m = _mises(props)
        lib().orc_set_mises(self.h, int(material), ctypes.byref(m))


def svk_point(K, mu, F):
    """P (3x3) and dP/dF (9x9, (ij)(kl)) of the St-Venant-Kirchhoff material."""
    P = np.zeros(9)
    A = np.zeros(81)
    lib().orc_svk_point(K, mu, _p(np.ascontiguousarray(F, dtype=np.float64).reshape(9)),
                        _p(P), _p(A))
    return P.reshape(3, 3), A.reshape(9, 9)


def mises_update(props, step, Fn, Fn1, hist_n=None):
    """One mm01 material point (kinematics + mm01 + cnst1 + cep2A); F 3x3 row-major."""
    m = _mises(props)
    P = np.zeros(9)
    A = np.zeros(81)
    sig = np.zeros(6)
    cep = np.zeros(36)
    h1 = np.zeros(HIST_WORDS)
    fn = np.ascontiguousarray(Fn, dtype=np.float64).reshape(9)
    fn1 = np.ascontiguousarray(Fn1, dtype=np.float64).reshape(9)
    hn = None if hist_n is None else np.ascontiguousarray(hist_n, dtype=np.float64)
    lib().orc_mises_update(ctypes.byref(m), step, _p(fn), _p(fn1), _p(hn), _p(h1), _p(P),
                           _p(A), _p(sig), _p(cep))
    return dict(P=P, A=A.reshape(9, 9), sig=sig, cep=cep.reshape(6, 6), hist=h1)


def voxel_update(crystal, kocks, tstep, step, it, Fn, Fn1, hist_n=None):
    """One material point (kinematics + mm10 + cep2A); F as 3x3 row-major."""
    c = crystal_array([crystal])
    P = np.zeros(9)
    A = np.zeros(81)
    sig = np.zeros(6)
    cep = np.zeros(36)
    h1 = np.zeros(HIST_WORDS_MRR if crystal["h_type"] in (4, 7) else HIST_WORDS)
    k = np.ascontiguousarray(kocks, dtype=np.float64)
    fn = np.ascontiguousarray(Fn, dtype=np.float64).reshape(9)
    fn1 = np.ascontiguousarray(Fn1, dtype=np.float64).reshape(9)
    hn = None if hist_n is None else np.ascontiguousarray(hist_n, dtype=np.float64)
    its = lib().orc_voxel_update(c, _p(k), tstep, step, it, _p(fn), _p(fn1), _p(hn),
                                 _p(h1), _p(P), _p(A), _p(sig), _p(cep))
    return dict(P=P, A=A.reshape(9, 9), sig=sig, cep=cep.reshape(6, 6), hist=h1,
                iters=its)


def mrr_interaction(slip_type=1):
    """The Ma-Roters-Raabe forest and parallel interaction matrices (12 x 12 each) of a
    12-system slip type (1 fcc, 2 bcc, 6 roters, 7 bcc12)."""
    G = np.zeros(144)
    H = np.zeros(144)
    lib().orc_mrr_interaction(int(slip_type), _p(G), _p(H))
    return G.reshape(12, 12), H.reshape(12, 12)


def mrr_residual(crystal, kocks, D, tinc, x, hist_n=None):
    """Ma-Roters-Raabe local residual (18) and Jacobian (18 x 18) at x = (sigma, rho)."""
    c = crystal_array([crystal])
    R = np.zeros(18)
    J = np.zeros(324)
    hn = None if hist_n is None else np.ascontiguousarray(hist_n, dtype=np.float64)
    rc = lib().orc_mrr_residual(c, _p(np.ascontiguousarray(kocks, dtype=np.float64)),
                                _p(np.ascontiguousarray(D, dtype=np.float64)), float(tinc),
                                _p(hn), _p(np.ascontiguousarray(x, dtype=np.float64)), _p(R),
                                _p(J))
    assert rc == 0
    return R, J.reshape(18, 18)


def polar(F):
    R = np.zeros(9)
    lib().orc_polar(_p(np.ascontiguousarray(F, dtype=np.float64).reshape(9)), _p(R))
    return R.reshape(3, 3)


def crystal_setup(crystal, kocks):
    c = crystal_array([crystal])
    ns = {8: 48, 3: 1, 9: 6, 10: 18}.get(crystal.get("slip_type", 1), 12)
    C = np.zeros(36)
    ms = np.zeros(6 * ns)
    qs = np.zeros(3 * ns)
    lib().orc_crystal_setup(c, _p(np.ascontiguousarray(kocks, dtype=np.float64)), _p(C),
                            _p(ms), _p(qs))
    return C.reshape(6, 6), ms.reshape(ns, 6), qs.reshape(ns, 3)


def fft3(x, sign=-1):
    """3-D complex DFT (first index fastest).  Input shaped (N, N, N) in C order means
    the LAST numpy axis is the fastest memory axis."""
    N = x.shape[0]
    re = np.ascontiguousarray(x.real, dtype=np.float64)
    im = np.ascontiguousarray(x.imag, dtype=np.float64)
    lib().orc_fft3(N, _p(re), _p(im), sign)
    return re + 1j * im
