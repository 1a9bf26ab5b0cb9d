"""The C-ABI library builds, loads and exports every entry point include/cpfft_gpu.h
declares; argument checks that run before any device work behave as documented.
No GPU is needed (no call here reaches CUDA)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "cpfft_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cpfft_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("cpfft_init", "cpfft_stress_update", "cpfft_green_apply", "cpfft_cg",
                     "cpfft_nr3_step", "cpfft_sync_to_host", "cpfft_commit_step",
                     "cpfft_finalize", "cpfft_tangent_homo"):
        assert required in names


def test_library_exports_every_declared_symbol(gpulib):
    lib = gpulib.LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r" T (cpfft_[a-z0-9_]+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    L = gpulib.load_library()
    for n in declared_functions():
        assert hasattr(L, n)
        assert n in gpulib.SIGNATURES


def test_calls_before_init_fail_cleanly(gpulib):
    L = gpulib.load_library()
    L.cpfft_finalize()
    x = np.zeros(9)
    assert L.cpfft_stress_update(1, 0, None, None, None, None) == -7
    assert L.cpfft_commit_step() == -7
    assert L.cpfft_nr3_step(1, x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                            np.zeros(9, dtype=np.int32).ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                            1e-6, 1e-10, 10, None, None) == -7
    assert b"cpfft_init" in L.cpfft_last_error()


def test_init_rejects_bad_arguments(gpulib):
    from cpfft_gb300 import rve
    L = gpulib.load_library()
    cr = gpulib.crystal_struct([dict(rve.FCC_VOCE)])
    ml = np.ones(8, dtype=np.int32)
    ka = np.zeros(24)
    P = ctypes.POINTER
    mlp = ml.ctypes.data_as(P(ctypes.c_int))
    kap = ka.ctypes.data_as(P(ctypes.c_double))
    assert L.cpfft_init(1, mlp, kap, cr, 1, 1.0, 0) == -5       # N too small
    assert L.cpfft_init(2, mlp, kap, cr, 1, -1.0, 0) == -5      # tstep
    assert L.cpfft_init(2, mlp, kap, cr, 1, 1.0, 7) == -5       # mapping
    bad = dict(rve.FCC_VOCE)
    bad["slip_type"] = 11  # halite: no slip table
    assert L.cpfft_init(2, mlp, kap, gpulib.crystal_struct([bad]), 1, 1.0, 0) == -5
    ml2 = ml.copy()
    ml2[3] = 5
    assert L.cpfft_init(2, ml2.ctypes.data_as(P(ctypes.c_int)), kap, cr, 1, 1.0, 0) == -5


@pytest.mark.parametrize("bad", [dict(eta_max=1.0), dict(coupled_bc=3),
                                 dict(equilibrium_tol=-1e-6), dict(equilibrium_tol=np.inf),
                                 dict(tangent_tol=1.5)])
def test_batch_refuses_newton_options_out_of_range(gpulib, bad):
    """cpfft_batch_solve_newton checks its options before any RVE starts (no GPU call)."""
    L = gpulib.load_library()
    nt = gpulib.Newton(**dict(dict(equilibrium_tol=1e-6, eta_max=1e-2, tangent_tol=1e-2,
                                   coupled_bc=2), **bad))
    rv = (gpulib.Rve * 1)()
    assert L.cpfft_batch_solve_newton(rv, 1, 1, 0, 0, 0, ctypes.byref(nt), 1e-6, 1e-10, 20,
                                      1) == -5
    assert b"Newton option" in L.cpfft_last_error()
    with pytest.raises(ValueError):
        gpulib.batch_solve([], newton=dict(eta=1e-2))


def test_product_path_does_not_reference_the_oracle():
    for dirpath, _, files in os.walk(os.path.join(ROOT, "cpfft_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert "pyoracle" not in text and "cpfft_oracle" not in text, f


def test_stats_mirrors_match_the_header():
    """cpfft_stats is filled by both the library and the oracle: the ctypes mirrors must
    have the header's fields in order (a shorter mirror would be overrun)."""
    import cpfft_gb300
    from oracle import pyoracle
    src = open(os.path.join(ROOT, "include", "cpfft_gpu.h")).read()
    body = re.search(r"typedef struct cpfft_stats \{(.*?)\} cpfft_stats;", src, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    ctype = {"int": ctypes.c_int, "double": ctypes.c_double, "long long": ctypes.c_longlong}
    fields = [(m.group(2), ctype[m.group(1)])
              for m in re.finditer(r"(long long|int|double)\s+(\w+);", body)]
    for mirror in (cpfft_gb300.Stats, pyoracle.Stats):
        assert [(n, t) for n, t in mirror._fields_] == fields


def test_ctypes_signatures_match_the_header_arity(gpulib):
    """Every ctypes signature takes as many arguments as the header's prototype."""
    src = open(os.path.join(ROOT, "include", "cpfft_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    for m in re.finditer(r"\b(cpfft_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", src):
        name, params = m.group(1), m.group(2).strip()
        n = 0 if params in ("", "void") else params.count(",") + 1
        assert len(gpulib.SIGNATURES[name][1]) == n, (name, n, gpulib.SIGNATURES[name][1])


def test_struct_layouts_match_the_c_compiler(tmp_path):
    """Every struct of the boundary has, in the ctypes mirrors, the size and field offsets
    gcc gives it from include/cpfft_gpu.h (a probe program compiled here), and the history
    width constant agrees."""
    import cpfft_gb300
    from oracle import pyoracle
    mirrors = {"cpfft_crystal": [cpfft_gb300.Crystal, pyoracle.Crystal],
               "cpfft_mises": [cpfft_gb300.Mises, pyoracle.Mises],
               "cpfft_stats": [cpfft_gb300.Stats, pyoracle.Stats],
               "cpfft_rve": [cpfft_gb300.Rve], "cpfft_newton": [cpfft_gb300.Newton]}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "cpfft_gpu.h"',
             'int main(void) {', 'printf("HIST %d\\n", CPFFT_HIST_WORDS);',
             'printf("HISTMRR %d\\n", CPFFT_HIST_WORDS_MRR);']
    for name, ms in mirrors.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (name, name))
        for f, _ in ms[0]._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines += ["return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        parts = ln.split()
        if len(parts) == 2:
            got[parts[0]] = int(parts[1])
        elif len(parts) == 3:
            got[(parts[0], parts[1])] = int(parts[2])
    assert got["HIST"] == cpfft_gb300.HIST_WORDS == pyoracle.HIST_WORDS
    assert got["HISTMRR"] == cpfft_gb300.HIST_WORDS_MRR == pyoracle.HIST_WORDS_MRR
    for name, ms in mirrors.items():
        for m in ms:
            assert ctypes.sizeof(m) == got[(name, "size")], (name, m)
            for f, _ in m._fields_:
                assert getattr(m, f).offset == got[(name, f)], (name, f)
