"""Element result files (ouelestr / oupestr, src/ouresult.f:140-300): the GPU's Fortran
E15.6 formatter and the wes/wee line layout against the oracle's restatement
(oracle/flat_ref.py), byte for byte."""
import os

import numpy as np
import pytest

from cpfft_gb300 import rve
from oracle import flat_ref


def test_oracle_e15_known_answers():
    cases = {123.456: "   0.123456E+03", -0.001: "  -0.100000E-02", 0.0: "   0.000000E+00",
             1.0: "   0.100000E+01", 1234565.0: "   0.123456E+07",  # tie: to even
             1234575.0: "   0.123458E+07", 999999.5: "   0.100000E+07",
             -2.5e-29: "  -0.250000E-28", 7.0e5: "   0.700000E+06", 1e100: "   0.100000+101"}
    for v, s in cases.items():
        assert flat_ref.e15_6(v) == s, (v, flat_ref.e15_6(v), s)


def adversarial_values(n, seed):
    rng = np.random.default_rng(seed)
    mags = 10.0 ** rng.uniform(-29.9, 7.0, n)
    x = mags * rng.choice([-1.0, 1.0], n)
    ties = np.array([1234565.0, 1234575.0, 999999.5, 99999.95, 0.5, 2.5, 1e5, 1e6, 1e-5,
                     123456.5, 123457.5, 2.0 ** -40, 2.0 ** 20, 3.0, 1.0 / 3.0])
    near = np.concatenate([np.nextafter(ties, 0.0), np.nextafter(ties, np.inf)])
    return np.concatenate([x, ties, -ties, near, [0.0, -0.0]])


@pytest.mark.gpu
def test_gpu_e15_formatter(gpulib):
    x = adversarial_values(200_000, 5)
    got = gpulib.format_e15(x)
    bad = [(v, g, flat_ref.e15_6(v)) for v, g in zip(x, got) if g != flat_ref.e15_6(v)]
    assert not bad, bad[:5]


@pytest.mark.gpu
def test_gpu_flat_files(gpulib, tmp_path):
    N = 9
    r = rve.make_rve(N, 4, 51)
    load = rve.uniaxial_tension(0.02, 20)
    s = gpulib.Solver(N, r.mat_list, r.kocks, r.crystals, 1.0, gpulib.G_REF_SHIFT)
    try:
        s.nr3_begin(1e-10)
        for step in (1, 2):
            s.nr3_step(step, load.BC_all[step - 1], load.isNBC, 1e-6, 1e-10, 20)
        _, _, H = s.fields(history=True)
        for quantity, word0, nvals in ((2, 0, 26), (1, 23, 22)):
            text = s.format_flat(quantity).decode()
            assert text == flat_ref.flat_text(H[word0:word0 + 6], nvals)
            s.write_flat(quantity, 2, "rve9", str(tmp_path))
            name = ("wes" if quantity == 2 else "wee") + "00002_text"
            lines = open(os.path.join(tmp_path, name)).read().split("\n")
            assert lines[0] == "#" and lines[6] == "#"
            assert lines[1].startswith("#  WARP3D element results: ")
            assert lines[3] == "#  Model nodes, elements: %8d%8d" % ((N + 1) ** 3, N ** 3)
            assert lines[5] == "#  Load(time) step: %8d" % 2
            assert "\n".join(lines[7:]) == text
        # ouresult writes the same two element files and the nodal file
        sub = tmp_path / "ouresult"
        sub.mkdir()
        s.ouresult(2, (100.0, 100.0, 100.0), "rve9", str(sub))
        assert sorted(os.listdir(sub)) == ["wee00002_text", "wes00002_text", "wnd00002_text"]
        for name in ("wee00002_text", "wes00002_text"):
            a = open(os.path.join(tmp_path, name)).read().split("\n")
            b = open(os.path.join(sub, name)).read().split("\n")
            assert a[:4] + a[5:] == b[:4] + b[5:]  # all but the date line
        u = s.f2disp((100.0, 100.0, 100.0))
        body = open(os.path.join(sub, "wnd00002_text")).read().split("\n")[7:-1]
        assert len(body) == (N + 1) ** 3
        assert body[5] == "".join(flat_ref.e15_6(0.0 if abs(x) < 1e-30 else x) for x in u[5])
    finally:
        s.close()
