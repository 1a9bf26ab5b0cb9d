"""The benchmark's bookkeeping without a GPU: its defaults (the fast form's Newton options,
the workload it names), the roofline arithmetic of the stress kernel (explicit passes by
P_bar mode, no flop model for the dislocation-density kernel) and the per-step counts."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def default_args(*argv):
    return bench.make_parser().parse_args(list(argv))


def test_defaults_name_the_fast_form():
    a = default_args()
    assert (a.N, a.grains, a.seed, a.mode, a.material) == (128, 256, 3, "mixed", "voce")
    assert a.tol_nr == 1e-6 and a.tol_equil == 1e-6 and a.inexact == 1e-2
    assert a.coupled_bc and a.implicit_first and a.tangent_tol == 1e-2
    cfg = bench.config_dict(a, "gb300")
    assert cfg["p_bar_update"].startswith("inside the Newton iteration")
    assert cfg["tolerances"]["tangent_homo"] == 1e-2
    assert "Voce" in cfg["workload"]
    ref = bench.config_dict(a, "reference")
    assert ref["p_bar_update"] == "nested loop (the reference's)"
    assert ref["tolerances"]["inexact_newton_eta_max"] == 0.0
    nested = bench.config_dict(default_args("--nested-bc"), "gb300")
    assert nested["p_bar_update"] == "nested loop (the reference's)"


def fake_run(material="voce", explicit=(0, 0)):
    N3 = 128 ** 3
    st = [dict(stress_updates=4, n_green32=100, n_green64=10, n_green32_timed=20,
               t_green32=0.01, t_green64=0.01, t_stress_kernel=0.19, t_cg_graph=0.07,
               nbc_iters=1, local_iters=2.9 * 4 * N3, predict_iters=0, newton_iters=3,
               cg_iters=150, res_equil=1e-8, res_fft=1e-8, local_fallbacks=0,
               t_device=0.32)] * 2
    return {"stats": st, "N3": N3, "explicit_passes": list(explicit), "material": material}


def test_stress_roofline_counts_explicit_passes():
    peaks = {"hbm_gbs": 6786.2}
    r0, _ = bench.roofline(fake_run(explicit=(0, 0)), 128, peaks, "measured", 1.255)
    r1, _ = bench.roofline(fake_run(explicit=(1, 1)), 128, peaks, "measured", 1.255)
    assert r0["kernel"].startswith("stress update")
    fl = bench.STRESS_FLOPS
    N3 = 128 ** 3
    # two passes move from the implicit base to the explicit cost
    diff = (r0["algorithmic_flops_per_launch"] - r1["algorithmic_flops_per_launch"]) * 8
    assert diff == pytest.approx(2 * N3 * (fl["implicit_base"] - fl["explicit"]))
    assert 0 < r0["frac"] < 1.5


def test_no_flop_model_for_the_density_kernel():
    r, _ = bench.roofline(fake_run("mrr"), 128, {"hbm_gbs": 6786.2}, "measured", 1.255)
    assert r["frac"] is None and r["traffic"] is None
    assert "stress_kernel_mrr_32" in r["flop_model"]


def test_counts_report_device_time_per_step():
    c = bench.counts(fake_run())
    assert c["stress_passes_per_step"] == 4.0
    assert c["s_device_per_step"] == [0.32, 0.32]
    assert c["newton"] == [3, 3]
