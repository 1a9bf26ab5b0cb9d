"""The Voce law's known answer, which needs no reference output: mm10_h_voche
(src/mm10_b.f:1888-1912) is a backward-Euler step of
d(tau_tilde) = theta_0 (1 - (tau_tilde - tau_y) / tau_v)^m sum |d gamma|, whose only fixed
point is tau_y + tau_v, approached from below.  A crystal with one slip system (slip_type
single: direction x, plane normal y) sheared along it accumulates slip without bound, so
its slip resistance climbs monotonically towards tau_y + tau_v and never passes it."""
import numpy as np
import pytest

from cpfft_gb300 import rve


@pytest.mark.parametrize("voce_m", [1.0, 2.0])
def test_voce_saturates_at_tau_y_plus_tau_v(oracle, voce_m):
    cr = dict(rve.FCC_VOCE, slip_type=3, voce_m=voce_m)
    sat = cr["tau_y"] + cr["tau_v"]
    F0, hist, tt = np.eye(3), None, []
    for step in range(1, 801):             # simple shear F12 to 2.0
        F1 = F0.copy()
        F1[0, 1] += 2.5e-3
        r = oracle.voxel_update(cr, np.zeros(3), 1.0, step, 1, F0, F1, hist)
        assert r["iters"] >= 0, step
        hist, F0 = r["hist"], F1
        tt.append(hist[6])
    tt = np.array(tt)
    assert tt[0] > cr["tau_y"] and np.all(np.diff(tt) >= 0.0) and tt.max() < sat
    # m = 1 approaches exponentially (sat - tt = tau_v exp(-theta_0 G / tau_v)), m = 2
    # algebraically (1 / (sat - tt) = 1 / tau_v + theta_0 G / tau_v^2), G the accumulated
    # slip (about 1.3 of the 2.0 shear here)
    assert sat - tt[-1] < (0.01 if voce_m == 1.0 else 0.2) * cr["tau_v"]
