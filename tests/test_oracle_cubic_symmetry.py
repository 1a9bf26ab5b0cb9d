"""Cubic symmetry of the oracle's crystals, a known answer that needs no reference output:
FCC {111}<110> and BCC {110},{112},{123}<111> slip with cubic elasticity are invariant
under the 24 proper rotations of the cube, so a lattice orientation g and S g (S acting in
the crystal frame) must give the same P, dP/dF and hardening, step after step.  The
check pins the slip tables (src/mod_crystals.f:438-811, 812-1207), the Kocks-angle
convention and the stiffness rotation together, and the dislocation-density laws'
interaction matrices: S permutes the slip systems and flips some slip directions, so
only a law that treats every system alike survives it.

MTS's tangent is the exception: the reference hands mm10_a_mult_type_4 the whole
symtqmat array (src/mm10_a.f:770-772), so each system's JA term reads system 1's column,
and which system is "system 1" changes under S.  Its P stays invariant."""
import itertools

import numpy as np
import pytest

from cpfft_gb300 import rve

I3 = np.eye(3)
KOCKS = np.array([20.0, 35.0, 70.0])
F1 = I3 + 2e-3 * np.array([[1.0, 0.3, -0.2], [0.1, -0.4, 0.25], [-0.15, 0.2, -0.5]])
CRYSTALS = {"voce": rve.FCC_VOCE, "mts": rve.MTS_FCC, "mrr": rve.MRR_FCC,
            "ornl": rve.ORNL_FCC, "bcc48": rve.BCC48_DECK,
            "bcc_voce": dict(rve.FCC_VOCE, slip_type=2),
            "roters_voce": dict(rve.FCC_VOCE, slip_type=6),
            "bcc12_voce": dict(rve.FCC_VOCE, slip_type=7),
            "bcc_mrr": dict(rve.MRR_FCC, slip_type=2)}


def cube_rotations():
    out = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            S = np.zeros((3, 3))
            for i, j in enumerate(perm):
                S[i, j] = signs[i]
            if np.linalg.det(S) > 0:
                out.append(S)
    return out


def two_steps(oracle, cr, kocks):
    a = oracle.voxel_update(cr, kocks, 1.0, 1, 1, I3, F1)
    b = oracle.voxel_update(cr, kocks, 1.0, 2, 1, F1, F1 @ F1, a["hist"])
    return a, b


def rel(x, y):
    return np.abs(x - y).max() / np.abs(y).max()


def test_cube_has_24_rotations():
    ops = cube_rotations()
    assert len(ops) == 24
    assert all(np.allclose(S @ S.T, I3) for S in ops)


@pytest.mark.parametrize("name", sorted(CRYSTALS))
def test_equivalent_orientations_respond_alike(oracle, name):
    cr = CRYSTALS[name]
    g = rve.kocks_matrix(KOCKS)[0]
    a1, a2 = two_steps(oracle, cr, KOCKS)
    assert a1["iters"] > 0 and a2["iters"] > 0      # the steps are plastic
    for S in cube_rotations():
        kocks = rve.matrix_to_kocks((S @ g)[None])[0]
        b1, b2 = two_steps(oracle, cr, kocks)
        assert rel(b1["P"], a1["P"]) < 1e-12 and rel(b2["P"], a2["P"]) < 1e-12
        if name == "mts":
            assert rel(b1["A"], a1["A"]) < 1e-3
        else:
            assert rel(b1["A"], a1["A"]) < 1e-12 and rel(b2["A"], a2["A"]) < 1e-12
        if name in ("mrr", "ornl", "bcc_mrr"):
            # the twelve densities after two steps: the same multiset, systems permuted
            rho_a = np.sort(a2["hist"][31:43])
            rho_b = np.sort(b2["hist"][31:43])
            assert rel(rho_b, rho_a) < 1e-12
