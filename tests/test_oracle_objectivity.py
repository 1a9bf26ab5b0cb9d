"""Frame indifference of the oracle's material point, a known answer that needs no
reference output: a step F -> Q F after a rigid rotation step I -> Q must give Q P and
the tangent rotated on its spatial legs.

The kinematics (src/drive_eps_sig.f:200-325: mid-step polar rotation, unrotated rate of
deformation, Cauchy stress rotated back with R_{n+1}, pull-back to P and dP/dF) are
exactly objective, and so is mm01, whose update lives wholly in the unrotated frame.
mm10 is objective up to its lattice-spin term: the residual and J11 contract the
unrotated stress with spin vectors rotated by the current polar rotation
(qc = rt2rvw(R Rp^T) qs, src/mm10_a.f:866-876, used by mm10_form_wp src/mm10_b.f:1304-1374
and mm10_formJ11 :205), so a superposed rotation changes a plastic step's P by a little
more than rotating it; in the elastic range the spin term vanishes with the slip."""
import numpy as np
import pytest
from scipy.spatial.transform import Rotation

from cpfft_gb300 import rve

I3 = np.eye(3)
AXIS = np.array([0.3, -0.5, 0.8]) / np.linalg.norm([0.3, -0.5, 0.8])
KOCKS = np.array([30.0, 50.0, 70.0])


def rotation(angle):
    return Rotation.from_rotvec(angle * AXIS).as_matrix()


def rotated_pair(update, Q, F):
    """(step 1: I -> F) and (step 1: I -> Q, rigid; step 2: Q -> Q F)."""
    a = update(1, I3, F, None)
    r = update(1, I3, Q, None)
    b = update(2, Q, Q @ F, r["hist"])
    return a, r, b


def frame_errors(Q, a, b):
    P, Pq = a["P"].reshape(3, 3), b["P"].reshape(3, 3)
    A, Aq = a["A"].reshape(3, 3, 3, 3), b["A"].reshape(3, 3, 3, 3)
    Arot = np.einsum("ia,kb,aJbL->iJkL", Q, Q, A)
    return (np.abs(Pq - Q @ P).max() / np.abs(P).max(),
            np.abs(Aq - Arot).max() / np.abs(A).max())


@pytest.mark.parametrize("angle", [1e-3, 0.05, 0.5, 2.0])
@pytest.mark.parametrize("mat", [0, 1])
@pytest.mark.parametrize("scale", [1e-4, 1e-2])
def test_mm01_is_frame_indifferent(oracle, angle, mat, scale):
    """Both of the deck's bilinear materials, elastic (1e-4) and plastic (1e-2) steps."""
    props = rve.MM01_DECK[mat]
    rng = np.random.default_rng(11)
    F = I3 + scale * (np.diag([1.0, -0.4, -0.4]) + 0.2 * rng.standard_normal((3, 3)))
    Q = rotation(angle)

    def update(step, Fn, Fn1, h):
        return oracle.mises_update(props, step, Fn, Fn1, h)

    a, r, b = rotated_pair(update, Q, F)
    assert np.abs(r["P"]).max() < 1e-10 * props["e"]   # a rigid rotation stresses nothing
    eP, eA = frame_errors(Q, a, b)
    assert eP < 1e-10 and eA < 1e-12, (eP, eA)


@pytest.mark.parametrize("crystal", ["voce", "mts", "mrr"])
def test_rigid_rotation_step_keeps_the_state(oracle, crystal):
    """A step I -> Q: the midpoint rate of deformation is the Cayley transform's symmetric
    part, zero, so the stress stays at round-off and the plastic rotation at I."""
    cr = {"voce": rve.FCC_VOCE, "mts": rve.MTS_FCC, "mrr": rve.MRR_FCC}[crystal]
    r = oracle.voxel_update(cr, KOCKS, 1.0, 1, 1, I3, rotation(0.5))
    assert np.abs(r["P"]).max() < 1e-9
    Rp = r["hist"][7:16].reshape(3, 3)
    assert np.abs(Rp - I3).max() < 1e-14


@pytest.mark.parametrize("angle", [0.05, 0.5])
@pytest.mark.parametrize("scale", [1e-5, 1e-4])
def test_mm10_elastic_range_is_frame_indifferent(oracle, angle, scale):
    F = I3 + scale * np.diag([1.0, -0.4, -0.4])
    Q = rotation(angle)

    def update(step, Fn, Fn1, h):
        return oracle.voxel_update(rve.FCC_VOCE, KOCKS, 1.0, step, 1, Fn, Fn1, h)

    a, _, b = rotated_pair(update, Q, F)
    eP, _ = frame_errors(Q, a, b)
    assert eP < 1e-9, eP


def test_mm10_plastic_step_carries_the_spin_term(oracle):
    """A plastic step (strain 1e-3): within 1e-4 of objective, but not to round-off, and
    the departure grows with the superposed angle (the qc term)."""
    F = I3 + 1e-3 * np.diag([1.0, -0.4, -0.4])

    def update(step, Fn, Fn1, h):
        return oracle.voxel_update(rve.FCC_VOCE, KOCKS, 1.0, step, 1, Fn, Fn1, h)

    errs = []
    for angle in (0.05, 0.5):
        Q = rotation(angle)
        a, _, b = rotated_pair(update, Q, F)
        errs.append(frame_errors(Q, a, b)[0])
    assert 1e-8 < errs[0] < errs[1] < 1e-4, errs


def test_zero_first_increment_leaves_plastic_rotation_zero(oracle):
    """The reference's early return for a point with no stress and no strain increment
    (no_load, src/mm10_a.f:2682-2689, :1132-1135) skips mm10_update_rotation, so np1%Rp
    keeps the zero of mm10_setup_np1 (:1712-1718).  Committed, that state has no slip
    geometry: the next step differs from the same step taken from the virgin state."""
    cr = rve.FCC_VOCE
    z = oracle.voxel_update(cr, KOCKS, 1.0, 1, 1, I3, I3)
    assert np.all(z["hist"][7:16] == 0.0)
    F = I3 + 1e-3 * np.diag([1.0, -0.4, -0.4])
    virgin = oracle.voxel_update(cr, KOCKS, 1.0, 1, 1, I3, F)
    after = oracle.voxel_update(cr, KOCKS, 1.0, 2, 1, I3, F, z["hist"])
    assert np.abs(after["P"] - virgin["P"]).max() > 1e-2 * np.abs(virgin["P"]).max()
