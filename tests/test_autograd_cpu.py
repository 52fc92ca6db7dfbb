"""CPU tests of the pose algebra behind the differentiable projection (deepdrr_gb300.autograd)."""
import numpy as np
import pytest

from deepdrr_gb300.autograd import _skew, left_jacobian, rigid_motion, rotation


def _log(R):
    """Rotation vector of a rotation matrix (angles below pi)."""
    c = np.clip((np.trace(R) - 1.0) / 2.0, -1.0, 1.0)
    th = np.arccos(c)
    if th < 1e-12:
        return np.zeros(3)
    return th / (2 * np.sin(th)) * np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])


@pytest.mark.parametrize("w", [np.zeros(3), np.array([0.3, -0.2, 0.5]), np.array([1e-7, 2e-7, 0.0]),
                               np.array([-1.1, 0.4, 2.0])])
def test_rotation_is_orthonormal_and_matches_the_exponential(w):
    R = rotation(w)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-13)
    assert np.isclose(np.linalg.det(R), 1.0, atol=1e-13)
    # matrix exponential by series
    K = _skew(w)
    E, term = np.eye(3), np.eye(3)
    for k in range(1, 40):
        term = term @ K / k
        E = E + term
    assert np.allclose(R, E, atol=1e-12)


@pytest.mark.parametrize("w", [np.zeros(3), np.array([0.3, -0.2, 0.5]), np.array([-1.1, 0.4, 2.0])])
def test_left_jacobian_composes_small_rotations(w):
    J = left_jacobian(w)
    rng = np.random.default_rng(0)
    for _ in range(3):
        dw = rng.standard_normal(3) * 1e-6
        lhs = _log(rotation(w + dw) @ rotation(w).T)
        assert np.allclose(lhs, J @ dw, atol=1e-11)


def test_rigid_motion_turns_about_the_centre():
    c = np.array([10.0, -5.0, 3.0])
    T = rigid_motion([1.0, 2.0, 3.0, 0.1, 0.2, -0.3], c)
    # the centre moves by the translation only
    assert np.allclose(T[:3, :3] @ c + T[:3, 3], c + [1.0, 2.0, 3.0])
    assert np.allclose(rigid_motion(np.zeros(6), c), np.eye(4))
