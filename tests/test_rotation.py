"""rotate_galaxy: the oracle against the reference's known answers
(tests/test_galaxy_alignment.py, tests/test_core_rotation.py), the index-padding
property of the reference's inertia tensor, the step's config checks, and the CUDA
kernels against the oracle."""

import numpy as np
import pytest

import oracle
from helpers import to_dev

UNIT = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])


def test_inertia_tensor_known_answer():  # test_galaxy_alignment.py:75-90
    np.testing.assert_allclose(oracle.moment_of_inertia_tensor(UNIT, np.ones(3), 2.0),
                               np.diag([2.0, 2.0, 2.0]))


def test_inertia_tensor_index_padding():
    # particle 0 at (1,0,0) inside, particle 2 outside r = 2: jnp.where(size=3) pads the
    # selection with index 0, so particle 0 is counted twice
    pos = np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [5.0, 0.0, 0.0]])
    I = oracle.moment_of_inertia_tensor(pos, np.ones(3), 2.0)
    expect = 2 * np.diag([0.0, 1.0, 1.0]) + np.diag([1.0, 0.0, 1.0])
    np.testing.assert_allclose(I, expect)


def test_euler_and_rotate_known_answers():  # test_galaxy_alignment.py:127-198
    np.testing.assert_allclose(oracle.euler_rotation_matrix(90.0, 0.0, 0.0),
                               [[1, 0, 0], [0, 0, -1], [0, 1, 0]], atol=1e-12)
    np.testing.assert_allclose(oracle.rotation_matrix_from_inertia_tensor(np.diag([1.0, 2, 3])),
                               np.eye(3), atol=1e-12)
    pos, vel = oracle.rotate_galaxy(UNIT, UNIT[[1, 2, 0]], np.ones(3), 2.0, 90.0, 0.0, 0.0)
    np.testing.assert_allclose(pos, [[1, 0, 0], [0, 0, -1], [0, 1, 0]], atol=1e-7)
    # the velocities follow the same row-vector product (v . R)
    np.testing.assert_allclose(vel, UNIT[[1, 2, 0]] @ oracle.euler_rotation_matrix(90, 0, 0),
                               atol=1e-7)


def test_rotation_step_config_messages():  # tests/test_core_rotation.py:14-73
    from rubix_gb300.core import get_galaxy_rotation

    with pytest.raises(ValueError, match="Rotation information not provided in galaxy config"):
        get_galaxy_rotation({"galaxy": {}})
    for missing in ("alpha", "beta", "gamma"):
        rot = {k: 0 for k in ("alpha", "beta", "gamma") if k != missing}
        with pytest.raises(ValueError, match=f"{missing} not provided in rotation information"):
            get_galaxy_rotation({"galaxy": {"rotation": rot}})
    with pytest.raises(ValueError, match="Invalid type provided in rotation information"):
        get_galaxy_rotation({"galaxy": {"rotation": {"type": "invalid"}}})
    for cfg in ({"type": "face-on"}, {"type": "edge-on"}, {"alpha": 45, "beta": 30, "gamma": 15}):
        f = get_galaxy_rotation({"galaxy": {"rotation": cfg}})
        assert callable(f) and f.__name__ == "rotate_galaxy"


def test_host_matrices_match_oracle():
    from rubix_gb300.core import rotation as rot

    for a, b, g in ((0, 0, 0), (90, 0, 0), (45, 30, 15), (-20, 170, 33)):
        np.testing.assert_allclose(rot.euler_rotation_matrix(a, b, g),
                                   oracle.euler_rotation_matrix(a, b, g), atol=1e-15)


@pytest.mark.gpu
def test_inertia_and_rotation_kernels():
    import torch

    from rubix_gb300 import ops, synth

    p = synth.make_galaxy(20000, seed=9)
    hmr = 4.0
    I = ops.inertia_tensor(to_dev(p.coords), to_dev(p.mass), hmr).cpu().numpy()
    Io = oracle.moment_of_inertia_tensor(p.coords, p.mass, hmr)
    np.testing.assert_allclose(I, Io, rtol=1e-9, atol=1e-9 * np.abs(Io).max())
    M = oracle.rotation_matrix_from_inertia_tensor(Io) @ oracle.euler_rotation_matrix(30, 10, 5)
    got = ops.rotate_vectors(to_dev(p.velocity), M).cpu().numpy()
    want = (p.velocity.astype(np.float64) @ M).astype(np.float32)
    np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-6 * np.abs(want).max())
    torch.cuda.synchronize()
