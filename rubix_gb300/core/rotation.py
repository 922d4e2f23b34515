"""Step rotate_galaxy (rubix/core/rotation.py:11-117; galaxy/alignment.py:66-265) on
the CUDA inertia-tensor and rotation kernels.

Same config keys, validation messages and closure name as rubix: the galaxy is turned
into the principal frame of its moment-of-inertia tensor within the stellar half-mass
radius (eigenvectors in ascending eigenvalue order), then rotated by the Euler angles
alpha, beta, gamma (degrees, R = R_z R_y R_x; "face-on" = (0, 0, 0), "edge-on" =
(90, 0, 0)).  Positions and velocities are row vectors multiplied by the matrices, as
rubix does (jnp.dot(positions, R)).  The 3x3 eigen-decomposition runs on the host
(numpy.linalg.eigh) after one small device-to-host copy of the tensor.
"""

from __future__ import annotations

from typing import Callable

import numpy as np
import torch

from .. import ops
from ..logging import get_logger
from .data import RubixData, device_of, to_device


def euler_rotation_matrix(alpha: float, beta: float, gamma: float) -> np.ndarray:
    """alignment.py:162-205: R_z(gamma) R_y(beta) R_x(alpha), angles in degrees."""
    a, b, g = np.deg2rad([alpha, beta, gamma])
    Rx = np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])
    Ry = np.array([[np.cos(b), 0, np.sin(b)], [0, 1, 0], [-np.sin(b), 0, np.cos(b)]])
    Rz = np.array([[np.cos(g), -np.sin(g), 0], [np.sin(g), np.cos(g), 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def rotation_matrix_from_inertia_tensor(I) -> np.ndarray:
    """alignment.py:123-138: eigenvectors of I as columns, ascending eigenvalues."""
    w, v = np.linalg.eigh(np.asarray(I, dtype=np.float64))
    return v[:, np.argsort(w)]


def get_galaxy_rotation(config: dict, handoff=None) -> Callable:
    """rubix/core/rotation.py:11-117.  With ``handoff`` (a ``core.telescope.FrameHandoff``
    whose ``rotation`` is set) the matrix is derived here and the turn itself runs in the
    spaxel_assignment pass that follows."""
    if "rotation" not in config["galaxy"]:
        raise ValueError("Rotation information not provided in galaxy config")
    logger = get_logger(config.get("logger", None))
    rot = config["galaxy"]["rotation"]
    if "type" in rot:
        if rot["type"] not in ["face-on", "edge-on"]:
            raise ValueError("Invalid type provided in rotation information")
        alpha, beta, gamma = (0.0, 0.0, 0.0) if rot["type"] == "face-on" else (90.0, 0.0, 0.0)
    else:
        for key in ["alpha", "beta", "gamma"]:
            if key not in rot:
                raise ValueError(f"{key} not provided in rotation information")
        alpha, beta, gamma = rot["alpha"], rot["beta"], rot["gamma"]
    R_euler = euler_rotation_matrix(alpha, beta, gamma)
    types = config.get("data", {}).get("args", {}).get("particle_type", ["stars"])

    def rotate_galaxy(rubixdata: RubixData) -> RubixData:
        logger.info(f"Rotating galaxy with alpha={alpha}, beta={beta}, gamma={gamma}")
        dev = device_of(config)
        hmr = rubixdata.galaxy.halfmassrad_stars if rubixdata.galaxy is not None else None
        if hmr is None:
            raise ValueError("rotate_galaxy needs rubixdata.galaxy.halfmassrad_stars")
        hmr = float(np.asarray(hmr.cpu() if isinstance(hmr, torch.Tensor) else hmr).reshape(-1)[0])
        for particle_type in ["stars", "gas"]:
            if particle_type not in types:
                continue
            comp = getattr(rubixdata, particle_type)
            assert comp.coords is not None, f"Coordinates not found for {particle_type}. "
            assert comp.velocity is not None, f"Velocities not found for {particle_type}. "
            assert comp.mass is not None, f"Masses not found for {particle_type}. "
            coords = to_device(comp.coords, dev)
            vel = to_device(comp.velocity, dev)
            mass = to_device(comp.mass, dev)
            I = ops.inertia_tensor(coords, mass, hmr).cpu().numpy()
            M = rotation_matrix_from_inertia_tensor(I) @ R_euler
            if handoff is not None and handoff.rotation:
                handoff.matrix[particle_type] = (M, coords, vel)
                continue
            comp.coords = ops.rotate_vectors(coords, M)
            comp.velocity = ops.rotate_vectors(vel, M)
        return rubixdata

    return rotate_galaxy
