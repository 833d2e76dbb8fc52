"""Self-interaction integrals S and the diagonal shift k^2 alpha S / V.

Host-side scalars, restated from the reference:
  2D: Transmission2D.py:12-36 (``self_interaction_integral_scalar`` /
      ``_vector``), scatterer volume pi a^2;
  3D: Transmission3D.py:13-37, scatterer volume 4 pi a^3 / 3.
"""
from __future__ import annotations

import numpy as np
import scipy.special as sps

_EG = np.euler_gamma


def si_2d_scalar(k0, radius, self_interaction_type="Rayleigh"):
    volume = np.pi * radius ** 2
    if self_interaction_type == "full":
        return -1 / (k0 * k0) + 0.5j * volume * sps.hankel1(1, k0 * radius) / (k0 * radius)
    if self_interaction_type == "Rayleigh":
        return (-1.0 * radius ** 2 / 4.0) * (2.0 * _EG - 1.0 + 2.0 * np.log(k0 * radius / 2.0) - 1j * np.pi)
    raise NotImplementedError


def si_2d_vector(k0, radius, self_interaction_type="Rayleigh"):
    volume = np.pi * radius ** 2
    if self_interaction_type == "full":
        return -1 / (k0 * k0) + 0.25j * volume * sps.hankel1(1, k0 * radius) / (k0 * radius)
    if self_interaction_type == "Rayleigh":
        return -1 / (2.0 * k0 * k0) - (radius ** 2 / 8.0) * (2.0 * _EG - 1.0 + 2.0 * np.log(k0 * radius / 2.0)
                                                             - 1j * np.pi)
    raise NotImplementedError


def si_3d_vector(k0, radius, self_interaction_type="Rayleigh"):
    volume = 4.0 * np.pi * radius ** 3 / 3.0
    if self_interaction_type == "full":
        return (1.0 / k0 ** 2) * ((2.0 / 3.0) * np.exp(1j * k0 * radius) * (1 - 1j * k0 * radius) - 1.0)
    if self_interaction_type == "Rayleigh":
        return -1.0 / (3.0 * k0 ** 2) + radius ** 2 / 3.0 + 1j * k0 * volume / (6.0 * np.pi)
    raise NotImplementedError


def si_3d_scalar(k0, radius, self_interaction_type="Rayleigh"):
    volume = 4.0 * np.pi * radius ** 3 / 3.0
    if self_interaction_type == "full":
        return (1.0 / k0 ** 2) * (np.exp(1j * k0 * radius) * (1 - 1j * k0 * radius) - 1.0)
    if self_interaction_type == "Rayleigh":
        return radius ** 2 / 2.0 + 1j * k0 * volume / (4.0 * np.pi)
    raise NotImplementedError


SELF_TERM = {"2d_vector": si_2d_vector, "2d_scalar": si_2d_scalar,
             "3d_vector": si_3d_vector, "3d_scalar": si_3d_scalar}


def volume(kind, radius):
    return np.pi * radius * radius if kind.startswith("2d") else 4 * np.pi * radius ** 3 / 3


def self_over_volume(kind, k0, radius, self_interaction_type="Rayleigh"):
    return complex(SELF_TERM[kind](k0, radius, self_interaction_type)) / volume(kind, radius)


def diagonal_shift(kind, k0, alpha, radius, self_interaction=True, self_interaction_type="Rayleigh",
                   reference_rounding=True):
    """k^2 alpha S/V as subtracted from the diagonal of M.

    The reference multiplies this scalar by ``torch.eye(dims)``, a float32
    tensor, so the value it subtracts is rounded to complex64
    (Transmission2D.py:228, :739; Transmission3D.py:203, :715).  With
    ``reference_rounding`` (the default) the same rounding is applied here so
    that results match the reference's; without it the exact value is used.
    """
    if not self_interaction:
        return 0j
    s = complex(alpha * k0 * k0 * self_over_volume(kind, k0, radius, self_interaction_type))
    if reference_rounding:
        s = complex(np.complex64(s))
    return s
