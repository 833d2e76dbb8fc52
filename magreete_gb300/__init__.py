"""magreete_gb300: coupled-dipole multiple scattering on one NVIDIA GB300.

A GB300-native engine behind the MAGreeTe solver-class API.  The public
classes live in the ``Transmission2D`` / ``Transmission3D`` modules (same
names as the reference's); the device building blocks are in ``engine``.
"""
from .Transmission2D import Transmission2D_scalar, Transmission2D_vector  # noqa: F401
from .Transmission3D import Transmission3D_scalar, Transmission3D_vector  # noqa: F401

__version__ = "0.1.0"
