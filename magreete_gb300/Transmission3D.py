"""GB300 drop-in for the reference module ``Transmission3D`` (3D coupled dipoles).

Same public names as the reference module: ``self_interaction_integral_vector``,
``self_interaction_integral_scalar``, ``Transmission3D_vector`` and
``Transmission3D_scalar``.
"""
from __future__ import annotations

from . import sources as _src
from .selfterm import si_3d_scalar as self_interaction_integral_scalar  # Transmission3D.py:26-37
from .selfterm import si_3d_vector as self_interaction_integral_vector  # Transmission3D.py:13-24
from .solver import CoupledDipoleSolver, _home_device

__all__ = ["Transmission3D_vector", "Transmission3D_scalar", "self_interaction_integral_scalar",
           "self_interaction_integral_vector"]


class _Transmission3D(CoupledDipoleSolver):
    def greens(self, r, k0, periodic="", regularize=False, radius=0.0):
        """Green's tensor of separations r (N, M, 3) (Transmission3D.py:47-77, :573-601),
        evaluated by the GPU kernel."""
        return self._greens_of_separations(r, k0, periodic, regularize, radius)

    def G0(self, points, k0, print_statement="", regularize=False, radius=0.0):
        """(dM, dN) propagator; points=None gives the scatterer matrix with zero self blocks
        (Transmission3D.py:240-268, :751-777)."""
        return self._G0_dense(points, k0, print_statement, regularize, radius)


class Transmission3D_vector(_Transmission3D):
    """3x3 dyadic Green's function (Transmission3D.py:39-564)."""
    kind = "3d_vector"

    def generate_source(self, points, k0, u, p, w, print_statement=""):
        """Incident field at points (M, 3) for directions u and polarisations p (R, 3)
        (Transmission3D.py:79-145)."""
        home = _home_device(points)
        return _src.source_3d(self.kind, self.source, self._pts(points), k0, u, p, w).to(home)


class Transmission3D_scalar(_Transmission3D):
    """Scalar 3D Green's function (Transmission3D.py:565-1078)."""
    kind = "3d_scalar"

    def generate_source(self, points, k0, u, w, print_statement=""):
        """Incident field at points (M, 3) for directions u (R, 3) (Transmission3D.py:603-658)."""
        home = _home_device(points)
        return _src.source_3d(self.kind, self.source, self._pts(points), k0, u, None, w).to(home)
