"""GB300 drop-in for the reference module ``Transmission2D`` (2D coupled dipoles).

Same public names as the reference module: ``self_interaction_integral_scalar``,
``self_interaction_integral_vector``, ``Transmission2D_vector`` (TE) and
``Transmission2D_scalar`` (TM).
"""
from __future__ import annotations

import torch

from . import sources as _src
from .selfterm import si_2d_scalar as self_interaction_integral_scalar  # Transmission2D.py:12-23
from .selfterm import si_2d_vector as self_interaction_integral_vector  # Transmission2D.py:25-36
from .solver import CoupledDipoleSolver, _as_tensor, _home_device

__all__ = ["Transmission2D_vector", "Transmission2D_scalar", "self_interaction_integral_scalar",
           "self_interaction_integral_vector"]


class _Transmission2D(CoupledDipoleSolver):
    def torch_hankel1(self, nu, x):
        """H_nu(x) = J_nu(x) + i Y_nu(x) for nu = 0, 1 (Transmission2D.py:46-61)."""
        x = _as_tensor(x)
        if nu == 0:
            return torch.special.bessel_j0(x) + 1j * torch.special.bessel_y0(x)
        if nu == 1:
            return torch.special.bessel_j1(x) + 1j * torch.special.bessel_y1(x)
        exit("torch Hankel function only implemented for orders 0 and 1!")

    def torch_greens(self, r, k0, periodic="", regularize=False, radius=0.0):
        """Green's tensor of separations r (N, M, 2) (Transmission2D.py:63-91, :595-618),
        evaluated by the GPU kernel."""
        return self._greens_of_separations(r, k0, periodic, regularize, radius)

    def generate_source(self, points, k0, thetas, w, print_statement=""):
        """Incident field at points (M, 2) for directions thetas (Transmission2D.py:93-174, :620-685)."""
        if self.source in ("beam", "plane", "point"):
            self._say(f"Calculating {self.source.capitalize()} Source at k0L/2pi = {self._k_label(k0)} ({print_statement})")
        home = _home_device(points)
        E0 = _src.source_2d(self.kind, self.source, self._pts(points), k0, thetas, w)
        return E0.to(home)


class Transmission2D_vector(_Transmission2D):
    """TE polarisation, 2x2 dyadic Green's function (Transmission2D.py:38-569)."""
    kind = "2d_vector"

    def G0_vector(self, points, k0, print_statement="", regularize=False, radius=0.0):
        """(2M, 2N) TE propagator; points=None gives the scatterer matrix with zero self blocks
        (Transmission2D.py:263-280)."""
        return self._G0_dense(points, k0, print_statement, regularize, radius)


class Transmission2D_scalar(_Transmission2D):
    """TM polarisation, scalar Green's function (Transmission2D.py:570-1065)."""
    kind = "2d_scalar"

    def G0(self, points, k0, print_statement="", regularize=False, radius=0.0):
        """(M, N) TM propagator (Transmission2D.py:777-785); self pairs are not zeroed."""
        return self._G0_dense(points, k0, print_statement, regularize, radius, zero_self=False)
