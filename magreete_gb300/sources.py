"""Incident fields (generate_source) evaluated on the GPU.

Vectorised over all incidence directions at once (the reference loops over
angles in Python).  Float32 roundings the reference performs are kept so
that results agree with it bit-for-bit in the inputs and to rounding in the
outputs:
  * 2D TE polarisation u = (sin(-theta), cos(-theta)) is stored in a float32
    tensor (Transmission2D.py:112, :116);
  * the 2D TE point-dipole moment sqrt(I) * (0, 1) is a float32 tensor
    (Transmission2D.py:162).
"""
from __future__ import annotations

import numpy as np
import torch

from . import engine as E


def _angles(thetas, device):
    th = np.asarray(thetas, dtype=np.float64).reshape(-1)
    c, s = np.cos(-th), np.sin(-th)
    return torch.from_numpy(c).to(device), torch.from_numpy(s).to(device)


def source_2d(kind, source, points, k0, thetas, w):
    """generate_source of Transmission2D_vector (Transmission2D.py:93-174) and
    Transmission2D_scalar (:620-685).  points: (M, 2) float64 on the GPU."""
    dev = points.device
    M = points.shape[0]
    R = len(np.asarray(thetas).reshape(-1))
    if source is None:
        shape = (M, 2, R) if kind == "2d_vector" else (M, R)
        return torch.zeros(shape, dtype=torch.complex128, device=dev)
    if source not in ("beam", "plane", "point"):
        raise NotImplementedError
    c, s = _angles(thetas, dev)
    x, y = points[:, 0:1], points[:, 1:2]
    rpar = c[None, :] * x - s[None, :] * y     # (rot @ p)[0], rot = [[c, -s], [s, c]]
    rperp = s[None, :] * x + c[None, :] * y
    if source == "plane":
        E0 = torch.exp(1j * rpar * k0)
    elif source == "beam":
        a = 2 * rperp / (w * w * k0)
        E0 = torch.exp(1j * rpar * k0 - (rperp ** 2 / (w * w * (1 + 1j * a)))) / torch.sqrt(1 + 1j * a)
    else:
        return _point_source_2d(kind, points, k0, c, s)
    if kind == "2d_vector":
        u = torch.stack([s, c]).to(torch.float32).to(torch.float64)  # (2, R), float32-rounded
        E0 = E0.reshape(M, 1, R) * u
    return E0.to(torch.complex128)


def _point_source_2d(kind, points, k0, c, s):
    """Point dipole at distance 2 (Transmission2D.py:145-166, :662-677): the
    Green's function from (-2, 0) in the frame rotated by -theta."""
    dev = points.device
    M, R = points.shape[0], c.shape[0]
    dist = 2.0
    intensity = 1.0 * k0 * dist * 2.0 * np.pi
    loc = torch.tensor([[-dist, 0.0]], dtype=torch.float64, device=dev)
    x, y = points[:, 0], points[:, 1]
    out = torch.zeros((M, 2, R) if kind == "2d_vector" else (M, R), dtype=torch.complex128, device=dev)
    for t in range(R):
        rr = torch.stack([c[t] * x - s[t] * y, s[t] * x + c[t] * y], 1).contiguous()
        G = E.assemble_propagator(kind, rr, loc, k0)          # (d*M, d)
        if kind == "2d_vector":
            mom = float(np.float32(np.sqrt(intensity)))
            e = G.reshape(M, 2, 2)[:, :, 1] * mom               # G @ (0, mom)
            rot_t = torch.tensor([[c[t], s[t]], [-s[t], c[t]]], dtype=torch.complex128, device=dev)  # rot.T
            out[:, :, t] = (rot_t @ e.T).T
        else:
            out[:, t] = np.sqrt(intensity) * G.reshape(M)
    return out


def polarisation_vectors(p):
    """pvec rebuilt from p via (theta, phi) (Transmission3D.py:102-104): (3, R)."""
    phi = torch.atan2(p[:, 1], p[:, 0])
    th = torch.arccos(p[:, 2])
    return torch.stack([torch.sin(th) * torch.cos(phi), torch.sin(th) * torch.sin(phi), p[:, 2]])


def source_3d(kind, source, points, k0, u, p, w):
    """generate_source of Transmission3D_vector (Transmission3D.py:79-145) and
    Transmission3D_scalar (:603-658).  u, p: (R, 3) float64."""
    dev = points.device
    M = points.shape[0]
    u = torch.as_tensor(u).to(device=dev, dtype=torch.float64)
    R = u.shape[0]
    if source is None:
        return torch.zeros((M, u.shape[1], R) if kind == "3d_vector" else (M, u.shape[1]), dtype=torch.complex128,
                           device=dev)
    if source == "point":
        # both 3D point sources fail inside the reference (Transmission3D.py:136, :649)
        raise NotImplementedError("the 3D point source is not available in the reference implementation")
    if source not in ("beam", "plane"):
        raise NotImplementedError
    rpara = points @ u.T
    if source == "plane":
        E0 = torch.exp(1j * rpara * k0)
    else:
        rperp = torch.linalg.norm(points.reshape(-1, 3, 1) - rpara.reshape(M, 1, R) * u.T.reshape(1, 3, -1), dim=1)
        a = 2 * rperp / (w * w * k0)
        E0 = torch.exp(1j * rpara * k0 - (rperp ** 2 / (w * w * (1 + 1j * a)))) / torch.sqrt(1 + 1j * a)
    if kind == "3d_vector":
        pv = polarisation_vectors(torch.as_tensor(p).to(device=dev, dtype=torch.float64))
        E0 = E0.reshape(M, 1, -1) * pv.reshape(1, 3, -1)
    return E0.to(torch.complex128)
