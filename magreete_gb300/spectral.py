"""Spectral tools of the solver classes: the eigenvalues of the scatterer
Green's matrix and of the system matrix, and what the reference derives from
them (compute_hamiltonian_DOS, compute_eigenvalues_and_scatterer_LDOS,
compute_eigenmodes_IPR; Transmission2D.py:455-569, :955-1060;
Transmission3D.py:442-564, :951-1070).

These are dense non-Hermitian eigenproblems.  The Green's matrix comes from
the GPU assembly (the classes' G0 / G0_vector); the eigensolver is LAPACK's,
on the host, as in the reference (torch.linalg.eigvals / eig on complex128).
The functions below take that matrix and return what the reference's methods
return, with its per-class constants and in its order of operations; the
classes add the file output.
"""
import numpy as np
import torch


def _host(G):
    return G.detach().to(device="cpu", dtype=torch.complex128)


def hamiltonian_matrix(kind, G, k0):
    """The near-resonant Hamiltonian of the Green's matrix G (scatterer pairs):
    c G with zero diagonal, c = 8 (2D TE), 4 (2D TM), 6 pi / k0 (3D vector),
    4 pi / k0 (3D scalar) (Transmission2D.py:466, :966; Transmission3D.py:453,
    :962)."""
    G = _host(G)
    if kind == "2d_vector":
        H = 8 * G
    elif kind == "2d_scalar":
        H = 4 * G
    elif kind == "3d_vector":
        H = 6 * np.pi * G / k0
    else:
        H = 4 * np.pi * G / k0
    H.fill_diagonal_(0)
    return H


def hamiltonian_dos(kind, G, k0, deltas):
    """DOS of the resolvent at deltas - 1j from the eigenvalues of the
    Hamiltonian (Transmission2D.py:468-477).  Returns (dos, eigenvalues)."""
    lambdas = torch.linalg.eigvals(hamiltonian_matrix(kind, G, k0))
    resonance = torch.as_tensor(deltas).detach().cpu() - 1j
    resolvant = torch.mean(1 / (resonance.reshape(-1, 1) - lambdas.reshape(1, -1)), dim=-1)
    return torch.imag(resolvant) / np.pi, lambdas


def system_matrix(G, k0, alpha, shift):
    """M = I - k^2 alpha G with diagonal 1 - shift, as the spectral methods
    build it (Transmission2D.py:497-503): `shift` is the self-interaction term
    k^2 alpha S / V rounded as the reference rounds it (selfterm.diagonal_shift),
    0 without self-interaction."""
    M = -alpha * k0 * k0 * _host(G)
    M.fill_diagonal_(1)
    if shift != 0:
        M.diagonal().sub_(shift)
    return M


def scatterer_ldos_factor(kind, M, n_points, k0, alpha):
    """Im of the trace term sum((1 - d)^2 / d) / N over the eigenvalues d of M,
    times 4 / (k^2 alpha) (2D), 2 pi / (k^3 alpha) (3D vector) or
    4 pi / (k^3 alpha) (3D scalar) (Transmission2D.py:505-515;
    Transmission3D.py:491-501, :1001-1009).  Returns (factor, eigenvalues)."""
    deltas = torch.linalg.eigvals(M)
    f = ((1 - deltas) ** 2 / deltas).sum() / n_points
    if kind.startswith("2d"):
        f *= 4.0 / (k0 ** 2 * alpha)
    elif kind == "3d_vector":
        f *= 2.0 * np.pi / (k0 ** 3 * alpha)
    else:
        f *= 4.0 * np.pi / (k0 ** 3 * alpha)
    return torch.imag(f), deltas


def mode_constants(kind, alpha, radius):
    """(kares, gamma0, scale, volume) of the 3D classes' dimensionless
    eigenvalues (Transmission3D.py:517-522, :1027-1032)."""
    volume = 4 * np.pi * (radius ** 3) / 3
    if kind == "3d_vector":
        kares = np.sqrt(1.0 + 3.0 / np.real(alpha / volume))
        gamma0 = (2.0 / 9.0) * (1 + 3.0 / np.real(alpha / volume))
        return kares, gamma0, 6.0, volume
    kares = np.sqrt(2.0 / np.real(alpha / volume))
    gamma0 = 4.0 / (3.0 * np.real(alpha / volume))
    return kares, gamma0, 4.0, volume


def eigenmodes(kind, M, k0, alpha, radius):
    """Eigenmodes of M with their inverse participation ratios
    sum |v|^4 / (sum |v|^2)^2 (Transmission2D.py:536-537).  The eigenvalues
    are returned as 1 - k^2 alpha d (2D, Transmission2D.py:540) or, in 3D, as
    (1 - d) / (k^2 alpha) made dimensionless with the resonance constants
    (Monsarrat's form, Transmission3D.py:515-525).  Returns (values, vectors,
    IPRs), unsorted."""
    deltas, vectors = torch.linalg.eig(M)
    iprs = torch.sum(torch.abs(vectors ** 4), dim=0) / (torch.sum(torch.abs(vectors ** 2), dim=0)) ** 2
    if kind.startswith("2d"):
        values = 1.0 - k0 ** 2 * alpha * deltas
    else:
        kares, gamma0, scale, volume = mode_constants(kind, alpha, radius)
        lambdas = (1.0 - deltas) / (k0 ** 2 * alpha)
        values = scale * volume * k0 ** 2 * lambdas / (kares * gamma0)
    return values, vectors, iprs


def sort_modes(values, vectors, iprs, sorting_type="IPR"):
    """Largest IPR first ('IPR') or smallest damping Im(value) first
    ('damping'); anything else raises NotImplementedError, as the reference
    (Transmission2D.py:548-560)."""
    if sorting_type == "IPR":
        iprs, order = torch.sort(iprs, descending=True)
        return values[order], vectors[:, order], iprs
    if sorting_type == "damping":
        order = torch.argsort(torch.imag(values), descending=False)
        return values[order], vectors[:, order], iprs[order]
    raise NotImplementedError


def mean_resonance_ratio(kind, values, k0, alpha, radius):
    """The 3D classes' printed diagnostic mean((g/2) / ((k a - w)^2 + (g/2)^2)) / pi
    with g = gamma0 Im(l) / 2, w = kares - gamma0 Re(l) / 2 over the
    dimensionless eigenvalues l (Transmission3D.py:551-554)."""
    kares, gamma0, _, _ = mode_constants(kind, alpha, radius)
    gamman = gamma0 * np.imag(values.numpy()) / 2
    omegan = kares - gamma0 * np.real(values.numpy()) / 2
    ratio = (gamman / 2) / ((k0 * radius - omegan) ** 2 + (gamman / 2) ** 2)
    return float(np.mean(ratio) / np.pi)
