"""Drop-in solver classes with the reference's Transmission2D/3D API.

``CoupledDipoleSolver`` holds the shared logic; the four public classes in
``Transmission2D.py`` / ``Transmission3D.py`` only fix the Green's-function
kind and the source signature.  Method names, argument meanings, output
shapes, dtypes (complex128) and the reference's edge-case behaviour are kept
(see each method's reference citation).  Inputs may be CPU or CUDA tensors
(or numpy arrays); the work runs on the GPU and results come back on the
device the caller's data came from, so the unmodified ``magreete.py`` driver
(which calls ``.numpy()`` on results) keeps working.

Engine options beyond the reference API (keyword-only, or environment):
  precision: "fp64" (plain method, default) or "mixed" (complex64 LU +
             double-float iterative refinement to ``tol``);
             env MAGREETE_PRECISION.
  verbose:   print the reference's progress lines (default off).
"""
from __future__ import annotations

import os

import numpy as np
import torch

from . import engine as E
from . import selfterm
from . import spectral as SP


def _as_tensor(x):
    if isinstance(x, torch.Tensor):
        return x
    return torch.as_tensor(np.asarray(x))


def _home_device(*xs):
    """Device results are returned on: CPU unless an input was a CUDA tensor."""
    for x in xs:
        if isinstance(x, torch.Tensor) and x.is_cuda:
            return x.device
    return torch.device("cpu")


def periodic_wrap(r, periodic, dim):
    """Separations r (..., dim) wrapped into [-1/2, 1/2) along the periodic
    axes, (r + 1/2) mod 1 - 1/2 with a floored modulo, as a new float64
    tensor (the reference edits its argument in place).  The 2D classes honour
    exactly one of 'x' / 'y' (Transmission2D.py:74-81, :605-612: an 'xy'
    string wraps nothing); the 3D classes wrap every axis named
    (Transmission3D.py:58-69, :584-595)."""
    r = _as_tensor(r).to(torch.float64).clone()
    if periodic:
        axes = {"x": 0, "y": 1, "z": 2}
        if dim == 2:
            sel = [axes[periodic]] if periodic in ("x", "y") else []
        else:
            sel = [axes[c] for c in "xyz" if c in periodic]
        for a in sel:
            r[..., a] = torch.remainder(r[..., a] + 0.5, 1.0) - 0.5
    return r


class CoupledDipoleSolver:
    kind = None  # "2d_vector" | "2d_scalar" | "3d_vector" | "3d_scalar"

    def __init__(self, points, source="beam", *, precision=None, verbose=False, tol=E.DEFAULT_TOL,
                 max_iter=E.DEFAULT_MAX_ITER, reference_rounding=True):
        dim, d = E.KIND_DIMS[self.kind]
        self.dim, self.d = dim, d
        self.r = _as_tensor(points).reshape(-1, dim)
        self.N = self.r.shape[0]
        self.source = source
        self.precision = precision or os.environ.get("MAGREETE_PRECISION", "fp64")
        if self.precision not in ("fp64", "mixed"):
            raise ValueError(f"precision must be 'fp64' or 'mixed', not {self.precision!r}")
        self.verbose = verbose
        self.tol, self.max_iter = tol, max_iter
        self.reference_rounding = reference_rounding
        self.last_stats = {}
        self._dev = E.device_of(self.r)
        self._r_dev = E.points_to(self.r, self._dev, dim)

    # ------------------------------------------------------------ helpers
    def _say(self, msg):
        if self.verbose:
            print(msg)

    def _k_label(self, k0):
        return str(np.round(k0 / (2.0 * np.pi), 1))

    def _pts(self, points):
        return E.points_to(points, self._dev, self.dim)

    def _shift(self, k0, alpha, radius, self_interaction, si_type):
        return selfterm.diagonal_shift(self.kind, k0, alpha, radius, self_interaction, si_type,
                                       self.reference_rounding)

    def _factorization(self, k0, alpha, radius, self_interaction, si_type):
        return E.SystemFactorization(self.kind, self._r_dev, k0, alpha * k0 * k0,
                                     self._shift(k0, alpha, radius, self_interaction, si_type),
                                     self.precision, self.tol, self.max_iter)

    # ------------------------------------------------------------ Green's functions
    def _greens_of_separations(self, r, k0, periodic="", regularize=False, radius=0.0):
        """Green's tensor for an array of separations r (..., dim)."""
        r = periodic_wrap(r, periodic, self.dim)
        lead = r.shape[:-1]
        seps = E.points_to(r, self._dev, self.dim)
        origin = torch.zeros((1, self.dim), dtype=torch.float64, device=self._dev)
        G = E.assemble_propagator(self.kind, seps, origin, k0, 1.0, regularize, radius)
        G = G.reshape(*lead, self.d, self.d) if self.d > 1 else G.reshape(*lead)
        return G.to(_home_device(r))

    def _G0_dense(self, points, k0, print_statement="", regularize=False, radius=0.0, zero_self=None):
        """Dense propagator between `points` (None: the scatterers) and the
        scatterers, shape (d*M, d*N) complex128 (G0_vector / G0)."""
        self._say(f"Calculating Green's function at k0L/2pi = {self._k_label(k0)} ({print_statement})")
        tg = self._r_dev if points is None else self._pts(points)
        if tg.shape[0] == 0:
            # no target points: an empty (0, d*N) propagator, as the reference's
            return torch.zeros((0, self.d * self.N), dtype=torch.complex128, device=_home_device(points, self.r))
        G = E.assemble_propagator(self.kind, tg, self._r_dev, k0, 1.0, regularize, radius)
        if zero_self is None:
            zero_self = points is None
        if zero_self:
            d = self.d
            idx = torch.arange(self.N, device=self._dev)
            Gv = G.view(self.N, d, self.N, d)
            Gv[idx, :, idx, :] = 0
        return G.to(_home_device(points, self.r))

    # ------------------------------------------------------------ solve
    def solve(self, k0, alpha, radius, E0, self_interaction=True, self_interaction_type="Rayleigh"):
        """Fields at the scatterers: (I - k^2 alpha G) Ek = E0, Transmission2D.py:207-231 / :718-744,
        Transmission3D.py:181-206 / :693-718.  Returns (d*N, R) complex128 (or (N,) for a 1-D
        scalar source)."""
        selfterm.SELF_TERM[self.kind](k0, radius, self_interaction_type)  # NotImplementedError as the reference
        self._say(f"Calculating Green's function at k0L/2pi = {self._k_label(k0)} (solve)")
        home = _home_device(E0, self.r)
        E0t = _as_tensor(E0)
        flat = E0t.dim() == 1
        B = E0t.reshape(self.d * self.N, -1).to(device=self._dev, dtype=torch.complex128).contiguous()
        if B.shape[1] == 0:
            # no incident fields: the reference's solve returns an empty (d*N, 0) tensor
            self.last_stats = {}
            return torch.zeros((self.d * self.N, 0), dtype=torch.complex128, device=home)
        stats = {}
        X = E.solve_system(self.kind, self._r_dev, k0, alpha * k0 * k0,
                           self._shift(k0, alpha, radius, self_interaction, self_interaction_type), B,
                           self.precision, self.tol, self.max_iter, stats)
        self.last_stats = stats
        if flat:
            X = X.reshape(-1)
        return X.to(home)

    # ------------------------------------------------------------ propagate
    def _propagate_common(self, points, k0, alpha, src_field, E0_meas, regularize, radius, ss):
        home = _home_device(points, src_field, E0_meas, self.r)
        pts_t = _as_tensor(points).reshape(-1, self.dim).to(torch.float64)
        det = self._pts(pts_t)
        M, d = det.shape[0], self.d
        src = _as_tensor(src_field).to(device=self._dev, dtype=torch.complex128)
        flat = src.dim() == 1 and d == 1
        src2 = src.reshape(d * self.N, -1)
        R = src2.shape[1]
        E0d = _as_tensor(E0_meas).to(device=self._dev, dtype=torch.complex128)
        out = E.propagate(self.kind, det, self._r_dev, k0, alpha * k0 * k0, src2, E0d.reshape(d * M, R),
                          regularize, radius, self.precision)
        out = out.reshape(M, d, R) if d > 1 else out.reshape(M, R)
        flag = out[:, 0, 0] if d > 1 else out[:, 0]
        bad = torch.nonzero(torch.isnan(flag)).reshape(-1)
        if bad.numel():
            self._fix_rows(out, bad.tolist(), pts_t, src2, E0d, regularize, radius, ss)
        if flat:
            out = out.reshape(M)
        return out.to(home)

    def _fix_rows(self, out, rows, pts, src2, E0d, regularize, radius, ss):
        """Detectors that coincide with (or, regularised, lie within `radius` of) a
        scatterer take a field from that scatterer: Transmission2D.py:192-203,
        :703-714, :248-259; Transmission3D.py:165-177, :677-689, :225-236.
        QUIRKS kept: the 2D TE propagate() indexes the (2N, R) field by the
        scatterer index and broadcasts it to both components; propagate_ss()
        indexes E0_meas by the scatterer index."""
        r = self.r.to(torch.float64).cpu()
        for j in rows:
            p = pts[j].cpu()
            dist = torch.linalg.norm(r - p, dim=-1)
            if regularize:
                cand = torch.nonzero(dist <= radius).reshape(-1)
                idx = int(torch.argmin(dist)) if cand.numel() > 1 else int(cand[0])
            else:
                idx = int(torch.nonzero(torch.all(r - p == 0, dim=-1)).reshape(-1)[0])
            if ss:
                out[j] = E0d[idx]
            elif self.kind == "3d_vector":
                out[j] = src2.reshape(self.N, 3, -1)[idx]
            else:
                out[j] = src2[idx]   # 2D TE: row idx of the (2N, R) array (reference quirk)

    def propagate(self, points, Ek, k0, alpha, E0, regularize=False, radius=0.0):
        """E = k^2 alpha G0(points) Ek + E0 (Transmission2D.py:176-205, :687-716;
        Transmission3D.py:147-179, :660-691).  Matrix-free on the GPU."""
        self._say(f"Calculating Green's function at k0L/2pi = {self._k_label(k0)} (propagate)")
        return self._propagate_common(points, k0, alpha, Ek, E0, regularize, radius, False)

    def propagate_ss(self, points, k0, alpha, E0_meas, E0_scat, regularize=False, radius=0.0):
        """Single-scattering field (Transmission2D.py:233-261, :746-775;
        Transmission3D.py:208-238, :720-749).  E0_scat may be (N, d, R) or
        (d*N, R)."""
        self._say(f"Calculating Green's function at k0L/2pi = {self._k_label(k0)} (propagate_ss)")
        return self._propagate_common(points, k0, alpha, E0_scat, E0_meas, regularize, radius, True)

    # ------------------------------------------------------------ DOS
    _DOS_PREF = {"2d_vector": lambda k0, a: 4.0 * k0 * k0 * a, "2d_scalar": lambda k0, a: 4.0 * k0 * k0 * a,
                 "3d_vector": lambda k0, a: 2.0 * np.pi * k0 * a, "3d_scalar": lambda k0, a: 4.0 * np.pi * k0 * a}

    def _dos_terms(self, fac, measure_points, k0, radius, self_interaction, si_type, regularize):
        """Per-row g_i M^-1 g_i^T for the rows g_i of G0(measure_points):
        solve M Y = Gm^T (LU solve with d*P right-hand sides) and take the
        column dots of Gm^T and Y.  Same value as the reference's
        sum((Gm^T Gm) * inverse(M)) / diag(Gm W Gm^T), without forming the inverse."""
        mp = self._pts(measure_points)
        fill = selfterm.self_over_volume(self.kind, k0, radius, si_type) if self_interaction else 0j
        GmT = E.assemble_propagator(self.kind, mp, self._r_dev, k0, 1.0, regularize, radius, nan_fill=fill,
                                    transpose=True)
        Y = fac.solve(GmT)
        return E.column_dots(GmT, Y)

    def mean_DOS_measurements(self, measure_points, k0, alpha, radius, self_interaction=True,
                              self_interaction_type="Rayleigh", regularize=False, discard_absorption=False):
        """Mean DOS over measurement points (Transmission2D.py:282-336, :787-841;
        Transmission3D.py:270-323, :779-832).  Returns a 0-d float64 tensor."""
        P = _as_tensor(measure_points).reshape(-1, self.dim).shape[0]
        self._say(f"Computing mean DOS using {P} points at k0L/2pi = {self._k_label(k0)}")
        if P == 0:
            # the reference averages over no points: 0 / 0 = nan
            selfterm.SELF_TERM[self.kind](k0, radius, self_interaction_type)
            return torch.tensor(float("nan"), dtype=torch.float64, device=_home_device(measure_points, self.r))
        fac = self._factorization(k0, alpha, radius, self_interaction, self_interaction_type)
        dots = self._dos_terms(fac, measure_points, k0, radius, self_interaction, self_interaction_type, regularize)
        total = dots.sum() / P
        a = np.real(alpha) if discard_absorption else alpha
        val = torch.imag(total * complex(self._DOS_PREF[self.kind](k0, a)))
        return val.to(_home_device(measure_points, self.r))

    def _ldos_from_dots(self, dots, P, k0, alpha, discard_absorption):
        """Shapes as the reference: (P, 1) for the vector kinds (reshape(M, d, -1).sum(1),
        Transmission2D.py:387-388), (P,) for the scalar kinds."""
        a = np.real(alpha) if discard_absorption else alpha
        v = torch.imag(dots * complex(self._DOS_PREF[self.kind](k0, a)))
        return v.reshape(P, self.d, -1).sum(1) if self.d > 1 else v

    def LDOS_measurements(self, measure_points, k0, alpha, radius, self_interaction=True,
                          self_interaction_type="Rayleigh", regularize=False, discard_absorption=False):
        """LDOS at each measurement point (Transmission2D.py:338-390, :843-890;
        Transmission3D.py:325-376, :834-886)."""
        P = _as_tensor(measure_points).reshape(-1, self.dim).shape[0]
        if P == 0:
            # the reference fails reshaping an empty propagator (a RuntimeError)
            raise RuntimeError("LDOS_measurements needs at least one measurement point")
        fac = self._factorization(k0, alpha, radius, self_interaction, self_interaction_type)
        dots = self._dos_terms(fac, measure_points, k0, radius, self_interaction, self_interaction_type, regularize)
        return self._ldos_from_dots(dots, P, k0, alpha, discard_absorption).to(_home_device(measure_points, self.r))

    def batch_LDOS_measurements(self, batches, k0, alpha, radius, self_interaction=True,
                                self_interaction_type="Rayleigh", regularize=False, discard_absorption=False):
        """LDOS over batches of points with one factorisation (Transmission2D.py:392-453;
        Transmission3D.py:379-439)."""
        fac = self._factorization(k0, alpha, radius, self_interaction, self_interaction_type)
        outs = []
        for b in range(len(batches)):
            self._say("Batch " + str(b + 1))
            pts = batches[b]
            P = _as_tensor(pts).reshape(-1, self.dim).shape[0]
            dots = self._dos_terms(fac, pts, k0, radius, self_interaction, self_interaction_type, regularize)
            outs.append(self._ldos_from_dots(dots, P, k0, alpha, discard_absorption))
        return torch.cat(outs).to(_home_device(batches[0] if len(batches) else None, self.r))

    # ------------------------------------------------------------ spectral tools
    # Dense non-Hermitian eigenproblems: the Green's matrix from the GPU
    # assembly, LAPACK's eigensolver on the host as in the reference
    # (spectral.py).  Results are returned on the device of the points.  The
    # reference's plots of compute_eigenmodes_IPR (utils.plot_IPR_damping_values)
    # are not drawn: no plotting library is part of this engine.
    def _spectral_system(self, k0, alpha, radius, self_interaction, si_type):
        G = self._G0_dense(None, k0, "DOS eigvals")
        return SP.system_matrix(G, k0, alpha, self._shift(k0, alpha, radius, self_interaction, si_type))

    def compute_hamiltonian_DOS(self, k0, deltas, file_name, write_eigenvalues=True):
        """DOS of the near-resonant Hamiltonian built from the scatterer Green's
        matrix, at the detunings `deltas` (Transmission2D.py:455-477, :955-977;
        Transmission3D.py:442-464, :951-973).  Writes the eigenvalues to
        <file_name>_hamiltonian_lambdas_<k0L/2pi>_vector.csv (the name every
        reference class uses)."""
        k0_ = self._k_label(k0)
        self._say(f"Computing Hamiltonian DOS od {self.N} points at k0L/2pi = {k0_}")
        dos, lambdas = SP.hamiltonian_dos(self.kind, self._G0_dense(None, k0, "Hamiltonian DOS"), k0, deltas)
        if write_eigenvalues:
            np.savetxt(file_name + "_hamiltonian_lambdas_" + k0_ + "_vector.csv",
                       np.stack([lambdas.real.numpy(), lambdas.imag.numpy()]).T)
        return dos.to(_home_device(self.r))

    def compute_eigenvalues_and_scatterer_LDOS(self, k0, alpha, radius, file_name, self_interaction=True,
                                               self_interaction_type="Rayleigh", write_eigenvalues=True):
        """The LDOS at the scatterers from the eigenvalues d of the system
        matrix, Im(c sum((1 - d)^2 / d) / N) (Transmission2D.py:479-515,
        :979-1015; Transmission3D.py:466-501, :975-1009).  Writes the
        eigenvalues to <file_name>_deltas_<k0L/2pi>[_vector|_scalar].csv as the
        reference names them."""
        k0_ = self._k_label(k0)
        self._say(f"Computing spectrum and scatterer LDOS using {self.N} points at k0L/2pi = {k0_}")
        M = self._spectral_system(k0, alpha, radius, self_interaction, self_interaction_type)
        factor, deltas = SP.scatterer_ldos_factor(self.kind, M, self.N, k0, alpha)
        if write_eigenvalues:
            suffix = {"2d_vector": "_vector.csv", "2d_scalar": "_scalar.csv"}.get(self.kind, ".csv")
            np.savetxt(file_name + "_deltas_" + k0_ + suffix, np.stack([deltas.real.numpy(), deltas.imag.numpy()]).T)
        return factor.to(_home_device(self.r))

    def compute_eigenmodes_IPR(self, k0, alpha, radius, file_name, self_interaction=True,
                               self_interaction_type="Rayleigh", number_eigenmodes=1, write_eigenvalues=True,
                               sorting_type="IPR"):
        """Eigenmodes of the system matrix with their inverse participation
        ratios, sorted by IPR or by damping (Transmission2D.py:517-569,
        :1017-1060; Transmission3D.py:503-564, :1011-1070).  Returns (values,
        the first number_eigenmodes eigenvectors, IPRs); the unsorted values
        and IPRs go to <file_name>_deltas_<k0L/2pi>.csv (2D) or
        <file_name>_lambdas_<k0L/2pi>.csv (3D)."""
        k0_ = self._k_label(k0)
        self._say(f"Computing spectrum and scatterer LDOS using {self.N} points at k0L/2pi = {k0_}")
        M = self._spectral_system(k0, alpha, radius, self_interaction, self_interaction_type)
        values, vectors, iprs = SP.eigenmodes(self.kind, M, k0, alpha, radius)
        if write_eigenvalues:
            name = "_deltas_" if self.kind.startswith("2d") else "_lambdas_"
            np.savetxt(file_name + name + k0_ + ".csv",
                       np.stack([values.real.numpy(), values.imag.numpy(), iprs.numpy()]).T)
        values, vectors, iprs = SP.sort_modes(values, vectors, iprs, sorting_type)
        if self.kind.startswith("3d"):
            self._say(str(SP.mean_resonance_ratio(self.kind, values, k0, alpha, radius)))
        home = _home_device(self.r)
        return values.to(home), vectors[:, 0:number_eigenmodes].to(home), iprs.to(home)
