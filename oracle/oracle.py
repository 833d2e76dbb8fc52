"""CPU oracle for the coupled-dipole solve path -- TEST INFRASTRUCTURE ONLY.

This module restates, in plain numpy/scipy float64 / complex128 arithmetic, the
reference MAGreeTe functions that make up the accelerated path.  It exists so
that tests, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` have an independent CPU answer to check the CUDA path against.
Nothing in the ``magreete_gb300`` package imports it, and the product path
never calls it.

Each function names the reference file:line it follows (paths relative to the
MAGreeTe project root).  Reference quirks are reproduced on purpose and are
marked ``QUIRK``; the CUDA path mirrors the same behaviour.

Parity of this restatement is pinned against outputs of the reference itself
(``tests/golden/*.npz``, produced by ``tests/golden/make_golden.py`` which
imports the unmodified reference classes).

Layout conventions (same as the reference):
  * points are (N, d) float64, d = 2 or 3;
  * the interaction matrix is (dN, dN) with row/column index ``d*i + a``
    (``Transmission2D.py:279``, ``Transmission3D.py:267``);
  * fields at scatterers are (dN, R) complex128, detector fields (M, d, R)
    for vector kinds and (M, R) for scalar kinds.
"""
from __future__ import annotations

import concurrent.futures as _cf
import os

import numpy as np
import scipy.special as sps

EULER_GAMMA = np.euler_gamma

KINDS = ("2d_vector", "2d_scalar", "3d_vector", "3d_scalar")


def kind_dims(kind):
    """(spatial dimension, field components per scatterer) for a kind."""
    return {"2d_vector": (2, 2), "2d_scalar": (2, 1),
            "3d_vector": (3, 3), "3d_scalar": (3, 1)}[kind]


# ---------------------------------------------------------------------------
# self-interaction integrals
# ---------------------------------------------------------------------------

def self_interaction_2d_scalar(k0, radius, kind="Rayleigh"):
    """Transmission2D.py:12-23 (TM self term S; the matrix uses S / (pi a^2))."""
    volume = np.pi * radius ** 2
    if kind == "full":
        return -1.0 / (k0 * k0) + 0.5j * volume * sps.hankel1(1, k0 * radius) / (k0 * radius)
    if kind == "Rayleigh":
        return (-radius ** 2 / 4.0) * (2.0 * EULER_GAMMA - 1.0 + 2.0 * np.log(k0 * radius / 2.0) - 1j * np.pi)
    raise NotImplementedError


def self_interaction_2d_vector(k0, radius, kind="Rayleigh"):
    """Transmission2D.py:25-36 (TE self term)."""
    volume = np.pi * radius ** 2
    if kind == "full":
        return -1.0 / (k0 * k0) + 0.25j * volume * sps.hankel1(1, k0 * radius) / (k0 * radius)
    if kind == "Rayleigh":
        return (-1.0 / (2.0 * k0 * k0)
                - (radius ** 2 / 8.0) * (2.0 * EULER_GAMMA - 1.0 + 2.0 * np.log(k0 * radius / 2.0) - 1j * np.pi))
    raise NotImplementedError


def self_interaction_3d_vector(k0, radius, kind="Rayleigh"):
    """Transmission3D.py:13-24."""
    volume = 4.0 * np.pi * radius ** 3 / 3.0
    if kind == "full":
        return (1.0 / k0 ** 2) * ((2.0 / 3.0) * np.exp(1j * k0 * radius) * (1 - 1j * k0 * radius) - 1.0)
    if kind == "Rayleigh":
        return -1.0 / (3.0 * k0 ** 2) + radius ** 2 / 3.0 + 1j * k0 * volume / (6.0 * np.pi)
    raise NotImplementedError


def self_interaction_3d_scalar(k0, radius, kind="Rayleigh"):
    """Transmission3D.py:26-37."""
    volume = 4.0 * np.pi * radius ** 3 / 3.0
    if kind == "full":
        return (1.0 / k0 ** 2) * (np.exp(1j * k0 * radius) * (1 - 1j * k0 * radius) - 1.0)
    if kind == "Rayleigh":
        return radius ** 2 / 2.0 + 1j * k0 * volume / (4.0 * np.pi)
    raise NotImplementedError


def scatterer_volume(kind, radius):
    """Disk area in 2D (Transmission2D.py:226), ball volume in 3D (Transmission3D.py:202)."""
    if kind.startswith("2d"):
        return np.pi * radius * radius
    return 4.0 * np.pi * radius ** 3 / 3.0


def self_term_over_volume(kind, k0, radius, si_type="Rayleigh"):
    """S/V, the diagonal correction used by solve() and mean_DOS_measurements()."""
    f = {"2d_vector": self_interaction_2d_vector, "2d_scalar": self_interaction_2d_scalar,
         "3d_vector": self_interaction_3d_vector, "3d_scalar": self_interaction_3d_scalar}[kind]
    return complex(f(k0, radius, si_type)) / scatterer_volume(kind, radius)


# ---------------------------------------------------------------------------
# Green's functions (pairwise, dense)
# ---------------------------------------------------------------------------

# Which Bessel-function implementation the 2D Green's functions use.
#   "exact": scipy.special j0/y0/j1/y1 (Cephes double precision, ~1e-15).
#   "torch": torch.special.bessel_{j0,y0,j1,y1}, the calls the reference makes
#            (Transmission2D.py:54-59).  In torch 2.x these are accurate to
#            only ~2.4e-6 (relative to the sqrt(2/(pi x)) envelope) for
#            5 <= x <= 10, and ~1e-9 up to x = 25: the large-argument branch
#            evaluates its Q denominator with the leading coefficient of a
#            monic polynomial dropped.  This mode reproduces the reference's
#            own numbers; "exact" is the FP64 oracle the GPU path is held to.
BESSEL_MODE = "exact"


def _hankel1_01(x):
    """H0(x), H1(x) = J + iY, as in torch_hankel1 (Transmission2D.py:46-61)."""
    with np.errstate(all="ignore"):
        if BESSEL_MODE == "torch":
            import torch
            t = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64))
            j0, y0 = torch.special.bessel_j0(t).numpy(), torch.special.bessel_y0(t).numpy()
            j1, y1 = torch.special.bessel_j1(t).numpy(), torch.special.bessel_y1(t).numpy()
        else:
            j0, y0, j1, y1 = sps.j0(x), sps.y0(x), sps.j1(x), sps.y1(x)
        return j0 + 1j * y0, j1 + 1j * y1


def greens_2d_vector(r, k0, regularize=False, radius=0.0):
    """TE dyadic Green's function, Transmission2D.py:63-91.

    r: (M, N, 2) separations.  Returns (M, N, 2, 2) complex128.
    QUIRK (Transmission2D.py:86-89): ``regularize`` compares k*R with radius.
    At R == 0 every entry of the block is NaN (0/0 in R^R/R^2)."""
    with np.errstate(all="ignore"):
        R = np.sqrt(np.sum(r * r, axis=-1))
        RxR = r[..., :, None] * r[..., None, :] / (R * R)[..., None, None]
        kR = R * k0
        if regularize:
            kR = np.where(kR < radius, 0.0, kR)
        h0, h1 = _hankel1_01(kR)
        I2 = np.eye(2)
        return 0.25j * ((I2 - RxR) * h0[..., None, None] - (I2 - 2 * RxR) * (h1 / kR)[..., None, None])


def greens_2d_scalar(r, k0, regularize=False, radius=0.0):
    """TM scalar Green's function (i/4) H0(kR), Transmission2D.py:595-618.
    ``regularize`` compares the distance R with radius (:615-616)."""
    with np.errstate(all="ignore"):
        R = np.sqrt(np.sum(r * r, axis=-1))
        if regularize:
            R = np.where(R < radius, 0.0, R)
        h0, _ = _hankel1_01(R * k0)
        return 0.25j * h0


def greens_3d_vector(r, k0, regularize=False, radius=0.0):
    """3D dyadic Green's function, Transmission3D.py:47-77:
    [I - R^R - (I - 3 R^R)(1/(ikR) + 1/(kR)^2)] e^{ikR} / (4 pi R)."""
    with np.errstate(all="ignore"):
        R = np.sqrt(np.sum(r * r, axis=-1))[..., None, None]
        RxR = r[..., :, None] * r[..., None, :] / (R * R)
        if regularize:
            R = np.where(R < radius, 0.0, R)
        I3 = np.eye(3)
        kR = k0 * R
        return (I3 - RxR - (I3 - 3 * RxR) * (1.0 / (1j * kR) + kR ** -2.0)) * np.exp(1j * kR) / (4 * np.pi * R)


def greens_3d_scalar(r, k0, regularize=False, radius=0.0):
    """3D scalar Green's function e^{ikR}/(4 pi R), Transmission3D.py:573-601."""
    with np.errstate(all="ignore"):
        R = np.sqrt(np.sum(r * r, axis=-1))
        if regularize:
            R = np.where(R < radius, 0.0, R)
        return np.exp(1j * k0 * R) / (4 * np.pi * R)


_GREENS = {"2d_vector": greens_2d_vector, "2d_scalar": greens_2d_scalar,
           "3d_vector": greens_3d_vector, "3d_scalar": greens_3d_scalar}


def periodic_wrap(kind, r, periodic=""):
    """Minimum-image wrap of separations into [-1/2, 1/2) along the periodic
    axes: (r + 1/2) mod 1 - 1/2 with a floored modulo.
    QUIRK: the 2D classes honour exactly periodic == 'x' or 'y' (an 'xy'
    string wraps nothing, Transmission2D.py:74-81, :605-612); the 3D classes
    wrap every axis named in the string (Transmission3D.py:58-69, :584-595).
    Returns a new array (the reference edits its argument in place)."""
    r = np.array(r, dtype=np.float64, copy=True)
    dim, _ = kind_dims(kind)
    axes = ([{"x": 0, "y": 1}[periodic]] if periodic in ("x", "y") else []) if dim == 2 else \
        [a for a, c in enumerate("xyz") if c in periodic]
    for a in axes:
        r[..., a] = np.mod(r[..., a] + 0.5, 1.0) - 0.5
    return r


def greens_separations(kind, r, k0, periodic="", regularize=False, radius=0.0):
    """torch_greens / greens of the solver classes on an array of separations
    (Transmission2D.py:63-91, :595-618; Transmission3D.py:47-77, :573-601):
    the periodic wrap, then the kind's Green's function."""
    return _GREENS[kind](periodic_wrap(kind, r, periodic), k0, regularize=regularize, radius=radius)


# Row blocks of the dense Green's tensor are evaluated on all host threads
# (numpy releases the GIL inside its elementwise loops), as the reference's
# torch operations use every intra-op thread.  Each entry is computed by the
# same elementwise expression either way, so the result does not depend on
# the split.
THREADS = os.cpu_count() or 1


def _greens_rows(kind, P, scat, k0, regularize, radius):
    M = P.shape[0]
    f = _GREENS[kind]
    if THREADS <= 1 or M * scat.shape[0] < 1 << 18:
        return f(P[:, None, :] - scat[None, :, :], k0, regularize=regularize, radius=radius)
    step = -(-M // (4 * THREADS))
    blocks = [(a, min(M, a + step)) for a in range(0, M, step)]
    first = f(P[:1, None, :] - scat[None, :, :], k0, regularize=regularize, radius=radius)
    out = np.empty((M,) + first.shape[1:], first.dtype)

    def one(ab):
        a, b = ab
        out[a:b] = f(P[a:b, None, :] - scat[None, :, :], k0, regularize=regularize, radius=radius)

    with _cf.ThreadPoolExecutor(THREADS) as ex:
        list(ex.map(one, blocks))
    return out


def G0(kind, scat, k0, points=None, regularize=False, radius=0.0):
    """Dense propagator matrix, following G0_vector (Transmission2D.py:263-280),
    G0 (Transmission2D.py:777-785), G0 (Transmission3D.py:240-268, 751-777).

    points=None means scatterer-scatterer, with the self pairs set to zero
    (the reference's Python loop, Transmission2D.py:277-278).  QUIRK: the 2D
    scalar class never zeroes its self pairs (it is called with points=self.r,
    Transmission2D.py:733); its diagonal is overwritten by fill_diagonal_ in
    solve(), so the value there does not matter for the system matrix.
    Returns (d*M, d*N) complex128 with index d*i + a.
    """
    dim, d = kind_dims(kind)
    self_pairs = points is None
    P = scat if self_pairs else points
    g = _greens_rows(kind, P, scat, k0, regularize, radius)
    M, N = P.shape[0], scat.shape[0]
    if self_pairs and kind != "2d_scalar":
        idx = np.arange(N)
        g[idx, idx] = 0
    if d == 1:
        return g.astype(np.complex128)
    return np.transpose(g, (0, 2, 1, 3)).reshape(d * M, d * N).astype(np.complex128)


def system_matrix(kind, scat, k0, alpha, radius, self_interaction=True, si_type="Rayleigh"):
    """M = I - k^2 alpha G with diagonal 1 - k^2 alpha S/V, as built inside
    solve() (Transmission2D.py:222-228, 733-739; Transmission3D.py:197-203, 709-715)."""
    G = G0(kind, scat, k0)
    Mt = -alpha * k0 * k0 * G
    np.fill_diagonal(Mt, 1.0)
    if self_interaction:
        Mt[np.diag_indices_from(Mt)] -= diagonal_self_shift(kind, k0, alpha, radius, si_type)
    return Mt


def diagonal_self_shift(kind, k0, alpha, radius, si_type="Rayleigh"):
    """k^2 alpha S/V as the reference subtracts it from the diagonal.

    QUIRK (Transmission2D.py:228, :739; Transmission3D.py:203, :715): the
    scalar is multiplied by ``torch.eye(dims)``, whose default dtype is
    float32, so the product is a complex64 tensor: the shift is rounded to
    single precision (real and imaginary parts separately) before it is
    subtracted from the complex128 matrix."""
    s = complex(alpha * k0 * k0 * self_term_over_volume(kind, k0, radius, si_type))
    return complex(np.complex64(s))


# ---------------------------------------------------------------------------
# sources
# ---------------------------------------------------------------------------

def source_2d(kind, source, points, k0, thetas, w):
    """generate_source for the 2D classes: Transmission2D.py:93-174 (TE) and
    :620-685 (TM).  Plane and Gaussian-beam sources; 'point' and None too.
    Returns (M, 2, R) for TE and (M, R) for TM."""
    thetas = np.asarray(thetas, dtype=np.float64)
    M, R = points.shape[0], len(thetas)
    if source is None:
        return np.zeros((M, 2, R) if kind == "2d_vector" else (M, R), np.complex128)
    if source not in ("plane", "beam", "point"):
        raise NotImplementedError
    E = np.zeros((M, R), np.complex128) if source != "point" or kind == "2d_scalar" \
        else np.zeros((M, 2, R), np.complex128)
    # QUIRK (Transmission2D.py:112,116): the TE polarisation u is held in a
    # float32 torch tensor, so its components are rounded to float32.
    u = np.zeros((2, R), np.float32)
    for t, th in enumerate(thetas):
        c, s = np.cos(-th), np.sin(-th)
        u[:, t] = (s, c)
        rot = np.array([[c, -s], [s, c]])
        rr = points @ rot.T  # (rparallel, rperp)
        if source == "plane":
            E[:, t] = np.exp(1j * rr[:, 0] * k0)
        elif source == "beam":
            a = 2 * rr[:, 1] / (w * w * k0)
            E[:, t] = np.exp(1j * rr[:, 0] * k0 - (rr[:, 1] ** 2 / (w * w * (1 + 1j * a)))) / np.sqrt(1 + 1j * a)
        else:  # point dipole at distance 2 (Transmission2D.py:145-166, :662-677)
            dist = 2.0
            if kind == "2d_vector":
                intensity = k0 * dist * 2.0 * np.pi
                loc = dist * np.array([-1.0, 0.0])
                # QUIRK (Transmission2D.py:162): the moment is built on a
                # float32 torch.tensor, so its magnitude is rounded to float32
                mom = np.float32(np.sqrt(intensity)) * np.array([0.0, 1.0], np.float32)
                g = greens_2d_vector(rr.reshape(-1, 1, 2) - loc.reshape(1, -1, 2), k0)[:, 0]
                e = g @ mom.astype(np.complex128)
                E[:, :, t] = (rot.T.astype(np.complex128) @ e.T).T
            else:
                intensity = k0 * dist * 2.0 * np.pi
                loc = dist * np.array([-1.0, 0.0])
                E[:, t] = np.sqrt(intensity) * greens_2d_scalar(rr.reshape(-1, 1, 2) - loc.reshape(1, -1, 2), k0).reshape(M)
    if kind == "2d_vector" and source != "point":
        E = E.reshape(M, 1, R) * u.astype(np.float64)
    return E


def polarisation_vectors(p):
    """pvec rebuilt from p through (theta, phi), Transmission3D.py:102-104."""
    phi = np.arctan2(p[:, 1], p[:, 0])
    th = np.arccos(p[:, 2])
    return np.stack([np.sin(th) * np.cos(phi), np.sin(th) * np.sin(phi), p[:, 2]])


def source_3d(kind, source, points, k0, u, p, w):
    """generate_source for the 3D classes: Transmission3D.py:79-145 (vector)
    and :603-658 (scalar).  Returns (M, 3, R) or (M, R)."""
    M, R = points.shape[0], u.shape[0]
    if source is None:
        return np.zeros((M, u.shape[1], R) if kind == "3d_vector" else (M, u.shape[1]), np.complex128)
    rpara = points @ u.T
    if source == "plane":
        E = np.exp(1j * rpara * k0)
    elif source == "beam":
        rperp = np.linalg.norm(points.reshape(-1, 3, 1) - rpara.reshape(M, 1, R) * u.T.reshape(1, 3, -1), axis=1)
        a = 2 * rperp / (w * w * k0)
        E = np.exp(1j * rpara * k0 - (rperp ** 2 / (w * w * (1 + 1j * a)))) / np.sqrt(1 + 1j * a)
    else:
        # QUIRK: both 3D point sources fail inside the reference: the vector
        # one calls a method that does not exist (Transmission3D.py:136), the
        # scalar one calls .type() on a numpy float (Transmission3D.py:649).
        raise NotImplementedError
    if kind == "3d_vector":
        pv = polarisation_vectors(p)
        E = E.reshape(M, 1, -1) * pv.reshape(1, 3, -1)
    return E


# ---------------------------------------------------------------------------
# solve / propagate / DOS
# ---------------------------------------------------------------------------

def solve(kind, scat, k0, alpha, radius, E0, self_interaction=True, si_type="Rayleigh"):
    """Transmission*D solve(): LU solve of M Ek = E0 for all columns
    (Transmission2D.py:207-231, 718-744; Transmission3D.py:181-206, 693-718)."""
    _, d = kind_dims(kind)
    Mt = system_matrix(kind, scat, k0, alpha, radius, self_interaction, si_type)
    return np.linalg.solve(Mt, np.asarray(E0).reshape(d * scat.shape[0], -1))


def _nan_fix(kind, scat, points, out, src, regularize, radius, src_is_scatterer_field):
    """Row fix-up for detectors whose G row is NaN (Transmission2D.py:192-203,
    :703-714; Transmission3D.py:165-177, :677-689).

    ``src`` is Ek for propagate() and E0_meas for propagate_ss().
    QUIRK (2D TE, Transmission2D.py:201,203): Ek (2N, R) is indexed by the
    scatterer index and broadcast to both components.
    QUIRK (propagate_ss, Transmission2D.py:257,259): E0_meas is indexed by the
    scatterer index."""
    _, d = kind_dims(kind)
    flag = out[:, 0, 0] if out.ndim == 3 else out[:, 0]
    for j in np.nonzero(np.isnan(flag))[0]:
        dist = np.linalg.norm(scat - points[j], axis=-1)
        if regularize:
            cand = np.nonzero(dist <= radius)[0]
            idx = int(np.argmin(dist)) if cand.size > 1 else int(cand[0])
        else:
            idx = int(np.nonzero(np.all(scat - points[j] == 0, axis=-1))[0][0])
        if src_is_scatterer_field and kind == "3d_vector":
            out[j] = src.reshape(scat.shape[0], 3, -1)[idx]
        elif src_is_scatterer_field and kind == "3d_scalar":
            out[j] = src.reshape(scat.shape[0], -1)[idx]
        else:
            out[j] = src[idx]
    return out


def propagate(kind, scat, points, Ek, k0, alpha, E0, regularize=False, radius=0.0):
    """E(det) = k^2 alpha G0(det, scat) Ek + E0(det) (Transmission2D.py:176-205,
    :687-716; Transmission3D.py:147-179, :660-691)."""
    _, d = kind_dims(kind)
    G = G0(kind, scat, k0, points=points, regularize=regularize, radius=radius)
    with np.errstate(all="ignore"):
        out = alpha * k0 * k0 * (G @ Ek)
    M = points.shape[0]
    out = out.reshape(M, d, -1) + E0 if d > 1 else out.reshape(M, -1) + E0
    return _nan_fix(kind, scat, points, out, Ek, regularize, radius, True)


def propagate_ss(kind, scat, points, k0, alpha, E0_meas, E0_scat, regularize=False, radius=0.0):
    """Single-scattering propagate (Transmission2D.py:233-261, :746-775;
    Transmission3D.py:208-238, :720-749)."""
    _, d = kind_dims(kind)
    G = G0(kind, scat, k0, points=points, regularize=regularize, radius=radius)
    with np.errstate(all="ignore"):
        out = alpha * k0 * k0 * (G @ np.asarray(E0_scat).reshape(d * scat.shape[0], -1))
    M = points.shape[0]
    out = out.reshape(M, d, -1) + E0_meas if d > 1 else out.reshape(M, -1) + E0_meas
    return _nan_fix(kind, scat, points, out, E0_meas, regularize, radius, False)


DOS_PREFACTOR = {
    # Transmission2D.py:333 and :838
    "2d_vector": lambda k0, a: 4.0 * k0 * k0 * a,
    "2d_scalar": lambda k0, a: 4.0 * k0 * k0 * a,
    # Transmission3D.py:320 and :829
    "3d_vector": lambda k0, a: 2.0 * np.pi * k0 * a,
    "3d_scalar": lambda k0, a: 4.0 * np.pi * k0 * a,
}


def measurement_propagator(kind, scat, measure_points, k0, radius, self_interaction=True,
                           si_type="Rayleigh", regularize=False):
    """G0(measure, scat) with NaN entries replaced by S/V (or 0), the loop in
    mean_DOS_measurements (Transmission2D.py:314-323; Transmission3D.py:301-310).
    QUIRK: for vector kinds every entry of a coincident d x d block is NaN, so
    the whole block (off-diagonals included) becomes S/V."""
    Gm = G0(kind, scat, k0, points=measure_points, regularize=regularize, radius=radius)
    bad = np.isnan(Gm)
    if bad.any():
        Gm[bad] = self_term_over_volume(kind, k0, radius, si_type) if self_interaction else 0.0
    return Gm


def mean_dos(kind, scat, measure_points, k0, alpha, radius, self_interaction=True,
             si_type="Rayleigh", regularize=False, discard_absorption=False):
    """mean_DOS_measurements (Transmission2D.py:282-336, :787-841;
    Transmission3D.py:270-323, :779-832):
    Im(pref * sum((Gm^T Gm) * W) / P) with W = M^-1."""
    Mt = system_matrix(kind, scat, k0, alpha, radius, self_interaction, si_type)
    W = np.linalg.inv(Mt)
    Gm = measurement_propagator(kind, scat, measure_points, k0, radius, self_interaction, si_type, regularize)
    val = np.sum((Gm.T @ Gm) * W) / measure_points.shape[0]
    a = np.real(alpha) if discard_absorption else alpha
    return float(np.imag(val * DOS_PREFACTOR[kind](k0, a)))


def ldos(kind, scat, measure_points, k0, alpha, radius, self_interaction=True,
         si_type="Rayleigh", regularize=False, discard_absorption=False):
    """LDOS_measurements (Transmission2D.py:338-390; Transmission3D.py:325-376):
    per point Im(pref * diag(Gm W Gm^T)) summed over the d components."""
    _, d = kind_dims(kind)
    Mt = system_matrix(kind, scat, k0, alpha, radius, self_interaction, si_type)
    W = np.linalg.inv(Mt)
    Gm = measurement_propagator(kind, scat, measure_points, k0, radius, self_interaction, si_type, regularize)
    v = np.einsum("ij,ji->i", Gm @ W, Gm.T)
    a = np.real(alpha) if discard_absorption else alpha
    v = np.imag(v * DOS_PREFACTOR[kind](k0, a))
    return v.reshape(measure_points.shape[0], d, -1).sum(1) if d > 1 else v


def relative_residual(Mt, X, B):
    """||B - M X||_F / ||B||_F in float64."""
    return float(np.linalg.norm(B - Mt @ X) / np.linalg.norm(B))
