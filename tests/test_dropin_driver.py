"""The drop-in as the reference driver uses it, on the GPU.

The driver imports ``Transmission2D`` / ``Transmission3D`` and ``hickle`` as
top-level modules (magreete.py:1-20).  Here those names are aliased to the
drop-in modules and to ``magreete_gb300.fieldcache``, and the driver's
per-frequency call sequences are replayed with its argument types (torch
point tensors, numpy angles, ``onp.array`` / ``.numpy()`` on the results):
  * transmission, magreete.py:325-400: generate_source at the scatterers and
    at the 360 / Fibonacci detectors, solve, ``hkl.dump`` of
    ``[Ej, [alpha, k0], points, thetas]``, propagate; then the
    ``plot_transmission`` re-run from the cache (magreete.py:404-431);
  * mean DOS, magreete.py:871-896.
Every saved array is compared with the oracle.

Also here: the Green's tensors of separation arrays with each periodic
option against the reference's own outputs, a Hankel-function sweep over
kR in [1e-4, 1e3] against scipy, the single-scatterer (dressed
polarisability) solve and the symmetry of the assembled system.
"""
import math
import os
import sys

import numpy as np
import pytest
import scipy.special as sps
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL = {"fp64": 1e-10, "mixed": 1e-8}


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(autouse=True)
def exact_bessel():
    O.BESSEL_MODE = "exact"
    yield


@pytest.fixture
def driver_modules(monkeypatch):
    """sys.modules as a driver run would see them with the drop-in installed."""
    import magreete_gb300.Transmission2D as T2
    import magreete_gb300.Transmission3D as T3
    import magreete_gb300.fieldcache as fc
    monkeypatch.setitem(sys.modules, "Transmission2D", T2)
    monkeypatch.setitem(sys.modules, "Transmission3D", T3)
    monkeypatch.setitem(sys.modules, "hickle", fc)
    yield


def _scene(ndim, N, seed):
    rng = np.random.default_rng(seed)
    if ndim == 2:
        r = np.sqrt(rng.random(N))
        t = 2 * np.pi * rng.random(N)
        pts = np.stack([r * np.cos(t), r * np.sin(t)], 1)
    else:
        pts = rng.random((N, 3)) - 0.5
    phi = 0.05 if ndim == 2 else 0.1
    volume = (np.pi if ndim == 2 else 1.0) * phi / N
    radius = np.sqrt(volume / np.pi) if ndim == 2 else np.cbrt(3 * volume / (4 * np.pi))
    alpha = volume * (1.6 ** 2 - 1) + 0j
    return torch.from_numpy(pts), radius, alpha


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("ndim", [2, 3])
def test_driver_transmission_sequence(driver_modules, tmp_path, monkeypatch, ndim, precision):
    monkeypatch.setenv("MAGREETE_PRECISION", precision)
    import hickle as hkl
    import numpy as onp
    from Transmission2D import Transmission2D_vector
    from Transmission3D import Transmission3D_vector
    np_ = torch
    points, radius, alpha0 = _scene(ndim, 180 if ndim == 2 else 120, 3 + ndim)
    L, beam_waist, self_interaction, regularize = 1.0, 0.2, True, False
    thetas = onp.arange(6) / 6 * 2 * onp.pi
    solver = Transmission2D_vector(points, source="plane") if ndim == 2 else \
        Transmission3D_vector(points, source="plane")
    if ndim == 2:
        tm = onp.arange(360) / 360 * 2 * np.pi
        measurement_points = np_.from_numpy(2.0 * L * onp.vstack([onp.cos(tm), onp.sin(tm)]).T)
    else:
        golden = onp.pi * (onp.sqrt(5.0) - 1.0)
        i = onp.arange(200)
        z = 1 - (i / 199) * 2
        measurement_points = np_.from_numpy(3.0 * L * onp.stack([onp.cos(i * golden) * onp.sqrt(1 - z ** 2),
                                                                 onp.sin(i * golden) * onp.sqrt(1 - z ** 2), z]).T)
        u = np_.from_numpy(onp.stack([onp.cos(thetas), onp.sin(thetas), onp.zeros(len(thetas))]).T)
        e_alt = np_.zeros(u.shape)
        e_alt[:, 2] = 1
        p = e_alt * onp.cos(0.0) + onp.stack([onp.sin(thetas), -onp.cos(thetas), onp.zeros(len(thetas))]).T * 0.0
    k0range = [2 * onp.pi * 4.0, 2 * onp.pi * 4.5]
    file_name = str(tmp_path / "run")
    Eall, saved = [], []
    for k0 in k0range:
        alpha = alpha0
        if ndim == 2:
            E0_scat = solver.generate_source(points, k0, thetas, beam_waist, print_statement="Source at scatterers")
            E0_meas = solver.generate_source(measurement_points, k0, thetas, beam_waist,
                                             print_statement="Source at measurement points")
        else:
            E0_scat = solver.generate_source(points, k0, u, p, beam_waist, print_statement="Source at scatterers")
            E0_meas = solver.generate_source(measurement_points, k0, u, p, beam_waist,
                                             print_statement="Source at measurement points")
        Ej = solver.solve(k0, alpha, radius, E0_scat, self_interaction=self_interaction,
                          self_interaction_type="Rayleigh")
        k0_ = onp.round(onp.real(k0 * L / (2 * onp.pi)), 1)
        fname = file_name + "_Ek_k0_" + str(k0_) + "_0.hkl"
        hkl.dump([onp.array(Ej), onp.array([alpha, k0]), onp.array(points), onp.array(thetas)], fname)
        saved.append(fname)
        Ek = solver.propagate(measurement_points, Ej, k0, alpha, E0_meas, regularize=regularize, radius=radius)
        Eall.append(Ek.numpy())
    hkl.dump([onp.array(Eall), onp.array(k0range), onp.array(thetas)], file_name + "_transmission_0.hkl")

    # the oracle on the same inputs
    pts = points.numpy()
    det = measurement_points.numpy()
    for k0, fname, E_meas in zip(k0range, saved, Eall):
        if ndim == 2:
            E0s = O.source_2d("2d_vector", "plane", pts, k0, thetas, beam_waist)
            E0d = O.source_2d("2d_vector", "plane", det, k0, thetas, beam_waist)
        else:
            E0s = O.source_3d("3d_vector", "plane", pts, k0, u.numpy(), p.numpy(), beam_waist)
            E0d = O.source_3d("3d_vector", "plane", det, k0, u.numpy(), p.numpy(), beam_waist)
        kind = "2d_vector" if ndim == 2 else "3d_vector"
        Ek_ref = O.solve(kind, pts, k0, alpha0, radius, E0s)
        Ed_ref = O.propagate(kind, pts, det, Ek_ref, k0, alpha0, E0d)
        Ej_saved, params, pts_saved, th_saved = hkl.load(fname)
        assert rel(Ej_saved, Ek_ref) < TOL[precision]
        assert complex(params[0]) == alpha0 and float(np.real(params[1])) == k0
        assert np.array_equal(pts_saved, pts) and np.array_equal(th_saved, thetas)
        assert rel(E_meas, Ed_ref) < TOL[precision]
        # plot_transmission re-run: fields from the cache, propagated again
        Ej2 = np_.from_numpy(Ej_saved)
        if ndim == 2:
            E0_meas = solver.generate_source(measurement_points, k0, th_saved.astype(onp.float64), beam_waist)
        else:
            E0_meas = solver.generate_source(measurement_points, k0, u, p, beam_waist)
        Ek2 = solver.propagate(measurement_points, Ej2, k0, alpha0, E0_meas, regularize=regularize, radius=radius)
        assert rel(Ek2.numpy(), E_meas) < 1e-13
    Eall_saved, k_saved, _ = hkl.load(file_name + "_transmission_0.hkl")
    assert np.array_equal(Eall_saved, np.array(Eall)) and np.allclose(k_saved, k0range)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("ndim", [2, 3])
def test_driver_dos_sequence(driver_modules, monkeypatch, ndim, precision):
    monkeypatch.setenv("MAGREETE_PRECISION", precision)
    import numpy as onp
    from Transmission2D import Transmission2D_vector
    from Transmission3D import Transmission3D_vector
    points, radius, alpha = _scene(ndim, 200 if ndim == 2 else 120, 11 + ndim)
    solver = Transmission2D_vector(points, source="plane") if ndim == 2 else \
        Transmission3D_vector(points, source="plane")
    from magreete_gb300 import workloads as W
    measurement_points = W.ball_points(50, 5, ndim)
    measurement_points *= 1.0 / 2
    DOSall, k0_range = [], []
    k0range = [2 * onp.pi * 3.5, 2 * onp.pi * 4.0, 2 * onp.pi * 4.5]
    for k0 in k0range:
        dos = solver.mean_DOS_measurements(measurement_points, k0, alpha, radius, regularize=False,
                                           self_interaction=True, self_interaction_type="Rayleigh")
        DOSall.append(dos.numpy())
        k0_range.append(onp.round(onp.real(k0 / (2 * onp.pi)), 1))
    table = onp.stack([k0_range, DOSall]).T
    kind = "2d_vector" if ndim == 2 else "3d_vector"
    tol = 1e-9 if precision == "fp64" else 1e-8
    for row, k0 in zip(table, k0range):
        ref = O.mean_dos(kind, points.numpy(), measurement_points.numpy(), k0, alpha, radius)
        assert abs(row[1] - ref) <= tol * abs(ref)


@pytest.mark.parametrize("kind", O.KINDS)
def test_greens_separations_periodic_vs_reference(kind):
    """torch_greens / greens on the reference's separation arrays, free and with
    each periodic option, and regularised, against the reference's own outputs
    (Transmission2D.py:63-91, :595-618; Transmission3D.py:47-77, :573-601).
    2D is held to the torch-Bessel accuracy of the reference (2e-6), 3D to 1e-12;
    both also to the oracle (exact Bessel functions)."""
    from magreete_gb300 import Transmission2D_scalar, Transmission2D_vector, Transmission3D_scalar, Transmission3D_vector
    cls = {"2d_vector": Transmission2D_vector, "2d_scalar": Transmission2D_scalar,
           "3d_vector": Transmission3D_vector, "3d_scalar": Transmission3D_scalar}[kind]
    z = np.load(os.path.join(GOLD, f"golden_greens_{kind}.npz"))
    r, k0 = z["r"], float(z["k0"])
    dim = 2 if kind.startswith("2d") else 3
    s = cls(torch.zeros((3, dim), dtype=torch.float64))
    fn = s.torch_greens if dim == 2 else s.greens
    tol_ref = 2e-6 if dim == 2 else 1e-12
    tol_orc = 1e-11 if dim == 2 else 1e-13
    for i, per in enumerate(z["periodic_options"]):
        G = fn(torch.from_numpy(r), k0, periodic=str(per))
        assert tuple(G.shape) == z[f"G_{i}"].shape
        assert rel(G, z[f"G_{i}"]) < tol_ref, per
        assert rel(G, O.greens_separations(kind, r, k0, periodic=str(per))) < tol_orc, per
    G = fn(torch.from_numpy(r), k0, regularize=True, radius=float(z["radius_reg"])).numpy()
    ref = z["G_reg"]
    fin = np.isfinite(ref)
    assert np.array_equal(np.isfinite(G), fin)
    assert rel(G[fin], ref[fin]) < tol_ref


@pytest.mark.parametrize("kind", ["2d_scalar", "2d_vector"])
def test_hankel_sweep_small_to_large_kR(kind):
    """H0 / H1 inside the 2D Green's tensors for kR from 1e-4 to 1e3 (400
    log-spaced values, separations along a skew direction) against scipy's
    hankel1: each tensor within 1e-11 of its own norm."""
    from magreete_gb300 import Transmission2D_scalar, Transmission2D_vector
    cls = Transmission2D_scalar if kind == "2d_scalar" else Transmission2D_vector
    k0 = 2 * np.pi * 3.0
    kR = np.logspace(-4, 3, 400)
    d = np.array([math.cos(0.3), math.sin(0.3)])
    r = (kR / k0)[:, None] * d[None, :]
    s = cls(torch.zeros((2, 2), dtype=torch.float64))
    G = s.torch_greens(torch.from_numpy(r.reshape(400, 1, 2)), k0).numpy().reshape(400, -1)
    h0, h1 = sps.hankel1(0, kR), sps.hankel1(1, kR)
    if kind == "2d_scalar":
        ref = (0.25j * h0).reshape(400, 1)
    else:
        RR = d[:, None] * d[None, :]
        I2 = np.eye(2)
        ref = 0.25j * ((I2 - RR)[None] * h0[:, None, None] - (I2 - 2 * RR)[None] * (h1 / kR)[:, None, None])
        ref = ref.reshape(400, 4)
    err = np.linalg.norm(G - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert err.max() < 1e-11, (kR[err.argmax()], err.max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", O.KINDS)
def test_single_scatterer_dressed_polarisability(kind, precision):
    """N = 1: the solve is E0 / (1 - k^2 alpha S/V), the dressed
    polarisability (the self-term shift rounded as the reference rounds it)."""
    from magreete_gb300 import Transmission2D_scalar, Transmission2D_vector, Transmission3D_scalar, Transmission3D_vector
    cls = {"2d_vector": Transmission2D_vector, "2d_scalar": Transmission2D_scalar,
           "3d_vector": Transmission3D_vector, "3d_scalar": Transmission3D_scalar}[kind]
    dim, d = O.kind_dims(kind)
    pt = torch.tensor([[0.1] * dim], dtype=torch.float64)
    s = cls(pt, source="plane", precision=precision)
    k0, radius = 2 * np.pi * 2.0, 0.05
    alpha = (np.pi * radius ** 2 if dim == 2 else 4 / 3 * np.pi * radius ** 3) * (1.6 ** 2 - 1) + 0.001j
    E0 = torch.randn(d, 3, dtype=torch.complex128, generator=torch.Generator().manual_seed(1))
    Ek = s.solve(k0, alpha, radius, E0)
    shift = O.diagonal_self_shift(kind, k0, alpha, radius)
    assert rel(Ek, E0.numpy() / (1 - shift)) < (1e-14 if precision == "fp64" else 1e-10)


@pytest.mark.parametrize("kind", O.KINDS)
def test_system_matrix_is_complex_symmetric(kind):
    """M^T = M exactly, in every output format, for a random geometry."""
    from magreete_gb300 import engine as E
    dim, _ = O.kind_dims(kind)
    pts = torch.rand(301, dim, dtype=torch.float64, generator=torch.Generator().manual_seed(4)).cuda()
    M128, = E.assemble_system(kind, pts, 2 * np.pi * 5, 0.01 + 0.002j, 0.1 - 0.01j, ("c128",))
    Mdf, M64 = E.assemble_system(kind, pts, 2 * np.pi * 5, 0.01 + 0.002j, 0.1 - 0.01j, ("cdf", "c64"))
    assert torch.equal(M128, M128.T)
    assert torch.equal(M64, M64.T)
    assert torch.equal(Mdf, Mdf.transpose(0, 1))
