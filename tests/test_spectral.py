"""Spectral tools of the drop-in classes (compute_hamiltonian_DOS,
compute_eigenvalues_and_scatterer_LDOS, compute_eigenmodes_IPR) against the
reference's own outputs (tests/golden/golden_spectral_<kind>.npz, written by
make_golden.py --spectral).

CPU tests: the Green's matrix comes from the oracle (its "torch" Bessel mode
reproduces the reference's 2D matrices to ~1e-15), the eigensolver is the
host LAPACK the reference uses, and the class methods run on a solver object
whose GPU assembly is replaced by that matrix.  Eigenvalues are compared as
sets (nearest match), eigenvectors up to a phase.
"""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from magreete_gb300 import selfterm
from magreete_gb300 import spectral as SP

GOLD = os.path.join(os.path.dirname(__file__), "golden")
KINDS = ("2d_vector", "2d_scalar", "3d_vector", "3d_scalar")


@pytest.fixture(autouse=True)
def torch_bessel():
    old = O.BESSEL_MODE
    O.BESSEL_MODE = "torch"
    yield
    O.BESSEL_MODE = old


def load(kind):
    z = np.load(os.path.join(GOLD, f"golden_spectral_{kind}.npz"))
    return {k: z[k] for k in z.files}


def green(kind, g):
    return torch.from_numpy(O.G0(kind, g["points"], float(g["k0"])))


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def same_set(a, b, tol):
    """Every value of b has a value of a within tol (relative to max |b|), and
    the sizes agree."""
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    assert a.shape == b.shape
    scale = np.abs(b).max()
    d = np.abs(a[:, None] - b[None, :]).min(axis=0)
    assert d.max() <= tol * scale, d.max() / scale


def csv_values(arr):
    arr = np.atleast_2d(arr)
    return arr[:, 0] + 1j * arr[:, 1]


@pytest.mark.parametrize("kind", KINDS)
def test_hamiltonian_dos(kind):
    g = load(kind)
    k0 = float(g["k0"])
    dos, lambdas = SP.hamiltonian_dos(kind, green(kind, g), k0, torch.from_numpy(g["deltas_grid"]))
    assert rel(dos.numpy(), g["hamiltonian_dos"]) < 1e-10
    name = [k for k in g if k.startswith("csv:") and "hamiltonian_lambdas" in k][0]
    same_set(lambdas.numpy(), csv_values(g[name]), 1e-11)


@pytest.mark.parametrize("kind", KINDS)
def test_scatterer_ldos_factor(kind):
    g = load(kind)
    k0, alpha, radius = float(g["k0"]), complex(g["alpha"]), float(g["radius"])
    N = g["points"].shape[0]
    G = green(kind, g)
    for self_interaction, key in ((True, "ldos_factor"), (False, "ldos_factor_no_self")):
        shift = selfterm.diagonal_shift(kind, k0, alpha, radius, self_interaction, "Rayleigh")
        M = SP.system_matrix(G, k0, alpha, shift)
        if self_interaction:
            # the same system matrix the solve builds (oracle restatement)
            assert rel(M.numpy(), O.system_matrix(kind, g["points"], k0, alpha, radius)) < 1e-15
        f, deltas = SP.scatterer_ldos_factor(kind, M, N, k0, alpha)
        assert abs(float(f) - float(g[key])) <= 1e-9 * abs(float(g[key]))
    name = [k for k in g if k.startswith("csv:_deltas_")][0]
    shift = selfterm.diagonal_shift(kind, k0, alpha, radius, True, "Rayleigh")
    _, deltas = SP.scatterer_ldos_factor(kind, SP.system_matrix(G, k0, alpha, shift), N, k0, alpha)
    same_set(deltas.numpy(), csv_values(g[name]), 1e-11)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("sorting", ["IPR", "damping"])
def test_eigenmodes_ipr(kind, sorting):
    g = load(kind)
    k0, alpha, radius = float(g["k0"]), complex(g["alpha"]), float(g["radius"])
    shift = selfterm.diagonal_shift(kind, k0, alpha, radius, True, "Rayleigh")
    M = SP.system_matrix(green(kind, g), k0, alpha, shift)
    values, vectors, iprs = SP.eigenmodes(kind, M, k0, alpha, radius)
    # the unsorted values and IPRs, as written to the CSV
    name = [k for k in g if k.startswith(f"csv:_{sorting}_")][0]
    written = np.atleast_2d(g[name])
    same_set(values.numpy(), written[:, 0] + 1j * written[:, 1], 1e-10)
    assert rel(np.sort(iprs.numpy()), np.sort(written[:, 2])) < 1e-9
    v, V, p = SP.sort_modes(values, vectors, iprs, sorting)
    gv, gV, gp = g[f"ipr_{sorting}_values"], g[f"ipr_{sorting}_vectors"], g[f"ipr_{sorting}_iprs"]
    assert rel(p.numpy(), gp) < 1e-9
    assert rel(v.numpy(), gv) < 1e-9
    # the first modes, up to a phase each
    for j in range(gV.shape[1]):
        overlap = abs(np.vdot(V[:, j].numpy(), gV[:, j])) / (np.linalg.norm(V[:, j].numpy()) * np.linalg.norm(gV[:, j]))
        assert overlap > 1 - 1e-9, (j, overlap)
    with pytest.raises(NotImplementedError):
        SP.sort_modes(values, vectors, iprs, "energy")


def _cpu_solver(kind, g):
    """A drop-in class object on the CPU whose Green's matrix comes from the
    oracle (the GPU assembly replaced)."""
    from magreete_gb300 import Transmission2D_scalar, Transmission2D_vector, Transmission3D_scalar, \
        Transmission3D_vector
    cls = {"2d_vector": Transmission2D_vector, "2d_scalar": Transmission2D_scalar,
           "3d_vector": Transmission3D_vector, "3d_scalar": Transmission3D_scalar}[kind]
    s = cls.__new__(cls)
    dim = 2 if kind.startswith("2d") else 3
    s.dim, s.d = dim, (1 if kind.endswith("scalar") else dim)
    s.r = torch.from_numpy(g["points"])
    s.N = s.r.shape[0]
    s.verbose = False
    s.reference_rounding = True
    s._G0_dense = lambda points, k0, statement="", **kw: green(kind, g)
    return s


@pytest.mark.parametrize("kind", KINDS)
def test_class_methods_write_the_reference_files(kind, tmp_path):
    """The three methods of the class return the reference's values and write
    its files, under its names, with the same contents."""
    g = load(kind)
    k0, alpha, radius = float(g["k0"]), complex(g["alpha"]), float(g["radius"])
    s = _cpu_solver(kind, g)
    base = str(tmp_path / "spec")
    dos = s.compute_hamiltonian_DOS(k0, torch.from_numpy(g["deltas_grid"]), base)
    assert rel(dos.numpy(), g["hamiltonian_dos"]) < 1e-10
    f = s.compute_eigenvalues_and_scatterer_LDOS(k0, alpha, radius, base)
    assert abs(float(f) - float(g["ldos_factor"])) <= 1e-9 * abs(float(g["ldos_factor"]))
    f0 = s.compute_eigenvalues_and_scatterer_LDOS(k0, alpha, radius, base + "_ns", self_interaction=False,
                                                  write_eigenvalues=False)
    assert abs(float(f0) - float(g["ldos_factor_no_self"])) <= 1e-9 * abs(float(g["ldos_factor_no_self"]))
    for sorting in ("IPR", "damping"):
        v, V, p = s.compute_eigenmodes_IPR(k0, alpha, radius, base + "_" + sorting, number_eigenmodes=3,
                                           sorting_type=sorting)
        assert V.shape == g[f"ipr_{sorting}_vectors"].shape
        assert rel(v.numpy(), g[f"ipr_{sorting}_values"]) < 1e-9
        assert rel(p.numpy(), g[f"ipr_{sorting}_iprs"]) < 1e-9
    written = sorted("csv:" + n[len("spec"):] for n in os.listdir(tmp_path))
    assert written == sorted(k for k in g if k.startswith("csv:"))
    for key in written:
        ours = np.atleast_2d(np.loadtxt(os.path.join(tmp_path, "spec" + key[4:])))
        ref = np.atleast_2d(g[key])
        same_set(ours[:, 0] + 1j * ours[:, 1], ref[:, 0] + 1j * ref[:, 1], 1e-10)
        if ref.shape[1] == 3:
            assert rel(np.sort(ours[:, 2]), np.sort(ref[:, 2])) < 1e-9
    with pytest.raises(NotImplementedError):
        s.compute_eigenmodes_IPR(k0, alpha, radius, base + "_bad", sorting_type="energy")
