"""Host-side math of the drop-in on CPU against the reference's golden outputs:
incident fields (plane, beam; torch ops that run on the points' device), the
self-interaction integrals and the diagonal shift with the reference's
complex64 rounding, and the reference's errors for unknown types."""
import os

import numpy as np
import pytest
import torch

from magreete_gb300 import selfterm
from magreete_gb300 import sources as S

GOLD = os.path.join(os.path.dirname(__file__), "golden")
KINDS = ["2d_vector", "2d_scalar", "3d_vector", "3d_scalar"]


def load(kind):
    z = np.load(os.path.join(GOLD, f"golden_{kind}.npz"))
    return {k: z[k] for k in z.files}


def rel(a, b):
    return float(np.linalg.norm((np.asarray(a) - b).ravel()) / np.linalg.norm(b.ravel()))


def source(kind, g, which, pts):
    k0, w = float(g["k0"]), float(g["beam_w"])
    if kind.startswith("2d"):
        return S.source_2d(kind, which, pts, k0, g["thetas"], w)
    p = torch.from_numpy(g["p"]) if kind == "3d_vector" else None
    return S.source_3d(kind, which, pts, k0, torch.from_numpy(g["u"]), p, w)


@pytest.mark.parametrize("kind", KINDS)
def test_plane_and_beam_sources_match_reference(kind):
    g = load(kind)
    pts = torch.from_numpy(g["points"])
    E0 = source(kind, g, "plane", pts)
    assert E0.dtype == torch.complex128 and tuple(E0.shape) == g["E0_scat"].shape
    assert rel(E0.numpy(), g["E0_scat"]) <= 1e-14
    assert rel(source(kind, g, "plane", torch.from_numpy(g["det"])).numpy(), g["E0_det"]) <= 1e-14
    assert rel(source(kind, g, "beam", pts).numpy(), g["E0_scat_beam"]) <= 1e-14


@pytest.mark.parametrize("kind", KINDS)
def test_self_terms_match_reference(kind):
    g = load(kind)
    k0, a = float(g["k0"]), float(g["radius"])
    for t, key, tol in (("Rayleigh", "si_rayleigh", 1e-14), ("full", "si_full", 1e-12)):
        ref = complex(g[key])
        assert abs(complex(selfterm.SELF_TERM[kind](k0, a, t)) - ref) <= tol * abs(ref)
    with pytest.raises(NotImplementedError):
        selfterm.SELF_TERM[kind](k0, a, "unknown")


@pytest.mark.parametrize("kind", KINDS)
def test_diagonal_shift_rounding(kind):
    g = load(kind)
    k0, a, alpha = float(g["k0"]), float(g["radius"]), complex(g["alpha"])
    exact = selfterm.diagonal_shift(kind, k0, alpha, a, reference_rounding=False)
    assert exact == pytest.approx(alpha * k0 * k0 * complex(g["si_rayleigh"]) / selfterm.volume(kind, a), rel=1e-14)
    rounded = selfterm.diagonal_shift(kind, k0, alpha, a)
    # the reference multiplies by a float32 identity: the shift is a complex64 value
    assert rounded == complex(np.complex64(exact))
    assert selfterm.diagonal_shift(kind, k0, alpha, a, self_interaction=False) == 0j


def test_unknown_source_raises():
    g = load("2d_vector")
    pts = torch.from_numpy(g["points"])
    with pytest.raises(NotImplementedError):
        S.source_2d("2d_vector", "laser", pts, float(g["k0"]), g["thetas"], 1.0)
    g3 = load("3d_vector")
    with pytest.raises(NotImplementedError):
        S.source_3d("3d_vector", "point", torch.from_numpy(g3["points"]), float(g3["k0"]),
                    torch.from_numpy(g3["u"]), torch.from_numpy(g3["p"]), 1.0)


@pytest.mark.parametrize("kind", KINDS)
def test_periodic_wrap_matches_reference_semantics(kind):
    """The drop-in's wrap of separations (host side of torch_greens / greens)
    equals the oracle's restatement for every periodic option the reference
    fixtures hold, and leaves its input untouched."""
    from oracle import oracle as O
    from magreete_gb300.solver import periodic_wrap
    z = np.load(os.path.join(GOLD, f"golden_greens_{kind}.npz"))
    dim = 2 if kind.startswith("2d") else 3
    r = torch.from_numpy(z["r"].copy())
    for per in list(z["periodic_options"]) + ["z", "yz"]:
        w = periodic_wrap(r, str(per), dim)
        assert torch.equal(w, torch.from_numpy(O.periodic_wrap(kind, z["r"], str(per)))), per
        assert w.abs().max() <= 1.2
    assert torch.equal(r, torch.from_numpy(z["r"]))
    if dim == 2:
        assert torch.equal(periodic_wrap(r, "xy", 2), r)      # the 2D classes ignore 'xy'


@pytest.mark.parametrize("kind", KINDS)
def test_solve_without_incident_fields_returns_empty(kind, monkeypatch):
    """solve() with zero right-hand sides returns an empty (d*N, 0) complex128
    tensor, as the reference's linalg.solve does, without any device work (the
    device lookup is pointed at the CPU here; no library call is reached)."""
    import magreete_gb300 as M
    from magreete_gb300 import engine as E
    monkeypatch.setattr(E, "device_of", lambda *t: torch.device("cpu"))
    cls = {"2d_vector": M.Transmission2D_vector, "2d_scalar": M.Transmission2D_scalar,
           "3d_vector": M.Transmission3D_vector, "3d_scalar": M.Transmission3D_scalar}[kind]
    g = load(kind)
    s = cls(torch.from_numpy(g["points"]), source="plane")
    d = s.d
    E0 = torch.zeros((s.N, d, 0) if d > 1 else (s.N, 0), dtype=torch.complex128)
    X = s.solve(float(g["k0"]), complex(g["alpha"]), float(g["radius"]), E0)
    assert X.shape == (d * s.N, 0) and X.dtype == torch.complex128 and X.device.type == "cpu"
    with pytest.raises(NotImplementedError):
        s.solve(float(g["k0"]), complex(g["alpha"]), float(g["radius"]), E0, self_interaction_type="other")


@pytest.mark.parametrize("kind", KINDS)
def test_dos_at_no_points_as_reference(kind, monkeypatch):
    """Mean DOS over zero measurement points is nan (the reference's 0 / 0);
    LDOS at zero points raises RuntimeError, as the reference does.  Both are
    decided on the host before any device work."""
    import magreete_gb300 as M
    from magreete_gb300 import engine as E
    monkeypatch.setattr(E, "device_of", lambda *t: torch.device("cpu"))
    cls = {"2d_vector": M.Transmission2D_vector, "2d_scalar": M.Transmission2D_scalar,
           "3d_vector": M.Transmission3D_vector, "3d_scalar": M.Transmission3D_scalar}[kind]
    g = load(kind)
    s = cls(torch.from_numpy(g["points"]), source="plane")
    none = torch.zeros((0, s.dim), dtype=torch.float64)
    k0, alpha, a = float(g["k0"]), complex(g["alpha"]), float(g["radius"])
    v = s.mean_DOS_measurements(none, k0, alpha, a)
    assert v.dim() == 0 and v.dtype == torch.float64 and torch.isnan(v)
    with pytest.raises(NotImplementedError):
        s.mean_DOS_measurements(none, k0, alpha, a, self_interaction_type="other")
    with pytest.raises(RuntimeError):
        s.LDOS_measurements(none, k0, alpha, a)


@pytest.mark.parametrize("kind", KINDS)
def test_G0_to_no_points_is_empty(kind, monkeypatch):
    """G0 / G0_vector towards zero target points: an empty (0, d*N) complex128
    propagator, as the reference returns (decided on the host)."""
    import magreete_gb300 as M
    from magreete_gb300 import engine as E
    monkeypatch.setattr(E, "device_of", lambda *t: torch.device("cpu"))
    cls = {"2d_vector": M.Transmission2D_vector, "2d_scalar": M.Transmission2D_scalar,
           "3d_vector": M.Transmission3D_vector, "3d_scalar": M.Transmission3D_scalar}[kind]
    g = load(kind)
    s = cls(torch.from_numpy(g["points"]), source="plane")
    fn = s.G0_vector if kind == "2d_vector" else s.G0
    G = fn(torch.zeros((0, s.dim), dtype=torch.float64), float(g["k0"]))
    assert G.shape == (0, s.d * s.N) and G.dtype == torch.complex128 and G.device.type == "cpu"


@pytest.mark.parametrize("kind", KINDS)
def test_sources_for_no_incidences_have_the_reference_shapes(kind):
    """Zero angles / directions give empty fields shaped like the reference's:
    (N, d, 0) for the vector kinds, (N, 0) for the scalar kinds."""
    g = load(kind)
    pts = torch.from_numpy(g["points"])
    N, vec = pts.shape[0], kind.endswith("vector")
    d = int(kind[0]) if vec else 1
    for which in ("plane", "beam"):
        if kind.startswith("2d"):
            E0 = S.source_2d(kind, which, pts, float(g["k0"]), np.array([]), 0.2)
        else:
            u = torch.zeros((0, 3), dtype=torch.float64)
            E0 = S.source_3d(kind, which, pts, float(g["k0"]), u, u if vec else None, 0.2)
        assert tuple(E0.shape) == ((N, d, 0) if vec else (N, 0)) and E0.dtype == torch.complex128


@pytest.mark.parametrize("kind", KINDS)
def test_class_attributes_and_options(kind, monkeypatch):
    """The reference's attributes (.r, .N, .source), the engine options and
    their validation, without device work."""
    import magreete_gb300 as M
    from magreete_gb300 import engine as E
    monkeypatch.setattr(E, "device_of", lambda *t: torch.device("cpu"))
    cls = {"2d_vector": M.Transmission2D_vector, "2d_scalar": M.Transmission2D_scalar,
           "3d_vector": M.Transmission3D_vector, "3d_scalar": M.Transmission3D_scalar}[kind]
    g = load(kind)
    pts = torch.from_numpy(g["points"])
    s = cls(pts)
    assert s.source == "beam" and s.N == pts.shape[0] and torch.equal(s.r, pts)
    assert s.precision == "fp64"
    assert cls(g["points"], source="plane", precision="mixed").precision == "mixed"   # numpy input too
    monkeypatch.setenv("MAGREETE_PRECISION", "mixed")
    assert cls(pts).precision == "mixed"
    with pytest.raises(ValueError):
        cls(pts, precision="fp16")
    # the spectral tools take the reference's parameters (Transmission2D.py:455, :479, :517)
    import inspect
    params = {name: list(inspect.signature(getattr(s, name)).parameters)
              for name in ("compute_hamiltonian_DOS", "compute_eigenvalues_and_scatterer_LDOS",
                           "compute_eigenmodes_IPR")}
    assert params["compute_hamiltonian_DOS"] == ["k0", "deltas", "file_name", "write_eigenvalues"]
    assert params["compute_eigenvalues_and_scatterer_LDOS"] == [
        "k0", "alpha", "radius", "file_name", "self_interaction", "self_interaction_type", "write_eigenvalues"]
    assert params["compute_eigenmodes_IPR"] == [
        "k0", "alpha", "radius", "file_name", "self_interaction", "self_interaction_type", "number_eigenmodes",
        "write_eigenvalues", "sorting_type"]
