"""Full-field images and the field cache (host logic on CPU; one GPU test).

The CPU tests restate the driver's formulas (magreete.py:575-581 grid,
:652 angle lookup, :698-713 field components, :391/:412 cache objects)
element by element and compare."""
import math
import os

import numpy as np
import pytest
import torch

from magreete_gb300 import fieldcache as fc
from magreete_gb300 import fields as F

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_grid_points_2d():
    pts = F.grid_points(2, 5, 3, L=2.0, window_width=1.5).numpy()
    assert pts.shape == (15, 2) and pts.dtype == np.float64
    r = 5 / 3
    for iy in range(3):
        for ix in range(5):
            x = (ix * r / 4 - r / 2) * 3.0
            y = (iy / 2 - 0.5) * 3.0
            assert pts[iy * 5 + ix] == pytest.approx([x, y], abs=1e-15)


@pytest.mark.parametrize("slice_coordinate, zero_axis", [(0, 2), (1, 0), (2, 1)])
def test_grid_points_3d_slices(slice_coordinate, zero_axis):
    pts = F.grid_points(3, 4, 4, L=1.0, slice_coordinate=slice_coordinate).numpy()
    assert pts.shape == (16, 3)
    assert np.all(pts[:, zero_axis] == 0.0)
    others = [a for a in range(3) if a != zero_axis]
    assert all(np.unique(pts[:, a]).size == 4 for a in others)


def test_column_of_angle():
    thetas = np.linspace(0, 2 * np.pi, 8, endpoint=False)
    assert F.column_of_angle(thetas, thetas[5] + 1e-6) == 5
    assert F.column_of_angle(torch.from_numpy(thetas), thetas[0]) == 0
    with pytest.raises(ValueError):
        F.column_of_angle(thetas, 0.1)


def test_field_components_2d():
    g = np.random.default_rng(3)
    P = 50
    E = g.normal(size=(P, 2)) + 1j * g.normal(size=(P, 2))
    pts = g.normal(size=(P, 2))
    amp, lon, tra = F.field_components(torch.from_numpy(E), torch.from_numpy(pts))
    for i in range(P):
        phi = math.atan2(pts[i, 1], pts[i, 0])
        assert amp[i].item() == pytest.approx(math.sqrt(abs(E[i, 0]) ** 2 + abs(E[i, 1]) ** 2), rel=1e-14)
        assert complex(lon[i]) == pytest.approx(E[i, 0] * math.cos(phi) - E[i, 1] * math.sin(phi), rel=1e-13)
        assert complex(tra[i]) == pytest.approx(E[i, 0] * math.sin(phi) + E[i, 1] * math.cos(phi), rel=1e-13)


def test_field_components_3d():
    g = np.random.default_rng(4)
    P = 40
    E = g.normal(size=(P, 3)) + 1j * g.normal(size=(P, 3))
    pts = g.normal(size=(P, 3))
    amp, lon, tra = F.field_components(torch.from_numpy(E), torch.from_numpy(pts))
    for i in range(P):
        v = pts[i] / np.linalg.norm(pts[i])
        l_ref = np.sum(E[i] * v)
        assert amp[i].item() == pytest.approx(np.linalg.norm(E[i]), rel=1e-14)
        assert complex(lon[i]) == pytest.approx(l_ref, rel=1e-13)
        assert tra[i].item() == pytest.approx(np.linalg.norm(E[i] - l_ref * v), rel=1e-13)


def test_fieldcache_list_roundtrip(tmp_path):
    g = np.random.default_rng(5)
    Ej = g.normal(size=(30, 4)) + 1j * g.normal(size=(30, 4))
    params = np.array([0.3 + 0.01j, 2 * np.pi * 10])
    points = g.normal(size=(15, 2))
    thetas = np.linspace(0, np.pi, 4)
    path = str(tmp_path / "run_Ek_k0_10.0_0.hkl")
    fc.dump([Ej, params, torch.from_numpy(points), thetas], path)
    assert os.path.isfile(path)          # the driver checks for exactly this name
    Ej2, params2, _, thetas2 = fc.load(path)
    assert np.array_equal(Ej2, Ej) and Ej2.dtype == np.complex128
    assert np.array_equal(params2, params)
    alpha, k0 = params2
    assert complex(alpha) == 0.3 + 0.01j and k0.real == 2 * np.pi * 10
    assert np.array_equal(thetas2, thetas)


def test_fieldcache_array_and_tuple(tmp_path):
    a = np.arange(12.0).reshape(3, 4)
    p = str(tmp_path / "points.hkl")
    fc.dump(a, p)
    b = fc.load(p)
    assert isinstance(b, np.ndarray) and np.array_equal(a, b)
    assert np.array_equal(fc.load(p)[:, 0:2], a[:, 0:2])      # utils.py:808 slices the loaded points
    t = str(tmp_path / "t.hkl")
    fc.dump((a, a + 1), t)
    out = fc.load(t)
    assert isinstance(out, tuple) and np.array_equal(out[1], a + 1)


def test_fieldcache_rejects_hdf5(tmp_path):
    p = tmp_path / "real.hkl"
    p.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes(64))
    with pytest.raises(ValueError):
        fc.load(str(p))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["2d_vector", "3d_vector"])
def test_full_fields_one_call_matches_per_angle(kind):
    """One propagate call over the grid for several incidences equals the
    driver's per-angle calls and the FP64 oracle."""
    from oracle import oracle as O
    from magreete_gb300 import Transmission2D_vector, Transmission3D_vector
    O.BESSEL_MODE = "exact"
    z = np.load(os.path.join(GOLD, f"golden_{kind}.npz"))
    g = {k: z[k] for k in z.files}
    k0, alpha, w = float(g["k0"]), complex(g["alpha"]), float(g["beam_w"])
    pts_s = torch.from_numpy(g["points"])
    dim = 2 if kind.startswith("2d") else 3
    s = (Transmission2D_vector if dim == 2 else Transmission3D_vector)(pts_s, source="plane")
    Ek = torch.from_numpy(g["Ek"])
    grid = F.grid_points(dim, 24, 16, L=2.0 * float(np.abs(g["points"]).max()), window_width=1.0)
    R = Ek.shape[1]
    cols = [0, R // 2, R - 1]

    def source(c):
        if dim == 2:
            return s.generate_source(grid, k0, g["thetas"][c], w)
        return s.generate_source(grid, k0, torch.from_numpy(g["u"][c]), torch.from_numpy(g["p"][c]), w)

    E0 = source(cols)
    E = F.full_fields(s, grid, Ek, cols, E0, k0, alpha)
    assert E.shape == E0.shape and not torch.isnan(E).any()
    for a, c in enumerate(cols):
        Ea = s.propagate(grid, Ek[:, c].unsqueeze(-1), k0, alpha, source([c]))
        assert torch.allclose(E[..., a], Ea[..., 0], rtol=0, atol=1e-12 * Ea.abs().max().item())
    ref = O.propagate(kind, g["points"], grid.numpy(), g["Ek"][:, cols], k0, alpha, E0.numpy())
    diff = np.linalg.norm((E.numpy() - ref).ravel()) / np.linalg.norm(ref.ravel())
    assert diff < 1e-10
    amp, lon, tra = F.field_components(E[..., 0], grid)
    assert amp.shape == (grid.shape[0],) and torch.isfinite(amp).all()
