"""Pin the CPU oracle against golden vectors produced by the reference itself."""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")

# The reference's 2D Green's functions use torch.special Bessel functions,
# which carry up to ~2.4e-6 (envelope-relative) error for 5 <= kR <= 10.  The
# oracle reproduces them exactly in "torch" mode (pinned here at 1e-11); in
# "exact" mode (the FP64 oracle the GPU path is held to) 2D results differ
# from the reference's by that defect, bounded below by TOL_2D_EXACT.
TOL_2D_EXACT = 2e-6


@pytest.fixture(params=["torch", "exact"], autouse=True)
def bessel_mode(request):
    old = O.BESSEL_MODE
    O.BESSEL_MODE = request.param
    yield request.param
    O.BESSEL_MODE = old


def tol(kind, strict):
    if kind.startswith("2d") and O.BESSEL_MODE == "exact":
        return TOL_2D_EXACT
    return strict


def load(kind):
    z = np.load(os.path.join(GOLD, f"golden_{kind}.npz"))
    return {k: z[k] for k in z.files}


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("kind", O.KINDS)
def test_self_terms(kind):
    g = load(kind)
    f = {"2d_vector": O.self_interaction_2d_vector, "2d_scalar": O.self_interaction_2d_scalar,
         "3d_vector": O.self_interaction_3d_vector, "3d_scalar": O.self_interaction_3d_scalar}[kind]
    k0, a = float(g["k0"]), float(g["radius"])
    assert abs(f(k0, a, "Rayleigh") - complex(g["si_rayleigh"])) <= 1e-14 * abs(complex(g["si_rayleigh"]))
    assert abs(f(k0, a, "full") - complex(g["si_full"])) <= 1e-12 * abs(complex(g["si_full"]))
    with pytest.raises(NotImplementedError):
        f(k0, a, "bogus")


@pytest.mark.parametrize("kind", O.KINDS)
def test_greens_matrix(kind):
    g = load(kind)
    pts = g["points"][:12]
    if kind == "2d_scalar":
        G = O.G0(kind, pts, float(g["k0"]), points=pts)
        off = ~np.eye(12, dtype=bool)
        assert rel(G[off], g["G_small"][off]) < tol(kind, 1e-13)
    else:
        G = O.G0(kind, pts, float(g["k0"]))
        assert rel(G, g["G_small"]) < tol(kind, 1e-13)


@pytest.mark.parametrize("kind", O.KINDS)
def test_sources(kind):
    g = load(kind)
    dim, d = O.kind_dims(kind)
    k0, w = float(g["k0"]), float(g["beam_w"])
    if dim == 2:
        E = O.source_2d(kind, "plane", g["points"], k0, g["thetas"], w)
        Eb = O.source_2d(kind, "beam", g["points"], k0, g["thetas"], w)
        Ep = O.source_2d(kind, "point", g["points"], k0, g["thetas"], w)
        assert rel(Ep, g["E0_scat_point"]) < tol(kind, 1e-13)
    else:
        E = O.source_3d(kind, "plane", g["points"], k0, g["u"], g["p"], w)
        Eb = O.source_3d(kind, "beam", g["points"], k0, g["u"], g["p"], w)
        with pytest.raises(NotImplementedError):
            O.source_3d(kind, "point", g["points"], k0, g["u"], g["p"], w)
    assert rel(E, g["E0_scat"]) < 1e-14
    assert rel(Eb, g["E0_scat_beam"]) < 1e-14


@pytest.mark.parametrize("kind", O.KINDS)
def test_solve(kind):
    g = load(kind)
    args = (kind, g["points"], float(g["k0"]), complex(g["alpha"]), float(g["radius"]), g["E0_scat"])
    assert rel(O.solve(*args), g["Ek"]) < tol(kind, 1e-12)
    assert rel(O.solve(*args, self_interaction=False), g["Ek_no_self"]) < tol(kind, 1e-12)
    assert rel(O.solve(*args, si_type="full"), g["Ek_full"]) < tol(kind, 1e-12)


@pytest.mark.parametrize("kind", O.KINDS)
def test_propagate(kind):
    g = load(kind)
    k0, alpha, a = float(g["k0"]), complex(g["alpha"]), float(g["radius"])
    E = O.propagate(kind, g["points"], g["det"], g["Ek"], k0, alpha, g["E0_det"])
    assert not np.isnan(E).any()
    assert rel(E, g["E_det"]) < tol(kind, 1e-12)
    E = O.propagate(kind, g["points"], g["det"], g["Ek"], k0, alpha, g["E0_det"], regularize=True, radius=a)
    assert rel(E, g["E_det_reg"]) < tol(kind, 1e-12)
    E = O.propagate_ss(kind, g["points"], g["det"], k0, alpha, g["E0_det"], g["E0_scat"])
    assert rel(E, g["E_ss"]) < tol(kind, 1e-12)


@pytest.mark.parametrize("kind", O.KINDS)
def test_mean_dos_and_ldos(kind):
    g = load(kind)
    k0, alpha, a = float(g["k0"]), complex(g["alpha"]), float(g["radius"])
    t = tol(kind, 1e-11)
    d = O.mean_dos(kind, g["points"], g["dos_pts"], k0, alpha, a)
    assert abs(d - float(g["dos"])) <= t * abs(float(g["dos"]))
    d = O.mean_dos(kind, g["points"], g["dos_pts_hit"], k0, alpha, a)
    assert abs(d - float(g["dos_hit"])) <= t * abs(float(g["dos_hit"]))
    d = O.mean_dos(kind, g["points"], g["dos_pts"], k0, alpha, a, regularize=True, discard_absorption=True)
    assert abs(d - float(g["dos_reg"])) <= t * abs(float(g["dos_reg"]))
    l = O.ldos(kind, g["points"], g["dos_pts"][:8], k0, alpha, a)
    assert rel(l, g["ldos"]) < t


def test_known_answers():
    """Single scatterer: Ek = E0 / (1 - k^2 alpha S/V); M is complex symmetric."""
    k0, a = 2 * np.pi * 3.0, 0.03
    for kind in O.KINDS:
        dim, d = O.kind_dims(kind)
        V = O.scatterer_volume(kind, a)
        alpha = V * (1.6 ** 2 - 1)
        pts = np.zeros((1, dim))
        E0 = np.ones((d, 2), np.complex128)
        Ek = O.solve(kind, pts, k0, alpha, a, E0)
        ref = E0 / (1 - O.diagonal_self_shift(kind, k0, alpha, a))
        assert rel(Ek, ref) < 1e-14
        rng = np.random.default_rng(0)
        P = rng.random((20, dim))
        Mt = O.system_matrix(kind, P, k0, alpha, a)
        assert rel(Mt, Mt.T) < 1e-14


@pytest.mark.parametrize("kind", O.KINDS)
def test_greens_of_separations_periodic_and_regularised(kind):
    """torch_greens / greens on an array of separations (free, each periodic
    option, regularised) against the reference's outputs.  Non-finite entries
    (a regularised separation at zero) must sit in the same places."""
    z = np.load(os.path.join(GOLD, f"golden_greens_{kind}.npz"))
    r, k0 = z["r"], float(z["k0"])
    for i, per in enumerate(z["periodic_options"]):
        G = O.greens_separations(kind, r, k0, periodic=str(per))
        assert G.shape == z[f"G_{i}"].shape
        assert rel(G, z[f"G_{i}"]) < tol(kind, 1e-13), per
    G = O.greens_separations(kind, r, k0, regularize=True, radius=float(z["radius_reg"]))
    ref = z["G_reg"]
    fin = np.isfinite(ref)
    assert np.array_equal(np.isfinite(G), fin) and not fin.all()
    assert rel(G[fin], ref[fin]) < tol(kind, 1e-13)
    # the reference's wrap changes the answer: periodic and free calls differ
    assert not np.allclose(z["G_0"], z["G_1"])
