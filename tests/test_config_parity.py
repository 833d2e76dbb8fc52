"""GPU parity at the sizes of the benchmark configurations, against the CPU oracle.

The oracle (numpy/scipy complex128, exact Bessel functions) runs on the host
in the test itself, on the same seeded inputs as the GPU:
  * 2D TE, N = 1000 in the unit disk, k0 L = 2 pi 20, 64 plane-wave angles,
    360 detectors on the ring at 2L, mean DOS at 8 frequencies over 1000
    points (Transmission2D.py:93-231, :176-205, :282-336; magreete.py:371-400,
    :885-892);
  * 3D dyadic, N = 4000 in the unit cube (n = 12000), k0 L = 2 pi 10,
    32 directions x 2 polarisations, 1024 Fibonacci detectors
    (Transmission3D.py:79-206, :147-179);
  * the large strong-scattering 3D case (unit ball, n = 2.0, k0 L = 2 pi 15,
    128 right-hand sides) at N = 2000 (n = 6000), fields and mean DOS: the
    full N = 20000 case does not fit the host oracle, and its FP64 answer is
    the GPU's plain method, which this test holds to the oracle first.

Tolerances (relative, Frobenius over all fields; DOS per frequency):
  plain FP64 method 1e-10 (DOS 1e-9); mixed method 1e-8.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "mixed": 1e-8}
TOL_DOS = {"fp64": 1e-9, "mixed": 1e-8}


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(autouse=True)
def exact_bessel():
    O.BESSEL_MODE = "exact"
    yield


def oracle_request(prob):
    """Incident fields, fields at the scatterers and detector fields of the oracle."""
    pts, det = prob.points.numpy(), prob.detectors.numpy()
    if prob.kind.startswith("2d"):
        E0s = O.source_2d(prob.kind, "plane", pts, prob.k0, prob.thetas, 0.2)
        E0d = O.source_2d(prob.kind, "plane", det, prob.k0, prob.thetas, 0.2)
    else:
        E0s = O.source_3d(prob.kind, "plane", pts, prob.k0, prob.u.numpy(), prob.p.numpy(), 0.2)
        E0d = O.source_3d(prob.kind, "plane", det, prob.k0, prob.u.numpy(), prob.p.numpy(), 0.2)
    Ek = O.solve(prob.kind, pts, prob.k0, prob.alpha, prob.radius, E0s)
    Ed = O.propagate(prob.kind, pts, det, Ek, prob.k0, prob.alpha, E0d)
    return E0s, Ek, Ed


def gpu_request(prob, precision):
    """The same request through the drop-in classes, as the driver makes it:
    generate_source x2 -> solve -> propagate (magreete.py:371-400)."""
    from magreete_gb300 import Transmission2D_vector, Transmission3D_vector
    pts, det = prob.points, prob.detectors
    if prob.kind.startswith("2d"):
        s = Transmission2D_vector(pts, source="plane", precision=precision)
        E0s = s.generate_source(pts, prob.k0, prob.thetas, 0.2)
        E0d = s.generate_source(det, prob.k0, prob.thetas, 0.2)
    else:
        s = Transmission3D_vector(pts, source="plane", precision=precision)
        E0s = s.generate_source(pts, prob.k0, prob.u, prob.p, 0.2)
        E0d = s.generate_source(det, prob.k0, prob.u, prob.p, 0.2)
    Ek = s.solve(prob.k0, prob.alpha, prob.radius, E0s)
    stats = dict(s.last_stats)
    Ed = s.propagate(det, Ek, prob.k0, prob.alpha, E0d)
    return s, E0s, Ek, Ed, stats


@pytest.fixture(scope="module")
def cfg1():
    from magreete_gb300 import workloads as W
    prob = W.cfg1()
    return prob, oracle_request(prob)


@pytest.fixture(scope="module")
def cfg2():
    from magreete_gb300 import workloads as W
    prob = W.cfg2()
    return prob, oracle_request(prob)


@pytest.fixture(scope="module")
def ball2000():
    from magreete_gb300 import workloads as W
    prob = W.ball_problem(2000, 4, 15.0)
    return prob, oracle_request(prob)


def check_request(prob, ref, precision):
    E0s_ref, Ek_ref, Ed_ref = ref
    s, E0s, Ek, Ed, stats = gpu_request(prob, precision)
    assert rel(E0s, E0s_ref) < 1e-13
    assert Ek.shape == Ek_ref.shape and Ed.shape == Ed_ref.shape
    assert rel(Ek, Ek_ref) < TOL[precision]
    assert rel(Ed, Ed_ref) < TOL[precision]
    if precision == "mixed":
        assert stats["rel_residual"] <= 1e-10
    return s, Ek


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_2d_te_N1000_transmission(cfg1, precision):
    """64 angles, 360 detectors."""
    prob, ref = cfg1
    assert prob.n == 2000 and prob.nrhs == 64 and prob.detectors.shape[0] == 360
    check_request(prob, ref, precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_2d_te_N1000_mean_dos_8_frequencies(cfg1, precision):
    """Mean DOS over 1000 points in the disk of radius L/2 at k0 L / 2 pi =
    18.5 .. 22 (the driver's loop, magreete.py:885-892)."""
    from magreete_gb300 import Transmission2D_vector
    from magreete_gb300 import workloads as W
    prob, _ = cfg1
    mp = W.dos_points_cfg1()
    s = Transmission2D_vector(prob.points, source="plane", precision=precision)
    for k0 in W.dos_frequencies_cfg1():
        got = float(s.mean_DOS_measurements(mp, k0, prob.alpha, prob.radius))
        ref = O.mean_dos(prob.kind, prob.points.numpy(), mp.numpy(), k0, prob.alpha, prob.radius)
        assert abs(got - ref) <= TOL_DOS[precision] * abs(ref), (k0, got, ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_3d_N4000_transmission(cfg2, precision):
    """n = 12000, 64 right-hand sides, 1024 detectors."""
    prob, ref = cfg2
    assert prob.n == 12000 and prob.nrhs == 64 and prob.detectors.shape[0] == 1024
    check_request(prob, ref, precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_3d_ball_strong_scattering_N2000(ball2000, precision):
    """n = 2.0, 128 right-hand sides: fields, and the mean DOS at 40 points."""
    from magreete_gb300 import workloads as W
    prob, ref = ball2000
    assert prob.nrhs == 128
    s, _ = check_request(prob, ref, precision)
    mp = 0.5 * W.ball_points(40, 77)
    got = float(s.mean_DOS_measurements(mp, prob.k0, prob.alpha, prob.radius))
    want = O.mean_dos(prob.kind, prob.points.numpy(), mp.numpy(), prob.k0, prob.alpha, prob.radius)
    assert abs(got - want) <= TOL_DOS[precision] * abs(want)
