"""Seeded synthetic workloads (point patterns, frequencies, sources, detectors).

The reference has no benchmark suite; these generators produce inputs with
the shapes and distributions of its own driver and samplers, seeded with a
CPU ``torch.Generator`` so every run (CPU or GPU) sees bit-identical points:
  * uniform points in the unit disk: r = sqrt(U2), phi = 2 pi U1
    (utils.uniform_unit_disk_picking, utils.py:85-98);
  * uniform points in a cube [-1/2, 1/2]^3 (lattices.poisson, lattices.py:29-31);
  * points in the unit ball as the reference draws them: x / sqrt(|x|^2 + E),
    x Gaussian, E exponential with mean 1 (utils.uniform_unit_ball_picking,
    utils.py:100-115).  The method it cites is uniform for E of mean 2; with
    mean 1 the points sit further out (E[r^3] = 0.63 instead of 0.5), and the
    workload keeps the reference's distribution;
  * detectors: a ring of 360 at radius 2L (magreete.py:351-353) or a
    Fibonacci sphere (utils.fibonacci_sphere, utils.py:117-136);
  * polarisability of a small dielectric object alpha = V (n^2 - 1)
    (utils.alpha_small_dielectric_object, utils.py:67-83).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np
import torch


def _gen(seed):
    return torch.Generator().manual_seed(int(seed))


def disk_points(N, seed, L=1.0):
    g = _gen(seed)
    u1 = torch.rand(N, dtype=torch.float64, generator=g)
    u2 = torch.rand(N, dtype=torch.float64, generator=g)
    return torch.stack([torch.sqrt(u2) * torch.cos(2 * math.pi * u1), torch.sqrt(u2) * torch.sin(2 * math.pi * u1)], 1) * L


def cube_points(N, seed):
    return torch.rand(N, 3, dtype=torch.float64, generator=_gen(seed)) - 0.5


def ball_points(N, seed, dim=3):
    g = _gen(seed)
    normals = torch.randn(N, dim, dtype=torch.float64, generator=g)
    exps = -torch.log(torch.rand(N, 1, dtype=torch.float64, generator=g))
    proxies = torch.cat([normals, torch.sqrt(exps)], 1)
    return normals / torch.linalg.norm(proxies, dim=-1).reshape(N, 1)


def ring(M=360, radius=2.0):
    t = np.arange(M) / M * 2 * np.pi
    return torch.from_numpy(radius * np.stack([np.cos(t), np.sin(t)], 1))


def fibonacci_sphere(M=1024, radius=1.0):
    golden = np.pi * (np.sqrt(5.0) - 1.0)
    i = np.arange(M)
    z = 1 - (i / (M - 1)) * 2
    rr = np.sqrt(1 - z ** 2)
    th = i * golden
    return torch.from_numpy(radius * np.stack([np.cos(th) * rr, np.sin(th) * rr, z], 1))


def directions_3d(n_dirs, pol_angles=(0.0, np.pi / 2)):
    """n_dirs directions in the Oxy plane x polarisation angles, as
    utils.vector_3d_u_and_p (utils.py:138-162): R = n_dirs * len(pol_angles)."""
    th = np.arange(n_dirs) / n_dirs * 2 * np.pi
    us, ps = [], []
    for pa in pol_angles:
        u = np.stack([np.cos(th), np.sin(th), np.zeros_like(th)], 1)
        e_alt = np.zeros_like(u)
        e_alt[:, 2] = 1
        e_az = np.stack([np.sin(th), -np.cos(th), np.zeros_like(th)], 1)
        us.append(u)
        ps.append(e_alt * np.cos(pa) + e_az * np.sin(pa))
    return torch.from_numpy(np.concatenate(us)), torch.from_numpy(np.concatenate(ps))


@dataclasses.dataclass
class Problem:
    """One coupled-dipole solve: geometry, frequency, sources, detectors."""
    kind: str
    points: torch.Tensor          # (N, dim) float64, CPU
    k0: float
    alpha: complex
    radius: float
    thetas: np.ndarray = None     # 2D incidence angles
    u: torch.Tensor = None        # 3D directions (R, 3)
    p: torch.Tensor = None        # 3D polarisations (R, 3)
    detectors: torch.Tensor = None
    arrival: float = 0.0          # seconds after the stream starts
    requery_of: int = -1          # index of the request whose geometry this one reuses
    seed: int = 0

    @property
    def N(self):
        return self.points.shape[0]

    @property
    def d(self):
        return {"2d_vector": 2, "2d_scalar": 1, "3d_vector": 3, "3d_scalar": 1}[self.kind]

    @property
    def n(self):
        return self.d * self.N

    @property
    def nrhs(self):
        return len(self.thetas) if self.kind.startswith("2d") else self.u.shape[0]


def disk_problem(N, seed, kL_over_2pi, n_ref=1.6, phi=0.05, n_angles=64, kind="2d_vector", n_det=360):
    """2D TE in the unit disk (the 2D transmission config)."""
    V = phi * math.pi / N
    a = math.sqrt(V / math.pi)
    return Problem(kind, disk_points(N, seed), 2 * math.pi * kL_over_2pi, complex(V * (n_ref ** 2 - 1)), a,
                   thetas=np.arange(n_angles) / n_angles * 2 * np.pi, detectors=ring(n_det, 2.0), seed=seed)


def cube_problem(N, seed, kL_over_2pi, n_ref=1.6, phi=0.1, n_dirs=32, kind="3d_vector", n_det=1024):
    """3D dyadic in the unit cube (the 3D transmission config)."""
    V = phi / N
    a = (3 * V / (4 * math.pi)) ** (1 / 3)
    u, p = directions_3d(n_dirs)
    return Problem(kind, cube_points(N, seed), 2 * math.pi * kL_over_2pi, complex(V * (n_ref ** 2 - 1)), a,
                   u=u, p=p, detectors=fibonacci_sphere(n_det, 3.0), seed=seed)


def cfg1():
    """2D TE, N=1000 in the unit disk, k0 L = 2 pi 20, n=1.6, phi=0.05, 64 angles, 360 detectors."""
    return disk_problem(1000, 1, 20.0)


def cfg2():
    """3D dyadic, N=4000 in the unit cube, k0 L = 2 pi 10, n=1.6, phi=0.1, 32 dirs x 2 pols, 1024 detectors."""
    return cube_problem(4000, 2, 10.0)


def sweep_2d(count=256, seed=1000):
    """Batched 2D sweep: `count` TE disk instances, N uniform in [500, 4000]
    (seeded per instance), k0 L uniform in [2 pi 5, 2 pi 30], 16 angles,
    phi = 0.05, n = 1.6."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        N = int(rng.integers(500, 4001))
        kl = float(rng.uniform(5.0, 30.0))
        out.append(disk_problem(N, seed + i, kl, n_angles=16))
    return out


def ball_problem(N, seed, kL_over_2pi, n_ref=2.0, phi=0.1, n_dirs=64, kind="3d_vector", n_det=1024):
    """3D dyadic in the unit ball (the large strong-scattering config): phi is
    the volume fraction of the ball, n = 2.0."""
    V = phi * (4 * math.pi / 3) / N
    a = (3 * V / (4 * math.pi)) ** (1 / 3)
    u, p = directions_3d(n_dirs)
    return Problem(kind, ball_points(N, seed), 2 * math.pi * kL_over_2pi, complex(V * (n_ref ** 2 - 1)), a,
                   u=u, p=p, detectors=fibonacci_sphere(n_det, 3.0), seed=seed)


def cfg4():
    """3D dyadic, N=20000 in the unit ball, k0 L = 2 pi 15, n=2.0, phi=0.1, 64 dirs x 2 pols."""
    return ball_problem(20000, 4, 15.0)


def dos_frequencies_cfg1():
    """k0 L / 2 pi = 18.5, 19, ..., 22 (the driver's 0.5 step, magreete.py:243)."""
    return [2 * math.pi * f for f in np.arange(18.5, 22.01, 0.5)]


def dos_points_cfg1(P=1000, seed=11):
    """P points uniform in the disk of radius L/2 (magreete.py:877-878)."""
    return 0.5 * disk_points(P, seed)


def serving_stream(n_requests, seed=5, rate=200.0, n_min=500, n_max=16000, requery=0.2):
    """Mixed 2D/3D request stream: Poisson arrivals at `rate`/s, N log-uniform
    in [n_min, n_max], k0 L uniform in [2 pi 5, 2 pi 25], 1-64 right-hand
    sides, a fraction `requery` re-using an earlier request's geometry at a
    new frequency.  2D requests follow the disk config, 3D the cube config."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate)
        kL = rng.uniform(5.0, 25.0)
        R = int(rng.integers(1, 65))
        if out and rng.random() < requery:
            j = int(rng.integers(0, len(out)))
            base = out[j]
            prob = dataclasses.replace(base, k0=2 * math.pi * kL, arrival=t, requery_of=j)
            if base.kind.startswith("2d"):
                prob.thetas = np.arange(R) / R * 2 * np.pi
            else:
                u, p = directions_3d(max(1, R // 2) if R > 1 else 1, (0.0, np.pi / 2) if R > 1 else (0.0,))
                prob.u, prob.p = u, p
            out.append(prob)
            continue
        N = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        s = int(seed * 100003 + i)
        if rng.random() < 0.5:
            prob = disk_problem(N, s, kL, n_angles=R)
        else:
            nd = max(1, R // 2) if R > 1 else 1
            prob = cube_problem(N, s, kL, n_dirs=nd)
            if R == 1:
                u, p = directions_3d(1, (0.0,))
                prob.u, prob.p = u, p
        prob.arrival = t
        out.append(prob)
    return out
