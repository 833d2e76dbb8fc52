"""Generate golden vectors from the unmodified MAGreeTe reference classes.

Run from the repository root on a machine that has the reference checkout:

    python tests/golden/make_golden.py /root/reference            # golden_<kind>.npz
    python tests/golden/make_golden.py /root/reference --greens   # golden_greens_<kind>.npz
    python tests/golden/make_golden.py /root/reference --spectral # golden_spectral_<kind>.npz

The reference imports ``hickle``, ``matplotlib`` and ``cmasher`` at module
level; none of them is used on the solve path, so empty stand-in modules are
registered before the import.  Inputs are small seeded point patterns; every
array the tests need (inputs and reference outputs) is written to one
``golden_<kind>.npz`` file per solver class.  The committed fixtures are the
ground truth that pins both the CPU oracle and the CUDA path.
"""
import contextlib
import io
import os
import sys
import types

import numpy as np


def _stub_modules():
    for name in ["hickle", "matplotlib", "matplotlib.pyplot", "matplotlib.colors", "cmasher"]:
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["matplotlib"].use = lambda *a, **k: None
    sys.modules["matplotlib.pyplot"].rc = lambda *a, **k: None
    sys.modules["cmasher"].ember = None


def _points_disk(rng, n, L=1.0):
    u1, u2 = rng.random(n), rng.random(n)
    return np.stack([np.sqrt(u2) * np.cos(2 * np.pi * u1), np.sqrt(u2) * np.sin(2 * np.pi * u1)], 1) * L


def _points_ball(rng, n):
    g = rng.standard_normal((n, 3))
    e = rng.exponential(size=(n, 1))
    return g / np.sqrt(np.sum(g * g, 1, keepdims=True) + e)


def main(ref_path):
    _stub_modules()
    sys.path.insert(0, ref_path)
    import torch
    import utils  # first: utils and the solver modules import each other
    from Transmission2D import Transmission2D_vector, Transmission2D_scalar
    from Transmission2D import self_interaction_integral_vector as si2v, self_interaction_integral_scalar as si2s
    from Transmission3D import Transmission3D_vector, Transmission3D_scalar
    from Transmission3D import self_interaction_integral_vector as si3v, self_interaction_integral_scalar as si3s

    out_dir = os.path.dirname(os.path.abspath(__file__))
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a))

    cases = {
        "2d_vector": (Transmission2D_vector, 2, 150, 2 * np.pi * 6.0, 1.6 + 0.0j, 0.05),
        "2d_scalar": (Transmission2D_scalar, 2, 150, 2 * np.pi * 6.0, 1.6 + 0.01j, 0.05),
        "3d_vector": (Transmission3D_vector, 3, 90, 2 * np.pi * 3.0, 1.6 + 0.0j, 0.1),
        "3d_scalar": (Transmission3D_scalar, 3, 90, 2 * np.pi * 3.0, 1.6 + 0.02j, 0.1),
    }
    for seed, (kind, (cls, dim, N, k0, n_ref, phi)) in enumerate(cases.items()):
        rng = np.random.default_rng(100 + seed)
        if dim == 2:
            pts = _points_disk(rng, N)
            volume = phi * np.pi / N
            radius = np.sqrt(volume / np.pi)
        else:
            pts = rng.random((N, 3)) - 0.5
            volume = phi / N
            radius = np.cbrt(3 * volume / (4 * np.pi))
        alpha = complex(utils.alpha_small_dielectric_object(n_ref, volume))
        R = 5
        thetas = np.arange(R) / R * 2 * np.pi + 0.1
        # detectors: ring / sphere at 2L, plus two that sit exactly on scatterers,
        # plus one within `radius` of a scatterer (for the regularised case)
        if dim == 2:
            ring = 2.0 * np.stack([np.cos(np.arange(24) / 24 * 2 * np.pi), np.sin(np.arange(24) / 24 * 2 * np.pi)], 1)
        else:
            ring = 2.0 * utils.fibonacci_sphere(24)
        near = pts[7] + 0.3 * radius / np.sqrt(dim)
        det = np.concatenate([ring, pts[[3, 11]], near[None]], 0)
        dos_pts = 0.5 * (_points_disk(rng, 40) if dim == 2 else _points_ball(rng, 40))
        dos_pts_hit = np.concatenate([dos_pts, pts[[5]]], 0)

        solver = cls(T(pts), source="plane")
        res = {}
        with contextlib.redirect_stdout(io.StringIO()):
            if dim == 2:
                E0s = solver.generate_source(T(pts), k0, thetas, 0.2)
                E0d = solver.generate_source(T(det), k0, thetas, 0.2)
                solver.source = "beam"
                E0s_beam = solver.generate_source(T(pts), k0, thetas, 0.2)
                solver.source = "point"
                E0s_point = solver.generate_source(T(pts), k0, thetas, 0.2)
                solver.source = "plane"
                u = p = np.zeros((0, 3))
            else:
                u, p = utils.vector_3d_u_and_p(thetas, polarization_angle_radians=0.3)
                u, p = u.numpy(), p.numpy()
                if kind == "3d_vector":
                    E0s = solver.generate_source(T(pts), k0, T(u), T(p), 0.2)
                    E0d = solver.generate_source(T(det), k0, T(u), T(p), 0.2)
                    solver.source = "beam"
                    E0s_beam = solver.generate_source(T(pts), k0, T(u), T(p), 0.2)
                    E0s_point = torch.zeros(1)
                else:
                    E0s = solver.generate_source(T(pts), k0, T(u), 0.2)
                    E0d = solver.generate_source(T(det), k0, T(u), 0.2)
                    solver.source = "beam"
                    E0s_beam = solver.generate_source(T(pts), k0, T(u), 0.2)
                    # the 3D point sources fail inside the reference
                    # (Transmission3D.py:136 and :649), so none is recorded
                    E0s_point = torch.zeros(1)
                solver.source = "plane"
            Ek = solver.solve(k0, alpha, radius, E0s)
            Ek_rayleigh_off = solver.solve(k0, alpha, radius, E0s, self_interaction=False)
            Ek_full = solver.solve(k0, alpha, radius, E0s, self_interaction_type="full")
            Ed = solver.propagate(T(det), Ek, k0, alpha, E0d)
            Ed_reg = solver.propagate(T(det), Ek, k0, alpha, E0d, regularize=True, radius=radius)
            # the 3D vector propagate_ss multiplies by E0_scat without reshaping it
            # (Transmission3D.py:223), so it is handed the (3N, R) form here
            Ess = solver.propagate_ss(T(det), k0, alpha, E0d, E0s.reshape(E0s.shape[0] * (3 if kind == "3d_vector" else 1), -1)
                                      if kind == "3d_vector" else E0s)
            dos = solver.mean_DOS_measurements(T(dos_pts), k0, alpha, radius)
            dos_hit = solver.mean_DOS_measurements(T(dos_pts_hit), k0, alpha, radius)
            dos_reg = solver.mean_DOS_measurements(T(dos_pts), k0, alpha, radius, regularize=True, discard_absorption=True)
            ldos = solver.LDOS_measurements(T(dos_pts[:8]), k0, alpha, radius)
            # the scatterer-scatterer propagator of a 12-point subset
            small = cls(T(pts[:12]), source="plane")
            if kind == "2d_vector":
                G_small = small.G0_vector(None, k0)
            elif kind == "2d_scalar":
                G_small = small.G0(T(pts[:12]), k0)
            else:
                G_small = small.G0(None, k0)
        si = {"2d_vector": si2v, "2d_scalar": si2s, "3d_vector": si3v, "3d_scalar": si3s}[kind]
        res.update(
            points=pts, k0=k0, alpha=alpha, radius=radius, thetas=thetas, u=u, p=p, det=det,
            dos_pts=dos_pts, dos_pts_hit=dos_pts_hit, beam_w=0.2,
            E0_scat=E0s.numpy(), E0_det=E0d.numpy(), E0_scat_beam=E0s_beam.numpy(), E0_scat_point=E0s_point.numpy(),
            Ek=Ek.numpy(), Ek_no_self=Ek_rayleigh_off.numpy(), Ek_full=Ek_full.numpy(),
            E_det=Ed.numpy(), E_det_reg=Ed_reg.numpy(), E_ss=Ess.numpy(),
            dos=float(dos), dos_hit=float(dos_hit), dos_reg=float(dos_reg), ldos=ldos.numpy(),
            G_small=G_small.numpy(),
            si_rayleigh=complex(si(k0, radius, "Rayleigh")), si_full=complex(si(k0, radius, "full")),
        )
        path = os.path.join(out_dir, f"golden_{kind}.npz")
        np.savez_compressed(path, **res)
        print("wrote", path, os.path.getsize(path), "bytes")


def main_greens(ref_path):
    """golden_greens_<kind>.npz: the classes' Green's function on an array of
    separations (torch_greens / greens), free and with each periodic option,
    plus one regularised call in which the shortest separation falls under the
    threshold.  Separate files, so the fixtures above stay as they are."""
    _stub_modules()
    sys.path.insert(0, ref_path)
    import torch
    import utils  # noqa: F401 -- first: utils and the solver modules import each other
    from Transmission2D import Transmission2D_vector, Transmission2D_scalar
    from Transmission3D import Transmission3D_vector, Transmission3D_scalar

    out_dir = os.path.dirname(os.path.abspath(__file__))
    classes = {"2d_vector": (Transmission2D_vector, 2, ("", "x", "y", "xy")),
               "2d_scalar": (Transmission2D_scalar, 2, ("", "x", "y", "xy")),
               "3d_vector": (Transmission3D_vector, 3, ("", "x", "xy", "xyz")),
               "3d_scalar": (Transmission3D_scalar, 3, ("", "x", "xy", "xyz"))}
    k0 = 2 * np.pi * 3.0
    for seed, (kind, (cls, dim, options)) in enumerate(classes.items()):
        rng = np.random.default_rng(500 + seed)
        r = rng.uniform(-1.2, 1.2, size=(5, 4, dim))
        r[0, 0] = 0.01                       # a short separation for the regularised call
        # the 2D vector class compares k*R with the radius (a quirk), the others R
        radius_reg = 0.5 if kind == "2d_vector" else 0.03
        solver = cls(torch.from_numpy(rng.random((3, dim))), source="plane")
        fn = solver.torch_greens if dim == 2 else solver.greens
        res = {"r": r, "k0": k0, "radius_reg": radius_reg, "periodic_options": np.array(options)}
        with contextlib.redirect_stdout(io.StringIO()):
            for i, per in enumerate(options):
                # the reference wraps its argument in place: hand it a copy
                res[f"G_{i}"] = fn(torch.from_numpy(r.copy()), k0, periodic=per).numpy()
            res["G_reg"] = fn(torch.from_numpy(r.copy()), k0, regularize=True, radius=radius_reg).numpy()
        path = os.path.join(out_dir, f"golden_greens_{kind}.npz")
        np.savez_compressed(path, **res)
        print("wrote", path, os.path.getsize(path), "bytes")


def main_spectral(ref_path):
    """golden_spectral_<kind>.npz: the spectral tools of each class
    (compute_hamiltonian_DOS, compute_eigenvalues_and_scatterer_LDOS,
    compute_eigenmodes_IPR with both sortings) on a small seeded pattern: their
    return values and the CSV files they write.  The plots of
    compute_eigenmodes_IPR (utils.plot_IPR_damping_values, matplotlib) are
    replaced by a no-op."""
    import tempfile
    _stub_modules()
    sys.path.insert(0, ref_path)
    import torch
    import utils
    from Transmission2D import Transmission2D_vector, Transmission2D_scalar
    from Transmission3D import Transmission3D_vector, Transmission3D_scalar
    utils.plot_IPR_damping_values = lambda *a, **k: None

    out_dir = os.path.dirname(os.path.abspath(__file__))
    cases = {
        "2d_vector": (Transmission2D_vector, 2, 40, 2 * np.pi * 4.0, 1.6 + 0.0j, 0.05),
        "2d_scalar": (Transmission2D_scalar, 2, 40, 2 * np.pi * 4.0, 1.6 + 0.01j, 0.05),
        "3d_vector": (Transmission3D_vector, 3, 24, 2 * np.pi * 2.0, 1.6 + 0.0j, 0.1),
        "3d_scalar": (Transmission3D_scalar, 3, 24, 2 * np.pi * 2.0, 1.6 + 0.02j, 0.1),
    }
    for seed, (kind, (cls, dim, N, k0, n_ref, phi)) in enumerate(cases.items()):
        rng = np.random.default_rng(900 + seed)
        if dim == 2:
            pts = _points_disk(rng, N)
            volume = phi * np.pi / N
            radius = np.sqrt(volume / np.pi)
        else:
            pts = rng.random((N, 3)) - 0.5
            volume = phi / N
            radius = np.cbrt(3 * volume / (4 * np.pi))
        alpha = complex(utils.alpha_small_dielectric_object(n_ref, volume))
        deltas_grid = np.linspace(-3.0, 3.0, 13)
        solver = cls(torch.from_numpy(pts), source="plane")
        res = {"points": pts, "k0": k0, "alpha": alpha, "radius": radius, "deltas_grid": deltas_grid}
        with tempfile.TemporaryDirectory() as tmp, contextlib.redirect_stdout(io.StringIO()):
            base = os.path.join(tmp, "spec")
            dos = solver.compute_hamiltonian_DOS(k0, torch.from_numpy(deltas_grid), base)
            res["hamiltonian_dos"] = dos.numpy()
            res["ldos_factor"] = float(solver.compute_eigenvalues_and_scatterer_LDOS(k0, alpha, radius, base))
            res["ldos_factor_no_self"] = float(solver.compute_eigenvalues_and_scatterer_LDOS(
                k0, alpha, radius, base + "_ns", self_interaction=False, write_eigenvalues=False))
            for sorting in ("IPR", "damping"):
                vals, vecs, iprs = solver.compute_eigenmodes_IPR(k0, alpha, radius, base + "_" + sorting,
                                                                 number_eigenmodes=3, sorting_type=sorting)
                res[f"ipr_{sorting}_values"] = vals.numpy()
                res[f"ipr_{sorting}_vectors"] = vecs.numpy()
                res[f"ipr_{sorting}_iprs"] = iprs.numpy()
            # the files written, by name relative to the base
            for name in sorted(os.listdir(tmp)):
                key = "csv:" + name[len("spec"):]
                res[key] = np.loadtxt(os.path.join(tmp, name))
        path = os.path.join(out_dir, f"golden_spectral_{kind}.npz")
        np.savez_compressed(path, **res)
        print("wrote", path, os.path.getsize(path), "bytes", sorted(k for k in res if k.startswith("csv:")))


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref = args[0] if args else os.environ.get("MAGREETE_REFERENCE", "reference")
    if "--greens" in sys.argv:
        main_greens(ref)
    elif "--spectral" in sys.argv:
        main_spectral(ref)
    else:
        main(ref)
