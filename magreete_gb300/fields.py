"""Full-field images: fields on a pixel grid around the sample.

The MAGreeTe driver images |E| and its longitudinal / transverse parts on a
``ngridx x ngridy`` grid (magreete.py:570-741).  It splits the grid into
batches and calls ``propagate`` once per batch and per plotted angle, because
the reference builds the dense (grid x scatterers) Green's matrix in host
memory.  ``propagate`` here is matrix-free on the GPU (propagator rows are
built in chunks of at most 1 GiB), so the whole grid and every plotted angle
go in ONE call, with the angles as right-hand-side columns.

    pts = grid_points(2, 301, 301, L, window_width)
    cols = [column_of_angle(thetas, a) for a in thetas_plot]
    E0 = solver.generate_source(pts, k0, thetas[cols], w)        # (P, d, A)
    E = full_fields(solver, pts, Ej, cols, E0, k0, alpha)        # (P, d, A)
    amp, lon, tra = field_components(E[..., 0], pts)
"""
from __future__ import annotations

import numpy as np
import torch


def grid_points(ndim, ngridx, ngridy, L, window_width=1.0, slice_coordinate=0):
    """The driver's image grid (magreete.py:575-581), float64 (ngridy * ngridx, ndim).

    x spans [-r/2, r/2] with r = ngridx / ngridy and y spans [-1/2, 1/2], both
    times L * window_width; points run along x first.  In 3D the grid is the
    plane z = 0 with the coordinates rolled by ``slice_coordinate`` (0: z = 0,
    1: x = 0, 2: y = 0)."""
    ratio = ngridx / ngridy
    xs = np.linspace(0, ratio, ngridx) - ratio / 2.0
    ys = np.linspace(0, 1, ngridy) - 0.5
    if ndim == 2:
        x, y = np.meshgrid(xs, ys)
        pts = np.vstack([x.ravel(), y.ravel()]).T
    elif ndim == 3:
        x, y, z = np.roll(np.meshgrid(xs, ys, [0.0]), slice_coordinate, axis=0)
        pts = np.vstack([x.ravel(), y.ravel(), z.ravel()]).T
    else:
        raise ValueError(f"ndim must be 2 or 3, not {ndim}")
    return torch.from_numpy(pts * L * window_width)


def column_of_angle(thetas, angle):
    """Column of ``thetas`` holding ``angle`` (magreete.py:652: the first
    with (theta - angle)^2 < 1e-8)."""
    th = np.asarray(thetas.cpu() if isinstance(thetas, torch.Tensor) else thetas, dtype=np.float64).ravel()
    hits = np.nonzero((th - float(angle)) ** 2 < 1e-8)[0]
    if hits.size == 0:
        raise ValueError(f"angle {angle} is not one of the solved incidences")
    return int(hits[0])


def full_fields(solver, points, Ej, columns, E0, k0, alpha, regularize=False, radius=0.0):
    """Total field at ``points`` for the incidences ``columns`` of the solved
    fields ``Ej`` (n, R), in one ``propagate`` call.

    E0: incident field at ``points`` for those incidences, as the solver's
    ``generate_source`` returns it: (P, d, A) for vector waves, (P, A) for
    scalar waves.  Returns the same shape as E0 (the driver's per-angle
    ``E_meas``, magreete.py:672, stacked along the last axis)."""
    Ej = torch.as_tensor(Ej)
    cols = torch.as_tensor(list(columns), dtype=torch.long, device=Ej.device)
    return solver.propagate(points, Ej.index_select(1, cols), k0, alpha, E0, regularize=regularize,
                            radius=radius)


def field_components(E, points):
    """Amplitude, longitudinal and transverse parts of a vector field E (P, d)
    at points (P, d), as the driver plots them (magreete.py:698-713).

    amplitude    sqrt(sum_a |E_a|^2);
    2D: with phi = atan2(y, x), longitudinal = E_x cos(phi) - E_y sin(phi),
        transverse = E_x sin(phi) + E_y cos(phi) (complex);
    3D: with v = points / |points|, longitudinal = sum_a E_a v_a (complex),
        transverse = |E - longitudinal v| (real)."""
    E = torch.as_tensor(E)
    pts = torch.as_tensor(points, dtype=torch.float64).to(E.device)
    amplitude = torch.sqrt(torch.sum(torch.abs(E) ** 2, dim=-1))
    if E.shape[-1] == 2:
        phi = torch.atan2(pts[:, 1], pts[:, 0])
        longitudinal = E[:, 0] * torch.cos(phi) - E[:, 1] * torch.sin(phi)
        transverse = E[:, 0] * torch.sin(phi) + E[:, 1] * torch.cos(phi)
    elif E.shape[-1] == 3:
        v = pts / torch.linalg.norm(pts, dim=-1).unsqueeze(-1)
        longitudinal = torch.sum(E * v, dim=1)
        transverse = torch.sqrt(torch.sum(torch.abs(E - longitudinal.reshape(-1, 1) * v) ** 2, dim=1))
    else:
        raise ValueError(f"vector fields have 2 or 3 components, not {E.shape[-1]}")
    return amplitude, longitudinal, transverse
