"""Request-level solve pipeline and the serving loop.

A request (``workloads.Problem``) is one coupled-dipole solve: incident
fields at the scatterers and detectors, system assembly, LU, (refined)
solve for all right-hand sides, and matrix-free propagation to the
detectors -- the ``generate_source`` -> ``solve`` -> ``propagate`` sequence
the reference driver runs per frequency (magreete.py:371-400).
"""
from __future__ import annotations

import dataclasses
import time

import torch

from . import engine as E
from . import selfterm
from . import sources as S


@dataclasses.dataclass
class Result:
    Ek: torch.Tensor          # (n, R) complex128 fields at the scatterers
    E_det: torch.Tensor       # (M*d, R) complex128 detector fields
    iterations: int = 0
    rel_residual: float = float("nan")
    latency: float = float("nan")


def incident_fields(prob, pts, det):
    if prob.kind.startswith("2d"):
        E0s = S.source_2d(prob.kind, "plane", pts, prob.k0, prob.thetas, 0.2)
        E0d = S.source_2d(prob.kind, "plane", det, prob.k0, prob.thetas, 0.2)
    else:
        E0s = S.source_3d(prob.kind, "plane", pts, prob.k0, prob.u, prob.p, 0.2)
        E0d = S.source_3d(prob.kind, "plane", det, prob.k0, prob.u, prob.p, 0.2)
    return E0s, E0d


def solve_problem(prob, precision="mixed", pts=None, det=None, tol=E.DEFAULT_TOL):
    """Run one request on the current CUDA stream; inputs already on the device
    when pts/det are given."""
    dev = torch.device("cuda", torch.cuda.current_device())
    pts = prob.points.to(dev) if pts is None else pts
    det = prob.detectors.to(dev) if det is None else det
    E0s, E0d = incident_fields(prob, pts, det)
    n = prob.n
    R = prob.nrhs
    coef = prob.alpha * prob.k0 * prob.k0
    shift = selfterm.diagonal_shift(prob.kind, prob.k0, prob.alpha, prob.radius)
    stats = {}
    X = E.solve_system(prob.kind, pts, prob.k0, coef, shift, E0s.reshape(n, R).contiguous(), precision, tol,
                       E.DEFAULT_MAX_ITER, stats)
    Ed = E.propagate(prob.kind, det, pts, prob.k0, coef, X, E0d.reshape(-1, R), precision=precision)
    return Result(X, Ed, stats.get("iterations", 0), stats.get("rel_residual", float("nan")))


def matrix_bytes(prob, precision="mixed"):
    """Device bytes a request holds at its peak (matrix copies + right-hand sides)."""
    n, R = prob.n, prob.nrhs
    per = 16 if precision == "fp64" else 24
    return per * n * n + 6 * 16 * n * R + (1 << 20)


def serve_sequential(problems, precision="mixed", device_inputs=None, start=None):
    """Serve requests one at a time in arrival order.  Returns results with
    latency = completion - arrival (seconds from `start`)."""
    start = time.perf_counter() if start is None else start
    out = []
    for i, prob in enumerate(problems):
        now = time.perf_counter() - start
        if prob.arrival > now:
            time.sleep(prob.arrival - now)
        pts, det = device_inputs[i] if device_inputs is not None else (None, None)
        res = solve_problem(prob, precision, pts, det)
        torch.cuda.current_stream().synchronize()
        res.latency = time.perf_counter() - start - prob.arrival
        out.append(res)
    return out
