"""Device-side building blocks over the C ABI (torch tensors as device memory).

Every function here takes and returns CUDA tensors and enqueues work on the
current torch CUDA stream through ``libmagreete_gb300.so``.  There is no CPU
path: a missing library or a non-CUDA tensor is an error.

Precision methods
-----------------
``"fp64"`` (the plain method, the drop-in default): complex128 assembly,
complex128 LU with partial pivoting, complex128 triangular solves.

``"mixed"``: one assembly pass writes the matrix in complex64 (for the LU) and
in double-float form (for residuals); the LU runs in complex64 and iterative
refinement brings the solution to a relative residual ``tol`` (1e-10 by
default), i.e. complex128-level accuracy.  The residuals run on the tensor
cores (a digit-split product of the double-float matrix).  The LU chooses its
pivots within each 64-row diagonal tile (no exchange between CTAs); when the
refinement cannot use such factors (or a tile pivot is exactly zero) the
matrix is factored again with partial pivoting.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib as L

KIND_CODE = {"2d_vector": L.MGT_2D_VECTOR, "2d_scalar": L.MGT_2D_SCALAR,
             "3d_vector": L.MGT_3D_VECTOR, "3d_scalar": L.MGT_3D_SCALAR}
KIND_DIMS = {"2d_vector": (2, 2), "2d_scalar": (2, 1), "3d_vector": (3, 3), "3d_scalar": (3, 1)}

DEFAULT_TOL = 1e-10
DEFAULT_MAX_ITER = 10


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _need_cuda(t, name):
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")


def device_of(*tensors):
    for t in tensors:
        if isinstance(t, torch.Tensor) and t.is_cuda:
            return t.device
    if not torch.cuda.is_available():
        raise RuntimeError("magreete_gb300 needs a CUDA GPU; none is available")
    return torch.device("cuda", torch.cuda.current_device())


def points_to(points, device, dim):
    p = torch.as_tensor(points)
    p = p.reshape(-1, dim).to(device=device, dtype=torch.float64).contiguous()
    return p


def workspace(nbytes, device):
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


# ------------------------------------------------------------------ assembly

def assemble_system(kind, points, k0, coef, shift, formats=("c128",)):
    """M = I - coef * G with diagonal 1 - shift, written in each of
    ``formats`` ("c128", "c64", "cdf").  Returns a tuple of tensors; "cdf"
    comes back as a float32 tensor of shape (n, n, 4)."""
    lib = L.load()
    _need_cuda(points, "points")
    dim, d = KIND_DIMS[kind]
    N = points.shape[0]
    n = d * N
    outs, specs = [], []
    for f in formats:
        if f == "c128":
            t = torch.empty((n, n), dtype=torch.complex128, device=points.device)
            specs.append((t, n, L.MGT_C128))
        elif f == "c64":
            # rows padded to a multiple of 16 elements (128 B): the tensor-core
            # LU update needs 16-byte aligned rows
            ld = (n + 15) // 16 * 16
            t = torch.empty((n, ld), dtype=torch.complex64, device=points.device)[:, :n]
            specs.append((t, ld, L.MGT_C64))
        elif f == "cdf":
            t = torch.empty((n, n, 4), dtype=torch.float32, device=points.device)
            specs.append((t, n, L.MGT_CDF))
        else:
            raise ValueError(f"unknown format {f}")
        outs.append(t)
    if len(specs) > 2:
        raise ValueError("at most two formats per assembly pass")
    s2 = specs[1] if len(specs) > 1 else (None, 0, 0)
    coef = complex(coef)
    shift = complex(shift)
    L.check(lib.mgt_assemble_system(KIND_CODE[kind], _ptr(points), N, float(k0), coef.real, coef.imag,
                                    shift.real, shift.imag, _ptr(specs[0][0]), specs[0][1], specs[0][2],
                                    _ptr(s2[0]), s2[1], s2[2], _stream()), "mgt_assemble_system")
    return tuple(outs)


def assemble_propagator(kind, targets, sources, k0, coef=1.0, regularize=False, radius=0.0,
                        nan_fill=None, transpose=False):
    """Dense coef * G(t - s) (d*T x d*S complex128), or its transpose.
    nan_fill=None keeps NaN where the reference has NaN; a complex value
    replaces every entry of such a block."""
    lib = L.load()
    _need_cuda(targets, "targets")
    dim, d = KIND_DIMS[kind]
    T, S = targets.shape[0], sources.shape[0]
    shape = (d * S, d * T) if transpose else (d * T, d * S)
    out = torch.empty(shape, dtype=torch.complex128, device=targets.device)
    coef = complex(coef)
    fill = complex(nan_fill) if nan_fill is not None else 0j
    L.check(lib.mgt_assemble_propagator(KIND_CODE[kind], _ptr(targets), T, _ptr(sources), S, float(k0),
                                        coef.real, coef.imag, int(bool(regularize)), float(radius),
                                        L.MGT_NAN_KEEP if nan_fill is None else L.MGT_NAN_FILL,
                                        fill.real, fill.imag, int(bool(transpose)), _ptr(out), shape[1],
                                        _stream()), "mgt_assemble_propagator")
    return out


# ------------------------------------------------------------------ LU

class LUFactors:
    """In-place LU factors with their row permutation and workspace."""

    def __init__(self, lu, perm, work, dtype_code, pivoting="partial"):
        self.lu, self.perm, self.work, self.dtype_code = lu, perm, work, dtype_code
        self.pivoting = pivoting

    @property
    def n(self):
        return self.lu.shape[0]


PIVOTING = {"partial": L.MGT_PIVOT_PARTIAL, "tile": L.MGT_PIVOT_TILE}


def lu_factor(A, check_singular=True, pivoting="partial", options=None):
    """Factor A (complex128 or complex64, n x n, CUDA) in place.

    pivoting: "partial" (LAPACK's row interchanges, the reference's pivot
    sequence) or "tile" (complex64: pivots chosen within each 64-row
    diagonal tile, no exchange between CTAs; for the refined mixed method).
    options: an _lib.LuOptions for the other per-call choices."""
    lib = L.load()
    _need_cuda(A, "A")
    n = A.shape[0]
    code = {torch.complex128: L.MGT_C128, torch.complex64: L.MGT_C64}[A.dtype]
    nb = ctypes.c_size_t()
    L.check(lib.mgt_lu_workspace_bytes(code, n, ctypes.byref(nb)), "mgt_lu_workspace_bytes")
    work = workspace(nb.value, A.device)
    perm = torch.empty(n, dtype=torch.int32, device=A.device)
    opt = options if options is not None else L.LuOptions()
    opt.pivoting = PIVOTING[pivoting] if options is None else opt.pivoting
    L.check(lib.mgt_lu_factor_ex(code, _ptr(A), n, A.stride(0), _ptr(perm), _ptr(work), work.numel(),
                                 ctypes.byref(opt), _stream()), "mgt_lu_factor_ex")
    f = LUFactors(A, perm, work, code, "tile" if opt.pivoting == L.MGT_PIVOT_TILE else "partial")
    if check_singular:
        status_check(f)
    return f


def lu_info(f):
    """(device error, first zero pivot) of a factorisation; synchronises the stream."""
    lib = L.load()
    st = (ctypes.c_int32 * 2)()
    L.check(lib.mgt_workspace_status(_ptr(f.work), st, _stream()), "mgt_workspace_status")
    return st[0], st[1]


def status_check(f):
    lib = L.load()
    st = (ctypes.c_int32 * 2)()
    L.check(lib.mgt_workspace_status(_ptr(f.work), st, _stream()), "mgt_workspace_status")
    if st[0] != 0:
        raise L.MagreeteError(st[0], "mgt_lu_factor (device)")
    if st[1] != 0:
        raise torch.linalg.LinAlgError(
            f"linalg.solve: The solver failed because the input matrix is singular (zero pivot at column {st[1]}).")


def lu_solve(f, B):
    """X = A^-1 B with LU factors f; B (n x R) of the factors' dtype."""
    lib = L.load()
    B = B.contiguous()
    X = torch.empty_like(B)
    nb = ctypes.c_size_t()
    L.check(lib.mgt_lu_solve_workspace_bytes(f.dtype_code, f.n, B.shape[1], ctypes.byref(nb)),
            "mgt_lu_solve_workspace_bytes")
    work = workspace(nb.value, B.device)
    L.check(lib.mgt_lu_solve(f.dtype_code, _ptr(f.lu), f.n, f.lu.stride(0), _ptr(f.perm), _ptr(B), B.shape[1],
                             _ptr(X), B.shape[1], B.shape[1], _ptr(work), work.numel(), _stream()), "mgt_lu_solve")
    return X


class RefineContext:
    """The refinement's hold on M: its digits (the tensor-core residual's
    operand, 14 B per entry) made once by mgt_refine_prepare in a refinement
    workspace for up to max_nrhs columns, after which the double-float copy
    may be freed.  Where the tensor-core residual is unavailable it keeps the
    double-float matrix instead."""

    def __init__(self, Mdf, max_nrhs=64):
        lib = L.load()
        self.n = Mdf.shape[0]
        self.max_nrhs = int(max_nrhs)
        nb = ctypes.c_size_t()
        L.check(lib.mgt_refine_workspace_bytes(self.n, self.max_nrhs, ctypes.byref(nb)), "mgt_refine_workspace_bytes")
        self.work = workspace(nb.value, Mdf.device)
        st = lib.mgt_refine_prepare(_ptr(Mdf), self.n, self.n, self.max_nrhs, _ptr(self.work), self.work.numel(),
                                    _stream())
        if st == L.MGT_ERR_UNSUPPORTED:
            self.Mdf, self.work = Mdf, None
        else:
            L.check(st, "mgt_refine_prepare")
            self.Mdf = None


def solve_refined(M, f, B, tol=DEFAULT_TOL, max_iter=DEFAULT_MAX_ITER, require=True):
    """Refined solve of M X = B (B complex128 n x R) with complex64 factors f.
    M: the double-float matrix, or a RefineContext (right-hand sides wider
    than it was prepared for are solved in blocks of columns).  Returns
    (X, iterations, rel_residual)."""
    if isinstance(M, RefineContext):
        if M.work is None:
            return solve_refined(M.Mdf, f, B, tol, max_iter, require)
        return _solve_prepared(M, f, B, tol, max_iter, require)
    Mdf = M
    lib = L.load()
    n = f.n
    B = B.contiguous()
    R = B.shape[1]
    nb = ctypes.c_size_t()
    L.check(lib.mgt_refine_workspace_bytes(n, R, ctypes.byref(nb)), "mgt_refine_workspace_bytes")
    work = workspace(nb.value, B.device)
    X = torch.empty_like(B)
    it = ctypes.c_int(0)
    rr = ctypes.c_double(0.0)
    st = lib.mgt_solve_refined(_ptr(Mdf), n, _ptr(f.lu), f.lu.stride(0), _ptr(f.perm), n, _ptr(B), R, _ptr(X), R,
                               R, float(tol), int(max_iter), _ptr(work), work.numel(), ctypes.byref(it),
                               ctypes.byref(rr), _stream())
    if st == L.MGT_ERR_NOT_CONVERGED and not require:
        return X, it.value, rr.value
    L.check(st, f"mgt_solve_refined (iterations {it.value}, relative residual {rr.value:.3e})")
    return X, it.value, rr.value


def _solve_prepared(ctx, f, B, tol, max_iter, require):
    lib = L.load()
    n = f.n
    B = B.contiguous()
    R = B.shape[1]
    X = torch.empty_like(B)
    its, sq = [], 0.0
    for c0 in range(0, R, ctx.max_nrhs):
        Bc = B[:, c0:c0 + ctx.max_nrhs].contiguous()
        Xc = torch.empty_like(Bc)
        rc = Bc.shape[1]
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        st = lib.mgt_solve_refined(None, n, _ptr(f.lu), f.lu.stride(0), _ptr(f.perm), n, _ptr(Bc), rc, _ptr(Xc), rc,
                                   rc, float(tol), int(max_iter), _ptr(ctx.work), ctx.work.numel(), ctypes.byref(it),
                                   ctypes.byref(rr), _stream())
        if not (st == L.MGT_ERR_NOT_CONVERGED and not require):
            L.check(st, f"mgt_solve_refined (iterations {it.value}, relative residual {rr.value:.3e})")
        X[:, c0:c0 + rc] = Xc
        its.append(it.value)
        if rc == R:
            return X, it.value, rr.value
        sq += (rr.value * torch.linalg.norm(Bc).item()) ** 2
    nb = torch.linalg.norm(B).item()
    return X, max(its), (sq ** 0.5 / nb if nb > 0 else sq ** 0.5)


def residual(Mdf, X, B):
    lib = L.load()
    n, R = B.shape
    nb = ctypes.c_size_t()
    L.check(lib.mgt_residual_workspace_bytes(n, R, ctypes.byref(nb)), "mgt_residual_workspace_bytes")
    work = workspace(nb.value, B.device)
    Rr = torch.empty_like(B)
    X, B = X.contiguous(), B.contiguous()
    L.check(lib.mgt_residual(_ptr(Mdf), n, n, _ptr(X), R, _ptr(B), R, _ptr(Rr), R, R, _ptr(work), work.numel(),
                             _stream()), "mgt_residual")
    return Rr


class ResidualOperator:
    """R = B - M X for a fixed double-float M and any number of X (up to
    max_nrhs columns each): M's digits are made once (mgt_residual_prepare)
    and every call applies them (mgt_residual_apply, tensor cores only)."""

    def __init__(self, Mdf, max_nrhs):
        self.lib = L.load()
        self.n = Mdf.shape[0]
        self.max_nrhs = max_nrhs
        nb = ctypes.c_size_t()
        L.check(self.lib.mgt_residual_workspace_bytes(self.n, max_nrhs, ctypes.byref(nb)),
                "mgt_residual_workspace_bytes")
        self.work = workspace(nb.value, Mdf.device)
        L.check(self.lib.mgt_residual_prepare(_ptr(Mdf), self.n, self.n, _ptr(self.work), self.work.numel(),
                                              _stream()), "mgt_residual_prepare")

    def __call__(self, X, B):
        n, R = B.shape
        if n != self.n or R > self.max_nrhs:
            raise ValueError(f"shape {tuple(B.shape)} does not fit an operator of order {self.n} "
                             f"with at most {self.max_nrhs} right-hand sides")
        X, B = X.contiguous(), B.contiguous()
        Rr = torch.empty_like(B)
        L.check(self.lib.mgt_residual_apply(n, _ptr(X), R, _ptr(B), R, _ptr(Rr), R, R, _ptr(self.work),
                                            self.work.numel(), _stream()), "mgt_residual_apply")
        return Rr


# ------------------------------------------------------------------ system solve

def solve_system(kind, points, k0, coef, shift, E0, precision="fp64", tol=DEFAULT_TOL,
                 max_iter=DEFAULT_MAX_ITER, stats=None):
    """Solve (I - coef G) X = E0 with diagonal 1 - shift.  E0: (n, R)
    complex128 CUDA.  Returns X (n, R) complex128."""
    if precision == "fp64":
        (M,) = assemble_system(kind, points, k0, coef, shift, ("c128",))
        f = lu_factor(M)
        X = lu_solve(f, E0)
        if stats is not None:
            stats.update(method="fp64", iterations=0)
        return X
    if precision == "mixed":
        Mdf, M32 = assemble_system(kind, points, k0, coef, shift, ("cdf", "c64"))
        # the digits replace the double-float copy before the LU needs its memory
        ctx = RefineContext(Mdf, E0.shape[1])
        del Mdf
        f, X, it, rr = mixed_factor_solve(ctx, M32, E0, _fresh(kind, points, k0, coef, shift), tol, max_iter)
        if stats is not None:
            stats.update(method="mixed", iterations=it, rel_residual=rr, pivoting=f.pivoting)
        return X
    raise ValueError(f"unknown precision {precision!r} (expected 'fp64' or 'mixed')")


def mixed_factor(M32, fresh_m32):
    """complex64 LU of M32 with tile pivoting; with partial pivoting of a fresh
    copy (fresh_m32() returns one) when a tile pivot is exactly zero."""
    f = lu_factor(M32, check_singular=False, pivoting="tile")
    err, info = lu_info(f)
    if err != 0:
        raise L.MagreeteError(err, "mgt_lu_factor_ex (device)")
    if info == 0:
        return f
    return lu_factor(fresh_m32(), pivoting="partial")


def mixed_factor_solve(Mdf, M32, B, fresh_m32, tol=DEFAULT_TOL, max_iter=DEFAULT_MAX_ITER):
    """Factor M32 (tile pivoting first) and refine M X = B against the
    double-float Mdf (or a RefineContext made from it); if the refinement
    does not reach tol on tile-pivoted factors, factor a fresh copy with
    partial pivoting and refine again.  Returns (factors, X, iterations,
    relative residual)."""
    f = mixed_factor(M32, fresh_m32)
    X, it, rr = solve_refined(Mdf, f, B, tol, max_iter, require=f.pivoting == "partial")
    if rr <= tol:
        return f, X, it, rr
    f = lu_factor(fresh_m32(), pivoting="partial")
    X, it, rr = solve_refined(Mdf, f, B, tol, max_iter)
    return f, X, it, rr


def _fresh(kind, points, k0, coef, shift):
    return lambda: assemble_system(kind, points, k0, coef, shift, ("c64",))[0]


class SystemFactorization:
    """Factorised system matrix kept resident for several right-hand sides
    (mean DOS, LDOS, frequency re-queries)."""

    def __init__(self, kind, points, k0, coef, shift, precision="fp64", tol=DEFAULT_TOL,
                 max_iter=DEFAULT_MAX_ITER):
        self.precision, self.tol, self.max_iter = precision, tol, max_iter
        if precision == "fp64":
            (M,) = assemble_system(kind, points, k0, coef, shift, ("c128",))
            self.Mdf = None
            self.f = lu_factor(M)
        elif precision == "mixed":
            Mdf, M32 = assemble_system(kind, points, k0, coef, shift, ("cdf", "c64"))
            self.ctx = RefineContext(Mdf, 64)
            self.Mdf = self.ctx.Mdf
            del Mdf
            self._fresh = _fresh(kind, points, k0, coef, shift)
            self.f = mixed_factor(M32, self._fresh)
        else:
            raise ValueError(f"unknown precision {precision!r}")
        self.last_iterations = 0
        self.last_residual = None

    def solve(self, B):
        if self.precision == "fp64":
            return lu_solve(self.f, B.to(torch.complex128))
        B = B.to(torch.complex128)
        X, it, rr = solve_refined(self.ctx, self.f, B, self.tol, self.max_iter, require=self.f.pivoting == "partial")
        if rr > self.tol:
            # tile-pivoted factors that refinement cannot use: partial pivoting from here on
            self.f = lu_factor(self._fresh(), pivoting="partial")
            X, it, rr = solve_refined(self.ctx, self.f, B, self.tol, self.max_iter)
        self.last_iterations, self.last_residual = it, rr
        return X


# ------------------------------------------------------------------ propagate

def propagate(kind, targets, sources, k0, coef, Ek, E0=None, regularize=False, radius=0.0, precision="fp64"):
    """coef * G(targets, sources) @ Ek + E0, matrix-free.  Ek (d*S, R),
    E0 (d*T, R) or None.  Returns (d*T, R) complex128."""
    lib = L.load()
    dim, d = KIND_DIMS[kind]
    T, S = targets.shape[0], sources.shape[0]
    Ek = Ek.reshape(d * S, -1).to(torch.complex128).contiguous()
    R = Ek.shape[1]
    if E0 is not None:
        E0 = E0.reshape(d * T, R).to(torch.complex128).contiguous()
    out = torch.empty((d * T, R), dtype=torch.complex128, device=targets.device)
    nb = ctypes.c_size_t()
    L.check(lib.mgt_propagate_workspace_bytes(KIND_CODE[kind], T, S, R, ctypes.byref(nb)),
            "mgt_propagate_workspace_bytes")
    work = workspace(nb.value, targets.device)
    coef = complex(coef)
    code = L.MGT_C128 if precision == "fp64" else L.MGT_CDF
    L.check(lib.mgt_propagate(KIND_CODE[kind], code, _ptr(targets), T, _ptr(sources), S, float(k0), coef.real,
                              coef.imag, int(bool(regularize)), float(radius), _ptr(Ek), R, _ptr(E0), R,
                              _ptr(out), R, R, _ptr(work), work.numel(), _stream()), "mgt_propagate")
    return out


def cgemm_sub(C, A, B, tensor_cores=True):
    """C -= A @ B in place (complex; C, A, B CUDA tensors of one dtype)."""
    lib = L.load()
    M, K = A.shape
    N = B.shape[1]
    code = {torch.complex128: L.MGT_C128, torch.complex64: L.MGT_C64}[C.dtype]
    nb = ctypes.c_size_t()
    L.check(lib.mgt_cgemm_workspace_bytes(max(M, N), ctypes.byref(nb)), "mgt_cgemm_workspace_bytes")
    work = workspace(nb.value, C.device)
    work[:256].zero_()
    L.check(lib.mgt_cgemm_sub(code, int(bool(tensor_cores)), M, N, K, _ptr(A), A.stride(0), _ptr(B), B.stride(0),
                              _ptr(C), C.stride(0), _ptr(work), work.numel(), _stream()), "mgt_cgemm_sub")
    st = int(work[:4].view(torch.int32)[0].item())
    if st != 0:
        raise L.MagreeteError(st, "mgt_cgemm_sub (device)")
    return C


def column_dots(A, B):
    """out[i] = sum_k A[k, i] B[k, i] (complex128)."""
    lib = L.load()
    A, B = A.contiguous(), B.contiguous()
    n, c = A.shape
    out = torch.empty(c, dtype=torch.complex128, device=A.device)
    L.check(lib.mgt_column_dots(_ptr(A), c, _ptr(B), c, n, c, _ptr(out), _stream()), "mgt_column_dots")
    return out
