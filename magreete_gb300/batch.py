"""Batched sweeps: many independent solves of uneven size in one CUDA-graph launch.

A sweep over disorder realisations or frequencies (the driver's per-copy and
per-k0 loops, magreete.py:114, :371) is a set of independent requests.  A
``BatchedSweep`` groups them, preallocates every device buffer of a group,
and captures the whole group -- assembly, complex64 LU, refined solve (one
correction) and the final residual norms -- into one CUDA graph whose
instances run as concurrent branches on `branches` streams.  One
``replay()`` then launches the group.  Instances whose certified relative
residual is still above the tolerance after the graph get further
corrections outside it, and, if those do not reach it either, a fresh
factorisation with partial pivoting.

Every factorisation carries its own options (``_lib.LuOptions``): nothing
here changes the library's process-wide tuning, so a sweep and a server in
one process do not affect each other.  With tile pivoting (the default) the
LU has no spin-waits between CTAs at all; with partial pivoting the panels
launch without the cooperative attribute (capturable) and each is limited to
its share of the SMs.

The autotuner (``autotune``) times the group's graph for a few settings of
the concurrent-branch count, the pivoting and the LU's outer block width,
keeps the fastest, and caches the choice per size bucket.
"""
from __future__ import annotations

import ctypes
import json
import math
import os
import time

import torch

from . import _lib as L
from . import engine as E
from . import selfterm
from . import sources as S

TUNE_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "magreete_gb300_tuning.json")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class _Instance:
    """Device buffers of one request of a batch."""

    def __init__(self, prob, dev, lib, lu_options):
        self.prob = prob
        self.lu_options = lu_options
        n, R = prob.n, prob.nrhs
        self.pts = prob.points.to(dev)
        ld = (n + 15) // 16 * 16
        self.M32 = torch.empty((n, ld), dtype=torch.complex64, device=dev)[:, :n]
        self.Mdf = torch.empty((n, n, 4), dtype=torch.float32, device=dev)
        self.perm = torch.empty(n, dtype=torch.int32, device=dev)
        nb = ctypes.c_size_t()
        L.check(lib.mgt_lu_workspace_bytes(L.MGT_C64, n, ctypes.byref(nb)), "mgt_lu_workspace_bytes")
        self.luw = torch.empty(max(nb.value, 256), dtype=torch.uint8, device=dev)
        L.check(lib.mgt_refine_workspace_bytes(n, R, ctypes.byref(nb)), "mgt_refine_workspace_bytes")
        self.rw = torch.empty(max(nb.value, 256), dtype=torch.uint8, device=dev)
        # incident fields are computed once, eagerly: they hold host-to-device
        # copies of the direction tables, which a graph capture does not allow
        if prob.kind.startswith("2d"):
            E0 = S.source_2d(prob.kind, "plane", self.pts, prob.k0, prob.thetas, 0.2)
        else:
            E0 = S.source_3d(prob.kind, "plane", self.pts, prob.k0, prob.u, prob.p, 0.2)
        self.B = E0.reshape(n, R).contiguous()
        self.X = torch.empty((n, R), dtype=torch.complex128, device=dev)
        self.norms = torch.zeros(2, dtype=torch.float64, device=dev)

    def bytes(self):
        return sum(t.numel() * t.element_size() for t in (self.M32, self.Mdf, self.luw, self.rw, self.B, self.X)) + \
            self.M32.shape[0] * 16 * 8

    def enqueue(self, lib, stream_ptr, corrections=1, options=None):
        """Stream-ordered solve: assembly, LU, refined solve, norms."""
        p = self.prob
        n, R = p.n, p.nrhs
        coef = complex(p.alpha * p.k0 * p.k0)
        shift = complex(selfterm.diagonal_shift(p.kind, p.k0, p.alpha, p.radius))
        L.check(lib.mgt_assemble_system(E.KIND_CODE[p.kind], _ptr(self.pts), p.N, float(p.k0), coef.real, coef.imag,
                                        shift.real, shift.imag, _ptr(self.Mdf), n, L.MGT_CDF, _ptr(self.M32),
                                        self.M32.stride(0), L.MGT_C64, stream_ptr), "mgt_assemble_system")
        # M's digits for every residual of this solve (corrections and norms
        # then pass no matrix); the double-float matrix itself where the
        # tensor-core residual is unavailable
        st = lib.mgt_refine_prepare(_ptr(self.Mdf), n, n, R, _ptr(self.rw), self.rw.numel(), stream_ptr)
        if st == L.MGT_ERR_UNSUPPORTED:
            self.mref = _ptr(self.Mdf)
        else:
            L.check(st, "mgt_refine_prepare")
            self.mref = None
        opt = options if options is not None else self.lu_options
        L.check(lib.mgt_lu_factor_ex(L.MGT_C64, _ptr(self.M32), n, self.M32.stride(0), _ptr(self.perm),
                                     _ptr(self.luw), self.luw.numel(), ctypes.byref(opt), stream_ptr),
                "mgt_lu_factor_ex")
        L.check(lib.mgt_refine_start(_ptr(self.M32), self.M32.stride(0), _ptr(self.perm), n, _ptr(self.B), R,
                                     _ptr(self.X), R, R, _ptr(self.rw), self.rw.numel(), stream_ptr),
                "mgt_refine_start")
        for _ in range(corrections):
            self.correct(lib, stream_ptr)
        self.measure(lib, stream_ptr)

    def correct(self, lib, stream_ptr):
        p = self.prob
        n, R = p.n, p.nrhs
        L.check(lib.mgt_refine_correct(self.mref, n, _ptr(self.M32), self.M32.stride(0), _ptr(self.perm), n,
                                       _ptr(self.B), R, _ptr(self.X), R, R, _ptr(self.rw), self.rw.numel(),
                                       stream_ptr), "mgt_refine_correct")

    def measure(self, lib, stream_ptr):
        p = self.prob
        n, R = p.n, p.nrhs
        L.check(lib.mgt_refine_norms(self.mref, n, n, _ptr(self.B), R, _ptr(self.X), R, R, _ptr(self.rw),
                                     self.rw.numel(), ctypes.c_void_p(self.norms.data_ptr()), stream_ptr),
                "mgt_refine_norms")

    def rel_residual(self):
        b, r = self.norms.tolist()
        return math.sqrt(r / b) if b > 0 else math.sqrt(r)


class BatchedSweep:
    """One CUDA graph for a group of independent refined solves.

    problems:    workloads.Problem list (any kinds / sizes)
    branches:    concurrent graph branches (streams) the instances are spread over
    pivoting:    "tile" (default) or "partial" (see engine.lu_factor)
    outer_block: 128 (default) or 64, the complex64 LU's outer block width
    panel_rows:  rows per CTA of partial-pivoting panels (0: library default)
    """

    def __init__(self, problems, branches=8, tol=E.DEFAULT_TOL, device=None, pivoting="tile", outer_block=128,
                 panel_rows=0):
        self.lib = L.load()
        self.dev = device or torch.device("cuda", torch.cuda.current_device())
        self.tol = tol
        self.pivoting = pivoting
        sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
        if pivoting == "partial":
            # a panel CTA holds at most 220 KB of rows (complex64, 64 columns): the
            # largest instance needs ceil(8 n / 440) CTAs; keep the panels of all
            # branches within the SM count, so that no panel waits on another
            need = max(1, math.ceil(max(p.n for p in problems) / 440))
            self.branches = max(1, min(int(branches), sms // need))
        else:
            self.branches = max(1, int(branches))
        # launched without the cooperative attribute (capturable), no lookahead (capture)
        self.lu_options = L.LuOptions(pivoting=E.PIVOTING[pivoting], panel_rows=int(panel_rows),
                                      panel_max_ctas=max(1, sms // self.branches), cooperative=0, lookahead=0,
                                      outer_block=int(outer_block))
        # largest first, so that the long solves start early in every branch
        order = sorted(range(len(problems)), key=lambda i: -problems[i].n)
        self.order = order
        self.inst = [_Instance(problems[i], self.dev, self.lib, self.lu_options) for i in order]
        self.graph = None
        self.refactored = 0

    def _enqueue_all(self):
        main = torch.cuda.current_stream()
        streams = [torch.cuda.Stream(self.dev) for _ in range(self.branches)]
        for st in streams:
            st.wait_stream(main)
        for k, inst in enumerate(self.inst):
            st = streams[k % self.branches]
            with torch.cuda.stream(st):
                inst.enqueue(self.lib, ctypes.c_void_p(st.cuda_stream))
        for st in streams:
            main.wait_stream(st)

    def warmup(self):
        """One eager run (initialises kernels' one-time attributes; required before capture)."""
        self._enqueue_all()
        torch.cuda.synchronize(self.dev)

    def capture(self):
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode="thread_local"):
            self._enqueue_all()
        return self

    def replay(self):
        """Launch the captured group and finish stragglers eagerly.  Returns
        (iterations beyond the graph per instance, relative residuals)."""
        self.graph.replay()
        torch.cuda.synchronize(self.dev)
        extra, res = [], []
        sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        for inst in self.inst:
            k = 0
            rr = inst.rel_residual()
            while rr > self.tol and k < E.DEFAULT_MAX_ITER:
                inst.correct(self.lib, sp)
                inst.measure(self.lib, sp)
                torch.cuda.synchronize(self.dev)
                nr = inst.rel_residual()
                k += 1
                if not nr < 0.9 * rr:
                    rr = nr
                    break
                rr = nr
            if not rr <= self.tol:
                # the refinement cannot use these factors: partial pivoting, eagerly
                inst.enqueue(self.lib, sp, corrections=1, options=L.LuOptions(pivoting=L.MGT_PIVOT_PARTIAL))
                torch.cuda.synchronize(self.dev)
                rr = inst.rel_residual()
                while rr > self.tol and k < 2 * E.DEFAULT_MAX_ITER:
                    inst.correct(self.lib, sp)
                    inst.measure(self.lib, sp)
                    torch.cuda.synchronize(self.dev)
                    rr = inst.rel_residual()
                    k += 1
                self.refactored += 1
            extra.append(k)
            res.append(rr)
        return extra, res

    def solutions(self):
        """Fields at the scatterers, in the order the problems were given."""
        out = [None] * len(self.inst)
        for pos, i in enumerate(self.order):
            out[i] = self.inst[pos].X
        return out


def _bucket(problems):
    n = max(p.n for p in problems)
    return f"n<={2 ** math.ceil(math.log2(max(n, 2)))}"


def autotune(problems, branch_options=(4, 8, 16), pivoting_options=("tile", "partial"), outer_options=(128, 64),
             reps=1, cache=TUNE_CACHE):
    """Pick (branches, pivoting, outer block width) for groups like `problems`
    by timing graph replays; the choice is cached per size bucket.  Returns
    the dict (keyword arguments of BatchedSweep plus the timings)."""
    key = _bucket(problems)
    try:
        with open(cache) as f:
            table = json.load(f)
    except (OSError, ValueError):
        table = {}
    if key in table and {"branches", "pivoting", "outer_block"} <= set(table[key]):
        return table[key]
    results = []
    for piv in pivoting_options:
        for ob in outer_options:
            for br in branch_options:
                sw = BatchedSweep(problems, branches=br, pivoting=piv, outer_block=ob)
                sw.warmup()
                sw.capture()
                sw.replay()
                t0 = time.perf_counter()
                for _ in range(reps):
                    sw.replay()
                dt = (time.perf_counter() - t0) / reps
                results.append({"pivoting": piv, "outer_block": ob, "branches": br, "seconds": dt})
                del sw
                torch.cuda.empty_cache()
    best = dict(min(results, key=lambda r: r["seconds"]), candidates=results)
    table[key] = best
    try:
        os.makedirs(os.path.dirname(cache), exist_ok=True)
        with open(cache, "w") as f:
            json.dump(table, f, indent=1)
    except OSError:
        pass
    return best
