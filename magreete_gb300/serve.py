"""Request-level solve pipeline and the continuous-batching server.

A request (``workloads.Problem``) is one coupled-dipole solve: incident
fields at the scatterers and detectors, system assembly, LU, (refined)
solve for all right-hand sides, and matrix-free propagation to the
detectors -- the ``generate_source`` -> ``solve`` -> ``propagate`` sequence
the reference driver runs per frequency (magreete.py:371-400).

``Server`` keeps several requests in flight on one GPU: each of ``slots``
worker threads owns a CUDA stream and takes the oldest waiting request as
soon as its device memory fits in the HBM budget, so requests that arrive
while others are running are admitted as slots and memory free up, and their
kernels overlap on the device (a latency-bound panel factorisation of one
request runs beside the tensor-core updates of another).  Geometries stay
resident on the device for re-queries; a re-query at a frequency whose
factorisation is still cached reuses it.
"""
from __future__ import annotations

import collections
import concurrent.futures as cf
import dataclasses
import threading
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
    reused_factorization: bool = False


def incident_fields(prob, pts, det):
    if prob.kind.startswith("2d"):
        E0s = S.source_2d(prob.kind, "plane", pts, prob.k0, prob.thetas, 0.2)
        E0d = S.source_2d(prob.kind, "plane", det, prob.k0, prob.thetas, 0.2)
    else:
        E0s = S.source_3d(prob.kind, "plane", pts, prob.k0, prob.u, prob.p, 0.2)
        E0d = S.source_3d(prob.kind, "plane", det, prob.k0, prob.u, prob.p, 0.2)
    return E0s, E0d


def solve_problem(prob, precision="mixed", pts=None, det=None, tol=E.DEFAULT_TOL, factorization=None):
    """Run one request on the current CUDA stream; inputs already on the device
    when pts/det are given.  With `factorization` (an engine.SystemFactorization
    of the same geometry and frequency) the assembly and LU are skipped."""
    dev = torch.device("cuda", torch.cuda.current_device())
    pts = prob.points.to(dev) if pts is None else pts
    det = prob.detectors.to(dev) if det is None else det
    E0s, E0d = incident_fields(prob, pts, det)
    n, R = prob.n, prob.nrhs
    coef = prob.alpha * prob.k0 * prob.k0
    B = E0s.reshape(n, R).contiguous()
    if factorization is None:
        shift = selfterm.diagonal_shift(prob.kind, prob.k0, prob.alpha, prob.radius)
        stats = {}
        X = E.solve_system(prob.kind, pts, prob.k0, coef, shift, B, precision, tol, E.DEFAULT_MAX_ITER, stats)
        it, rr = stats.get("iterations", 0), stats.get("rel_residual", float("nan"))
    else:
        X = factorization.solve(B)
        it, rr = factorization.last_iterations, factorization.last_residual
    Ed = E.propagate(prob.kind, det, pts, prob.k0, coef, X, E0d.reshape(-1, R), precision=precision)
    return Result(X, Ed, it, rr if rr is not None else float("nan"), reused_factorization=factorization is not None)


def matrix_bytes(prob, precision="mixed"):
    """Device bytes a request holds at its peak: the matrix copies (24 B / entry
    mixed: complex64 LU + double-float residual copy; 16 B fp64), the
    tensor-core split buffers of the LU's update (12 KB per row: K up to 256,
    sized for fp32 splits), the triangular solves' partial sums (24 B per row
    and right-hand side, rounded up to 64 of them), the right-hand-side blocks and
    the propagation workspace (double-float propagator rows, at most 1 GiB at
    a time, and the double-float copy of the fields), the split-K partial sums
    of the residual (at most 16 splits) and the digits of the tensor-core
    residual: the right-hand sides' (56 KB per 32 rows and 32 right-hand
    sides) and, in the mixed method, the matrix's (14 B per entry, rows padded
    to 128) and the propagator rows' (14 B per entry of a chunk)."""
    n, R = prob.n, prob.nrhs
    per = 16 if precision == "fp64" else 24
    T = prob.detectors.shape[0] if prob.detectors is not None else 0
    chunk = min(1 << 30, 16 * prob.d * n * T)
    prop = chunk + 16 * n * R + (chunk * 14 // 16 if precision != "fp64" else 0)
    partial = 16 * 16 * n * max(R, 64)
    digits = 57344 * -(-n // 32) * -(-R // 32)
    if precision != "fp64":
        digits += 14 * (-(-n // 128) * 128) * (-(-n // 32) * 32)
    split = 12288 * n + 24 * n * (-(-R // 64) * 64)
    return per * n * n + split + 8 * 16 * n * R + prop + partial + digits + (64 << 20)


def serve_sequential(problems, precision="mixed", device_inputs=None, start=None):
    """Serve requests one at a time in arrival order (the plain one-at-a-time
    path).  Returns results with latency = completion - arrival."""
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


class Admission:
    """Device-memory admission for the server, thread-safe and free of CUDA
    calls: requests wait in arrival order and the oldest is admitted once its
    bytes fit the budget next to those in use (no request overtakes an older
    one that does not fit yet).  Cached objects (factorisations) hold bytes
    too, least recently used first out: when the cache outgrows its size,
    and whenever the waiting request would fit without them."""

    def __init__(self, budget):
        self.budget = int(budget)
        self.in_use = 0
        self.cv = threading.Condition()
        self.queue = collections.deque()
        self.closed = False
        self.cache = collections.OrderedDict()     # key -> (object, bytes held)

    def put(self, item, need):
        """Queue ``item`` needing ``need`` bytes; MemoryError if it can never fit."""
        if need > self.budget:
            raise MemoryError(f"request needs {need} B, above the HBM budget of {self.budget} B")
        with self.cv:
            self.queue.append((item, need))
            self.cv.notify_all()

    def take(self):
        """Block until the oldest request fits, admit it and return (item, need);
        None once closed and drained."""
        with self.cv:
            while True:
                if self.queue:
                    need = self.queue[0][1]
                    # cached objects give way to a waiting request
                    while self.in_use + need > self.budget and self.cache:
                        _, (_, held) = self.cache.popitem(last=False)
                        self.in_use -= held
                    if self.in_use + need <= self.budget:
                        self.in_use += need
                        return self.queue.popleft()
                elif self.closed:
                    return None
                self.cv.wait()

    def release(self, need):
        with self.cv:
            self.in_use -= need
            self.cv.notify_all()

    def cache_get(self, key):
        with self.cv:
            hit = self.cache.get(key)
            if hit is None:
                return None
            self.cache.move_to_end(key)
            return hit[0]

    def cache_put(self, key, obj, held, limit):
        """Keep ``obj`` (holding ``held`` bytes) under ``key``; at most ``limit``
        objects stay cached."""
        with self.cv:
            old = self.cache.pop(key, None)
            if old is not None:
                self.in_use -= old[1]
            self.cache[key] = (obj, held)
            self.in_use += held
            while len(self.cache) > limit:
                _, (_, h) = self.cache.popitem(last=False)
                self.in_use -= h
            self.cv.notify_all()

    def close(self):
        with self.cv:
            self.closed = True
            self.cv.notify_all()


class Server:
    """Continuous-batching solve server on one GPU.

    slots:       requests in flight at once (one worker thread + CUDA stream each)
    hbm_budget:  bytes of device memory the in-flight requests may hold
                 (default: 85% of the free memory at start)
    precision:   "mixed" (default) or "fp64"
    host_results: copy each result to host memory before completing it
    factor_cache: factorisations kept for re-queries at the same frequency
                 (they count against the budget and give way to waiting requests)
    """

    def __init__(self, slots=4, hbm_budget=None, precision="mixed", host_results=False, factor_cache=0):
        if not torch.cuda.is_available():
            raise RuntimeError("magreete_gb300.Server needs a CUDA GPU")
        self.device = torch.device("cuda", torch.cuda.current_device())
        free, _ = torch.cuda.mem_get_info(self.device)
        # memory the caching allocator holds but no tensor uses is free for requests too
        free += torch.cuda.memory_reserved(self.device) - torch.cuda.memory_allocated(self.device)
        self.budget = int(hbm_budget if hbm_budget is not None else 0.85 * free)
        self.admission = Admission(self.budget)
        self.precision = precision
        self.host_results = host_results
        self.lock = threading.Lock()
        self.resident = collections.OrderedDict()     # geometry key -> (pts, det) on device
        self.factor_cache = factor_cache
        self.h2d_bytes = 0
        self.d2h_bytes = 0
        self.start = time.perf_counter()
        self.workers = [threading.Thread(target=self._run, args=(i,), daemon=True) for i in range(slots)]
        for w in self.workers:
            w.start()

    @property
    def in_use(self):
        """Bytes the admitted requests and cached factorisations hold."""
        return self.admission.in_use

    # ---------------------------------------------------------------- API
    def submit(self, prob, pts=None, det=None):
        """Queue a request; returns a Future of its Result.  pts / det: device
        copies of the inputs when the caller already holds them."""
        fut = cf.Future()
        try:
            self.admission.put((prob, pts, det, fut), matrix_bytes(prob, self.precision))
        except MemoryError as e:
            fut.set_exception(e)
        return fut

    def close(self):
        self.admission.close()
        for w in self.workers:
            w.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---------------------------------------------------------------- internals
    def _geometry(self, prob, pts, det):
        if pts is not None and det is not None:
            return pts, det
        key = (prob.kind, prob.seed, prob.N)
        with self.lock:
            hit = self.resident.get(key)
            if hit is not None:
                self.resident.move_to_end(key)
                return hit
        pts = prob.points.to(self.device, non_blocking=False)
        det = prob.detectors.to(self.device, non_blocking=False)
        with self.lock:
            self.h2d_bytes += prob.points.numel() * 8 + prob.detectors.numel() * 8
            self.resident[key] = (pts, det)
            while len(self.resident) > 64:
                self.resident.popitem(last=False)
        return pts, det

    def _factorization(self, prob, pts):
        """Cached factorisation for (geometry, k0), built on a miss.  Cached
        factorisations count against the HBM budget until evicted."""
        key = (prob.kind, prob.seed, prob.N, prob.k0)
        fac = self.admission.cache_get(key)
        if fac is not None:
            return fac, True
        shift = selfterm.diagonal_shift(prob.kind, prob.k0, prob.alpha, prob.radius)
        fac = E.SystemFactorization(prob.kind, pts, prob.k0, prob.alpha * prob.k0 * prob.k0, shift, self.precision)
        self.admission.cache_put(key, fac, matrix_bytes(prob, self.precision), self.factor_cache)
        return fac, False

    def _run(self, slot):
        torch.cuda.set_device(self.device)
        stream = torch.cuda.Stream(self.device)
        with torch.cuda.stream(stream):
            while True:
                got = self.admission.take()
                if got is None:
                    return
                (prob, pts, det, fut), need = got
                try:
                    pts, det = self._geometry(prob, pts, det)
                    fac, hit = self._factorization(prob, pts) if self.factor_cache else (None, False)
                    res = solve_problem(prob, self.precision, pts, det, factorization=fac)
                    res.reused_factorization = hit
                    if self.host_results:
                        res.Ek = res.Ek.cpu()
                        res.E_det = res.E_det.cpu()
                        with self.lock:
                            self.d2h_bytes += (res.Ek.numel() + res.E_det.numel()) * 16
                    stream.synchronize()
                    res.latency = time.perf_counter() - self.start - prob.arrival
                    self.admission.release(need)
                    fut.set_result(res)
                except BaseException as e:  # noqa: BLE001 -- reported through the future
                    self.admission.release(need)
                    fut.set_exception(e)


def serve_stream(problems, slots=4, precision="mixed", device_inputs=None, host_results=False, server=None):
    """Feed `problems` to a Server at their arrival times (seconds from now)
    and wait for all results."""
    own = server is None
    srv = server or Server(slots=slots, precision=precision, host_results=host_results)
    srv.start = time.perf_counter()
    futs = []
    for i, prob in enumerate(problems):
        now = time.perf_counter() - srv.start
        if prob.arrival > now:
            time.sleep(prob.arrival - now)
        pts, det = device_inputs[i] if device_inputs is not None else (None, None)
        futs.append(srv.submit(prob, pts, det))
    out = [f.result() for f in futs]
    if own:
        srv.close()
    return out
