#!/usr/bin/env python
"""Benchmark: solves/s and p50/p99 latency of the mixed-N coupled-dipole request stream.

Workload (one "step" = one window of the stream): requests arrive as a
Poisson process (mean 200/s); half are 2D TE (unit disk, phi 0.05) and half
3D dyadic (unit cube, phi 0.1) problems, N log-uniform in [500, 16000],
k0 L uniform in [2 pi 5, 2 pi 25], 1-64 incident fields each, 20% re-query an
earlier geometry at a new frequency.  Each request is solved with the mixed
method (complex64 LU + double-float refinement to a 1e-10 relative residual)
and propagated to 360 (2D) / 1024 (3D) detectors.

value:  requests/s with inputs resident in HBM (all ranks' requests / max time).
e2e:    the same windows through the public Server API with host inputs and
        host results, copies inside the timed region.
subset: the GPU's solves/s on exactly the requests the CPU arms run whole
        (order n = dN <= 12000 of every timed window).
vs_plain_fp64: the plain FP64 GPU method, one request at a time, against the
        mixed server on the requests of order n <= 16000 of four timed windows,
        with the field error of every mixed result against FP64.
sweep:  the 256-instance batched 2D sweep in captured CUDA graphs.

--impl reference times the reference algorithm's CPU implementation (the
numpy/scipy port in oracle/; the reference itself cannot travel) on the CPU
subset of every timed window, each request run whole.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

WORKLOAD = ("serving stream (continuous batching, 4 requests in flight): Poisson 200 req/s, 50/50 2D-TE disk / 3D-dyadic cube, N log-uniform [500,16000], "
            "k0L U[2pi*5, 2pi*25], 1-64 RHS, 20% geometry re-queries at a new k0; mixed method refined to 1e-10; "
            "detectors 360 ring (2D) / 1024 Fibonacci sphere (3D)")
METRIC = "solves/s (mixed-N 2D/3D request stream, refined to 1e-10 relative residual)"
# DRAM bytes / algorithmic bytes of the trailing update, from an ncu capture of one
# full-size launch (3D N=4000, M = 11616, N = 8032 complex, K = 256: 1.575 GB of DRAM
# traffic vs 1.533 GB algorithmic)
TRAFFIC_RATIO = 1.03


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--requests", type=int, default=8, help="requests per step (window)")
    ap.add_argument("--slots", type=int, default=4, help="requests in flight in the server")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the plain-FP64 comparison, the batched sweep and the CPU extrapolation")
    ap.add_argument("--phases", action="store_true",
                    help="print per-phase device times of the transmission configs instead of the stream bench")
    ap.add_argument("--only", default=None, help="with --phases: one case label, e.g. 3d_N4000:mixed")
    ap.add_argument("--sweep", type=int, default=0,
                    help="run the batched 2D sweep with this many instances (graph replays) instead")
    ap.add_argument("--group", type=int, default=32, help="with --sweep: instances per captured graph")
    ap.add_argument("--compare-fp64", action="store_true",
                    help="the timed windows served by the mixed server and by the plain FP64 method one request "
                         "at a time: throughput, latency and field error of the mixed results against FP64")
    ap.add_argument("--cfg4-fp64", action="store_true",
                    help="the large strong-scattering 3D case, mixed against the plain FP64 method (fields, DOS)")
    ap.add_argument("--cfg4-n", type=int, default=20000, help="with --cfg4-fp64: number of points")
    ap.add_argument("--cfg4-methods", default="mixed,fp64",
                    help="with --cfg4-fp64: the methods to run ('mixed' alone skips the FP64 answer and the "
                         "comparison)")
    ap.add_argument("--case", default=None, choices=sorted(KERNEL_CASES),
                    help="run one small kernel workload twice and exit (the profiles' capture commands)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device):
    """Largest value of x over the ranks of the default process group (the
    timed region of the slowest replica); x itself with one rank."""
    if world <= 1:
        return float(x)
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.rows, self.proc = index, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for nm, v in zip(names, r[4:8]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), float(j["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def windows(steps, warmup, per_step, rank):
    from magreete_gb300 import workloads as W
    return [W.serving_stream(per_step, seed=7919 * (s + 1) + 104729 * rank) for s in range(warmup + steps)]


# ------------------------------------------------------------------ CPU (reference algorithm)

# The CPU legs run whole requests only: the requests of order n = d N <= 12000
# of each window (about two thirds of them, ~3.5 minutes on 16 host cores for
# 20 windows; the larger ones take up to ten minutes each on the host).  The GPU line reports its own solves/s on exactly these requests
# under "subset", so the two arms can be compared like for like.
CPU_SUBSET_N = 12000
# The plain FP64 GPU method, one request at a time, on the requests of order
# n <= 16000 of the first four timed windows (~30 s of complex128 LU).
FP64_SUBSET_N = 16000
FP64_SUBSET_WINDOWS = 4
SUBSET_NOTE = (f"requests of order n = dN <= {CPU_SUBSET_N} of every timed window, run whole on the CPU "
               f"(the GPU arm's 'subset' key: the same requests on the GPU)")


def subset_indices(window, n_max):
    return [i for i, p in enumerate(window) if p.n <= n_max]


def host_info():
    """Host CPU model, thread count and the BLAS numpy calls (for the CPU lines)."""
    info = {"threads": os.cpu_count(), "machine": platform.machine()}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                info["cpu_model"] = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    try:
        cfg = np.show_config(mode="dicts")
        blas = cfg["Build Dependencies"]["blas"]
        info["blas"] = f"{blas.get('name')} {blas.get('version', '')}".strip()
    except Exception:
        pass
    info["numpy"] = np.__version__
    return info


def cpu_request_time(prob):
    """Seconds the numpy/scipy port of the reference algorithm takes for one
    request, run whole: sources at the scatterers and detectors, complex128
    solve (LAPACK, all host threads), propagation to the detectors."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    pts, det = prob.points.numpy(), prob.detectors.numpy()
    if prob.kind.startswith("2d"):
        E0s = O.source_2d(prob.kind, "plane", pts, prob.k0, prob.thetas, 0.2)
        E0d = O.source_2d(prob.kind, "plane", det, prob.k0, prob.thetas, 0.2)
    else:
        E0s = O.source_3d(prob.kind, "plane", pts, prob.k0, prob.u.numpy(), prob.p.numpy(), 0.2)
        E0d = O.source_3d(prob.kind, "plane", det, prob.k0, prob.u.numpy(), prob.p.numpy(), 0.2)
    Ek = O.solve(prob.kind, pts, prob.k0, prob.alpha, prob.radius, E0s)
    O.propagate(prob.kind, pts, det, Ek, prob.k0, prob.alpha, E0d)
    return time.perf_counter() - t0


def cpu_measure(wins):
    """Every CPU-subset request of `wins`, run whole: (requests, seconds, per-window seconds)."""
    count, per = 0, []
    t0 = time.perf_counter()
    for w in wins:
        ts = time.perf_counter()
        for i in subset_indices(w, CPU_SUBSET_N):
            cpu_request_time(w[i])
            count += 1
        per.append(time.perf_counter() - ts)
    return count, time.perf_counter() - t0, per


def cpu_extrapolate(problems):
    """A labelled extrapolation, not a measurement: the port's time for every
    request of `problems` (the larger ones included), costed as
    (8/3 n^3 + 8 n^2 R) / rate + b n^2 with the complex128 LAPACK rate measured
    at n = 4000 and b fitted per dimension to whole requests at small N."""
    from magreete_gb300 import workloads as W
    rng = np.random.default_rng(0)
    n0, r0 = 4000, 64
    A = rng.standard_normal((n0, n0)) + 1j * rng.standard_normal((n0, n0)) + n0 * np.eye(n0)
    B = rng.standard_normal((n0, r0)) + 0j
    np.linalg.solve(A[:500, :500], B[:500])
    t0 = time.perf_counter()
    np.linalg.solve(A, B)
    rate = (8 / 3 * n0 ** 3 + 8 * n0 ** 2 * r0) / (time.perf_counter() - t0)
    del A
    fits, meas = {}, []
    for dim, sizes in (("2d", (500, 1000)), ("3d", (300, 600))):
        xs, ys = [], []
        for N in sizes:
            prob = (W.disk_problem(N, 17 + N, 15.0, n_angles=32) if dim == "2d"
                    else W.cube_problem(N, 17 + N, 15.0, n_dirs=16))
            t = cpu_request_time(prob)
            xs.append(float(prob.n) ** 2)
            ys.append(max(t - (8 / 3 * prob.n ** 3 + 8 * prob.n ** 2 * prob.nrhs) / rate, 0.0))
            meas.append((dim, N, round(t, 3)))
        fits[dim] = float(np.dot(xs, ys) / np.dot(xs, xs))
    t = sum((8 / 3 * p.n ** 3 + 8 * p.n ** 2 * p.nrhs) / rate + fits["2d" if p.kind.startswith("2d") else "3d"] * p.n ** 2
            for p in problems)
    return {"value": len(problems) / t, "unit": "solves/s", "kind": "extrapolation (not a measurement)",
            "lapack_gflops_n4000": rate / 1e9, "calibration_requests": meas,
            "model": "(8/3 n^3 + 8 n^2 R)/rate + b n^2 per request, b fitted per dimension"}


def config_dict(args):
    """The workload description both arms print (the same dict in both lines)."""
    return {"workload": WORKLOAD, "requests_per_step": args.requests,
            "l2": "inputs larger than L2 (matrices 24 n^2 bytes on the GPU)", "subset": SUBSET_NOTE}


def run_reference(args, rank, world):
    """The reference algorithm on the host cores (numpy/scipy port, complex128
    LAPACK with all host threads): each step runs the CPU-subset requests of
    one window whole; value = those requests / the wall time of the K steps.
    Warm-up steps run the smallest subset request of each warm-up window."""
    if rank != 0:
        return
    wins = windows(args.steps, args.warmup, args.requests, 0)
    for w in wins[:args.warmup]:
        idx = subset_indices(w, CPU_SUBSET_N)
        if idx:
            cpu_request_time(min((w[i] for i in idx), key=lambda p: p.n))
    count, wall, per = cpu_measure(wins[args.warmup:])
    val = count / wall
    info = host_info()
    sample = (f"numpy/scipy port of the reference algorithm (oracle/; complex128 solve + propagate, "
              f"{info['threads']} host threads, {info.get('blas', 'numpy BLAS')}): {count} requests of order "
              f"n <= {CPU_SUBSET_N} from the {args.steps} timed windows, each run whole and timed")
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "complex128",
            "data": "synthetic", "config": config_dict(args),
            "cpu_baseline": {"value": val, "unit": "solves/s", "cores": info["threads"], "kind": "port",
                             "sample": sample, "requests": count, "seconds": wall, "host": info,
                             "seconds_per_step": per},
            "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU

def e2e_class_api(problems, precision):
    """The requests one at a time through the drop-in solver classes with numpy
    inputs and CPU results (the reference's plugin boundary): generate_source
    -> solve -> propagate, as the reference driver runs them per frequency.
    Returns (seconds, host-to-device bytes, device-to-host bytes)."""
    from magreete_gb300 import Transmission2D_vector, Transmission3D_vector
    h2d = d2h = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for prob in problems:
        pts, det = prob.points.numpy(), prob.detectors.numpy()
        if prob.kind.startswith("2d"):
            s = Transmission2D_vector(pts, source="plane", precision=precision)
            E0s = s.generate_source(pts, prob.k0, prob.thetas, 0.2)
            E0d = s.generate_source(det, prob.k0, prob.thetas, 0.2)
        else:
            s = Transmission3D_vector(pts, source="plane", precision=precision)
            u, p = prob.u.numpy(), prob.p.numpy()
            E0s = s.generate_source(pts, prob.k0, u, p, 0.2)
            E0d = s.generate_source(det, prob.k0, u, p, 0.2)
        Ek = s.solve(prob.k0, prob.alpha, prob.radius, E0s)
        Ed = s.propagate(det, Ek, prob.k0, prob.alpha, E0d)
        # points copied in three times (class, two sources), the detectors twice;
        # sources, fields and detector fields each cross once per direction
        h2d += 3 * pts.nbytes + 2 * det.nbytes + E0s.numel() * 16 + Ek.numel() * 16 + E0d.numel() * 16
        d2h += E0s.numel() * 16 + E0d.numel() * 16 + Ek.numel() * 16 + Ed.numel() * 16
    torch.cuda.synchronize()
    return time.perf_counter() - t0, h2d, d2h


def serve_windows(srv, wins, dev_inputs=None):
    """Serve each window's requests at their arrival times; (results, seconds)."""
    from magreete_gb300 import serve
    res = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k, w in enumerate(wins):
        res += serve.serve_stream(w, device_inputs=dev_inputs[k] if dev_inputs is not None else None, server=srv)
    torch.cuda.synchronize()
    return res, time.perf_counter() - t0


def pick(wins, dev_inputs, n_max):
    """The requests of order n <= n_max of each window (and their device inputs)."""
    sw, sd = [], []
    for w, di in zip(wins, dev_inputs):
        idx = subset_indices(w, n_max)
        sw.append([w[i] for i in idx])
        sd.append([di[i] for i in idx])
    return sw, sd


def lat_stats(res):
    lat = sorted(1e3 * r.latency for r in res)
    return {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))}


def rel_err(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def vs_plain_fp64(srv, wins, dev_inputs):
    """The mixed server against the plain FP64 method run one request at a
    time, on the FP64 subset: solves/s, latency, and the field error of every
    mixed result against the FP64 one."""
    from magreete_gb300 import serve
    sw, sd = pick(wins, dev_inputs, FP64_SUBSET_N)
    mixed, t_mixed = serve_windows(srv, sw, sd)
    plain = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for w, di in zip(sw, sd):
        plain += serve.serve_sequential(w, "fp64", di)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    n = sum(len(w) for w in sw)
    ek = [rel_err(m.Ek, p.Ek) for m, p in zip(mixed, plain)]
    ed = [rel_err(m.E_det, p.E_det) for m, p in zip(mixed, plain)]
    return {"sample": f"requests of order n <= {FP64_SUBSET_N} of the first {len(sw)} timed windows",
            "requests": n, "sizes": [(p.kind[:2], p.n, p.nrhs) for w in sw for p in w],
            "mixed_served": {"solves_per_s": n / t_mixed, "seconds": t_mixed, "latency_ms": lat_stats(mixed),
                             "max_rel_residual": max(r.rel_residual for r in mixed)},
            "plain_fp64_one_at_a_time": {"solves_per_s": n / t_plain, "seconds": t_plain,
                                         "latency_ms": lat_stats(plain)},
            "ratio": t_plain / t_mixed,
            "max_field_err_vs_fp64": {"Ek": max(ek), "E_det": max(ed)}}


def update_roofline(dom_n, dom_ms, dom_flops, dom_bytes, hbm, bf16, src):
    """Roofline entry of the trailing update from its timed windows (count,
    total ms, algorithmic flops and bytes) and the measured peaks (copy GB/s,
    bf16 TFLOP/s).  The windows run with K = 128 (one block) or K = 256 (a
    pair of blocks).  Per algorithmic flop a window moves 16 B of complex64 C
    per 8 K flops and issues three F16 split products, so its roof is the
    larger of (algorithmic bytes / copy bandwidth) and (3 x flops / bf16
    peak): HBM at K = 128, tensor at K = 256.  For the windows together the
    larger of the two totals is taken (a lower bound of the roof time, so the
    fraction is conservative)."""
    gbs = (dom_bytes / (dom_ms * 1e-3) / 1e9) if dom_ms > 0 else None
    tflops = (dom_flops / (dom_ms * 1e-3) / 1e12) if dom_ms > 0 else None
    t_hbm = dom_bytes / (hbm * 1e9) if hbm else 0.0
    t_tc = 3 * dom_flops / (bf16 * 1e12) if bf16 else 0.0
    tensor_bound = t_tc >= t_hbm
    return {"kernel": "tc::cgemm_split3_kernel<F16x2> + operand splits (LU trailing update, tcgen05 kind::f16, "
                      "128 x 256 tiles, K = 256 for paired blocks, else 128)",
            "bound": "tensor" if tensor_bound else "hbm",
            "achieved": tflops if tensor_bound else gbs,
            "peak": bf16 / 3 if tensor_bound else hbm,
            "unit": "TFLOP/s" if tensor_bound else "GB/s",
            "frac": ((t_tc if tensor_bound else t_hbm) / (dom_ms * 1e-3)) if dom_ms > 0 else None,
            "hbm_achieved_gbs": gbs, "hbm_peak_gbs": hbm,
            "hbm_frac": (gbs / hbm) if gbs else None,
            "traffic": (dom_bytes / dom_n * TRAFFIC_RATIO) if dom_n else None,
            "peak_source": (f"bf16_tflops of {src} peaks / 3 (three kind::f16 split products per algorithmic "
                            f"flop)" if tensor_bound else f"hbm_gbs of {src} peaks (copy bandwidth)"),
            "algorithmic_bytes_per_launch": dom_bytes / dom_n if dom_n else None,
            "algorithmic_flops_per_launch": dom_flops / dom_n if dom_n else None,
            "launches": dom_n, "avg_launch_ms": dom_ms / dom_n if dom_n else None,
            "achieved_tflops": tflops,
            "tensor_peak_tflops": bf16,
            "tensor_frac": (3 * tflops / bf16) if tflops else None,
            "tensor_note": "three kind::f16 split products per algorithmic flop; tensor_frac = 3 x achieved / "
                           f"bf16_tflops of {src} peaks",
            "measured": "CUDA events around each launch on its stream, sequential pass over the first timed window"}


def secondary_rooflines():
    """The two other kernels with large shares of the stream, timed alone with
    CUDA events after the timed region:
      * the tensor-core refinement residual R = B - M X (3D N=4000: n = 12000,
        64 right-hand sides).  Its algorithmic work is the 28 digit-pair real
        products of the FP16 digit split, 224 n^2 R tensor flops (8 n^2 R per
        product), held to the measured bf16 (= fp16) dense peak;
      * the complex64 LU of order 2000 (2D N=1000), where the trailing update is
        small and the time is the panel chain's latency, tile and partial
        pivoting."""
    from magreete_gb300 import engine as E, selfterm
    from magreete_gb300 import workloads as W
    hbm, bf16, src = measured_peaks()
    dev = torch.device("cuda")
    out = {}
    prob = W.cfg2()
    pts = prob.points.to(dev)
    coef = prob.alpha * prob.k0 ** 2
    shift = selfterm.diagonal_shift(prob.kind, prob.k0, prob.alpha, prob.radius)
    (Mdf,) = E.assemble_system(prob.kind, pts, prob.k0, coef, shift, ("cdf",))
    n, R = prob.n, prob.nrhs
    gen = torch.Generator(device=dev).manual_seed(5)
    X = torch.randn(n, R, dtype=torch.complex128, device=dev, generator=gen)
    B = torch.randn(n, R, dtype=torch.complex128, device=dev, generator=gen)
    op = E.ResidualOperator(Mdf, R)
    for _ in range(2):
        op(X, B)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    e0.record()
    for _ in range(reps):
        op(X, B)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    e0.record()
    for _ in range(reps):
        E.residual(Mdf, X, B)
    e1.record()
    torch.cuda.synchronize()
    ms_call = e0.elapsed_time(e1) / reps
    tflop = 224.0 * n * n * R / 1e12
    nbytes = 14.0 * n * n + 3 * 16.0 * n * R
    out["residual_tc"] = {"kernel": "rtc::residual_tc_kernel (+ the right-hand sides' scales and digits, reduction "
                                    "of the K splits); M's digits made beforehand (mgt_residual_prepare)",
                          "bound": "tensor", "n": n, "nrhs": R, "ms": ms,
                          "achieved": tflop / (ms * 1e-3), "peak": bf16, "unit": "TFLOP/s",
                          "frac": tflop / (ms * 1e-3) / bf16,
                          "algorithmic_tflop": tflop,
                          "hbm_achieved_gbs": nbytes / (ms * 1e-3) / 1e9, "hbm_peak_gbs": hbm,
                          "hbm_frac": nbytes / (ms * 1e-3) / 1e9 / hbm,
                          "peak_source": f"bf16_tflops of {src} peaks (kind::f16 runs at the bf16 rate); "
                                         "224 n^2 R flops = 28 digit-pair products of the 7-digit split",
                          "complex_macs_per_s": float(n) * n * R / (ms * 1e-3),
                          "one_call_ms_with_digit_pass": ms_call,
                          "measured": "CUDA events over 5 applications of mgt_residual_apply, after 2"}
    del Mdf, X, B, op
    prob = W.cfg1()
    pts = prob.points.to(dev)
    coef = prob.alpha * prob.k0 ** 2
    shift = selfterm.diagonal_shift(prob.kind, prob.k0, prob.alpha, prob.radius)
    (M32,) = E.assemble_system(prob.kind, pts, prob.k0, coef, shift, ("c64",))
    for piv in ("tile", "partial"):
        ts = []
        for rep in range(4):
            A = torch.empty_strided(M32.size(), M32.stride(), dtype=M32.dtype, device=dev)
            A.copy_(M32)
            torch.cuda.synchronize()
            e0.record()
            E.lu_factor(A, check_singular=False, pivoting=piv)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        lu_ms = min(ts[1:])
        out[f"lu_panel_{piv}"] = {"bound": "latency (the panel chain)", "n": prob.n, "pivoting": piv,
                                  "lu_ms": lu_ms, "us_per_column": 1e3 * lu_ms / prob.n,
                                  "note": "complex64 LU of order 2000; the trailing update is a small part of it"}
    return out


def sweep_measure(count, group):
    """The batched 2D sweep (TE disk, N uniform in [500, 4000], 16 angles):
    groups of instances captured into one CUDA graph each, concurrency,
    pivoting and LU block width chosen by the autotuner on the first group;
    instances/s over graph replays (one warm replay per group first)."""
    from magreete_gb300 import batch
    from magreete_gb300 import workloads as W
    probs = W.sweep_2d(count)
    groups = [probs[i:i + group] for i in range(0, len(probs), group)]
    best = batch.autotune(groups[0])
    choice = {k: best[k] for k in ("branches", "pivoting", "outer_block")}
    t_total, worst, extra_total, flops, refactored = 0.0, 0.0, 0, 0.0, 0
    for g in groups:
        sw = batch.BatchedSweep(g, **choice)
        sw.warmup()
        sw.capture()
        sw.replay()
        torch.cuda.synchronize()
        sw.refactored = 0
        t0 = time.perf_counter()
        extra, res = sw.replay()
        t_total += time.perf_counter() - t0
        worst = max(worst, max(res))
        extra_total += sum(extra)
        refactored += sw.refactored
        flops += sum(8 / 3 * p.n ** 3 for p in g)
        del sw
        torch.cuda.empty_cache()
    return {"case": "batched 2D sweep", "instances": len(probs), "group": group,
            "autotune": {k: v for k, v in best.items() if k != "candidates"}, "candidates": best.get("candidates"),
            "seconds": t_total, "instances_per_s": len(probs) / t_total,
            "lu_tflops_effective": flops / t_total / 1e12, "max_rel_residual": worst,
            "corrections_after_graph": extra_total, "refactored_with_partial_pivoting": refactored}


def run_ours(args, rank, world, local):
    import magreete_gb300  # noqa: F401
    from magreete_gb300 import _lib
    from magreete_gb300 import serve

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    _lib.load()
    wins = windows(args.steps, args.warmup, args.requests, rank)
    dev_inputs = [[(p.points.to(dev), p.detectors.to(dev)) for p in w] for w in wins]
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    srv = serve.Server(slots=args.slots, precision=args.precision)
    for w, di in zip(wins[:args.warmup], dev_inputs[:args.warmup]):
        serve.serve_stream(w, device_inputs=di, server=srv)
    torch.cuda.synchronize()
    # ---- timed region: device-resident inputs
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    _lib.diag_reset(enable_timing=True)
    clocks.start()
    t0 = time.perf_counter()
    lat, iters, rres = [], [], []
    for w, di in zip(wins[args.warmup:], dev_inputs[args.warmup:]):
        res = serve.serve_stream(w, device_inputs=di, server=srv)
        lat += [r.latency for r in res]
        iters += [r.iterations for r in res]
        rres += [r.rel_residual for r in res]
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    clk = clocks.stop()
    launches, mix_n, mix_ms, mix_flops, mix_bytes = _lib.diag_read()
    # the dominant kernel's own rate: the first timed window once more, one request
    # at a time, with CUDA events around every trailing-update launch
    _lib.diag_reset(enable_timing=True)
    serve.serve_sequential(wins[args.warmup], args.precision, dev_inputs[args.warmup])
    torch.cuda.synchronize()
    _, dom_n, dom_ms, dom_flops, dom_bytes = _lib.diag_read()
    _lib.diag_reset(enable_timing=False)
    barrier()
    elapsed = max_over_ranks(elapsed, world, dev)
    n_req = args.steps * args.requests * world
    value = n_req / elapsed
    # ---- the CPU subset on the GPU (the requests the CPU arms run whole), served the same way
    sub_w, sub_d = pick(wins[args.warmup:], dev_inputs[args.warmup:], CPU_SUBSET_N)
    sub_res, sub_t = serve_windows(srv, sub_w, sub_d)
    n_sub = sum(len(w) for w in sub_w)
    subset = {"value": n_sub / sub_t, "unit": "solves/s", "requests": n_sub, "seconds": sub_t,
              "sample": SUBSET_NOTE, "latency_ms": lat_stats(sub_res)}
    # ---- the plain FP64 method on a subset of the timed windows
    fp64_cmp = None
    if not args.no_extras:
        fp64_cmp = vs_plain_fp64(srv, wins[args.warmup:args.warmup + FP64_SUBSET_WINDOWS],
                                 dev_inputs[args.warmup:args.warmup + FP64_SUBSET_WINDOWS])
    srv.close()
    # ---- e2e through the public API with host buffers
    e2e = e2e_api = None
    if not args.no_e2e:
        # the same windows through the public Server API with host inputs and host
        # results: points / detectors copied in, fields copied out, inside the timed region
        esrv = serve.Server(slots=args.slots, precision=args.precision, host_results=True)
        barrier()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for w in wins[args.warmup:]:
            serve.serve_stream(w, server=esrv)
        torch.cuda.synchronize()
        e_el = time.perf_counter() - t1
        h2d, d2h = esrv.h2d_bytes, esrv.d2h_bytes
        esrv.close()
        e_el = max_over_ranks(e_el, world, dev)
        e2e = {"value": n_req / e_el, "unit": "solves/s", "h2d_bytes_per_step": h2d // args.steps,
               "d2h_bytes_per_step": d2h // args.steps, "api": "magreete_gb300.serve.Server(host_results=True)"}
        # the first timed window through the drop-in classes, one request at a
        # time, after one untimed pass over it (the classes' first-use costs)
        e2e_class_api(wins[args.warmup], args.precision)
        t_api, h2d_api, d2h_api = e2e_class_api(wins[args.warmup], args.precision)
        e2e_api = {"value": len(wins[args.warmup]) / t_api, "unit": "solves/s", "requests": len(wins[args.warmup]),
                   "h2d_bytes": h2d_api, "d2h_bytes": d2h_api,
                   "api": "Transmission2D_vector / Transmission3D_vector: generate_source x2, solve, propagate; "
                          "numpy in, CPU tensors out; one request at a time (first timed window)"}
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    hbm, bf16, src = measured_peaks()
    roofline = update_roofline(dom_n, dom_ms, dom_flops, dom_bytes, hbm, bf16, src)
    roofline["in_mix_tflops"] = (mix_flops / (mix_ms * 1e-3) / 1e12) if mix_ms > 0 else None
    secondary = secondary_rooflines()
    sweep = None if args.no_extras else sweep_measure(256, 32)
    cpu = cpu_extra = None
    if world == 1:
        first = wins[args.warmup:args.warmup + 2]
        count, wall, _ = cpu_measure(first)
        info = host_info()
        cpu = {"value": count / wall, "unit": "solves/s", "cores": info["threads"], "kind": "port",
               "sample": f"numpy/scipy port of the reference algorithm (oracle/; complex128, {info['threads']} host "
                         f"threads, {info.get('blas', 'numpy BLAS')}): the {count} requests of order "
                         f"n <= {CPU_SUBSET_N} of the first {len(first)} timed windows, each run whole and timed",
               "requests": count, "seconds": wall, "host": info}
        if not args.no_extras:
            cpu_extra = cpu_extrapolate([p for w in wins[args.warmup:] for p in w])
    lat_ms = sorted(1e3 * x for x in lat)
    refinement = {"max_iterations": max(iters), "max_rel_residual": max(rres)}
    if fp64_cmp is not None:
        refinement["max_field_err_vs_fp64"] = dict(fp64_cmp["max_field_err_vs_fp64"],
                                                   sample=fp64_cmp["sample"])
    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "complex64 LU + double-float residual" if args.precision == "mixed" else "complex128",
            "data": "synthetic", "precision": args.precision, "parallelism": f"replicas x{world}",
            "config": config_dict(args),
            "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99))},
            "refinement": refinement, "subset": subset, "vs_plain_fp64": fp64_cmp, "sweep": sweep,
            "e2e": e2e, "e2e_class_api": e2e_api, "roofline": roofline, "roofline_other": secondary,
            "cpu_baseline": cpu, "cpu_full_stream_extrapolated": cpu_extra, "clocks": clk,
            "gpu_launches": launches}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_phases(args):
    """Per-phase device times (CUDA events) of one request: 2D TE N=1000 (64 RHS, 360 detectors),
    3D dyadic N=4000 (64 RHS, 1024 detectors) and 3D dyadic N=9000, both methods."""
    from magreete_gb300 import _lib, engine as E, selfterm, serve
    from magreete_gb300 import workloads as W
    _lib.load()
    dev = torch.device("cuda")

    def ev():
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        return e

    cases = [("2d_te_N1000", W.cfg1(), ("mixed", "fp64")), ("3d_N4000", W.cfg2(), ("mixed", "fp64")),
             ("3d_N9000", W.cube_problem(9000, 3, 15.0), ("mixed",)),
             ("3d_ball_N20000", W.cfg4(), ("mixed",))]
    only = args.only.split(":") if args.only else None
    if only and only[0] == "dos_2d_te_N1000":
        run_dos(only[1] if len(only) > 1 else None)
        return
    for label, prob, precs in cases:
        for prec in precs:
            if only and (label != only[0] or prec != only[1]):
                continue
            for rep in range(1 if label == "3d_ball_N20000" else 2):
                pts, det = prob.points.to(dev), prob.detectors.to(dev)
                coef = prob.alpha * prob.k0 ** 2
                shift = selfterm.diagonal_shift(prob.kind, prob.k0, prob.alpha, prob.radius)
                E0s, E0d = serve.incident_fields(prob, pts, det)
                n, R = prob.n, prob.nrhs
                B = E0s.reshape(n, R).contiguous()
                torch.cuda.synchronize()
                _lib.diag_reset(enable_timing=True)
                e0 = ev()
                if prec == "fp64":
                    (M,) = E.assemble_system(prob.kind, pts, prob.k0, coef, shift, ("c128",))
                    e1 = ev()
                    f = E.lu_factor(M, check_singular=False)
                    e2 = ev()
                    X = E.lu_solve(f, B)
                    it, rr = 0, None
                else:
                    Mdf, M32 = E.assemble_system(prob.kind, pts, prob.k0, coef, shift, ("cdf", "c64"))
                    e1 = ev()
                    f = E.lu_factor(M32, check_singular=False)
                    e2 = ev()
                    X, it, rr = E.solve_refined(Mdf, f, B)
                e3 = ev()
                E.propagate(prob.kind, det, pts, prob.k0, coef, X, E0d.reshape(-1, R), precision=prec)
                e4 = ev()
                torch.cuda.synchronize()
                extra = {}
                if prec == "mixed":
                    # components of the refined solve, timed on their own (outside the phases above)
                    t_a = ev()
                    E.lu_solve(f, B.to(torch.complex64))
                    t_b = ev()
                    E.residual(Mdf, X, B)
                    t_c = ev()
                    torch.cuda.synchronize()
                    extra = {"one_lu_solve_ms": t_a.elapsed_time(t_b), "one_residual_ms": t_b.elapsed_time(t_c)}
                _, dn, dms, dfl, dby = _lib.diag_read()
                _lib.diag_reset(enable_timing=False)
                if rep == 0 and label != "3d_ball_N20000":
                    continue
                lu = e1.elapsed_time(e2)
                print(json.dumps({"case": label, "precision": prec, "n": n, "nrhs": R,
                                  "assemble_ms": e0.elapsed_time(e1), "lu_ms": lu,
                                  "lu_tflops": 8 / 3 * n ** 3 / lu / 1e9, "solve_ms": e2.elapsed_time(e3),
                                  "refine_iterations": it, "rel_residual": rr, "propagate_ms": e3.elapsed_time(e4),
                                  "trailing_update": {"launches": dn, "ms": dms,
                                                      "tflops": dfl / dms / 1e9 if dms else None}, **extra}),
                      flush=True)


def run_dos(precision=None):
    """Mean DOS of the 2D TE N=1000 config at 8 frequencies (1000 points in the
    disk of radius L/2), both methods; their agreement and the time per
    frequency."""
    from magreete_gb300 import Transmission2D_vector, _lib
    from magreete_gb300 import workloads as W
    _lib.load()
    prob = W.cfg1()
    mp = W.dos_points_cfg1()
    out = {}
    for prec in ((precision,) if precision else ("mixed", "fp64")):
        s = Transmission2D_vector(prob.points.cuda(), source="plane", precision=prec)
        s.mean_DOS_measurements(mp.cuda(), W.dos_frequencies_cfg1()[0], prob.alpha, prob.radius)
        torch.cuda.synchronize()
        vals, t0 = [], time.perf_counter()
        for k0 in W.dos_frequencies_cfg1():
            vals.append(float(s.mean_DOS_measurements(mp.cuda(), k0, prob.alpha, prob.radius)))
        torch.cuda.synchronize()
        out[prec] = {"dos": vals, "ms_per_frequency": 1e3 * (time.perf_counter() - t0) / len(vals)}
    if "mixed" in out and "fp64" in out:
        a, b = np.array(out["mixed"]["dos"]), np.array(out["fp64"]["dos"])
        out["max_rel_diff_mixed_vs_fp64"] = float(np.max(np.abs(a - b) / np.abs(b)))
    print(json.dumps({"case": "dos_2d_te_N1000", "frequencies": len(W.dos_frequencies_cfg1()), "points": len(mp),
                      **out}), flush=True)


def run_sweep(args):
    """The batched 2D sweep alone (see sweep_measure)."""
    from magreete_gb300 import _lib
    _lib.load()
    print(json.dumps(sweep_measure(args.sweep, args.group)), flush=True)


def run_compare_fp64(args):
    """Mixed served stream vs the plain FP64 method one request at a time, on
    the same windows; field errors of every mixed result against FP64."""
    from magreete_gb300 import _lib, serve
    from magreete_gb300 import workloads as W
    _lib.load()
    dev = torch.device("cuda")
    wins = windows(args.steps, args.warmup, args.requests, 0)
    timed = [p for w in wins[args.warmup:] for p in w]
    # warm both methods up on small requests of each kind
    small = [W.disk_problem(500, 1, 10.0, n_angles=8), W.cube_problem(300, 2, 10.0, n_dirs=4)]
    for prec in ("mixed", "fp64"):
        serve.serve_sequential(small, prec)
    torch.cuda.synchronize()

    def lat_stats(res):
        lat = sorted(1e3 * r.latency for r in res)
        return float(np.percentile(lat, 50)), float(np.percentile(lat, 99))

    srv = serve.Server(slots=args.slots, precision="mixed")
    t0 = time.perf_counter()
    mixed = []
    for w in wins[args.warmup:]:
        mixed += serve.serve_stream(w, server=srv)
    torch.cuda.synchronize()
    t_mixed = time.perf_counter() - t0
    srv.close()
    t0 = time.perf_counter()
    plain = []
    for w in wins[args.warmup:]:
        plain += serve.serve_sequential(w, "fp64")
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0

    def rel(a, b):
        return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))
    ek = [rel(m.Ek, p.Ek) for m, p in zip(mixed, plain)]
    ed = [rel(m.E_det, p.E_det) for m, p in zip(mixed, plain)]
    m50, m99 = lat_stats(mixed)
    p50, p99 = lat_stats(plain)
    print(json.dumps({
        "mode": "compare_fp64", "workload": WORKLOAD, "requests": len(timed),
        "sizes": [(p.kind, p.n, p.nrhs) for p in timed],
        "mixed_served": {"solves_per_s": len(timed) / t_mixed, "seconds": t_mixed, "p50_ms": m50, "p99_ms": m99,
                         "slots": args.slots, "max_rel_residual": max(r.rel_residual for r in mixed)},
        "plain_fp64_one_at_a_time": {"solves_per_s": len(timed) / t_plain, "seconds": t_plain, "p50_ms": p50,
                                     "p99_ms": p99},
        "speedup": t_plain / t_mixed,
        "field_error_vs_fp64": {"max_rel_Ek": max(ek), "max_rel_E_det": max(ed)}}), flush=True)


def run_cfg4_fp64(args):
    """The large strong-scattering 3D case (unit ball, N = 20000, n = 60000,
    n_ref = 2.0, k0 L = 2 pi 15, 128 right-hand sides, 1024 detectors) with
    the mixed method and with the plain FP64 method (the FP64 answer at this
    size, which the host oracle cannot hold): the error of every field and of
    the mean DOS at 32 points in the ball of radius L/2, mixed against FP64,
    and the time of each."""
    from magreete_gb300 import Transmission3D_vector, _lib
    from magreete_gb300 import workloads as W
    _lib.load()
    prob = W.ball_problem(args.cfg4_n, 4, 15.0)
    mp = 0.5 * W.ball_points(32, 44)
    dev = torch.device("cuda")
    pts, det = prob.points.to(dev), prob.detectors.to(dev)
    out = {"case": f"3D ball N={prob.N} (n={prob.n}), n_ref 2.0, k0L 2pi*15, {prob.nrhs} RHS, "
                   f"{det.shape[0]} detectors; mean DOS at {len(mp)} points"}
    res = {}
    P = mp.shape[0]
    methods = [m for m in ("mixed", "fp64") if m in args.cfg4_methods.split(",")]
    for prec in methods:
        # one factorisation per method serves the fields and the DOS (the
        # classes' solve and mean_DOS_measurements would each factor: at this
        # size one FP64 LU takes minutes)
        s = Transmission3D_vector(pts, source="plane", precision=prec)
        E0s = s.generate_source(pts, prob.k0, prob.u, prob.p, 0.2)
        E0d = s.generate_source(det, prob.k0, prob.u, prob.p, 0.2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fac = s._factorization(prob.k0, prob.alpha, prob.radius, True, "Rayleigh")
        Ek = fac.solve(E0s.reshape(prob.n, -1).to(torch.complex128))
        Ed = s.propagate(det, Ek, prob.k0, prob.alpha, E0d)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        dots = s._dos_terms(fac, mp.to(dev), prob.k0, prob.radius, True, "Rayleigh", False)
        dos = float(torch.imag(dots.sum() / P * complex(s._DOS_PREF[s.kind](prob.k0, prob.alpha))))
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        res[prec] = (Ek.cpu(), Ed.cpu(), dos)
        out[prec] = {"factor_solve_propagate_s": t1 - t0, "mean_dos_s": t2 - t1, "mean_dos": dos,
                     "refine_iterations": getattr(fac, "last_iterations", 0),
                     "rel_residual": getattr(fac, "last_residual", None),
                     "pivoting": getattr(getattr(fac, "f", None), "pivoting", None)}
        del Ek, Ed, s, fac, dots
        torch.cuda.empty_cache()
    if len(res) < 2:
        print(json.dumps(out), flush=True)
        return
    (Em, Dm, dm), (Ef, Df, df) = res["mixed"], res["fp64"]
    col = lambda a, b: (torch.linalg.norm(a - b, dim=0) / torch.linalg.norm(b, dim=0)).max().item()
    out["error_mixed_vs_fp64"] = {
        "Ek_rel_frobenius": rel_err(Em, Ef), "Ek_worst_field": col(Em, Ef),
        "E_det_rel_frobenius": rel_err(Dm, Df), "E_det_worst_field": col(Dm.reshape(-1, prob.nrhs),
                                                                          Df.reshape(-1, prob.nrhs)),
        "mean_dos_rel": abs(dm - df) / abs(df)}
    print(json.dumps(out), flush=True)


# Small workloads of single kernels, each run twice (the second launch is the
# one a profile captures): 3D dyadic N = 2000 (n = 6000) assembly and
# tensor-core residual with 64 right-hand sides; the complex64 LU of 2D
# N = 1000 (n = 2000) and 3D N = 4000 (n = 12000), tile or partial pivoting.
KERNEL_CASES = ("assemble_3d_N2000", "residual_3d_N2000", "lu_2d_N1000_tile", "lu_2d_N1000_partial",
                "lu_3d_N4000_tile", "lu_3d_N4000_partial")


def run_case(name):
    from magreete_gb300 import engine as E, selfterm
    from magreete_gb300 import workloads as W
    dev = torch.device("cuda")
    if name.startswith("lu_"):
        prob = W.cfg1() if "2d_N1000" in name else W.cfg2()
    else:
        prob = W.cube_problem(2000, 2, 10.0)
    pts = prob.points.to(dev)
    coef = prob.alpha * prob.k0 ** 2
    shift = selfterm.diagonal_shift(prob.kind, prob.k0, prob.alpha, prob.radius)
    if name == "assemble_3d_N2000":
        for _ in range(2):
            out = E.assemble_system(prob.kind, pts, prob.k0, coef, shift, ("cdf", "c64"))
            torch.cuda.synchronize()
            del out
    elif name == "residual_3d_N2000":
        (Mdf,) = E.assemble_system(prob.kind, pts, prob.k0, coef, shift, ("cdf",))
        g = torch.Generator(device=dev).manual_seed(1)
        X = torch.randn(prob.n, 64, dtype=torch.complex128, device=dev, generator=g)
        B = torch.randn(prob.n, 64, dtype=torch.complex128, device=dev, generator=g)
        for _ in range(2):
            E.residual(Mdf, X, B)
    else:
        (M32,) = E.assemble_system(prob.kind, pts, prob.k0, coef, shift, ("c64",))
        for _ in range(2):
            E.lu_factor(M32.clone(), check_singular=False, pivoting=name.rsplit("_", 1)[1])
    torch.cuda.synchronize()
    print(json.dumps({"case": name, "ok": True}), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.case:
        run_case(args.case)
        return
    if args.compare_fp64:
        run_compare_fp64(args)
        return
    if args.cfg4_fp64:
        run_cfg4_fp64(args)
        return
    if args.phases:
        run_phases(args)
        return
    if args.sweep:
        run_sweep(args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
