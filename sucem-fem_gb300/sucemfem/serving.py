"""Continuous-batching server for driven ABC solves on one GPU.

Requests (box size, mesh divisions, basis order, k0, material seed) arrive
over time.  Host preparation (mesh, function space, LU symbolic analysis)
runs in a worker pool as soon as a request arrives; a scheduler admits
prepared requests in arrival order while a solve slot is free and the
request's device memory (LU arena + matrices + vectors, known exactly from
the symbolic analysis) fits the HBM budget; requests that can never fit are
rejected with a status.  Each slot is a thread with its own CUDA stream, so
the assembly, factorisation and refinement of several requests overlap on
the device.  Per-request results carry the solution, the refinement
residual, the status and the latency (arrival -> solution on the host).

Every request is computed by the same kernels on the same inputs whatever
else is in flight; only the order of a few floating-point additions in the
LU solve can differ, so a result alone and in a mix agree to the refinement
tolerance (tests/test_serving_gpu.py)."""
import math
import queue
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _device, autotune
from .Consts import c0, Z0
from .mesh import BoxMesh
from .Sources.point_source import evaluate_point_sources
from .solvers import DeviceCSR, RefinedDirectSolver, lu_for_space
from .space import FunctionSpace
from ._native import call, ptr


@dataclass
class DrivenRequest:
    rid: int
    cubes: int
    order: int
    size: float
    k0: float
    seed: int
    arrival: float = 0.0


@dataclass
class DrivenResult:
    rid: int
    status: str
    n_dofs: int = 0
    residual: float = float("nan")
    iterations: int = 0
    latency: float = float("nan")
    solve_seconds: float = float("nan")
    x: np.ndarray = field(default=None, repr=False)


def make_request_stream(n, rate, cubes=(6, 48), orders=(1, 2), wavelengths=(1.0, 6.0), size=1.0,
                        seed=0):
    """Poisson arrivals (mean ``rate`` per second), divisions log-uniform in
    ``cubes``, order uniform over ``orders``, k0 so that the box spans a
    uniform number of wavelengths in ``wavelengths``."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    lo, hi = np.log(cubes[0]), np.log(cubes[1] + 1)
    out = []
    for i in range(n):
        nc = int(min(cubes[1], max(cubes[0], math.floor(math.exp(rng.uniform(lo, hi))))))
        order = int(rng.choice(orders))
        w = rng.uniform(*wavelengths)
        out.append(DrivenRequest(i, nc, order, size, 2 * np.pi * w / size, int(rng.integers(1 << 30)),
                                 float(t[i])))
    return out


class _Prepared:
    def __init__(self, req, tuner=None):
        self.req = req
        mesh = BoxMesh(req.size, req.size, req.size, req.cubes, req.cubes, req.cubes)
        self.V = FunctionSpace(mesh, order=req.order)
        self.eps = np.random.default_rng(req.seed).uniform(1.0, 4.0, self.V.nt)
        self.lu = lu_for_space(self.V, leaf_size=96)
        if tuner is not None:
            # an LU plan tuned earlier for this size class (no trials here:
            # they would add to this request's latency)
            key = autotune.size_class(self.lu.info["n"], self.lu.info["nnz"],
                                      "c64_f%d" % self.lu.info["max_front"])
            plan = tuner.lookup("lu_plan", key)
            if plan is not None:
                self.lu.configure(*plan)
        n, nnz = self.V.n, self.V.nnz
        # complex64 arena + A32 + A64 + 3x pattern ints + solver vectors (~40 n complex128)
        self.bytes = (self.lu.info["arena"] * 8 + nnz * (8 + 16 + 4) + (n + 1) * 4 + n * 16 * 40
                      + self.lu.info["n"] * 16 * 2)


class SolveServer:
    def __init__(self, hbm_budget_bytes=None, slots=4, precision="fp32-ir", tol=1e-8,
                 prep_workers=4, keep_solutions=False, tuner=None):
        dev = _device.device()
        free, total = torch.cuda.mem_get_info(dev)
        self.budget = int(hbm_budget_bytes if hbm_budget_bytes is not None else 0.8 * free)
        self.slots = slots
        self.precision = precision
        self.tol = tol
        self.prep_workers = prep_workers
        self.keep = keep_solutions
        self.tuner = tuner
        self._lock = threading.Lock()
        self._reserved = 0
        self.stats = {}

    # -- one solve on the calling thread's stream ---------------------------
    def _solve(self, p):
        V, req = p.V, p.req
        dev = _device.device()
        stream = torch.cuda.Stream(dev)
        with torch.cuda.stream(stream):
            sp = stream.cuda_stream
            h = V.upload()
            e64 = torch.as_tensor(p.eps, dtype=torch.float64, device=dev)
            A64 = torch.empty(V.nnz, dtype=torch.complex128, device=dev)
            call("sucem_assemble_helmholtz", h, 8, ptr(e64), None, float(req.k0), ptr(A64), sp)
            indptr = torch.as_tensor(V.indptr.astype(np.int32), device=dev)
            indices = torch.as_tensor(V.indices, device=dev)
            rs = RefinedDirectSolver(DeviceCSR(indptr, indices, A64, V.n), p.lu)
            if self.precision == "fp64":
                rs.factor(A64, "c128")
            else:
                # the single-precision LU input: the FP64 matrix rounded
                # (one refinement iteration fewer than the FP32 assembly's)
                A32 = rs.vec.convert(A64, torch.empty(V.nnz, dtype=torch.complex64, device=dev))
                rs.factor(A32, "c64")
            c = req.size / 2
            _, dofs, con = evaluate_point_sources(V, np.array([[c, c, c]]), np.array([[0, 0, 1.0]]))
            b = np.zeros(V.n, dtype=np.complex128)
            b[dofs[0]] += -1j * req.k0 * Z0 * con[0]
            bd = torch.as_tensor(b, device=dev)
            x, info = rs.solve(bd, tol=self.tol, method="gmres", maxit=30)
            xh = x.cpu().numpy()
            stream.synchronize()
        return xh, info

    # -- serving loop ---------------------------------------------------------
    def run(self, requests, realtime=True, time_scale=1.0):
        """Serve ``requests`` (arrival times in seconds).  Returns results in
        request order."""
        t0 = time.perf_counter()
        results = {}
        prepared = queue.Queue()
        done_prep = threading.Event()

        def arrive_and_prepare():
            with ThreadPoolExecutor(self.prep_workers) as ex:
                futs = []
                for r in sorted(requests, key=lambda q: q.arrival):
                    if realtime:
                        wait = r.arrival * time_scale - (time.perf_counter() - t0)
                        if wait > 0:
                            time.sleep(wait)
                    futs.append(ex.submit(_Prepared, r, self.tuner))
                    futs[-1].add_done_callback(lambda f: prepared.put(f))
                for f in futs:
                    f.exception()
            done_prep.set()

        feeder = threading.Thread(target=arrive_and_prepare, daemon=True)
        feeder.start()
        work = queue.Queue()
        slot_sem = threading.Semaphore(self.slots)
        mem_cv = threading.Condition(self._lock)
        inflight_max = [0]
        inflight = [0]

        def arrival_of(req):
            return t0 + req.arrival * time_scale if realtime else t0

        def worker():
            while True:
                item = work.get()
                if item is None:
                    return
                p = item
                try:
                    ts = time.perf_counter()
                    xh, info = self._solve(p)
                    te = time.perf_counter()
                    res = DrivenResult(p.req.rid, "ok" if info["converged"] else "not_converged",
                                       p.V.n, info["residual"], info["iterations"],
                                       te - arrival_of(p.req), te - ts, xh if self.keep else None)
                except Exception as exc:  # report and keep serving
                    res = DrivenResult(p.req.rid, "error: %s" % exc, p.V.n)
                finally:
                    with mem_cv:
                        self._reserved -= p.bytes
                        inflight[0] -= 1
                        mem_cv.notify_all()
                    slot_sem.release()
                    p.lu = None
                results[p.req.rid] = res

        threads = [threading.Thread(target=worker, daemon=True) for _ in range(self.slots)]
        for t in threads:
            t.start()
        pending = []
        n_total = len(requests)
        n_seen = 0
        prep_errors = []
        while n_seen < n_total:
            fut = prepared.get()
            n_seen += 1
            exc = fut.exception()
            if exc is not None:
                prep_errors.append("preparation: %s" % exc)
                continue
            p = fut.result()
            if p.bytes > self.budget:
                results[p.req.rid] = DrivenResult(p.req.rid, "rejected: needs %.1f GB > budget %.1f GB"
                                                  % (p.bytes / 1e9, self.budget / 1e9), p.V.n)
                continue
            slot_sem.acquire()
            with mem_cv:
                while self._reserved + p.bytes > self.budget:
                    mem_cv.wait()
                self._reserved += p.bytes
                inflight[0] += 1
                inflight_max[0] = max(inflight_max[0], inflight[0])
            work.put(p)
        for _ in threads:
            work.put(None)
        for t in threads:
            t.join()
        wall = time.perf_counter() - t0
        ok = [r for r in results.values() if r.status == "ok"]
        lat = sorted(r.latency for r in ok)
        self.stats = {
            "requests": n_total, "completed": len(ok),
            "rejected": sum(1 for r in results.values() if r.status.startswith("rejected")),
            "wall_s": wall, "solves_per_s": len(ok) / wall if wall > 0 else 0.0,
            "p50_ms": 1e3 * lat[len(lat) // 2] if lat else None,
            "p99_ms": 1e3 * lat[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)] if lat else None,
            "max_inflight": inflight_max[0], "budget_bytes": self.budget,
            "not_converged": sum(1 for r in results.values() if r.status == "not_converged"),
            "errors": sum(1 for r in results.values() if r.status.startswith("error")) + len(prep_errors),
            "error_sample": ([r.status for r in results.values() if r.status.startswith("error")]
                             + prep_errors)[:3],
        }
        return [results[r.rid] for r in requests if r.rid in results]
