"""Benchmark of the GB300 N1curl system-matrix + solve path.

Workload (one "step" = one driven solve): the driven ABC box of 1 m with
20x20x20 cubes x 6 tets (48,000 tets), N1curl order 2 (n = 316,120,
nnz = 13,419,440), eps_r ~ U[1,4) per cell (seed 0), k0 = 2*pi/0.4 m,
unit z-directed dipole at the box centre; solve (S - k0^2 T + j k0 B) x = b
to 1e-10 relative residual.  Inputs are synthetic (no dataset exists for
this path); the LU arena (12.6 GB) and the matrices are far larger than L2.

FP32+IR step (the headline): FP64 assembly of A (the refinement matrix),
its rounding to complex64 as the LU input, complex64 multifrontal LU,
FGMRES in complex128 to the tolerance.  The plain FP64 path (complex128 LU)
is timed beside it.  The FP32 assembly kernel is timed on its own (L2
flushed before each launch) for its HBM roofline.

--impl reference: the reference's CPU path for this workload is the oracle
assembly (its forms restated in numpy) and a scipy direct solve (SuperLU in
place of the reference's UMFPACK).  The direct solve of this 20^3 order-2
system does not finish in bounded time on host cores (splu with the
MMD_AT_PLUS_A ordering ran out of a 30-minute limit; COLAMD likewise), and
the reference's default iterative route (BiCGStab + spilu(1e-8, 10)) fails
with an exactly singular factor.  The reference line therefore carries no
solves/s value, with that reason, and times the part of the path that does
finish on the same configuration: the assembly of S, T and B (elems/s).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "sucem-fem_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np

N_CUBES = 20
ORDER = 2
SEED = 0
WAVELENGTH = 0.4
C0 = 299792458.0
TOL = 1e-10
METRIC = "solves/s (driven ABC 20^3 order 2, 1e-10 rel. residual, FP32 LU + FP64 refinement)"


def workload(n_cubes=N_CUBES):
    from sucemfem.mesh import BoxMesh
    mesh = BoxMesh(1.0, 1.0, 1.0, n_cubes, n_cubes, n_cubes)
    eps = np.random.default_rng(SEED).uniform(1.0, 4.0, mesh.num_cells())
    k0 = 2 * np.pi / WAVELENGTH
    return mesh, eps, k0


def config_dict(extra=None):
    d = {"workload": "driven ABC box 1 m, 20^3 cubes x 6 tets (48,000 tets), N1curl order 2, "
                     "eps_r~U[1,4) seed 0, k0=2pi/0.4, z dipole at the centre; solve to 1e-10",
         "tets": 6 * N_CUBES ** 3, "order": ORDER, "tolerance": TOL,
         "l2": "inputs larger than L2 (LU arena 12.6 GB); assembly timed with a 512 MB flush"}
    if extra:
        d.update(extra)
    return d


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    def __init__(self):
        self.samples = []
        self._proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(int(os.environ.get("LOCAL_RANK", "0"))),
                 "--query-gpu=" + q, "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self._proc = None

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(s[0]) for s in self.samples if num(s[0]) is not None]
        mx = [num(s[1]) for s in self.samples if num(s[1]) is not None]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if s[3 + i].lower() in ("active", "1", "yes")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def profiled_traffic(kernel):
    """DRAM bytes per launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get(kernel)
    return None


REFERENCE_SOLVE_REASON = (
    "the reference's CPU solve of this 20^3 order-2 driven system (n=316,120, nnz=13.4M) does not "
    "finish in bounded time: scipy splu (the stand-in for the reference's UMFPACK route) with the "
    "MMD_AT_PLUS_A ordering ran out of a 1800 s limit (8 x86 host cores; SuperLU is single-threaded), "
    "COLAMD likewise, and the reference's default BiCGStab + spilu(drop 1e-8, fill 10) fails with an "
    "exactly singular factor")


def cpu_assembly_sample(n_cubes=N_CUBES):
    """The oracle (the reference's forms restated in numpy, FP64) assembling
    S, T and B of the full benchmark configuration once: elems/s."""
    from oracle import fem
    mesh, eps, _ = workload(n_cubes)
    coords, cells = mesh.coordinates(), mesh.cells()
    t0 = time.perf_counter()
    A = fem.assemble(coords, cells, ORDER, eps_r=eps)
    dt = time.perf_counter() - t0
    return len(cells) / dt, dt, A.n


def assembly_bytes(V):
    """Minimum HBM bytes of one fused complex64 assembly launch: read cell
    connectivity (16 B/tet), eps_r (4 B/tet) and FP32 coordinates (12 B per
    vertex); write every CSR value once (8 B complex64)."""
    return V.nt * 16 + V.nt * 4 + V.nv * 12 + V.nnz * 8


def percentile(v, q):
    v = sorted(v)
    if not v:
        return None
    k = (len(v) - 1) * q / 100.0
    lo, hi = int(np.floor(k)), int(np.ceil(k))
    return v[lo] + (v[hi] - v[lo]) * (k - lo)


def replica_rate(total_ms, steps, device=None):
    """Whole-job rate of independent replicas (one per rank): the timed
    total of every rank, the maximum over ranks (the slowest replica bounds
    the job) and world_size problems per step of that length.  Returns
    (solves/s, max total ms).  Without an initialised process group: one
    replica."""
    import torch
    world = 1
    if torch.distributed.is_available() and torch.distributed.is_initialized():
        world = torch.distributed.get_world_size()
        t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    return world / (total_ms / steps * 1e-3), total_ms


def run_gpu(args):
    import torch
    from sucemfem import _device, _native
    from sucemfem._native import call, ptr
    from sucemfem.Sources.point_source import evaluate_point_sources
    from sucemfem.solvers import DeviceCSR, RefinedDirectSolver, lu_for_space
    from sucemfem.space import FunctionSpace

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    _device.set_device(local)
    dev = _device.device()
    lib = _native.lib()

    mesh, eps, k0 = workload()
    V = FunctionSpace(mesh, order=ORDER)
    h = V.upload()
    lu = lu_for_space(V)
    from sucemfem import autotune
    tuner = autotune.Autotuner()
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    d_eps32 = torch.as_tensor(eps, dtype=torch.float32, device=dev)
    d_eps64 = torch.as_tensor(eps, dtype=torch.float64, device=dev)
    A32 = torch.empty(V.nnz, dtype=torch.complex64, device=dev)
    A64 = torch.empty(V.nnz, dtype=torch.complex128, device=dev)
    indptr = torch.as_tensor(V.indptr.astype(np.int32), device=dev)
    indices = torch.as_tensor(V.indices, device=dev)
    Acsr = DeviceCSR(indptr, indices, A64, V.n)
    Z0 = 4e-7 * np.pi * C0
    _, dofs, con = evaluate_point_sources(V, np.array([[0.5, 0.5, 0.5]]), np.array([[0, 0, 1.0]]))
    b_h = np.zeros(V.n, dtype=np.complex128)
    b_h[dofs[0]] += -1j * k0 * Z0 * con[0]
    b = torch.as_tensor(b_h, device=dev)

    def solve_step(precision, b_dev, ev=None):
        call("sucem_assemble_helmholtz", h, 8, ptr(d_eps64), None, float(k0), ptr(A64), sp)
        rs = RefinedDirectSolver(Acsr, lu)
        if ev is not None:
            ev[0].record(stream)
        if precision == "fp64":
            rs.factor(A64, "c128")
        else:
            # the LU input: the FP64 matrix rounded to complex64 (the
            # refinement needs the FP64 matrix anyway; the FP32 assembly's
            # matrix, timed below on its own, costs one more iteration)
            rs.vec.convert(A64, A32)
            rs.factor(A32, "c64")
        if ev is not None:
            ev[1].record(stream)
        x, info = rs.solve(b_dev, tol=TOL, method="gmres", maxit=30)
        return x, info

    def timed(precision, steps, warmup):
        for _ in range(warmup):
            solve_step(precision, b)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        lat, fac, infos = [], [], []
        l0 = lib.sucem_launch_count()
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            x, info = solve_step(precision, b, (f0, f1))
            e1.record(stream)
            torch.cuda.synchronize()
            lat.append(e0.elapsed_time(e1))
            fac.append(f0.elapsed_time(f1))
            infos.append(info)
        launches = lib.sucem_launch_count() - l0
        return lat, fac, infos, launches, x

    # LU plan (super-panel width, tensor-core panel threshold) from the
    # autotuner: cached per device and size class, else timed trials now,
    # before the timed region
    call("sucem_assemble_helmholtz", h, 4, ptr(d_eps32), None, float(k0), ptr(A32), sp)
    trials0 = tuner.trials
    if args.lu_plan:
        # a fixed plan (profiling runs: no autotuning trials before the steps)
        plan = tuple(int(v) for v in args.lu_plan.split(","))
        lu.configure(*plan)
    else:
        plan = autotune.tune_lu(lu, A32, "c64", tuner)
    clocks = ClockSampler()
    clocks.start()
    time.sleep(0.3)
    lat32, fac32, inf32, launches32, x32 = timed("fp32-ir", args.steps, args.warmup)
    clk = clocks.stop()
    # the dominant kernel (tensor-core Schur updates) of the last timed
    # factorisation: CUDA events recorded around its launches on the stream
    tc = lu.kernel_stats()
    value, total_ms = replica_rate(sum(lat32), args.steps, dev)

    # e2e: host b in (pinned), x back to host, through the same public
    # calls; measured right after the device-timed steps (same warm state:
    # the FP64 path below re-plans the factor's device buffers), after one
    # untimed warm-up iteration of its own
    b_pin = torch.as_tensor(b_h).pin_memory()
    x_pin = torch.empty(V.n, dtype=torch.complex128).pin_memory()
    e2e = []
    if world > 1:
        torch.distributed.barrier()
    for it in range(1 + max(2, min(args.steps, 5))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        bd = b_pin.to(dev, non_blocking=True)
        x, _ = solve_step("fp32-ir", bd)
        x_pin.copy_(x, non_blocking=True)
        torch.cuda.synchronize()
        if it > 0:
            e2e.append(time.perf_counter() - t0)
    n64 = max(1, args.fp64_steps)
    lat64, fac64, inf64, _, x64 = timed("fp64", n64, 1)

    # assembly kernel alone (HBM roofline), L2 flushed before each launch
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    asm = []
    for i in range(args.asm_reps + 3):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call("sucem_assemble_helmholtz", h, 4, ptr(d_eps32), None, float(k0), ptr(A32), sp)
        e1.record(stream)
        torch.cuda.synchronize()
        if i >= 3:
            asm.append(e0.elapsed_time(e1))
    del flush


    hbm, bf16, peak_kind = measured_peaks()
    mean_ms = total_ms / args.steps
    e2e_value, _ = replica_rate(1e3 * sum(e2e), len(e2e), dev)
    lu_flops = lu.info["flops"] * 8.0  # complex multiply-add = 8 real flops
    fac_ms = statistics.mean(fac32)
    fac_tflops = lu_flops / (fac_ms * 1e-3) / 1e12
    tc_tflops = tc["flops"] / (tc["ms"] * 1e-3) / 1e12 if tc["ms"] > 0 else 0.0
    tc_flops_launch = tc["flops"] / max(1, tc["launches"])
    # DRAM bytes of all tensor-core launches of one factorisation (ncu)
    # (the events around each tensor-core launch also cover its operand
    # pre-split kernel, so both kernels' bytes count)
    tc_bytes = [profiled_traffic("tc_update_kernel_per_factorisation"),
                profiled_traffic("tc_presplit_kernel_per_factorisation")]
    tc_traffic = sum(tc_bytes) / max(1, tc["launches"]) if all(tc_bytes) else None
    asm_ms = statistics.mean(asm)
    asm_gbs = assembly_bytes(V) / (asm_ms * 1e-3) / 1e9
    rel_diff = float(torch.linalg.norm(x32 - x64) / torch.linalg.norm(x64))
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 LU / c128 refinement", "data": "synthetic (seeded structured mesh)",
        "config": config_dict({"parallelism": "replicas" if world > 1 else "single",
                               "n_dofs": V.n, "nnz": V.nnz, "lu_fronts": lu.info["nodes"],
                               "lu_levels": lu.info["levels"],
                               "lu_largest_front": lu.info["max_front"]}),
        "latency_ms": {"p50": percentile(lat32, 50), "p99": percentile(lat32, 99)},
        "refinement": {"iterations": [i["iterations"] for i in inf32],
                       "residual": max(i["residual"] for i in inf32),
                       "converged": all(i["converged"] for i in inf32),
                       "perturbed_pivots": int(lu.perturbed())},
        "fp64_path": {"solves_per_s": 1e3 / statistics.mean(lat64),
                      "ms_per_solve": statistics.mean(lat64),
                      "factor_ms": statistics.mean(fac64),
                      "residual": max(i["residual"] for i in inf64),
                      "steps": n64},
        "speedup_fp32ir_vs_fp64": statistics.mean(lat64) / statistics.mean(lat32),
        "solution_rel_diff_fp32ir_vs_fp64": rel_diff,
        "factor_ms": fac_ms,
        "roofline": {"bound": "tensor", "achieved": tc_tflops, "peak": bf16, "unit": "TFLOP/s",
                     "frac": tc_tflops / bf16, "peak_source": peak_kind + " (bf16 tensor)",
                     "traffic": tc_traffic,
                     "kernel": "tc_update_kernel (complex64 Schur updates, tcgen05 kind::tf32, "
                               "3xTF32 split) with its tc_presplit_kernel (operand TF32 hi/lo "
                               "chunk images, read by bulk async copies)",
                     "launches_per_factor": tc["launches"],
                     "ms_per_factor": tc["ms"],
                     "algorithmic_flops_per_launch": tc_flops_launch,
                     "ceiling_3xtf32": bf16 / 2 / 3,
                     "frac_of_3xtf32_ceiling": tc_tflops / (bf16 / 2 / 3),
                     "note": "achieved = algorithmic complex flops (8 per multiply-add) / event time; "
                             "the tensor cores execute 3x that in TF32 (half the bf16 rate)"},
        "lu_factor": {"ms": fac_ms, "tflops": fac_tflops, "algorithmic_flops": lu_flops},
        "assembly": {"elems_per_s": V.nt / (asm_ms * 1e-3), "ms": asm_ms,
                     "roofline": {"bound": "hbm", "achieved": asm_gbs, "peak": hbm,
                                  "unit": "GB/s", "frac": asm_gbs / hbm,
                                  "peak_source": peak_kind,
                                  "traffic": profiled_traffic("assemble_entities_kernel<2,float,1,1>"),
                                  "algorithmic_bytes_per_launch": assembly_bytes(V),
                                  "kernel": "assemble_entities_kernel<2,float,1,1> + "
                                            "cell_geometry_kernel"}},
        "e2e": {"value": e2e_value, "unit": "solves/s",
                "h2d_bytes_per_step": int(V.n * 16), "d2h_bytes_per_step": int(V.n * 16)},
        "gpu_launches": int(launches32),
        "clocks": clk,
        "lu_plan": {"superpanel": int(plan[0]), "panel_min_k": int(plan[1]),
                    "autotune_trials_this_run": tuner.trials - trials0,
                    "note": ("given by --lu-plan" if args.lu_plan else
                             "chosen by sucemfem.autotune from timed factorisations (cached per "
                             "device and size class)")},
    }
    if not args.no_secondary and world == 1:
        # the batched-eigen and serving configurations, each with its own
        # clock record (after the headline's timed region); the headline's
        # factor (its last factorisation was the FP64 one, 25 GB) and
        # matrices are released first, so the server's HBM budget sees the
        # whole device
        import gc
        del lu, Acsr, A32, A64, x32, x64
        gc.collect()
        torch.cuda.empty_cache()
        line["eigen_batch"] = measure_eigen_batch(args.cavities, with_oracle=True)
        torch.cuda.empty_cache()
        line["serve"] = measure_serve(args, tuner)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline():
    """The reference's CPU path on the benchmark configuration, as far as it
    finishes: the FP64 oracle assembly of the 20^3 order-2 S, T, B (one
    pass, ~15-30 s on one host core).  Its unit is the assembly half of the
    metric (elems/s); the solve half has no CPU value (see
    REFERENCE_SOLVE_REASON)."""
    rate, dt, n = cpu_assembly_sample()
    return {"value": rate, "unit": "elems/s", "cores": 1, "kind": "port",
            "sample": "FP64 oracle assembly (numpy restatement of the reference's forms) of S, T "
                      "and B of the full 20^3 order-2 configuration (48,000 tets, n=%d), one pass "
                      "of %.1f s" % (n, dt),
            "solve": {"value": None, "unit": "solves/s", "reason": REFERENCE_SOLVE_REASON}}


def run_reference(args):
    """The reference arm: no solves/s value on this configuration (the CPU
    solve does not finish, REFERENCE_SOLVE_REASON); the assembly part of
    the path timed on the same configuration.  Rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    base = cpu_baseline()
    line = {"impl": "reference", "metric": METRIC, "value": None, "unit": "solves/s",
            "reason": REFERENCE_SOLVE_REASON,
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": 1, "warmup": 0,
            "higher_is_better": True, "dtype": "c128", "data": "synthetic",
            "config": config_dict({"n_dofs": 316120, "nnz": 13419440, "cubes": N_CUBES}),
            "cpu_baseline": base,
            "assembly": {"elems_per_s": base["value"], "unit": "elems/s"},
            "e2e": {"value": None, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_kernel_case(args):
    """Small single-kernel cases for profiling (no JSON contract): 'factor'
    runs warmup+steps complex64 LU factorisations of the driven matrix,
    'lu-solve' one factorisation then warmup+steps LU solves (the
    preconditioner application of every FGMRES iteration; device-timed
    mean reported), 'assemble' the fused FP32 assembly, at --cubes^3 and
    --order."""
    import torch
    from sucemfem import _device
    from sucemfem._native import call, ptr
    from sucemfem.solvers import lu_for_space
    from sucemfem.space import FunctionSpace
    dev = _device.device()
    mesh, eps, k0 = workload(args.cubes)
    V = FunctionSpace(mesh, order=args.order)
    h = V.upload()
    d_eps = torch.as_tensor(eps, dtype=torch.float32, device=dev)
    A = torch.empty(V.nnz, dtype=torch.complex64, device=dev)
    sp = _device.stream_ptr()
    lu = lu_for_space(V) if args.only in ("factor", "lu-solve") else None
    out = {"case": args.only, "cubes": args.cubes, "order": args.order, "n": V.n, "nnz": V.nnz,
           "runs": args.warmup + args.steps}
    if args.only == "lu-solve":
        call("sucem_assemble_helmholtz", h, 4, ptr(d_eps), None, float(k0), ptr(A), sp)
        lu.factor(A, "c64")
        g = torch.Generator(device="cpu").manual_seed(0)
        b = torch.complex(torch.randn(V.n, generator=g, dtype=torch.float64),
                          torch.randn(V.n, generator=g, dtype=torch.float64)).to(dev)
        x = torch.empty_like(b)
        for _ in range(args.warmup):
            lu.solve(b, x)
        stream = torch.cuda.current_stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            lu.solve(b, x)
        e1.record(stream)
        torch.cuda.synchronize()
        out["ms_per_solve"] = e0.elapsed_time(e1) / max(1, args.steps)
    else:
        for _ in range(args.warmup + args.steps):
            call("sucem_assemble_helmholtz", h, 4, ptr(d_eps), None, float(k0), ptr(A), sp)
            if lu is not None:
                lu.factor(A, "c64")
        torch.cuda.synchronize()
    print(json.dumps(out))


def jittered_box(n, frac=0.2, seed=0):
    """Unit box of n^3 cubes x 6 tets with every interior vertex moved by
    U(-frac*h, frac*h) per coordinate (h = 1/n)."""
    from sucemfem.mesh import BoxMesh, Mesh
    m = BoxMesh(1.0, 1.0, 1.0, n, n, n)
    x = m.coordinates().copy()
    interior = np.all((x > 1e-12) & (x < 1 - 1e-12), axis=1)
    d = np.random.default_rng(seed).uniform(-frac / n, frac / n, size=x.shape)
    x[interior] += d[interior]
    return Mesh(x, m.cells())


def run_precision(args):
    """Large-mesh precision case: jittered 60^3 box (1,296,000 tets), orders 1
    and 2: per-entry FP32-vs-FP64 error of S, T, B; fused FP32 assembly
    throughput against the HBM roofline (outputs far larger than L2);
    order-1 FP32 LU + FP64 FGMRES solve to 1e-8; and, on the 40^3 order-1
    box, the FP32+refinement solution against the plain FP64 GPU solution."""
    import torch
    from sucemfem import _device
    from sucemfem._native import call, ptr
    from sucemfem.solvers import DrivenSolver
    from sucemfem.space import FunctionSpace
    dev = _device.device()
    hbm, _, peak_kind = measured_peaks()
    out = {"case": "precision", "cubes": args.cubes}
    mesh = jittered_box(args.cubes)
    eps = np.random.default_rng(1).uniform(1.0, 4.0, mesh.num_cells())
    k0 = 2 * np.pi / WAVELENGTH
    for order in (1, 2):
        V = FunctionSpace(mesh, order=order)
        h = V.upload()
        ip = torch.as_tensor(V.indptr, device=dev)
        rows = torch.repeat_interleave(torch.arange(V.n, device=dev), ip[1:] - ip[:-1])
        errs = {}
        for name in ("S", "T", "B"):
            v = {}
            for rb in (8, 4):
                dt = torch.float64 if rb == 8 else torch.float32
                bufs = {k: torch.empty(V.nnz, dtype=dt, device=dev) if k == name else None for k in "STB"}
                de = torch.as_tensor(eps, dtype=dt, device=dev)
                call("sucem_assemble", h, rb, ptr(de), None, ptr(bufs["S"]), ptr(bufs["T"]),
                     ptr(bufs["B"]), _device.stream_ptr())
                v[rb] = bufs[name].double()
                del bufs
            a = v[8].abs()
            rowmax = torch.zeros(V.n, dtype=torch.float64, device=dev).scatter_reduce(
                0, rows, a, reduce="amax")
            floor = (1.0 if name == "B" else 1e-6) * a.max()
            scale = torch.maximum(rowmax[rows], floor)
            e = (v[4] - v[8]).abs() / scale
            errs[name] = {"max": float(e.max()), "median": float(e.median())}
            del v, a, e, scale
        d_eps = torch.as_tensor(eps, dtype=torch.float32, device=dev)
        A = torch.empty(V.nnz, dtype=torch.complex64, device=dev)
        times = []
        for i in range(3 + 10):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            call("sucem_assemble_helmholtz", h, 4, ptr(d_eps), None, float(k0), ptr(A),
                 _device.stream_ptr())
            e1.record()
            torch.cuda.synchronize()
            if i >= 3:
                times.append(e0.elapsed_time(e1))
        ms = statistics.mean(times)
        gbs = assembly_bytes(V) / (ms * 1e-3) / 1e9
        out["order%d" % order] = {
            "n_dofs": V.n, "nnz": V.nnz, "fp32_vs_fp64_entry_error": errs,
            "assembly": {"ms": ms, "elems_per_s": V.nt / (ms * 1e-3), "achieved_gbs": gbs,
                         "frac_of_hbm": gbs / hbm, "peak_source": peak_kind}}
        del A, rows, ip
        if order == 1:
            from sucemfem.Sources.point_source import evaluate_point_sources
            Z0 = 4e-7 * np.pi * C0
            _, dofs, con = evaluate_point_sources(V, np.array([[0.5, 0.5, 0.5]]), np.array([[0, 0, 1.0]]))
            b = np.zeros(V.n, dtype=np.complex128)
            b[dofs[0]] += -1j * k0 * Z0 * con[0]
            ds = DrivenSolver(V, eps_r=eps)
            t0 = time.perf_counter()
            x, info = ds.solve(k0, b, precision="fp32-ir", tol=1e-8)
            torch.cuda.synchronize()
            out["order1"]["solve_fp32_ir"] = {"seconds": time.perf_counter() - t0,
                                              "iterations": info["iterations"],
                                              "residual": info["residual"],
                                              "lu_arena_gb": ds.lu.info["arena"] * 8 / 1e9,
                                              "lu_tflop": ds.lu.info["flops"] * 8 / 1e12}
            del ds, x
        del V
        torch.cuda.empty_cache()
    # solution error vs the FP64 GPU path on a size where the FP64 LU is cheap
    small = jittered_box(args.precision_solve_cubes)
    eps_s = np.random.default_rng(2).uniform(1.0, 4.0, small.num_cells())
    from sucemfem.Sources.point_source import evaluate_point_sources
    Vs = FunctionSpace(small, order=1)
    Z0 = 4e-7 * np.pi * C0
    _, dofs, con = evaluate_point_sources(Vs, np.array([[0.5, 0.5, 0.5]]), np.array([[0, 0, 1.0]]))
    b = np.zeros(Vs.n, dtype=np.complex128)
    b[dofs[0]] += -1j * k0 * Z0 * con[0]
    ds = DrivenSolver(Vs, eps_r=eps_s)
    x32, i32 = ds.solve(k0, b, precision="fp32-ir", tol=1e-8)
    x64, i64 = ds.solve(k0, b, precision="fp64", tol=1e-12)
    out["solution_vs_fp64"] = {"cubes": args.precision_solve_cubes, "order": 1, "n_dofs": Vs.n,
                               "rel_error": float(torch.linalg.norm(x32 - x64) / torch.linalg.norm(x64)),
                               "fp32_ir_residual": i32["residual"], "fp64_residual": i64["residual"],
                               "fp32_ir_s": i32["seconds"], "fp64_s": i64["seconds"]}
    del ds, x32, x64
    torch.cuda.empty_cache()

    # order 2.  The LU requirement of the 60^3 order-2 system from the
    # symbolic analysis (host only): far beyond the device, so the largest
    # jittered order-2 box whose complex64 LU fits is solved FP32+IR to 1e-8
    # instead, and FP32+IR is compared with the FP64 path where the complex128
    # LU fits too.
    from sucemfem.solvers import lu_for_space
    free_b, total_b = torch.cuda.mem_get_info()
    V60 = FunctionSpace(mesh, order=2)
    lu60 = lu_for_space(V60)
    out["order2_lu_requirement"] = {
        "cubes": args.cubes, "n_dofs": V60.n, "nnz": V60.nnz,
        "lu_arena_gb_c64": lu60.info["arena"] * 8 / 1e9, "lu_tflop": lu60.info["flops"] * 8 / 1e12,
        "largest_front": lu60.info["max_front"], "device_gb": total_b / 1e9,
        "fits": lu60.info["arena"] * 8 < free_b}
    del lu60, V60

    def order2_case(cubes, seed, precisions):
        m2 = jittered_box(cubes)
        e2 = np.random.default_rng(seed).uniform(1.0, 4.0, m2.num_cells())
        V2 = FunctionSpace(m2, order=2)
        _, dofs2, con2 = evaluate_point_sources(V2, np.array([[0.5, 0.5, 0.5]]), np.array([[0, 0, 1.0]]))
        b2 = np.zeros(V2.n, dtype=np.complex128)
        b2[dofs2[0]] += -1j * k0 * Z0 * con2[0]
        ds2 = DrivenSolver(V2, eps_r=e2)
        res = {"cubes": cubes, "order": 2, "n_dofs": V2.n, "nnz": V2.nnz,
               "lu_arena_gb_c64": ds2.lu.info["arena"] * 8 / 1e9,
               "lu_tflop": ds2.lu.info["flops"] * 8 / 1e12}
        xs = {}
        for prec, tol in precisions:
            x2, inf2 = ds2.solve(k0, b2, precision=prec, tol=tol)
            torch.cuda.synchronize()
            res[prec] = {"seconds": inf2["seconds"], "iterations": inf2["iterations"],
                         "residual": inf2["residual"], "tolerance": tol}
            xs[prec] = x2
        if len(xs) == 2:
            res["rel_error_fp32_ir_vs_fp64"] = float(torch.linalg.norm(xs["fp32-ir"] - xs["fp64"]) /
                                                     torch.linalg.norm(xs["fp64"]))
        del ds2, xs
        torch.cuda.empty_cache()
        return res

    out["order2_solve"] = order2_case(args.precision_solve2_cubes, 3, [("fp32-ir", 1e-8)])
    out["order2_solution_vs_fp64"] = order2_case(args.precision_fp64_cubes2, 4,
                                                 [("fp32-ir", 1e-8), ("fp64", 1e-12)])
    print(json.dumps(out))


def run_postproc(args):
    """Post-processing case on the --cubes^3 order --order box (default 20^3
    order 2): a seeded random complex field, then, device-timed with CUDA
    events after a warm-up, the surface power flux, the surface NTFF over
    360 directions in one launch pair, the variational NTFF over 36
    directions, the variational flux, the field at 100,000 points and the
    EM functional; beside them the FP64 oracle on a bounded sample (the
    same calls on the 6^3 box), timed on the host."""
    import torch
    from sucemfem import _device
    from sucemfem.PostProcessing import CalcEMFunctional, Reconstruct
    from sucemfem.PostProcessing.power_flux import SurfaceFlux, VariationalSurfaceFlux
    from sucemfem.PostProcessing.surface_ntff import NTFF
    from sucemfem.PostProcessing.variational_ntff import NTFF as VNTFF
    from sucemfem.space import FunctionSpace
    dev = _device.device()
    stream = torch.cuda.current_stream(dev)
    mesh, eps, k0 = workload(args.cubes)
    V = FunctionSpace(mesh, order=args.order)
    rng = np.random.default_rng(0)
    x = torch.as_tensor(rng.standard_normal(V.n) + 1j * rng.standard_normal(V.n), device=dev)
    freq = k0 * C0 / (2 * np.pi)
    th360 = np.linspace(0.5, 179.5, 360)
    ph360 = np.linspace(0.0, 359.0, 360)
    pts = rng.uniform(0.01, 0.99, (100000, 3))

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    sf = SurfaceFlux(V)
    sf.set_k0(k0)
    sf.set_dofs(x)
    vf = VariationalSurfaceFlux(V)
    vf.set_k0(k0)
    vf.set_dofs(x)
    nt = NTFF(V)
    nt.set_frequency(freq)
    nt.set_dofs(x)
    vn = VNTFF(V)
    vn.set_frequency(freq)
    vn.set_dofs(x)
    rc = Reconstruct(V)
    rc.set_dof_values(x)
    fu = CalcEMFunctional(V)
    fu.set_k0(k0)
    fu.set_E_dofs(x)
    fu.set_g_dofs(x)
    out = {"case": "postproc", "cubes": args.cubes, "order": args.order, "n_dofs": V.n,
           "tets": V.nt, "exterior_facets": V.n_ext_facets,
           "data": "synthetic (seeded random complex field)"}
    ms = timed(sf.calc_flux)
    out["surface_flux"] = {"ms": ms, "facets_per_s": V.n_ext_facets / (ms * 1e-3)}
    ms = timed(lambda: nt.calc_pts(th360, ph360))
    out["surface_ntff_360_directions"] = {"ms": ms, "directions_per_s": 360 / (ms * 1e-3)}
    ms = timed(lambda: vn.calc_pts(th360[::10], ph360[::10]), reps=1)
    out["variational_ntff_36_directions"] = {"ms": ms, "directions_per_s": 36 / (ms * 1e-3)}
    ms = timed(vf.calc_flux)
    out["variational_flux"] = {"ms": ms}
    ms = timed(lambda: rc.reconstruct_points(pts))
    out["reconstruct_100k_points"] = {"ms": ms, "points_per_s": 1e5 / (ms * 1e-3)}
    ms = timed(fu.calc_functional)
    out["em_functional"] = {"ms": ms, "tets_per_s": V.nt / (ms * 1e-3)}
    if not args.no_cpu_baseline:
        from oracle import fem as ofem, postproc as opp
        cm, _, _ = workload(6)
        A = ofem.assemble(cm.coordinates(), cm.cells(), args.order)
        xs = rng.standard_normal(A.n) + 1j * rng.standard_normal(A.n)
        t0 = time.perf_counter()
        opp.surface_flux(cm.coordinates(), cm.cells(), args.order, A.topo, A.dofmap, xs, k0)
        t1 = time.perf_counter()
        opp.ntff(cm.coordinates(), cm.cells(), args.order, A.topo, A.dofmap, xs, freq,
                 th360[:36], ph360[:36])
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"kind": "port", "cores": 1,
                               "sample": "FP64 oracle on the 6^3 box (%d tets)" % len(cm.cells()),
                               "surface_flux_s": t1 - t0, "surface_ntff_36_directions_s": t2 - t1}
    print(json.dumps(out))


def eigen_cavities(ncav, seed=0):
    """The batched-cavity configuration: ncav PEC boxes, sides U[0.3,1.5] m,
    divisions U{4..24} per axis, eps_r U[1,4] per cell (one stacked mesh,
    boxes side by side)."""
    from sucemfem.mesh import BoxMesh
    rng = np.random.default_rng(seed)
    boxes, coords, cells, seg_cells, off, x0 = [], [], [], [], 0, 0.0
    for k in range(ncav):
        L = rng.uniform(0.3, 1.5, 3)
        n = rng.integers(4, 25, 3)
        m = BoxMesh(L[0], L[1], L[2], int(n[0]), int(n[1]), int(n[2]), origin=(x0, 0.0, 0.0))
        x0 += L[0] + 0.5
        boxes.append((m.coordinates(), m.cells()))
        coords.append(m.coordinates())
        cells.append(m.cells() + off)
        off += len(m.coordinates())
        seg_cells.append(np.full(m.num_cells(), k))
    return boxes, np.concatenate(coords), np.concatenate(cells), np.concatenate(seg_cells), rng


def oracle_cavity_k2(coords, cells, eps, nev, sigma=1.0):
    """FP64 CPU oracle: the nev smallest k^2 above sigma of a PEC cavity
    (oracle assembly, PEC DOFs removed, scipy shift-invert eigsh)."""
    import scipy.sparse.linalg as spl
    from oracle import fem
    A = fem.assemble(coords, cells, 1, eps_r=eps, with_abc=False)
    pec = fem.pec_dofs(A.topo, 1)
    keep = np.setdiff1d(np.arange(A.n), pec)
    S = A.S[keep][:, keep].tocsc()
    T = A.T[keep][:, keep].tocsc()
    # shift-invert: 'LA' on nu = 1/(k^2 - sigma) picks the k^2 just above
    # sigma (the gradient null space, k^2 = 0, lies below it)
    w = spl.eigsh(S, M=T, k=nev, sigma=sigma, which="LA", return_eigenvectors=False)
    return np.sort(w)


def measure_eigen_batch(ncav, with_oracle=False, nev=6):
    """Batched cavities through one space, one assembly launch, one FP32 LU
    of the stacked problem and one batched shift-invert Lanczos for the nev
    smallest k^2 above sigma=1 of every cavity (FP64 Lanczos/RR), wall time
    from assembly to eigenvalues on the host; with_oracle: the largest
    relative k^2 error against the FP64 oracle on the three cavities with
    the fewest cells."""
    import torch
    from sucemfem import _device
    from sucemfem._native import call, ptr
    from sucemfem.eigen import BatchedShiftInvertLanczos
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    dev = _device.device()
    boxes, coords, cells, seg_cells, rng = eigen_cavities(ncav)
    t0 = time.perf_counter()
    V = FunctionSpace(Mesh(coords, cells), order=1)
    dof_seg = np.zeros(V.n, dtype=np.int64)
    dof_seg[V.cell_dofs.ravel()] = np.repeat(seg_cells, 6)
    eps = rng.uniform(1.0, 4.0, V.nt)
    t_host = time.perf_counter() - t0
    clocks = ClockSampler()
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    S = torch.empty(V.nnz, dtype=torch.float64, device=dev)
    T = torch.empty_like(S)
    d_eps = torch.as_tensor(eps, device=dev)
    call("sucem_assemble", V.upload(), 8, ptr(d_eps), None, ptr(S), ptr(T), None, _device.stream_ptr())
    sol = BatchedShiftInvertLanczos(V, S, T, V.boundary_dofs, 1.0, dof_segment=dof_seg)
    t2 = time.perf_counter()
    k2, _ = sol.solve(nev)
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    clk = clocks.stop()
    out = {"cavities": ncav, "tets": V.nt, "n_dofs": V.n, "nev": nev,
           "cavity_solves_per_s": ncav / (t3 - t1), "seconds": t3 - t1,
           "host_build_s": t_host, "setup_s": t2 - t1, "solve_s": t3 - t2,
           "lanczos_steps": sol.stats.get("m"), "lu_arena_gb": sol.lu.info["arena"] * 4 / 1e9,
           "precision": "FP32 LU (tensor-core updates) + FP64 Lanczos and Rayleigh-Ritz",
           "clocks": clk}
    if with_oracle:
        sizes = [len(c) for _, c in boxes]
        order = np.argsort(sizes)[:3]
        starts = np.concatenate([[0], np.cumsum(sizes)])
        errs = []
        for k in order:
            bc, bcells = boxes[k]
            ek = eps[starts[k]:starts[k + 1]]
            ref = oracle_cavity_k2(bc, bcells, ek, nev)
            got = np.sort(k2[k])[:len(ref)]
            errs.append(float(np.max(np.abs(got - ref) / ref)))
        out["max_rel_k2_error_vs_oracle"] = max(errs)
        out["oracle_cavities"] = [int(k) for k in order]
    return out


def run_eigen_batch(args):
    print(json.dumps(dict(case="eigen-batch", **measure_eigen_batch(args.cavities,
                                                                     with_oracle=True))))


def measure_serve(args, tuner=None):
    """The serving configuration: a Poisson stream (mean args.serve_rate per
    second) of driven ABC-box solves, divisions log-uniform in [6,
    args.serve_max_cubes], order 1 or 2 at 50/50, k0 so that the box spans
    1-6 wavelengths, complex64 LU + FP64 refinement to 1e-8, through the
    continuous-batching server with HBM-budget admission (slot count from
    the autotuner); the first args.serve_requests requests of the stream;
    beside it the same kind of requests one at a time on the plain FP64
    path (a sample)."""
    from sucemfem import autotune
    from sucemfem.serving import SolveServer, make_request_stream
    tuner = tuner or autotune.Autotuner()
    reqs = make_request_stream(args.serve_requests, args.serve_rate,
                               cubes=(6, args.serve_max_cubes), seed=0)
    # slot count: timed trials on a small fixed sample of the stream's kind
    # (divisions 6-16), cached per device
    sample = make_request_stream(12, 1000.0, cubes=(6, 16), seed=1)

    def run_sample(slots):
        t0 = time.perf_counter()
        SolveServer(slots=slots, tol=1e-8).run(sample, realtime=False)
        return time.perf_counter() - t0
    trials0 = tuner.trials
    slots = autotune.tune_slots(run_sample, tuner, key="serve_driven_abc")
    clocks = ClockSampler()
    clocks.start()
    srv = SolveServer(slots=slots, tol=1e-8, tuner=tuner)
    res = srv.run(reqs, realtime=True)
    clk = clocks.stop()
    n64 = min(len(reqs), args.serve_fp64_sample)
    one = SolveServer(slots=1, precision="fp64", tol=1e-8)
    one.run(reqs[:n64], realtime=False)
    ok = [r for r in res if r.status == "ok"]
    return {"requests": len(reqs), "rate_per_s": args.serve_rate,
            "stream": "first %d requests of the seeded Poisson stream (%.1f s of arrivals)"
                      % (len(reqs), reqs[-1].arrival if reqs else 0.0),
            "cubes": [6, args.serve_max_cubes], "orders": [1, 2], "wavelengths": [1, 6],
            "slots": slots, "slot_trials_this_run": tuner.trials - trials0,
            "solves_per_s": srv.stats["solves_per_s"], "p50_ms": srv.stats["p50_ms"],
            "p99_ms": srv.stats["p99_ms"], "completed": srv.stats["completed"],
            "rejected": srv.stats["rejected"], "not_converged": srv.stats["not_converged"],
            "errors": srv.stats["errors"], "error_sample": srv.stats["error_sample"],
            "max_inflight": srv.stats["max_inflight"],
            "max_residual": max(r.residual for r in ok) if ok else None,
            "fp64_one_at_a_time": {"requests": n64, "solves_per_s": one.stats["solves_per_s"],
                                   "p50_ms": one.stats["p50_ms"]},
            "clocks": clk}


def run_serve(args):
    print(json.dumps(dict(case="serve", **measure_serve(args))))


def run_high_order(args):
    """N1curl orders 3 and 4: the entry-gather assembly of S, T and B on a
    20^3 (order 3) and 16^3 (order 4) box with eps_r ~ U[1,4), FP32 and
    FP64, device-timed after a warm-up (outputs far larger than L2), against
    the HBM roofline of its algorithmic bytes (every value of S, T, B
    written once and the per-entry gather lists read once); then the
    reference's two higher-order cavity cases (order 3 on the 4^3 unit cube,
    order 4 on a 1 x 0.5 x 0.25 prism of 8 x 4 x 2 cubes), ten modes above
    sigma = 1.1 each, wall-timed solve_problem after a warm-up solve, with
    the largest relative error of k/pi against the analytic wavenumbers."""
    import torch
    from sucemfem import _device
    from sucemfem._native import call, ptr
    from sucemfem.BoundaryConditions import PECWallsBoundaryCondition
    from sucemfem.mesh import BoxMesh
    from sucemfem.ProblemConfigurations.EMVectorWaveEigenproblem import DefaultEigenSolver, EigenProblem
    from sucemfem.space import FunctionSpace
    dev = _device.device()
    stream = torch.cuda.current_stream(dev)
    hbm, _, peak_kind = measured_peaks()
    out = {"case": "high-order", "data": "synthetic (structured boxes, seeded eps_r)", "assembly": [],
           "cavities": []}
    for order, nc in ((3, 20), (4, 16)):
        V = FunctionSpace(BoxMesh(1.0, 1.0, 1.0, nc, nc, nc), order=order)
        h = V.upload()
        eps = np.random.default_rng(0).uniform(1, 4, V.nt)
        nd = V.ndof_cell
        for rb, dt in ((4, torch.float32), (8, torch.float64)):
            S, T, B = (torch.empty(V.nnz, dtype=dt, device=dev) for _ in range(3))
            d_eps = torch.as_tensor(eps, dtype=dt, device=dev)

            def go():
                call("sucem_assemble", h, rb, ptr(d_eps), None, ptr(S), ptr(T), ptr(B),
                     _device.stream_ptr())
            for _ in range(3):
                go()
            torch.cuda.synchronize()
            reps = 10
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(reps):
                go()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            alg = 3 * V.nnz * rb + V.nt * nd * nd * 4 + (2 * V.nnz + 1) * 4 + V.nt * (16 + rb)
            gbs = alg / (ms * 1e-3) / 1e9
            out["assembly"].append({
                "order": order, "cubes": nc, "tets": V.nt, "n_dofs": V.n, "nnz": V.nnz,
                "real_bytes": rb, "ms": ms, "tets_per_s": V.nt / (ms * 1e-3),
                "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                             "frac": gbs / hbm, "peak_source": peak_kind,
                             "algorithmic_bytes": alg}})
            del S, T, B
    for order, dims, mesh in ((3, (1.0, 1.0, 1.0), BoxMesh(1.0, 1.0, 1.0, 4, 4, 4)),
                              (4, (1.0, 0.5, 0.25), BoxMesh(1.0, 0.5, 0.25, 8, 4, 2))):
        pec = PECWallsBoundaryCondition()
        pec.init_with_mesh(mesh)
        ep = EigenProblem()
        ep.set_mesh(mesh)
        ep.set_basis_order(order)
        ep.set_boundary_conditions(pec)
        ep.init_problem()
        es = DefaultEigenSolver()
        es.set_eigenproblem(ep)
        es.set_sigma(1.1)
        es.solve_problem(10)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w, _ = es.solve_problem(10)
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        k = np.sort(np.sqrt(1.0 / w.real + 1.1) / np.pi)
        a, b, d = dims
        ana = []
        for m in range(6):
            for n in range(6):
                for l in range(6):
                    i = (m, n, l)
                    kk = np.sqrt((m / a) ** 2 + (n / b) ** 2 + (l / d) ** 2)
                    if i.count(0) < 2:
                        ana.append(kk)
                    if i.count(0) == 0:
                        ana.append(kk)
        ana = np.sort(ana)[:10]
        out["cavities"].append({"order": order, "box": dims, "n_dofs": ep.get_global_dimension(),
                                "seconds": sec, "max_rel_err_k": float(np.max(np.abs(k - ana) / ana))})
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default="solve",
                    choices=["solve", "factor", "lu-solve", "assemble", "serve", "precision",
                             "eigen-batch", "postproc", "high-order"],
                    help="profiling cases: factor / assemble at --cubes, --order; serve; precision")
    ap.add_argument("--precision-solve-cubes", type=int, default=30)
    ap.add_argument("--precision-solve2-cubes", type=int, default=40,
                    help="jittered order-2 box solved FP32+IR in --only precision")
    ap.add_argument("--precision-fp64-cubes2", type=int, default=24,
                    help="jittered order-2 box where FP32+IR is compared with the FP64 path")
    ap.add_argument("--cavities", type=int, default=256)
    ap.add_argument("--serve-requests", type=int, default=300)
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-max-cubes", type=int, default=48)
    ap.add_argument("--serve-fp64-sample", type=int, default=10)
    ap.add_argument("--no-secondary", action="store_true",
                    help="headline solve only (no batched-eigen and serving keys)")
    ap.add_argument("--cubes", type=int, default=N_CUBES)
    ap.add_argument("--order", type=int, default=ORDER)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--asm-reps", type=int, default=50)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lu-plan", default="",
                    help="SUPERPANEL,PANEL_MIN_K: a fixed LU plan instead of the autotuner's")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.only == "serve":
        run_serve(args)
    elif args.only == "precision":
        run_precision(args)
    elif args.only == "eigen-batch":
        run_eigen_batch(args)
    elif args.only == "postproc":
        run_postproc(args)
    elif args.only == "high-order":
        run_high_order(args)
    elif args.only != "solve":
        run_kernel_case(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
