"""Benchmark of the GB300 N1curl system-matrix + solve path.

Workload (one "step"): the driven ABC box of 1 m with 20x20x20 cubes x 6
tets (48,000 tets), N1curl order 2, eps_r ~ U[1,4) per cell (seeded),
k0 = 2*pi/0.4 m: assembly of A = S - k0^2 T + j k0 B on the CSR pattern
(n = 316,120, nnz = 13,419,440).  Inputs are synthetic (no dataset exists
for this path).  L2 is flushed (512 MB write) before every timed step.

Prints one JSON line (see the key list in main()).  --impl reference runs
the CPU restatement of the reference's assembly (the oracle port) on a
bounded sample of the same workload.
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


def workload():
    from sucemfem.mesh import BoxMesh
    mesh = BoxMesh(1.0, 1.0, 1.0, N_CUBES, N_CUBES, N_CUBES)
    eps = np.random.default_rng(SEED).uniform(1.0, 4.0, mesh.num_cells())
    k0 = 2 * np.pi / WAVELENGTH
    return mesh, eps, k0


def config_dict(extra=None):
    d = {"workload": "driven ABC box 1 m, 20^3 cubes x 6 tets (48,000 tets), N1curl order 2, "
                     "eps_r~U[1,4) seed 0, k0=2pi/0.4; assemble A=S-k0^2T+jk0B (complex64)",
         "tets": 6 * N_CUBES ** 3, "order": ORDER, "l2": "flushed (512 MB write) before each step"}
    if extra:
        d.update(extra)
    return d


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    def __init__(self):
        self.samples = []
        self._stop = threading.Event()
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
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
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
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernel):
    """DRAM bytes per launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get(kernel)
    return None


def algorithmic_bytes(V):
    """Minimum HBM bytes of one fused complex64 assembly launch: read cell
    connectivity (16 B/tet), eps_r (4 B/tet) and FP32 coordinates (12 B per
    vertex); write every CSR value once (8 B complex64)."""
    return V.nt * 16 + V.nt * 4 + V.nv * 12 + V.nnz * 8


def run_gpu(args):
    import torch
    from sucemfem import _device
    from sucemfem._native import call, ptr
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

    mesh, eps, k0 = workload()
    V = FunctionSpace(mesh, order=ORDER)
    h = V.upload()
    d_eps = torch.as_tensor(eps, dtype=torch.float32, device=dev)
    A = torch.empty(V.nnz, dtype=torch.complex64, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def step():
        call("sucem_assemble_helmholtz", h, 4, ptr(d_eps), None, float(k0), ptr(A), sp)

    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler()
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    per = [a.elapsed_time(b) for a, b in ev]  # ms
    total_ms = sum(per)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    clk = clocks.stop()

    # e2e through the host-buffer C-ABI: eps in, A back to pinned host memory
    eps_h = torch.as_tensor(eps, dtype=torch.float32).pin_memory()
    A_h = torch.empty(V.nnz, dtype=torch.complex64).pin_memory()
    d_eps2 = torch.empty_like(d_eps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        d_eps2.copy_(eps_h, non_blocking=True)
        call("sucem_assemble_helmholtz", h, 4, ptr(d_eps2), None, float(k0), ptr(A), sp)
        A_h.copy_(A, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps

    mean_ms = total_ms / args.steps
    elems = V.nt * world
    value = elems / (mean_ms * 1e-3)
    peak, peak_kind = measured_peaks()
    ab = algorithmic_bytes(V)
    achieved = ab / (statistics.mean(per) * 1e-3) / 1e9
    line = {
        "metric": "elems/s assembled (S-k0^2T+jk0B, order 2, FP32)",
        "value": value, "unit": "elems/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (complex64 output)",
        "data": "synthetic (seeded structured mesh, eps_r~U[1,4))",
        "config": config_dict({"parallelism": "replicas" if world > 1 else "single",
                               "n_dofs": V.n, "nnz": V.nnz}),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": profiled_traffic("assemble_rows_kernel<2,float,true,1>"),
                     "algorithmic_bytes_per_launch": ab,
                     "kernel": "assemble_rows_kernel<2,float,true,1>"},
        "e2e": {"value": V.nt / e2e_s, "unit": "elems/s",
                "h2d_bytes_per_step": int(eps_h.numel() * 4),
                "d2h_bytes_per_step": int(A_h.numel() * 8)},
        "gpu_launches": args.steps,
        "clocks": clk,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, sample_s=args.cpu_sample_s)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_baseline(args, sample_s=15.0):
    """Oracle (numpy FP64 restatement of the reference's assembly) on a
    bounded sample: the first cells of the same mesh, timed repeatedly."""
    from oracle import fem
    mesh, eps, k0 = workload()
    coords, cells = mesh.coordinates(), mesh.cells()
    ncell = 2000
    sub = cells[:ncell]
    t0 = time.perf_counter()
    reps = 0
    while True:
        A = fem.assemble(coords, sub, ORDER, eps_r=eps[:ncell])
        L = fem.lhs_matrix(A.S, A.T, A.B, k0 * C0 / (2 * np.pi))
        reps += 1
        if time.perf_counter() - t0 > sample_s:
            break
    dt = (time.perf_counter() - t0) / reps
    return {"value": ncell / dt, "unit": "elems/s", "cores": 1, "kind": "port",
            "sample": "oracle assembly + LHS combine of the first %d of 48,000 cells, %d reps"
                      % (ncell, reps)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(args, sample_s=0.5)
    for _ in range(args.steps):
        vals.append(cpu_baseline(args, sample_s=max(1.0, args.cpu_sample_s / max(args.steps, 1))))
    v = statistics.mean(x["value"] for x in vals)
    line = {"impl": "reference", "metric": "elems/s assembled (S-k0^2T+jk0B, order 2, FP32)",
            "value": v, "unit": "elems/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "dtype": "f64", "data": "synthetic", "config": config_dict(),
            "cpu_baseline": {"value": v, "unit": "elems/s", "cores": 1, "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": v, "unit": "elems/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample-s", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
