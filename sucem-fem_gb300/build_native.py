"""Build libsucem_gb300.so in-tree with nvcc for sm_103a.

Compiles every translation unit in parallel (one -gencode, no cmake) and
links a shared library next to this file: sucem-fem_gb300/libsucem_gb300.so.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "libsucem_gb300.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")

CU = ["abi.cu", "assemble.cu", "linalg.cu"]
CPP = ["space.cpp", "schedule.cpp", "mf_symbolic.cpp"]


def _sources():
    srcs = [os.path.join(CSRC, f) for f in CU + CPP]
    extra = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu") and f not in CU)
    return srcs + [os.path.join(CSRC, f) for f in extra]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    tables = os.path.join(CSRC, "n1curl_tables.h")
    tables_hi = os.path.join(CSRC, "n1curl_tables_hi.h")
    contract = os.path.join(CSRC, "n1curl_contract.h")
    if not all(os.path.exists(p) for p in (tables, tables_hi, contract)):
        _run([sys.executable, os.path.join(CSRC, "gen_tables.py"), tables, tables_hi, contract])
    srcs = _sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "sucem_gb300.h"))
    newest_dep = max(os.path.getmtime(p) for p in srcs + headers)
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= newest_dep:
        return OUT
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp",
              "-I", os.path.join(ROOT, "include")]
    jobs = []
    objs = []
    for s in srcs:
        obj = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(obj)
        if s.endswith(".cu"):
            cmd = [NVCC] + ARCH + common + ["-lineinfo", "-c", s, "-o", obj]
        else:
            cmd = [NVCC] + common + ["-x", "cu", "-c", s, "-o", obj] + ARCH
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    tmp = OUT + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", tmp] + objs)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
