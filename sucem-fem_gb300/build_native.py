"""Build libsucem_gb300.so in-tree with nvcc for sm_103a.

Compiles every translation unit in parallel (one -gencode, no cmake) and
links a shared library next to this file: sucem-fem_gb300/libsucem_gb300.so.
"""
import concurrent.futures as cf
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "libsucem_gb300.so")
# objects per host architecture: a tree copied to another machine never links them
BUILD = os.path.join(HERE, "_build", platform.machine() or "host")
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


def _local_deps(path, seen=None):
    """The file and the local headers it includes (recursively)."""
    import re
    seen = set() if seen is None else seen
    if path in seen or not os.path.exists(path):
        return seen
    seen.add(path)
    with open(path, errors="replace") as f:
        for m in re.finditer(r'^\s*#\s*include\s+"([^"]+)"', f.read(), re.M):
            _local_deps(os.path.normpath(os.path.join(os.path.dirname(path), m.group(1))), seen)
    return seen


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
        if (not force and os.path.exists(obj) and
                os.path.getmtime(obj) >= max(os.path.getmtime(p) for p in _local_deps(s))):
            continue  # object newer than its source and the headers it includes
        if s.endswith(".cu"):
            cmd = [NVCC] + ARCH + common + ["-lineinfo", "-c", s, "-o", obj]
        else:
            cmd = [NVCC] + common + ["-x", "cu", "-c", s, "-o", obj] + ARCH
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, len(jobs)))) as ex:
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
