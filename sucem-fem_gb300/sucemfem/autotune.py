"""A small autotuner for the schedule choices of the GPU path.

It picks, per problem-size class and device, from timed trials:

* the super-panel width and the tensor-core panel threshold of the
  single-precision LU factorisation (``tune_lu``), the two choices that
  trade tensor-core work against re-reading the trailing blocks of the
  fronts;
* the number of concurrent solve slots of the serving loop
  (``tune_slots``), which trades overlap on the device against memory and
  host threads.

Choices are cached in a JSON file keyed by device name and a size class, so
a process (or a later one) reuses them without new trials.  The trial
function is a parameter: tests drive the cache logic with fake timings on
the CPU.  The reference has no counterpart (its solvers take fixed
parameters, sucemfem/Utilities/LinalgSolvers.py:107-127).
"""
import json
import math
import os
import threading
import time

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "sucem_gb300", "autotune.json")

# the candidates of the LU plan: (super-panel width, tensor-core panel threshold)
LU_CANDIDATES = [(128, 64), (192, 64), (256, 64), (384, 64), (512, 64), (768, 64), (256, 128),
                 (512, 128), (512, 1 << 30)]
SLOT_CANDIDATES = [2, 4, 6, 8]


def size_class(n, nnz=0, extra=""):
    """Size class of a problem: the number of unknowns and nonzeros rounded
    to a quarter power of two (problems within ~19 % share a choice)."""
    def q(x):
        return "%.2f" % (round(4 * math.log2(max(x, 1))) / 4)
    return "n%s_z%s%s" % (q(n), q(nnz), ("_" + extra) if extra else "")


def device_name():
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(torch.cuda.current_device()).replace(" ", "_")
    except Exception:  # no torch / no device: a host-only key
        pass
    return "host"


class Autotuner:
    """Timed-trial choice with a persistent cache.

    ``choose(kind, key, candidates, measure, repeats)`` returns the cached
    choice for (device, kind, key) or, on a miss, times every candidate
    with ``measure(candidate) -> seconds`` (``repeats`` times, the minimum
    counts), keeps the fastest, writes it to the cache file and returns it.
    """

    def __init__(self, path=None, device=None, enabled=True):
        self.path = path or os.environ.get("SUCEM_AUTOTUNE_CACHE", DEFAULT_CACHE)
        self.device = device or device_name()
        self.enabled = enabled
        self._lock = threading.Lock()
        self._data = None
        self.trials = 0  # candidate measurements made by this object

    def _load(self):
        if self._data is None:
            try:
                with open(self.path) as f:
                    self._data = json.load(f)
            except (OSError, ValueError):
                self._data = {}
        return self._data

    def _save(self):
        d = os.path.dirname(self.path)
        if d:
            os.makedirs(d, exist_ok=True)
        tmp = self.path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(self._data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)

    def _key(self, kind, key):
        return "%s|%s|%s" % (self.device, kind, key)

    def lookup(self, kind, key):
        with self._lock:
            e = self._load().get(self._key(kind, key))
        return None if e is None else _untuple(e["choice"])

    def choose(self, kind, key, candidates, measure, repeats=2):
        hit = self.lookup(kind, key)
        if hit is not None or not self.enabled:
            return hit if hit is not None else candidates[0]
        times = []
        for c in candidates:
            best = float("inf")
            for _ in range(max(1, repeats)):
                best = min(best, float(measure(c)))
                self.trials += 1
            times.append(best)
        k = min(range(len(candidates)), key=lambda i: times[i])
        with self._lock:
            self._load()[self._key(kind, key)] = {
                "choice": list(candidates[k]) if isinstance(candidates[k], tuple) else candidates[k],
                "seconds": times[k],
                "trials": {str(c): t for c, t in zip(candidates, times)},
                "when": time.time()}
            self._save()
        return candidates[k]


def _untuple(v):
    return tuple(v) if isinstance(v, list) else v


def tune_lu(lu, values, dtype, tuner=None, candidates=None, repeats=2, stream=None):
    """Choose the LU plan (super-panel width, panel threshold) for this
    matrix's size class by timing factorisations of ``values`` (CUDA events
    on the stream), configure ``lu`` with it and return it.  Single
    precision only (the double-precision factorisation has no tensor-core
    plan)."""
    import torch
    if dtype not in ("f32", "c64"):
        return lu.params
    tuner = tuner or Autotuner()
    key = size_class(lu.info["n"], lu.info["nnz"], "%s_f%d" % (dtype, lu.info["max_front"]))

    def measure(cand):
        lu.configure(*cand)
        lu.factor(values, dtype, stream=stream)  # first factor of a plan builds it
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        lu.factor(values, dtype, stream=stream)
        e1.record()
        torch.cuda.synchronize()
        lu.check()
        return e0.elapsed_time(e1) * 1e-3

    choice = tuner.choose("lu_plan", key, candidates or LU_CANDIDATES, measure, repeats=repeats)
    lu.configure(*choice)
    return choice


def tune_slots(run_sample, tuner=None, key="serve", candidates=None):
    """Choose the serving slot count: ``run_sample(slots) -> seconds`` serves
    a fixed request sample with that many slots; the fastest count is kept."""
    tuner = tuner or Autotuner()
    return tuner.choose("serve_slots", key, candidates or SLOT_CANDIDATES, run_sample, repeats=1)
