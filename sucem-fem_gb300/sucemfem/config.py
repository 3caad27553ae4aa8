"""Precision knobs of the GPU path.

ASSEMBLY_REAL_BYTES: 8 (FP64, the drop-in default: same numbers as the
reference's DOLFIN assembly to ~1e-15) or 4 (FP32, the fast path; per-entry
error vs FP64 is reported by the tests and the bench)."""
ASSEMBLY_REAL_BYTES = 8
