"""Vector helpers of sucemfem/Utilities/Geometry.py:22-28."""
import numpy as np


def vector_length(vec):
    """Euclidean length of ``vec``."""
    v = np.asarray(vec, dtype=np.float64)
    return float(np.sqrt(np.dot(v, v)))


def unit_vector(vec):
    """``vec`` scaled to unit length."""
    v = np.asarray(vec, dtype=np.float64)
    return v / vector_length(v)
