"""sucemfem/PostProcessing/circuit.py:18-25."""
import numpy as np


def S11(Zl, Z0):
    """Reflection coefficient (Zl - Z0) / (Zl + Z0) of a load Zl on a line of
    characteristic impedance Z0 (element-wise for arrays)."""
    z = np.asarray(Zl)
    return (z - Z0) / (z + Z0)
