"""sucemfem/Utilities/Optimization.py:24-39 switches DOLFIN's form-compiler
optimisation.  Here the element tensors are precomputed reference tables
contracted by hand-written kernels, so there is no form compiler to tune:
the call is accepted for scripts that make it and changes nothing."""


def set_dolfin_optimisation(enable=True):
    """Accepted for compatibility; returns the requested setting."""
    return bool(enable)
