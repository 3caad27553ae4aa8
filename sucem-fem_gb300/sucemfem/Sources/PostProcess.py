"""Voltage along a straight line (sucemfem/Sources/PostProcess.py:26-66):
the line integral of E . l_hat from start to end, by Romberg integration
over the unit parameter interval (scipy.integrate.romberg with its default
tolerances, which the reference calls and current SciPy no longer ships,
is restated in ``romberg``).  ``ComplexVoltageAlongLine`` evaluates the
field of a DOF vector on the GPU, every Romberg level's new points in one
batched reconstruction; the real and imaginary parts keep separate
integration tables and stopping tests, as two separate calls would."""
import warnings

import numpy as np

from ..Utilities.Geometry import unit_vector, vector_length


def romberg(f, a, b, tol=1.48e-8, rtol=1.48e-8, divmax=10):
    """Romberg integrals of the columns of a vectorised integrand.

    f(t) takes an array of abscissae and returns an array of shape (len(t),)
    or (len(t), m).  Row i of every column's table halves the trapezoid
    step (2^i intervals) and Richardson-extrapolates; a column stops when
    its last two diagonal entries differ by less than tol or rtol times the
    latest (at most divmax halvings, then the last value is returned with a
    warning).  Returns a float, or an array of m floats."""
    h = float(b - a)
    y = np.asarray(f(np.array([a, b], dtype=np.float64)), dtype=np.float64)
    vec = y.ndim == 2
    y = y.reshape(2, -1)
    m = y.shape[1]
    prev = [[0.5 * h * (y[0, j] + y[1, j])] for j in range(m)]
    result = [p[0] for p in prev]
    done = [False] * m
    for i in range(1, divmax + 1):
        n = 1 << (i - 1)
        h *= 0.5
        t = a + h * (2.0 * np.arange(n) + 1.0)
        s = np.asarray(f(t), dtype=np.float64).reshape(n, -1).sum(axis=0)
        for j in range(m):
            if done[j]:
                continue
            row = [0.5 * prev[j][0] + h * s[j]]
            for k in range(1, i + 1):
                row.append(row[k - 1] + (row[k - 1] - prev[j][k - 1]) / (4.0 ** k - 1.0))
            err = abs(row[i] - prev[j][i - 1])
            prev[j], result[j] = row, row[i]
            if err < tol or err < rtol * abs(row[i]):
                done[j] = True
        if all(done):
            break
    if not all(done):
        warnings.warn("romberg: divmax (%d) exceeded before convergence" % divmax)
    return np.array(result) if vec else result[0]


class VoltageAlongLine(object):
    """Voltage of a real field given as a callable fn(x, y, z) -> E (3)."""

    def __init__(self, field_function):
        self.field_function = field_function

    def calculate_voltage(self, start_pt, end_pt):
        start = np.asarray(start_pt, dtype=np.float64)
        delta = np.asarray(end_pt, dtype=np.float64) - start
        l_hat = unit_vector(delta)
        fn = self.field_function

        def integrand(t):
            return np.array([np.dot(l_hat, fn(*(start + delta * ti))) for ti in t])
        return romberg(integrand, 0.0, 1.0) * vector_length(delta)


class ComplexVoltageAlongLine(object):
    """Complex voltage of the field of a DOF vector of ``function_space``."""

    def __init__(self, function_space):
        self.function_space = function_space

    def set_dofs(self, dofs):
        from ..PostProcessing.PostProcessing import Reconstruct
        self.dofs = dofs
        self.reconstruct = Reconstruct(self.function_space)
        self.reconstruct.set_dof_values(dofs)

    def calculate_voltage(self, start_pt, end_pt):
        start = np.asarray(start_pt, dtype=np.float64)
        delta = np.asarray(end_pt, dtype=np.float64) - start
        l_hat = unit_vector(delta)

        def integrand(t):
            E = self.reconstruct.reconstruct_points(start[None, :] + np.outer(t, delta))
            v = E @ l_hat
            return np.stack([v.real, v.imag], axis=1)
        re, im = romberg(integrand, 0.0, 1.0)
        return (re + 1j * im) * vector_length(delta)
