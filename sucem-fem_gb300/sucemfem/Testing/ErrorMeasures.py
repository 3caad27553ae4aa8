"""Error measures of sucemfem/Testing/ErrorMeasures.py:22-60 (percentages;
note that both sum the squared relative errors without a square root or a
mean, which the names do not say)."""
import numpy as np


def _terms(actual, desired, extra_error):
    err = np.abs(np.asarray(actual) - np.asarray(desired))
    extra = np.zeros_like(err) if extra_error is None else np.abs(np.asarray(extra_error))
    return err, extra


def normalised_RMS(actual, desired, extra_error=None):
    """100 * sum(((|actual - desired|)/|actual|)^2 + (|extra|/|actual|)^2)."""
    err, extra = _terms(actual, desired, extra_error)
    a = np.abs(np.asarray(actual))
    return 100 * np.sum((err / a) ** 2 + (extra / a) ** 2)


def max_normalised_RMS(actual, desired, extra_error=None):
    """As ``normalised_RMS`` with every term normalised by max |actual|, so
    values of actual near zero do not dominate."""
    err, extra = _terms(actual, desired, extra_error)
    m = np.abs(np.asarray(actual)).max()
    return 100 * np.sum((err / m) ** 2 + (extra / m) ** 2)
