"""Saving and loading matrices as MATLAB .mat files
(sucemfem/Utilities/MatrixIO.py:24-85), through scipy.io."""
import os

import numpy as np


def check_path(path, create=True):
    """True when ``path`` exists after the call (created if missing and
    ``create``; with ``create`` False a missing path also answers True, as
    the reference's helper does)."""
    if not os.path.exists(path) and create:
        os.makedirs(path)
    return True


def save_scipy_matrix_as_mat(path, name, matrix):
    """Writes ``matrix`` (sparse or dense) to ``path/name.mat`` under the
    variable ``name``."""
    import scipy.io
    if not check_path(path):
        return False
    # the file is name.mat whatever the SciPy version's extension default
    scipy.io.savemat(os.path.join(path, name + ".mat"), {name: matrix}, oned_as="column")
    return True


def load_scipy_matrix_from_mat(path, name):
    """The variable ``name`` of ``path/name.mat``: CSR for a sparse matrix,
    the ndarray otherwise; None when the file does not exist."""
    import scipy.io
    filename = os.path.join(path, name)
    if not os.path.exists(filename + ".mat"):
        return None
    data = scipy.io.loadmat(filename + ".mat")[name]
    return data if isinstance(data, np.ndarray) else data.tocsr()
