"""File helpers of sucemfem/Testing/Paths.py:22-41, used by the reference's
tests to find their data next to the test module."""
import os


def get_module_path(modfile):
    """Directory of the module whose ``__file__`` is ``modfile``."""
    return os.path.dirname(modfile)


def get_module_path_filename(filename, modfile):
    """``filename`` in the directory of the module ``modfile``."""
    return os.path.join(get_module_path(modfile), filename)


def get_module_path_file(filename, modfile, mode="r"):
    """Open ``filename`` in the directory of the module ``modfile``."""
    return open(get_module_path_filename(filename, modfile), mode)
