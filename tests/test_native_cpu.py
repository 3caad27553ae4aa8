"""CPU-side checks of the native library: it loads, exports every entry
point the header declares, and its host builder (entities, DOF map, CSR
pattern, boundary DOFs) is bit-exact against the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from oracle import fem

HEADER = os.path.join(ROOT, "include", "sucem_gb300.h")


def _declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(
        r"^\s*(?:int|void|const char\*|int64_t|long long)\s+(sucem_\w+)\s*\(", txt, re.M)))


def test_library_exports_every_declared_symbol():
    from sucemfem import _native
    lib = _native.lib()
    names = _declared()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.sucem_version() == 1


def _space(coords, cells, order):
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    return FunctionSpace(Mesh(coords, cells), order=order)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("mesh", ["inscribed", "cube322", "jitter3"])
def test_builder_matches_oracle(order, mesh):
    if mesh == "inscribed":
        coords, cells = fem.inscribed_tet()
    elif mesh == "cube322":
        coords, cells = fem.box_mesh(1.0, 0.5, 0.75, 3, 2, 2)
    else:
        coords, cells = fem.unit_cube(3, 3, 3)
        coords = fem.jitter_interior(coords, cells, 1 / 3, 0.2, seed=0)
        # scrambled vertex order inside each cell must not matter
        rng = np.random.default_rng(1)
        cells = np.array([rng.permutation(c) for c in cells])
    V = _space(coords, cells, order)
    topo = fem.Topology(np.sort(cells, axis=1))
    dm, n = fem.dofmap(topo, order)
    ip, ix = fem.sparsity(dm, n)
    assert V.n == n and V.nnz == len(ix)
    assert np.array_equal(V.cell_dofs, dm)
    assert np.array_equal(V.indptr, ip)
    assert np.array_equal(V.indices, ix)
    assert np.array_equal(np.sort(V.boundary_dofs), fem.pec_dofs(topo, order))
    assert V.n_ext_facets == len(topo.exterior_faces())


def test_builder_rejects_bad_input():
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    coords, cells = fem.unit_cube(1, 1, 1)
    bad = cells.copy()
    bad[0, 0] = 99
    with pytest.raises(ValueError, match="out of range"):
        FunctionSpace(Mesh(coords, bad), order=1)
    with pytest.raises(ValueError):
        FunctionSpace(Mesh(coords, cells), order=5)
    with pytest.raises(ValueError):
        FunctionSpace(Mesh(coords, cells), order=0)
    rep = cells.copy()
    rep[0, 1] = rep[0, 0]
    with pytest.raises(ValueError, match="degenerate"):
        FunctionSpace(Mesh(coords, rep), order=1)


def test_config1_sizes():
    coords, cells = fem.box_mesh(1.0, 0.5, 0.75, 8, 4, 6)
    V1 = _space(coords, cells, 1)
    V2 = _space(coords, cells, 2)
    assert (V1.n, V1.nnz) == (1674, 23658)
    assert (V2.n, V2.nnz) == (8372, 330856)
