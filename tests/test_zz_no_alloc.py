"""The allocation-free compaction count against the ordinary one.

sucem_compact_count_noalloc exists for callers that cannot allocate device
memory when they need the compaction (a serving loop that reserved its
whole HBM budget for resident problems, or a host whose device memory
belongs to another allocator): its row-count scratch is a fixed array inside
the library instead of a caller buffer.  This file is collected last so a
stop-at-first-failure run has already run everything else; it also passes
on its own in a fresh process."""
import numpy as np
import pytest

from oracle import fem

pytestmark = pytest.mark.gpu


def _space_and_values(seed):
    import torch
    from sucemfem import _device
    from sucemfem._native import call, ptr
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    coords, cells = fem.box_mesh(1.0, 0.7, 0.5, 5, 4, 3)
    V = FunctionSpace(Mesh(coords, cells), order=2)
    A = torch.empty(V.nnz, dtype=torch.complex128, device=_device.device())
    eps = torch.as_tensor(np.random.default_rng(seed).uniform(1, 4, V.nt), device=_device.device())
    call("sucem_assemble_helmholtz", V.upload(), 8, ptr(eps), None, 7.0, ptr(A), _device.stream_ptr())
    # plant exact zeros so the compaction has something to drop
    drop = np.random.default_rng(seed + 1).random(V.nnz) < 0.3
    A[torch.as_tensor(drop, device=A.device)] = 0
    return V, A


def _count(V, A, noalloc):
    import torch
    from sucemfem import _device
    from sucemfem._native import call, ptr
    out = torch.full((V.n + 1,), -7, dtype=torch.int32, device=_device.device())
    if noalloc:
        call("sucem_compact_count_noalloc", V.upload(), 3, ptr(A), ptr(out), _device.stream_ptr())
    else:
        work = torch.empty(V.n, dtype=torch.int32, device=_device.device())
        call("sucem_compact_count", V.upload(), 3, ptr(A), ptr(out), ptr(work), _device.stream_ptr())
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_count_matches_the_allocating_one_twice():
    for seed in (0, 5):  # two calls in a row, different data each time
        V, A = _space_and_values(seed)
        ref = _count(V, A, noalloc=False)
        got = _count(V, A, noalloc=True)
        assert np.array_equal(got, ref)
        keep = (A != 0).cpu().numpy()
        assert got[-1] == int(keep.sum())


def test_noalloc_rejects_too_many_rows():
    import torch
    from sucemfem import _device
    from sucemfem._native import call, ptr
    from sucemfem.mesh import BoxMesh
    from sucemfem.space import FunctionSpace
    V = FunctionSpace(BoxMesh(1, 1, 1, 56, 56, 56), order=1)
    assert V.n > (1 << 20)
    A = torch.zeros(V.nnz, dtype=torch.complex64, device=_device.device())
    out = torch.empty(V.n + 1, dtype=torch.int32, device=_device.device())
    with pytest.raises(ValueError, match="at most"):
        call("sucem_compact_count_noalloc", V.upload(), 2, ptr(A), ptr(out), _device.stream_ptr())
