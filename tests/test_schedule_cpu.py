"""Host checks of the order-1/2 assembly schedule (the work plan of the
entity-per-lane assembly kernel), no GPU needed.

The kernel's data flow is replayed in numpy: every lane of every warp task
takes its entity's incident cells step by step (local entity index major),
adds the oracle's element-matrix rows of that local entity at the column
slots of the step record, and the rows are compared with the oracle's CSR
matrices S, T and B.  This pins that every incidence is visited exactly
once, that the slots point at the right CSR columns and that boundary
entities (the only ones with ABC entries) are in the boundary tasks."""
import numpy as np
import pytest

from oracle import fem


def _space(coords, cells, order):
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    return FunctionSpace(Mesh(coords, cells), order=order)


def _replay(V, ref, order):
    sch = V.assembly_schedule()
    ent, meta, words = sch["task_ent"], sch["task_meta"], sch["step_words"]
    nd = V.ndof_cell
    dpe = order
    ne = V.ne
    ip = V.indptr
    coords, cells = V.mesh().coordinates(), V.cells
    S_e, T_e = fem.element_matrices(coords, cells, order, np.ones(V.nt), np.ones(V.nt))
    fc, flf = ref.topo.exterior_facets()
    B_e = fem.facet_matrices(coords, cells, order, fc, flf)
    ext = {}
    for i, (c, f) in enumerate(zip(fc, flf)):
        ext.setdefault(int(c), []).append((int(f), i))
    edge_verts = [(2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1)]
    out = {k: np.zeros(V.nnz) for k in "STB"}
    visits = 0
    n_int = sch["n_tasks_interior"]
    for t in range(len(ent)):
        trip = np.frombuffer(meta[t, 1:3].tobytes(), dtype=np.uint8)
        face = bool(meta[t, 3] & 1)
        s = int(meta[t, 0])
        for le in range(8):
            for _ in range(int(trip[le])):
                blk = words[s]
                s += 1
                for lane in range(32):
                    c = int(np.int32(blk[0, lane]))
                    k = int(ent[t, lane])
                    if c < 0:
                        continue
                    assert k >= 0
                    assert (k >= ne) == face
                    visits += 1
                    slots = [(int(blk[1 + b // 4, lane]) >> (8 * (b % 4))) & 255 for b in range(nd)]
                    for j in range(dpe):
                        a = 12 + 2 * le + j if face else dpe * le + j
                        pos = ip[dpe * k + j] + np.array(slots)
                        np.add.at(out["S"], pos, S_e[c, a])
                        np.add.at(out["T"], pos, T_e[c, a])
                        if t >= n_int:
                            for f, i in ext.get(c, []):
                                holds = (f == le) if face else (f not in edge_verts[le])
                                if holds:
                                    np.add.at(out["B"], pos, B_e[i, a])
    return out, visits


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("jitter", [False, True])
def test_schedule_replay_matches_oracle(order, jitter):
    coords, cells = fem.box_mesh(1.0, 0.8, 0.6, 3, 3, 2)
    if jitter:
        coords = fem.jitter_interior(coords, cells, 1.0 / 3, 0.2, 7)
    V = _space(coords, cells, order)
    ref = fem.assemble(coords, cells, order)
    got, visits = _replay(V, ref, order)
    assert visits == V.nt * (6 if order == 1 else 10)
    for k, R in (("S", ref.S), ("T", ref.T), ("B", ref.B)):
        scale = np.abs(R.data).max()
        assert np.abs(got[k] - R.data).max() <= 1e-13 * scale, k


def test_schedule_tasks_cover_entities_once_and_group_by_kind():
    coords, cells = fem.box_mesh(1.0, 1.0, 1.0, 4, 3, 3)
    V = _space(coords, cells, 2)
    sch = V.assembly_schedule()
    ent = sch["task_ent"]
    ids = ent[ent >= 0]
    assert np.array_equal(np.sort(ids), np.arange(V.ne + V.nf))
    for t in range(len(ent)):
        lanes = ent[t][ent[t] >= 0]
        assert len(lanes) > 0
        assert np.all((lanes >= V.ne) == bool(sch["task_meta"][t, 3] & 1))
