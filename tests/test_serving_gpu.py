"""Continuous-batching server: every request converges, results are the
same alone and in the mix (solutions within 1e-7 relative for a 1e-10
refinement tolerance; only the order of some floating-point additions can
differ), admission respects the HBM budget and rejects what cannot fit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mix():
    from sucemfem.serving import DrivenRequest
    reqs = []
    for i, (nc, order) in enumerate([(5, 1), (4, 2), (7, 1), (6, 2), (8, 1), (5, 2)]):
        reqs.append(DrivenRequest(i, nc, order, 1.0, 2 * np.pi * (1.0 + 0.5 * i), 100 + i, 0.01 * i))
    return reqs


def test_mix_equals_alone_and_converges():
    from sucemfem.serving import SolveServer
    reqs = _mix()
    srv = SolveServer(slots=3, tol=1e-10, keep_solutions=True)
    res = srv.run(reqs, realtime=False)
    assert [r.status for r in res] == ["ok"] * len(reqs)
    assert all(r.residual <= 1e-10 for r in res)
    assert srv.stats["completed"] == len(reqs)
    for i in (1, 4):
        alone = SolveServer(slots=1, tol=1e-10, keep_solutions=True).run([reqs[i]], realtime=False)[0]
        x, y = res[i].x, alone.x
        assert np.linalg.norm(x - y) / np.linalg.norm(y) <= 1e-7


def test_budget_admission_and_rejection():
    from sucemfem.serving import SolveServer, _Prepared
    reqs = _mix()
    need = [_Prepared(r).bytes for r in reqs]
    budget = int(sorted(need)[-2] * 1.01)       # the largest request cannot fit
    srv = SolveServer(hbm_budget_bytes=budget, slots=3, tol=1e-8)
    res = srv.run(reqs, realtime=False)
    big = int(np.argmax(need))
    assert res[big].status.startswith("rejected")
    assert all(r.status == "ok" for i, r in enumerate(res) if i != big)
    assert srv.stats["rejected"] == 1


def test_single_request_matches_oracle():
    import scipy.sparse.linalg as spl
    from oracle import fem
    from sucemfem.serving import DrivenRequest, SolveServer
    req = DrivenRequest(0, 4, 2, 1.0, 2 * np.pi * 2.0, 7, 0.0)
    res = SolveServer(slots=1, tol=1e-11, keep_solutions=True).run([req], realtime=False)[0]
    coords, cells = fem.box_mesh(1.0, 1.0, 1.0, 4, 4, 4)
    eps = np.random.default_rng(7).uniform(1.0, 4.0, len(cells))
    A = fem.assemble(coords, cells, 2, eps_r=eps)
    f = req.k0 * 299792458 / (2 * np.pi)
    L = fem.lhs_matrix(A.S, A.T, A.B, f)
    d, v = fem.point_source_contrib(coords, cells, 2, A.topo, A.dofmap, np.array([.5, .5, .5]),
                                    np.array([0, 0, 1.0]))
    xr = spl.spsolve(L.tocsc(), fem.rhs_vector(A.n, f, d, v))
    assert np.linalg.norm(res.x - xr) / np.linalg.norm(xr) < 1e-9
