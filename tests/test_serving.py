"""Serving engine (grmp_server_*): continuous admission of Poisson /
reaction-diffusion requests of mixed size and element type.

* every result equals the same request served alone (bit for bit: launch
  shapes and the SpMV configuration come from the request's own sizes);
* results match the oracle's FP64 sparse-direct solution to 1e-10;
* the HBM budget admits requests one at a time when only one fits, and a
  request larger than the budget is refused at submission.
"""
import types

import numpy as np
import pytest

from parity_helpers import oracle_system

pytestmark = pytest.mark.gpu


def _workload(G, n=10, seed=3, dofs_max=6e4):
    from grmp_gb300 import serve as SV
    return SV.make_workload(n, seed=seed, dofs_max=dofs_max)


def test_served_results_same_alone_and_in_the_mix(G):
    from grmp_gb300 import serve as SV
    reqs = _workload(G)
    xs_mix, sts_mix, _ = SV.run(reqs, nslots=4, realtime=False)
    assert all(s["rc"] == 0 for s in sts_mix), [s["rc"] for s in sts_mix]
    assert len({s["slot"] for s in sts_mix}) > 1          # several workers took part
    for r, xm in zip(reqs, xs_mix):
        xa, sa, _ = SV.run([r], nslots=1, realtime=False)
        assert sa[0]["rc"] == 0
        assert np.array_equal(xa[0], xm)


def test_served_solutions_match_oracle(G, O):
    from grmp_gb300 import serve as SV
    reqs = sorted(_workload(G, n=8, seed=5, dofs_max=2e4), key=lambda r: r.ndofs)[:4]
    xs, sts, _ = SV.run(reqs, nslots=2, realtime=False)
    for r, x, st in zip(reqs, xs, sts):
        assert st["rc"] == 0
        prob = types.SimpleNamespace(FES=r.FES, operators=r.operators(), rhs=r.rhs(), fixed=r.fixed)
        _, Apen, _, bpen = oracle_system(G, O, prob)
        uo = O.solve_direct(Apen, bpen)
        err = np.linalg.norm(x - uo) / np.linalg.norm(uo)
        assert err <= 1e-10, (r.dim, r.order, r.ndofs, err, st)


def test_budget_serialises_and_refuses(G):
    from grmp_gb300 import serve as SV
    from grmp_gb300 import _lib as L
    reqs = _workload(G, n=4, seed=7, dofs_max=3e4)
    # a budget that holds one request at a time: all complete, none overlap
    srv = SV.Server(0, hbm_budget_bytes=int(1.2 * max(SV.estimate_bytes(r) for r in reqs)), nslots=4)
    try:
        ids = [srv.submit(r) for r in reqs]
        outs = [srv.wait(i, r.ndofs) for i, r in zip(ids, reqs)]
        assert all(rc == 0 for rc, _, _ in outs)
        big = _workload(G, n=1, seed=8, dofs_max=3e4)[0]
        tiny = SV.Server(0, hbm_budget_bytes=1 << 20, nslots=1)
        try:
            with pytest.raises(L.GrmpError) as ei:
                tiny.submit(big)
            assert ei.value.code == L.ERR_BUDGET
        finally:
            tiny.close()
    finally:
        srv.close()
