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


def _cold(reqs):
    import dataclasses
    return [dataclasses.replace(r, mesh_key=0, device_dofmap=False) for r in reqs]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_resident_results_match_cold_requests(G):
    """Requests on a pool of three meshes: with residency most of them reuse
    a slot's mesh, DoF map, pattern and solver workspace.  A resident pattern
    is built with unit coefficients (it serves every later coefficient field),
    so it may hold a few stored entries whose cold pattern drops as exact
    zeros of that request's coefficients: the solutions agree with the cold
    requests' to the serving tolerance, and a replay of the same sequence on
    one slot is bit-identical."""
    from grmp_gb300 import serve as SV
    reqs = SV.make_pooled_workload(12, nmeshes=3, seed=11, dofs_max=5e4)
    xs_res, sts_res, _ = SV.run(reqs, nslots=2, realtime=False)
    assert all(s["rc"] == 0 for s in sts_res), [s["rc"] for s in sts_res]
    assert sum(s["resident"] for s in sts_res) >= 12 - 2 * 3   # at most one cold start per mesh and slot
    xs_cold, sts_cold, _ = SV.run(_cold(reqs), nslots=2, realtime=False)
    assert not any(s["resident"] for s in sts_cold)
    for xr, xc in zip(xs_res, xs_cold):
        assert _rel(xr, xc) <= 1e-10
    xa, sa, _ = SV.run(reqs, nslots=1, realtime=False)
    xb, sb, _ = SV.run(reqs, nslots=1, realtime=False)
    assert [s["resident"] for s in sa] == [s["resident"] for s in sb]
    for a, b in zip(xa, xb):
        assert np.array_equal(a, b)


def test_device_dofmap_requests_equal_host_dofmap(G):
    """Requests without CellDofs and Dirichlet lists (both built on the
    device) give the host-numbered requests' solutions bit for bit, and with
    residency the same to the serving tolerance."""
    import dataclasses
    from grmp_gb300 import serve as SV
    reqs = SV.make_pooled_workload(8, nmeshes=4, seed=12, dofs_max=4e4, device_dofmap=True)
    one_off = [dataclasses.replace(r, mesh_key=0) for r in reqs]
    xs_dev, sts_dev, _ = SV.run(one_off, nslots=2, realtime=False)
    assert all(s["rc"] == 0 for s in sts_dev)
    xs_host, _, _ = SV.run(_cold(reqs), nslots=2, realtime=False)
    for r, xd, xh, st in zip(reqs, xs_dev, xs_host, sts_dev):
        assert st["ndofs"] == r.ndofs
        assert np.array_equal(xd, xh)
    xs_res, sts_res, _ = SV.run(reqs, nslots=2, realtime=False)
    assert all(s["rc"] == 0 for s in sts_res) and any(s["resident"] for s in sts_res)
    for xr, xh in zip(xs_res, xs_host):
        assert _rel(xr, xh) <= 1e-10


def test_resident_entries_are_evicted_under_budget(G):
    """A budget that holds about two requests: resident entries of idle slots
    are dropped as new meshes arrive, and every request completes."""
    from grmp_gb300 import serve as SV
    reqs = SV.make_pooled_workload(10, nmeshes=5, seed=13, dofs_max=3e4)
    budget = int(2.2 * max(SV.estimate_bytes(r) for r in reqs))
    xs, sts, _ = SV.run(reqs, nslots=2, hbm_budget_bytes=budget, realtime=False)
    assert all(s["rc"] == 0 for s in sts), [s["rc"] for s in sts]
    xs_cold, _, _ = SV.run(_cold(reqs), nslots=1, realtime=False)
    for a, b in zip(xs, xs_cold):
        assert _rel(a, b) <= 1e-10


def test_large_request_near_two_million_dofs(G):
    """One 3D P2 request of ~1.8M DoFs (60^3 Kuhn cubes) through the server:
    the mixed result against the FP64 one (1e-10 relative, the serving
    tolerance), then the same mesh resubmitted with new coefficients runs on
    its resident data and equals a cold run of it."""
    import dataclasses
    from grmp_gb300 import serve as SV
    rng = np.random.default_rng(21)
    r = SV.build_request(rng, dofs_min=1.7e6, dofs_max=1.9e6, dim=3, order=2)
    assert 1.5e6 <= r.ndofs <= 2.1e6
    xs_m, st_m, _ = SV.run([r], nslots=1, mode="mixed", realtime=False)
    xs_f, st_f, _ = SV.run([r], nslots=1, mode="fp64", realtime=False)
    assert st_m[0]["rc"] == 0 and st_f[0]["rc"] == 0
    assert np.linalg.norm(xs_m[0] - xs_f[0]) <= 1e-10 * np.linalg.norm(xs_f[0])
    r2 = dataclasses.replace(r, kappa=np.exp(rng.standard_normal(r.kappa.size)))
    xs2, st2, _ = SV.run([r, r2], nslots=1, realtime=False)
    assert st2[1]["resident"] == 1
    xc, _, _ = SV.run([r2], nslots=1, realtime=False)
    assert np.array_equal(xs2[1], xc[0])
