"""Serving loop: Poisson-process arrivals of Poisson / reaction-diffusion solves.

Request mix (seeded): dimension 2 or 3, element H1P1 or H1P2 (uniform), DoF
count log-uniform in [1e3, 2e6], per-cell kappa = exp(N(0,1)) as
BilinearForm([Gradient, Gradient], Action(kappa[cell] * input; "I")), with
probability 1/2 a ReactionOperator(alpha), alpha uniform in [0, 10], an
8-mode Fourier right-hand side and homogeneous Dirichlet data on the whole
boundary.  Requests are served by the library's serving engine
(grmp_server_*): slots with their own streams, admission by an HBM budget,
mixed-precision solves to a relative residual that gives <= 1e-10 relative
error against FP64.

Pooled workload (make_pooled_workload): the requests draw their mesh from a
small pool and vary the coefficients and right-hand side, like the
reference's parameter sweeps and time steps on one grid; with a mesh key the
server keeps each mesh's DoF map, pattern and solver workspace resident and
such requests run only assembly and solve.
"""
from __future__ import annotations

import ctypes
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from . import api
from .fespace import FESpace, H1P1, H1P2
from .mesh import grid_unitsquare, grid_unitcube_kuhn
from .problems import fourier_modes


@dataclass
class ServeRequest:
    dim: int
    order: int
    n: int
    FES: FESpace
    kappa: np.ndarray
    alpha: float
    amp: np.ndarray
    k: np.ndarray
    fixed: np.ndarray
    arrival_s: float = 0.0
    meta: dict = field(default_factory=dict)
    mesh_key: int = 0            # non-zero: data stay resident in the server under this key
    device_dofmap: bool = False  # DoF map and boundary DoFs built on the device (no host arrays)

    @property
    def ndofs(self) -> int:
        return self.FES.ndofs

    def operators(self):
        ops = [api.BilinearForm([api.Gradient, api.Gradient], api.CellCoefficient(self.kappa),
                                APT=api.APT_SymmetricBilinearForm)]
        if self.alpha > 0:
            ops.append(api.ReactionOperator(self.alpha))
        return ops

    def rhs(self):
        return api.LinearForm(api.Identity, api.DataFunction.fourier(self.amp, self.k))


def mesh_size_for(dofs: float, dim: int, order: int) -> int:
    """Number of subdivisions per axis whose DoF count is closest to `dofs`."""
    side = dofs ** (1.0 / dim)                 # DoFs per axis ~ (order n + 1)
    return max(2, int(round((side - 1) / order)))


STATUS_TIMEOUT = 7   # GRMP_ERR_TIMEOUT

_grid_cache: dict = {}
_space_cache: dict = {}


def build_request(rng: np.random.Generator, dofs_min=1e3, dofs_max=2e6, dim=None, order=None,
                  resident: bool = True) -> ServeRequest:
    dim = int(rng.integers(2, 4)) if dim is None else dim
    order = int(rng.integers(1, 3)) if order is None else order
    target = math.exp(rng.uniform(math.log(dofs_min), math.log(dofs_max)))
    n = mesh_size_for(target, dim, order)
    key = (dim, n)
    if key not in _grid_cache:
        _grid_cache[key] = grid_unitsquare(n) if dim == 2 else grid_unitcube_kuhn(n)
    g = _grid_cache[key]
    skey = (dim, n, order)
    if skey not in _space_cache:
        _space_cache[skey] = FESpace(H1P1(1) if order == 1 else H1P2(1, dim), g)
    FES = _space_cache[skey]
    kappa = np.exp(rng.standard_normal(g.ncells))
    alpha = float(rng.uniform(0, 10)) if rng.random() < 0.5 else 0.0
    amp, k = fourier_modes(rng, dim)
    return ServeRequest(dim, order, n, FES, kappa, alpha, amp, k, FES.boundary_dofs(),
                        mesh_key=mesh_key(dim, n, order) if resident else 0)


def mesh_key(dim: int, n: int, order: int) -> int:
    """Residency key of the unit square / Kuhn cube grid with n subdivisions and element order."""
    return (dim << 40) | (order << 32) | n


def make_pooled_workload(nrequests: int, nmeshes: int = 8, seed: int = 0, mean_interarrival_s: float = 0.05,
                         dofs_min=1e3, dofs_max=2e6, device_dofmap: bool = False):
    """Requests on a pool of `nmeshes` problems (dimension, element, size and
    whether a reaction term is present drawn as in make_workload), with fresh
    kappa, reaction coefficient and right-hand side per request and the pool
    entry's residency key."""
    rng = np.random.default_rng(seed)
    pool = []
    for _ in range(nmeshes):
        dim, order = int(rng.integers(2, 4)), int(rng.integers(1, 3))
        target = math.exp(rng.uniform(math.log(dofs_min), math.log(dofs_max)))
        pool.append((dim, order, mesh_size_for(target, dim, order), bool(rng.random() < 0.5)))
    reqs, t = [], 0.0
    for _ in range(nrequests):
        dim, order, n, reaction = pool[int(rng.integers(0, nmeshes))]
        key = (dim, n)
        if key not in _grid_cache:
            _grid_cache[key] = grid_unitsquare(n) if dim == 2 else grid_unitcube_kuhn(n)
        g = _grid_cache[key]
        skey = (dim, n, order)
        if skey not in _space_cache:
            _space_cache[skey] = FESpace(H1P1(1) if order == 1 else H1P2(1, dim), g)
        FES = _space_cache[skey]
        kappa = np.exp(rng.standard_normal(g.ncells))
        alpha = float(rng.uniform(0.1, 10)) if reaction else 0.0
        amp, k = fourier_modes(rng, dim)
        r = ServeRequest(dim, order, n, FES, kappa, alpha, amp, k, FES.boundary_dofs(),
                         mesh_key=mesh_key(dim, n, order), device_dofmap=device_dofmap)
        t += float(rng.exponential(mean_interarrival_s))
        r.arrival_s = t
        reqs.append(r)
    return reqs


def make_workload(nrequests: int, seed: int = 0, mean_interarrival_s: float = 0.05, dofs_max=2e6,
                  resident: bool = True):
    """Requests with Poisson-process arrival times (exponential gaps); with
    `resident` each carries the residency key of its grid and element, so
    requests that land on an already served mesh size reuse its device data."""
    rng = np.random.default_rng(seed)
    reqs, t = [], 0.0
    for _ in range(nrequests):
        r = build_request(rng, dofs_max=dofs_max, resident=resident)
        t += float(rng.exponential(mean_interarrival_s))
        r.arrival_s = t
        reqs.append(r)
    return reqs


class Server:
    """The library's serving engine (grmp_server_*)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 150 << 30, nslots: int = 4):
        self.lib = L.load()
        self.h = ctypes.c_void_p()
        rc = self.lib.grmp_server_create(device, hbm_budget_bytes, nslots, ctypes.byref(self.h))
        if rc:
            raise L.GrmpError(rc, "grmp_server_create")

    def submit(self, r: ServeRequest, mode: str = "mixed", reltol: float = 1e-11) -> int:
        q, keep = make_request(r, mode, reltol)
        rid = ctypes.c_int64()
        rc = self.lib.grmp_server_submit(self.h, ctypes.byref(q), ctypes.byref(rid))
        if rc:
            raise L.GrmpError(rc, "grmp_server_submit")
        return rid.value

    def wait(self, rid: int, ndofs: int | None = None, timeout_s: float = -1.0):
        """(status, solution, stats) of request rid; ndofs None asks the server
        for the solution's length first (a device-built DoF map)."""
        st = L.RequestStats()
        if ndofs is None:
            rc = self.lib.grmp_server_wait(self.h, rid, timeout_s, None, ctypes.byref(st))
            if rc == STATUS_TIMEOUT:
                return rc, None, None
            ndofs = st.ndofs   # 0 for a request that failed before its DoF map
        x = np.empty(ndofs)
        rc = self.lib.grmp_server_wait(self.h, rid, timeout_s, x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                       ctypes.byref(st))
        return rc, x, {"status": st.status, "slot": st.slot, "iterations": st.iterations,
                       "outer": st.outer_iterations, "relres": st.final_relres, "queue_ms": st.queue_ms,
                       "run_ms": st.run_ms, "latency_ms": st.latency_ms, "solve_ms": st.solve_ms,
                       "ndofs": st.ndofs, "resident": st.resident}

    def close(self):
        if self.h:
            self.lib.grmp_server_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


def estimate_bytes(r: ServeRequest) -> int:
    """The server's admission estimate for request r (grmp_server_request_bytes)."""
    lib = L.load()
    q, keep = make_request(r)
    v = ctypes.c_size_t()
    rc = lib.grmp_server_request_bytes(ctypes.byref(q), ctypes.byref(v))
    if rc:
        raise L.GrmpError(rc, "grmp_server_request_bytes")
    return v.value


def make_request(r: ServeRequest, mode: str = "mixed", reltol: float = 1e-11):
    """grmp_request for r; returns (request, arrays it points into)."""
    FES, g = r.FES, r.FES.xgrid
    q = L.Request()
    keep = []

    def arr(a, dt):
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a.ctypes.data_as(ctypes.POINTER(np.ctypeslib.as_ctypes_type(dt)))

    q.dim = g.dim
    q.nverts = g.nverts
    q.coords = arr(g.coords, np.float64)
    q.ncells = g.ncells
    q.cells = arr(g.cells, np.int32)
    q.fe_kind = FES.FEType.kind
    q.ncomponents = FES.FEType.ncomponents
    if r.device_dofmap:
        q.ndofs = 0
        q.celldofs = None
    else:
        q.ndofs = FES.ndofs
        q.celldofs = arr(FES.celldofs, np.int32)
    ops = r.operators()
    terms = (L.BilinearTerm * len(ops))()
    for i, o in enumerate(ops):
        terms[i] = o.term()
    keep.append(ops)
    q.nterms = len(ops)
    q.terms = terms
    lf = r.rhs()
    q.rhs = lf.rhs()
    keep.append(lf)
    if r.device_dofmap:
        q.nfixed = -1
        q.fixed = None
    else:
        q.nfixed = r.fixed.size
        q.fixed = arr(r.fixed, np.int32)
    s = api.GB300PCG(mode=mode, reltol=reltol, abstol=0.0)
    q.solve = s.params()
    q.mesh_key = r.mesh_key
    return q, keep


def run(reqs, nslots: int = 4, hbm_budget_bytes: int = 150 << 30, mode: str = "mixed", reltol: float = 1e-11,
        realtime: bool = True):
    """Submit the requests at their arrival times (realtime) or all at once;
    returns (solutions, per-request stats, makespan seconds)."""
    srv = Server(0, hbm_budget_bytes, nslots)
    try:
        t0 = time.perf_counter()
        ids = []
        for r in reqs:
            if realtime:
                dt = r.arrival_s - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
            ids.append(srv.submit(r, mode, reltol))
        xs, sts = [], []
        for r, rid in zip(reqs, ids):
            rc, x, st = srv.wait(rid, None if r.device_dofmap else r.ndofs)
            st["rc"] = rc
            xs.append(x)
            sts.append(st)
        makespan = time.perf_counter() - t0
    finally:
        srv.close()
    return xs, sts, makespan


def summarize(reqs, sts, makespan):
    lat = np.array([s["latency_ms"] for s in sts])
    dofs = sum(r.ndofs for r in reqs)
    return {"requests": len(reqs), "dofs": int(dofs), "makespan_s": makespan, "dof_per_s": dofs / makespan,
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "max": float(lat.max())},
            "failed": int(sum(1 for s in sts if s["rc"] != 0)),
            "resident_hits": int(sum(1 for s in sts if s.get("resident")))}
