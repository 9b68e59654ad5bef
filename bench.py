#!/usr/bin/env python3
"""Benchmark: DoF/s of assembly + solve at <= 1e-10 relative error against
FP64, mixed-precision versus plain FP64 on the GPU, with p50/p99 latency.

Workload (default): 3D Poisson, unit cube 64^3 Kuhn tetrahedra (1,572,864
cells), H1P2 (2,146,689 DoFs), per-cell kappa = exp(N(0,1)) (seed 0),
f = 8 seeded Fourier modes, homogeneous Dirichlet.  One step = FP64 (+ FP32)
assembly of the matrix, the right-hand side, Dirichlet elimination and the
solve; inputs (mesh, pattern, kappa) are resident in HBM when a timed step
starts.  The matrix (~490 MB FP64) and its FP32 copy exceed the 129 MB L2, so
no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 64]

Under torchrun (N > 1) every rank solves its own replica (the path does not
shard: replicas only, weak scaling); rank 0 prints the JSON line.
"""
from __future__ import annotations

import argparse
import ctypes
import dataclasses
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "gradientrobustmultiphysics.jl_gb300")
METRIC = "DoF/s assembly+solve at 1e-10 rel err vs FP64: mixed vs plain GPU; p50/p99 latency"


def _package():
    if "grmp_gb300" in sys.modules:
        return sys.modules["grmp_gb300"]
    spec = importlib.util.spec_from_file_location("grmp_gb300", os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["grmp_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, single: bool = False):
        self.ws, self.rank, self.local = (1, 0, dist_env()[2]) if single else dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo")
            self.td = td

    @classmethod
    def single(cls):
        """This process alone (the bounded summaries the headline run adds)."""
        return cls(single=True)

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join("/tmp", f"grmp_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names[1:], p[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


# ------------------------------------------------------------------ CPU baseline (oracle port)
WORKLOADS = {
    # name: (description, default size n, CPU sample size, solve tolerance for <= 1e-10 error vs FP64)
    "poisson3d": ("poisson3d_P2_kuhn{n}_lognormal_kappa", 64, 64, 1e-11),
    "poisson2d": ("poisson2d_P2_{n}x{n}_kappa1e-3", 128, 128, 1e-11),
    "elasticity2d": ("elasticity2d_P2vec_{n}x{n}_mu1_lambda1e3", 256, 32, 1e-12),
}


def make_problem(P, args, seed: int, n: int = None):
    """The workload's LinearProblem at size n (default: the workload's)."""
    n = n or args.n or WORKLOADS[args.workload][1]
    if args.workload == "poisson2d":
        return P.poisson2d(n)
    if args.workload == "elasticity2d":
        return P.elasticity2d(n, seed=seed)
    return P.poisson3d(n, seed=seed)


def cpu_port_step(prob, reltol: float):
    """The workload's assembly + solve on the host cores with the oracle: the
    reference's item loop (each row's additions in the reference's order; rows
    split among OpenMP threads, bit-identical to one thread), the penalised
    Dirichlet rows, then FP64 Jacobi-CG (OpenMP) to `reltol`.  Returns
    (dofs, seconds, assembly_s, solve_s, iterations, A, b, x)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    FES = prob.FES
    g = FES.xgrid
    fe = 1 if FES.FEType.kind == 1 else 2
    nc = FES.FEType.ncomponents
    t0 = time.perf_counter()
    M = O.Matrix(FES.ndofs)
    for op in prob.operators:
        if op.op_kind == 1:
            act = O.ACT_CELLSCALE if op.cell_coef is not None else O.ACT_NONE
            M.add_bilinear(g.coords, g.cells, fe, nc, FES.celldofs, O.OP_GRADIENT, op.symmetric, op.factor, act,
                           op.cell_coef)
        elif op.op_kind == 2:
            act = O.ACT_CELLSCALE if op.cell_coef is not None else O.ACT_NONE
            M.add_bilinear(g.coords, g.cells, fe, nc, FES.celldofs, O.OP_IDENTITY, op.symmetric, op.factor, act,
                           op.cell_coef)
        else:
            M.add_bilinear(g.coords, g.cells, fe, nc, FES.celldofs, O.OP_SYMGRAD, op.symmetric, op.factor,
                           O.ACT_HOOKE2D if g.dim == 2 else O.ACT_HOOKE3D, mu=op.params[0], lam=op.params[1])
    b = np.zeros(FES.ndofs)
    f = prob.rhs.f
    O.assemble_linear(b, g.coords, g.cells, fe, nc, FES.celldofs, f.kind, f.params, prob.rhs.factor,
                      f.bonus_quadorder)
    M.penalize(prob.fixed)
    A = M.csr()
    bb = O.penalized_rhs(b, prob.fixed)
    t1 = time.perf_counter()
    x, it, rr = O.solve_cg(A, bb, reltol)
    t2 = time.perf_counter()
    return FES.ndofs, t2 - t0, t1 - t0, t2 - t1, it, A, bb, x


# sample of the single-core CPU baseline per workload (bounded to a few seconds
# of one core; the all-core baseline runs the full workload)
SINGLE_CORE_N = {"poisson3d": 24, "poisson2d": 128, "elasticity2d": 16}


def cpu_single_core(P, args, n: int = None) -> dict:
    """The oracle port on ONE host core (the reference assembles in one Julia
    task, src/assemblypatterns/bilinearform.jl:226), on a bounded sample of
    the workload: assembly in the reference's item-loop order + FP64
    Jacobi-CG to the workload's tolerance."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    n = n or SINGLE_CORE_N[args.workload]
    O.set_threads(1)
    try:
        d, dt, ta, ts, it, _, _, _ = cpu_port_step(make_problem(P, args, args.seed, n), args.reltol)
    finally:
        O.set_threads(0)
    return {"value": d / dt, "unit": "DoF/s", "cores": 1, "kind": "port",
            "sample": f"{WORKLOADS[args.workload][0].format(n=n)}, {d} DoFs: oracle assembly {ta:.2f}s + "
                      f"1-thread FP64 Jacobi-CG {ts:.2f}s ({it} it)"}


def oracle_reference(prob, reltol: float) -> dict:
    """The CPU baseline and the independent FP64 reference solution of the
    workload, from the oracle alone (nothing of the GPU library): one timed
    cpu_port_step (assembly + FP64 CG to `reltol`), then, untimed, iterative
    refinement of that CG solution with residuals in double-double until the
    correction is below 2 ulp (oracle.solve_refined)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    d, dt, ta, ts, it, A, bb, x = cpu_port_step(prob, reltol)
    t0 = time.perf_counter()
    xr, info = O.solve_refined(A, bb, inner_reltol=1e-6, x0=x)
    info["refine_s"] = time.perf_counter() - t0
    return {"dofs": d, "seconds": dt, "assembly_s": ta, "solve_s": ts, "iterations": it, "x": xr, "info": info}


# the reference arm's timed steps stop once they have taken this long (at least 3 are run)
REFERENCE_TIME_BUDGET_S = 150.0


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    _package()   # host-side mesh / DoF-map code (pure Python; nothing runs on the GPU)
    from grmp_gb300 import problems as P
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    prob = make_problem(P, args, args.seed, args.cpu_n)
    # untimed steps as requested, up to the three the timing rules ask for (CPU code warms
    # up with its first touch of memory; more would only lengthen the run)
    warm = min(args.warmup, 3)
    for _ in range(warm):
        cpu_port_step(prob, args.reltol)
    times, dofs, its = [], 0, 0
    for _ in range(args.steps):
        dofs, dt, _, _, its, _, _, _ = cpu_port_step(prob, args.reltol)
        times.append(dt)
        if len(times) >= 3 and sum(times) > REFERENCE_TIME_BUDGET_S:
            break
    v = dofs / statistics.mean(times)
    same = args.cpu_n == args.n
    line = {"metric": METRIC, "value": v, "unit": "DoF/s", "n_gpus": args.gpus, "steps": len(times),
            "steps_requested": args.steps, "warmup": warm, "warmup_requested": args.warmup,
            "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "impl": "reference",
            "config": {"workload": workload_name(args) + ("" if same else f" (sample: n = {args.cpu_n})"),
                       "ndofs": dofs, "same_config": same, "reltol": args.reltol},
            "cpu_baseline": {"value": v, "unit": "DoF/s", "cores": cores, "kind": "port",
                             "sample": f"{WORKLOADS[args.workload][0].format(n=args.cpu_n)} ({dofs} DoFs): oracle "
                                       f"assembly (reference item loop, rows split over {cores} threads, "
                                       f"bit-identical to one thread) + {cores}-thread FP64 Jacobi-CG to relative "
                                       f"residual {args.reltol:g} ({its} it); steps stop after "
                                       f"{REFERENCE_TIME_BUDGET_S:g} s (Julia reference not runnable here)"},
            "e2e": {"value": v, "unit": "DoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm
# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) of one
# persistent-solver launch on the 48^3 case divided by pcg_bytes() of the
# same launch (summaries under profiles/):
#   k_pcg_mixed (packed pairs, 10408): 180.78 GB / 185.73 GB
#   k_pcg_mixed_duo (two-run 16-bit columns, 60208; 768 iterations, 11
#     refinements): 153.315 GB / 185.260 GB
#   k_pcg_mixed_duo_keep (Jacobi-scaled two-run columns, A p kept on chip,
#     66404, the autotuner's choice at 64^3; 763 iterations, 13
#     refinements): 141.091 GB / 184.752 GB (65208: 138.241 / 185.124)
TRAFFIC_RATIO = {"k_pcg_mixed": (163.612 + 17.166) / 185.732,
                 "k_pcg_mixed_duo": (137.023 + 16.292) / 185.260,
                 "k_pcg_mixed_duo_keep": (131.944 + 9.147) / 184.752}


def duo_family(cfg: int) -> bool:
    """spmv_config reads the two-run 16-bit column copy (60xxx-65xxx grid-wide,
    80xxx one cluster)."""
    return 60000 <= cfg < 70000 or 80000 <= cfg < 90000


def pcg_kernel(cfg: int) -> str:
    if 64000 <= cfg < 67000:
        return "k_pcg_mixed_duo_keep"
    if duo_family(cfg):
        return "k_pcg_mixed_duo"
    if 20000 <= cfg < 40000:
        return "k_pcg_mixed_staged"
    return "k_pcg_mixed"


def pcg_bytes(stats: dict, n: int, nnz: int, mixed: bool) -> float:
    """Algorithmic DRAM bytes of one persistent PCG launch, by the CSR
    definition (int32 column indices) whatever the storage format: per inner
    FP32 iteration the matrix once (4-byte value + 4-byte column per entry)
    and the vector traffic of Jacobi-PCG's update phase (seven 8-byte streams
    per row); per FP64 refinement one FP64 residual.  A format or kernel that
    moves fewer bytes shows as DRAM traffic below these bytes."""
    it, outer = stats["iterations"], stats["outer_iterations"]
    if mixed:
        per_it = 8.0 * nnz + 56.0 * n
        per_outer = 12.0 * nnz + 64.0 * n
        return it * per_it + (outer + 1) * per_outer
    return it * (12.0 * nnz + 108.0 * n) + 2 * (12.0 * nnz + 36.0 * n)


def workload_name(args) -> str:
    return WORKLOADS[args.workload][0].format(n=args.n)


def setup_timings(ctx, FES, prob) -> dict:
    """One-time setup costs, reported beside the per-step numbers (which
    exclude them): the host's mesh generation and dofmap + boundary DoFs
    (the FESpace constructor's role) against the same dofmap and boundary
    DoFs built on the device from the uploaded mesh (grmp_space_create_on_device,
    grmp_space_boundary_dofs; results checked equal to the host's)."""
    from grmp_gb300 import fespace as F
    from grmp_gb300 import mesh as M
    g = FES.xgrid
    out = {}
    n = getattr(prob, "meta", {}).get("n")
    if n:
        t0 = time.perf_counter()
        g2 = M.grid_unitcube_kuhn(n) if g.dim == 3 else M.grid_unitsquare(n)
        out["mesh_host"] = 1e3 * (time.perf_counter() - t0)
    else:
        g2 = type(g)(g.coords, g.cells, name="copy")
    t0 = time.perf_counter()
    H = F.FESpace(FES.FEType, g2)
    fixed_h = H.boundary_dofs()
    out["dofmap_boundary_host"] = 1e3 * (time.perf_counter() - t0)
    t0 = time.perf_counter()
    ctx.mesh(g2)
    out["mesh_upload"] = 1e3 * (time.perf_counter() - t0)
    t0 = time.perf_counter()
    D = ctx.space_on_device(FES.FEType, g2, download=False)
    fixed_d = ctx.boundary_dofs(D)
    out["dofmap_boundary_device"] = 1e3 * (time.perf_counter() - t0)
    cd = np.empty_like(H.celldofs)
    ctx.check(ctx.lib.grmp_space_celldofs(ctx.space(D), cd.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
    if D.ndofs != H.ndofs or not np.array_equal(cd, H.celldofs) or not np.array_equal(fixed_d, fixed_h):
        raise RuntimeError("device dofmap differs from the host's")
    ctx.release(D)
    return out


def run_ours(args):
    dist = Dist()
    G = _package()
    from grmp_gb300 import build as B
    from grmp_gb300 import problems as P
    from grmp_gb300 import _lib as L
    B.build()
    import torch
    dev = dist.local
    torch.cuda.set_device(dev)
    ctx = G.GB300Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)
    prob = make_problem(P, args, args.seed + dist.rank)
    FES = prob.FES
    ndofs = FES.ndofs
    setup_ms = setup_timings(ctx, FES, prob)
    op = prob.operators[0]
    dev_terms = None
    if op.cell_coef is not None:
        # resident inputs: the per-cell coefficient in a device vector (read in place)
        kdev = G.FEVector.__new__(G.FEVector)
        kdev.ctx = ctx
        kdev.h = ctypes.c_void_p()
        ctx.check(ctx.lib.grmp_vector_create(ctx.h, FES.xgrid.ncells, ctypes.byref(kdev.h)))
        kap = np.ascontiguousarray(op.cell_coef, dtype=np.float64)
        ctx.check(ctx.lib.grmp_vector_upload(kdev.h, kap.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        kptr = ctypes.c_void_p()
        ctx.check(ctx.lib.grmp_vector_device_ptr(kdev.h, ctypes.byref(kptr)))
        t = op.term()
        t.cell_coef = ctypes.cast(kptr, ctypes.POINTER(ctypes.c_double))
        t.coef_on_device = 1
        dev_terms = (L.BilinearTerm * 1)(t)
    t0 = time.perf_counter()
    A = G.FEMatrix(ctx, FES, prob.operators)
    setup_ms["pattern_device"] = 1e3 * (time.perf_counter() - t0)
    b = G.FEVector(ctx, FES)
    x = G.FEVector(ctx, FES)
    nnz = A.nnz

    direct = args.solver == "direct"

    def step(mode: str, host_inputs: bool = False):
        # FP32 element matrices feed the FP32 PCG; the FP32 factorisation reads the FP64 values
        needs32 = mode == "mixed" and not direct
        # one walk of the incidence lists fills both precisions when both are needed
        prec = G.FP64_FP32 if needs32 else G.FP64
        if host_inputs:
            G.assemble(A, prob.operators, prec)
        elif dev_terms is not None:
            ctx.check(ctx.lib.grmp_assemble_bilinear(A.h, 1, dev_terms, prec))
        else:   # scalar operator parameters: nothing per cell to upload
            G.assemble(A, prob.operators, prec)
        b.fill(0.0)
        G.assemble(b, prob.rhs)
        G.apply_dirichlet(A, b, prob.fixed, None, G.DIRICHLET_ELIMINATE)
        smode = {"fp64": "direct", "mixed": "mixed_direct"}[mode] if direct else mode
        s = G.GB300PCG(mode=smode, reltol=args.reltol, abstol=0.0, inner_reltol=args.inner_reltol,
                       spmv_config=args.spmv_config if smode == "mixed" else 0)
        st = s.solve(A, b, x)
        out = x.entries if host_inputs else None
        return st, out

    # The error reference: for the PCG workloads the oracle's own FP64 solution
    # (CPU assembly + refined CG, computed at the end, untimed); for the
    # direct-solver workload (near-incompressible elasticity, where Jacobi-CG
    # does not converge) the library's FP64 multifrontal solve with refinement.
    uref, ref_desc = None, None
    if direct:
        G.assemble(A, prob.operators, G.FP64)
        b.fill(0.0)
        G.assemble(b, prob.rhs)
        G.apply_dirichlet(A, b, prob.fixed, None, G.DIRICHLET_ELIMINATE)
        ref = G.GB300PCG(mode="direct", reltol=args.ref_reltol, abstol=0.0, maxiter=200000)
        ref_st = ref.solve(A, b, x, raise_on_error=False)
        uref = x.entries
        ref_desc = f"GPU FP64 multifrontal direct solve, refined to relres {ref_st['final_relres']:.1e}"

    results = {}
    if args.profile:
        # profiling run: the mixed path only, no host-side extras (for ncu)
        for k in range(max(3, args.warmup) + args.steps):
            st, _ = step("mixed")
            # iteration counts let a capture's DRAM bytes be set against the algorithmic bytes
            print(json.dumps({"profile_step": k, "ndofs": ndofs, "nnz": nnz, "iterations": st["iterations"],
                              "outer": st["outer_iterations"], "spmv_config": st["spmv_config"],
                              "algorithmic_bytes": pcg_bytes(st, ndofs, nnz, True)}), flush=True)
        torch.cuda.synchronize()
        ctx.close()
        dist.close()
        return 0
    for mode in ("fp64", "mixed"):
        for _ in range(max(3, args.warmup)):
            step(mode)
        dist.barrier()
        torch.cuda.synchronize()
        clk = ClockSampler(dev) if mode == "mixed" else None
        if clk:
            clk.start()
        l0 = ctypes.c_uint64()
        ctx.check(ctx.lib.grmp_context_launches(ctx.h, ctypes.byref(l0)))
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        stats = []
        t0 = time.perf_counter()
        for k in range(args.steps):
            ev[k][0].record(stream)
            st, _ = step(mode)
            ev[k][1].record(stream)
            stats.append(st)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        dist.barrier()
        l1 = ctypes.c_uint64()
        ctx.check(ctx.lib.grmp_context_launches(ctx.h, ctypes.byref(l1)))
        clocks = clk.stop() if clk else None
        ms = [e[0].elapsed_time(e[1]) for e in ev]
        tot = dist.max(sum(ms) / 1e3)
        results[mode] = {"ms": ms, "total_s": tot, "wall_s": wall, "stats": stats, "u": x.entries,
                         "launches": int(l1.value - l0.value), "clocks": clocks}
    # end-to-end through the host-buffer API (kappa from host, solution back to host)
    for _ in range(max(3, args.warmup)):
        step("mixed", host_inputs=True)
    dist.barrier()
    torch.cuda.synchronize()
    e2e_ms = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step("mixed", host_inputs=True)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_tot = dist.max(sum(e2e_ms) / 1e3)
    dist.barrier()

    mixed, plain = results["mixed"], results["fp64"]
    world_dofs = ndofs * dist.ws * args.steps
    value = world_dofs / mixed["total_s"]
    plain_value = world_dofs / plain["total_s"]
    # roofline of the dominant kernel (persistent mixed PCG)
    st_last = mixed["stats"][-1]
    kb = pcg_bytes(st_last, ndofs, nnz, True)
    kname = pcg_kernel(st_last["spmv_config"])
    kms = statistics.mean([s["solve_ms"] for s in mixed["stats"]])
    achieved = kb / (kms / 1e3) / 1e9
    pk = peaks()
    peak = float(pk["hbm_gbs"]) if pk else 6800.0
    tpab = TRAFFIC_RATIO.get(kname)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": kb * tpab if tpab else None,
                "traffic_source": (f"ncu dram__bytes_read+write of {kname} "
                                   f"on the 48^3 case ({tpab:.3f} x its algorithmic bytes), scaled to this launch"
                                   if tpab else "not captured for this configuration"),
                "kernel": f"{kname} (persistent)",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if pk else "fallback 6800 GB/s"}
    if direct:
        roofline = None   # factorisation-bound (FP32 / FP64 pipes), no HBM roofline line for this solver
    cpu = None
    oracle_info = None
    if dist.rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        cores = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        if direct:
            cprob = make_problem(P, args, args.seed, args.cpu_n)
            d, dt, ta, ts, it, _, _, _ = cpu_port_step(cprob, args.reltol)
        else:
            # the full workload on the host cores: the CPU baseline, and the oracle's solution as the error reference
            ref = oracle_reference(prob, args.reltol)
            d, dt, ta, ts, it = ref["dofs"], ref["seconds"], ref["assembly_s"], ref["solve_s"], ref["iterations"]
            uref = ref["x"]
            oracle_info = ref["info"]
            ref_desc = (f"oracle FP64 (CPU assembly; Jacobi-CG + {oracle_info['refinements']} refinements with "
                        f"double-double residuals; last correction {oracle_info['last_correction']:.1e}, "
                        f"relres {oracle_info['relres']:.1e})")
        cpu = {"value": d / dt, "unit": "DoF/s", "cores": cores, "kind": "port",
               "sample": f"{WORKLOADS[args.workload][0].format(n=args.cpu_n if direct else args.n)}, {d} DoFs: "
                         f"oracle assembly (reference item loop, rows over {cores} threads) {ta:.2f}s + "
                         f"{cores}-thread FP64 Jacobi-CG {ts:.2f}s ({it} it)",
               "single_core": cpu_single_core(P, args)}
    errs = {}
    for mode in ("mixed", "fp64"):
        errs[mode] = (float(np.linalg.norm(results[mode]["u"] - uref) / np.linalg.norm(uref))
                      if uref is not None else None)
    p = sorted(mixed["ms"])
    line = {"metric": METRIC, "value": value, "unit": "DoF/s", "n_gpus": dist.ws, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": statistics.mean(mixed["ms"]), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32-inner/f64-outer", "data": "synthetic (seeded)",
            "config": {"workload": workload_name(args), "ndofs": ndofs, "nnz": nnz,
                       "ncells": FES.xgrid.ncells, "global_batch": dist.ws, "parallelism": f"replicas{dist.ws}",
                       "l2": "inputs larger than L2 (matrix FP64+FP32 > 129 MB)", "reltol": args.reltol,
                       "inner_reltol": args.inner_reltol, "solver": args.solver},
            "latency_ms": {"p50": p[len(p) // 2], "p99": p[min(len(p) - 1, int(0.99 * len(p)))]},
            "rel_err_vs_fp64": {"mixed": errs["mixed"], "plain": errs["fp64"], "reference": ref_desc},
            "plain_fp64": {"value": plain_value, "ms_per_step": statistics.mean(plain["ms"]),
                           "iterations": plain["stats"][-1]["iterations"]},
            "mixed_vs_plain": value / plain_value,
            "solver": {"iterations": st_last["iterations"], "outer": st_last["outer_iterations"],
                       "spmv_config": st_last["spmv_config"], "grid_blocks": st_last["grid_blocks"]},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": world_dofs / e2e_tot, "unit": "DoF/s",
                    "h2d_bytes_per_step": int(sum(o.cell_coef.size * 8 for o in prob.operators
                                                  if o.cell_coef is not None) + prob.rhs.f.params.size * 8),
                    "d2h_bytes_per_step": int(ndofs * 8)},
            "gpu_launches": mixed["launches"],
            "clocks": mixed["clocks"],
            "setup_ms": setup_ms}
    ctx.close()
    if dist.rank == 0 and not args.no_extras and args.workload == "poisson3d":
        # the other configurations, bounded, on the same run's record
        line["configs"] = run_extras(args)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def _timed(stream, fn, steps: int, warmup: int):
    """warmup + steps calls of fn, each step bracketed by CUDA events on the
    library's stream; returns (ms per step, last result)."""
    import torch
    r = None
    for _ in range(warmup):
        r = fn()
    torch.cuda.synchronize()
    ms = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return ms, r


def summary_linear(G, P, prob, modes, reltol: float, steps: int, warmup: int, reference: str, cpu: bool):
    """One LinearProblem in a plain and a mixed solver mode (assembly + rhs +
    Dirichlet + solve per step); errors against the oracle's sparse-direct
    FP64 solve of the penalised system (reference "oracle"), or against the
    library's FP64 multifrontal solve refined to 1e-14 ("gpu_direct", for
    near-incompressible elasticity, whose Jacobi-CG the oracle cannot
    converge and whose sparse-direct solve does not fit the time bound)."""
    import torch
    ctx = G.GB300Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream, device=0)
    sysd = P.DeviceSystem(ctx, prob, mixed=True)
    ndofs = prob.FES.ndofs
    out = {"ndofs": ndofs, "steps": steps, "warmup": warmup, "reltol": reltol}
    sols = {}
    for mode in modes:
        sysd.mixed = mode == "mixed"   # FP32 element matrices only for the FP32 PCG
        solver = G.GB300PCG(mode=mode, reltol=reltol, abstol=0.0)
        ms, st = _timed(stream, lambda: sysd.assemble_and_solve(solver), steps, warmup)
        sols[mode] = sysd.x.entries
        out[mode] = {"value": ndofs / (statistics.mean(ms) / 1e3), "ms_per_step": statistics.mean(ms),
                     "iterations": st["iterations"], "spmv_config": st["spmv_config"],
                     "solve_ms": st["solve_ms"], "grid_blocks": st["grid_blocks"],
                     "us_per_iteration": (1e3 * st["solve_ms"] / st["iterations"]) if st["iterations"] else None}
    plain, mixed = modes
    out["mixed_vs_plain"] = out[mixed]["value"] / out[plain]["value"]
    uref, desc = None, None
    if reference == "gpu_direct":
        sysd.mixed = False
        sysd.assemble_and_solve(G.GB300PCG(mode="direct", reltol=1e-14, abstol=0.0))
        uref, desc = sysd.x.entries, "GPU FP64 multifrontal direct solve refined to 1e-14"
    ctx.close()
    if cpu or reference == "oracle":
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        d, dt, ta, ts, it, A, bb, _ = cpu_port_step(prob, reltol)
        if cpu:
            out["cpu_baseline"] = {"value": d / dt, "unit": "DoF/s", "cores": os.cpu_count() or 1, "kind": "port",
                                   "sample": f"full problem: oracle assembly {ta:.2f}s + FP64 Jacobi-CG {ts:.2f}s"}
        if reference == "oracle":
            uref, desc = O.solve_direct(A, bb), "oracle sparse-direct (SuperLU) FP64 solve of the penalised system"
    out["rel_err_vs_fp64"] = {m: float(np.linalg.norm(sols[m] - uref) / np.linalg.norm(uref)) for m in modes}
    out["rel_err_vs_fp64"]["reference"] = desc
    return out


def run_extras(args) -> dict:
    """Bounded summaries of the other configurations, attached to the
    headline line so that one default run records them: 2D P2 Poisson 128^2
    (FP64 vs mixed PCG), 2D P2 elasticity 256^2 with lambda = 1e3 (FP64 vs
    FP32-factor multifrontal), the 2048-problem batched Stokes solve, and the
    serving loop (Poisson arrivals, then the same requests at saturation in
    mixed and plain FP64 mode).  Each entry records its own wall time."""
    import copy
    G = _package()
    from grmp_gb300 import problems as P
    out = {}
    t0 = time.perf_counter()
    out["poisson2d_P2_128x128"] = summary_linear(G, P, P.poisson2d(128), ("fp64", "mixed"), 1e-11, 5, 3, "oracle",
                                                 True)
    out["poisson2d_P2_128x128"]["wall_s"] = time.perf_counter() - t0
    # which bound: the FP64 values + columns of this matrix (395,265 nonzeros,
    # ~4.7 MB) and its vectors stay in the 129 MB L2 between iterations, so a
    # solver iteration is bounded by its grid-wide synchronisations (three per
    # FP64 iteration, two per mixed one) and the dependent gathers, not by HBM
    out["poisson2d_P2_128x128"]["bound"] = ("latency: L2-resident system; per-iteration time set by the persistent "
                                            "solver's grid barriers and dependent gathers, not by HBM bandwidth")
    t0 = time.perf_counter()
    out["elasticity2d_P2vec_256x256_lambda1e3"] = summary_linear(
        G, P, P.elasticity2d(256, seed=args.seed), ("direct", "mixed_direct"), 1e-12, 3, 3, "gpu_direct", False)
    out["elasticity2d_P2vec_256x256_lambda1e3"]["wall_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    a = copy.copy(args)
    a.workload, a.steps, a.warmup, a.dim, a.nprob = "stokes-batch", 3, 3, 2, 2048
    st = run_stokes(a, emit=False)
    out["stokes_BR_P0_batch2048"] = {k: st[k] for k in ("value", "unit", "ms_per_step", "config", "solver",
                                                        "rel_err_vs_oracle", "cpu_baseline", "latency_ms",
                                                        "mixed_direct", "mixed_vs_plain")}
    out["stokes_BR_P0_batch2048"]["wall_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    a = copy.copy(args)
    a.workload = "serve"
    sv = run_serve(a, emit=False)
    out["serve_64_requests"] = {k: sv[k] for k in ("value", "unit", "config", "latency_ms", "failed", "run_ms_p50",
                                                   "queue_ms_p50", "saturated", "mixed_vs_plain",
                                                   "max_rel_diff_mixed_vs_fp64", "pooled_8_meshes")}
    out["serve_64_requests"]["wall_s"] = time.perf_counter() - t0
    return out


def run_stokes(args, emit: bool = True):
    """Batched gradient-robust Stokes: 2048 BR/P0 problems (8x8 .. 96x96
    squares, nu log-uniform in [1e-4, 1], penalty 1e4), iterated penalty with
    one FP64 multifrontal factorisation per problem; a step = FP64 assembly
    of all problems + reconstructed rhs + Dirichlet + the batched solve.
    The error is measured against the oracle's sparse-direct sweeps on the
    problems the CPU baseline samples."""
    dist = Dist() if emit else Dist.single()
    G = _package()
    from grmp_gb300 import build as B
    from grmp_gb300 import stokes as S
    B.build()
    import torch
    torch.cuda.set_device(dist.local)
    ctx = G.GB300Context(dist.local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dist.local)
    if args.dim == 3:
        # n^3 Kuhn cubes, n log-uniform in [2, 6] (201 to 3,837 velocity DoFs per problem; the
        # per-problem direct solver stages its largest front in shared memory, 969 DoFs at n = 6)
        prob = S.make_batch(nproblems=args.nprob, nmin=2, nmax=6, seed=args.seed + dist.rank, dim=3)
    else:
        prob = S.make_batch(nproblems=args.nprob, seed=args.seed + dist.rank)
    sysd = S.StokesBatchSystem(ctx, prob, mixed=False, direct=True)
    ndofs = prob.V.ndofs + prob.mesh.ncells

    def step():
        sysd.assemble()
        st = sysd.solve(sweeps=args.sweeps, reltol=args.stokes_reltol, maxiter=1, sweep_tol=0.0,
                        raise_on_error=False)
        ctx.check(st["rc"])   # a refused or failed solve ends the run, it is never timed
        return st

    for _ in range(max(3, args.warmup)):
        st = step()
    dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(dist.local)
    clk.start()
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    clocks = clk.stop()
    tot = dist.max(sum(ms) / 1e3)
    value = ndofs * dist.ws * args.steps / tot
    u_direct, p_direct = sysd.velocity().copy(), sysd.pressure().copy()
    # the mixed option: an FP32 factor per problem preconditioning FP64 CG
    # (FP64 factor as the per-problem fallback), one warm-up and one timed step
    sysm = S.StokesBatchSystem(ctx, prob, solver="mixed_direct")
    mixed_line = None
    for rep in range(2):
        sysm.assemble()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        stm = sysm.solve(sweeps=args.sweeps, reltol=args.stokes_reltol, maxiter=1, sweep_tol=0.0,
                         raise_on_error=False)
        e1.record(stream)
        torch.cuda.synchronize()
        ctx.check(stm["rc"])
        mms = e0.elapsed_time(e1)
    um, pm = sysm.velocity(), sysm.pressure()
    ro, co = prob.V.row_offsets, prob.mesh.cell_offsets
    dmax = max(max(np.linalg.norm(um[ro[k]:ro[k + 1]] - u_direct[ro[k]:ro[k + 1]]) /
                   max(np.linalg.norm(u_direct[ro[k]:ro[k + 1]]), 1e-300),
                   np.linalg.norm(pm[co[k]:co[k + 1]] - p_direct[co[k]:co[k + 1]]) /
                   max(np.linalg.norm(p_direct[co[k]:co[k + 1]]), 1e-300)) for k in range(prob.nproblems))
    mixed_line = {"value": ndofs / (mms / 1e3), "ms_per_step": mms, "fp64_fallbacks": stm["fp64_fallbacks"],
                  "cg_iterations_total": int(stm["total_iterations"]), "max_rel_diff_vs_fp64_direct": float(dmax),
                  "solver": "FP32 multifrontal factor per problem preconditioning FP64 CG (FP64 factor fallback)"}
    del sysm
    cpu = None
    if dist.rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        sample = np.argsort(prob.sizes)[::max(1, len(prob.sizes) // 8)][:8]
        t0 = time.perf_counter()
        dd = 0
        uo_s = {}
        for k in sample:
            g = prob.mesh.parts[k]
            uo_s[k] = O.stokes_iterated_penalty(g, prob.nus[k], prob.lam, prob.terms[k], sweeps=args.sweeps)
            dd += (prob.V.row_offsets[k + 1] - prob.V.row_offsets[k]) + g.ncells
        dt = time.perf_counter() - t0
        u_g, p_g = u_direct, p_direct
        eu, ep = [], []
        for k, (uo, po, _) in uo_s.items():
            r0, r1 = prob.V.row_offsets[k], prob.V.row_offsets[k + 1]
            c0, c1 = prob.mesh.cell_offsets[k], prob.mesh.cell_offsets[k + 1]
            eu.append(float(np.linalg.norm(u_g[r0:r1] - uo) / np.linalg.norm(uo)))
            ep.append(float(np.linalg.norm(p_g[c0:c1] - po) / np.linalg.norm(po)))
        err = {"velocity_max": max(eu), "pressure_max": max(ep), "problems": len(eu),
               "nu_range": [float(min(prob.nus[k] for k in uo_s)), float(max(prob.nus[k] for k in uo_s))],
               "reference": f"oracle sparse-direct (SuperLU) iterated-penalty sweeps ({args.sweeps})"}
        cpu = {"value": dd / dt, "unit": "DoF/s", "cores": 1, "kind": "port",
               "sample": f"{len(sample)} problems of the batch (every {max(1, len(prob.sizes) // 8)}th by size), "
                         f"{dd} DoFs: oracle assembly + SuperLU sparse-direct sweeps ({args.sweeps})"}
    p = sorted(ms)
    line = {"metric": "DoF/s batched Stokes assembly+solve (velocity+pressure DoFs)", "value": value,
            "unit": "DoF/s", "n_gpus": dist.ws, "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": statistics.mean(ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"stokes_BR_P0_batch{args.nprob}" + ("_3d" if args.dim == 3 else ""),
                       "velocity_dofs": prob.V.ndofs,
                       "cells": prob.mesh.ncells, "sweeps": args.sweeps, "reltol": args.stokes_reltol,
                       "solver": "FP64 multifrontal Cholesky per problem, factored once per step"},
            "latency_ms": {"p50": p[len(p) // 2], "p99": p[min(len(p) - 1, int(0.99 * len(p)))]},
            "solver": {k: st[k] for k in ("max_iterations", "max_sweeps", "failed", "max_relres", "solve_ms")},
            "mixed_direct": mixed_line,
            "mixed_vs_plain": (mixed_line["value"] / value) if mixed_line else None,
            "rel_err_vs_oracle": err if dist.rank == 0 and not args.no_cpu else None,
            "cpu_baseline": cpu, "clocks": clocks}
    ctx.close()
    if not emit:
        return line
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def run_serve(args, emit: bool = True):
    """Serving loop: Poisson-process arrivals of 2D/3D Poisson and
    reaction-diffusion requests (H1P1/H1P2, 1e3..2e6 DoFs), 4 slots, HBM
    budget 150 GB, mixed-precision solves; DoF/s and p50/p99 latency.  The
    same requests are then submitted all at once in mixed and in plain FP64
    mode (serving capacity of each, and the largest relative difference
    between the two solutions of a request)."""
    dist = Dist() if emit else Dist.single()
    G = _package()
    from grmp_gb300 import build as B
    from grmp_gb300 import serve as SV
    B.build()
    reqs = SV.make_workload(args.nreq, seed=args.seed + dist.rank, mean_interarrival_s=args.interarrival,
                            dofs_max=2e6)
    SV.run(reqs[:4], nslots=args.slots, realtime=False)          # warm-up: module load, pools
    clk = ClockSampler(dist.local)
    clk.start()
    xs, sts, makespan = SV.run(reqs, nslots=args.slots, hbm_budget_bytes=150 << 30, realtime=True)
    clocks = clk.stop()
    summ = SV.summarize(reqs, sts, makespan)
    # capacity: the same requests submitted at once, mixed and plain FP64 serving
    sat = {}
    sols = {}
    for mode in ("mixed", "fp64"):
        xm, sm, mk = SV.run(reqs, nslots=args.slots, hbm_budget_bytes=150 << 30, mode=mode, realtime=False)
        ss = SV.summarize(reqs, sm, mk)
        sat[mode] = {"dof_per_s": ss["dof_per_s"], "makespan_s": mk, "failed": ss["failed"],
                     "latency_ms": ss["latency_ms"]}
        sols[mode] = xm
    rel = [float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)) for a, b in zip(sols["mixed"], sols["fp64"])]
    # pooled: the same number of requests on 8 meshes of 1e3..2e5 DoFs (fresh
    # coefficients and right-hand side each; setup is a large share of such
    # requests), submitted at once with and without residency
    pooled = SV.make_pooled_workload(args.nreq, nmeshes=8, seed=args.seed + 100 + dist.rank, dofs_max=2e5,
                                     device_dofmap=True)
    SV.run(pooled[:2], nslots=args.slots, realtime=False)
    pool = {}
    psol = {}
    for kind, rr in (("resident", pooled), ("cold", [dataclasses.replace(r, mesh_key=0, device_dofmap=False)
                                                     for r in pooled])):
        xp, sp, mk = SV.run(rr, nslots=args.slots, hbm_budget_bytes=150 << 30, realtime=False)
        ss = SV.summarize(rr, sp, mk)
        pool[kind] = {"dof_per_s": ss["dof_per_s"], "makespan_s": mk, "failed": ss["failed"],
                      "latency_ms": ss["latency_ms"], "resident_hits": ss["resident_hits"],
                      "run_ms_p50": float(np.percentile([s["run_ms"] for s in sp], 50))}
        psol[kind] = xp
    pool["meshes"] = 8
    pool["dofs"] = int(sum(r.ndofs for r in pooled))
    pool["resident_vs_cold"] = pool["resident"]["dof_per_s"] / pool["cold"]["dof_per_s"]
    pool["max_rel_diff_vs_cold"] = max(float(np.linalg.norm(a - b) / np.linalg.norm(b))
                                       for a, b in zip(psol["resident"], psol["cold"]))
    line = {"metric": "serving DoF/s and p50/p99 latency (Poisson-process arrivals)", "value": summ["dof_per_s"],
            "unit": "DoF/s", "n_gpus": dist.ws, "steps": 1, "warmup": 1, "ms_per_step": 1e3 * makespan,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32-inner/f64-outer",
            "data": "synthetic (seeded)",
            "config": {"workload": f"serve_{args.nreq}_requests", "slots": args.slots, "hbm_budget_gb": 150,
                       "mean_interarrival_s": args.interarrival, "dofs": summ["dofs"]},
            "latency_ms": summ["latency_ms"], "failed": summ["failed"],
            "run_ms_p50": float(np.percentile([s["run_ms"] for s in sts], 50)),
            "queue_ms_p50": float(np.percentile([s["queue_ms"] for s in sts], 50)),
            "saturated": sat, "mixed_vs_plain": sat["mixed"]["dof_per_s"] / sat["fp64"]["dof_per_s"],
            "max_rel_diff_mixed_vs_fp64": max(rel), "pooled_8_meshes": pool, "clocks": clocks}
    if not emit:
        return line
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=0, help="mesh size (0: the workload's own)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--reltol", type=float, default=0.0, help="solve tolerance (0: the workload's own)")
    ap.add_argument("--ref-reltol", type=float, default=1e-14)
    ap.add_argument("--inner-reltol", type=float, default=0.1)
    ap.add_argument("--spmv-config", type=int, default=0,
                    help="SpMV configuration of the mixed solver (0: autotuned per matrix)")
    ap.add_argument("--cpu-n", type=int, default=0, help="CPU sample mesh size (0: the workload's own)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline only: skip the bounded summaries of the other configurations")
    ap.add_argument("--profile", action="store_true", help="mixed path only, no timing output (for ncu)")
    ap.add_argument("--workload", default="poisson3d",
                    choices=["poisson3d", "poisson2d", "elasticity2d", "stokes-batch", "serve"],
                    help="poisson3d: the headline line; the others print their own lines")
    ap.add_argument("--solver", default="", choices=["", "pcg", "direct"],
                    help="pcg: Jacobi-PCG (plain FP64 / mixed FP32-inner); direct: multifrontal Cholesky "
                         "(plain FP64 / FP32 factor preconditioning FP64 CG); default per workload")
    ap.add_argument("--nprob", type=int, default=2048)
    ap.add_argument("--sweeps", type=int, default=6)
    ap.add_argument("--dim", type=int, default=2, choices=[2, 3], help="stokes-batch: 2D or 3D problems")
    ap.add_argument("--stokes-reltol", type=float, default=1e-12)
    ap.add_argument("--nreq", type=int, default=64)
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--interarrival", type=float, default=0.05)
    args = ap.parse_args()
    if args.workload in WORKLOADS:
        args.n = args.n or WORKLOADS[args.workload][1]
        args.cpu_n = args.cpu_n or WORKLOADS[args.workload][2]
        args.solver = args.solver or ("direct" if args.workload == "elasticity2d" else "pcg")
        args.reltol = args.reltol or WORKLOADS[args.workload][3]
    args.reltol = args.reltol or 1e-11
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "stokes-batch":
        return run_stokes(args)
    if args.workload == "serve":
        return run_serve(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
