"""bench.py's reference arm (the oracle port timed on the host cores) runs
without a GPU and prints the JSON line the benchmark contract asks for."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("workload,n", [("poisson3d", 6), ("poisson2d", 16), ("elasticity2d", 8)])
def test_reference_arm_prints_contract_line(workload, n):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          workload, "--cpu-n", str(n), "--steps", "1", "--warmup", "0"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_algorithmic_bytes_follow_the_csr_definition():
    """The roofline's algorithmic bytes are Jacobi-PCG's over int32 CSR
    whatever storage format the solver used: the same launch counts the same
    bytes for the packed-pair, two-run-column and row-state configurations."""
    B = _bench_module()
    n, nnz = 1000, 25000
    st = {"iterations": 10, "outer_iterations": 2}
    want = 10 * (8.0 * nnz + 56.0 * n) + 3 * (12.0 * nnz + 64.0 * n)
    for cfg in (10408, 20204, 60208, 65208, 66404, 70204, 80204):
        assert B.pcg_bytes(dict(st, spmv_config=cfg), n, nnz, True) == want
    assert B.pcg_bytes(dict(st, spmv_config=408), n, nnz, False) == 10 * (12.0 * nnz + 108.0 * n) + 2 * (
        12.0 * nnz + 36.0 * n)


def test_roofline_kernel_names_and_traffic_ratios():
    """Each configuration family maps to the persistent kernel it launches,
    and every kernel the benchmark can pick has a captured traffic ratio
    below 1 (it moves no more than the CSR-definition bytes)."""
    B = _bench_module()
    assert B.pcg_kernel(10408) == "k_pcg_mixed"
    assert B.pcg_kernel(20204) == "k_pcg_mixed_staged"
    assert B.pcg_kernel(60208) == "k_pcg_mixed_duo"
    for cfg in (64208, 65208, 66404):
        assert B.pcg_kernel(cfg) == "k_pcg_mixed_duo_keep"
    assert B.pcg_kernel(80204) == "k_pcg_mixed_duo"
    for k in ("k_pcg_mixed", "k_pcg_mixed_duo", "k_pcg_mixed_duo_keep"):
        assert 0.5 < B.TRAFFIC_RATIO[k] < 1.0


def test_single_core_cpu_baseline():
    """The one-core CPU baseline runs the oracle port with one OpenMP thread
    and restores all threads afterwards."""
    import types
    B = _bench_module()
    import grmp_gb300.problems as P
    args = types.SimpleNamespace(workload="poisson3d", seed=0, reltol=1e-11, n=None)
    out = B.cpu_single_core(P, args, n=4)
    assert out["cores"] == 1 and out["value"] > 0 and out["kind"] == "port"
    assert "729 DoFs" in out["sample"]
