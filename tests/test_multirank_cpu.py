"""The N > 1 path of bench.py on the CPU, world size 2 over gloo: the
replica harness (barrier, max over ranks of the timed seconds; only rank 0
prints) and the reference arm under torch.distributed.run (rank 0 alone
runs and prints one line, the other rank exits 0 without work).  The
benchmark's problems are independent replicas, so no collective touches the
data path; these are the only collectives it has."""
import json
import os
import socket
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _torchrun(args, timeout=600):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, OMP_NUM_THREADS="1")
    return subprocess.run(cmd, capture_output=True, text=True, timeout=timeout, cwd=ROOT, env=env)


def test_replica_harness_takes_the_max_over_ranks(tmp_path):
    script = tmp_path / "harness.py"
    script.write_text(textwrap.dedent(f"""
        import json, sys
        sys.path.insert(0, {ROOT!r})
        import bench
        d = bench.Dist()
        d.barrier()
        t = d.max(1.5 + d.rank)          # each rank's own "seconds"
        d.barrier()
        if d.rank == 0:
            print(json.dumps({{"ws": d.ws, "max": t}}), flush=True)
        d.close()
    """))
    out = _torchrun([str(script)], timeout=300)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [json.loads(x) for x in out.stdout.splitlines() if x.startswith("{")]
    assert lines == [{"ws": 2, "max": 2.5}]


def test_reference_arm_under_two_ranks_prints_once():
    pytest.importorskip("scipy")
    out = _torchrun([os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--workload",
                     "poisson2d", "--cpu-n", "8", "--steps", "1", "--warmup", "0"])
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [json.loads(x) for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["value"] > 0
