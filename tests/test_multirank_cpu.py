"""The multi-rank path of bench.py on the CPU (gloo, world size 2): shots are
independent, so ranks share nothing but a barrier and the max of their timed
regions; and the reference arm under torchrun prints one line, from rank 0."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        bench.barrier(dist)
        q.put((rank, bench.max_over_ranks(dist, 1.5 + rank)))
        bench.barrier(dist)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 2.5, 1: 2.5}


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--grid", "24x24x24", "--nt", "20", "--cpu-sample-steps", "2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"


def test_reference_arm_loads_no_product_library():
    """The reference arm builds its survey, random boundary, sinc tables and
    source stencil from the oracle: libsepx.so is never mapped and no module
    of the product that binds it is imported."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', "
            "'--warmup', '0', '--grid', '24x24x24', '--nt', '20', '--cpu-sample-steps', '2']; "
            "runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPPED', 'libsepx.so' in maps, 'libsepx_oracle.so' in maps); "
            "print('MODS', sorted(m for m in sys.modules if m.startswith('sep_code_gb300')))")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = r.stdout.splitlines()
    assert "MAPPED False True" in out, r.stdout
    mods = [ln for ln in out if ln.startswith("MODS")][0]
    assert "_lib" not in mods and "gpu_funcs" not in mods and "model" not in mods.replace(
        "sep_code_gb300.surveys", ""), mods
    line = json.loads([ln for ln in out if ln.startswith("{")][0])
    assert line["impl"] == "reference" and line["config"]["padded_grid"]
