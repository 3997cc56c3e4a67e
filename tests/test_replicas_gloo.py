"""The N > 1 path of bench.py (independent replicas, one per rank): the job
time is the max over ranks and the job value counts every rank's nodes.
Two gloo ranks on the CPU."""
import os

import pytest


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(100.0 + 50.0 * rank, dist)
    dist.barrier()
    q.put((rank, t, bench.job_value(1000, 10, world, t)))
    dist.destroy_process_group()


def test_max_over_ranks_and_job_value_two_ranks():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [o[1] for o in out] == [150.0, 150.0]
    assert out[0][2] == pytest.approx(2 * 1000 * 10 / 0.150 / 1e6)


@pytest.mark.parametrize("workload", ["bgk_d3q19_f64_256", "turbulent_d3q27_f32_256",
                                      "entropic_learned_512"])
def test_reference_arm_prints_the_contract_line(workload):
    """`bench.py --impl reference` (the reference's CPU algorithm, the C
    restatement, on the host cores): one JSON line with the arm's metric,
    unit, cpu_baseline and a zero-copy e2e, on CPU."""
    import json
    import subprocess
    import sys
    from conftest import ROOT
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--workload", workload, "--steps", "1", "--warmup", "3", "--grid", "24"],
                       capture_output=True, text=True, timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "MLUPS" and d["value"] > 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"] == {"value": d["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert d["config"]["workload"] == workload and d["config"]["grid"] == [24, 24, 24]
    # a grid other than the workload's is named as the difference
    assert d["config"]["same_config"] is False and "grid 24x24x24" in d["config"]["differences"][0]
    if workload.startswith("entropic"):  # the GPU arm's solver, and one reference-solver step
        assert "residual" in d["config"]["alpha_solver"]
        assert d["reference_alpha_solver"]["value"] > 0
