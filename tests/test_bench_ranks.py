"""The benchmark's multi-rank host logic on the CPU (two gloo ranks): each
rank drives its own local GPU (replicas, no data-path collective) and the
job's time is the slowest rank's, exchanged as one scalar."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, bench.device(), bench.rank_max(1.5 + rank), bench.dist_env()))
    finally:
        dist.destroy_process_group()


def test_two_ranks_pick_their_gpu_and_share_the_slowest_time():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [0, 1]           # rank i drives local GPU i
    assert [o[2] for o in out] == [2.5, 2.5]       # max over ranks
    assert [o[3] for o in out] == [(0, 0, 2), (1, 1, 2)]


def test_one_rank_needs_no_process_group(monkeypatch):
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    import bench
    assert bench.device() == 0 and bench.rank_max(3.25) == 3.25


def test_reference_arm_line_on_the_cpu():
    # the reference arm times the reference's own kernels built for the CPU,
    # here from the scenario's initial depth (no wet spin-up)
    import json
    import subprocess
    import sys
    from oracle import oracle as O
    if O.ref_lib() is None:
        pytest.skip("reference CPU build unavailable")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "LOCAL_RANK", "WORLD_SIZE")}
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--size", "256", "--steps", "3",
                          "--warmup", "5", "--spinup-s", "0"], cwd=root, env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "reference" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["cells"] == 256 * 256
    assert line["steps"] == 3 and line["warmup"] == 5  # both counts honoured exactly


def test_gpus_flag_spawns_local_ranks_and_prints_one_line():
    # --gpus 2 without a launcher starts two local ranks; rank 0 alone runs
    # the reference arm and prints the one line, the other rank exits 0
    import json
    import subprocess
    import sys
    from oracle import oracle as O
    if O.ref_lib() is None:
        pytest.skip("reference CPU build unavailable")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "LOCAL_RANK", "WORLD_SIZE", "MASTER_PORT")}
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--size", "128",
                          "--steps", "3", "--warmup", "5", "--spinup-s", "0"], cwd=root, env=env,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["n_gpus"] == 2 and line["impl"] == "reference"
    assert line["steps"] == 3 and line["warmup"] == 5


def test_cpu_baseline_falls_back_to_the_port(monkeypatch):
    # without the reference's own CPU build the baseline times the oracle's
    # restatement of its kernels and says so
    import bench
    from oracle import oracle as O
    sc = bench.workload_config2(128)
    if O.ref_lib() is not None:
        v, _, n, kind, _ = bench.cpu_baseline_sample(sc, 3, 1, 2)
        assert kind == "reference" and n == 3 and v > 0
    monkeypatch.setattr(O, "ref_lib", lambda: None)
    v, secs, n, kind, what = bench.cpu_baseline_sample(sc, 3, 1, 2)
    assert kind == "port" and n == 3 and v > 0 and secs > 0 and "restatement" in what


def test_fp32_only_cells_counts_leave_one_out():
    """The conditioning check of the precision report on planted peaks: a
    cell that only the FP32 run moves is FP32-only; a cell that one perturbed
    run alone moves counts against that run in the leave-one-out test."""
    import bench
    shape = (6, 7)
    base = np.zeros(shape)
    res = {"fp64": {"peak": base}}
    for k in ("fp32", "p1", "p2", "p3"):
        res[k] = {"peak": base.copy()}
    res["fp32"]["peak"][0, 0] = 0.005    # FP32 alone
    res["fp32"]["peak"][1, 1] = 0.002    # FP32 and p1
    res["p1"]["peak"][1, 1] = 0.003
    res["p2"]["peak"][2, 2] = 0.004      # p2 alone
    res["p3"]["peak"][3, 3] = 0.0005     # under the tolerance
    out = bench.fp32_only_cells(res, tol=0.001)
    assert out["cells_fp32_over_tol"] == 2 and out["cells_sensitive_union"] == 2
    assert out["cells_fp32_only"] == 1
    assert out["worst_fp32_only"][0] == {"row": 0, "col": 0, "err_m": 0.005, "perturbed_max_err_m": 0.0,
                                         "peak_fp64_m": 0.0}
    p = out["perturbations"]
    assert p["p1"]["own_cells_unexplained_by_the_others"] == 1 and p["p1"]["own_worst_unexplained_m"] == 0.003
    assert p["p1"]["fp32_cells_unexplained_by_the_others"] == 2
    assert p["p2"]["own_cells_unexplained_by_the_others"] == 1 and p["p2"]["own_worst_unexplained_m"] == 0.004
    assert p["p2"]["fp32_cells_unexplained_by_the_others"] == 1
    assert p["p3"]["own_cells_unexplained_by_the_others"] == 0 and p["p3"]["own_worst_unexplained_m"] == 0.0
    assert p["p3"]["fp32_worst_unexplained_m"] == 0.005
    loo = out["leave_one_out"]
    assert loo["perturbed_runs_max"] == 1 and loo["perturbed_worst_m_max"] == 0.004


def test_benchmark_workloads_follow_their_configs():
    """The batched and served legs' synthetic inputs have the shapes the
    workloads name: batched, sides log-uniform in [128, 2048] with a
    three-class Manning raster and 1-6 h of rain; served, sides in
    [256, 4096] with the precision workload's generator (uniform n 0.03,
    5-min gamma hyetograph) and 0.5-6 h durations, scaled as asked."""
    import bench
    b = bench.make_batch_specs(12, 128, 2048, 4)
    assert all(128 <= s["dem"].shape[0] == s["dem"].shape[1] <= 2048 for s in b)
    assert all(set(np.unique(s["manning_classes"])) <= {0, 1, 2} for s in b)
    assert all(len(s["manning_table"]) == 3 and 3600.0 <= s["t_end"] <= 6 * 3600.0 for s in b)
    v = bench.make_served_specs(6, 6, t_scale=0.25)
    assert all(256 <= s["dem"].shape[0] == s["dem"].shape[1] <= 4096 for s in v)
    assert all(s["manning"] == 0.03 and "manning_classes" not in s for s in v)
    assert all(s["dtrain"] == 300.0 and 0.5 * 3600 * 0.25 <= s["t_end"] <= 6 * 3600 * 0.25 for s in v)
    # the plane falls towards the south edge (row 0 is the north row)
    assert all(s["dem"][0].mean() > s["dem"][-1].mean() for s in v)
