"""bench.py's JSON-line contract: the reference arm on the host cores, the multi-rank
timing reduction over a gloo process group, and (on a GPU) both ops at small scale."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _run(args, env=None, timeout=600):
    e = dict(os.environ)
    e.update(env or {})
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT, env=e,
                         capture_output=True, text=True, timeout=timeout)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    return [json.loads(l) for l in lines]


@pytest.mark.parametrize("cfg", ["config1", "config4", "config5"])
def test_reference_arm_line(cfg):
    (line,) = _run(["--impl", "reference", "--config", cfg, "--scale", "0.001", "--steps", "2",
                    "--warmup", "1", "--cpu-seconds", "0.5"])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["config"]["op"] == ("upper_bound" if cfg == "config4" else "search_idxs (C++ order)")
    assert "cores" in line["cpu_baseline"] and "sample" in line["cpu_baseline"]


def test_contig_subset_workload_keeps_density():
    """--contigs: configuration 3 on a subset of contigs with its share of intervals and
    queries (the same intervals and hits per query as the full configuration)."""
    import bench
    from superintervals_gb300 import workloads as W
    full = sum(c[1] for c in W.HUMAN_CONTIGS)
    sub = [c for c in W.HUMAN_CONTIGS if c[0] in ("chr21", "chr22")]
    wl = bench.make_workload("config3", 0.01, 0, "chr21,chr22")
    assert len(wl.seg) - 1 == 2
    share = sum(c[1] for c in sub) / full
    assert wl.n == int(50_000_000 * 0.01 * share) and wl.nq == int(50_000_000 * 0.01 * share)
    with pytest.raises(SystemExit):
        bench.make_workload("config3", 0.01, 0, "chr21,chrZ")


def test_reference_arm_two_ranks_prints_once():
    """Under torchrun only rank 0 runs the host baseline and prints; rank 1 exits 0."""
    out = subprocess.run(
        [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
         "--master-addr", "127.0.0.1", "--master-port", "29531", os.path.join(ROOT, "bench.py"),
         "--impl", "reference", "--config", "config1", "--scale", "0.001", "--steps", "1", "--warmup", "1",
         "--cpu-seconds", "0.3", "--gpus", "2"],
        cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1 and json.loads(lines[0])["impl"] == "reference"


def _max_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    q.put((rank, bench.max_over_ranks(10.0 + 5.0 * rank, dist)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_max_worker, args=(r, 2, 29533, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 15.0, 1: 15.0}


def test_ranks_get_their_own_batches():
    import bench
    w0 = bench.make_workload("config3", 0.0002, 0)
    w1 = bench.make_workload("config3", 0.0002, 1)
    assert w0.nq == w1.nq and (w0.starts == w1.starts).all()          # the same index replica
    assert not (w0.q_starts == w1.q_starts).all()                     # a different query batch
    assert sorted(zip(w0.q_starts, w0.q_ends, w0.q_contig)) == sorted(zip(w1.q_starts, w1.q_ends, w1.q_contig))


@pytest.mark.gpu
def test_bench_search_line_gpu():
    (line,) = _run(["--config", "config3", "--scale", "0.01", "--steps", "3", "--warmup", "3",
                    "--cpu-seconds", "0.5"])
    assert line["value"] > 0 and line["gpu_launches"] > 0
    for k in ("roofline", "cpu_baseline", "e2e", "clocks", "plain_gpu"):
        assert k in line, k
    assert 0 < line["roofline"]["frac"] < 2
    assert line["parity_sample_ok"] is True      # the timed result's first queries against the oracle


@pytest.mark.gpu
def test_bench_upper_bound_line_gpu():
    (line,) = _run(["--config", "config4", "--scale", "0.01", "--steps", "3", "--warmup", "3",
                    "--cpu-seconds", "0.5"])
    assert line["oracle_sample_identical"]
    assert all(v["identical_to_binary"] for v in line["providers"].values())
    # the headline is the sorted batch: min/max, keys (which also count the sort's digits), digit
    # offsets, three sort passes, prepare and the scatter back per step; per query it is one
    # kernel per step
    assert line["gpu_launches"] == 3 * 8 and "e2e" in line and "cpu_baseline" in line
    assert line["providers"]["binary"]["path"] == "per_query"
    assert line["providers"]["learned+sorted"]["path"] == "sorted_batch"


@pytest.mark.gpu
def test_bench_serving_line_gpu():
    (line,) = _run(["--config", "config5", "--scale", "0.005", "--requests", "60", "--rate", "2000",
                    "--cpu-seconds", "0.5"])
    assert line["value"] > 0 and line["gpu_launches"] > 0
    assert 0 < line["latency_ms"]["p50"] <= line["latency_ms"]["p99"]
    assert "plain_gpu" in line and "cpu_baseline" in line and "e2e" in line


@pytest.mark.parametrize("op", ["intersect", "difference", "coverage", "keys", "bed_ingest"])
def test_reference_arm_rows(op):
    (line,) = _run(["--impl", "reference", "--op", op, "--scale", "0.002", "--cpu-seconds", "0.3"])
    assert line["impl"] == "reference" and line["value"] > 0 and line["config"]["op"] == op


@pytest.mark.gpu
@pytest.mark.parametrize("op", ["intersect", "difference", "coverage", "keys", "count", "bed_ingest"])
def test_bench_rows_gpu(op):
    (line,) = _run(["--op", op, "--scale", "0.004", "--steps", "2", "--warmup", "1", "--cpu-seconds", "0.3"])
    assert line["value"] > 0 and line["gpu_launches"] > 0 and "cpu_baseline" in line


def test_emit_traffic_figures_match_their_profile():
    """roofline.traffic is the per-unit DRAM traffic of the emit kernel, measured with ncu and
    summarised under profiles/, scaled by the run's pairs and queries: the constants in bench.py
    must be the ones that summary states."""
    import bench
    text = open(os.path.join(ROOT, "profiles", "k_tiles_config3_dram.md")).read()
    assert f"**{bench.EMIT_DRAM_WRITE_PER_PAIR:.3f} B**" in text
    assert f"**{bench.EMIT_DRAM_READ_PER_QUERY:.1f} B**" in text
