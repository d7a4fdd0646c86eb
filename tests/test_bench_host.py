"""bench.py's multi-rank logic on the CPU (no GPU): two gloo ranks agree on
the slowest rank's time, the whole-job throughput counts every rank's
units against it, and a non-zero rank of the reference arm exits at once
without output (rank 0 alone times and prints the reference)."""
import json
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir, times):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    ms = bench.max_over_ranks(times[rank], world, device="cpu")
    dist.barrier()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"ms": ms}, f)
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    times = [4.5, 6.25]
    mp.start_processes(_rank_main, args=(2, _free_port(), str(tmp_path), times), nprocs=2, join=True,
                       start_method="spawn")
    got = [json.load(open(tmp_path / f"rank{r}.json"))["ms"] for r in range(2)]
    assert got == [6.25, 6.25]
    units_per_rank = 262144
    value = units_per_rank * 2 / (got[0] * 1e-3)  # the value bench.py reports for 2 ranks
    assert value == pytest.approx(2 * 262144 / 6.25e-3)


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(3.5, 1) == 3.5


def test_reference_arm_other_ranks_exit_without_work(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        workload, steps, warmup, gpus = "render", 2, 3, 2

    assert bench.run_reference(Args()) == 0
    assert capsys.readouterr().out == ""
