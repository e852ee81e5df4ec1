"""bench.py's multi-GPU logic (independent replicas, one per rank) on CPU ranks over
gloo: the timed figure is the slowest rank's, the throughput sums the replicas, and
the reference arm prints from rank 0 only."""
import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest
import torch.multiprocessing as mp

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, torch.device("cpu"))
    out[rank] = (ms, bench.replica_throughput(1000.0, world, ms))
    dist.destroy_process_group()


def test_replicas_report_the_slowest_rank_and_sum_the_work():
    world = 2
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world,
                           start_method="spawn")
        res = dict(out)
    assert res[0] == res[1]
    ms, rate = res[0]
    assert ms == 15.0
    assert rate == pytest.approx(world * 1000.0 / 15e-3)


def test_single_process_keeps_its_own_time():
    assert bench.max_over_ranks(3.5, None, None) == 3.5


def test_reference_arm_prints_on_rank_zero_only(monkeypatch):
    args = type("A", (), dict(workload="deshade_128x128x128", warmup=0, steps=1,
                              ref_sample_iterations=1, gpus=2))()
    monkeypatch.setenv("RANK", "1")
    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference_arm(args) == 0
    assert buf.getvalue() == ""
    monkeypatch.setenv("RANK", "0")
    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference_arm(args) == 0
    line = json.loads(buf.getvalue())
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def test_unknown_extras_are_refused_before_device_work(monkeypatch, capsys):
    """An unknown --extras name stops the bench at argument parsing, before it touches
    a device (this runs on the CPU)."""
    monkeypatch.setattr(sys, "argv", ["bench.py", "--extras", "adjoint,bogus"])
    with pytest.raises(SystemExit) as e:
        bench.main()
    assert e.value.code == 2
    assert "bogus" in capsys.readouterr().err


def test_adjoint_kernel_names_map_to_iteration_kernels(monkeypatch, capsys):
    """--adjoint-kernel picks the context's iteration kernel for the adjoint extras (it
    also picks the reverse sweep's passes); an unknown name stops at argument parsing."""
    import ambient_image_processor_gb300 as pkg
    assert bench.ADJOINT_KERNELS == {"auto": pkg.KERNEL_AUTO, "two_pass": pkg.KERNEL_TWO_PASS,
                                     "shifted": pkg.KERNEL_FUSED_SHIFTED}
    monkeypatch.setattr(sys, "argv", ["bench.py", "--adjoint-kernel", "fused_register"])
    with pytest.raises(SystemExit) as e:
        bench.main()
    assert e.value.code == 2
    assert "adjoint-kernel" in capsys.readouterr().err
