"""Convergence metrics and the alpha search on the GPU against the reference
(golden fixtures from its kernels, float statistics) and the FP64 oracle."""
import os
import subprocess

import numpy as np
import pytest

import ambient_image_processor_gb300 as pkg
import oracle
from ambient_image_processor_gb300 import build as pkg_build
from ambient_image_processor_gb300.phantoms import tissue_phantom_3d
from conftest import load_golden, rel_l2

pytestmark = pytest.mark.gpu

NAMES = ["convergence3d", "convergence3d_mask", "convergence3d_d1"]


@pytest.mark.parametrize("name", NAMES)
def test_convergence_metrics_match_reference(gpu_lib, name):
    """The device sums are FP64 over FP32 shading fields; the reference sums in float.
    Tolerances: measured differences of the FP64 oracle from the reference are
    3e-6 (NCC), 2e-6 (time-TV), 5e-4 and 3e-6 (the two series' TVs)."""
    g = load_golden(name)
    lam, a0, a1, it, interval = g["params"]
    ncc, tv, mt = pkg.convergence_test(g["f"], lam, a0, a1, int(it), int(interval),
                                       mask=g.get("mask"))
    assert len(ncc) == len(g["ncc"])
    assert np.abs(ncc - g["ncc"]).max() < 2e-5
    assert (np.abs(tv - g["time_tv"]) / np.abs(g["time_tv"])).max() < 2e-5
    assert abs(mt[0] - g["metric_tv"][0]) <= 5e-3 * abs(g["metric_tv"][0])
    assert abs(mt[1] - g["metric_tv"][1]) <= 1e-4 * abs(g["metric_tv"][1])


def test_convergence_metrics_match_fp64_oracle(gpu_lib):
    f = tissue_phantom_3d(16, 24, 32, seed=9)
    ncc, tv, mt = pkg.convergence_test(f, 1.0, 2.0, 1.0, 30, 3)
    o_ncc, o_tv, o_mt = oracle.convergence_test(f.astype(np.float64), 1.0, 2.0, 1.0, 30, 3)
    assert len(ncc) == len(o_ncc) == 8  # checks at 3, 6, ..., 27: eight pairs after the first
    assert np.abs(ncc - o_ncc).max() < 1e-5
    assert rel_l2(tv, o_tv) < 1e-5
    assert abs(mt[1] - o_mt[1]) <= 1e-4 * o_mt[1]


def test_convergence_optimization_runs_the_reference_search(gpu_lib):
    """Decade search, ratio search and the final 500-iteration deshade."""
    f = tissue_phantom_3d(12, 20, 24, seed=10)
    a0, a1, u, l, r = pkg.convergence_optimization(f, 1.0)
    assert a1 in [np.float32(10.0 ** -i) for i in range(11)]
    ratios = [1, 1.5, 1.8, 2, 2.2, 2.3, 2.35, 2.4, 2.45]
    assert any(abs(a0 - k * a1) <= 1e-6 * a0 for k in ratios)
    ou, ol, orr = oracle.process_tgv2_l1(f, 1.0, a0, a1, 500, dtype=np.float32)
    assert rel_l2(u, ou) < 1e-4 and rel_l2(r, orr) < 1e-4


def test_convergence_program_writes_the_metric_file(gpu_lib, tmp_path):
    g = load_golden("convergence3d")
    lam, a0, a1, it, _ = g["params"]
    d, h, w = g["f"].shape
    g["f"].tofile(str(tmp_path / "f.raw"))
    out = str(tmp_path / "metric.txt")
    exe = pkg_build.CONVERGENCE_CLI
    assert os.path.exists(exe)
    r = subprocess.run([exe, str(tmp_path / "f.raw"), repr(float(lam)), repr(float(a0)),
                        repr(float(a1)), str(int(it)), out, f"--raw={w}x{h}x{d}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    vals = [float(x) for x in open(out).read().split()]
    assert len(vals) == 2
    assert abs(vals[0] - g["metric_tv"][0]) <= 5e-3 * abs(g["metric_tv"][0])
    assert abs(vals[1] - g["metric_tv"][1]) <= 1e-4 * abs(g["metric_tv"][1])
