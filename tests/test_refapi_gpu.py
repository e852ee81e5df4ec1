"""The reference-signature C++ layer (libtgvdct_refapi.so) and the terminal program,
called the way the reference's own C++ calls them, against the reference's kernels
(golden fixtures) and the oracle."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from ambient_image_processor_gb300 import build as pkg_build
from conftest import ROOT, load_golden, rel_l2

TOL = 1e-5
CLI = pkg_build.CLI


def write_mha(path, a, element_type="MET_FLOAT", local=True):
    d, h, w = a.shape
    hdr = ("ObjectType = Image\nNDims = 3\nBinaryData = True\nBinaryDataByteOrderMSB = False\n"
           "CompressedData = False\nElementSpacing = 1 1 1\n"
           f"DimSize = {w} {h} {d}\nElementType = {element_type}\n")
    dtype = {"MET_FLOAT": np.float32, "MET_USHORT": np.uint16, "MET_DOUBLE": np.float64}[
        element_type]
    data = np.ascontiguousarray(a, dtype).tobytes()
    if local:
        with open(path, "wb") as fh:
            fh.write((hdr + "ElementDataFile = LOCAL\n").encode() + data)
    else:
        raw = path[:-4] + ".raw"
        with open(path, "w") as fh:
            fh.write(hdr + f"ElementDataFile = {os.path.basename(raw)}\n")
        with open(raw, "wb") as fh:
            fh.write(data)


def read_mha(path):
    with open(path, "rb") as fh:
        blob = fh.read()
    head, _, rest = blob.partition(b"ElementDataFile = LOCAL\n")
    fields = dict(line.split(" = ", 1) for line in head.decode().splitlines() if " = " in line)
    dims = [int(x) for x in fields["DimSize"].split()]
    assert fields["ElementType"] == "MET_FLOAT"
    shape = tuple(reversed(dims))
    return np.frombuffer(rest, np.float32).reshape(shape)


# ---- CPU: argument handling and file reading, no device needed ------------------

def test_cli_usage_and_missing_files(tmp_path):
    if not os.path.exists(CLI):
        pkg_build.build()
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode == 1 and "parameter:" in r.stdout
    r = subprocess.run([CLI, str(tmp_path / "nope.mha"), "1", "2", "1", "10", "16", "u.mha",
                        "l.mha", "r.mha"], capture_output=True, text=True)
    assert r.returncode == 2
    f = np.ones((3, 4, 5), np.float32)
    write_mha(str(tmp_path / "f.mha"), f)
    r = subprocess.run([CLI, str(tmp_path / "f.mha"), "1", "2", "1", "10", "16",
                        str(tmp_path / "nomask.mha"), "u.mha", "l.mha", "r.mha"],
                       capture_output=True, text=True)
    assert r.returncode == 3


# ---- GPU -------------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("element_type,local", [("MET_FLOAT", True), ("MET_USHORT", False),
                                                ("MET_DOUBLE", True)])
def test_cli_deshade_matches_reference(gpu_lib, tmp_path, element_type, local):
    g = load_golden("process3d")
    lam, a0, a1, it = g["params"]
    f = g["f"]
    if element_type == "MET_USHORT":  # integer input: the reference reads it as float too
        f = np.round(f * 1000).astype(np.float32)
    write_mha(str(tmp_path / ("f.mha" if local else "f.mhd")), f, element_type, local)
    src = str(tmp_path / ("f.mha" if local else "f.mhd"))
    outs = [str(tmp_path / n) for n in ("u.mha", "l.mha", "r.mha")]
    r = subprocess.run([CLI, src, repr(float(lam)), repr(float(a0)), repr(float(a1)),
                        str(int(it)), "16", *outs], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    u, l, rr = (read_mha(p) for p in outs)
    if element_type == "MET_USHORT":
        ou, ol, orr = oracle.process_tgv2_l1(f, lam, a0, a1, int(it), dtype=np.float32)
    else:
        ou, ol, orr = g["denoised"], g["shading"], g["deshaded"]
    assert rel_l2(u, ou) < TOL and rel_l2(l, ol) < 1e-4 and rel_l2(rr, orr) < TOL


@pytest.mark.gpu
def test_cli_masked_deshade_matches_oracle(gpu_lib, tmp_path):
    """With a mask the reference program runs the masked processor with clamp and
    background add-back (tgv2_deshade_main.cpp:73-86)."""
    g = load_golden("masked3d_odd")
    lam, a0, a1, it = g["params"]
    write_mha(str(tmp_path / "f.mha"), g["f"])
    write_mha(str(tmp_path / "m.mha"), g["mask"])
    outs = [str(tmp_path / n) for n in ("u.mha", "l.mha", "r.mha")]
    r = subprocess.run([CLI, str(tmp_path / "f.mha"), repr(float(lam)), repr(float(a0)),
                        repr(float(a1)), str(int(it)), "16", str(tmp_path / "m.mha"), *outs],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    u, l, rr = (read_mha(p) for p in outs)
    ou, ol, orr = oracle.process_tgv2_l1_masked(g["f"], g["mask"], lam, a0, a1, int(it),
                                                add_background_back=True, dtype=np.float32)
    assert rel_l2(u, ou) < TOL and rel_l2(l, ol) < 1e-4 and rel_l2(rr, orr) < TOL


@pytest.mark.gpu
def test_reference_signature_templates(gpu_lib, tmp_path):
    """A C++ program using the reference's launcher templates links against
    libtgvdct_refapi.so and gets the reference's results."""
    exe = str(tmp_path / "refapi_driver")
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "refapi_driver.cpp"), "-o", exe,
                        "-L", pkg_build.OUT, "-ltgvdct_refapi", "-ltgvdct",
                        f"-Wl,-rpath,{pkg_build.OUT}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    g = load_golden("masked3d")
    lam, a0, a1, it = g["params"]
    f, mask = g["f"], g["mask"]
    d, h, w = f.shape
    (tmp_path / "in").mkdir()
    (tmp_path / "out").mkdir()
    f.tofile(str(tmp_path / "in" / "f.raw"))
    mask.tofile(str(tmp_path / "in" / "mask.raw"))
    r = subprocess.run([exe, str(tmp_path / "in"), str(tmp_path / "out"), str(w), str(h), str(d),
                        repr(float(lam)), repr(float(a0)), repr(float(a1)), str(int(it))],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    it = int(it)
    assert f"callbacks {(it - 1) // 7} last {7 * ((it - 1) // 7)}" in r.stdout

    def out(name):
        return np.fromfile(str(tmp_path / "out" / (name + ".raw")), np.float32).reshape(f.shape)

    ou, ovx, ovy, ovz = oracle.tgv2_deshade(f, lam, a0, a1, it, dtype=np.float32)
    assert rel_l2(out("u"), ou) < TOL and rel_l2(out("vz"), ovz) < TOL
    assert rel_l2(out("u_double"), ou) < TOL
    assert rel_l2(out("l"), oracle.integrate_poisson_dct(out("vx"), out("vy"), out("vz"))) < 1e-4
    assert rel_l2(out("u_l1"), ou) < TOL
    ou2, *_ = oracle.tgv2_deshade(f, lam, a0, a1, it, data_term="l2", dtype=np.float32)
    assert rel_l2(out("u_l2"), ou2) < TOL
    assert rel_l2(out("u_masked"), g["u"]) < TOL and rel_l2(out("vx_masked"), g["v_x"]) < TOL
