"""Builds libtgvdct.so (the C-ABI library) and the terminal programs for sm_103a.

Every CUDA translation unit is compiled by nvcc for ``sm_103a`` only, in
parallel, then linked into ``ambient_image_processor_gb300/_build/libtgvdct.so``.
No cmake, no torch extension machinery: the library exposes plain ``extern "C"``
symbols declared in ``include/tgvdct.h``.  On top of it, g++ builds the host-only
reference-signature layer ``libtgvdct_refapi.so`` (``include/tgvdct_reference_api.hpp``)
and the terminal programs ``tgv2_deshade_application``,
``tgv2_deshade_convergence_test_application`` and
``tgvk_deshade_downsampled_application``.

    python -m ambient_image_processor_gb300.build
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libtgvdct.so")
REFAPI = os.path.join(PKG, "refapi")
REFAPI_LIB = os.path.join(OUT, "libtgvdct_refapi.so")
OUT_CHECKED = os.path.join(PKG, "_build_checked")
LIB_CHECKED = os.path.join(OUT_CHECKED, "libtgvdct_checked.so")
CLI = os.path.join(OUT, "tgv2_deshade_application")
CONVERGENCE_CLI = os.path.join(OUT, "tgv2_deshade_convergence_test_application")
DOWNSAMPLED_CLI = os.path.join(OUT, "tgvk_deshade_downsampled_application")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
               "--expt-relaxed-constexpr"]

# translation unit -> extra flags
UNITS = {
    # -fmad=false keeps the reference's rounding sequence: only the explicit
    # __fmaf_rn calls (the reference's fmaf) fuse.
    "tgv_kernels.cu": ["-fmad=false"],
    "dct_kernels.cu": [],
    "capi.cu": [],
    "noalloc.cu": [],
    "dct_tc.cu": [],
    "dct_tc2.cu": [],
    "metrics.cu": [],
    # the adjoint recomputes forward predicates (prox branch, projection activity)
    # and must round exactly like tgv_kernels.cu
    "adjoint.cu": ["-fmad=false"],
    # the FP64 resize follows ITK's operation sequence, on the device and in its host
    # tables (g++ contracts a*b+c into FMA on aarch64 unless told not to)
    "resize.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout[-4000:]
                           + r.stderr[-8000:])
    return r


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, jobs: int = 8,
          checked: bool = False) -> str:
    """Compile libtgvdct.so and the host tools; with checked=True, instead compile
    libtgvdct_checked.so (kernels with bounds checks, -DTGV_CHECK_BOUNDS) into
    _build_checked/."""
    out = OUT_CHECKED if checked else OUT
    lib = LIB_CHECKED if checked else LIB
    os.makedirs(out, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "tgvdct.h"))
    objs, cmds = [], []
    for unit, extra in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(out, unit + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers, __file__]):
            flags = [*extra, "-DTGV_CHECK_BOUNDS"] if checked else extra
            cmds.append([nvcc(), *ARCH, *NVCC_COMMON, *flags, "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        for r in ex.map(_run, cmds):
            if verbose and r.stderr:
                print(r.stderr)
    if force or cmds or _stale(lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", lib, *objs])
    if not checked:
        build_host(force)
    return lib


def build_host(force: bool = False) -> None:
    """The host-only C++ on top of libtgvdct.so (portable flags: x86_64 and aarch64)."""
    cxx = os.environ.get("CXX", "g++")
    flags = ["-O2", "-std=c++17", "-Wall", "-Wextra", "-I", INCLUDE, "-I", REFAPI]
    link = ["-L", OUT, "-ltgvdct", "-Wl,-rpath,$ORIGIN"]
    hdrs = [os.path.join(INCLUDE, "tgvdct.h"), os.path.join(INCLUDE, "tgvdct_reference_api.hpp"),
            os.path.join(REFAPI, "metaimage.hpp"), __file__]
    api_src = [os.path.join(REFAPI, "reference_api.cpp")]
    if force or _stale(REFAPI_LIB, [*api_src, *hdrs, LIB]):
        _run([cxx, *flags, "-fPIC", "-shared", "-o", REFAPI_LIB, *api_src, *link])
    cli_src = [os.path.join(REFAPI, "tgv2_deshade_main.cpp"), os.path.join(REFAPI, "metaimage.cpp")]
    if force or _stale(CLI, [*cli_src, *hdrs, LIB]):
        _run([cxx, *flags, "-o", CLI, *cli_src, *link])
    conv_src = [os.path.join(REFAPI, "tgv2_deshade_convergence_test_main.cpp"),
                os.path.join(REFAPI, "metaimage.cpp")]
    if force or _stale(CONVERGENCE_CLI, [*conv_src, *hdrs, LIB]):
        _run([cxx, *flags, "-o", CONVERGENCE_CLI, *conv_src, *link])
    ds_src = [os.path.join(REFAPI, "tgvk_deshade_downsampled_main.cpp"),
              os.path.join(REFAPI, "metaimage.cpp")]
    if force or _stale(DOWNSAMPLED_CLI, [*ds_src, *hdrs, LIB]):
        _run([cxx, *flags, "-o", DOWNSAMPLED_CLI, *ds_src, *link])


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
