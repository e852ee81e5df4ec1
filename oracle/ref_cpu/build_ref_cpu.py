"""TEST INFRASTRUCTURE — builds the reference's own TGV-DCT kernels for the CPU.

Recipe: read the reference's unmodified CUDA sources where they lie
(``<reference>/source/modules/{tgv_cuda,tgv_deshade,cuda_image_operations}/*.cu``),
rewrite each kernel launch ``k<<<grid, block>>>(args);`` into
``ref_launch(grid, block, [&]{ k(args); });`` (the only non-C++ syntax they use),
write the rewritten translation units to a temporary directory outside the
repository, and compile them with g++ against ``shim/`` (a host-only stand-in
for the CUDA runtime) together with ``ref_harness.cpp``.  The only output is
``oracle/_ref/libref_cpu.so`` (git-ignored).  Nothing here is product code and
the rewritten sources are deleted after the build.

Usage: python oracle/ref_cpu/build_ref_cpu.py [--reference /path/to/reference]
"""
from __future__ import annotations

import argparse
import os
import re
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT_DIR = os.path.join(ORACLE, "_ref")
# the reference checkout: TGVDCT_REFERENCE_ROOT, else "reference" beside the repository
DEFAULT_REFERENCE = os.environ.get(
    "TGVDCT_REFERENCE_ROOT", os.path.join(os.path.dirname(os.path.dirname(ORACLE)), "reference"))

MODULE_DIRS = ("tgv_cuda", "tgv_deshade", "tgv_deshade_masked", "cuda_image_operations")
# translation units that provide the launchers ref_harness.cpp calls
UNITS = (
    "tgv_deshade/tgv2_l1_deshade.cu",
    "tgv_deshade/tgv2_l1_deshade_2d.cu",
    "tgv_cuda/tgv2_l2.cu",
    "cuda_image_operations/divergence.cu",
    "cuda_image_operations/divergence_2d.cu",
    "cuda_image_operations/cosine_transform.cu",
    "cuda_image_operations/inverse_cosine_transform.cu",
    "cuda_image_operations/solve_poisson_in_cosine_domain.cu",
    "cuda_image_operations/subtract.cu",
    "cuda_image_operations/clamp_negative_values.cu",
    "cuda_image_operations/multiply.cu",
    "cuda_image_operations/add.cu",
    "cuda_image_operations/invert.cu",
    "tgv_deshade_masked/tgv2_l1_deshade_masked.cu",
    "tgv_deshade_masked/tgv2_l1_deshade_masked_2d.cu",
)

_LAUNCH = re.compile(r"\b([A-Za-z_]\w*)\s*<<<(.*?)>>>\s*\(", re.S)


def _matching_paren(text: str, open_idx: int) -> int:
    depth = 0
    for i in range(open_idx, len(text)):
        c = text[i]
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
            if depth == 0:
                return i
    raise ValueError("unbalanced parentheses in kernel launch")


def rewrite_launches(text: str) -> tuple[str, int]:
    out, pos, count = [], 0, 0
    while True:
        m = _LAUNCH.search(text, pos)
        if not m:
            out.append(text[pos:])
            break
        name, cfg = m.group(1), m.group(2)
        open_idx = m.end() - 1
        close_idx = _matching_paren(text, open_idx)
        args = text[open_idx + 1:close_idx]
        out.append(text[pos:m.start()])
        out.append(f"ref_launch({cfg}, [&]() {{ {name}({args}); }})")
        pos = close_idx + 1
        count += 1
    return "".join(out), count


def build(reference: str, jobs: int = 8, verbose: bool = True) -> str:
    modules = os.path.join(reference, "source", "modules")
    if not os.path.isdir(modules):
        raise FileNotFoundError(f"reference sources not found under {modules}")
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = tempfile.mkdtemp(prefix="ref_cpu_")
    try:
        incs = []
        for sub in MODULE_DIRS:
            src_dir = os.path.join(modules, sub)
            dst_dir = os.path.join(tmp, sub)
            os.makedirs(dst_dir)
            incs.append(dst_dir)
            for name in sorted(os.listdir(src_dir)):
                if not name.endswith(".cu"):
                    continue
                with open(os.path.join(src_dir, name), encoding="utf-8") as fh:
                    text, _ = rewrite_launches(fh.read())
                with open(os.path.join(dst_dir, name), "w", encoding="utf-8") as fh:
                    fh.write(text)
        flags = ["-O2", "-std=c++14", "-fPIC", "-ffp-contract=off", "-w", "-x", "c++"]
        inc_flags = ["-I", os.path.join(HERE, "shim")]
        for d in incs:
            inc_flags += ["-I", d]
        objs = []
        cmds = []
        for unit in UNITS:
            obj = os.path.join(tmp, unit.replace("/", "__") + ".o")
            objs.append(obj)
            cmds.append(["g++", *flags, *inc_flags, "-c", os.path.join(tmp, unit), "-o", obj])
        harness_obj = os.path.join(tmp, "ref_harness.o")
        objs.append(harness_obj)
        cmds.append(["g++", "-O2", "-std=c++14", "-fPIC", "-ffp-contract=off",
                     "-I", os.path.join(HERE, "shim"), "-c",
                     os.path.join(HERE, "ref_harness.cpp"), "-o", harness_obj])

        def run(cmd):
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stderr[-4000:])

        with ThreadPoolExecutor(max_workers=jobs) as ex:
            list(ex.map(run, cmds))
        lib = os.path.join(OUT_DIR, "libref_cpu.so")
        run(["g++", "-shared", "-o", lib, *objs])
        if verbose:
            print(f"built {lib}")
        return lib
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=DEFAULT_REFERENCE)
    args = ap.parse_args()
    build(args.reference)
    return 0


if __name__ == "__main__":
    sys.exit(main())
