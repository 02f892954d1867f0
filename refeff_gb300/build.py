"""Build the GB300 FMS library (refeff_gb300/build/librefeff_fms.so) with nvcc.

Every translation unit is compiled for sm_103a only, in parallel, then linked
into one shared library that exports the C ABI of include/refeff_fms.h.
Host code is compiled with -ffp-contract=off so that the cluster preparation
keeps the reference's unfused f32 arithmetic on both x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "build"
LIB = BUILD / "librefeff_fms.so"
SOURCES = ["g0t_build.cu", "batched_lu.cu", "tc_update.cu", "fms_host.cu", "fms_files.cu", "noalloc.cu", "mkgtr.cu", "iterative.cu", "sweeps.cu", "debye.cu", "bicgstab.cu", "precond_mlp.cu", "ff2x.cu", "feff_inp.cu", "autotune.cu", "tc_residual.cu"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def common_flags() -> list[str]:
    return [ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
            "--expt-relaxed-constexpr", f"-I{CSRC}", f"-I{ROOT / 'include'}"]


def _compile(src: Path, obj: Path, verbose: bool) -> None:
    cmd = [nvcc(), *common_flags(), "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "refeff_fms.h"]
    newest = max(p.stat().st_mtime for p in deps)
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    objs = [BUILD / (Path(s).stem + ".o") for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        futs = [ex.submit(_compile, CSRC / s, o, verbose) for s, o in zip(SOURCES, objs)]
        for f in futs:
            f.result()
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
