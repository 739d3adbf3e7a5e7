"""In-tree build of libb2g.so (sm_103a) and of the test oracles.

    python box2d-optimized_gb300/build.py          # engine + oracle (+ reference oracle if present)

Translation units compile in parallel: the CUDA sources with nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), the host sources with nvcc's host compiler.
Float contraction is disabled on both sides (``--fmad=false``, ``-ffp-contract=off``) so that
the device arithmetic rounds exactly like a CPU evaluation of the same formulas.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libb2g.so"
# The reference checkout the test oracle oracle/_ref is compiled from: B2G_REF_ROOT, else a
# `reference` directory beside this repository; skipped when neither holds its sources.
REF_SOURCES = Path(os.environ.get("B2G_REF_ROOT") or (ROOT.parent / "reference"))

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off",
              f"-I{ROOT / 'include'}", f"-I{PKG / 'include'}"]
CU_SOURCES = ["solve.cu", "solve_wide.cu", "solve_cluster.cu", "kernels.cu", "compact.cu", "query.cu", "engine.cu", "pairs.cu", "toi.cu"]
CPP_SOURCES = ["shapes.cpp", "facade.cpp", "server.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run_parallel(cmds: list[list[str]]) -> None:
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out.decode(errors="replace")))
    if failed:
        msg = "\n\n".join(f"$ {' '.join(c)}\n{o}" for c, o in failed)
        raise RuntimeError(f"build failed:\n{msg}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build_engine(force: bool = False) -> Path:
    nvcc = _nvcc()
    OUT.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "b2g_capi.h",
               PKG / "include" / "box2d" / "box2d.h", PKG / "scenes" / "scenes.h",
               PKG / "scenes" / "scenes_joints.h"]
    cmds, objs = [], []
    for src in CU_SOURCES + CPP_SOURCES:
        obj = OUT / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            if src.endswith(".cu"):
                cmds.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
            else:
                cmds.append([nvcc, "-x", "c++", *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)])
    if cmds:
        _run_parallel(cmds)
    if force or cmds or _stale(LIB, objs):
        _run_parallel([[nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]])
    return LIB


def build_oracle() -> None:
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    if (REF_SOURCES / "src" / "dynamics" / "b2_world.cpp").exists():
        subprocess.run(["make", "-s", "-j8", "-C", str(ROOT / "oracle"), "ref", f"REF_ROOT={REF_SOURCES}"],
                       check=True)


def build(force: bool = False) -> None:
    build_engine(force)
    build_oracle()


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(LIB)
