"""In-tree build of libsmg (host C++ + sm_103a CUDA), the ClusterSM CLI and the
oracle checker library.  Compiles translation units in parallel, links with
nvcc, and skips units whose object is newer than every input.

    python -m clustersm_gb300.build            # library, CLI, oracle
    SMG_CHECKED=1 python -m clustersm_gb300.build   # self-checking library

The self-checking library (lib_checked/libsmg.so, load it with SMG_LIB_PATH)
bounds-checks the kernels' indexed accesses, records the first violation
(site code and two values, readable with smg_debug_check_join/_filter) and
skips the access instead of making it.
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
INCLUDE = ROOT / "include"
CHECKED = os.environ.get("SMG_CHECKED") == "1"
LIBDIR = PKG / ("lib_checked" if CHECKED else "lib")
BINDIR = PKG / "bin"
OBJDIR = LIBDIR / "obj"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "lib"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SRCS = ["io.cpp", "gen.cpp", "plan.cpp", "serve.cpp"]
CUDA_SRCS = ["api.cu", "filter.cu", "join.cu", "noalloc.cu", "graph_build.cu"]
HEADERS = [INCLUDE / "smg.h"] + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh"))


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _stale(out: Path, inputs) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(i).stat().st_mtime > t for i in inputs if Path(i).exists())


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _compile(src: Path, obj: Path, extra=()):
    if not _stale(obj, [src, *HEADERS]):
        return ""
    obj.parent.mkdir(parents=True, exist_ok=True)
    if src.suffix == ".cu":
        cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-I", str(INCLUDE), "-I", str(CSRC),
               "-Xcompiler", "-fPIC,-fopenmp,-Wall", "--expt-relaxed-constexpr", "-c", str(src),
               "-o", str(obj), *extra]
    else:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-I", str(INCLUDE),
               "-I", str(CSRC), "-I", "/usr/local/cuda/include", "-c", str(src), "-o", str(obj), *extra]
    return _run(cmd)


def build(verbose: bool = False, jobs: int | None = None, ptxas_verbose: bool = False) -> dict:
    """Build everything; returns paths of the produced artefacts."""
    jobs = jobs or max(2, os.cpu_count() or 2)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    BINDIR.mkdir(parents=True, exist_ok=True)
    ORACLE_LIB.mkdir(parents=True, exist_ok=True)
    units = [(CSRC / s, OBJDIR / (s + ".o")) for s in HOST_SRCS + CUDA_SRCS if (CSRC / s).exists()]
    extra_cu = (["-Xptxas", "-v"] if ptxas_verbose else []) + (["-DSMG_CHECKED"] if CHECKED else [])
    logs = []
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(_compile, s, o, extra_cu if s.suffix == ".cu" else ()) for s, o in units]
        futs.append(ex.submit(_build_oracle))
        for f in futs:
            logs.append(f.result())
    lib = LIBDIR / "libsmg.so"
    objs = [o for _, o in units]
    if _stale(lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-Xcompiler", "-fopenmp",
              "-lgomp", "-lcudart"])
    cli_src = CSRC / "cli_main.cpp"
    cli = BINDIR / "ClusterSM"
    if not CHECKED and cli_src.exists() and _stale(cli, [cli_src, lib, *HEADERS]):
        _run(["g++", "-O2", "-std=c++17", "-I", str(INCLUDE), str(cli_src), "-o", str(cli),
              "-L", str(LIBDIR), "-lsmg", "-Wl,-rpath,$ORIGIN/../lib"])
    if verbose:
        for l in logs:
            if l:
                print(l, file=sys.stderr)
    return {"lib": str(lib), "cli": str(cli), "oracle": str(ORACLE_LIB / "liboracle.so"),
            "log": "".join(logs)}


def _build_oracle() -> str:
    src = ORACLE_DIR / "oracle.cpp"
    out = ORACLE_LIB / "liboracle.so"
    if not _stale(out, [src, ORACLE_DIR / "oracle.h", INCLUDE / "smg.h"]):
        return ""
    return _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-Wall", "-I", str(INCLUDE),
                 str(src), "-o", str(out)])


if __name__ == "__main__":
    res = build(verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv)
    print(res["lib"])
    if "--ptxas" in sys.argv:
        print(res["log"])
