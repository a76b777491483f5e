"""In-tree build of the native libraries.

Two shared objects are produced inside the package (``teufel_gb300/_lib``):

* ``libteufel_gb300.so`` -- the CUDA field-integration kernels and the C-ABI
  declared in ``include/teufel_cuda.h`` (nvcc, sm_103a only);
* ``libteufel_harness.so`` -- the host-side synthetic trajectory source
  (Vay pusher restatement and seeded bunch sampler, g++/OpenMP).

Everything is compiled with one ``-gencode`` and without cmake so that a
fresh machine builds in well under a minute.  A library is rebuilt when any of
its sources is newer than the output.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
INCLUDE = ROOT / "include"

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

CUDA_LIB = LIBDIR / "libteufel_gb300.so"
HARNESS_LIB = LIBDIR / "libteufel_harness.so"

CU_SOURCES = ["teufel_abi.cu", "teufel_batch.cu", "lw_fp64.cu", "lw_fp32_main.cu",
              "lw_fp32_warp.cu", "lw_fp32_pair.cu", "lw_support.cu", "lw_noalloc.cu",
              "lw_snapshot.cu", "lw_track.cu"]
CU_HEADERS = ["lw_common.cuh", "lw_internal.h", "lw_fp32_point.cuh"]


def _newer(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(map(str, cmd)) + "\n" + r.stdout)
    return r.stdout


def build_harness(force: bool = False) -> Path:
    src = CSRC / "trajgen.cpp"
    LIBDIR.mkdir(exist_ok=True)
    if force or _newer(HARNESS_LIB, [src]):
        tmp = HARNESS_LIB.with_suffix(".so.tmp")
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared",
              "-o", str(tmp), str(src)])
        os.replace(tmp, HARNESS_LIB)
    return HARNESS_LIB


def nvcc_flags(extra=()):
    return [NVCC, GENCODE, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
            "-Xcompiler", "-fPIC,-O3", f"-I{INCLUDE}", f"-I{CSRC}", *extra]


def build_cuda(force: bool = False, verbose_ptxas: bool = False) -> Path:
    LIBDIR.mkdir(exist_ok=True)
    srcs = [CSRC / s for s in CU_SOURCES]
    deps = srcs + [CSRC / h for h in CU_HEADERS] + [INCLUDE / "teufel_cuda.h"]
    if not (force or _newer(CUDA_LIB, deps)):
        return CUDA_LIB
    objdir = LIBDIR / "obj"
    objdir.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []

    def compile_one(s: Path):
        obj = objdir / (s.stem + ".o")
        return _run(nvcc_flags(extra) + ["-c", str(s), "-o", str(obj)]), obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(compile_one, srcs))
    if verbose_ptxas:
        for out, _ in results:
            sys.stdout.write(out)
    tmp = CUDA_LIB.with_suffix(".so.tmp")
    _run([NVCC, GENCODE, "-shared", "-o", str(tmp), *[str(o) for _, o in results]])
    os.replace(tmp, CUDA_LIB)
    return CUDA_LIB


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        futs = [ex.submit(build_cuda, force), ex.submit(build_harness, force)]
        for f in futs:
            f.result()
