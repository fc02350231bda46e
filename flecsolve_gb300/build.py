"""In-tree build of the native parts.

* ``_build/libfsproblems.so`` -- the seeded problem generators (plain C, host
  only, compiled with ``-ffp-contract=off`` so they give the same bits on
  every host).
* ``_build/libfsgpu.so`` -- the CUDA kernels, the device solver loops and the
  C ABI declared in ``include/fsgpu.h``, compiled for sm_103a only.
* ``oracle/`` -- the CPU checker (``make -C oracle``), and the reference
  drivers when the reference library is available: given by the
  ``FLECSOLVE_REF`` environment variable (a flecsolve checkout, which is then
  also staged into the git-ignored ``baseline/_ref``), or already staged
  there.

Everything is compiled directly with gcc / nvcc (no cmake), translation units
in parallel, so a cold build takes about a minute.
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
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr",
              "-I", str(INCLUDE), "-I", str(CSRC)]

CU_SOURCES = ["context.cu", "spmv.cu", "krylov.cu", "gmres.cu", "batched.cu", "blockcg.cu",
              "adjoint.cu", "noalloc.cu", "matrix_market.cu", "nka.cu", "fvm.cu",
              "bdf.cu", "generic.cu", "parcsr.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfsgpu.so")


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(map(str, cmd))}\n{r.stdout}")
    return r.stdout


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_problems(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "libfsproblems.so"
    src = CSRC / "problems.c"
    if force or _stale(out, [src]):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
              "-fno-fast-math", "-o", str(out), str(src), "-lm"])
    return out


def build_gpu(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "libfsgpu.so"
    headers = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    srcs = [CSRC / s for s in CU_SOURCES if (CSRC / s).exists()]
    nvcc = _nvcc()
    objs = []

    def compile_one(src: Path):
        obj = BUILD / (src.stem + ".o")
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            log = _run(cmd)
            if verbose and log:
                sys.stdout.write(log)
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    if force or _stale(out, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(out), *map(str, objs),
              "-lcudart", "-Xcompiler", "-fPIC"])
    return out


def build_cpp_tests(force: bool = False) -> Path:
    """The C++ API test (tests/cpp) against the in-tree libraries."""
    out = BUILD / "test_krylov_api"
    src = ROOT / "tests" / "cpp" / "test_krylov_api.cc"
    deps = [src, INCLUDE / "fsgpu.h", INCLUDE / "flecsolve_gb300" / "flecsolve.hh",
            BUILD / "libfsgpu.so", BUILD / "libfsproblems.so"]
    if force or _stale(out, deps):
        _run(["g++", "-std=c++17", "-O2", "-I", str(INCLUDE), str(src), "-o", str(out),
              "-L", str(BUILD), "-lfsgpu", "-lfsproblems", f"-Wl,-rpath,{BUILD}"])
    return out


def build_template_test(force: bool = False):
    """flecsolve's own solver templates over the device policy
    (tests/cpp/test_flecsolve_templates.cc), built where a flecsolve checkout
    is staged (baseline/_ref); None elsewhere."""
    ref = ROOT / "baseline" / "_ref"
    if not (ref / "flecsolve").is_dir():
        return None
    out = BUILD / "test_flecsolve_templates"
    src = ROOT / "tests" / "cpp" / "test_flecsolve_templates.cc"
    deps = [src, INCLUDE / "fsgpu.h", INCLUDE / "flecsolve_gb300" / "flecsolve_device.hh",
            BUILD / "libfsgpu.so"]
    if force or _stale(out, deps):
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(INCLUDE),
              "-I", str(ROOT / "oracle" / "ref_shim"), "-I", str(ref), str(src), "-o", str(out),
              "-L", str(BUILD), "-lfsgpu", f"-Wl,-rpath,{BUILD}"])
    return out


def build_oracle() -> None:
    oracle = str(ROOT / "oracle")
    ref = os.environ.get("FLECSOLVE_REF")
    if ref:
        _run(["make", "-s", "-C", oracle, "stage", f"REF={Path(ref).resolve()}"])
    _run(["make", "-s", f"-j{max(1, min(8, os.cpu_count() or 1))}", "-C", oracle, "ref"])


def build_all(force: bool = False, verbose: bool = False) -> None:
    build_problems(force)
    build_oracle()
    build_gpu(force, verbose)
    build_cpp_tests(force)
    build_template_test(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print("built", BUILD)
