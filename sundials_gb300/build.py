"""Build recipe for the GB300 library and the test oracle.

* ``sundials_gb300/lib/libsundials_gb300.so`` -- every ``csrc/*.cu`` compiled
  by nvcc for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``),
  one translation unit per process in parallel, linked into one C-ABI
  shared library (static CUDA runtime, hidden symbols except the exported
  ``extern "C"`` API).
* ``oracle/_build/liboracle.so`` -- the C restatements under ``oracle/``
  (test infrastructure), compiled with ``-ffp-contract=off``.
* ``oracle/_ref/libsundials_ref.so`` -- the reference's own serial sources,
  compiled by ``oracle/Makefile`` when they are present on this machine.

Run ``python -m sundials_gb300.build`` (or ``__graft_entry__.build()``).
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
OBJ = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libsundials_gb300.so"
ORACLE = ROOT / "oracle"
ORACLE_LIB = ORACLE / "_build" / "liboracle.so"
REFERENCE_SRC = Path(os.environ.get("SUNGB300_REFERENCE", "/root/reference"))

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
    "-Xcompiler", "-fvisibility=hidden", "-diag-suppress", "177",
    "-I", str(ROOT / "include"),
]


# Extra flags per translation unit: the exact-arithmetic batched integrator
# must not contract products and sums into FMAs.
PER_FILE_FLAGS = {
    "batch_bdf_exact.cu": ["-fmad=false"],
    "sunlinsol_blocklu_gb300.cu": ["-fmad=false"],
    # host-side Givens QR and norm tests rounded like the reference's C
    "sunlinsol_spgmr_gb300.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "heat2d_gb300.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "robertson_gb300.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "bruss3d_gb300.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n"
                           f"{res.stdout}\n{res.stderr}")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_library(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    OBJ.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    sources = sorted(CSRC.glob("*.cu"))
    jobs = []
    for src in sources:
        obj = OBJ / (src.stem + ".o")
        if _stale(obj, [src] + headers):
            jobs.append([nvcc, *NVCC_FLAGS, *PER_FILE_FLAGS.get(src.name, []), "-c", str(src),
                         "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    objs = [OBJ / (s.stem + ".o") for s in sources]
    if jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    srcs = sorted(ORACLE.glob("*_port.c"))
    out = ORACLE_LIB
    out.parent.mkdir(parents=True, exist_ok=True)
    if _stale(out, srcs + list(ORACLE.glob("*.h"))):
        cc = os.environ.get("CC", "gcc")
        _run([cc, "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
              "-o", str(out), *map(str, srcs), "-lm"])
    if verbose:
        print(f"built {out}")
    return out


def build_reference(verbose: bool = False) -> Path | None:
    """Compile the reference's serial path when its sources are on this machine."""
    if not (REFERENCE_SRC / "src" / "cvode" / "cvode.c").exists():
        return None
    jobs = str(os.cpu_count() or 4)
    _run(["make", "-s", "-C", str(ORACLE), f"REF={REFERENCE_SRC}", "-j", jobs, "ref"])
    lib = ORACLE / "_ref" / "libsundials_ref.so"
    if verbose:
        print(f"built {lib}")
    return lib


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_library, verbose), ex.submit(build_oracle, verbose),
                ex.submit(build_reference, verbose)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
