"""Build the in-tree native libraries.

* ``proteuscfd_gb300/libpcfd.so``: the product (CUDA kernels for sm_103a and the
  C ABI of ``include/pcfd.h``), compiled with nvcc.
* ``oracle/liboracle.so``: the CPU checker used by the tests (plain C, gcc).
* ``oracle/_ref/libref_pin.so``: the reference's own self-contained headers
  (``ucs/matrix.h``, ``ucs/geometry.h``) compiled from their source tree, only
  where that tree is present; it pins the oracle's LU and geometry routines.

Objects are rebuilt only when a source is newer than the output.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "proteuscfd_gb300"
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "libpcfd.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "liboracle.so"
REF_DIR = ORACLE_DIR / "_ref"
REF_LIB = REF_DIR / "libref_pin.so"
# The reference checkout, for the optional reference-side build below; unset: skipped.
REFERENCE_SRC = Path(os.environ["PCFD_REFERENCE_SRC"]) if os.environ.get("PCFD_REFERENCE_SRC") else None

# Host code rounds each operation on its own (no fused multiply-add, which
# aarch64 compilers form by default), as the reference's x86 build does, so
# host preprocessing gives the same bits on both machines.
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpcfd.so")


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run_all(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("build failed: %s\n%s" % (" ".join(map(str, c)), out))


def build_library(verbose: bool = False) -> Path:
    """Compile libpcfd.so (CUDA + host C++) for sm_103a."""
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "pcfd.h"]
    if not _stale(LIB, cu + cpp + headers + [Path(__file__)]):
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    cmds, objs = [], []
    for src in cu:
        obj = BUILD / (src.stem + ".cu.o")
        cmds.append([nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
        objs.append(obj)
    for src in cpp:
        obj = BUILD / (src.stem + ".cpp.o")
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall", "-c",
                     str(src), "-o", str(obj)])
        objs.append(obj)
    _run_all(cmds)
    tmp = LIB.with_suffix(".so.tmp")
    _run_all([[nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *map(str, objs), "-o", str(tmp)]])
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure)."""
    csrcs = [ORACLE_DIR / "oracle.c", ORACLE_DIR / "learned.c", ORACLE_DIR / "chem.c", ORACLE_DIR / "mesh.c"]
    srcs = csrcs + [ORACLE_DIR / "oracle.h", ROOT / "include" / "pcfd.h"]
    if _stale(ORACLE_LIB, srcs + [Path(__file__)]):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        # -ffp-contract=off: every operation rounded on its own, as in the
        # reference's x86 build, on the Arm machine too (whose compiler would
        # otherwise fuse multiply-adds and move the oracle off the reference's bits)
        _run_all([["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off"] + [str(c) for c in csrcs] +
                  ["-o", str(tmp), "-lm"]])
        os.replace(tmp, ORACLE_LIB)
        if verbose:
            print("built", ORACLE_LIB)
    return ORACLE_LIB


def build_ref_pin(verbose: bool = False):
    """Compile the reference's self-contained matrix/geometry headers when
    PCFD_REFERENCE_SRC names a checkout of the reference; skipped otherwise."""
    if REFERENCE_SRC is None:
        if verbose:
            print("PCFD_REFERENCE_SRC unset: reference-side build skipped")
        return None
    ucs = REFERENCE_SRC / "ucs"
    if not (ucs / "matrix.h").exists():
        raise RuntimeError("PCFD_REFERENCE_SRC=%s holds no ucs/matrix.h" % REFERENCE_SRC)
    src = ORACLE_DIR / "ref_pin.cpp"
    deps = [src, ucs / "matrix.h", ucs / "geometry.h"]
    if _stale(REF_LIB, deps):
        REF_DIR.mkdir(exist_ok=True)
        tmp = REF_LIB.with_suffix(".so.tmp")
        _run_all([["g++", "-O0", "-std=c++11", "-fPIC", "-shared", "-I", str(ucs), str(src), "-o", str(tmp)]])
        os.replace(tmp, REF_LIB)
        if verbose:
            print("built", REF_LIB)
    return REF_LIB


def build_all(verbose: bool = False) -> None:
    build_library(verbose)
    build_oracle(verbose)
    build_ref_pin(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
