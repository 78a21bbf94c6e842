"""Build recipes (no cmake): the CUDA library for sm_103a, its serial emulation
build for the CPU test suite, and the test oracles.

Everything is built in-tree:
  parafrost_gb300/_lib/libsigma_gb300.so   product (nvcc, sm_103a)
  parafrost_gb300/_lib/libsigma_emu.so     kernel-logic emulation (g++, CPU tests only)
  oracle/_build/libsigma_oracle.so         CPU restatement (test oracle)
  oracle/_ref/sigma_ref                    compiled reference harness (only where the reference sources exist)
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libsigma_gb300.so")
EMU = os.path.join(LIBDIR, "libsigma_emu.so")
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "libsigma_oracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list, cwd: str = ROOT) -> None:
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}")


def _sources() -> list:
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cu", ".cuh", ".h"))]


def _stale(target: str, deps: list) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_cuda(force: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    deps = _sources() + [os.path.join(ROOT, "include", "sigma_gb300.h")]
    if force or _stale(LIB, deps):
        _run([_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
              os.path.join(CSRC, "sigma.cu"), "-o", LIB + ".tmp"])
        os.replace(LIB + ".tmp", LIB)
    return LIB


def build_emu(force: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    deps = _sources() + [os.path.join(ROOT, "include", "sigma_gb300.h")]
    if force or _stale(EMU, deps):
        _run(["g++", "-x", "c++", "-std=c++17", "-O2", "-DSIGMA_EMU", "-fPIC", "-shared",
              os.path.join(CSRC, "sigma.cu"), "-o", EMU + ".tmp"])
        os.replace(EMU + ".tmp", EMU)
    return EMU


def build_oracle(force: bool = False) -> str:
    src = os.path.join(ROOT, "oracle", "sigma_oracle.cpp")
    deps = [src, os.path.join(ROOT, "oracle", "dump.h"), os.path.join(ROOT, "include", "sigma_gb300.h"),
            os.path.join(CSRC, "introsort.cuh"), os.path.join(CSRC, "device.cuh")]
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    if force or _stale(ORACLE_SO, deps):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", src, "-o", ORACLE_SO + ".tmp"])
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def build_reference(refdir: str | None = None) -> str | None:
    """Compile the reference CPU simplifier harness when the reference sources exist:
    their location is `refdir`, else the PARAFROST_REF environment variable."""
    refdir = refdir or os.environ.get("PARAFROST_REF")
    if not refdir or not os.path.isdir(os.path.join(refdir, "src", "cpu")):
        return None
    _run(["make", "-s", "-f", os.path.join("oracle", "ref.mk"), f"REFDIR={refdir}", f"-j{os.cpu_count() or 4}"])
    return os.path.join(ROOT, "oracle", "_ref", "sigma_ref")


def build_dropin(refdir: str | None = None) -> str | None:
    """Compile the drop-in harness (the reference solver calling this repository's C
    ABI through include/sigma_gb300.hpp, linked to the emulation build) when the
    reference sources exist."""
    refdir = refdir or os.environ.get("PARAFROST_REF")
    if not refdir or not os.path.isdir(os.path.join(refdir, "src", "cpu")):
        return None
    _run(["make", "-s", "-f", os.path.join("oracle", "ref.mk"), f"REFDIR={refdir}", "dropin"])
    return os.path.join(ROOT, "oracle", "_ref", "sigma_dropin")


def build_all(with_cuda: bool = True, refdir: str | None = None) -> dict:
    out = {}
    jobs = {"oracle": build_oracle, "emu": build_emu}
    if with_cuda:
        jobs["cuda"] = build_cuda
    with ThreadPoolExecutor(max_workers=len(jobs) + 1) as ex:
        futs = {k: ex.submit(f) for k, f in jobs.items()}
        ref = ex.submit(build_reference, refdir)
        for k, f in futs.items():
            out[k] = f.result()
        out["reference"] = ref.result()
    out["dropin"] = build_dropin(refdir) if out["reference"] else None
    return out
