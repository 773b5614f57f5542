"""Build recipes for libgi.so (the product), the CPU oracle and the reference
kernels used as a test oracle.

Everything is compiled in-tree:
  giant-impact_gb300/lib/libgi.so      sm_103a kernels + C ABI (product)
  oracle/libgi_oracle.so               CPU oracle (test infrastructure)
  oracle/_ref/libgiref.so              the reference's own kernels, extracted
                                       from its sources (test infrastructure)
  oracle/_ref/libgirefhost.so          the reference's own host steps, likewise
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
ORACLE = os.path.join(ROOT, "oracle")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["gi_force_pair.cu", "gi_force_ipt1.cu", "gi_force_ipt2.cu", "gi_force_ipt4.cu",
              "gi_force_ipt8.cu",
              "gi_grid.cu", "gi_aux.cu", "gi_api.cu", "gi_noalloc.cu",
              "gi_server.cu", "gi_cluster.cu", "gi_drivers.cu", "gi_splat.cu"]
CPP_SOURCES = ["gi_host.cpp", "gi_formats.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str], log: str | None = None) -> None:
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if log:
        with open(log, "w") as f:
            f.write(" ".join(cmd) + "\n" + p.stdout)
    if p.returncode != 0:
        raise RuntimeError(f"build step failed ({p.returncode}): {' '.join(cmd)}\n{p.stdout[-6000:]}")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, "gi_api.h")]


def host_fma_flags() -> list[str]:
    # fmaf() must be a hardware instruction for the oracle's speed; results
    # do not depend on it (fmaf is correctly rounded either way).
    return ["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []


def build_libgi(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xptxas", "-v", "-I", INCLUDE, "-c", s, "-o", o]
            jobs.append((cmd, os.path.join(BUILD, src + ".log")))
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE,
                   "-c", s, "-o", o]
            jobs.append((cmd, os.path.join(BUILD, src + ".log")))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, c, l) for c, l in jobs]:
            f.result()
    lib = os.path.join(LIBDIR, "libgi.so")
    if force or jobs or _stale(lib, objs):
        _run([nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", lib],
             os.path.join(BUILD, "link.log"))
    return lib


def build_oracle(force: bool = False) -> str:
    src = os.path.join(ORACLE, "gi_oracle.c")
    lib = os.path.join(ORACLE, "libgi_oracle.so")
    if force or _stale(lib, [src, os.path.join(ORACLE, "gi_oracle.h")]):
        _run(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              *host_fma_flags(), src, "-o", lib, "-lm"])
    return lib


def build_ref(force: bool = False) -> str | None:
    """Reference kernels: extracted from the reference sources when they are
    present, then compiled; on a machine without the reference the copy
    extracted earlier (oracle/_ref/*.inc) is compiled."""
    sys.path.insert(0, ORACLE)
    try:
        import build_ref  # oracle/build_ref.py
    finally:
        sys.path.pop(0)
    return build_ref.build(nvcc(), ARCH, force=force)


def build_ref_host(force: bool = False) -> str | None:
    """The reference's own host steps, cut from its sources and compiled for
    the CPU (test infrastructure); None where no cut is available."""
    sys.path.insert(0, ORACLE)
    try:
        import build_ref  # oracle/build_ref.py
    finally:
        sys.path.pop(0)
    return build_ref.build_host(force=force)


def build_all(force: bool = False) -> dict:
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        f_gi = ex.submit(build_libgi, force)
        f_or = ex.submit(build_oracle, force)
        f_ref = ex.submit(build_ref, force)
        f_host = ex.submit(build_ref_host, force)
        return {"libgi": f_gi.result(), "oracle": f_or.result(), "ref": f_ref.result(),
                "ref_host": f_host.result()}


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
