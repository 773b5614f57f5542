"""Recipe: build the reference's own force/move kernels as a test oracle.

TEST INFRASTRUCTURE.  The reference's drivers include GLUT/OpenGL headers and
link -lGL, so the whole files are never compiled.  Instead the kernels and
their constant structs are cut out of the reference sources, where they lie,
by line range:

  Code/ImpactCode/impactAddTime.cu                         3-28, 245-394
  Code/GenerateTargetImpactorCode/generateTargetImpactor.cu 2-31, 486-664

into oracle/_ref/*.inc (git-ignored; never committed), and compiled together
with oracle/ref_launch.cu (extern "C" launchers written for this project)
for sm_103a with the reference's optimisation level (-O3, no fast math)
into oracle/_ref/libgiref.so.

The reference's host steps of building and setting up an impact are cut the
same way and compiled for the CPU with oracle/ref_host.cpp (the globals and
vector types they use, and extern "C" entry points) into
oracle/_ref/libgirefhost.so:

  Code/GenerateTargetImpactorCode/generateTargetImpactorBasicFunctions.h
      29-237 (centre of mass, radius, mean velocity, angular momentum),
      407-506 (spinBody, zeroOutTargetImpactorDrift)
  Code/ImpactCode/impactInitialization.cu
      183-391 (readImpactSetupParameters, setupInitialConditions)  Each cut is checked against the lines it must
start and end with, so a moved line range fails loudly instead of compiling
the wrong code.  Where the reference is absent (the GPU host), the cuts made
earlier are compiled as they are.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# Where the reference checkout lies: GI_REFERENCE_DIR, else the location of
# the read-only checkout on the build machine.  Machines without it (the GPU
# host) compile the cuts made earlier.
REFERENCE = os.environ.get("GI_REFERENCE_DIR", "/root/reference")


def reference_dir() -> str | None:
    """The reference checkout, or None where it is absent."""
    return REFERENCE if os.path.isdir(REFERENCE) else None

# (source, first line, last line, expected text at first kernel/struct line, output)
CUTS = [
    ("Code/ImpactCode/impactAddTime.cu", 3, 28,
     {4: "struct forceCollisionKernalConstantsStruct", 22: "struct moveCollisionKernalConstantsStruct"},
     "ref_impact_structs.inc"),
    ("Code/ImpactCode/impactAddTime.cu", 245, 394,
     {245: "__global__ void getForcesCollisionSingleGPU", 379: "__global__ void moveBodiesCollisionSingleGPU"},
     "ref_impact_kernels.inc"),
    ("Code/GenerateTargetImpactorCode/generateTargetImpactor.cu", 2, 31,
     {3: "struct forceSeperateKernalConstantsStruct", 23: "struct moveSeperateKernalConstantsStruct"},
     "ref_generate_structs.inc"),
    ("Code/GenerateTargetImpactorCode/generateTargetImpactor.cu", 486, 664,
     {486: "__global__ void getForcesSeperate", 628: "__global__ void moveBodiesDampedSeperate"},
     "ref_generate_kernels.inc"),
]


HOST_CUTS = [
    ("Code/GenerateTargetImpactorCode/generateTargetImpactorBasicFunctions.h", 29, 237,
     {29: "double4 getCenterOfMass(int scope)"}, "ref_generate_getters.inc"),
    ("Code/GenerateTargetImpactorCode/generateTargetImpactorBasicFunctions.h", 407, 506,
     {407: "void spinBody(int bodyId, float4 spinVector)", 472: "void zeroOutTargetImpactorDrift()"},
     "ref_generate_spin_drift.inc"),
    ("Code/ImpactCode/impactInitialization.cu", 183, 391,
     {183: "void readImpactSetupParameters()", 260: "void setupInitialConditions()"},
     "ref_impact_setup.inc"),
]


def extract() -> bool:
    if not os.path.isdir(REFERENCE):
        return False
    os.makedirs(OUT, exist_ok=True)
    for rel, a, b, expect, out in CUTS + HOST_CUTS:
        with open(os.path.join(REFERENCE, rel), encoding="latin-1") as f:
            lines = f.read().split("\n")
        for ln, text in expect.items():
            if not lines[ln - 1].lstrip().startswith(text):
                raise RuntimeError(f"{rel}:{ln} is not '{text}' -- reference line ranges moved")
        if not lines[b - 1].strip().startswith("}"):
            raise RuntimeError(f"{rel}:{b} does not close a block")
        body = "\n".join(lines[a - 1:b]) + "\n"
        with open(os.path.join(OUT, out), "w") as f:
            f.write(f"// cut from {rel}:{a}-{b} at build time; not part of the repository\n")
            f.write(f"#line {a} \"{rel}\"\n")
            f.write(body)
    return True


def build(nvcc: str, arch: list[str], force: bool = False) -> str | None:
    extract()
    incs = [os.path.join(OUT, c[4]) for c in CUTS]
    if not all(os.path.exists(p) for p in incs):
        return None
    src = os.path.join(HERE, "ref_launch.cu")
    lib = os.path.join(OUT, "libgiref.so")
    deps = incs + [src]
    if not force and os.path.exists(lib) and all(os.path.getmtime(d) <= os.path.getmtime(lib) for d in deps):
        return lib
    cmd = [nvcc, *arch, "-O3", "-shared", "-Xcompiler", "-fPIC", "-I", OUT, src, "-o", lib]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    with open(os.path.join(OUT, "build.log"), "w") as f:
        f.write(" ".join(cmd) + "\n" + p.stdout)
    if p.returncode != 0:
        raise RuntimeError("reference kernel build failed:\n" + p.stdout[-4000:])
    return lib


def build_host(force: bool = False) -> str | None:
    """The reference's host steps (HOST_CUTS) with oracle/ref_host.cpp, for the
    CPU, without FMA contraction (the reference's host code is compiled for
    x86-64, where it has none)."""
    extract()
    incs = [os.path.join(OUT, c[4]) for c in HOST_CUTS]
    if not all(os.path.exists(p) for p in incs):
        return None
    src = os.path.join(HERE, "ref_host.cpp")
    lib = os.path.join(OUT, "libgirefhost.so")
    deps = incs + [src]
    if not force and os.path.exists(lib) and all(os.path.getmtime(d) <= os.path.getmtime(lib) for d in deps):
        return lib
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-I", OUT,
           src, "-o", lib]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    with open(os.path.join(OUT, "build_host.log"), "w") as f:
        f.write(" ".join(cmd) + "\n" + p.stdout)
    if p.returncode != 0:
        raise RuntimeError("reference host build failed:\n" + p.stdout[-4000:])
    return lib


if __name__ == "__main__":
    import shutil
    print(build(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc",
                ["-gencode", "arch=compute_103a,code=sm_103a"], force=True))
