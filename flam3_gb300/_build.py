"""Builds libflam3gpu.so in-tree: nvcc for the CUDA kernels (sm_103a only),
gcc for the C host driver, translation units compiled in parallel.

Usage: python -m flam3_gb300._build [--force] [--define NAME ...] [--out PATH]

--define adds a preprocessor macro to the CUDA sources (for example
F3G_FAST_MATH); --out writes the library elsewhere (its objects go to a
sibling build directory), so variants can sit beside the default build and
be loaded with FLAM3GPU_LIB=PATH.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libflam3gpu.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + CSRC,
                     "-I" + os.path.join(ROOT, "include")]
CC_FLAGS = ["-O2", "-std=gnu11", "-ffp-contract=off", "-fPIC", "-Wall", "-Wno-unused-function", "-I" + os.path.join(ROOT, "include"),
            "-I" + CSRC, "-I" + os.path.join(CUDA_HOME, "include")]


def sources():
    cu = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    c = sorted(os.path.join(CSRC, "host", f) for f in os.listdir(os.path.join(CSRC, "host")) if f.endswith(".c"))
    return cu, c


def headers():
    out = []
    for d in (CSRC, os.path.join(CSRC, "host"), os.path.join(ROOT, "include")):
        out += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".cuh"))]
    return out


def _obj(src, bdir=BUILD):
    return os.path.join(bdir, os.path.basename(src) + ".o")


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(force=False, verbose=False, defines=(), out=None):
    lib = out or LIB
    bdir = BUILD if out is None else os.path.splitext(lib)[0] + "_build"
    os.makedirs(bdir, exist_ok=True)
    cu, c = sources()
    hdrs = headers()
    dflags = ["-D" + d for d in defines]
    jobs = []
    for s in cu:
        o = _obj(s, bdir)
        if force or _stale(o, [s] + hdrs):
            jobs.append([NVCC] + NVCC_FLAGS + dflags + ["-c", s, "-o", o])
    for s in c:
        o = _obj(s, bdir)
        if force or _stale(o, [s] + hdrs):
            jobs.append(["gcc"] + CC_FLAGS + dflags + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
            for msg in ex.map(_compile, jobs):
                if verbose and msg:
                    print(msg)
    objs = [_obj(s, bdir) for s in cu + c]
    if force or jobs or _stale(lib, objs):
        tmp = lib + ".tmp"
        _compile([NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lpthread", "-lm"])
        os.replace(tmp, lib)
    return lib


def build_oracle(reference=None):
    """Builds the test oracle (oracle/liboracle.so) and, when `reference`
    (or the FLAM3_REFERENCE environment variable) names a reference source
    tree that exists, oracle/_ref from it.  Test infrastructure only."""
    od = os.path.join(ROOT, "oracle")
    make = shutil.which("make")
    subprocess.run([make, "-C", od, "port", "liboracle_fast.so"], check=True, capture_output=True)
    ref = reference or os.environ.get("FLAM3_REFERENCE")
    if ref and os.path.isfile(os.path.join(ref, "flam3.c")):
        subprocess.run([make, "-C", od, "ref", "REF=" + ref], check=True, capture_output=True)
        if os.path.exists(LIB):
            # the reference's CLIs relinked onto libflam3gpu (the drop-in)
            subprocess.run([make, "-C", od, "dropin", "REF=" + ref], check=True, capture_output=True)


if __name__ == "__main__":
    argv = sys.argv[1:]
    defs = [argv[i + 1] for i, a in enumerate(argv) if a == "--define"]
    outp = [argv[i + 1] for i, a in enumerate(argv) if a == "--out"]
    print(build(force="--force" in argv, verbose=True, defines=defs, out=os.path.abspath(outp[0]) if outp else None))
