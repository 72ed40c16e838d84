"""Build recipe for libtsqr_gb300.so and the test_tsqr / test_qr command lines.

Everything is compiled in-tree into tsqr_gb300/_build/ with nvcc for sm_103a
only (one -gencode), translation units in parallel.  No CMake, no torch
extension machinery: the library is a plain C-ABI shared object.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
CLI = os.path.join(HERE, "cli")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "libtsqr_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-Xptxas", "-warn-spills"]

SOURCES = ["tsqr.cu", "blocked_qr.cu", "abi.cu", "noalloc.cu", "tc_apply.cu", "tc_gemm.cu", "batched.cu", "check.cu",
           "implicit.cu"]


def nvcc():
    for c in ("/usr/local/cuda/bin/nvcc", shutil.which("nvcc") or ""):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _deps():
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h")):
                out.append(os.path.join(d, f))
    return out


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_lib(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    objs = []
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for s in SOURCES:
            src = os.path.join(CSRC, s)
            obj = os.path.join(BUILD, s.replace(".cu", ".o"))
            objs.append(obj)
            cmd = [nvcc()] + ARCH + NVFLAGS + ["-I", INCLUDE, "-c", src, "-o", obj]
            jobs.append(ex.submit(_run, cmd))
        logs = [j.result() for j in jobs]
    # ptxas's spill report of each unit (-warn-spills), read by the build
    # hygiene test
    for s, l in zip(SOURCES, logs):
        with open(os.path.join(BUILD, s.replace(".cu", ".ptxas.log")), "w") as f:
            f.write(l)
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    tmp = LIB + ".tmp"
    _run([nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs +
         ["-Xlinker", "-rpath,/usr/local/cuda/lib64"])
    os.replace(tmp, LIB)
    return LIB


def build_cli(force=False):
    """test_tsqr / test_qr: the reference's `m n dtype` command lines
    (test_tsqr.cu:112-131, test_qr.cu:112-131) over libtsqr_gb300.so."""
    os.makedirs(BUILD, exist_ok=True)
    outs = []
    if not os.path.isdir(CLI):
        return outs
    for name in ("test_tsqr", "test_qr"):
        src = os.path.join(CLI, "cli_main.cpp")
        out = os.path.join(BUILD, name)
        if force or _stale(out, [src, LIB, os.path.join(INCLUDE, "tsqr_gb300.h")]):
            define = "-DTSQR_CLI_QR=1" if name == "test_qr" else "-DTSQR_CLI_QR=0"
            _run(["g++", "-O2", "-std=c++17", define, "-I", INCLUDE, "-I", "/usr/local/cuda/include", src,
                  "-o", out + ".tmp", "-L", BUILD, "-ltsqr_gb300", "-Wl,-rpath," + BUILD,
                  "-L/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"])
            os.replace(out + ".tmp", out)
        outs.append(out)
    return outs


def build_all(force=False, verbose=False):
    lib = build_lib(force, verbose)
    clis = build_cli(force)
    return {"lib": lib, "cli": clis}


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv, verbose="-v" in sys.argv))
