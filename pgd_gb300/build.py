"""Build recipe for the native library and the `pgd` command line tool.

Compiles every translation unit for sm_103a in parallel and links, in tree:
    pgd_gb300/lib/libpgd_gb300.so   the C-ABI library (include/pgd_gb300.h)
    pgd_gb300/bin/pgd               the drop-in command line tool
No cmake; nvcc and g++ only.  Run as `python -m pgd_gb300.build`.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libpgd_gb300.so")
CLI = os.path.join(BINDIR, "pgd")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home():
    h = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if h and os.path.isdir(h):
        return h
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


CUDA = cuda_home()
NVCC = os.path.join(CUDA, "bin", "nvcc")

CU_SOURCES = ["graph_build.cu", "decompose.cu", "ingest.cu"]
CPP_SOURCES = ["api.cpp", "closing.cpp", "gen.cpp", "serve.cpp"]
CLI_SOURCES = ["graphlet_core.cpp", "pgd_cli.cpp"]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".hpp"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def compile_jobs(verbose_ptxas=False):
    hdrs = _headers()
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        cmd = [NVCC, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC,
               "--expt-relaxed-constexpr", "-c", s, "-o", o]
        if verbose_ptxas:
            cmd.insert(3, "-Xptxas=-v")
        jobs.append((o, [s] + hdrs, cmd))
    for src in CPP_SOURCES + CLI_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I" + INCLUDE, "-I" + CSRC,
               "-I" + os.path.join(CUDA, "include"), "-c", s, "-o", o]
        if src == "closing.cpp":
            cmd.insert(1, "-ffp-contract=off")
        if src == "gen.cpp":
            cmd.insert(1, "-fopenmp")
        jobs.append((o, [s] + hdrs, cmd))
    return jobs


def build(force=False, verbose=False, verbose_ptxas=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    jobs = [(o, deps, cmd) for (o, deps, cmd) in compile_jobs(verbose_ptxas) if force or not _newer(o, deps)]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        outs = list(ex.map(lambda j: _run(j[2]), jobs))
    if verbose:
        for (o, _, cmd), out in zip(jobs, outs):
            print(" ".join(cmd))
            if out.strip():
                print(out)
    lib_objs = [os.path.join(BUILD, s + ".o") for s in CU_SOURCES + CPP_SOURCES]
    if force or not _newer(LIB, lib_objs):
        _run([NVCC, ARCH, "-shared", "-cudart", "shared", "-o", LIB] + lib_objs +
             ["-Xcompiler", "-fopenmp", "-Xlinker", "-rpath," + os.path.join(CUDA, "lib64")])
    cli_objs = [os.path.join(BUILD, s + ".o") for s in CLI_SOURCES]
    if force or not _newer(CLI, cli_objs + [LIB]):
        _run(["g++", "-o", CLI] + cli_objs + ["-L" + LIBDIR, "-lpgd_gb300", "-Wl,-rpath,$ORIGIN/../lib"])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, verbose_ptxas="--ptxas" in sys.argv)
    print("built", LIB, CLI)
