"""Build the pphpc_gb300 shared library, the pp_gb300 command-line tool and
the CPU oracle (test infrastructure).

Every CUDA translation unit is compiled for sm_103a only
(`-gencode arch=compute_103a,code=sm_103a`), in parallel, then linked with
the host C code into ``pphpc_gb300/libpphpc_gb300.so`` (CUDA runtime linked
statically). Builds are incremental on file modification times.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpphpc_gb300.so")
CLI = os.path.join(PKG, "pp_gb300")
ORACLE_SRC = os.path.join(ROOT, "oracle", "pp_oracle.c")
ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "libpp_oracle.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                  "-Xcompiler", "-Wall"]
CU_SOURCES = ["pp_kernels.cu", "pp_radix.cu", "pp_world.cu", "pp_serve.cu",
              "pp_noalloc.cu", "pp_fused.cu", "pp_tune.cu", "pp_alloc.cu"]
C_SOURCES = ["pp_host.c"]
HEADERS = ["pp_device.cuh", "pp_kernels.cuh", "pp_block.cuh", "pp_world.cuh",
           "pp_act.cuh"]


_ELF_MACHINE = {"x86_64": 62, "aarch64": 183, "arm64": 183}


def native_ok(path):
    """True if `path` is an ELF file built for this machine's architecture
    (a binary copied from another architecture, or an emptied one, is not)."""
    import platform
    import struct
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    want = _ELF_MACHINE.get(platform.machine())
    return want is None or struct.unpack("<H", head[18:20])[0] == want


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    if target.endswith((".o", ".so")) or os.access(target, os.X_OK):
        if not native_ok(target):
            return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def build_library(verbose=False, extra_nvflags=()):
    os.makedirs(OBJ, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS]
    hdrs.append(os.path.join(ROOT, "include", "pphpc.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        if _newer(o, [s] + hdrs):
            jobs.append([NVCC] + NVFLAGS + list(extra_nvflags) + ["-c", s, "-o", o])
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".c", ".o"))
        objs.append(o)
        if _newer(o, [s] + hdrs):
            jobs.append(["gcc", "-O2", "-std=c11", "-fPIC", "-Wall", "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                sys.stdout.write(out)
    if _newer(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs)
    main_c = os.path.join(CSRC, "pp_main.c")
    if _newer(CLI, [main_c, LIB]):
        _run(["gcc", "-O2", "-std=gnu11", "-Wall", "-o", CLI, main_c,
              "-L" + PKG, "-lpphpc_gb300", "-Wl,-rpath,$ORIGIN"])
    return LIB


ORACLE_LIB_OMP = os.path.join(ROOT, "oracle", "_build", "libpp_oracle_omp.so")


def build_oracle(omp=False):
    """The oracle (test infrastructure); with omp, the same source with its
    independent loops on OpenMP threads (identical results), used only to
    generate the long full-size fixtures."""
    lib = ORACLE_LIB_OMP if omp else ORACLE_LIB
    os.makedirs(os.path.dirname(lib), exist_ok=True)
    hdr = os.path.join(ROOT, "oracle", "pp_oracle.h")
    if _newer(lib, [ORACLE_SRC, hdr]):
        extra = ["-fopenmp", "-DPPO_OMP"] if omp else []
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-Wall"] + extra +
             ["-o", lib, ORACLE_SRC])
    return lib


def build_all(verbose=False):
    lib = build_library(verbose=verbose)
    build_oracle()
    # the reference's own CPU kernels (test and baseline infrastructure),
    # when the reference tree or its preprocessed kernels are present
    sys.path.insert(0, ROOT)
    from oracle.ref import build_ref
    build_ref.build_all()
    return lib


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print(LIB)
