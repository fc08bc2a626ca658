"""Recipe that builds the reference's own CPU algorithm into oracle/_ref/.

TEST AND BASELINE INFRASTRUCTURE ONLY: the checker side of the statistical
parity tests and the timed CPU baseline. The product never loads it.

The reference's CPU path (opencl/pp/pp_cpu.c + pp_cpu.cl) needs an OpenCL
CPU runtime, cf4ocl2, cl_ops and GLib, none of which exist here, and its
build runs cmake. Its kernels, however, are plain OpenCL C over a handful of
built-ins. This recipe compiles them UNMODIFIED, straight from the
reference tree, as C++ for the host:

  1. preprocess oracle/ref/pp_cpu_kernels.cpp -- ocl_compat.hpp (the
     OpenCL built-ins and the RNG of cl_ops restated for a host), then the
     reference's pp_common.cl and pp_cpu.cl from <reference>/opencl/pp --
     into oracle/_ref/pp_cpu_kernels.ii (needs the reference tree);
  2. compile that translation unit with oracle/ref/pp_cpu_host.cpp (the
     reference host's work sizes and launch loop, with OpenMP threads as
     work items) into oracle/_ref/libpp_cpu_ref.so;
  3. the same with the in-cell shuffle compiled out (-DMAX_AGENT_SHUF=1, the
     reference's own switch) into oracle/_ref/libpp_cpu_ref_noshuf.so, for
     the test that pins the oracle's actions to the reference's step2.

oracle/_ref/ is not committed. Where the reference tree is absent (a GPU
host gets a copy of this working tree without it), step 1 is skipped and the
preprocessed file carried over from the build host is compiled; it includes
no system header, so it compiles on either architecture.

The reference tree's location is $PPHPC_REFERENCE, else /root/reference.

  python oracle/ref/build_ref.py      # prints the library path
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
KERNELS = os.path.join(HERE, "pp_cpu_kernels.cpp")
COMPAT = os.path.join(HERE, "ocl_compat.hpp")
HOST = os.path.join(HERE, "pp_cpu_host.cpp")
II = os.path.join(OUT, "pp_cpu_kernels.ii")
LIB = os.path.join(OUT, "libpp_cpu_ref.so")
# the same kernels with the in-cell shuffle compiled out (MAX_AGENT_SHUF 1,
# the reference's own switch, pp_cpu.cl:640): a cell's list order is then
# its acting order, which the act pin test sets
II_NOSHUF = os.path.join(OUT, "pp_cpu_kernels_noshuf.ii")
LIB_NOSHUF = os.path.join(OUT, "libpp_cpu_ref_noshuf.so")
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall"]


def reference_root():
    return os.environ.get("PPHPC_REFERENCE", "/root/reference")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), p.stdout))


def _build_one(ii, lib, defines):
    from pphpc_gb300.build import native_ok
    src = os.path.join(reference_root(), "opencl", "pp")
    cl = [os.path.join(src, "pp_common.cl"), os.path.join(src, "pp_cpu.cl")]
    if all(os.path.exists(f) for f in cl):
        if _stale(ii, [KERNELS, COMPAT] + cl):
            _run(["g++"] + CXXFLAGS + defines + ["-E", "-P", "-I", src, KERNELS, "-o", ii])
    elif not os.path.exists(ii):
        return None
    if _stale(lib, [ii, HOST]) or not native_ok(lib):
        _run(["g++"] + CXXFLAGS + ["-shared", "-fopenmp", ii, HOST, "-o", lib])
    return lib


def build(noshuf=False):
    """Build oracle/_ref/libpp_cpu_ref.so (or, with noshuf, the variant with
    the in-cell shuffle compiled out); returns its path, or None when
    neither the reference tree nor a preprocessed copy is available."""
    sys.path.insert(0, os.path.dirname(ORACLE))
    os.makedirs(OUT, exist_ok=True)
    if noshuf:
        return _build_one(II_NOSHUF, LIB_NOSHUF, ["-DMAX_AGENT_SHUF=1"])
    return _build_one(II, LIB, [])


def build_all():
    lib = build()
    build(noshuf=True)
    return lib


if __name__ == "__main__":
    print(build_all())
