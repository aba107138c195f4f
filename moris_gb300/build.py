"""Build libfem_gpu.so in-tree (moris_gb300/_build/) for sm_103a.

Host translation units are compiled with the system C++ compiler, CUDA
translation units with nvcc for ``-gencode arch=compute_103a,code=sm_103a``
only; all compiles run in parallel and the result is linked by nvcc.
Portable host flags only, so that the same recipe builds on x86_64 and on the
aarch64 GPU hosts.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfem_gpu.so")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

HOST_SRCS = ["fem_tables.cpp", "fem_host.cpp", "fem_hmr.cpp", "fem_xtk.cpp", "fem_vis.cpp"]
CUDA_SRCS = ["fem_device.cu", "fem_solver.cu", "fem_probe.cu", "fem_learned_pc.cu", "fem_cluster.cu", "fem_sensitivity.cu",
             "fem_multigrid.cu", "fem_xtk_device.cu", "fem_hmr_device.cu"]
# the device XFEM decomposition reproduces the host's floating-point results,
# which are compiled without contraction
EXTRA_FLAGS = {"fem_xtk_device.cu": ["-fmad=false"]}


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, s) for s in HOST_SRCS + CUDA_SRCS]


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "fem_gpu.h"))
    return hs


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _sources() + _headers() + [__file__])


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I" + os.path.join(os.path.dirname(HERE), "include")]
    jobs = []
    for s in HOST_SRCS:
        o = os.path.join(OUT, s + ".o")
        jobs.append(["g++", "-std=c++17", "-O3", "-fPIC", "-pthread", "-Wall", "-Wextra", "-Wno-unused-parameter",
                     "-ffp-contract=off", *inc, "-c", os.path.join(CSRC, s), "-o", o])
    for s in CUDA_SRCS:
        o = os.path.join(OUT, s + ".o")
        jobs.append([nvcc, GENCODE, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
                     *EXTRA_FLAGS.get(s, []), *inc, "-c", os.path.join(CSRC, s), "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        results = list(ex.map(run, jobs))
    for cmd, r in results:
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("compile failed: " + " ".join(cmd[-3:]))
        if verbose:
            sys.stderr.write(r.stderr)
    objs = [os.path.join(OUT, s + ".o") for s in HOST_SRCS + CUDA_SRCS]
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc, GENCODE, "-shared", "-o", tmp, *objs, "-lpthread"], capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose="-v" in sys.argv))
