"""Builds the in-tree shared objects.

    liblp_gpu.so     CUDA kernels + C ABI (sm_103a only)        lidar-processing-v2_gb300/csrc/*.cu
    liblp_synth.so   seeded synthetic scan generator (host)      lidar-processing-v2_gb300/csrc/lp_synth.cpp
    oracle/liblp_oracle.so   CPU parity oracle (test infrastructure)
    oracle/_ref/libref.so    reference sources + stand-in headers (only where the reference tree exists)

Translation units compile in parallel; objects go to lidar-processing-v2_gb300/_build/.
Device code uses --fmad=false and host code -ffp-contract=off so that no multiply-add is
contracted anywhere on the exact-arithmetic path.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(REPO, "include")

CUDA_TUS = ["lp_common.cu", "lp_segment.cu", "lp_cluster.cu", "lp_hull.cu", "lp_dror.cu", "lp_kdtree.cu", "lp_api.cu",
            "lp_serve.cu", "lp_io.cu", "lp_split.cu", "lp_wire.cu", "lp_objects.cu", "lp_tune.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_gpu(verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    flags = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                    "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC]
    if ptxas_info:
        flags += ["-Xptxas", "-v"]
    objs, jobs = [], []
    for tu in CUDA_TUS:
        src = os.path.join(CSRC, tu)
        obj = os.path.join(BUILD, tu.replace(".cu", ".o"))
        objs.append(obj)
        if ptxas_info or _stale(obj, [src] + headers):
            jobs.append([nvcc()] + flags + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            print(o)
    lib = os.path.join(HERE, "liblp_gpu.so")
    if _stale(lib, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", lib] + objs)
    return lib


def build_example():
    """C++ drop-in example (cpp/example_processor.cpp) linked against liblp_gpu.so."""
    src = os.path.join(HERE, "cpp", "example_processor.cpp")
    hdr = os.path.join(HERE, "cpp", "lidar_processing_gpu.hpp")
    exe = os.path.join(HERE, "example_processor")
    lib = os.path.join(HERE, "liblp_gpu.so")
    if _stale(exe, [src, hdr, lib]):
        _run(["g++", "-std=c++17", "-O2", "-I" + INCLUDE, "-I" + os.path.join(HERE, "cpp"), src, "-o", exe,
              "-L" + HERE, "-llp_gpu", "-Wl,-rpath," + HERE])
    return exe


def build_synth():
    src = os.path.join(CSRC, "lp_synth.cpp")
    lib = os.path.join(HERE, "liblp_synth.so")
    if _stale(lib, [src]):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", src, "-o", lib])
    return lib


def build_oracle():
    src = os.path.join(REPO, "oracle", "lp_oracle.cpp")
    lib = os.path.join(REPO, "oracle", "liblp_oracle.so")
    headers = [os.path.join(REPO, "oracle", f) for f in ("eigen_svd2.h", "introsort.h")]
    if _stale(lib, [src, os.path.join(INCLUDE, "lidar_gb300.h")] + headers):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I" + INCLUDE, src, "-o", lib])
    ref_script = os.path.join(REPO, "oracle", "build_ref.sh")
    ref_lib = os.path.join(REPO, "oracle", "_ref", "libref.so")
    # the recipe finds the reference tree itself (REF_ROOT) and builds nothing where it is absent
    shims = [os.path.join(dp, f) for dp, _, fs in os.walk(os.path.join(REPO, "oracle", "shim")) for f in fs]
    extra = [os.path.join(REPO, "oracle", f) for f in ("ref_capi.cpp", "ring_ref_prelude.h", "ring_ref_capi.inc")]
    if _stale(ref_lib, shims + headers + extra + [ref_script]):
        _run(["bash", ref_script])
    return lib


def build_all(verbose=False):
    with ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_gpu, verbose), ex.submit(build_synth), ex.submit(build_oracle)]
        out = [f.result() for f in futs]
    out.append(build_example())
    return out


if __name__ == "__main__":
    print(build_all(verbose="-v" in sys.argv))
    if "--ptxas" in sys.argv:
        build_gpu(verbose=True, ptxas_info=True)
