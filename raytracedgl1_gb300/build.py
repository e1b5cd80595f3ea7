"""Builds the native libraries in-tree (no cmake, no pip):

* ``raytracedgl1_gb300/lib/librgdn.so`` — the sm_103a CUDA kernels and the C ABI of
  ``include/rgdn.h`` (nvcc, one translation unit per storage mode, compiled in parallel);
* ``raytracedgl1_gb300/lib/librgdn_scene.so`` — the host-side synthetic scene generator;
* ``oracle/librgdn_oracle.so`` — the CPU oracle (test infrastructure, built beside the product
  so the checker exists wherever the tests run).

Rebuilds only what is older than its sources. ``python -m raytracedgl1_gb300.build`` or
``build_all()``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
ORACLE_DIR = os.path.join(ROOT, "oracle")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no contraction of a*b+c, so threshold decisions match an IEEE evaluation.
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-O3", "-I" + INCLUDE, "-I" + CSRC]
CU_SOURCES = ["rgdn_api.cu", "rgdn_mode_ref.cu", "rgdn_mode_f32.cu", "rgdn_mode_f16.cu",
              "rgdn_mode_bf16.cu", "rgdn_noalloc.cu", "rgdn_batch.cu", "rgdn_serve.cu", "rgdn_fast_ref.cu", "rgdn_fast_f32.cu",
              "rgdn_fast_f16.cu", "rgdn_fast_bf16.cu"]
# No translation unit lets the compiler contract a*b+c on its own: where the kernels want a
# fused multiply-add they say so (__fmaf_rn), so every instantiation of a kernel body (the
# single-frame and the batched kernels) computes the same bits.
FMAD_TRUE: set[str] = set()
HEADERS = ["rgdn_internal.h", "rgdn_kernels.cuh", "rgdn_codec.h", "rgdn_host.h"]

LIB_RGDN = os.path.join(LIBDIR, "librgdn.so")
LIB_SCENE = os.path.join(LIBDIR, "librgdn_scene.so")
LIB_ORACLE = os.path.join(ORACLE_DIR, "librgdn_oracle.so")


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librgdn.so")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def build_rgdn(force: bool = False, jobs: int | None = None) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "rgdn.h")]
    objs, todo = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            flags = [f if f != "--fmad=false" or src not in FMAD_TRUE else "--fmad=true" for f in NVCC_FLAGS]
            todo.append([nvcc] + flags + ["-c", s, "-o", o])
    if todo:
        with ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, todo))
    if force or todo or _stale(LIB_RGDN, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB_RGDN] + objs)
    return LIB_RGDN


def build_scene(force: bool = False) -> str:
    os.makedirs(LIBDIR, exist_ok=True)
    src = os.path.join(CSRC, "scene_gen.cpp")
    deps = [src, os.path.join(CSRC, "rgdn_codec.h"), os.path.join(INCLUDE, "rgdn.h")]
    if force or _stale(LIB_SCENE, deps):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-I" + INCLUDE, src, "-o", LIB_SCENE,
              "-lpthread"])
    return LIB_SCENE


def build_oracle(force: bool = False) -> str:
    src = os.path.join(ORACLE_DIR, "rgdn_oracle.cpp")
    deps = [src, os.path.join(INCLUDE, "rgdn.h")]
    if force or _stale(LIB_ORACLE, deps):
        # -ffp-contract=off: IEEE evaluation without fused multiply-add, like the GPU build
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I" + INCLUDE,
              src, "-o", LIB_ORACLE, "-lpthread"])
    return LIB_ORACLE


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_rgdn, force), ex.submit(build_scene, force),
                ex.submit(build_oracle, force)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built:", LIB_RGDN, LIB_SCENE, LIB_ORACLE)
