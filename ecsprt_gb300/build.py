"""Build libecsgpu.so (CUDA, sm_103a), libecshost.so (host C) and the
re-hosted programs pic and solver in-tree.

Translation units compile in parallel; a unit is rebuilt only when its
source, a shared header or the flags change.  Run as a module
(``python -m ecsprt_gb300.build``) or call :func:`build`.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
INCLUDE = ROOT / "include"
OUT = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-Xptxas",
    "-warn-spills",
    f"-I{INCLUDE}",
    f"-I{CSRC}",
]
CC_FLAGS = ["-O2", "-fPIC", "-std=gnu11", "-Wall", "-Wextra", "-Wno-unused-parameter", f"-I{INCLUDE}"]

GPU_SOURCES = ["ecs_api.cu", "ecs_particles.cu", "ecs_grid.cu", "ecs_solver.cu", "ecs_noalloc.cu", "ecs_serve.cu"]
HOST_SOURCES = ["ecs_options.c", "ecs_io.c"]
GPU_HOST_SOURCES = ["ecs_ops.c"]  # host C linked into libecsgpu (operator slots)
# the reference's programs re-hosted on the libraries: program -> main source
PROGRAMS = {"pic": "ecs_pic_main.c", "solver": "ecs_solver_main.c"}
DRIVER_SOURCES = ["ecs_driver.c"]

LIBGPU = OUT / "libecsgpu.so"
LIBHOST = OUT / "libecshost.so"


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libecsgpu")
    return cand


def _digest(paths, flags) -> str:
    h = hashlib.sha256(" ".join(flags).encode())
    for p in paths:
        h.update(Path(p).read_bytes())
    return h.hexdigest()


def _compile(cmd, obj: Path, stamp: Path, digest: str, verbose: bool):
    if obj.exists() and stamp.exists() and stamp.read_text() == digest:
        return None
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    stamp.write_text(digest)
    return r.stderr


def build(verbose: bool = False, jobs: int | None = None) -> dict:
    OUT.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    headers = sorted(list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))
    tasks = []
    gpu_objs = []
    for src in GPU_SOURCES:
        s = CSRC / src
        obj = OUT / (s.stem + ".o")
        flags = NVCC_FLAGS + ["-c", str(s), "-o", str(obj)]
        tasks.append(([nvcc] + flags, obj, OUT / (s.stem + ".stamp"), _digest([s] + headers, flags)))
        gpu_objs.append(obj)
    host_objs = []
    cc = shutil.which("gcc") or "cc"
    for src in GPU_HOST_SOURCES:
        s = HOST / src
        obj = OUT / (s.stem + ".gpuhost.o")
        flags = CC_FLAGS + ["-c", str(s), "-o", str(obj)]
        tasks.append(([cc] + flags, obj, OUT / (s.stem + ".gpuhost.stamp"), _digest([s] + headers, flags)))
        gpu_objs.append(obj)
    for src in HOST_SOURCES:
        s = HOST / src
        obj = OUT / (s.stem + ".host.o")
        flags = CC_FLAGS + ["-c", str(s), "-o", str(obj)]
        tasks.append(([cc] + flags, obj, OUT / (s.stem + ".host.stamp"), _digest([s] + headers, flags)))
        host_objs.append(obj)
    warnings = []
    with ThreadPoolExecutor(max_workers=jobs or max(1, min(len(tasks), os.cpu_count() or 4))) as ex:
        for w in ex.map(lambda t: _compile(*t, verbose), tasks):
            if w:
                warnings.append(w)
    link_gpu = [nvcc] + ARCH + ["-shared", "-o", str(LIBGPU)] + [str(o) for o in gpu_objs] + ["-lcudart", "-lpthread"]
    if not LIBGPU.exists() or any(o.stat().st_mtime > LIBGPU.stat().st_mtime for o in gpu_objs):
        r = subprocess.run(link_gpu, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {r.stderr}")
    link_host = [cc, "-shared", "-o", str(LIBHOST)] + [str(o) for o in host_objs] + ["-lm"]
    if not LIBHOST.exists() or any(o.stat().st_mtime > LIBHOST.stat().st_mtime for o in host_objs):
        r = subprocess.run(link_host, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host link failed: {r.stderr}")
    programs = {}
    for prog, main in PROGRAMS.items():
        srcs = [HOST / main] + [HOST / d for d in DRIVER_SOURCES]
        exe = OUT / prog
        flags = CC_FLAGS + [f"-I{HOST}"] + [str(x) for x in srcs] + [
            "-o", str(exe), f"-L{OUT}", "-lecsgpu", "-lecshost", "-lm", "-Wl,-rpath,$ORIGIN"]
        stamp = OUT / (prog + ".stamp")
        digest = _digest(srcs + headers + [LIBGPU, LIBHOST], flags)
        if not (exe.exists() and stamp.exists() and stamp.read_text() == digest):
            r = subprocess.run([cc] + flags, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link of {prog} failed: {r.stderr}")
            stamp.write_text(digest)
        programs[prog] = str(exe)
    if verbose:
        for w in warnings:
            sys.stderr.write(w)
    return {"gpu": str(LIBGPU), "host": str(LIBHOST), "programs": programs, "warnings": warnings}


if __name__ == "__main__":
    info = build(verbose=True)
    print(info["gpu"])
    print(info["host"])
