"""In-tree build of the CUDA front-end library (sm_103a) and the C++ adapter test.

The library is compiled with ``--fmad=false`` and host ``-ffp-contract=off``:
the front-end's arithmetic contract is IEEE binary32 with no contraction, so
the kernels stay bit-identical to the CPU oracle.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libuslam.so")
BUILD_DIR = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-lineinfo", "-O3", "--fmad=false", "-std=c++17",
    "-Xcompiler", "-fPIC,-ffp-contract=off",
    "-I", os.path.join(REPO, "include"),
]
SOURCES = ["kernels.cu", "runtime.cu", "server.cu", "noalloc.cu", "ransac.cu", "triangulate.cu", "bf_tc.cu",
           "win_tc.cu"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libuslam.so")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


STAMP = os.path.join(BUILD_DIR, "built_on.txt")


def _machine_tag(nvcc: str) -> str:
    """Host architecture and compiler version the objects are built with."""
    r = subprocess.run([nvcc, "--version"], capture_output=True, text=True)
    last = [ln for ln in r.stdout.splitlines() if ln.strip()][-1:] or ["?"]
    return f"{platform.machine()} | {last[0].strip()}"


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compile csrc/*.cu into libuslam.so (translation units in parallel).

    Objects and the library built on another machine (another host
    architecture or compiler, as when a checkout is copied to a GPU host) are
    never reused: the stamp written beside the objects names where they were
    built, and a mismatch forces a full rebuild from source."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    tag = _machine_tag(nvcc)
    prev = open(STAMP).read().strip() if os.path.exists(STAMP) else None
    if prev != tag:
        if prev is not None or os.path.exists(LIB):
            print(f"uslam build: objects were built on [{prev}], this host is [{tag}]: rebuilding from source",
                  flush=True)
        force = True
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".hpp"))]
    headers += [os.path.join(REPO, "include", h) for h in os.listdir(os.path.join(REPO, "include"))]
    objs = []
    jobs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            jobs.append([nvcc, *NVCC_FLAGS, "-c", path, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    with open(STAMP, "w") as f:
        f.write(tag + "\n")
    if force:
        print(f"uslam build: compiled {len(jobs)} translation units and linked {LIB} on [{tag}]", flush=True)
    return LIB


def build_oracle(reference: str | None = None) -> None:
    """Build the CPU oracle and the reference matcher (from the checkout at
    `reference`, or from the copy staged beside the repository)."""
    cmd = ["make", "-s", "-C", os.path.join(REPO, "oracle")]
    if reference:
        cmd.append(f"USLAM_REFERENCE={reference}")
    # objects of another host architecture are never reused
    stamp = os.path.join(REPO, "oracle", "_ref", "built_on.txt")
    tag = platform.machine()
    if os.path.exists(os.path.join(REPO, "oracle")) and (not os.path.exists(stamp) or open(stamp).read().strip() != tag):
        cmd.insert(1, "-B")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.makedirs(os.path.dirname(stamp), exist_ok=True)
    with open(stamp, "w") as f:
        f.write(tag + "\n")


if __name__ == "__main__":
    build_library(verbose=True)
    build_oracle()
