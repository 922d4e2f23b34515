"""In-tree build of the rubix_gb300 CUDA library for sm_103a with nvcc.

``build()`` compiles every ``csrc/*.cu`` to an object in parallel and links
``librubix_gb300.so`` next to this file.  It is a no-op when the library is newer
than every source and header.  No cmake, one ``-gencode``.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJDIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(HERE, "librubix_gb300.so")
# bench-only measurement aid (the FP32 FMA-rate probe), kept out of the product library
PROBE_SRC = os.path.join(ROOT, "bench_fma_probe.cu")
PROBE_PATH = os.path.join(HERE, "librubix_gb300_probe.so")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    "--expt-relaxed-constexpr",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the rubix_gb300 CUDA library cannot be built")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    deps = sources()
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    deps.append(os.path.abspath(__file__))
    return deps


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(nvcc, src, verbose):
    obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-I", INCLUDE, "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the library if needed and return its path."""
    if not force and up_to_date():
        return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(OBJDIR, exist_ok=True)
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(nvcc, s, verbose), srcs))
    if verbose:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_probe(force: bool = False) -> str:
    """Compile bench.py's FP32 FMA-rate probe into its own small library (not part of
    librubix_gb300) if needed and return its path."""
    if (not force and os.path.exists(PROBE_PATH)
            and os.path.getmtime(PROBE_PATH) >= os.path.getmtime(PROBE_SRC)):
        return PROBE_PATH
    tmp = PROBE_PATH + ".tmp"
    cmd = [_nvcc(), *ARCH_FLAGS, *NVCC_FLAGS, "-shared", PROBE_SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {PROBE_SRC}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, PROBE_PATH)
    return PROBE_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_probe(force="--force" in sys.argv))
