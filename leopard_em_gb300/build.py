"""Build the in-tree CUDA library ``_build/libleopard_gb300.so`` for sm_103a.

Each translation unit under ``csrc/`` is compiled by its own nvcc process (in
parallel), then linked into one shared library with the CUDA runtime linked
statically, so the library loads on a machine without a GPU (symbol checks)
and carries no dependency on torch.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libleopard_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)
# measurement-only kernels (csrc/bench/*.cu), linked into a library of their own
PROBE_LIB_PATH = os.path.join(OUT_DIR, "libleopard_gb300_probe.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build leopard_em_gb300")
    return cand


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def probe_sources() -> list[str]:
    d = os.path.join(CSRC, "bench")
    return sorted(os.path.join(d, f) for f in os.listdir(d) if f.endswith(".cu"))


def _compile(src: str, extra: list[str]) -> str:
    tag = "bench_" if os.path.basename(os.path.dirname(src)) == "bench" else ""
    obj = os.path.join(OUT_DIR, tag + os.path.basename(src)[:-3] + ".o")
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr}")
    return obj


def _link(objs: list[str], path: str) -> None:
    tmp = path + ".tmp"
    cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, path)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    """Compile every csrc/*.cu and link the shared library (and the
    measurement probes of csrc/bench/ into their own library); returns the
    product library's path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    extra = list(extra_flags or [])
    srcs = sources()
    probes = probe_sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs) + len(probes), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs + probes))
    _link(objs[: len(srcs)], LIB_PATH)
    _link(objs[len(srcs):], PROBE_LIB_PATH)
    if verbose:
        print("built", LIB_PATH, "and", PROBE_LIB_PATH, file=sys.stderr)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
