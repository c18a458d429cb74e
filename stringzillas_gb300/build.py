"""Builds ``libszs_gb300.so`` in-tree with nvcc for sm_103a (GB300).

Each kernel family is its own translation unit so the template instantiations compile in parallel; the
bit-parallel unit is compiled once per plane count. Usage: ``python -m stringzillas_gb300.build [--force]``.
"""
from __future__ import annotations

import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys

PACKAGE_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PACKAGE_DIR)
CSRC = os.path.join(PACKAGE_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
OUT_DIR = os.path.join(PACKAGE_DIR, "_lib")
BUILD_DIR = os.path.join(PACKAGE_DIR, "_build")
LIBRARY = os.path.join(OUT_DIR, "libszs_gb300.so")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
                "-Xcompiler", "-fvisibility=hidden", "-I", INCLUDE, "-I", CSRC]

# (object name, source, extra flags)
UNITS = [
    ("engine", "engine.cu", []),
    ("planner", "planner.cu", []),
    ("kernels_dp", "kernels_dp.cu", []),
    ("kernels_dp16", "kernels_dp16.cu", []),
    ("kernels_dp16_compare", "kernels_dp16.cu", ["-DSZS_DP16_COMPARE_UNIT"]),
    ("kernels_band", "kernels_band.cu", ["-DSZS_BAND_ROWS=8"]),
    ("kernels_band4", "kernels_band.cu", ["-DSZS_BAND_ROWS=4"]),
    ("kernels_band16", "kernels_band16.cu", ["-DSZS_BAND16_ROWS=8"]),
    ("kernels_band16_4", "kernels_band16.cu", ["-DSZS_BAND16_ROWS=4"]),
    ("direct", "direct.cu", []),
    ("kernels_short8", "kernels_short.cu", ["-DSZS_SHORT_ROWS=8"]),
    ("kernels_short12", "kernels_short.cu", ["-DSZS_SHORT_ROWS=12"]),
    ("kernels_short16", "kernels_short.cu", ["-DSZS_SHORT_ROWS=16"]),
    ("probe", "probe.cu", []),
    ("static_scratch", "static_scratch.cu", []),
    ("server", "server.cu", []),
    ("utf8", "utf8.cu", []),
    ("fingerprints", "fingerprints.cu", []),
    ("myers_wide", "kernels_myers_wide.cu", []),
    ("myers_p2", "kernels_myers.cu", ["-DSZS_MYERS_PLANES=2"]),
    ("myers_table", "kernels_myers_table.cu", []),
    ("myers_chain", "kernels_myers_chain.cu", []),
    ("myers_p3", "kernels_myers.cu", ["-DSZS_MYERS_PLANES=3"]),
    ("myers_p5", "kernels_myers.cu", ["-DSZS_MYERS_PLANES=5"]),
    ("myers_p8", "kernels_myers.cu", ["-DSZS_MYERS_PLANES=8"]),
]


def nvcc() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    fallback = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(fallback):
        return fallback
    raise RuntimeError("nvcc not found: the GB300 engine has no CPU fallback and must be compiled with CUDA")


def nvcc_available() -> bool:
    try:
        nvcc()
        return True
    except RuntimeError:
        return False


def _sources_digest() -> str:
    digest = hashlib.sha256()
    for root in (CSRC, INCLUDE):
        for name in sorted(os.listdir(root)):
            path = os.path.join(root, name)
            if os.path.isfile(path):
                with open(path, "rb") as f:
                    digest.update(name.encode() + f.read())
    digest.update(" ".join(ARCH_FLAGS + COMMON_FLAGS).encode())
    return digest.hexdigest()


def _compile(unit, verbose):
    name, source, extra = unit
    obj = os.path.join(BUILD_DIR, name + ".o")
    cmd = [nvcc()] + ARCH_FLAGS + COMMON_FLAGS + extra + ["-c", os.path.join(CSRC, source), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"nvcc failed for {source} ({name}):\n{result.stdout}\n{result.stderr}")
    return obj, result.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles the library if its sources changed; returns the library path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    stamp = os.path.join(OUT_DIR, "libszs_gb300.stamp")
    digest = _sources_digest()
    if not force and os.path.exists(LIBRARY) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIBRARY
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as pool:
        outputs = list(pool.map(lambda u: _compile(u, verbose), UNITS))
    objects = [o for o, _ in outputs]
    if verbose:
        for _, log in outputs:
            sys.stderr.write(log)
    link = [nvcc()] + ARCH_FLAGS + ["-shared", "-o", LIBRARY] + objects + ["-lcudart"]
    result = subprocess.run(link, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"link failed:\n{result.stdout}\n{result.stderr}")
    with open(stamp, "w") as f:
        f.write(digest)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
