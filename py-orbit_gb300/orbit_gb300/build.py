"""Builds liborbit_gb300.so in-tree from py-orbit_gb300/csrc with nvcc for
sm_103a (one -gencode, translation units compiled in parallel)."""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(ROOT, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "liborbit_gb300.so")
SOURCES = ["bunch.cu", "teapot.cu", "sc2p5d.cu", "program.cu", "peaks.cu", "boundary.cu", "diag.cu", "batch.cu", "dn.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-Xptxas", "-O3"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _digest(paths, flags) -> str:
    """SHA-256 of the compiler flags and the contents of the given files."""
    h = hashlib.sha256(" ".join(flags).encode())
    for p in paths:
        h.update(p.encode())
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _stale(target: str, digest: str) -> bool:
    """A build output is stale unless it exists beside a stamp holding the
    digest of what it was built from (contents, not modification times: a
    copied tree with fresh times or an output carried over from another
    machine is rebuilt exactly when its inputs differ)."""
    stamp = target + ".sha256"
    if not (os.path.exists(target) and os.path.exists(stamp)):
        return True
    with open(stamp) as f:
        return f.read().strip() != digest


def _stamp(target: str, digest: str):
    with open(target + ".sha256", "w") as f:
        f.write(digest + "\n")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(os.path.dirname(ROOT), "include", "orbit_gb300.h"))
    return hs


def build_library(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    """Compile every translation unit and link the shared library; returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    flags = NVFLAGS + list(extra_flags or [])
    jobs = []
    objs = []
    digests = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        d = _digest([s] + sorted(hdrs), ARCH + flags + [platform.machine()])
        digests.append((o, d))
        if force or _stale(o, d):
            jobs.append([cc] + ARCH + flags + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(run, jobs):
                if verbose and out.strip():
                    print(out)
    for o, d in digests:
        _stamp(o, d)
    lib_digest = hashlib.sha256("".join(d for _, d in digests).encode()).hexdigest()
    if force or jobs or _stale(LIB_PATH, lib_digest):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        run([cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
        os.replace(tmp, LIB_PATH)
        _stamp(LIB_PATH, lib_digest)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build_library(force="--force" in sys.argv, verbose=True))
