"""Build recipe of libcarcgb300.so (in-tree, sm_103a only).

``python -m carcassonne_gb300.build`` compiles every translation unit under
``csrc/`` in parallel with nvcc and links them into
``carcassonne_gb300/_lib/libcarcgb300.so``.  Object files are cached by
content hash under ``_lib/obj`` so a rebuild only recompiles what changed.
"""
from __future__ import annotations

import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "libcarcgb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]


def nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_digest():
    h = hashlib.sha256()
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in sorted(os.listdir(d)):
            if f.endswith((".cuh", ".h")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(f.encode())
                    h.update(fh.read())
    h.update(" ".join(ARCH + FLAGS).encode())
    return h.hexdigest()


def _compile(src, hdr_digest, verbose):
    with open(src, "rb") as fh:
        key = hashlib.sha256(fh.read() + hdr_digest.encode()).hexdigest()[:16]
    obj = os.path.join(OBJDIR, os.path.basename(src) + "." + key + ".o")
    if os.path.exists(obj):
        return obj
    cmd = [nvcc(), *ARCH, *FLAGS, "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj + ".tmp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
    if verbose and (r.stdout.strip() or r.stderr.strip()):
        print(r.stdout, r.stderr, flush=True)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False):
    os.makedirs(OBJDIR, exist_ok=True)
    digest = _headers_digest()
    srcs = _sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(16, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, digest, verbose), srcs))
    out = lib_path()
    tmp = out + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, out)
    # drop stale objects
    keep = set(os.path.basename(o) for o in objs)
    for f in os.listdir(OBJDIR):
        if f not in keep:
            try:
                os.remove(os.path.join(OBJDIR, f))
            except OSError:
                pass
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
