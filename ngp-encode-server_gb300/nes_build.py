"""Builds libnes_gb300.so in-tree with nvcc for sm_103a.

Every translation unit is compiled in parallel (nvcc for .cu, g++ via nvcc
for .cpp), then linked into one shared library next to this file.  A stamp
of the sources and flags skips the build when nothing changed.

    python ngp-encode-server_gb300/nes_build.py [--force] [--verbose]
"""
import concurrent.futures as cf
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.normpath(os.path.join(HERE, "..", "include"))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnes_gb300.so")
SERVER_BIN = os.path.join(HERE, "nes_render_server")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-I", CSRC, "-I", INCLUDE]
CU_FLAGS = ARCH + COMMON + ["--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def _sources():
    out = []
    for name in sorted(os.listdir(CSRC)):
        if name.endswith((".cu", ".cpp")):
            out.append(os.path.join(CSRC, name))
    return out


def _stamp(srcs):
    h = hashlib.sha256()
    for p in sorted(os.listdir(CSRC)) + sorted(os.listdir(INCLUDE)):
        full = os.path.join(CSRC, p) if os.path.exists(os.path.join(CSRC, p)) else os.path.join(INCLUDE, p)
        with open(full, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    with open(os.path.join(HERE, "render_server.cpp"), "rb") as f:
        h.update(f.read())
    h.update(" ".join(CU_FLAGS).encode())
    return h.hexdigest()


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [NVCC] + CU_FLAGS + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC] + ARCH + COMMON + ["-x", "c++", "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (src, r.stdout, r.stderr))
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return obj


def build(force=False, verbose=False):
    """Compiles and links the library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    stamp = _stamp(srcs)
    stamp_file = os.path.join(BUILD, "stamp")
    if not force and os.path.exists(LIB) and os.path.exists(SERVER_BIN) and os.path.exists(stamp_file):
        with open(stamp_file) as f:
            if f.read() == stamp:
                return LIB
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    # The renderer endpoint for an unmodified neserver, linked to the library.
    cmd = ["g++", "-O2", "-std=c++17", "-I", INCLUDE, os.path.join(HERE, "render_server.cpp"), "-o", SERVER_BIN,
           "-L", HERE, "-lnes_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("render server link failed\n%s%s" % (r.stdout, r.stderr))
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
