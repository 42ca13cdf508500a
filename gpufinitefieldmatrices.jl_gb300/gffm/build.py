"""Build libgffm.so in-tree with nvcc for sm_103a (GB300).

Every CUDA translation unit under ``csrc/`` is compiled in parallel and linked
into ``lib/libgffm.so``.  The library links the CUDA runtime statically, so it
only needs the NVIDIA driver (libcuda) at run time.
"""
import concurrent.futures
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libgffm.so")
OBJ_DIR = os.path.join(PKG_ROOT, "_build")
REPO_ROOT = os.path.dirname(PKG_ROOT)
HEADER = os.path.join(REPO_ROOT, "include", "gffm.h")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "-Xcompiler", "-Wall"]


def nvcc_path():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: libgffm needs the CUDA toolkit to build")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [HEADER]
    return max(os.path.getmtime(f) for f in files)


def up_to_date():
    return os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= _deps()


def build(force=False, verbose=False, jobs=None):
    """Compile and link libgffm.so (skipped when it is newer than every source)."""
    if not force and up_to_date():
        return LIB_PATH
    nvcc = nvcc_path()
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = _sources()
    objs = [os.path.join(OBJ_DIR, os.path.basename(s)[:-3] + ".o") for s in srcs]

    def compile_one(src_obj):
        src, obj = src_obj
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s" % (os.path.basename(src), r.stderr[-8000:]))
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr[-8000:])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
