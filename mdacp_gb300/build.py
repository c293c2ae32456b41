"""Builds libmdg.so (the CUDA library behind include/mdg.h) in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel to an object file under
mdacp_gb300/_build/, then one link step produces mdacp_gb300/libmdg.so.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmdg.so")
# bounds-checked build (-DMDG_CHECK=1): the same sources, every gather and
# scatter index of the single-box path checked on the device
OBJ_CHECK = os.path.join(HERE, "_build_check")
LIB_CHECK = os.path.join(HERE, "libmdg_check.so")
SOURCES = ["mdg_cells.cu", "mdg_list.cu", "mdg_step.cu", "mdg_batch.cu", "mdg_api.cu", "mdg_adjoint.cu", "mdg_noalloc.cu",
           "mdg_io.cu", "mdg_init.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
                   *extra]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    # an equal time counts as newer: a source saved in the same clock tick as
    # the last build is rebuilt
    return any(os.path.getmtime(d) >= t for d in deps)


def build(force=False, verbose=False, extra_flags=(), check=False):
    """Compiles and links libmdg.so (libmdg_check.so with check=True) if any
    source is newer; returns its path."""
    obj_dir, lib_path = (OBJ_CHECK, LIB_CHECK) if check else (OBJ, LIB)
    if check:
        extra_flags = tuple(extra_flags) + ("-DMDG_CHECK=1",)
    os.makedirs(obj_dir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "mdg.h"))
    srcs = [os.path.join(CSRC, s) for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = [os.path.join(obj_dir, os.path.basename(s).replace(".cu", ".o")) for s in srcs]
    cc = nvcc()

    def compile_one(src, obj):
        if not force and not _stale(obj, [src] + headers):
            return None
        cmd = [cc, *_flags(extra_flags), "-c", src, "-o", obj + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        os.replace(obj + ".tmp", obj)
        return r.stderr if verbose else None

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        outs = list(ex.map(lambda a: compile_one(*a), zip(srcs, objs)))
    if verbose:
        for o in outs:
            if o:
                sys.stderr.write(o)
    if force or _stale(lib_path, objs):
        tmp = lib_path + ".tmp%d" % os.getpid()
        cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, lib_path)
    return lib_path


HOST = os.path.join(HERE, "host")
HOST_BIN = os.path.join(HERE, "mdg_mdacp")


def build_host(force=False):
    """Links the C++ host front-end (mdg_mdacp) against libmdg.so."""
    srcs = [os.path.join(HOST, f) for f in ("mdg_host.cpp", "mdg_mdacp.cpp")]
    deps = srcs + [os.path.join(HOST, "mdg_host.hpp"), os.path.join(ROOT, "include", "mdg.h"), LIB]
    if not force and not _stale(HOST_BIN, deps):
        return HOST_BIN
    cxx = shutil.which("g++") or "g++"
    tmp = HOST_BIN + ".tmp%d" % os.getpid()
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), *srcs, "-L", HERE, "-lmdg",
           "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host build failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, HOST_BIN)
    return HOST_BIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra_flags=["-Xptxas", "-v"] if "-v" in sys.argv else ()))
