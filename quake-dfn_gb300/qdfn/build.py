"""Build recipe of libqdfn.so (sm_103a only).

Each translation unit is compiled by its own nvcc process in parallel, then the
objects are linked into ``quake-dfn_gb300/lib/libqdfn.so`` (in-tree, git-ignored).
The per-TU flags keep IEEE FP64 semantics where the result must track the
reference (``--fmad=false``: no contraction of a*b+c, like Julia); kernels use
explicit ``fma`` only where a fused multiply-add is intended.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
LIBDIR = os.path.join(PKG_ROOT, "lib")
LIB_PATH = os.path.join(LIBDIR, "libqdfn.so")
OBJDIR = os.path.join(PKG_ROOT, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math",
          "-diag-suppress", "177"]
# translation unit -> extra flags
UNITS = {
    "api.cpp": [],
    "input.cpp": [],
    "assemble.cu": [],
    "assemble_rect.cu": ["--fmad=false"],
    "assemble_tri.cu": ["--fmad=false"],
    "sim.cu": ["--fmad=false"],
    "ensemble.cu": ["--fmad=false"],
    "noalloc.cu": ["--fmad=false"],
    "selfcheck.cu": ["--fmad=false"],
    "adjoint.cu": ["--fmad=false"],
    "hstruct.cu": ["--fmad=false"],
}


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libqdfn.so")


def _sources_newer(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    for root, _, files in os.walk(CSRC):
        for f in files:
            if os.path.getmtime(os.path.join(root, f)) > t:
                return True
    inc = os.path.join(os.path.dirname(PKG_ROOT), "include", "qdfn.h")
    return os.path.exists(inc) and os.path.getmtime(inc) > t


def build(force=False, verbose=False):
    """Compile and link libqdfn.so; returns its path."""
    if not force and not _sources_newer(LIB_PATH):
        return LIB_PATH
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    cc = nvcc()

    def compile_one(item):
        src, extra = item
        obj = os.path.join(OBJDIR, src + ".o")
        if src.endswith(".cpp"):  # host-only unit
            cmd = [cc] + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        else:
            cmd = [cc] + ARCH + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), out.stderr[-6000:]))
        if verbose:
            print(out.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS.items()))
    tmp = LIB_PATH + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("link failed:\n%s" % out.stderr[-4000:])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
