"""Build the CUDA library ``libpyqg_gb300.so`` in-tree for sm_103a.

``python -m pyqg_gb300.build`` (or ``__graft_entry__.build()``) compiles
``csrc/*.cu`` with nvcc into ``pyqg_gb300/lib/``.  Host code is compiled with
``-ffp-contract=off`` so host-side constant tables round identically on
x86-64 and aarch64.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIBNAME = "libpyqg_gb300.so"
ARCH = "103a"   # GB300 only: the kernels use tcgen05, TMA and sm_103a cluster features


def nvcc_path():
    cand = os.environ.get("NVCC") or shutil.which("nvcc")
    if cand:
        return cand
    default = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(default):
        return default
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith(".cu"))


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def build(verbose=False, extra_flags=()):
    """Compile each csrc/*.cu to an object in parallel, then link the
    shared library; returns its path."""
    from concurrent.futures import ThreadPoolExecutor
    os.makedirs(LIBDIR, exist_ok=True)
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    out = lib_path()
    tmp = out + ".tmp"
    common = [nvcc_path(), "-O3", "-std=c++17", "-lineinfo",
              "-gencode", "arch=compute_%s,code=sm_%s" % (ARCH, ARCH),
              "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
              "-Xptxas", "-O3",
              "-I", os.path.join(os.path.dirname(HERE), "include"), *extra_flags]

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src)[:-3] + ".o")
        res = subprocess.run(common + ["-c", src, "-o", obj], capture_output=True, text=True)
        return src, obj, res

    with ThreadPoolExecutor(max_workers=4) as ex:
        results = list(ex.map(compile_one, sources()))
    for src, obj, res in results:
        if verbose or res.returncode != 0:
            sys.stderr.write(res.stdout + res.stderr)
        if res.returncode != 0:
            raise RuntimeError("nvcc failed on %s (exit %d)" % (src, res.returncode))
    res = subprocess.run([nvcc_path(), "-shared", "-gencode", "arch=compute_%s,code=sm_%s" % (ARCH, ARCH),
                          *[o for _, o, _ in results], "-o", tmp], capture_output=True, text=True)
    if verbose or res.returncode != 0:
        sys.stderr.write(res.stdout + res.stderr)
    if res.returncode != 0:
        raise RuntimeError("nvcc link failed (exit %d)" % res.returncode)
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
