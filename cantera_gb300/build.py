"""Build recipe of the engine library ``cantera_gb300/_build/libgbchem.so``.

Every translation unit is compiled by nvcc for sm_103a only (one -gencode), the units in
parallel, then linked into one shared library with the C ABI of include/gbchem.h.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgbchem.so")
OUT_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(OUT_CHECKED, "libgbchem.so")
SOURCES = ["capi.cu", "kernels.cu", "kernels_x.cu", "krylov.cu", "krylov32.cu", "surrogate.cu", "umma.cu", "mechanism.cpp", "yaml_lite.cpp"]
HEADERS = ["devmech.h", "fastexp.h", "kernels.h", "kinetics.cuh", "mechanism.h", "nnmath.cuh", "surrogate.h",
           "yaml_lite.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in ("nvcc", "/usr/local/cuda/bin/nvcc"):
        try:
            subprocess.run([c, "--version"], capture_output=True, check=True)
            return c
        except (OSError, subprocess.CalledProcessError):
            pass
    raise RuntimeError("nvcc not found")


def _compile(nvcc, src, extra, OUT):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    cmd = [nvcc] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2",
                           "-I", os.path.join(HERE, "..", "include"), "-c", src, "-o", obj] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False, extra=None, checked=False):
    """Build the library (the bounds-checked variant with checked=True, into _build_checked)."""
    if checked:
        return _build(OUT_CHECKED, LIB_CHECKED, force, verbose, list(extra or []) + ["-DGBCHEM_CHECKED"])
    return _build(OUT, LIB, force, verbose, extra)


def _build(OUT, LIB, force, verbose, extra):
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(HERE, "..", "include", "gbchem.h"), os.path.abspath(__file__)]
    if not force and os.path.exists(LIB):
        if os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
            return LIB
    nvcc = _nvcc()
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(nvcc, s, extra, OUT), srcs))
    if verbose:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
