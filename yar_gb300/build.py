"""Build recipe for the native parts of yar_gb300 (no cmake, no setuptools).

Outputs, all in-tree and git-ignored:
  yar_gb300/libyar_gb300.so   the product: CUDA kernels for sm_103a + C ABI +
                              host kd-tree builder (include/yar_gpu.h)
  oracle/liboracle.so         test infrastructure: the C restatement used by the
                              tests and the CPU baseline leg of bench.py
  oracle/_ref/yar_ref         test infrastructure: the reference renderer built
                              from its own sources (oracle/build_ref.sh), when
                              they are available
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "yar_gb300")
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libyar_gb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no contraction, so device float arithmetic rounds like the
# reference's (MSVC /fp:precise, g++ -ffp-contract=off).  Division and sqrt
# stay IEEE (no fast-math flags).
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
             "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

CU_SOURCES = ["capi.cu", "cast.cu", "render.cu", "guide_mlp.cu", "guided.cu", "batch.cu", "direct.cu"]
CXX_SOURCES = ["kdtree_build.cpp"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".hpp", ".cuh"))]
    return hs


def build_product(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append([nvcc] + GENCODE + NVCC_FLAGS + ["-Xptxas", "-v", "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if jobs or _stale(LIB, objs):
        _run([nvcc] + GENCODE + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"])
    return LIB


def build_oracle():
    src = os.path.join(ORACLE_DIR, "yar_oracle.c")
    deps = [src, os.path.join(ORACLE_DIR, "yar_oracle.h"), os.path.join(ROOT, "include", "yar_gpu.h")]
    if _stale(ORACLE_LIB, deps):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread",
              "-I" + os.path.join(ROOT, "include"), src, "-o", ORACLE_LIB, "-lm"])
    return ORACLE_LIB


def reference_root():
    """The reference checkout: $YAR_REFERENCE_ROOT, else a `reference` folder
    beside this repository."""
    return os.environ.get("YAR_REFERENCE_ROOT") or os.path.join(os.path.dirname(ROOT), "reference")


def build_reference():
    """Build oracle/_ref from the reference sources when they are present."""
    script = os.path.join(ORACLE_DIR, "build_ref.sh")
    ref = reference_root()
    have_src = os.path.isdir(os.path.join(ref, "src", "ref")) or \
        os.path.isdir(os.path.join(ORACLE_DIR, "_ref", "src", "src", "ref"))
    if not have_src:
        return None
    binary = os.path.join(ORACLE_DIR, "_ref", "yar_ref")
    deps = [os.path.join(ORACLE_DIR, "ref_harness.cpp"), os.path.join(ORACLE_DIR, "ref_flatten.hpp"),
            os.path.join(ORACLE_DIR, "render_scene_gpu.cpp"), script, os.path.join(ROOT, "include", "yar_gpu.h"),
            os.path.join(CSRC, "yfs.hpp"), LIB]
    if os.path.exists(binary) and not _stale(binary, deps):
        try:  # an x86 binary copied to an aarch64 host does not run: rebuild
            subprocess.run([binary], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, timeout=30)
            return binary
        except OSError:
            pass
    _run(["bash", script, ref])
    return binary


def build_all(verbose=False):
    lib = build_product(verbose)
    build_oracle()
    try:
        build_reference()
    except RuntimeError as e:  # the reference is a checker; the product does not depend on it
        sys.stderr.write("warning: reference build failed: %s\n" % str(e)[:2000])
    return lib


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built", LIB)
