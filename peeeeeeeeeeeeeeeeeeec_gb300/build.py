"""Build the native libraries in-tree.

  libpeec_gb300.so   the sm_103a drop-in library (nvcc, one -gencode)
  libpeec_mesh.so    host-only synthetic mesher (gcc)
  oracle/liboracle.so and, when the reference's sources are present (staged
  into baseline/_ref/ by `make -C oracle stage`, which travels with the
  working tree), oracle/_ref/libpeec_ref*.so   the CPU checkers and the
  reference's own CPU build (make -C oracle)

Translation units compile in parallel; no cmake.  Host code is portable C
(no -march=native), so the same sources build on x86-64 and aarch64.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(REPO, "include")
ORACLE = os.path.join(REPO, "oracle")
STAGED_REFERENCE = os.path.join(REPO, "baseline", "_ref")

CUDA_SOURCES = ["runtime.cu", "assembly.cu", "lu.cu", "potential_helpers.cu", "harmonic.cu", "mixed.cu", "server.cu", "transient.cu", "rcs.cu", "incidence.cu", "matrix_export.cu", "sweep.cu", "multirhs.cu"]
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
    "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills",
    "-I" + INCLUDE, "-I" + CSRC,
]


def _nvcc():
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda_home, "bin", "nvcc")
    return path if os.path.exists(path) else (shutil.which("nvcc") or "nvcc")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def build_gpu_lib(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    sources = [s for s in CUDA_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = []

    def compile_one(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if _stale(o, [s] + headers):
            out = _run([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
            if verbose and out.strip():
                print(out)
        return o

    with cf.ThreadPoolExecutor(max_workers=len(sources)) as ex:
        objs = list(ex.map(compile_one, sources))
    lib = os.path.join(PKG, "libpeec_gb300.so")
    if _stale(lib, objs):
        _run([nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", lib] + objs
             + ["-lcudart"])
    return lib


def build_mesh_lib():
    src = os.path.join(CSRC, "meshgen.c")
    lib = os.path.join(PKG, "libpeec_mesh.so")
    if _stale(lib, [src] + _headers()):
        _run(["gcc", "-std=c17", "-O2", "-fPIC", "-shared", "-Wall", "-o", lib, src, "-lm"])
    return lib


def build_oracle():
    _run(["make", "-s", "-C", ORACLE, "all"])
    # refresh the staged copy where the reference is readable (the recipe
    # knows where), then build the reference from the staged copy
    ref = os.environ.get("PEEC_REFERENCE_DIR")
    _run(["make", "-s", "-C", ORACLE, "stage"] + (["REF=" + ref] if ref else []))
    if os.path.isdir(os.path.join(STAGED_REFERENCE, "src")):
        _run(["make", "-s", "-C", ORACLE, "ref"])


def build_all(verbose=False):
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_gpu_lib, verbose), ex.submit(build_mesh_lib), ex.submit(build_oracle)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built")
