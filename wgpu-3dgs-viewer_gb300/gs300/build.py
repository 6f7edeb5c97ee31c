"""Build the CUDA library libgs300.so in-tree for sm_103a.

Each translation unit is compiled by its own nvcc process (in parallel), then linked into
gs300/libgs300.so.  Flags that matter for results:
  * -fmad=false: no multiply-add contraction in device code; the kernels spell out every FMA
    they want with fmaf(), so FP32 results follow one fixed evaluation order;
  * -Xcompiler -ffp-contract=off: the same for host code (the frame uniforms);
  * no fast-math: IEEE division and square root.
"""
import concurrent.futures
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)  # wgpu-3dgs-viewer_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD_DIR = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libgs300.so")
SOURCES = ["gs_api.cu", "gs_preprocess.cu", "gs_sort.cu", "gs_raster.cu", "gs_ply.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _flags(ptxas_verbose=False):
    f = ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
        "-I", INCLUDE, "-I", CSRC,
    ]
    if ptxas_verbose:
        f += ["-Xptxas", "-v"]
    return f


def _deps():
    out = [os.path.join(CSRC, s) for s in os.listdir(CSRC)]
    out += [os.path.join(INCLUDE, s) for s in os.listdir(INCLUDE)]
    out.append(os.path.abspath(__file__))
    return out


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False, ptxas_verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        cmd = [cc] + _flags(ptxas_verbose) + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if ptxas_verbose or verbose:
            sys.stderr.write(r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))
