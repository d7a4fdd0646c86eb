"""In-tree build of libhairmsnn.so for GB300 (sm_103a only).

Every CUDA translation unit in csrc/ is compiled in parallel with
  nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3
and linked into hairmsnn_gb300/_lib/libhairmsnn.so with the static CUDA
runtime, so the library loads next to any PyTorch build without a system
libcudart.  Rebuilds only what changed (header changes rebuild everything).
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB_PATH = os.path.join(OUT_DIR, "libhairmsnn.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without multiply-add contraction (g++ contracts by
# default on aarch64 but not on x86-64): the procedural scenes, BVH builds and
# environment tables come out the same on both.
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-ffp-contract=off",
                     "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills",
                     "-I", os.path.join(ROOT, "include"), "-I", CSRC]


# Shading translation units evaluate ill-conditioned expressions of the
# reference's formulas (1 - sin^2 near grazing angles, cross products of
# nearly parallel vectors, exp(cos/v) with 1/v up to ~1e3): they are compiled
# without multiply-add contraction so every non-transcendental operation is
# rounded exactly as the reference's separately rounded operations.
PER_FILE_FLAGS = {
    "hm_bsdf.cu": ["-fmad=false"],
    "hm_shade.cu": ["-fmad=false"],
    "hm_nrc.cu": ["-fmad=false"],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.isfile(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h")) + glob.glob(os.path.join(ROOT, "include", "*.cuh"))


def _compile(src, newest_header, verbose, extra):
    obj = os.path.join(OBJ_DIR, os.path.basename(src) + ".o")
    if os.path.isfile(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), newest_header):
        return obj, False
    cmd = [nvcc(), *NVCC_FLAGS, *PER_FILE_FLAGS.get(os.path.basename(src), []), *extra, "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    return obj, True


def build(verbose: bool = False, extra_flags=()) -> str:
    """Compile csrc/*.cu and link libhairmsnn.so; returns the library path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    newest = max([os.path.getmtime(h) for h in _headers()] + [os.path.getmtime(__file__)])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, newest, verbose, list(extra_flags)), srcs))
    objs = [o for o, _ in results]
    changed = any(c for _, c in results)
    if changed or not os.path.isfile(LIB_PATH):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread", "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
