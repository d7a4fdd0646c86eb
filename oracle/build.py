"""Build recipes for the ORACLE (test infrastructure only).

* build_oracle(): oracle/hm_oracle*.cpp -> oracle/_build/libhmoracle.so, the
  CPU restatement that tests/, smoke() and bench.py's CPU-baseline leg use as
  the checker.  Plain g++, -ffp-contract=off, no CUDA.
* build_ref(): the reference's own code compiled unmodified on the host
  through the stand-ins in oracle/ref_shim/ (OWL / OptiX names, cyHairFile,
  nlohmann::json), into oracle/_ref/ (git-ignored): its header-only device
  math, its integrators (hair_msnn.cu, path_tracing.cu, nrc.cu) and its
  scene.cpp.  It pins the oracle restatement and makes the
  golden vectors under tests/golden/.  It needs the reference checkout
  (HM_REF_DIR, default /root/reference); where that is absent it is skipped
  and the committed golden vectors stand in for it.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("HM_REF_DIR", "/root/reference")
OUT_DIR = os.path.join(HERE, "_ref")
ORACLE_DIR = os.path.join(HERE, "_build")
ORACLE_LIB = os.path.join(ORACLE_DIR, "libhmoracle.so")
ORACLE_SOURCES = ["hm_oracle.cpp", "hm_oracle_render.cpp", "hm_oracle_mlp.cpp", "hm_oracle_scene.cpp"]
ORACLE_HEADERS = ["hm_oracle.h", "hm_oracle_math.h"]


def _stale(out, deps):
    if not os.path.isfile(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.isfile(d))


def build_oracle(verbose: bool = False) -> str:
    """Compile the oracle restatement into oracle/_build/libhmoracle.so."""
    os.makedirs(ORACLE_DIR, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in ORACLE_SOURCES]
    deps = srcs + [os.path.join(HERE, h) for h in ORACLE_HEADERS]
    if _stale(ORACLE_LIB, deps):
        tmp = ORACLE_LIB + ".tmp%d" % os.getpid()
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
               "-fno-fast-math", "-I", HERE, *srcs, "-o", tmp, "-lpthread"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB

# (output library, entry source, extra flags, links the oracle library).
# The integrator targets include the reference's own raygen sources
# (cuda/hair_msnn.cu, cuda/path_tracing.cu, cuda/nrc.cu); __CUDA_ARCH__ is defined only so
# that common.cuh declares its ray types (common.cuh:28-32), and traceRay is
# answered by the oracle library's BVH.
TARGETS = [
    ("libhmref_math.so", "ref_math_entry.cpp", [], False),
    ("libhmref_path.so", "ref_path_entry.cpp", ["-D__CUDA_ARCH__=860"], True),
    ("libhmref_pt.so", "ref_pt_entry.cpp", ["-D__CUDA_ARCH__=860"], True),
    ("libhmref_nrc.so", "ref_nrc_entry.cpp", ["-D__CUDA_ARCH__=860"], True),
    # scene.cpp (parseScene, extractHairData, generateEnvSamplingTables) with
    # stand-ins for cyHairFile and nlohmann::json
    ("libhmref_scene.so", "ref_scene_entry.cpp", [], False),
]


def ref_available() -> bool:
    return os.path.isfile(os.path.join(REF_DIR, "cuda_headers", "disney_hair.cuh"))


def build_ref(verbose: bool = False) -> list:
    """Compile every target whose entry source exists; returns built paths."""
    if not ref_available():
        if verbose:
            print("build_ref: reference checkout not found; skipped")
        return []
    os.makedirs(OUT_DIR, exist_ok=True)
    oracle_lib = build_oracle()
    built = []
    for lib, src, defs, link_oracle in TARGETS:
        src_path = os.path.join(HERE, "ref_shim", src)
        out = os.path.join(OUT_DIR, lib)
        deps = [src_path, os.path.join(HERE, "ref_shim", "hm_owl_shim.h"),
                os.path.join(HERE, "ref_shim", "ref_harness.h"), os.path.join(HERE, "ref_shim", "ref_eval_order.h"),
                os.path.join(HERE, "ref_shim", "cyHairFile.h"), os.path.join(HERE, "ref_shim", "json", "json.hpp"),
                os.path.join(HERE, "hm_oracle.h"), os.path.join(HERE, "hm_oracle.cpp")]
        if link_oracle:
            deps.append(oracle_lib)
        if not _stale(out, deps):
            built.append(out)
            continue
        link = ["-L", ORACLE_DIR, "-lhmoracle", "-Wl,-rpath,$ORIGIN/../_build"] if link_oracle else []
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
               "-fno-fast-math", "-fno-strict-aliasing", "-w", *defs,
               "-I", os.path.join(HERE, "ref_shim"), "-I", HERE,
               "-I", os.path.join(REF_DIR, "cuda_headers"), "-I", os.path.join(REF_DIR, "cuda"),
               "-I", os.path.join(REF_DIR, "headers"), "-I", REF_DIR,
               src_path, "-o", out, *link, "-Wl,-Bsymbolic", "-lpthread"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        built.append(out)
    return built


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_ref(verbose=True))
    sys.exit(0)
