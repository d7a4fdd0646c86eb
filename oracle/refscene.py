"""ctypes front end of the reference's scene.cpp compiled on the host (test
infrastructure only): generateEnvSamplingTables, LoadCemYuksel +
Scene::extractHairData and parseScene, from oracle/_ref/libhmref_scene.so
(oracle/build.py build_ref, with the stand-ins of oracle/ref_shim/ for
cyHairFile and nlohmann::json).  Exists only where the reference checkout is
present; available() says whether it does.
"""
import ctypes
import os

import numpy as np

from . import build as _build

F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
I32P = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lib = []

# hmr_parse_scene's value slots
PARSE_FIELDS = ["from_x", "from_y", "from_z", "at_x", "at_y", "at_z", "up_x", "up_y", "up_z", "cos_fovy", "bsdf",
                "sigma_a_r", "sigma_a_g", "sigma_a_b", "beta_m", "beta_n", "alpha", "gain_r", "gain_tt", "gain_trt",
                "gain_trrt", "pixar_factor", "has_env", "env_scale", "env_rotation", "has_directional",
                "n_directional", "mis", "env_pdf", "spp", "path_v1", "path_v2", "width", "height", "init_train",
                "has_hair", "has_surface"]
PARSE_TEXT = ["image_output", "stats_output", "config", "config2", "init_weights", "dual_scatter_precomputation"]


def lib():
    if _lib:
        return _lib[0]
    path = os.path.join(_build.OUT_DIR, "libhmref_scene.so")
    if not os.path.isfile(path):
        if not _build.ref_available():
            _lib.append(None)
            return None
        _build.build_ref()
    L = ctypes.CDLL(path)
    i32, cp = ctypes.c_int, ctypes.c_char_p
    L.hmr_env_tables.restype = None
    L.hmr_env_tables.argtypes = [i32, i32, F32P, F32P, F32P, F32P, F32P]
    L.hmr_hair_file.restype = i32
    L.hmr_hair_file.argtypes = [cp, F32P, i32, I32P, i32, I32P, F32P]
    L.hmr_parse_scene.restype = i32
    L.hmr_parse_scene.argtypes = [cp, F32P, F32P, ctypes.c_char_p, i32]
    _lib.append(L)
    return L


def available():
    try:
        return lib() is not None
    except OSError:
        return False


def env_tables(env):
    """generateEnvSamplingTables of an RGBA map [h, w, 4]: dict cpdf, ccdf
    [h, w + 1], mpdf, mcdf [h + 1]."""
    env = np.ascontiguousarray(env, np.float32)
    h, w = env.shape[:2]
    out = dict(cpdf=np.zeros((h, w + 1), np.float32), ccdf=np.zeros((h, w + 1), np.float32),
               mpdf=np.zeros(h + 1, np.float32), mcdf=np.zeros(h + 1, np.float32))
    lib().hmr_env_tables(w, h, env, out["cpdf"], out["ccdf"], out["mpdf"], out["mcdf"])
    return out


def hair_file(path, cap=1 << 20):
    """LoadCemYuksel + extractHairData: dict cp [n, 4] (xyz, width),
    segments [m], strands, bounds [7] (min, max, scale); None if the file
    does not load."""
    cp = np.zeros((cap, 4), np.float32)
    seg = np.zeros(cap, np.int32)
    info = np.zeros(3, np.int32)
    bounds = np.zeros(7, np.float32)
    n = lib().hmr_hair_file(str(path).encode(), cp, cap, seg, cap, info, bounds)
    if n < 0:
        return None
    return dict(cp=cp[:info[0]].copy(), segments=seg[:info[1]].copy(), strands=int(info[2]), bounds=bounds)


def parse_scene(path):
    """parseScene on a scene file: (result, dict of PARSE_FIELDS and
    PARSE_TEXT, directional lights [k, 6] (from, emit)); result 1 / 0, or -1
    when the JSON text does not parse."""
    vals = np.zeros(40, np.float32)
    lights = np.zeros((8, 6), np.float32)
    text = ctypes.create_string_buffer(1 << 16)
    r = lib().hmr_parse_scene(str(path).encode(), vals, lights, text, len(text))
    out = {k: float(vals[i]) for i, k in enumerate(PARSE_FIELDS)}
    parts = text.raw.split(b"\0")
    for i, k in enumerate(PARSE_TEXT):
        out[k] = parts[i].decode() if i < len(parts) else ""
    return r, out, lights[:int(out["n_directional"])].copy()
