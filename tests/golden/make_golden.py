"""Generate tests/golden/*.npz from the reference's OWN code.

The reference's header-only device math (random.cuh, disney_hair.cuh,
frostbite_anisotropic.cuh, curve_utils.cuh, utils.cuh) is compiled unmodified
on the host by oracle/build.py (build_ref) through the OWL/OptiX stand-ins in
oracle/ref_shim/, and called here through ctypes on seeded inputs.  The
outputs are the golden vectors the oracle restatement and the GPU kernels are
checked against.  Needs the reference checkout (where oracle/build.py looks
for it, or HM_REF_DIR); run:  python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import build as obuild  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def load_ref():
    libs = obuild.build_ref(verbose=True)
    path = [p for p in libs if p.endswith("libhmref_math.so")][0]
    L = ctypes.CDLL(path)
    i32, u32, f32 = ctypes.c_int, ctypes.c_uint32, ctypes.c_float
    L.ref_get_rng.restype = u32
    L.ref_get_rng.argtypes = [i32, u32, u32, u32, u32]
    L.ref_lcg_stream.restype = u32
    L.ref_lcg_stream.argtypes = [u32, i32, F32P]
    L.ref_setup_hair.argtypes = [F32P, F32P]
    L.ref_hair_eval.argtypes = [i32, F32P, F32P, F32P, F32P, F32P, F32P, F32P, F32P]
    L.ref_hair_sample.argtypes = [i32, F32P, F32P, F32P, F32P, F32P, F32P, F32P, F32P, F32P]
    L.ref_frostbite_ggx.argtypes = [F32P, F32P, F32P, f32, F32P]
    L.ref_sample_ggx.argtypes = [F32P, f32, F32P, F32P, F32P]
    L.ref_pdf_ggx.restype = f32
    L.ref_pdf_ggx.argtypes = [f32, F32P, F32P]
    L.ref_catrom_eval.argtypes = [F32P, f32, F32P, F32P]
    L.ref_orthonormal_basis.argtypes = [F32P, F32P]
    L.ref_uniform_sample_sphere.argtypes = [F32P, F32P]
    L.ref_power_heuristic.restype = f32
    L.ref_power_heuristic.argtypes = [f32, f32]
    for n in ("ref_luminance", "ref_spherical_theta", "ref_spherical_phi"):
        getattr(L, n).restype = f32
        getattr(L, n).argtypes = [F32P]
    return L


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


# Hair parameter sets: sigma_a[3], beta_m, beta_n, alpha(rad), gains R, TT, TRT, TRRT.
# alpha = 3.14159 * deg / 180 exactly as the scene parser (scene.cpp:207).
def hair_sets():
    d2r = lambda d: np.float32(np.float32(3.14159) * np.float32(d) / np.float32(180.0))
    return {
        "c1": np.array([0.06, 0.1, 0.2, 0.3, 0.3, d2r(2.0), 1, 1, 1, 1], np.float32),
        "dark": np.array([0.5, 0.8, 1.4, 0.45, 0.6, d2r(3.0), 1, 1, 1, 1], np.float32),
        "smooth_gain": np.array([0.02, 0.03, 0.05, 0.2, 0.15, d2r(0.0), 0.5, 1.5, 2.0, 0.7], np.float32),
        # beta_m < 0.1: the reference keeps FP32 here (oracle FP64 mode is compared separately)
        "thin": np.array([0.06, 0.1, 0.2, 0.08, 0.3, d2r(2.0), 1, 1, 1, 1], np.float32),
    }


def make_bsdf(L, rng, n=1024):
    out = {}
    for name, hp in hair_sets().items():
        wo, wi, t = unit(rng, n), unit(rng, n), unit(rng, n)
        h = rng.uniform(-1, 1, n).astype(np.float32)
        # include the edge cases the sampler clamps: u.y below 1e-5, u.w at 0
        u = rng.uniform(0, 1, (n, 4)).astype(np.float32)
        u[:8, 1] = np.float32(1e-7)
        u[8:16, 3] = 0.0
        u[16:24, 0] = np.float32(0.9999999)
        f = np.zeros((n, 3), np.float32)
        pdf = np.zeros(n, np.float32)
        hu = np.zeros(n, np.float32)
        L.ref_hair_eval(n, wo, wi, t, h, hp, f, pdf, hu)
        swi = np.zeros((n, 3), np.float32)
        sf = np.zeros((n, 3), np.float32)
        spdf = np.zeros(n, np.float32)
        shu = np.zeros(n, np.float32)
        L.ref_hair_sample(n, wo, t, h, u, hp, swi, sf, spdf, shu)
        setup = np.zeros(10, np.float32)
        L.ref_setup_hair(hp, setup)
        for k, v in dict(hp=hp, wo=wo, wi=wi, t=t, h_used=hu, u=u, f=f, pdf=pdf, setup=setup,
                         s_wi=swi, s_f=sf, s_pdf=spdf, s_h_used=shu).items():
            out[f"{name}_{k}"] = v
    return out


def make_rng(L, rng):
    frames = rng.integers(0, 100000, 64).astype(np.int32)
    px = rng.integers(0, 2048, 64).astype(np.uint32)
    py = rng.integers(0, 2048, 64).astype(np.uint32)
    states = np.zeros(64, np.uint32)
    draws = np.zeros((64, 32), np.float32)
    ends = np.zeros(64, np.uint32)
    for i in range(64):
        s = L.ref_get_rng(int(frames[i]) + 10007, int(px[i]), int(py[i]), 512, 512)
        states[i] = s
        ends[i] = L.ref_lcg_stream(s, 32, draws[i])
    return dict(rng_frame=frames, rng_px=px, rng_py=py, rng_state=states, rng_draws=draws,
                rng_end=ends)


def make_ggx(L, rng, n=512):
    wo = unit(rng, n)
    wo[:, 2] = np.abs(wo[:, 2])
    wi = unit(rng, n)
    color = rng.uniform(0, 1, (n, 3)).astype(np.float32)
    alpha = rng.uniform(0.01, 1.0, n).astype(np.float32) ** 2
    r2 = rng.uniform(0, 1, (n, 2)).astype(np.float32)
    f = np.zeros((n, 3), np.float32)
    L_ = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    pdf2 = np.zeros(n, np.float32)
    for i in range(n):
        L.ref_frostbite_ggx(wo[i], wi[i], color[i], float(alpha[i]), f[i])
        p = np.zeros(1, np.float32)
        L.ref_sample_ggx(r2[i], float(alpha[i]), wo[i], L_[i], p)
        pdf[i] = p[0]
        hvec = wo[i] + wi[i]
        hvec = (hvec / np.linalg.norm(hvec)).astype(np.float32)
        pdf2[i] = L.ref_pdf_ggx(float(alpha[i]), wo[i], np.ascontiguousarray(hvec))
    return dict(ggx_wo=wo, ggx_wi=wi, ggx_color=color, ggx_alpha=alpha, ggx_r2=r2, ggx_f=f,
                ggx_L=L_, ggx_pdf=pdf, ggx_hvec_pdf=pdf2)


def make_curves(L, rng, n=256):
    q = np.zeros((n, 16), np.float32)
    base = rng.normal(size=(n, 3))
    for k in range(4):
        q[:, 4 * k:4 * k + 3] = base + k * 0.1 + rng.normal(scale=0.02, size=(n, 3))
        q[:, 4 * k + 3] = rng.uniform(1e-3, 5e-3, n)
    u = rng.uniform(0, 1, n).astype(np.float32)
    u[:4] = 0.0
    u[4:8] = 1.0
    ps = (q[:, 4:7] + rng.normal(scale=0.01, size=(n, 3))).astype(np.float32)
    out = np.zeros((n, 24), np.float32)
    for i in range(n):
        L.ref_catrom_eval(q[i], float(u[i]), ps[i], out[i])
    return dict(crv_q=q, crv_u=u, crv_ps=ps, crv_out=out)


def make_utils(L, rng, n=256):
    nrm = unit(rng, n)
    nrm[0] = [0, 0, -1]
    nrm[1] = [0, 0, 1]
    basis = np.zeros((n, 18), np.float32)
    u2 = rng.uniform(0, 1, (n, 2)).astype(np.float32)
    sph = np.zeros((n, 3), np.float32)
    th = np.zeros(n, np.float32)
    ph = np.zeros(n, np.float32)
    lum = np.zeros(n, np.float32)
    rgb = rng.uniform(0, 2, (n, 3)).astype(np.float32)
    pw = np.zeros(n, np.float32)
    for i in range(n):
        L.ref_orthonormal_basis(nrm[i], basis[i])
        L.ref_uniform_sample_sphere(u2[i], sph[i])
        th[i] = L.ref_spherical_theta(nrm[i])
        ph[i] = L.ref_spherical_phi(nrm[i])
        lum[i] = L.ref_luminance(rgb[i])
        pw[i] = L.ref_power_heuristic(float(rgb[i, 0]), float(rgb[i, 1]))
    return dict(ut_n=nrm, ut_basis=basis, ut_u2=u2, ut_sphere=sph, ut_theta=th, ut_phi=ph,
                ut_rgb=rgb, ut_lum=lum, ut_power=pw)


def main():
    L = load_ref()
    rng = np.random.default_rng(20230605)
    data = {}
    data.update(make_rng(L, rng))
    data.update(make_bsdf(L, rng))
    data.update(make_ggx(L, rng))
    data.update(make_curves(L, rng))
    data.update(make_utils(L, rng))
    path = os.path.join(OUT, "ref_math_golden.npz")
    np.savez_compressed(path, **data)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
