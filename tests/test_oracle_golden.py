"""The oracle restatement against the reference's own compiled math.

tests/golden/ref_math_golden.npz holds outputs of the reference's headers
(random.cuh, disney_hair.cuh, frostbite_anisotropic.cuh, curve_utils.cuh,
utils.cuh) compiled unmodified on the host (tests/golden/make_golden.py).  The
oracle must reproduce every value bit for bit on the same CPU.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

HAIR_SETS = ["c1", "dark", "smooth_gain", "thin"]


def bits_equal(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return np.array_equal(a.view(np.uint32), b.view(np.uint32)) or np.array_equal(a, b)


def test_rng_streams_bit_exact(golden):
    L = po.lib()
    for i in range(len(golden["rng_frame"])):
        s = L.hmo_get_rng(int(golden["rng_frame"][i]) + 10007, int(golden["rng_px"][i]),
                          int(golden["rng_py"][i]), 512, 512)
        assert s == golden["rng_state"][i]
        draws, end = po.lcg_stream(s, 32)
        assert bits_equal(draws, golden["rng_draws"][i])
        assert end == golden["rng_end"][i]


@pytest.fixture(autouse=True)
def _reference_fp32_mode():
    # the reference keeps the M_p log branch in FP32 for every beta_m
    po.set_mp_force_fp32(True)
    yield
    po.set_mp_force_fp32(False)


@pytest.mark.parametrize("name", HAIR_SETS)
def test_setup_hair_shading(golden, name):
    assert bits_equal(po.setup_hair(golden[f"{name}_hp"]), golden[f"{name}_setup"])


@pytest.mark.parametrize("name", HAIR_SETS)
def test_hair_eval_bit_exact(golden, name):
    g = lambda k: golden[f"{name}_{k}"]
    f, pdf = po.hair_eval(g("wo"), g("wi"), g("t"), g("h_used"), g("hp"))
    assert bits_equal(f, g("f"))
    assert bits_equal(pdf, g("pdf"))


@pytest.mark.parametrize("name", HAIR_SETS)
def test_hair_sample_bit_exact(golden, name):
    g = lambda k: golden[f"{name}_{k}"]
    wi, f, pdf, _ = po.hair_sample(g("wo"), g("t"), g("s_h_used"), g("u"), g("hp"))
    assert bits_equal(wi, g("s_wi"))
    assert bits_equal(f, g("s_f"))
    assert bits_equal(pdf, g("s_pdf"))


def test_ggx_bit_exact(golden):
    L = po.lib()
    n = len(golden["ggx_alpha"])
    for i in range(n):
        wo, wi = golden["ggx_wo"][i], golden["ggx_wi"][i]
        a = float(golden["ggx_alpha"][i])
        f = np.zeros(3, np.float32)
        L.hmo_frostbite_ggx(wo, wi, golden["ggx_color"][i], a, f)
        assert bits_equal(f, golden["ggx_f"][i])
        l_out = np.zeros(3, np.float32)
        p = np.zeros(1, np.float32)
        L.hmo_sample_ggx(golden["ggx_r2"][i], a, wo, l_out, p)
        assert bits_equal(l_out, golden["ggx_L"][i])
        assert bits_equal(p, golden["ggx_pdf"][i:i + 1])
        hv = wo + wi
        hv = np.ascontiguousarray((hv / np.linalg.norm(hv)).astype(np.float32))
        assert bits_equal(np.float32(L.hmo_pdf_ggx(a, wo, hv)), golden["ggx_hvec_pdf"][i])


def test_catmull_rom_curve_bit_exact(golden):
    L = po.lib()
    for i in range(len(golden["crv_u"])):
        out = np.zeros(24, np.float32)
        L.hmo_curve_eval(1, golden["crv_q"][i], float(golden["crv_u"][i]), golden["crv_ps"][i], out)
        assert bits_equal(out, golden["crv_out"][i]), i


def test_utils_bit_exact(golden):
    L = po.lib()
    for i in range(len(golden["ut_theta"])):
        b = np.zeros(18, np.float32)
        L.hmo_orthonormal_basis(golden["ut_n"][i], b)
        assert bits_equal(b, golden["ut_basis"][i])
        s = np.zeros(3, np.float32)
        L.hmo_uniform_sample_sphere(golden["ut_u2"][i], s)
        assert bits_equal(s, golden["ut_sphere"][i])
        assert bits_equal(np.float32(L.hmo_spherical_theta(golden["ut_n"][i])), golden["ut_theta"][i])
        assert bits_equal(np.float32(L.hmo_spherical_phi(golden["ut_n"][i])), golden["ut_phi"][i])
        assert bits_equal(np.float32(L.hmo_luminance(golden["ut_rgb"][i])), golden["ut_lum"][i])
        pw = L.hmo_power_heuristic(float(golden["ut_rgb"][i, 0]), float(golden["ut_rgb"][i, 1]))
        assert bits_equal(np.float32(pw), golden["ut_power"][i])


def test_fp64_mp_branch_close_to_fp32_reference(golden):
    """beta_m < 0.1: the oracle's FP64 M_p branch differs from the reference's
    FP32 branch only by FP32 rounding (the reason FP64 is used there)."""
    po.set_mp_force_fp32(False)
    g = lambda k: golden[f"thin_{k}"]
    f, pdf = po.hair_eval(g("wo"), g("wi"), g("t"), g("h_used"), g("hp"))
    ref = g("f")
    scale = np.maximum(np.abs(ref), 1e-6 * np.abs(ref).max())
    assert np.max(np.abs(f - ref) / scale) < 2e-3
    assert not bits_equal(f, ref)  # the FP64 branch is really taken
