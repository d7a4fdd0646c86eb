"""Differentiable rendering by path replay (hm_render_diff_forward / _backward).

* Strand groups whose materials all equal the scene's render the ungrouped
  image bit for bit, and a detached render at the scene's own materials is
  the plain render bit for bit.
* Material gradients: for every group and every parameter (sigma_a r, g, b,
  beta_m, beta_n, alpha) the replayed dL/dtheta of L = <A, image> (A a
  random adjoint) matches central finite differences (eps = 1e-3, image
  sums in FP64) of detached renders, whose sampling stays at the scene's
  materials, to 1e-2 |fd| + 1e-3 max |fd|; in HairMSNN mode (BETA = 2, the
  cache frozen) and in plain path tracing.  beta_m is kept >= 0.6, where
  every lobe's M_p takes the direct branch (v > 0.1): the log-space branch
  switches LogI0 at x = 12 (disney_hair.cuh:70-75), a step that
  differences across it count as slope.
* Cache weights: the directional derivative dL/dW . d for a random d
  (relative steps, eps = 1e-4) matches central differences of renders with
  W +- eps d to 1e-2.
* Replays are deterministic (bit-identical gradients), and a forward that
  cannot be replayed is refused.
* 60 Adam steps on sigma_a (2 groups, L2 image loss against a target
  rendered at the true materials) recover it from a +-50% start.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

EPS = 1e-3
PARAMS = ["sigma_a_r", "sigma_a_g", "sigma_a_b", "beta_m", "beta_n", "alpha"]


@pytest.fixture(scope="module")
def R():
    from hairmsnn_gb300 import build, render
    build.build()
    return render


def materials(n, seed=0):
    rng = np.random.default_rng(seed)
    m = np.zeros((n, 10), np.float32)
    m[:, 0:3] = rng.uniform(0.08, 0.5, (n, 3))
    m[:, 3] = rng.uniform(0.6, 0.75, n)
    m[:, 4] = rng.uniform(0.3, 0.6, n)
    m[:, 5] = np.deg2rad(rng.uniform(1.0, 4.0, n))
    m[:, 6:10] = 1.0
    return m


def diff_cfg(R, res=64, strands=1500, groups=2, path_v2=8, mats=None):
    """Curly hair; the scene material is mats[0], and `groups` azimuthal
    strand groups (0: none) take mats[g]."""
    cfg = R.straight_hair_scene(res, res, strands=strands, control_points=24, path_v2=path_v2, triangles=4000,
                                sky_w=128, sky_h=64)
    p = cfg["hair"]["procedural"]
    p["type"] = "curly"
    p["helix_radius"] = 0.05
    p["helix_pitch"] = 0.2
    m = materials(max(groups, 1)) if mats is None else mats
    mat = lambda r: {"sigma_a": [float(x) for x in r[0:3]], "beta_m": float(r[3]), "beta_n": float(r[4]),
                     "alpha": float(np.rad2deg(r[5]))}
    cfg["hair"].update(mat(m[0]))
    if groups > 0:
        cfg["hair"]["groups"] = {"count": groups, "assign": "azimuth", "materials": [mat(r) for r in m]}
    return cfg


def make(R, mode, cfg, beta=2):
    s = R.Scene(cfg)
    r = R.Renderer(s, mode, beta=beta, train_records=1024, train=False, seed=3)
    return s, r


def test_groups_at_scene_material_and_detached_render_match_plain(R):
    m = materials(1)
    _, r1 = make(R, R.MSNN, diff_cfg(R, groups=0, mats=m))
    r1.diff_forward(4)
    ref = r1.read()
    s2, r2 = make(R, R.MSNN, diff_cfg(R, groups=3, mats=np.repeat(m, 3, axis=0)))
    r2.diff_forward(4)
    assert np.array_equal(r2.read(), ref)
    r2.diff_forward(4, eval_materials=s2.group_materials())
    assert np.array_equal(r2.read(), ref)


def loss_of(img, A):
    return float(np.sum(img * A))


@pytest.mark.parametrize("mode", ["msnn", "pt"])
def test_material_gradients_match_detached_finite_differences(R, mode):
    md = R.MSNN if mode == "msnn" else R.PT
    cfg = diff_cfg(R, groups=2)
    s, r = make(R, md, cfg)
    frames = 4
    A = np.random.default_rng(1).normal(size=(64, 64, 3))
    r.diff_forward(frames)
    grad = r.diff_backward(torch.from_numpy(A.astype(np.float32)).cuda())
    base = s.group_materials().astype(np.float64)
    fd = np.zeros((2, 6))
    for g in range(2):
        for k in range(6):
            vals = []
            for sgn in (1, -1):
                m = base.copy()
                m[g, k] += sgn * EPS
                r.diff_forward(frames, eval_materials=m)
                vals.append(loss_of(r.read(), A))
            fd[g, k] = (vals[0] - vals[1]) / (2 * EPS)
    tol = 1e-2 * np.abs(fd) + 1e-3 * np.abs(fd).max()
    bad = np.abs(grad - fd) > tol
    assert not bad.any(), (mode, grad, fd)


def test_cache_weight_gradient_matches_finite_differences(R):
    cfg = diff_cfg(R, groups=2)
    s, r = make(R, R.MSNN, cfg)
    net = r.cache()
    frames = 4
    A = np.random.default_rng(2).normal(size=(64, 64, 3))
    r.diff_forward(frames)
    r.diff_backward(torch.from_numpy(A.astype(np.float32)).cuda())
    dW = net.gradients().astype(np.float64)
    w0 = net.params().astype(np.float64)
    d = np.random.default_rng(3).normal(size=w0.shape) * (np.abs(w0) + 1e-2)
    # 1e-4 relative steps: at 1e-3 enough ReLU units change sign along d that
    # the central difference of the piecewise-linear network is 2% off
    eps = 1e-4
    vals = []
    for sgn in (1, -1):
        net.set_params((w0 + sgn * eps * d).astype(np.float32))
        r.diff_forward(frames)
        vals.append(loss_of(r.read(), A))
    net.set_params(w0.astype(np.float32))
    fd = (vals[0] - vals[1]) / (2 * eps)
    an = float(np.dot(dW, d))
    assert abs(an - fd) <= 1e-2 * abs(fd), (an, fd)


def test_replay_is_deterministic_and_guarded(R):
    cfg = diff_cfg(R, groups=2)
    s, r = make(R, R.MSNN, cfg)
    A = torch.randn(64, 64, 3, device="cuda")
    r.diff_forward(3)
    g1 = r.diff_backward(A)
    g2 = r.diff_backward(A)
    assert np.array_equal(g1, g2)
    assert np.isfinite(g1).all() and np.abs(g1).max() > 0
    r.diff_forward(3, eval_materials=s.group_materials())
    with pytest.raises(Exception):
        r.diff_backward(A)
    r.diff_forward(3)
    s.set_group_materials(s.group_materials())
    with pytest.raises(Exception):
        r.diff_backward(A)
    r.diff_forward(3)
    r.frame()
    with pytest.raises(Exception):
        r.diff_backward(A)


def test_sigma_a_fit_with_adam_recovers_materials(R):
    truth = materials(2, seed=5)
    cfg = diff_cfg(R, groups=2, mats=truth)
    s, r = make(R, R.MSNN, cfg)
    s.set_group_materials(truth)  # exact radians (the JSON's degrees convert with 3.14159)
    frames = 8
    r.diff_forward(frames)
    target = r.read()
    n = target.size
    start = truth.copy()
    start[:, 0:3] *= np.where(np.random.default_rng(6).random((2, 3)) < 0.5, 0.5, 1.5)
    x = torch.tensor(np.log(start[:, 0:3].astype(np.float64)), requires_grad=True)
    opt = torch.optim.Adam([x], lr=0.05)
    for _ in range(60):
        m = truth.copy()
        m[:, 0:3] = np.exp(x.detach().numpy())
        s.set_group_materials(m)
        r.diff_forward(frames)
        img = r.read()
        A = 2.0 * (img - target) / n
        g = r.diff_backward(torch.from_numpy(A.astype(np.float32)).cuda())
        opt.zero_grad()
        x.grad = torch.from_numpy(g[:, 0:3] * m[:, 0:3])  # d/d log(sigma_a)
        opt.step()
    err = np.abs(np.exp(x.detach().numpy()) - truth[:, 0:3]) / truth[:, 0:3]
    assert err.max() <= 0.05, err
