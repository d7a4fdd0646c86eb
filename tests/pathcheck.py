"""Per-path comparison of GPU paths with the oracle's (shared by the GPU
parity tests; see tests/test_gpu_paths.py for the criterion).

Logs are [P, slots, 12] float32 in the GPU's slot layout (slot 3k + j:
vertex k's extension ray j = 0, light-sample shadow ray 1, BSDF-sample shadow
ray 2): result (int bits), t, u, RNG state (uint bits), direction[3], kind
(int bits, -1 empty), origin[3], 0.
"""
import os

import numpy as np

from oracle import pyoracle as po

FINE = 2e-6            # rays (origin, direction) and hits (t relative, u) equal within this
COLOR_RTOL = 1e-5      # |gpu - oracle| <= COLOR_RTOL * |oracle| + COLOR_ATOL + SPREAD_K * spread
COLOR_ATOL = 1e-7
SPREAD_K = 2.0
PERTURBED = (1, -1, 2, 3, 4, 5)
SEPARATE_MAX = 0.06    # fraction of paths whose log separates from the oracle's (and no more than the
                       # oracle's perturbed runs separate from its own)
UNEXPLAINED_MAX = 0    # separated paths neither separated by the perturbed oracle runs nor within the bar


def oracle_slots(ev, nev, slots):
    """The oracle's sequential ray log [P, E, 12] (kind, result, t, u, o, d,
    rng, 0) in the GPU's slot layout [P, slots, 12] (result, t, u, rng, d,
    kind, o, 0); empty slots have kind -1."""
    P, E, _ = ev.shape
    out = np.zeros((P, slots, 12), np.float32)
    out.view(np.int32)[:, :, 7] = -1
    kind = ev[:, :, 0].view(np.int32)
    valid = np.arange(E)[None, :] < np.minimum(nev, E)[:, None]
    vert = np.cumsum((kind == 0) & valid, axis=1) - 1
    slot = 3 * vert + kind
    p_idx, e_idx = np.nonzero(valid & (slot < slots))
    s_idx = slot[p_idx, e_idx]
    src = ev[p_idx, e_idx]
    out[p_idx, s_idx] = np.stack([src[:, 1], src[:, 2], src[:, 3], src[:, 10], src[:, 7], src[:, 8], src[:, 9],
                                  src[:, 0], src[:, 4], src[:, 5], src[:, 6], src[:, 11]], axis=1)
    return out


def separation(a, b, tol=FINE):
    """Per path: do logs a and b agree within tol everywhere, and the first
    slot where they do not (slot count if they agree)."""
    ai, bi = a.view(np.int32), b.view(np.int32)
    ak = ai[:, :, 7]
    empty = (ak == -1) & (bi[:, :, 7] == -1)
    ext = ak == 0
    same = (ak == bi[:, :, 7]) & (ai[:, :, 0] == bi[:, :, 0])
    same &= ~ext | (ai[:, :, 3] == bi[:, :, 3])
    same &= ~ext | (np.abs(a[:, :, 1] - b[:, :, 1]) <= tol * np.abs(b[:, :, 1]) + tol)
    same &= ~ext | (np.abs(a[:, :, 2] - b[:, :, 2]) <= tol)
    same &= np.abs(a[:, :, 4:7] - b[:, :, 4:7]).max(-1) <= tol
    same &= np.abs(a[:, :, 8:11] - b[:, :, 8:11]).max(-1) <= tol
    ok = empty | same
    agree = ok.all(1)
    first = np.where(agree, a.shape[1], np.argmin(ok, axis=1))
    return agree, first


def oracle_runs(o, mode, max_events, **kw):
    """The oracle's frame (render_pixels_ev) unperturbed (key 0) and under
    each PERTURBED ulp setting."""
    runs = {}
    for k in (0,) + PERTURBED:
        po.set_ulp_perturb(k)
        try:
            col, nn_in, train, flags, ev, nev, _ = o.render_pixels_ev(mode, max_events=max_events, **kw)
        finally:
            po.set_ulp_perturb(0)
        runs[k] = dict(col=col.astype(np.float64), nn_in=nn_in, train=train.astype(np.float64), flags=flags,
                       log=oracle_slots(ev, nev, max_events), nev=nev)
    return runs


def traingen_oracle_runs(o, points, max_events, **kw):
    """oracle_runs for the scene-sample training pass
    (OracleScene.render_traingen_ev over records aiming at `points`); `col`
    holds each record's training target."""
    runs = {}
    for k in (0,) + PERTURBED:
        po.set_ulp_perturb(k)
        try:
            tin, tout, flags, ev, nev, _ = o.render_traingen_ev(points, max_events=max_events, **kw)
        finally:
            po.set_ulp_perturb(0)
        runs[k] = dict(col=tout.astype(np.float64), train_in=tin, flags=flags,
                       log=oracle_slots(ev, nev, max_events), nev=nev)
    return runs


def nrc_oracle_runs(o, max_events, every_nth, n_train, accum_id=0, c=0.01):
    """oracle_runs for the NRC G_BUFFER pass (OracleScene.render_nrc); `col`
    holds each path's G-buffer (radiance, throughput at the cache query),
    its cache-query row and, for a training pixel, its suffix's query row."""
    runs = {}
    for k in (0,) + PERTURBED:
        po.set_ulp_perturb(k)
        try:
            out = o.render_nrc(accum_id=accum_id, every_nth=every_nth, n_train=n_train, c=c, max_events=max_events)
        finally:
            po.set_ulp_perturb(0)
        col = np.concatenate([out["gbuf"][:, :6], out["query"], out["suffix_query"]], 1).astype(np.float64)
        runs[k] = dict(col=col, records=out["records"].astype(np.float64), tinfo=out["tinfo"],
                       hit=out["gbuf"][:, 6], log=oracle_slots(out["events"], out["n_events"], max_events),
                       nev=out["n_events"])
    return runs


def spread_of(runs, key):
    """Per path (and channel): how far the perturbed oracle runs move `key`."""
    o0 = runs[0][key]
    return np.max([np.abs(runs[k][key] - o0) for k in PERTURBED], axis=0)


def color_excess(got, ref, spread, extra=0.0):
    """> 0 where `got` misses the bar around `ref` (extra: an added
    tolerance, e.g. hit_normal_tolerance for surface normals)."""
    return np.abs(got - ref) - (COLOR_RTOL * np.abs(ref) + COLOR_ATOL + SPREAD_K * spread + extra)


def hit_normal_tolerance(g_log, o_log, radius):
    """Per path: how far a hair normal may turn between the two logs' hits.
    The normal points from the fibre's axis to the hit point, so a hit point
    that moves by dp along a fibre of radius r turns it by up to dp / r; dp
    is bounded by the largest difference of the extension hits' distance,
    direction (times t) and origin.  Four times that, in each component."""
    ext = g_log.view(np.int32)[:, :, 7] == 0
    t = np.abs(o_log[:, :, 1])
    dp = np.abs(g_log[:, :, 1] - o_log[:, :, 1]) + t * np.abs(g_log[:, :, 4:7] - o_log[:, :, 4:7]).max(-1) + \
        np.abs(g_log[:, :, 8:11] - o_log[:, :, 8:11]).max(-1)
    dp = np.where(ext & np.isfinite(dp), dp, 0.0).max(1)
    return 4.0 * dp / radius


def check_paths(g_log, g_col, runs, label, dump=None, extra_tol=0.0, separate_max=SEPARATE_MAX):
    """Applies the per-path criterion; returns the paths whose logs agree.
    extra_tol [P, m] (or a scalar): an added tolerance per path and column;
    separate_max: the cap on the fraction of separating paths."""
    o0 = runs[0]
    agree, first = separation(g_log, o0["log"])
    self_sep = np.zeros(len(agree), bool)
    for k in PERTURBED:
        self_sep |= ~separation(runs[k]["log"], o0["log"])[0]
    spread = spread_of(runs, "col")
    excess = color_excess(g_col, o0["col"], spread, extra_tol).max(1)
    strict = (np.abs(g_col - o0["col"]) <= COLOR_RTOL * np.abs(o0["col"]) + COLOR_ATOL).all(1)
    sep = ~agree
    unexplained = sep & ~self_sep & (excess > 0)
    bad = agree & (excess > 0)
    print(f"{label}: {len(agree)} paths; {sep.sum()} separate ({sep.mean():.3%}; the oracle's perturbed runs "
          f"separate {self_sep.mean():.3%} of its own), {unexplained.sum()} unexplained; of the others "
          f"{(agree & strict).sum()} within {COLOR_RTOL:g} relative, {(agree & ~strict).sum()} within the spread "
          f"bar, {bad.sum()} beyond it")
    if dump:
        os.makedirs(dump, exist_ok=True)
        np.savez_compressed(os.path.join(dump, label.replace(" ", "_").replace("=", "") + ".npz"), g_log=g_log,
                            g_col=g_col, **{f"o{k}_{n}": runs[k][n] for k in runs for n in ("log", "col", "nev")})
    assert not bad.any(), (label, np.nonzero(bad)[0][:10], excess[bad].max())
    assert sep.mean() <= min(separate_max, self_sep.mean()), (label, sep.mean(), self_sep.mean())
    assert unexplained.sum() <= UNEXPLAINED_MAX, (label, np.nonzero(unexplained)[0][:10], first[unexplained][:10])
    return agree
