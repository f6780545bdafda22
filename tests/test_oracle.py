"""The CPU oracle: the C restatement against the reference itself.

* MT19937 known answers (the generator every random draw of the reference
  goes through).
* Restatement vs the reference's own routines (oracle/_ref), bit for bit,
  on seeded systems -- runs where the reference sources are present.
* Restatement vs the golden fixtures made from the reference
  (tests/golden/) -- runs everywhere.
* Observables outside the step (acc_correl, oo_params) against both.
"""
import ctypes
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, load_golden
from mdspherocyl_gb300 import systems as S


def test_mt19937_known_answers(orc):
    rng = orc._rng_new(5489)
    try:
        first = orc._rng_u(rng) * 4294967296.0
        for _ in range(9998):
            orc._rng_u(rng)
        tenthousandth = orc._rng_u(rng) * 4294967296.0
    finally:
        orc._rng_free(rng)
    # init_genrand(5489): first output 3499211612; 10000th 4123659995 (the
    # value the C++ standard requires of std::mt19937)
    assert first == 3499211612.0
    assert tenthousandth == 4123659995.0
    # seed 0 is mapped to 4357 as GSL does
    a, b = orc._rng_new(0), orc._rng_new(4357)
    try:
        assert [orc._rng_u(a) for _ in range(5)] == [orc._rng_u(b) for _ in range(5)]
    finally:
        orc._rng_free(a)
        orc._rng_free(b)


def _sys(st, box):
    return oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, box)


def _systems():
    out = []
    spec, st = S.plain_c0(seed=5, n=48)
    out.append((st, spec.box, spec.alpha, spec.K_max, spec.ksq_max))
    rng = np.random.default_rng(6)
    st, box = S.make_system(n=40, phi=0.25, lengths=rng.uniform(1.5, 3.0, 40), mu=rng.uniform(0.5, 2, 40), seed=6)
    out.append((st, box, 5.5 / box[0], 5, 0))
    st, box = S.make_system(n=30, phi=0.1, lengths=np.full(30, 2.0), mu=np.full(30, 1.0), seed=7, aspect=(1.3, 0.8))
    dip = np.zeros((30, 2, 5))
    dip[:, 0] = [-0.6, 0.6, 0.8, 0.0, 1.2]
    dip[:, 1] = [0.4, 0.0, 0.0, 1.0, 0.7]
    st.dip = dip
    out.append((st, box, 4.0 / box[2], 4, 0))
    return out


@pytest.mark.parametrize("k", range(3))
def test_restatement_bitexact_vs_reference(ref, orc, k):
    st, box, alpha, K, ksq = _systems()[k]
    B = np.array([0.2, 0.5, -0.4])

    def both(fn):
        a, b = _sys(st, box), _sys(st, box)
        ra = fn(orc, a)
        rb = fn(ref, b)
        return a, b, ra, rb

    checks = {
        "force_sc": lambda o, s: o.force_sc(s, 3.0, 3.5),
        "force_dipR": lambda o, s: o.force_dipR(s, alpha),
        "force_dipK": lambda o, s: o.force_dipK(s, K, alpha, ksq),
        "force_dipK_sphere": lambda o, s: o.force_dipK(s, K, alpha, max(ksq, 2 * (K - 1) ** 2)),
        "ext_field": lambda o, s: o.ext_field(s, B),
        "moveX": lambda o, s: o.moveX(s, 1e-3),
        "moveP_first": lambda o, s: o.moveP(s, np.array([0.3, -0.1]), 1e-3, False),
        "moveP_last": lambda o, s: o.moveP(s, np.array([0.3, -0.1]), 1e-3, True),
        "renorm": lambda o, s: o.renorm(s),
        "self_ener": lambda o, s: o.self_ener(s),
    }
    for name, fn in checks.items():
        a, b, ra, rb = both(fn)
        for f in ("r", "p", "O", "l", "F", "T"):
            assert np.array_equal(getattr(a, f), getattr(b, f)), (name, f)
        fa = [np.ravel(np.asarray(x, dtype=float)) for x in (ra if isinstance(ra, tuple) else (ra,)) if x is not None]
        fb = [np.ravel(np.asarray(x, dtype=float)) for x in (rb if isinstance(rb, tuple) else (rb,)) if x is not None]
        for u, v in zip(fa, fb):
            assert np.array_equal(u, v), (name, u, v)


def test_seg_dist_special_cases_bitexact(ref, orc):
    """Parallel rods (all four end-point sentinels and the non-unique case),
    intersecting axis lines, and generic pairs."""
    n = 2
    base = dict(p=np.zeros((n, 3)), l=np.zeros((n, 3)), length=np.array([2.0, 3.0]), dia=np.ones(n),
                mass=np.ones(n), dip=np.zeros((n, 1, 5)))
    ez = np.eye(3)
    flip = np.array([[1, 0, 0], [0, -1, 0], [0, 0, -1.0]])
    tilt = np.array([[1, 0, 0], [0, 0.8, -0.6], [0, 0.6, 0.8]])
    cases = [
        (np.array([[0, 0, 0], [1.1, 0.25, 0]]), [ez, ez]),          # side by side (no unique pair)
        (np.array([[0, 0, 0], [0.3, 0, 3.0]]), [ez, ez]),           # end to end, same direction
        (np.array([[0, 0, 0], [0.3, 0, -3.0]]), [ez, ez]),
        (np.array([[0, 0, 0], [0.3, 0, 3.0]]), [ez, flip]),         # antiparallel, head to head
        (np.array([[0, 0, 0], [0.3, 0, -3.0]]), [ez, flip]),
        (np.array([[0, 0, 0], [0.0, 0, 0.5]]), [ez, tilt]),         # axis lines intersect
        (np.array([[0, 0, 0], [0.9, -0.4, 0.7]]), [ez, tilt]),
    ]
    for r, Os in cases:
        s = oracle.System(r, base["p"], np.stack(Os), base["l"], base["length"], base["dia"], base["mass"],
                          base["dip"], [20.0, 20.0, 20.0])
        a = orc.seg_dist(s, 0, 1)
        b = ref.seg_dist(s, 0, 1)
        assert a[0] == b[0] and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]), (r, a, b)


def test_clusters_and_neighbour_list_vs_reference(ref, orc):
    rng = np.random.default_rng(8)
    st, box = S.make_system(n=80, phi=0.22, lengths=rng.uniform(2, 3, 80), mu=np.ones(80), seed=8)
    for ms in (0.1, 0.5):
        a, b = _sys(st, box), _sys(st, box)
        la, nca, nxa = orc.clust_conf(a, ms, seed=3, skip=11)
        lb, nxb = ref.clust_conf(b, ms, seed=3, skip=11)
        assert np.array_equal(la, lb)
        assert nxa == nxb  # the same number of draws was taken
        assert nca == la.max() + 1
    ca, ia = orc.neigh_list(_sys(st, box), 3.0)
    cb, ib = ref.neigh_list(_sys(st, box), 3.0)
    assert np.array_equal(ca, cb) and np.array_equal(ia, ib)


def test_clusters_at_2048_rods_vs_reference(ref, orc):
    """The oracle's labelling visits only partners within reach of the
    geometric test; at 2048 dense polydisperse rods (many clusters, long
    rods beside short ones) the labels and the generator's position still
    equal the reference's, which tests every pair."""
    rng = np.random.default_rng(12)
    n = 2048
    st, box = S.make_system(n=n, phi=0.2, lengths=rng.uniform(2, 5, n), mu=np.ones(n), seed=12)
    for ms in (0.1, 0.8):
        la, nca, nxa = orc.clust_conf(_sys(st, box), ms, seed=4, skip=2)
        lb, nxb = ref.clust_conf(_sys(st, box), ms, seed=4, skip=2)
        assert np.array_equal(la, lb) and nxa == nxb and nca == la.max() + 1


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_restatement_matches_golden_fixtures(orc, path):
    g = load_golden(path)

    def mk():
        return oracle.System(g["r"], g["p"], g["O"], g["l"], g["length"], g["dia"], g["mass"], g["dip"], g["box"])

    alpha, K, ksq = float(g["alpha"]), int(g["K_max"]), int(g["ksq_max"])
    s = mk()
    ok, U, W, PT = orc.force_sc(s, 3.0, 3.5)
    assert ok == bool(g["sc_ok"])
    if ok:
        assert U == g["sc_U"] and W == g["sc_W"] and np.array_equal(PT, g["sc_PT"])
        assert np.array_equal(s.F, g["sc_F"]) and np.array_equal(s.T, g["sc_T"])
    s = mk()
    U, PT = orc.force_dipR(s, alpha)
    assert U == g["dipR_U"] and np.array_equal(PT, g["dipR_PT"])
    assert np.array_equal(s.F, g["dipR_F"]) and np.array_equal(s.T, g["dipR_T"])
    s = mk()
    U, PT = orc.force_dipK(s, K, alpha, ksq)
    assert U == g["dipK_U"] and np.array_equal(PT, g["dipK_PT"])
    assert np.array_equal(s.F, g["dipK_F"]) and np.array_equal(s.T, g["dipK_T"])
    s = mk()
    assert orc.ext_field(s, g["B"]) == g["ext_U"] and np.array_equal(s.T, g["ext_T"])
    assert orc.self_ener(mk()) == g["self_U"]
    for last in (0, 1):
        s = mk()
        s.F[:] = g["mp_F"]
        s.T[:] = g["mp_T"]
        K2, PT = orc.moveP(s, g["mp_xi"], float(g["dt"]), bool(last))
        assert np.array_equal(K2, g[f"mp{last}_K"]) and np.array_equal(PT, g[f"mp{last}_PT"])
        assert np.array_equal(s.p, g[f"mp{last}_p"]) and np.array_equal(s.l, g[f"mp{last}_l"])
    s = mk()
    orc.moveX(s, float(g["dt"]))
    assert np.array_equal(s.r, g["mx_r"]) and np.array_equal(s.O, g["mx_O"])
    s = mk()
    orc.renorm(s)
    assert np.array_equal(s.O, g["rn_O"])
    for ms in (0.1, 0.6):
        lab, nc, nxt = orc.clust_conf(mk(), ms, seed=1, skip=7)
        assert np.array_equal(lab, g[f"cl{ms}_labels"]) and nxt == g[f"cl{ms}_next"]
    counts, idx = orc.neigh_list(mk(), 3.5)
    assert np.array_equal(counts, g["nl_counts"]) and np.array_equal(idx, g["nl_idx"])
    _check_observables(orc, mk(), float(g["corr_bar_w"]), g["corr_hist"], g["oo_G1"], g["oo_G2"], g["oo_M"])


def _check_observables(orc, s, bar_w, hist, G1, G2, M):
    """acc_correl: counts exact, the other sums to FP64 rounding (the
    reference adds them under OpenMP atomics, in thread order); oo_params:
    M to FP64 rounding, G1 and G2 to 1e-6 (the reference's Q and its eigen
    solve are FP32, the restatement's solve is FP64)."""
    h = orc.acc_correl(s, bar_w, hist.shape[1])
    assert np.array_equal(h[0], hist[0])
    assert np.abs(h[1:] - hist[1:]).max() <= 1e-12 * max(1.0, hist[0].max())
    g1, g2, m = orc.oo_params(s)
    assert abs(g1 - G1) <= 1e-6 and abs(g2 - G2) <= 1e-6
    assert np.abs(m - M).max() <= 1e-12 * max(1.0, np.abs(M).max())


@pytest.mark.parametrize("k", range(3))
def test_observables_vs_reference(ref, orc, k):
    st, box, *_ = _systems()[k]
    bar_w = float(min(box)) / 150.0
    nbins = int(np.floor(np.sqrt(3.0) * float(min(box)) / (2.0 * bar_w)))
    hist = ref.acc_correl(_sys(st, box), bar_w, nbins)
    G1, G2, M = ref.oo_params(_sys(st, box))
    _check_observables(orc, _sys(st, box), bar_w, hist, G1, G2, M)
    # components: intra and inter histograms against the reference's own
    counts = [st.n // 3, st.n // 3, st.n - 2 * (st.n // 3)]
    hs = ref.acc_correl_species(_sys(st, box), counts, bar_w, nbins)
    ho = orc.acc_correl_species(_sys(st, box), counts, bar_w, nbins)
    assert np.array_equal(ho[:, 0], hs[:, 0])
    assert np.abs(ho - hs).max() <= 1e-12 * max(1.0, hs[:, 0].max())
    # accumulation over calls, as Hista accumulates over a run
    h2 = orc.acc_correl(_sys(st, box), bar_w, nbins, orc.acc_correl(_sys(st, box), bar_w, nbins))
    assert np.array_equal(h2[0], 2 * hist[0])
