"""Observables outside the step on the GPU (mdsc_correlations,
mdsc_order_params) against the reference's fixtures and the oracle.

Tolerances:
  pair counts (the 000 histogram): identical -- every pair in the
    reference's bin
  110, 112, 220 sums: |GPU - oracle| <= 5e-6 x (pairs in the bin) + 1e-7
    (each pair's term is FP32, ~4e-6 at worst, then fixed point 2^-24)
  G2: 1e-5, G1: 1e-4 (the reference's Q and eigen solve are FP32; G1 goes
    through the eigenvector, whose error grows as the eigenvalue gap shrinks)
  M: 1e-12 of sum |mu|
  a system's histogram in a batch of several: identical to the one alone
"""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN, load_golden
from mdspherocyl_gb300 import lib as L
from mdspherocyl_gb300 import systems as S


def _spec(st, box):
    return S.SystemSpec(n=st.n, box=np.asarray(box, dtype=np.float64), alpha=5.0 / min(box), K_max=4, ksq_max=0)


def _osys(st, box):
    return oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, box)


def _check_hist(h, want):
    assert h.shape == want.shape
    assert np.array_equal(h[0], want[0])
    pairs = want[0] / 2.0
    assert np.all(np.abs(h[1:] - want[1:]) <= 5e-6 * pairs + 1e-7)


def _nbins(box, bar_w):
    return int(np.floor(np.sqrt(3.0) * float(min(box)) / (2.0 * bar_w)))


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=[p.split("/")[-1] for p in GOLDEN])
def test_observables_vs_reference_fixtures(path):
    g = load_golden(path)
    st = S.SystemState(g["r"], g["p"], g["O"], g["l"], g["length"], g["dia"], g["mass"], g["dip"])
    with L.Batch([_spec(st, g["box"])], [st]) as bt:
        bar_w = float(g["corr_bar_w"])
        assert bt.correlation_bins(0, bar_w) == g["corr_hist"].shape[1]
        (h,) = bt.correlations(bar_w)
        assert h.shape[0] == 1
        _check_hist(h[0], g["corr_hist"])
        G1, G2, M = bt.order_params()
        assert abs(G2[0] - g["oo_G2"]) <= 1e-5
        assert abs(G1[0] - g["oo_G1"]) <= 1e-4
        scale = np.abs(g["dip"][:, :, 4]).sum()
        assert np.abs(M[0] - g["oo_M"]).max() <= 1e-12 * scale


def _mix():
    rng = np.random.default_rng(21)
    out = []
    st, box = S.make_system(n=3000, phi=0.12, lengths=rng.uniform(2, 4, 3000), mu=rng.uniform(0.5, 2, 3000),
                            seed=21, aspect=(1.3, 0.8))
    out.append((st, box))
    st, box = S.make_system(n=700, phi=0.2, lengths=np.full(700, 3.0), mu=np.ones(700), seed=22)
    dip = np.zeros((700, 2, 5))
    dip[:, 0] = [-0.6, 0.6, 0.8, 0.0, 1.2]
    dip[:, 1] = [0.4, 0.0, 0.0, 1.0, 0.7]
    st.dip = dip
    out.append((st, box))
    st, box = S.make_system(n=129, phi=0.1, lengths=np.full(129, 2.0), mu=np.ones(129), seed=23)
    out.append((st, box))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("bins", ["shared", "global"])
def test_correlations_mix_vs_oracle(orc, bins):
    systems = _mix()
    Lmax = max(float(min(b)) for _, b in systems)
    # fewer than 1024 bins in every system: shared-memory histograms; more: global
    bar_w = Lmax / 400.0 if bins == "shared" else Lmax / 1500.0
    with L.Batch([_spec(st, b) for st, b in systems], [st for st, _ in systems]) as bt:
        nb = [bt.correlation_bins(k, bar_w) for k in range(len(systems))]
        assert (max(nb) <= 1024) == (bins == "shared")
        hs = bt.correlations(bar_w)
        for k, (st, box) in enumerate(systems):
            assert nb[k] == _nbins(box, bar_w)
            want = orc.acc_correl(_osys(st, box), bar_w, nb[k])
            _check_hist(hs[k][0], want)
        # accumulation: a second call adds the same sums
        hs2 = bt.correlations(bar_w, hs)
        for k in range(len(systems)):
            assert np.array_equal(hs2[k], 2 * hs[k])
        G1, G2, M = bt.order_params()
        for k, (st, box) in enumerate(systems):
            g1, g2, m = orc.oo_params(_osys(st, box))
            assert abs(G2[k] - g2) <= 1e-5
            assert abs(G1[k] - g1) <= 1e-4
            assert np.abs(M[k] - m).max() <= 1e-12 * np.abs(st.dip[:, :, 4]).sum()
    # the same system alone: the same integers, so the same histogram
    st, box = systems[1]
    with L.Batch([_spec(st, box)], [st]) as bt:
        (h1,) = bt.correlations(bar_w)
        assert np.array_equal(h1, hs[1])
        _, G2a, Ma = bt.order_params()
        assert G2a[0] == G2[1] and np.array_equal(Ma[0], M[1])


def test_normalize_correlations():
    """nor_correl's normalisation (v25/functions.cpp:2472-2540) on a
    histogram of known counts (host arithmetic, no GPU)."""
    box = np.array([10.0, 10.0, 10.0])
    bar_w = 0.5
    nb = _nbins(box, bar_w)
    h = np.ones((1, 4, nb))
    pos, norm, g = L.normalize_correlations(h, [100], box=box, bar_w=bar_w, cor_cont=2.0)
    assert np.allclose(pos, (np.arange(nb) + 0.5) * bar_w)
    k = 3  # pos = 1.75 < L/2: the full shell
    assert norm[k] == pytest.approx(4 * np.pi * (pos[k] ** 2 * bar_w + bar_w ** 3 / 12))
    k = 12  # pos = 6.25 in [L/2, L/sqrt 2]: the shell cut by the box
    assert norm[k] == pytest.approx(4 * np.pi * pos[k] ** 2 * (3 * 10.0 / (2 * pos[k]) - 2) * bar_w)
    assert g[0, 1, 3] == pytest.approx(3.0 / (norm[3] * 2.0 * 100 * 99))
    # two species: the pair block over N_m N_n
    h2 = np.ones((3, 4, nb))
    _, _, g2 = L.normalize_correlations(h2, [30, 70], box=box, bar_w=bar_w, cor_cont=2.0)
    assert g2[2, 3, 5] == pytest.approx(5.0 / (norm[5] * 2.0 * 30 * 70))
    assert g2[0, 0, 5] == pytest.approx(1.0 / (norm[5] * 2.0 * 30 * 29))


@pytest.mark.gpu
def test_order_params_every_step(orc):
    """mdsc_step's G1, G2, M (FP32 terms, taken every step as the driver
    does) against the FP64 call and the oracle on the state after the step."""
    systems = _mix()
    with L.Batch([_spec(st, b) for st, b in systems], [st for st, _ in systems]) as bt:
        obs = bt.step(2)
        G1, G2, M = bt.order_params()
        for k, (st, box) in enumerate(systems):
            d = bt.download(k)
            s = oracle.System(d["r"], d["p"], d["O"], d["l"], st.length, st.dia, st.mass, st.dip, box)
            g1, g2, m = orc.oo_params(s)
            scale = np.abs(st.dip[:, :, 4]).sum()
            assert abs(obs[k]["G2"] - G2[k]) <= 1e-6 and abs(G2[k] - g2) <= 1e-5
            assert abs(obs[k]["G1"] - G1[k]) <= 1e-4 and abs(G1[k] - g1) <= 1e-4
            assert np.abs(np.array(obs[k]["M"]) - M[k]).max() <= 1e-6 * scale
            assert np.abs(M[k] - m).max() <= 1e-12 * scale


@pytest.mark.gpu
def test_correlations_species_vs_oracle(orc):
    """Several species per system: intra and inter histograms against the
    oracle's acc_correl with components (itself equal to the reference's,
    tests/test_oracle.py), in a batch with a one-species system."""
    systems = _mix()
    counts = {0: [1000, 1200, 800], 1: [300, 400]}
    bar_w = max(float(min(b)) for _, b in systems) / 300.0
    with L.Batch([_spec(st, b) for st, b in systems], [st for st, _ in systems]) as bt:
        for k, c in counts.items():
            bt.set_species(k, c)
        hs = bt.correlations(bar_w)
        for k, (st, box) in enumerate(systems):
            c = counts.get(k, [st.n])
            want = orc.acc_correl_species(_osys(st, box), c, bar_w, _nbins(box, bar_w))
            assert hs[k].shape == want.shape
            for q in range(want.shape[0]):
                intra = q < len(c)
                assert np.array_equal(hs[k][q][0], want[q][0])
                pairs = want[q][0] / (2.0 if intra else 1.0)
                assert np.all(np.abs(hs[k][q][1:] - want[q][1:]) <= 5e-6 * pairs + 1e-7)
