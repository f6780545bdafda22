"""Small-case exactness on hand-built configurations (tests/hand_configs.py):
every branch of spherocyl_dist (v25/functions.cpp:89-489) inside the WCA
range, in systems of 2 to 8 rods.

* CPU: the branches are all reached; the oracle equals the reference bit
  for bit on every pair's segment distance, on force_sc and on clust_conf.
  The reference's OpenMP loops never end below 16 particles per thread
  (schedule(dynamic, chunk) with chunk = floor(N / (16 threads)) = 0,
  v25/functions.cpp:1411-1414), so these cases run on its serial build --
  itself pinned bit for bit to the OpenMP build on the golden fixtures.
* GPU: mdsc_force_sc on all the systems in one batch against the oracle
  (FP64, the reference's arithmetic: <= 1e-12 of the system's largest
  value), and the cluster labels identical.
"""
import numpy as np
import pytest

import hand_configs as H
import oracle
from conftest import GOLDEN, load_golden

WCA2 = 2.0 ** (1.0 / 3.0)  # (2^(1/6) sigma)^2 for sigma = 1
MIN_S = (0.1, 0.6)


def _osys(c):
    n = len(c["length"])
    return oracle.System(c["r"], np.zeros((n, 3)), c["O"], np.zeros((n, 3)), c["length"], c["dia"], np.ones(n),
                         np.zeros((n, 1, 5)), c["box"])


def _wca_pairs(orc, c):
    s = _osys(c)
    n = len(c["length"])
    return [(i, j) for i in range(n) for j in range(i + 1, n) if orc.seg_dist(s, i, j)[0] < WCA2]


def test_every_branch_is_reached(orc):
    got = set()
    for c in H.build():
        for name, first, rods in c["pairs"]:
            if name in H.PAIRS:  # the pair lands in the branch it is named for
                want = "parallel-none" if name == "parallel-documented" else name
                assert H.branch(c, first, first + 1) == want, name
        for i, j in _wca_pairs(orc, c):
            got.add(H.branch(c, i, j))
        ok, U, W, PT = orc.force_sc(_osys(c), 3.0, 3.5)
        assert ok, c["members"]  # no overlap abort
    assert got == H.ALL_BRANCHES, H.ALL_BRANCHES - got


def test_serial_reference_build_equals_openmp_build(ref, ref_serial):
    """The serial build is the reference's arithmetic: bit for bit the
    OpenMP build (one thread) on every golden system (N >= 16)."""
    for path in GOLDEN:
        g = load_golden(path)

        def mk():
            return oracle.System(g["r"], g["p"], g["O"], g["l"], g["length"], g["dia"], g["mass"], g["dip"],
                                 g["box"])

        assert len(g["length"]) >= 16
        a, b = mk(), mk()
        x, y = ref.force_sc(a, 3.0, 3.5), ref_serial.force_sc(b, 3.0, 3.5)
        assert x[0] == y[0] and x[1] == y[1] and x[2] == y[2] and np.array_equal(x[3], y[3])
        assert np.array_equal(a.F, b.F) and np.array_equal(a.T, b.T)
        a, b = mk(), mk()
        x, y = ref.force_dipR(a, float(g["alpha"])), ref_serial.force_dipR(b, float(g["alpha"]))
        assert x[0] == y[0] and np.array_equal(x[1], y[1]) and np.array_equal(a.F, b.F)
        for ms in MIN_S:
            la, nxa = ref.clust_conf(mk(), ms, seed=5, skip=3)
            lb, nxb = ref_serial.clust_conf(mk(), ms, seed=5, skip=3)
            assert np.array_equal(la, lb) and nxa == nxb


def test_oracle_equals_reference_on_hand_configs(ref_serial, orc):
    ref = ref_serial
    for c in H.build():
        n = len(c["length"])
        a, b = _osys(c), _osys(c)
        for i in range(n):
            for j in range(i + 1, n):
                x, y = orc.seg_dist(a, i, j), ref.seg_dist(b, i, j)
                assert x[0] == y[0] and np.array_equal(x[1], y[1]) and np.array_equal(x[2], y[2]), \
                    (c["members"], i, j, x, y)
        x, y = orc.force_sc(a, 3.0, 3.5), ref.force_sc(b, 3.0, 3.5)
        assert x[0] and y[0]
        assert x[1] == y[1] and x[2] == y[2] and np.array_equal(x[3], y[3]), c["members"]
        assert np.array_equal(a.F, b.F) and np.array_equal(a.T, b.T), c["members"]
        for ms in MIN_S:
            la, nca, nxa = orc.clust_conf(_osys(c), ms, seed=5, skip=3)
            lb, nxb = ref.clust_conf(_osys(c), ms, seed=5, skip=3)
            assert np.array_equal(la, lb) and nxa == nxb, (c["members"], ms)


@pytest.mark.gpu
def test_gpu_force_sc_and_clusters_on_hand_configs(orc):
    from mdspherocyl_gb300 import lib as L
    from mdspherocyl_gb300 import systems as S

    confs = H.build()
    states = []
    for c in confs:
        n = len(c["length"])
        states.append(S.SystemState(c["r"], np.zeros((n, 3)), c["O"], np.zeros((n, 3)), c["length"], c["dia"],
                                    np.ones(n), np.zeros((n, 1, 5))))
    for ms in MIN_S:
        specs = [S.SystemSpec(n=len(c["length"]), box=c["box"], alpha=6.0 / H.BOX, K_max=3, ksq_max=0, min_s=ms)
                 for c in confs]
        with L.Batch(specs, states) as bt:
            bt.zero_forces()
            U, W, PT = bt.force_sc()
            for k, c in enumerate(confs):
                s = _osys(c)
                ok, u, w, pt = orc.force_sc(s, 3.0, 3.5)
                d = bt.download(k)
                scale = max(1.0, np.abs(s.F).max(), np.abs(s.T).max())
                assert abs(U[k] - u) <= 1e-12 * max(1.0, abs(u)), (c["members"], U[k], u)
                assert abs(W[k] - w) <= 1e-12 * max(1.0, abs(w)), (c["members"], W[k], w)
                assert np.abs(PT[k] - pt).max() <= 1e-12 * max(1.0, np.abs(pt).max()), c["members"]
                assert np.abs(d["F"] - s.F).max() <= 1e-12 * scale, (c["members"], d["F"], s.F)
                assert np.abs(d["T"] - s.T).max() <= 1e-12 * scale, (c["members"], d["T"], s.T)
                lab, nc = bt.clust_conf(k)
                want, ncw, _ = orc.clust_conf(_osys(c), ms, seed=1, skip=0)
                assert np.array_equal(lab, want) and nc == ncw, (c["members"], ms, lab, want)
