"""Cell-binned list builds (mdsc_set_list_cells) give the same lists as the
all-pairs scan, so every result is bit-identical with cells on and off:
systems with and without a cell grid, one and two dipoles per rod, a
real-space cutoff (its neighbour list is built in the same scan), a rod
cluster dense enough to overflow a cell (that system falls back to the
all-pairs scan), and the 32,768-rod configuration.  Rebuilds are forced
between stretches of steps (mdsc_neigh_list) so every build in the run
happens on both paths."""
import numpy as np
import pytest

from mdspherocyl_gb300 import lib as L
from mdspherocyl_gb300 import systems as S

pytestmark = pytest.mark.gpu


def _systems():
    rs = np.random.default_rng(41)
    out = []
    for k, (n, nd, rc) in enumerate(((4200, 1, 0.0), (5000, 1, 0.0), (90, 1, 0.0), (4400, 2, 0.0),
                                     (4096, 1, 3.5))):
        mu = np.full(n, float(rs.uniform(0.8, 1.8)))
        st, box = S.make_system(n=n, phi=float(rs.uniform(0.08, 0.22)), lengths=rs.uniform(2, 4, n), mu=mu,
                                seed=500 + k, temp=1.1)
        if nd == 2:  # two off-centre dipoles per rod
            d = np.zeros((n, 2, 5))
            d[:, 0] = st.dip[:, 0]
            d[:, 0, 0] = 0.5
            d[:, 1] = st.dip[:, 0]
            d[:, 1, 0] = -0.5
            st.dip = d
        spec = S.SystemSpec(n=n, box=box, alpha=6.0 / box[0], K_max=6, ksq_max=27, temp=1.1, rc_real=rc)
        if rc > 0:
            spec.alpha = 3.3 / rc
        out.append((spec, st))
    # a dense cluster of 4096 rods in a box 3x wider: its cells overflow
    n = 4096
    st, box = S.make_system(n=n, phi=0.25, lengths=np.full(n, 2.0), mu=np.full(n, 1.0), seed=590)
    big = box * 3.0
    spec = S.SystemSpec(n=n, box=big, alpha=6.0 / big[0], K_max=5, ksq_max=16)
    out.append((spec, st))
    return out


def _run(systems, cells, stretches=3, steps=15):
    with L.Batch([s for s, _ in systems], [t for _, t in systems]) as bt:
        bt.set_list_cells(cells)
        obs = None
        for _ in range(stretches):
            bt.neigh_list()
            obs = bt.step(steps)
        return [bt.download(k) for k in range(len(systems))], obs


def test_cells_and_all_pairs_give_the_same_bits():
    systems = _systems()
    a, oa = _run(systems, True)
    b, ob = _run(systems, False)
    for k in range(len(systems)):
        assert oa[k]["status"] == 0 and ob[k]["status"] == 0, k
        assert oa[k]["list_builds"] == ob[k]["list_builds"] >= 1, (k, oa[k]["list_builds"], ob[k]["list_builds"])
        for f in ("r", "p", "O", "l", "F", "T"):
            assert np.array_equal(a[k][f], b[k][f]), (k, f)
        for key in ("U_ss", "W_ss", "U_dipR", "U_dipK", "PT_ss", "PT_dipR", "K", "xi"):
            assert np.array_equal(np.asarray(oa[k][key]), np.asarray(ob[k][key])), (k, key)


def test_cells_at_32768_rods():
    spec, st = S.plain_c2()
    res = []
    for cells in (True, False):
        with L.Batch([spec], [st]) as bt:
            bt.set_list_cells(cells)
            bt.neigh_list()
            obs = bt.step(3)[0]
            d = bt.download(0)
            lab, nc = bt.clust_conf(0)
            res.append((d, obs, lab))
    (da, oa, la), (db, ob, lb) = res
    for f in ("r", "p", "O", "l", "F", "T"):
        assert np.array_equal(da[f], db[f]), f
    assert oa["U_ss"] == ob["U_ss"] and np.array_equal(la, lb)
