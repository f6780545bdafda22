"""Clusters by an energy criterion -- an extension: the reference's own test
is geometric (v25/functions.cpp:2987-3016), so this criterion has no
reference to pin it ("parity unpinned").  A bond is U_pair < -u_bond * T with
U_pair = force_sc's WCA pair energy + the bare dipole-dipole energy of every
dipole pair at the minimum image of the sites; labels are numbered as
clust_conf numbers them (v25/functions.cpp:2950-2970,3282-3313).

* CPU: the oracle's pair energy against a numpy form of the same formula;
  its labels against the components of the numpy bond graph, numbered by
  the reference's draw-and-label order.
* GPU: mdsc_set_cluster_energy systems beside geometric ones in one batch,
  one and two (off-centre, tilted) dipoles per rod: labels identical to the
  oracle's, in mdsc_clust_conf and in the clustering inside mdsc_step.
"""
import numpy as np
import pytest

import oracle
from mdspherocyl_gb300 import systems as S


def _two_dipoles(st, rng):
    """Two off-centre dipoles per rod: offsets +-L/4 along the axis,
    directions tilted from the axis, moments around 1.6."""
    n = len(st.length)
    dip = np.zeros((n, 2, 5))
    for w, sgn in enumerate((1.0, -1.0)):
        d = np.array([0.25 * rng.normal(), 0.25 * rng.normal(), 1.0])
        d /= np.linalg.norm(d)
        dip[:, w, 0] = sgn * st.length / 4
        dip[:, w, 1:4] = d
        dip[:, w, 4] = rng.uniform(1.3, 1.9, n)
    st.dip = dip
    return st


def _cases():
    rng = np.random.default_rng(21)
    out = []
    for k, (n, phi, mu2, nd2) in enumerate(((400, 0.25, 6.0, False), (700, 0.3, 4.0, True), (300, 0.2, 8.0, False))):
        st, box = S.make_system(n=n, phi=phi, lengths=rng.uniform(2.0, 3.5, n), mu=np.full(n, np.sqrt(mu2)),
                                seed=40 + k, temp=1.0)
        if nd2:
            st = _two_dipoles(st, rng)
        out.append((st, box, 1.0 + 0.2 * k))
    return out


def _osys(st, box):
    return oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, box)


def _numpy_pair_energy(orc, o, st, box, a, b):
    dsq, _, _ = orc.seg_dist(o, a, b)
    sig = (st.dia[a] + st.dia[b]) / 2
    U = 0.0
    if dsq < 2 ** (1 / 3) * sig * sig:
        x = (sig * sig / dsq) ** 3
        U = 4 * x * (x - 1) + 1
    for da in st.dip[a]:
        for db in st.dip[b]:
            if da[4] == 0 or db[4] == 0:
                continue
            pa = st.r[a] + da[0] * st.O[a][2]
            pb = st.r[b] + db[0] * st.O[b][2]
            oa, ob = st.O[a].T @ da[1:4], st.O[b].T @ db[1:4]
            r = pa - pb
            r -= box * np.floor(r / box + 0.5)
            r2 = r @ r
            U += da[4] * db[4] * (oa @ ob - 3 * (oa @ r) * (ob @ r) / r2) / r2 ** 1.5
    return U


def test_pair_energy_and_labels_on_cpu(orc):
    for st, box, u in _cases():
        o = _osys(st, box)
        n = len(st.length)
        rng = np.random.default_rng(0)
        for a, b in rng.integers(0, n, (40, 2)):
            if a == b:
                continue
            a, b = min(a, b), max(a, b)
            assert abs(orc.pair_energy(o, a, b) - _numpy_pair_energy(orc, o, st, box, a, b)) < 1e-10
        # pairs that can bond: |U_dd| <= 2 M_a M_b / (r - e_a - e_b)^3, U_WCA >= 0
        M = np.abs(st.dip[:, :, 4]).sum(axis=1)
        e = np.abs(st.dip[:, :, 0]).max(axis=1)
        dr = st.r[:, None, :] - st.r[None, :, :]
        dr -= box * np.floor(dr / box + 0.5)
        gap = np.sqrt((dr ** 2).sum(-1)) - e[:, None] - e[None, :]
        near = (gap <= 0) | (2 * M[:, None] * M[None, :] * 1.01 >= u * np.maximum(gap, 1e-9) ** 3)
        E = {}
        for a, b in zip(*np.nonzero(np.triu(near, 1))):
            en = orc.pair_energy(o, int(a), int(b))
            if en < -u:
                E[(int(a), int(b))] = en
        assert len(E) >= 3, len(E)  # the cases do form bonds
        # components of the bond graph
        parent = list(range(n))

        def root(x):
            while parent[x] != x:
                parent[x] = parent[parent[x]]
                x = parent[x]
            return x

        for a, b in E:
            ra, rb = root(a), root(b)
            if ra != rb:
                parent[max(ra, rb)] = min(ra, rb)
        comp = [root(x) for x in range(n)]
        # the reference's numbering: draw u, take the floor(u * remaining)-th
        # remaining particle in index order, label its component
        g = orc._rng_new(7)
        for _ in range(2):
            orc._rng_u(g)
        remaining, want, nc = list(range(n)), np.full(n, -1), 0
        while remaining:
            seed = remaining[int(np.floor(orc._rng_u(g) * len(remaining)))]
            members = [x for x in remaining if comp[x] == comp[seed]]
            want[members] = nc
            remaining = [x for x in remaining if comp[x] != comp[seed]]
            nc += 1
        nxt = orc._rng_u(g)
        orc._rng_free(g)
        lab, ncl, nx2 = orc.clust_energy(_osys(st, box), u, seed=7, skip=2)
        assert np.array_equal(lab, want) and ncl == nc and nx2 == nxt


@pytest.mark.gpu
def test_gpu_energy_labels_equal_oracle(orc):
    from mdspherocyl_gb300 import lib as L

    cases = _cases()
    specs = [S.SystemSpec(n=len(st.length), box=box, alpha=6.0 / box[0], K_max=5, ksq_max=0, temp=1.0)
             for st, box, _ in cases]
    # the same systems twice: energy criterion, then the reference's
    with L.Batch(specs + specs, [c[0] for c in cases] * 2) as bt:
        for k, (_, _, u) in enumerate(cases):
            bt.set_cluster_energy(k, u)
        for k, (st, box, u) in enumerate(cases):
            lab, nc = bt.clust_conf(k)
            want, ncw, _ = orc.clust_energy(_osys(st, box), u, seed=1, skip=0)
            assert np.array_equal(lab, want) and nc == ncw, k
            assert nc < len(st.length)  # bonds were found
            lab, nc = bt.clust_conf(len(cases) + k)
            want, ncw, _ = orc.clust_conf(_osys(st, box), 0.1, seed=1, skip=0)
            assert np.array_equal(lab, want) and nc == ncw, k
        # back to the reference's test: the generator goes on from where the
        # energy labelling left it (one draw per cluster)
        st, box, u = cases[0]
        drawn = orc.clust_energy(_osys(st, box), u, seed=1, skip=0)[1]
        bt.set_cluster_energy(0, 0.0)
        lab, nc = bt.clust_conf(0)
        want, ncw, _ = orc.clust_conf(_osys(st, box), 0.1, seed=1, skip=drawn)
        assert np.array_equal(lab, want) and nc == ncw


@pytest.mark.gpu
def test_gpu_energy_clusters_inside_the_step(orc):
    """cl_fr = 5: the step's own clustering uses the system's criterion, on
    the reference's schedule (step index % cl_fr == 0: after the 1st and the
    6th step); labels equal the oracle's on the state after those steps, the
    generator going on from one labelling to the next."""
    from mdspherocyl_gb300 import lib as L

    st, box, u = _cases()[0]
    spec = S.SystemSpec(n=len(st.length), box=box, alpha=6.0 / box[0], K_max=5, ksq_max=0, temp=1.0, cl_fr=5)
    drawn = 0
    with L.Batch([spec], [st]) as bt:
        bt.set_cluster_energy(0, u)
        for steps in (1, 5):
            bt.step(steps)
            d = bt.download(0)
            after = S.SystemState(d["r"], d["p"], d["O"], d["l"], st.length, st.dia, st.mass, st.dip)
            want, ncw, _ = orc.clust_energy(_osys(after, box), u, seed=1, skip=drawn)
            assert np.array_equal(d["clust"], want), steps
            drawn += ncw
