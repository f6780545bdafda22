"""Three and four dipoles per rod (MDSC_MAX_DIPOLES = 4): off-centre, tilted,
some with zero moment (a particle with fewer dipoles than its system's
count, as a species with fewer dipoles has in the reference).

* CPU: the oracle's real-space, k-space, field and self terms equal the
  reference's bit for bit.
* GPU: every force term within the bar of the path (RMS 1e-5), the same bits
  alone and beside one- and two-dipole systems, and 20 driver steps against
  the oracle's (total energy 1e-7).  The self energy is the sum of every
  particle's own term; the reference's self_ener takes particle 0 of each
  species times its count, which is the same only when a species' rods
  carry the same dipoles (as the reference's driver sets them).
"""
import numpy as np
import pytest

import oracle
from conftest import rms_rel
from mdspherocyl_gb300 import systems as S

TOL_F = 1e-5


def _many(nd, n, seed):
    rng = np.random.default_rng(seed)
    st, box = S.make_system(n=n, phi=0.15, lengths=rng.uniform(2.5, 4.0, n), mu=np.ones(n), seed=seed)
    dip = np.zeros((n, nd, 5))
    for w in range(nd):
        d = rng.normal(size=(n, 3)) * 0.3
        d[:, 2] += 1.0
        d /= np.linalg.norm(d, axis=1)[:, None]
        dip[:, w, 0] = (w - (nd - 1) / 2) / nd * st.length  # spread along the axis
        dip[:, w, 1:4] = d
        dip[:, w, 4] = rng.uniform(0.6, 1.2, n)
    dip[::5, nd - 1, 4] = 0.0  # every fifth rod one dipole short
    st.dip = dip
    spec = S.SystemSpec(n=n, box=box, alpha=6.5 / box[0], K_max=5, ksq_max=0, B=np.array([0.1, -0.2, 0.3]))
    return spec, st


def _osys(spec, st):
    return oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, spec.box)


def test_oracle_equals_reference_three_and_four_dipoles(ref, orc):
    for nd, seed in ((3, 61), (4, 62)):
        spec, st = _many(nd, 48, seed)
        a, b = _osys(spec, st), _osys(spec, st)
        x, y = orc.force_dipR(a, spec.alpha), ref.force_dipR(b, spec.alpha)
        assert x[0] == y[0] and np.array_equal(x[1], y[1]) and np.array_equal(a.F, b.F) and np.array_equal(a.T, b.T)
        a, b = _osys(spec, st), _osys(spec, st)
        x, y = orc.force_dipK(a, spec.K_max, spec.alpha), ref.force_dipK(b, spec.K_max, spec.alpha)
        assert x[0] == y[0] and np.array_equal(x[1], y[1]) and np.array_equal(a.F, b.F) and np.array_equal(a.T, b.T)
        a, b = _osys(spec, st), _osys(spec, st)
        assert orc.ext_field(a, spec.B) == ref.ext_field(b, spec.B) and np.array_equal(a.T, b.T)
        assert orc.self_ener(_osys(spec, st)) == ref.self_ener(_osys(spec, st))


@pytest.mark.gpu
def test_gpu_three_and_four_dipoles_vs_oracle(orc):
    from mdspherocyl_gb300 import lib as L

    cases = [_many(3, 300, 63), _many(4, 260, 64)]
    with L.Batch([c[0] for c in cases], [c[1] for c in cases]) as bt:
        for term in ("force_dipR", "force_dipK"):
            bt.zero_forces()
            U, PT = getattr(bt, term)()
            for k, (spec, st) in enumerate(cases):
                o = _osys(spec, st)
                Uo, PTo = (orc.force_dipR(o, spec.alpha) if term == "force_dipR"
                           else orc.force_dipK(o, spec.K_max, spec.alpha))
                d = bt.download(k)
                assert rms_rel(d["F"], o.F) < TOL_F and rms_rel(d["T"], o.T) < TOL_F, (term, k)
                assert rms_rel(PT[k], PTo) < TOL_F and abs(U[k] - Uo) < TOL_F * max(abs(Uo), 1.0), (term, k)
        bt.zero_forces()
        Ue = bt.ext_field()
        Us = bt.self_ener()
        for k, (spec, st) in enumerate(cases):
            o = _osys(spec, st)
            ue = orc.ext_field(o, spec.B)
            assert abs(Ue[k] - ue) <= 1e-7 * max(1.0, abs(ue)) and rms_rel(bt.download(k)["T"], o.T) < 1e-6
            # the sum over the particles of each one's own term; the reference's
            # self_ener takes particle 0 of a species times its count
            # (v25/functions.cpp:2027-2069), the same when a species' rods are alike
            want = sum(orc.self_ener(oracle.System(st.r[i:i + 1], st.p[i:i + 1], st.O[i:i + 1], st.l[i:i + 1],
                                                   st.length[i:i + 1], st.dia[i:i + 1], st.mass[i:i + 1],
                                                   st.dip[i:i + 1], spec.box)) for i in range(spec.n))
            assert abs(Us[k] - want) <= 1e-12 * max(1.0, abs(want))


@pytest.mark.gpu
def test_gpu_many_dipoles_alone_equals_in_batch():
    from mdspherocyl_gb300 import lib as L

    one_spec, one_st = S.plain_c0(seed=8, n=200)
    systems = [_many(4, 220, 65), (one_spec, one_st), _many(3, 180, 66)]
    alone = []
    for spec, st in systems:
        with L.Batch([spec], [st]) as bt:
            bt.step(15)
            alone.append(bt.download(0))
    with L.Batch([c[0] for c in systems], [c[1] for c in systems]) as bt:
        bt.step(15)
        for k in range(len(systems)):
            d = bt.download(k)
            for f in ("r", "p", "O", "l", "F", "T"):
                assert np.array_equal(d[f], alone[k][f]), (k, f)


@pytest.mark.gpu
def test_gpu_four_dipoles_trajectory_vs_oracle():
    from mdspherocyl_gb300 import lib as L

    spec, st = _many(4, 200, 67)
    orc = oracle.Oracle()
    o = _osys(spec, st)
    md = oracle.MDOracle(orc, o, dt=spec.dt, temp=spec.temp, Q=spec.Q, gamma=spec.gamma, xi0=spec.xi0,
                         sr_cut=3.0, K_max=spec.K_max, ksq_max=spec.ksq_max, alpha=spec.alpha, B=spec.B)
    with L.Batch([spec], [st]) as bt:
        for k in range(20):
            ob = bt.step(1)[0]
            assert md.step()
            mo = md.obs()
            # U_self is a constant, summed per particle here (see above)
            Ug = ob["U_ss"] + ob["U_dipR"] + ob["U_dipK"] + ob["U_ext"]
            Uo = mo["Uss"] + mo["UdipR"] + mo["UdipK"] + mo["Uext"]
            Kg, Ko = sum(ob["K"]), mo["K"].sum()
            assert abs((Ug + Kg) - (Uo + Ko)) <= 1e-7 * abs(Uo + Ko), (k, Ug + Kg, Uo + Ko)
        g = bt.download(0)
    for f in ("p", "l", "F", "T"):
        assert rms_rel(g[f], getattr(o, f)) < TOL_F, f
    assert np.abs(g["r"] - o.r).max() < 1e-8
