"""Real-space cutoff (mdsc_system_desc.rc_real > 0): the reference's own
force_dipR with tabul's table zeroed beyond rc (the survey's "cutoff mode":
config 1's real cutoff of 3.5 sigma), summed on the GPU over a neighbour
list of rods instead of all pairs.

* CPU: the oracle's masked force_dipR equals the reference's (its own
  routine, the table masked) bit for bit, with one axial and two
  off-centre dipoles per rod.
* GPU: forces, torques, energy and pressure tensor against that oracle
  (RMS relative <= 1e-5, the bar of the all-pairs path), in one batch with
  an all-pairs system; the same bits alone and in the batch; 40 steps
  against the oracle's driver step with the masked table.
"""
import numpy as np
import pytest

import oracle
from conftest import rms_rel
from mdspherocyl_gb300 import systems as S

TOL_F = 1e-5


def _two_dipoles(st, rng):
    n = len(st.length)
    dip = np.zeros((n, 2, 5))
    for w, sgn in enumerate((1.0, -1.0)):
        d = np.array([0.3 * rng.normal(), 0.3 * rng.normal(), 1.0])
        d /= np.linalg.norm(d)
        dip[:, w, 0] = sgn * st.length / 4
        dip[:, w, 1:4] = d
        dip[:, w, 4] = rng.uniform(0.9, 1.4, n)
    st.dip = dip
    return st


def _cases():
    """(spec, state): C1-like (L ~ U[2, 5], mu ~ volume, alpha = 7/L_box,
    rc = 3.5), a larger cutoff with two off-centre dipoles per rod."""
    rng = np.random.default_rng(17)
    out = []
    n = 600
    lengths = rng.uniform(2.0, 5.0, n)
    vol = np.pi * lengths / 4 + np.pi / 6
    st, box = S.make_system(n=n, phi=0.2, lengths=lengths, mu=vol * np.sqrt(3.0 / np.mean(vol ** 2)), seed=31)
    out.append((S.SystemSpec(n=n, box=box, alpha=7.0 / box[0], K_max=5, ksq_max=0, rc_real=3.5), st))
    n = 400
    st, box = S.make_system(n=n, phi=0.15, lengths=rng.uniform(2.0, 3.5, n), mu=np.ones(n), seed=32)
    st = _two_dipoles(st, rng)
    out.append((S.SystemSpec(n=n, box=box, alpha=9.0 / box[0], K_max=5, ksq_max=0, rc_real=5.0), st))
    return out


def _osys(spec, st):
    return oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, spec.box)


def test_masked_oracle_equals_reference(ref, orc):
    for spec, st in _cases():
        a, b = _osys(spec, st), _osys(spec, st)
        x = orc.force_dipR(a, spec.alpha, rc=spec.rc_real)
        y = ref.force_dipR(b, spec.alpha, rc=spec.rc_real)
        assert x[0] == y[0] and np.array_equal(x[1], y[1])
        assert np.array_equal(a.F, b.F) and np.array_equal(a.T, b.T)
        # and the cutoff matters: the all-pairs sum differs
        c = _osys(spec, st)
        z = orc.force_dipR(c, spec.alpha)
        assert rms_rel(a.F, c.F) > 1e-3


@pytest.mark.gpu
def test_gpu_cutoff_forces_vs_oracle(orc):
    from mdspherocyl_gb300 import lib as L

    cases = _cases()
    allp_spec, allp_st = S.plain_c0(seed=5, n=300)
    specs = [c[0] for c in cases] + [allp_spec]
    states = [c[1] for c in cases] + [allp_st]
    with L.Batch(specs, states) as bt:
        bt.zero_forces()
        U, PT = bt.force_dipR()
        for k, (spec, st) in enumerate(zip(specs, states)):
            o = _osys(spec, st)
            Uo, PTo = orc.force_dipR(o, spec.alpha, rc=spec.rc_real)
            d = bt.download(k)
            assert rms_rel(d["F"], o.F) < TOL_F, k
            assert rms_rel(d["T"], o.T) < TOL_F, k
            assert rms_rel(PT[k], PTo) < TOL_F, k
            assert abs(U[k] - Uo) < TOL_F * max(abs(Uo), 1.0), (k, U[k], Uo)


@pytest.mark.gpu
def test_gpu_cutoff_alone_equals_in_batch():
    """Cutoff and all-pairs systems, one and two dipoles per rod, in one
    batch: every system has the bits it has alone."""
    from mdspherocyl_gb300 import lib as L

    allp_spec, allp_st = S.plain_c0(seed=6, n=250)
    systems = [(allp_spec, allp_st)] + _cases()
    alone = []
    for spec, st in systems:
        with L.Batch([spec], [st]) as bt:
            bt.step(20)
            alone.append(bt.download(0))
    with L.Batch([c[0] for c in systems], [c[1] for c in systems]) as bt:
        bt.step(20)
        for k in range(len(systems)):
            d = bt.download(k)
            for f in ("r", "p", "O", "l", "F", "T"):
                assert np.array_equal(d[f], alone[k][f]), (k, f)


@pytest.mark.gpu
def test_gpu_cutoff_trajectory_vs_oracle():
    from mdspherocyl_gb300 import lib as L

    spec, st = _cases()[0]
    orc = oracle.Oracle()
    o = _osys(spec, st)
    md = oracle.MDOracle(orc, o, dt=spec.dt, temp=spec.temp, Q=spec.Q, gamma=spec.gamma, xi0=spec.xi0,
                         sr_cut=3.0, K_max=spec.K_max, ksq_max=spec.ksq_max, alpha=spec.alpha, B=spec.B,
                         rc_real=spec.rc_real)
    with L.Batch([spec], [st]) as bt:
        for k in range(40):
            ob = bt.step(1)[0]
            assert md.step()
            mo = md.obs()
            assert abs(ob["U_dipR"] - mo["UdipR"]) <= TOL_F * abs(mo["UdipR"]), (k, ob["U_dipR"], mo["UdipR"])
            Ug = ob["U_ss"] + ob["U_dipR"] + ob["U_dipK"] + ob["U_ext"] + ob["U_self"]
            Uo = mo["Uss"] + mo["UdipR"] + mo["UdipK"] + mo["Uext"] + mo["Uself"]
            Kg, Ko = sum(ob["K"]), mo["K"].sum()
            assert abs((Ug + Kg) - (Uo + Ko)) <= 1e-7 * abs(Uo + Ko), (k, Ug + Kg, Uo + Ko)
        g = bt.download(0)
    for f in ("p", "l", "F", "T"):
        assert rms_rel(g[f], getattr(o, f)) < TOL_F, f
    assert np.abs(g["r"] - o.r).max() < 1e-8
