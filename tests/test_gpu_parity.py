"""GPU path (C ABI, libmdsc.so) against the FP64 oracle and the reference.

Tolerances (the bar the GPU path is held to):
  forces and torques of the FP32 Ewald sums: RMS relative error <= 1e-5
  total energy of a step, E = K + U: relative error <= 1e-7
  potential energy U alone: relative error <= 1e-6 (the FP32 pair
    energies, each good to ~1e-7, are summed with cancellation)
  WCA (FP64, the reference's own arithmetic): <= 1e-12
  kicks and drifts (FP64): <= 1e-12; orientations after a drift: <= 1e-8
  cluster labels: identical
"""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN, load_golden, rms_rel
from mdspherocyl_gb300 import lib as L
from mdspherocyl_gb300 import systems as S

pytestmark = pytest.mark.gpu

TOL_F = 1e-5
TOL_E_TOTAL = 1e-7
TOL_U = 1e-6


def desc(n, nd, box, alpha, K, ksq, **kw):
    d = L.SystemDesc()
    d.n, d.nd = n, nd
    for a in range(3):
        d.box[a] = float(box[a])
    B = kw.get("B", (0.0, 0.0, 0.0))
    for a in range(3):
        d.B[a] = float(B[a])
    d.alpha, d.K_max, d.ksq_max = float(alpha), int(K), int(ksq)
    d.sr_cut = float(kw.get("sr_cut", 0.0))
    d.dt, d.temp, d.Q, d.gamma = kw.get("dt", 1e-3), kw.get("T", 1.0), kw.get("Q", 1.0), kw.get("gamma", 0.0)
    d.xi0 = kw.get("xi0", 0.0)
    d.min_s, d.cl_fr = kw.get("min_s", 0.1), kw.get("cl_fr", 0)
    d.thermo_seed[0], d.thermo_seed[1] = 1, 2
    d.cluster_seed, d.cluster_skip = kw.get("cluster_seed", 1), kw.get("cluster_skip", 0)
    return d


def state_of(g):
    return S.SystemState(g["r"], g["p"], g["O"], g["l"], g["length"], g["dia"], g["mass"], g["dip"])


def batch_of(g, **kw):
    st = state_of(g)
    d = desc(len(g["length"]), g["dip"].shape[1], g["box"], float(g["alpha"]), int(g["K_max"]),
             int(g["ksq_max"]), B=g["B"], **kw)
    return L.Batch([None], [st], descs=[d])


@pytest.mark.parametrize("path", GOLDEN, ids=[p.split("/")[-1] for p in GOLDEN])
def test_functions_vs_reference_fixtures(path):
    g = load_golden(path)
    n = len(g["length"])
    with batch_of(g) as bt:
        # force_sc: the reference's own FP64 arithmetic
        bt.zero_forces()
        U, W, PT = bt.force_sc()
        d = bt.download(0)
        assert abs(U[0] - g["sc_U"]) <= 1e-12 * max(1.0, abs(g["sc_U"]))
        assert abs(W[0] - g["sc_W"]) <= 1e-12 * max(1.0, abs(g["sc_W"]))
        assert np.abs(d["F"] - g["sc_F"]).max() <= 1e-12 * max(1.0, np.abs(g["sc_F"]).max())
        assert np.abs(d["T"] - g["sc_T"]).max() <= 1e-12 * max(1.0, np.abs(g["sc_T"]).max())
        # real-space Ewald
        bt.zero_forces()
        U, PT = bt.force_dipR()
        d = bt.download(0)
        assert rms_rel(d["F"], g["dipR_F"]) < TOL_F
        assert rms_rel(d["T"], g["dipR_T"]) < TOL_F
        assert rms_rel(PT[0], g["dipR_PT"]) < TOL_F
        assert abs(U[0] - g["dipR_U"]) < TOL_F * max(abs(g["dipR_U"]), 1.0)
        # reciprocal-space Ewald
        bt.zero_forces()
        U, PT = bt.force_dipK()
        d = bt.download(0)
        assert rms_rel(d["F"], g["dipK_F"]) < TOL_F
        assert rms_rel(d["T"], g["dipK_T"]) < TOL_F
        assert rms_rel(PT[0], g["dipK_PT"]) < TOL_F
        assert abs(U[0] - g["dipK_U"]) < TOL_F * max(abs(g["dipK_U"]), 1.0)
        # external field
        bt.zero_forces()
        U = bt.ext_field()
        d = bt.download(0)
        assert abs(U[0] - g["ext_U"]) <= 1e-7 * max(1.0, abs(g["ext_U"]))
        assert rms_rel(d["T"], g["ext_T"]) < 1e-6
        assert abs(bt.self_ener()[0] - g["self_U"]) <= 1e-12 * max(1.0, abs(g["self_U"]))
    # kicks and drift
    for last in (0, 1):
        with batch_of(g) as bt:
            bt.upload(0, state_of(g), F=g["mp_F"], T=g["mp_T"])
            K, PT = bt.moveP(g["mp_xi"], bool(last))
            d = bt.download(0)
            assert rms_rel(d["p"], g[f"mp{last}_p"]) < 1e-12
            assert rms_rel(d["l"], g[f"mp{last}_l"]) < 1e-12
            assert np.abs(K[0] - g[f"mp{last}_K"]).max() < 1e-11 * np.abs(g[f"mp{last}_K"]).max()
            if last:
                assert rms_rel(PT[0], g[f"mp{last}_PT"]) < 1e-12
    with batch_of(g) as bt:
        bt.moveX()
        d = bt.download(0)
        assert np.abs(d["r"] - g["mx_r"]).max() < 1e-12
        assert np.abs(d["O"] - g["mx_O"]).max() < 1e-8
    with batch_of(g) as bt:
        bt.renorm()
        d = bt.download(0)
        assert np.abs(d["O"] - g["rn_O"]).max() < 1e-14
    # clusters: labels of the reference, drawing from a generator seeded 1
    # and advanced 7 draws
    for ms in (0.1, 0.6):
        with batch_of(g, min_s=ms, cluster_seed=1, cluster_skip=7) as bt:
            lab, nc = bt.clust_conf(0)
            assert np.array_equal(lab, g[f"cl{ms}_labels"])
            assert nc == g[f"cl{ms}_labels"].max() + 1


def test_trajectory_vs_reference_driver():
    """30 steps against the reference driver itself (noisy thermostat,
    tilted off-axis dipole, field, clusters every 7 steps)."""
    import os
    from conftest import ROOT

    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "driver_trajectory.npz")))
    n = len(g["length"])
    box = g["box"]
    d = desc(n, 1, box, float(g["alpha"]), int(g["K_max"]), 0, B=g["B"], T=float(g["T"]), Q=float(g["Q"]),
             gamma=float(g["gamma"]), dt=float(g["dt"]), min_s=float(g["min_s"]), cl_fr=int(g["cl_fr"]))
    st = state_of(g)
    V = float(np.prod(box))
    with L.Batch([None], [st], descs=[d]) as bt:
        bt.set_thermostat(0, g["xi"], g["strn"])
        out = g["out"]
        for k in range(int(g["steps"])):
            o = bt.step(1)[0]
            K = (o["K"][0] + o["K"][1]) / n
            U = o["U_self"] / n + (o["U_ss"] + o["U_dipR"] + o["U_dipK"] + o["U_ext"]) / n
            assert abs(K - out[k][0]) <= 1e-7 * abs(out[k][0]) + 1e-11, (k, K, out[k][0])
            E, Eo = K + U, out[k][0] + out[k][1]
            assert abs(E - Eo) <= TOL_E_TOTAL * abs(Eo) + 2e-12, (k, E, Eo)
            assert abs(U - out[k][1]) <= TOL_U * abs(out[k][1]) + 2e-12, (k, U, out[k][1])
            assert abs(o["U_ss"] / n - out[k][3]) <= 1e-6 * abs(out[k][3]) + 2e-12
            assert abs(o["U_dipR"] / n - out[k][5]) <= TOL_F * abs(out[k][5]) + 2e-12
            assert abs(o["U_dipK"] / n - out[k][7]) <= TOL_F * abs(out[k][7]) + 2e-12
        fin = bt.download(0)
    assert np.abs(fin["r"] - g["fin_r"]).max() < 1e-9
    assert rms_rel(fin["p"], g["fin_p"]) < 1e-6
    assert rms_rel(fin["l"], g["fin_l"]) < 1e-6
    assert np.abs(fin["O"] - g["fin_O"]).max() < 1e-8
    assert np.array_equal(fin["clust"], g["fin_clust"])


def _oracle_md(spec, st, **kw):
    orc = oracle.Oracle()
    o = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, spec.box)
    md = oracle.MDOracle(orc, o, dt=spec.dt, temp=spec.temp, Q=spec.Q, gamma=spec.gamma, xi0=spec.xi0,
                         sr_cut=3.0, K_max=spec.K_max, ksq_max=spec.ksq_max, alpha=spec.alpha, B=spec.B, **kw)
    return o, md


def test_plain_system_50_steps_vs_oracle():
    spec, st = S.plain_c0(seed=4, n=200)
    spec.B = np.array([0.0, 0.3, 0.2])
    o, md = _oracle_md(spec, st)
    with L.Batch([spec], [st]) as bt:
        for k in range(50):
            ob = bt.step(1)[0]
            assert md.step()
            mo = md.obs()
            Ug = ob["U_ss"] + ob["U_dipR"] + ob["U_dipK"] + ob["U_ext"] + ob["U_self"]
            Uo = mo["Uss"] + mo["UdipR"] + mo["UdipK"] + mo["Uext"] + mo["Uself"]
            parts = {k2: ob[k1] - mo[k2] for k1, k2 in (("U_ss", "Uss"), ("U_dipR", "UdipR"),
                                                       ("U_dipK", "UdipK"), ("U_ext", "Uext"))}
            Kg, Ko = sum(ob["K"]), mo["K"].sum()
            assert abs(Kg - Ko) <= 1e-9 * Ko
            assert abs((Ug + Kg) - (Uo + Ko)) <= TOL_E_TOTAL * abs(Uo + Ko), (k, Ug + Kg, Uo + Ko, parts)
            assert abs(Ug - Uo) <= TOL_U * abs(Uo), (k, Ug, Uo, parts)
        g = bt.download(0)
    for f in ("p", "l", "F", "T"):
        assert rms_rel(g[f], getattr(o, f)) < TOL_F, f
    assert np.abs(g["r"] - o.r).max() < 1e-8


def test_batch_results_equal_alone():
    """Each system gives bit-identical results alone and inside a batch of
    different systems (no cross-system reduction anywhere)."""
    rs = np.random.default_rng(77)
    systems = []
    for k, n in enumerate((70, 150, 300, 64)):
        st, box = S.make_system(n=n, phi=float(rs.uniform(0.05, 0.2)), lengths=rs.uniform(2, 4, n),
                                mu=np.full(n, float(rs.uniform(0.8, 2.0))), seed=100 + k, temp=1.2)
        spec = S.SystemSpec(n=n, box=box, alpha=6.0 / box[0], K_max=7, ksq_max=36, temp=1.2,
                            B=np.array([0.0, 0.0, 0.1 * k]), gamma=0.5 * (k % 2))
        systems.append((spec, st))
    alone = []
    for spec, st in systems:
        with L.Batch([spec], [st]) as bt:
            ob = bt.step(12)[0]
            alone.append((ob, bt.download(0)))
    with L.Batch([s for s, _ in systems], [t for _, t in systems]) as bt:
        obs = bt.step(12)
        for k in range(len(systems)):
            d = bt.download(k)
            for f in ("r", "p", "O", "l", "F", "T"):
                assert np.array_equal(d[f], alone[k][1][f]), (k, f)
            for key in ("U_ss", "U_dipR", "U_dipK", "U_ext", "K", "PT_dipR", "PT_dipK", "xi"):
                assert np.array_equal(np.asarray(obs[k][key]), np.asarray(alone[k][0][key])), (k, key)


def test_split_kspace_gather_alone_equals_in_batch():
    """A system of 4096 rods runs its k-space gather in parts on separate
    blocks (a function of the system alone): it has the same bits alone and
    beside small systems, in both gather forms (one or two rods a thread),
    and its forces stay on the oracle's."""
    rs = np.random.default_rng(78)
    n = 4096
    st, box = S.make_system(n=n, phi=0.2, lengths=rs.uniform(2, 4, n), mu=np.full(n, 1.3), seed=120)
    big = S.SystemSpec(n=n, box=box, alpha=6.0 / box[0], K_max=5, ksq_max=0)
    small = []
    for k, m in enumerate((90, 200)):
        s2, b2 = S.make_system(n=m, phi=0.1, lengths=rs.uniform(2, 4, m), mu=np.full(m, 1.1), seed=130 + k)
        small.append((S.SystemSpec(n=m, box=b2, alpha=6.0 / b2[0], K_max=5, ksq_max=0), s2))
    results = []
    for kg in (0, 1):
        with L.Batch([big], [st]) as bt:
            bt.set_tuning(1, 256, 152 * 8, kg)
            bt.step(6)
            results.append(bt.download(0))
    with L.Batch([small[0][0], big, small[1][0]], [small[0][1], st, small[1][1]]) as bt:
        bt.step(6)
        results.append(bt.download(1))
    for f in ("r", "p", "O", "l", "F", "T"):
        assert np.array_equal(results[0][f], results[1][f]), ("forms", f)
        assert np.array_equal(results[0][f], results[2][f]), ("batch", f)
    with L.Batch([big], [st]) as bt:
        bt.zero_forces()
        bt.force_dipK()
        d = bt.download(0)
    o = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, box)
    orc = oracle.Oracle()
    orc.force_dipK(o, big.K_max, big.alpha, big.ksq_max)
    assert rms_rel(d["F"], o.F) < TOL_F and rms_rel(d["T"], o.T) < TOL_F


def test_noncubic_box_and_field_vs_oracle():
    rng = np.random.default_rng(31)
    n = 120
    st, box = S.make_system(n=n, phi=0.12, lengths=rng.uniform(2, 3.5, n), mu=rng.uniform(0.5, 2.0, n), seed=31,
                            aspect=(1.4, 0.7))
    spec = S.SystemSpec(n=n, box=box, alpha=6.0 / box.min(), K_max=6, ksq_max=0, B=np.array([0.3, -0.4, 1.1]))
    with L.Batch([spec], [st]) as bt:
        for name, call, ofn in (
            ("dipR", lambda: bt.force_dipR(), lambda o, s: o.force_dipR(s, spec.alpha)),
            ("dipK", lambda: bt.force_dipK(), lambda o, s: o.force_dipK(s, spec.K_max, spec.alpha, 0)),
        ):
            bt.zero_forces()
            U, PT = call()
            d = bt.download(0)
            s = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, box)
            Uo, PTo = ofn(oracle.Oracle(), s)
            assert rms_rel(d["F"], s.F) < TOL_F, name
            assert rms_rel(d["T"], s.T) < TOL_F, name
            assert abs(U[0] - Uo) < TOL_F * max(abs(Uo), 1.0), name


def test_c1_size_forces_vs_oracle():
    """N = 4096 at packing fraction 0.20 (the 4096-particle configuration):
    real- and reciprocal-space forces against the FP64 oracle."""
    spec, st = S.plain_c1()
    orc = oracle.Oracle()
    import os

    orc.set_threads(os.cpu_count() or 1)
    with L.Batch([spec], [st]) as bt:
        bt.zero_forces()
        U, PT = bt.force_dipR()
        d = bt.download(0)
        s = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, spec.box)
        Uo, PTo = orc.force_dipR(s, spec.alpha)
        assert rms_rel(d["F"], s.F) < TOL_F and rms_rel(d["T"], s.T) < TOL_F
        # 64 strips: the energy and pressure tensor come through the per-strip sums
        assert abs(U[0] - Uo) < 1e-5 * abs(Uo) and rms_rel(PT[0], PTo) < TOL_F
        bt.zero_forces()
        U, PT = bt.force_dipK()
        d = bt.download(0)
        s = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, spec.box)
        Uo, PTo = orc.force_dipK(s, spec.K_max, spec.alpha, spec.ksq_max)
        # the k-space gather in parts (4096 rods, one dipole each)
        assert rms_rel(d["F"], s.F) < TOL_F and rms_rel(d["T"], s.T) < TOL_F
        assert abs(U[0] - Uo) < 1e-5 * abs(Uo) and rms_rel(PT[0], PTo) < TOL_F


def test_c2_size_properties():
    """N = 32768 (the chain-forming configuration in a field): a step runs,
    pair forces cancel (Newton's third law), clusters cover every particle."""
    spec, st = S.plain_c2()
    with L.Batch([spec], [st]) as bt:
        bt.zero_forces()
        bt.force_dipR()
        F = bt.download(0)["F"]
        assert np.all(np.isfinite(F))
        assert np.abs(F.sum(0)).max() < 1e-4 * np.abs(F).sum(0).max()
        obs = bt.step(3)[0]
        assert obs["status"] == 0 and obs["step"] == 3
        lab, nc = bt.clust_conf(0)
        assert lab.min() == 0 and lab.max() == nc - 1 and len(np.unique(lab)) == nc


def test_overlap_reported_like_the_reference():
    """Two rods whose segments come closer than 0.7 sigma: force_sc's abort
    (v25/functions.cpp:1454-1465) surfaces as MDSC_ERR_OVERLAP."""
    n = 2
    r = np.array([[5.0, 5.0, 5.0], [5.5, 5.0, 5.0]])
    O = np.stack([np.eye(3), np.eye(3)])
    st = S.SystemState(r, np.zeros((n, 3)), O, np.zeros((n, 3)), np.full(n, 2.0), np.ones(n), np.ones(n),
                       np.zeros((n, 1, 5)))
    st.dip[:, 0, 3] = 1.0
    st.dip[:, 0, 4] = 1.0
    spec = S.SystemSpec(n=n, box=np.full(3, 12.0), alpha=0.5, K_max=3, ksq_max=0)
    with L.Batch([spec], [st]) as bt:
        with pytest.raises(L.MdscError) as e:
            bt.force_sc()
        assert e.value.code == 4


def test_table_range_rejected():
    spec = S.SystemSpec(n=4, box=np.full(3, 120.0), alpha=0.05, K_max=3, ksq_max=0)
    st = S.SystemState(np.random.default_rng(0).uniform(0, 120, (4, 3)), np.zeros((4, 3)),
                       np.stack([np.eye(3)] * 4), np.zeros((4, 3)), np.full(4, 2.0), np.ones(4), np.ones(4),
                       np.zeros((4, 1, 5)))
    with pytest.raises(L.MdscError) as e:
        L.Batch([spec], [st])
    assert e.value.code == 6
