"""The reference's own driver, built from its unmodified sources
(oracle/build_ref.sh), against the golden vectors the reference ships, and
the oracle's whole-step restatement against that driver."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
import refdriver
from conftest import REFERENCE
from mdspherocyl_gb300 import systems as S

V25 = os.path.join(REFERENCE, "v25")


def _need_driver(name):
    if not os.path.isdir(V25):
        pytest.skip("reference sources not present")
    path = os.path.join(oracle.REF_DIR, name)
    if not os.path.exists(path):
        oracle.build_ref()
    return path


def _physics(lines):
    return [ln.split("|")[1].split() for ln in lines if "|" in ln and ln[:1].isdigit()]


def test_v25_golden_vector():
    """v25/input.txt (N=100, two species, two off-axis dipoles per particle,
    noisy thermostat): iniPos.dat byte-exact, and the first 20 steps of
    output.dat equal to a segment the reference ships (every printed digit)."""
    drv = _need_driver("DSCmd_v25")
    with tempfile.TemporaryDirectory() as d:
        src = open(os.path.join(V25, "input.txt")).read().splitlines()
        src = [("No. of steps=\t\t1" if ln.startswith("No. of steps=") else
                "Steps before average=\t20" if ln.startswith("Steps before average=") else ln) for ln in src]
        open(os.path.join(d, "input.txt"), "w").write("\n".join(src) + "\n")
        subprocess.run([drv], cwd=d, env=dict(os.environ, OMP_NUM_THREADS="1"), stdout=subprocess.DEVNULL,
                       timeout=300, check=True)
        assert open(os.path.join(d, "iniPos.dat"), "rb").read() == open(os.path.join(V25, "iniPos.dat"), "rb").read()
        ours = _physics(open(os.path.join(d, "output.dat")).read().splitlines())[:20]
        shipped = open(os.path.join(V25, "output.dat")).read().splitlines()
        starts = [i for i, ln in enumerate(shipped) if ln.startswith("0.000100000000.")]
        assert any(_physics(shipped[s:s + 20]) == ours for s in starts)


def test_v251_run1_golden_vector():
    """v25/v251/run1 (N=500 rods, axial dipole, field, clusters every 10
    steps): conf.dat -- state and cluster labels -- and the other outputs
    byte-exact."""
    drv = _need_driver("DSCmd_v251")
    run1 = os.path.join(V25, "v251", "run1")
    with tempfile.TemporaryDirectory() as d:
        shutil.copy(os.path.join(run1, "input.txt"), d)
        subprocess.run([drv], cwd=d, env=dict(os.environ, OMP_NUM_THREADS="1"), stdout=subprocess.DEVNULL,
                       timeout=600, check=True)
        for f in ("conf.dat", "iniPos.dat", "counters.dat", "correlation.dat", "compConf.dat"):
            assert open(os.path.join(d, f), "rb").read() == open(os.path.join(run1, f), "rb").read(), f
        ours = _physics(open(os.path.join(d, "output.dat")).read().splitlines())
        shipped = _physics(open(os.path.join(run1, "output.dat")).read().splitlines())
        assert len(ours) >= 11 and ours[:11] == shipped[:11]


def driver_case(seed=21, n=60, steps=30, gamma=1.0, cl_fr=7):
    rng = np.random.default_rng(seed)
    st, box = S.make_system(n=n, phi=0.06, lengths=np.full(n, 2.5), mu=np.full(n, 1.4), seed=seed,
                            temp=1.0)
    dip = np.array([[0.3, 0.6, 0.0, 0.8, 1.4]])
    st.dip = np.broadcast_to(dip, (n, 1, 5)).copy()
    p = dict(T=1.0, Q=5.0, gamma=gamma, dt=1e-3, sr_cut=4.5, K=5, alpha=6.0 / box[0], B=np.array([0.1, 0.0, 0.6]),
             cl_fr=cl_fr, min_s=0.4, xi=np.array([0.2, -0.1]), strn=np.array([0.0, 0.0]), steps=steps)
    return st, box, p


def test_oracle_step_matches_reference_driver():
    """The oracle's restatement of the driver's loop body (thermostat with
    noise, renorm, kicks, drift, forces, list checks, clusters) against the
    reference driver restarted from the same state: every printed digit of
    every step, and the final state and cluster labels."""
    drv = _need_driver("DSCmd_v25")
    st, box, p = driver_case()
    n = st.n
    with tempfile.TemporaryDirectory() as d:
        refdriver.write_run(d, r=st.r, p=st.p, O=st.O, l=st.l, L=2.5, D=1.0, m=1.0, dip=st.dip[0], box=box,
                            xi=p["xi"], strn=p["strn"], steps=p["steps"], T=p["T"], Q=p["Q"], gamma=p["gamma"],
                            dt=p["dt"], sr_cut=p["sr_cut"], K=p["K"], alpha=p["alpha"], B=p["B"],
                            cl_fr=p["cl_fr"], min_s=p["min_s"])
        refdriver.run(d, drv)
        out = refdriver.read_output(d)
        fin = refdriver.read_conf(d, n, 1)
    assert len(out) == p["steps"]
    orc = oracle.Oracle()
    o = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, box)
    md = oracle.MDOracle(orc, o, dt=p["dt"], temp=p["T"], Q=p["Q"], gamma=p["gamma"], xi0=0.0, sr_cut=p["sr_cut"],
                         K_max=p["K"], ksq_max=0, alpha=p["alpha"], B=p["B"], cl_fr=p["cl_fr"], min_s=p["min_s"])
    md.set_thermostat(p["xi"], p["strn"])
    V = float(np.prod(box))
    for k in range(p["steps"]):
        assert md.step()
        ob = md.obs()
        K = (ob["K"][0] + ob["K"][1]) / n
        U = ob["Uself"] / n + (ob["Uss"] + ob["UdipR"] + ob["UdipK"] + ob["Uext"]) / n
        row = [K, U, None, ob["Uss"] / n, ob["Wss"] / (3 * V), ob["UdipR"] / n, ob["UdipR"] / V,
               ob["UdipK"] / n, ob["UdipK"] / V]
        for c, v in enumerate(row):
            if v is not None:
                assert abs(v - out[k][c]) <= 1.5e-12 + 1e-12 * abs(v), (k, c, v, out[k][c])
    assert np.abs(o.r - fin["r"]).max() < 1e-11
    assert np.abs(o.p - fin["p"]).max() < 1e-11
    assert np.abs(o.O - fin["O"]).max() < 1e-11
    assert np.abs(o.l - fin["l"]).max() < 1e-11
    assert np.array_equal(o.clust, fin["clust"])
    assert np.abs(ob["xi"] - fin["xi"]).max() < 1e-11
