"""Makes the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own routines (oracle/_ref/libmdsc_ref.so, compiled by
oracle/build_ref.sh from the reference's unmodified sources) on small
seeded systems and stores inputs and outputs in golden_*.npz.  These
fixtures travel with the repository, so the oracle restatement and the GPU
path can be checked against the reference where its sources are absent.

  python tests/golden/make_golden.py

run_v25/ and run_v251/ hold the files the reference's two drivers write on
their own example inputs, for the file-format and driver tests.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from mdspherocyl_gb300 import systems as S  # noqa: E402


def two_dipole_system(seed, n=48):
    """Rods with two off-axis dipoles each, as in the reference's own input
    (v25/input.txt: offsets -0.5 and 0.5, tilted directions)."""
    rng = np.random.default_rng(seed)
    lengths = rng.uniform(1.0, 2.0, n)
    st, box = S.make_system(n=n, phi=0.08, lengths=lengths, mu=np.ones(n), seed=seed)
    dip = np.zeros((n, 2, 5))
    dip[:, 0] = [-0.5, 0.81915204, 0.57357644, 0.0, 1.5]
    dip[:, 1] = [0.5, 1.0, 0.0, 0.0, 2.0]
    st.dip = dip
    return st, box


def cases():
    out = []
    spec, st = S.plain_c0(seed=11, n=64)
    out.append(("c0_n64", st, spec.box, spec.alpha, spec.K_max, spec.ksq_max))
    spec, st = S.plain_c0(seed=12, n=40)
    st.O = st.O.copy()
    out.append(("c0_n40_cube", st, spec.box, spec.alpha, 5, 0))
    st, box = two_dipole_system(13)
    out.append(("twodip_n48", st, box, 5.0 / box[0], 5, 0))
    # dense: contacts for force_sc and multi-particle clusters
    rng = np.random.default_rng(14)
    st, box = S.make_system(n=64, phi=0.25, lengths=rng.uniform(2, 3, 64), mu=np.full(64, 1.3), seed=14)
    out.append(("dense_n64", st, box, 6.0 / box[0], 6, 27))
    return out


def run_case(ref: oracle.Ref, name, st, box, alpha, K_max, ksq):
    def mk():
        return oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, box)

    d = dict(r=st.r, p=st.p, O=st.O, l=st.l, length=st.length, dia=st.dia, mass=st.mass, dip=st.dip,
             box=box, alpha=alpha, K_max=K_max, ksq_max=ksq)
    B = np.array([0.4, -0.3, 0.7])
    d["B"] = B
    s = mk()
    ok, U, W, PT = ref.force_sc(s, 3.0, 3.5)
    d.update(sc_ok=ok, sc_U=U, sc_W=W, sc_PT=PT, sc_F=s.F.copy(), sc_T=s.T.copy())
    s = mk()
    U, PT = ref.force_dipR(s, alpha)
    d.update(dipR_U=U, dipR_PT=PT, dipR_F=s.F.copy(), dipR_T=s.T.copy())
    s = mk()
    U, PT = ref.force_dipK(s, K_max, alpha, ksq)
    d.update(dipK_U=U, dipK_PT=PT, dipK_F=s.F.copy(), dipK_T=s.T.copy())
    s = mk()
    U = ref.ext_field(s, B)
    d.update(ext_U=U, ext_T=s.T.copy())
    d["self_U"] = ref.self_ener(mk())
    rng = np.random.default_rng(99)
    F0 = rng.normal(size=(st.n, 3))
    T0 = rng.normal(size=(st.n, 3))
    d.update(mp_F=F0, mp_T=T0, mp_xi=np.array([0.3, -0.2]), dt=1e-3)
    for last in (0, 1):
        s = mk()
        s.F[:] = F0
        s.T[:] = T0
        K, PT = ref.moveP(s, d["mp_xi"], 1e-3, bool(last))
        d.update({f"mp{last}_K": K, f"mp{last}_PT": PT, f"mp{last}_p": s.p.copy(), f"mp{last}_l": s.l.copy()})
    s = mk()
    ref.moveX(s, 1e-3)
    d.update(mx_r=s.r.copy(), mx_O=s.O.copy())
    s = mk()
    ref.renorm(s)
    d.update(rn_O=s.O.copy())
    for ms in (0.1, 0.6):
        s = mk()
        lab, nxt = ref.clust_conf(s, ms, seed=1, skip=7)
        d[f"cl{ms}_labels"] = lab
        d[f"cl{ms}_next"] = nxt
    counts, idx = ref.neigh_list(mk(), 3.5)
    d.update(nl_counts=counts, nl_idx=idx)
    # observables: pair correlations with ~170 bins, order parameters
    bar_w = float(min(box)) / 200.0
    nbins = int(np.floor(np.sqrt(3.0) * float(min(box)) / (2.0 * bar_w)))
    d.update(corr_bar_w=bar_w, corr_hist=ref.acc_correl(mk(), bar_w, nbins))
    G1, G2, M = ref.oo_params(mk())
    d.update(oo_G1=G1, oo_G2=G2, oo_M=M)
    return d


def driver_trajectory():
    """The reference driver (oracle/_ref/DSCmd_v25) restarted from a seeded
    state: 30 steps with a noisy thermostat, a tilted off-axis dipole, a
    field and clusters every 7 steps.  Stores the start, the printed
    per-step observables and the final conf.dat (state and labels)."""
    import tempfile

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import refdriver
    from test_reference_driver import driver_case

    st, box, p = driver_case()
    with tempfile.TemporaryDirectory() as d:
        refdriver.write_run(d, r=st.r, p=st.p, O=st.O, l=st.l, L=2.5, D=1.0, m=1.0, dip=st.dip[0], box=box,
                            xi=p["xi"], strn=p["strn"], steps=p["steps"], T=p["T"], Q=p["Q"], gamma=p["gamma"],
                            dt=p["dt"], sr_cut=p["sr_cut"], K=p["K"], alpha=p["alpha"], B=p["B"],
                            cl_fr=p["cl_fr"], min_s=p["min_s"])
        refdriver.run(d, os.path.join(oracle.REF_DIR, "DSCmd_v25"))
        out = refdriver.read_output(d)
        fin = refdriver.read_conf(d, st.n, 1)
    return dict(r=st.r, p=st.p, O=st.O, l=st.l, length=st.length, dia=st.dia, mass=st.mass, dip=st.dip,
                box=box, T=p["T"], Q=p["Q"], gamma=p["gamma"], dt=p["dt"], sr_cut=p["sr_cut"], K_max=p["K"],
                alpha=p["alpha"], B=p["B"], cl_fr=p["cl_fr"], min_s=p["min_s"], xi=p["xi"], strn=p["strn"],
                steps=p["steps"], out=out, fin_r=fin["r"], fin_p=fin["p"], fin_O=fin["O"], fin_l=fin["l"],
                fin_clust=fin["clust"], fin_xi=fin["xi"])


RUN_FILES = ("input.txt", "iniPos.dat", "conf.dat", "ran_state0F.dat", "ran_state1F.dat", "counters.dat",
             "correlation.dat",
             "ptens.dat", "magmom.dat", "output.dat", os.path.join("pos_vel", "pos_vel_0.dat"),
             os.path.join("pos_vel", "pos_vel_1.dat"))


def _edit_input(text, **kv):
    """v25/input.txt with some lines replaced (label prefix -> new line)."""
    out = []
    for ln in text.splitlines():
        for prefix, new in kv.items():
            if ln.startswith(prefix):
                ln = new
        out.append(ln)
    return "\n".join(out) + "\n"


def _run_stages(src, common, binary, outdir):
    """init (signal 0, 2 steps), restart (signal 1, 3 steps) and continue
    (signal 2, 2 steps) of one input in one directory, each stage's files
    copied to outdir/<stage>."""
    import shutil
    import subprocess
    import tempfile

    drv = os.path.join(oracle.REF_DIR, binary)
    stages = (("init", 0, 2), ("restart", 1, 3), ("continue", 2, 2))
    with tempfile.TemporaryDirectory() as d:
        for name, sig, steps in stages:
            text = _edit_input(src, **common, **{"No. of steps=": f"No. of steps=\t\t{steps}",
                                               "Signal=": f"Signal=\t\t\t{sig}"})
            open(os.path.join(d, "input.txt"), "w").write(text)
            if os.path.exists(os.path.join(d, "output.dat")):
                os.remove(os.path.join(d, "output.dat"))
            subprocess.run([drv], cwd=d, env=dict(os.environ, OMP_NUM_THREADS="1"), stdout=subprocess.DEVNULL,
                           timeout=1200, check=True)
            dst = os.path.join(HERE, outdir, name)
            os.makedirs(os.path.join(dst, "pos_vel"), exist_ok=True)
            for f in RUN_FILES:
                if os.path.exists(os.path.join(d, f)) and (f != "iniPos.dat" or sig == 0):
                    shutil.copy(os.path.join(d, f), os.path.join(dst, f))
            shutil.rmtree(os.path.join(d, "pos_vel"), ignore_errors=True)
            print("wrote", dst)


def run_files():
    """The reference driver's run files on its own example input
    (v25/input.txt: two species of 50 rods, two off-axis dipoles each),
    shortened: a new run of 2 steps with every output every step (init/),
    then a restart (signal 1) of 3 steps from its files (restart/) and a
    continuation (signal 2) of 2 steps (continue/)."""
    ref = oracle.reference_root()
    src = open(os.path.join(ref, "v25", "input.txt")).read()
    common = {"Histogram bar width=": "Histogram bar width=\t0.1", "corr. sum freq.=": "corr. sum freq.=\t1",
              "DiffCorr. frequency=": "DiffCorr. frequency=    1", "ViscCorr. frequency=": "ViscCorr. frequency=    1",
              "Steps before average=": "Steps before average=\t0", "clustering frequency=": "clustering frequency=\t2"}
    _run_stages(src, common, "DSCmd_v25", "run_v25")


def run_files_v251():
    """The same three stages with the later driver (v25/v251) on its own
    example (v25/v251/run1/input.txt: rods of length 9 with an axial dipole
    in a field), at 200 rods and the same density, clustering every step."""
    ref = oracle.reference_root()
    src = open(os.path.join(ref, "v25", "v251", "run1", "input.txt")).read()
    common = {"Histogram bar width=": "Histogram bar width=\t0.5", "corr. sum freq.=": "corr. sum freq.=\t1",
              "DiffCorr. frequency=": "DiffCorr. frequency=    1", "ViscCorr. frequency=": "ViscCorr. frequency=    1",
              "Steps before average=": "Steps before average=\t0", "clustering frequency=": "clustering frequency=\t1",
              "Printing frequency=": "Printing frequency=\t1", "No. of Particles=": "No. of Particles=\t200",
              "proximity dist.=": "proximity dist.=\t1.5"}
    _run_stages(src, common, "DSCmd_v251", "run_v251")


def main():
    if not os.path.exists(oracle.REF_SO):
        oracle.build_ref()
    ref = oracle.Ref()
    for name, st, box, alpha, K, ksq in cases():
        d = run_case(ref, name, st, box, alpha, K, ksq)
        path = os.path.join(HERE, f"golden_{name}.npz")
        np.savez_compressed(path, **d)
        print("wrote", path, os.path.getsize(path), "bytes")
    path = os.path.join(HERE, "driver_trajectory.npz")
    np.savez_compressed(path, **driver_trajectory())
    print("wrote", path, os.path.getsize(path), "bytes")
    run_files()
    run_files_v251()


if __name__ == "__main__":
    main()
