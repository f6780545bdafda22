"""The run loop (mdspherocyl_gb300/driver.py) on the GPU against the
reference's own driver: a restart (signal 1) and a continuation (signal 2)
of the reference's example input (two species, two off-axis dipoles per
rod), from the files the reference wrote, compared file by file with what
the reference wrote next (tests/golden/run_v25/).

Tolerances: the GPU's Ewald sums are FP32 (forces ~1e-6 relative), so
  energies per particle, pressures: 1e-5 relative (+1e-9)
  positions 1e-9, orientations 1e-8, momenta and angular momenta 1e-7
  generator states, cluster labels, counters, file layouts: identical
"""
import os
import shutil
import tempfile

import numpy as np
import pytest

from conftest import ROOT
from mdspherocyl_gb300 import files as F
from mdspherocyl_gb300.driver import Driver, layout

pytestmark = pytest.mark.gpu

GOLD = os.path.join(ROOT, "tests", "golden")
RUN = os.path.join(GOLD, "run_v25")


def _cmp_numbers(a, b, rel, abs_, what):
    ta, tb = a.split(), b.split()
    assert len(ta) == len(tb), (what, a, b)
    for x, y in zip(ta, tb):
        try:
            fx, fy = float(x), float(y)
        except ValueError:
            assert x == y, (what, a, b)
            continue
        assert abs(fx - fy) <= rel * abs(fy) + abs_, (what, x, y)


def _check_stage(d, stage, run=RUN):
    p = F.read_input(os.path.join(d, "input.txt"))
    ref = os.path.join(run, stage)
    # output.dat: one line per step (times of the run itself aside), then the report
    ours = open(os.path.join(d, "output.dat")).read().splitlines()
    theirs = open(os.path.join(ref, "output.dat")).read().splitlines()
    assert len(ours) == len(theirs)
    for a, b in zip(ours, theirs):
        if " | " in b and b[:1].isdigit() and b.split()[0].endswith("."):
            assert a.split()[0] == b.split()[0]  # Time
            _cmp_numbers(a.split(" | ")[1], b.split(" | ")[1], 1e-5, 1e-9, "output.dat")
        else:
            ta, tb = a.replace("+/-", " +/- "), b.replace("+/-", " +/- ")
            if "+/-" in a:  # averages; the fluctuations are differences of nearly equal sums
                va, vb = ta.split(), tb.split()
                assert len(va) == len(vb)
                for k, (x, y) in enumerate(zip(va, vb)):
                    if k + 1 < len(va) and va[k + 1] == "+/-":
                        _cmp_numbers(x, y, 1e-5, 1e-9, "report")
                    elif k > 0 and va[k - 1] == "+/-":
                        continue
                    else:
                        assert x == y
            else:
                _cmp_numbers(ta, tb, 1e-5, 1e-9, "report")
    # conf.dat
    length, dia, mass, dip, nd, nd_part = layout(p)
    a = F.read_conf(os.path.join(d, "conf.dat"), p.n_part, nd_part)
    b = F.read_conf(os.path.join(ref, "conf.dat"), p.n_part, nd_part)
    assert np.array_equal(a["box"], b["box"])
    assert np.abs(a["r"] - b["r"]).max() <= 1e-9
    assert np.abs(a["O"] - b["O"]).max() <= 1e-8
    assert np.abs(a["p"] - b["p"]).max() <= 1e-7 and np.abs(a["l"] - b["l"]).max() <= 1e-7
    assert np.array_equal(a["clust"], b["clust"])
    assert np.abs(a["xi"] - b["xi"]).max() <= 1e-9 and np.array_equal(a["strn"], b["strn"])
    # the generators drew the same numbers
    for k in range(2):
        x = open(os.path.join(d, f"ran_state{k}F.dat"), "rb").read()
        y = open(os.path.join(ref, f"ran_state{k}F.dat"), "rb").read()
        assert x[:4996] == y[:4996]
    # counters.dat: the clock and counters exactly, the sums to the tolerance
    ca = open(os.path.join(d, "counters.dat")).read().split()
    cb = open(os.path.join(ref, "counters.dat")).read().split()
    assert ca[:5] == cb[:5]
    _cmp_numbers(" ".join(ca[5:]), " ".join(cb[5:]), 1e-5, 1e-9, "counters.dat")
    # correlation.dat, ptens.dat, magmom.dat
    for f in ("correlation.dat", "ptens.dat", "magmom.dat"):
        la, lb = open(os.path.join(d, f)).read().splitlines(), open(os.path.join(ref, f)).read().splitlines()
        assert len(la) == len(lb), f
        for x, y in zip(la, lb):
            _cmp_numbers(x, y, 1e-5, 2e-8, f)


@pytest.mark.parametrize("variant", ["v25", "v251"])
def test_restart_and_continue_like_the_reference(variant):
    """v25: two species, off-axis dipoles; v251 (the later driver): rods of
    length 9 with an axial dipole in a field, clustering every step, the
    degree-of-polymerisation counters."""
    run = os.path.join(GOLD, f"run_{variant}")
    with tempfile.TemporaryDirectory() as d:
        for f in ("conf.dat", "ran_state0F.dat", "ran_state1F.dat", "counters.dat", "correlation.dat"):
            shutil.copy(os.path.join(run, "init", f), d)
        shutil.copy(os.path.join(run, "restart", "input.txt"), d)
        with open(os.devnull, "w") as devnull:
            assert Driver(d, out=devnull, variant=variant).run() == 0, open(os.path.join(d, "Error.dat")).read()
        _check_stage(d, "restart", run)
        shutil.copy(os.path.join(run, "continue", "input.txt"), d)
        os.remove(os.path.join(d, "output.dat"))
        with open(os.devnull, "w") as devnull:
            assert Driver(d, out=devnull, variant=variant).run() == 0, open(os.path.join(d, "Error.dat")).read()
        _check_stage(d, "continue", run)


def test_new_run_writes_every_file():
    """Signal 0: a configuration of its own, then the same files."""
    with tempfile.TemporaryDirectory() as d:
        shutil.copy(os.path.join(RUN, "init", "input.txt"), d)
        with open(os.devnull, "w") as devnull:
            assert Driver(d, out=devnull).run() == 0, open(os.path.join(d, "Error.dat")).read()
        for f in ("conf.dat", "ran_state0F.dat", "ran_state1F.dat", "counters.dat", "correlation.dat",
                  "ptens.dat", "magmom.dat", "output.dat", os.path.join("pos_vel", "pos_vel_0.dat")):
            assert os.path.getsize(os.path.join(d, f)) > 0, f
        assert open(os.path.join(d, "Error.dat")).read() == ""
        # time.dat in the reference's layout, from the GPU kernels' times
        lines = open(os.path.join(d, "time.dat")).read().splitlines()
        assert [ln.split(".")[0] for ln in lines] == ["X move time", "Force_ss time", "P move time", "correl"]
        assert all(float(ln.split("elap:")[1].split()[0]) > 0 for ln in lines[:3])


def test_new_run_lattice_is_the_references():
    """Signal 0: the lattice on the GPU is ini_pos's -- iniPos.dat byte for
    byte what the reference wrote for its own example (two species on one
    lattice: the second species takes the sites the first left free)."""
    with tempfile.TemporaryDirectory() as d:
        shutil.copy(os.path.join(RUN, "init", "input.txt"), d)
        with open(os.devnull, "w") as devnull:
            assert Driver(d, out=devnull).run() == 0, open(os.path.join(d, "Error.dat")).read()
        assert open(os.path.join(d, "iniPos.dat")).read() == open(os.path.join(RUN, "init", "iniPos.dat")).read()


def test_thermalize_momenta():
    """mdsc_thermalize: zero total momentum, the equipartition temperature
    within the sampling error, the same draws for the same seed."""
    from mdspherocyl_gb300 import lib as L
    from mdspherocyl_gb300 import systems as S

    rng = np.random.default_rng(3)
    st, box = S.make_system(n=3000, phi=0.1, lengths=rng.uniform(1, 3, 3000), mu=np.ones(3000), seed=3,
                            mass=rng.uniform(0.5, 2.0, 3000))
    spec = S.SystemSpec(n=3000, box=box, alpha=5.0 / box[0], K_max=4, ksq_max=0)
    with L.Batch([spec], [st]) as bt:
        bt.thermalize(0, 1.7, seed=11)
        a = bt.download(0)
        bt.thermalize(0, 1.7, seed=11)
        b = bt.download(0)
    assert np.array_equal(a["p"], b["p"]) and np.array_equal(a["l"], b["l"])
    assert np.abs(a["p"].sum(axis=0)).max() < 1e-10
    Kt = 0.5 * np.sum(a["p"] ** 2 / st.mass[:, None])
    assert abs(2 * Kt / (3 * 3000) - 1.7) < 0.05 * 1.7
    I = S.inertia(st.length, st.dia, st.mass)
    lb = np.einsum("nab,nb->na", st.O, a["l"])  # body frame
    Kr = 0.5 * np.sum(lb ** 2 / I)
    assert abs(2 * Kr / (3 * 3000) - 1.7) < 0.05 * 1.7


def test_library_knobs_in_the_run_loop():
    """The driver's own options -- a real-space cutoff, a spherical k-set,
    clusters by pair energy -- run the reference's example restart to the
    end with every file written; the energy criterion changes the labels."""
    run = os.path.join(GOLD, "run_v251")
    labels = {}
    for ce in (0.0, 0.5):
        with tempfile.TemporaryDirectory() as d:
            for f in ("conf.dat", "ran_state0F.dat", "ran_state1F.dat", "counters.dat", "correlation.dat"):
                shutil.copy(os.path.join(run, "init", f), d)
            shutil.copy(os.path.join(run, "restart", "input.txt"), d)
            p = F.read_input(os.path.join(d, "input.txt"))
            length, dia, mass, dip, nd, nd_part = layout(p)
            box = F.read_conf(os.path.join(d, "conf.dat"), p.n_part, nd_part)["box"]
            with open(os.devnull, "w") as devnull:
                drv = Driver(d, out=devnull, variant="v251", rc_real=0.4 * float(min(box)), ksq_max=16,
                             cl_energy=ce)
                assert drv.run() == 0, open(os.path.join(d, "Error.dat")).read()
            c = F.read_conf(os.path.join(d, "conf.dat"), p.n_part, nd_part)
            assert np.all(np.isfinite(c["r"])) and np.all(np.isfinite(c["p"]))
            labels[ce] = c["clust"]
            assert os.path.getsize(os.path.join(d, "output.dat")) > 0
    assert not np.array_equal(labels[0.0], labels[0.5])
