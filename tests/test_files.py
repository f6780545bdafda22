"""The reference's run files (mdspherocyl_gb300/files.py) against files its
own driver wrote (tests/golden/run_v25/, made by tests/golden/make_golden.py
from v25/input.txt: two species, two off-axis dipoles per rod).  No GPU."""
import math
import os
import tempfile

import numpy as np
import pytest

from conftest import ROOT
from mdspherocyl_gb300 import files as F
from mdspherocyl_gb300.driver import layout

GOLD = os.path.join(ROOT, "tests", "golden")
RUN = os.path.join(GOLD, "run_v25")
# both drivers' runs: v25 (two species, off-axis dipoles) and v251 (one species, field, clusters every step)
STAGES = tuple(f"{r}/{s}" for r in ("run_v25", "run_v251") for s in ("init", "restart", "continue"))


def _v251(stage):
    return stage.startswith("run_v251")


def _init(stage):
    return os.path.join(GOLD, stage.split("/")[0], "init")


def _nums(tokens):
    out = []
    for t in tokens:
        try:
            out.append(float(t))
        except ValueError:
            out.append(t)
    return out


def test_input_round_trip():
    p = F.read_input(os.path.join(RUN, "init", "input.txt"))
    assert (p.Nsteps, p.pre_steps, p.signal, p.n_part, p.iprint) == (2, 0, 0, [50, 50], 1)
    assert p.length == [1.0, 1.0] and p.mass == [1.0, 1.0] and p.dens == 0.005 and p.K_max == 10
    assert p.alpha == 0.75 and p.bar_w == 0.1 and p.Dt == 1e-4 and p.sr_cut == 3.1 and p.cl_fr == 2
    assert np.allclose(p.dip[0], [[-0.5, 0.81915204, 0.57357644, 0, 1.5], [0.5, 1, 0, 0, 2]])
    assert np.allclose(p.dip[1], [[-0.5, 0.81915204, -0.57357644, 0, 1.5], [0.5, 1, 0, 0, 2]])
    with tempfile.TemporaryDirectory() as d:
        F.write_input(os.path.join(d, "input.txt"), p)
        q = F.read_input(os.path.join(d, "input.txt"))
    for k, v in vars(p).items():
        w = getattr(q, k)
        if k == "dip":
            assert all(np.array_equal(a, b) for a, b in zip(v, w))
        else:
            assert np.array_equal(np.asarray(v), np.asarray(w)), k


@pytest.mark.parametrize("stage", STAGES)
def test_conf_round_trip(stage):
    """conf.dat read and written again: every token equal, except the lab
    dipole coordinates, which follow from r and O as printed (12 decimals)
    and so may differ by one unit in the last place."""
    p = F.read_input(os.path.join(GOLD, stage, "input.txt"))
    length, dia, mass, dip, nd, nd_part = layout(p)
    src = os.path.join(GOLD, stage, "conf.dat")
    c = F.read_conf(src, p.n_part, nd_part)
    assert c["r"].shape == (p.n_total, 3) and np.all(c["mass"] == 1.0)
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "conf.dat")
        F.write_conf(out, c["box"], c["r"], c["p"], c["O"], c["l"], mass, dip, c["clust"], c["xi"], c["strn"],
                     ndip=np.repeat(nd_part, p.n_part))
        a, b = open(src).read().splitlines(), open(out).read().splitlines()
    assert len(a) == len(b) and a[0] == b[0] and a[-2:] == b[-2:]
    for la, lb in zip(a[1:-2], b[1:-2]):
        ta, tb = la.split(" "), lb.split(" ")
        assert len(ta) == len(tb)
        head = 18 + 3  # r p O l, '', '|', mass
        assert ta[:head] == tb[:head] and ta[-1] == tb[-1]
        for x, y in zip(ta[head:-1], tb[head:-1]):
            if x in (".", "") or y in (".", ""):
                assert x == y
            else:
                assert abs(float(x) - float(y)) <= 2.5e-12


@pytest.mark.parametrize("stage", STAGES)
def test_generator_state_and_counters_round_trip(stage):
    with tempfile.TemporaryDirectory() as d:
        for k in range(2):
            src = os.path.join(GOLD, stage, f"ran_state{k}F.dat")
            mt, mti = F.read_mt_state(src)
            assert mt.shape == (624,) and 0 <= mti <= 624
            F.write_mt_state(os.path.join(d, "s.dat"), mt, mti)
            # the 4 bytes of struct padding after the position are whatever the
            # reference's memory held; everything before them is equal
            a, w = open(src, "rb").read(), open(os.path.join(d, "s.dat"), "rb").read()
            assert len(a) == len(w) == 5000 and a[:4996] == w[:4996]
        src = os.path.join(GOLD, stage, "counters.dat")
        got = F.read_counters(src, npc=_v251(stage))
        F.write_counters(os.path.join(d, "c.dat"), *got[:7], npc=got[7] if _v251(stage) else None)
        assert open(src).read() == open(os.path.join(d, "c.dat")).read()


def test_thermostat_state_continues_the_seeded_sequence():
    """ran_state0F.dat after the two steps of the new run: the thermostat's
    generator seeded 1 has drawn two uniforms per step (one normal pair,
    v25/functions.cpp:2196-2199) -- so the state is MT19937(1) advanced 4
    draws, and the refill happened at the first draw."""
    mt, mti = F.read_mt_state(os.path.join(RUN, "init", "ran_state0F.dat"))
    assert mti == 4
    # the state words after one refill of MT19937 seeded 1: its first output
    # tempered from word 0 must be the known first value 1791095845
    y = int(mt[0])
    y ^= y >> 11
    y ^= (y << 7) & 0x9d2c5680
    y ^= (y << 15) & 0xefc60000
    y ^= y >> 18
    assert y & 0xffffffff == 1791095845


@pytest.mark.parametrize("stage", STAGES)
def test_output_lines_and_report(stage):
    """output.dat: every step line printed again from its own values is the
    same line; the closing report rebuilt from counters.dat has the same
    text and, within the rounding counters.dat imposes, the same averages."""
    p = F.read_input(os.path.join(GOLD, stage, "input.txt"))
    lines = open(os.path.join(GOLD, stage, "output.dat")).read().splitlines()
    steps = [ln for ln in lines if " | " in ln and ln[:1].isdigit() and ln.split()[0].endswith(".")]
    assert len(steps) == p.Nsteps
    for ln in steps:
        head, vals = ln.split(" | ")
        t = head.split()
        v = [float(x) for x in vals.split()]
        var = F.Accumulator()
        (var.K, var.U, var.P, var.Uss, var.Pss, var.UdipR, var.PdipR, var.UdipK, var.PdipK) = v[:9]
        Mom = [math.sqrt(v[9]), 0.0, 0.0, math.sqrt(v[10]), 0.0, 0.0]
        again = F.output_line(float(t[0][:-1]), float(t[1]), float(t[2]), var, Mom)
        ta, tb = ln.split(), again.split()
        assert ta[:-2] == tb[:-2]  # the momentum squares pass through a square root here
        assert abs(float(ta[-1]) - float(tb[-1])) <= 1e-12 and abs(float(ta[-2]) - float(tb[-2])) <= 1e-12
    got = F.read_counters(os.path.join(GOLD, stage, "counters.dat"), npc=_v251(stage))
    Time, cont, Ntcf, Ntcv, mcont, AcT, AcTsq = got[:7]
    pol = got[7][1] / (p.n_total * got[7][0]) if _v251(stage) else None
    if p.signal == 0:
        Lz = (p.n_total / (p.ArLx * p.ArLy * p.dens)) ** (1.0 / 3)
        box = (p.ArLx * Lz, p.ArLy * Lz, Lz)
    else:
        box = tuple(float(x) for x in open(os.path.join(_init(stage), "conf.dat")).readline().split())
    rep = F.final_report(Time, AcT, AcTsq, cont, p, box, pol_deg=pol).splitlines()
    tail = lines[-len(rep):]
    assert tail[0] == "NVT ensemble"
    for a, b in zip(tail, rep):
        ta, tb = a.replace("+/-", " +/- ").split(), b.replace("+/-", " +/- ").split()
        assert len(ta) == len(tb), (a, b)
        prev = None
        for x, y in zip(_nums(ta), _nums(tb)):
            if isinstance(x, str) or isinstance(y, str):
                assert x == y, (a, b)
            elif prev != "+/-":  # averages; fluctuations cancel and are not reproducible from 12 decimals
                assert abs(x - y) <= 2e-5 * abs(x) + 1e-12, (a, b)
            prev = x if isinstance(x, str) else None


@pytest.mark.parametrize("stage", STAGES)
def test_correlation_file(stage):
    """correlation.dat read back into histograms and normalised again: the
    bin columns are the same text and the functions agree to the
    precision the file keeps."""
    p = F.read_input(os.path.join(GOLD, stage, "input.txt"))
    src = os.path.join(GOLD, stage, "correlation.dat")
    box = [float(x) for x in open(os.path.join(GOLD, stage, "conf.dat")).readline().split()]
    if p.signal == 0:
        Lz = (p.n_total / (p.ArLx * p.ArLy * p.dens)) ** (1.0 / 3)
        box = [p.ArLx * Lz, p.ArLy * Lz, Lz]
    Lmin = min(box)
    nbins = int(math.floor(math.sqrt(3.0) * Lmin / (2.0 * p.bar_w)))
    cor_cont, hist = F.read_correlation(src, p.n_part, nbins)
    nc = p.n_comp
    assert hist.shape == (nc + nc * (nc - 1) // 2, 4, nbins) and cor_cont > 0
    # intra counts: even integers; inter counts: integers
    assert np.allclose(hist[:nc, 0], np.round(hist[:nc, 0] / 2) * 2, atol=1e-3)
    assert np.allclose(hist[nc:, 0], np.round(hist[nc:, 0]), atol=1e-3)
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "c.dat")
        F.write_correlation(out, hist, p.n_part, Lmin, p.bar_w, cor_cont)
        a, b = open(src).read().splitlines(), open(out).read().splitlines()
    assert len(a) == len(b) == nbins
    for k, (la, lb) in enumerate(zip(a, b)):
        ta, tb = la.split(), lb.split()
        assert len(ta) == len(tb) and ta[1:4] == tb[1:4], (k, la, lb)
        for x, y in zip(_nums(ta[4:]), _nums(tb[4:])):
            if isinstance(x, str):
                assert x == y
            else:
                assert abs(x - y) <= 1e-5 * abs(x) + 2e-8, (k, x, y)


@pytest.mark.parametrize("stage", STAGES)
def test_ptens_magmom_pos_vel_lines(stage):
    with tempfile.TemporaryDirectory() as d:
        for ln in open(os.path.join(GOLD, stage, "ptens.dat")).read().splitlines():
            t = ln.split()
            v = [float(x) for x in t]
            assert F.ptens_line(v[0], np.array(v[1:10]), np.array(v[10:19])).rstrip("\n") == ln
        for ln in open(os.path.join(GOLD, stage, "magmom.dat")).read().splitlines():
            v = [float(x) for x in ln.split()]
            assert F.magmom_line(v[0], v[1:4]).rstrip("\n") == ln
        pv = os.path.join(_init(stage), "pos_vel", "pos_vel_0.dat")
        lines = open(pv).read().splitlines()
        rows = []
        for ln in lines[:-1]:
            a, b = ln.split(" | ")
            x, y = [float(v) for v in a.split()], [float(v) for v in b.split()]
            rows.append((x[:3], x[3:], y[:3], y[3:]))
        p = F.read_input(os.path.join(_init(stage), "input.txt"))
        assert len(rows) == sum(min(25, k) for k in p.n_part)  # up to 25 of each species
        F.write_pos_vel(os.path.join(d, "pv.dat"), rows, float(lines[-1]))
        assert open(os.path.join(d, "pv.dat")).read() == open(pv).read()


@pytest.mark.parametrize("run", ["run1", "run2"])
def test_shipped_restart_states(run):
    """The restart states the reference ships (v25/run1: 64-bit generator
    files of 5000 bytes; v25/run2: a 32-bit build's, 2500 bytes): input,
    configuration, counters and generator states read, the configuration
    written back token for token.  Runs where the reference is present."""
    from conftest import REFERENCE

    d = os.path.join(REFERENCE, "v25", run)
    if not os.path.isdir(d):
        pytest.skip("reference run directories not present")
    p = F.read_input(os.path.join(d, "input.txt"))
    length, dia, mass, dip, nd, nd_part = layout(p)
    c = F.read_conf(os.path.join(d, "conf.dat"), p.n_part, nd_part)
    assert c["r"].shape == (p.n_total, 3)
    assert np.allclose(np.einsum("nab,ncb->nac", c["O"], c["O"]), np.eye(3), atol=1e-8)  # orthonormal frames
    for k in range(2):
        mt, mti = F.read_mt_state(os.path.join(d, f"ran_state{k}F.dat"))
        assert 0 <= mti <= 624 and mt.dtype == np.uint32
    F.read_counters(os.path.join(d, "counters.dat"))
    with tempfile.TemporaryDirectory() as t:
        out = os.path.join(t, "conf.dat")
        F.write_conf(out, c["box"], c["r"], c["p"], c["O"], c["l"], mass, dip, c["clust"], c["xi"], c["strn"],
                     ndip=np.repeat(nd_part, p.n_part))
        a, b = open(os.path.join(d, "conf.dat")).read().split(), open(out).read().split()
    assert len(a) == len(b)
    diff = [(x, y) for x, y in zip(a, b) if x != y]
    # only lab dipole coordinates may differ, in the last printed place
    assert all(abs(float(x) - float(y)) <= 2.5e-12 for x, y in diff)
