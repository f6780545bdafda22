"""The reference's run files, read and written in its own formats.

mdSpherocyl keeps a run in plain files in its working directory; this module
reads and writes them byte for byte as the reference's iostream code does
(fixed 12 decimals where it sets them, C++'s default six significant digits
elsewhere), so a run can move between the reference and this library at any
restart point:

  input.txt          r_input        v25/functions.cpp:10-87
  conf.dat           print_conf / chrg_conf   v25/functions.cpp:1181-1296
  ran_state{0,1}{I,F}.dat  Thermostat::print_ran / read_ran  v25/classes.cpp:344-367
                     (gsl_rng_fwrite of GSL's mt19937 state)
  counters.dat       save_cont / chrg_cont   v25/functions.cpp:2220-2398
  output.dat         print_out / print_final v25/functions.cpp:2830-2948
  correlation.dat    nor_correl / chrg_correl v25/functions.cpp:2472-2600
  ptens.dat, magmom.dat  print_ptens / print_magmom v25/functions.cpp:2645-2700
  pos_vel/pos_vel_N.dat  pos_vel    v25/functions.cpp:2602-2643
  compConf.dat       savec_list     v25/functions.cpp:1336-1354
  iniPos.dat         ini_pos        v25/functions.cpp:584-597
"""
from __future__ import annotations

import math
import os
import struct
from dataclasses import dataclass, field

import numpy as np


def f12(x) -> str:
    """A value as iostream prints it after setiosflags(ios::fixed) and setprecision(12)."""
    return "%.12f" % float(x)


def g6(x) -> str:
    """A double as iostream prints it by default (six significant digits)."""
    return "%g" % float(x)


# ---------------------------------------------------------------------------
# input.txt
# ---------------------------------------------------------------------------
@dataclass
class RunInput:
    """The parameters r_input reads (v25/functions.cpp:10-87), per species
    where the reference keeps them per species."""

    Nsteps: int
    pre_steps: int
    signal: int
    n_part: list
    length: list
    diameter: list
    mass: list
    B: np.ndarray
    dens: float
    temp: float
    Q: float
    gamma: float
    ArLx: float
    ArLy: float
    Dt: float
    sr_cut: float
    K_max: int
    alpha: float
    bar_w: float
    corrf: int
    tcfd: int
    tcfv: int
    cl_fr: int
    min_s: float
    iprint: int
    dip: list = field(default_factory=list)  # per species an (nd, 5) array

    @property
    def n_comp(self) -> int:
        return len(self.n_part)

    @property
    def n_total(self) -> int:
        return int(sum(self.n_part))


def read_input(path: str) -> RunInput:
    """input.txt, token by token as r_input reads it: each label is skipped
    as the number of whitespace-separated words it has in the reference's
    own files."""
    toks = open(path).read().split()
    pos = [0]

    def skip(k):
        pos[0] += k

    def take(cast=float):
        v = toks[pos[0]]
        pos[0] += 1
        return cast(v)

    def take_int():
        return int(float(take(str)))

    skip(3)
    Nsteps = take_int()
    skip(3)
    pre_steps = take_int()
    skip(1)
    signal = take_int()
    skip(3)
    nc = take_int()
    skip(3)
    n_part = [take_int() for _ in range(nc)]
    skip(1)
    length = [take() for _ in range(nc)]
    skip(1)
    diameter = [take() for _ in range(nc)]
    skip(1)
    mass = [take() for _ in range(nc)]
    skip(2)
    B = np.array([take() for _ in range(3)])
    skip(1)
    dens = take()
    skip(1)
    temp = take()
    skip(1)
    Q = take()
    skip(1)
    gamma = take()
    skip(5)
    ArLx, ArLy = take(), take()
    skip(3)
    Dt = take()
    skip(2)
    sr_cut = take()
    skip(3)
    K_max = take_int()
    skip(2)
    alpha = take()
    skip(3)
    bar_w = take()
    skip(3)
    corrf = take_int()
    skip(2)
    tcfd = take_int()
    skip(2)
    tcfv = take_int()
    skip(2)
    cl_fr = take_int()
    skip(2)
    min_s = take()
    skip(2)
    iprint = take_int()
    skip(1)
    skip(5)
    dip = []
    for _ in range(nc):
        skip(1)
        nd = take_int()
        d = np.zeros((nd, 5))
        for j in range(nd):
            d[j, 0] = take()
            skip(1)
            d[j, 1:4] = [take(), take(), take()]
            skip(1)
            d[j, 4] = take()
        dip.append(d)
    return RunInput(Nsteps, pre_steps, signal, n_part, length, diameter, mass, B, dens, temp, Q, gamma, ArLx,
                    ArLy, Dt, sr_cut, K_max, alpha, bar_w, corrf, tcfd, tcfv, cl_fr, min_s, iprint, dip)


def write_input(path: str, p: RunInput) -> None:
    """input.txt in the layout of the reference's own example (the labels
    r_input skips, with the same word counts)."""
    r = repr
    lines = [
        f"No. of steps=\t\t{p.Nsteps}",
        f"Steps before average=\t{p.pre_steps}",
        f"Signal=\t\t\t{p.signal}",
        f"No. of components=\t{p.n_comp}",
        "No. of Particles=\t" + " ".join(str(int(x)) for x in p.n_part),
        "Lengths=\t\t" + " ".join(r(float(x)) for x in p.length),
        "Diameters=\t\t" + " ".join(r(float(x)) for x in p.diameter),
        "masses=\t\t  \t" + " ".join(r(float(x)) for x in p.mass),
        "Ext Mag.Field=          " + " ".join(r(float(x)) for x in p.B),
        f"Density=\t\t{r(float(p.dens))}",
        f"Temperature=\t\t{r(float(p.temp))}",
        f"Thermostat\"mass\"=\t{r(float(p.Q))}",
        f"Thermostat\"shearRate\"=\t{r(float(p.gamma))}",
        f"Lx, Ly asp.rat. to Lz=  {r(float(p.ArLx))} {r(float(p.ArLy))}",
        f"Time step size=\t\t{r(float(p.Dt))}",
        f"Cutoff dist(SRange)=\t{r(float(p.sr_cut))}",
        f"No. of Kvectors=        {int(p.K_max)}",
        f"Convergence param(a)=   {r(float(p.alpha))}",
        f"Histogram bar width=\t{r(float(p.bar_w))}",
        f"corr. sum freq.=\t{int(p.corrf)}",
        f"DiffCorr. frequency=    {int(p.tcfd)}",
        f"ViscCorr. frequency=    {int(p.tcfv)}",
        f"clustering frequency=\t{int(p.cl_fr)}",
        f"proximity dist.=\t{r(float(p.min_s))}",
        f"Printing frequency=\t{int(p.iprint)}",
        "",
        "dipoles:(No.of.dipoles)",
        "(position ; orientation ; dip.moment)",
    ]
    for k, d in enumerate(p.dip):
        lines.append(f"species{k + 1}: {len(d)}")
        for w in np.asarray(d, dtype=np.float64).reshape(-1, 5):
            lines.append(f"{r(float(w[0]))} ; {r(float(w[1]))} {r(float(w[2]))} {r(float(w[3]))} ; {r(float(w[4]))}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


# ---------------------------------------------------------------------------
# conf.dat
# ---------------------------------------------------------------------------
def dipoles_lab(r, O, dip):
    """Lab-frame dipole positions and directions of one particle, in the
    order of operations of Spherocyl::set_dip / rotate
    (v25/classes.cpp:148-173,291-303): pos = r + offset * axis,
    dir = O^T o_body accumulated from zero."""
    out = []
    for w in np.asarray(dip, dtype=np.float64).reshape(-1, 5):
        pos = [r[a] + w[0] * O[2][a] for a in range(3)]
        ori = []
        for m in range(3):
            acc = 0.0
            acc += O[0][m] * w[1]
            acc += O[1][m] * w[2]
            acc += O[2][m] * w[3]
            ori.append(acc)
        out.append((pos, ori, w[4]))
    return out


def write_conf(path: str, box, r, p, O, l, mass, dip, clust, xi, strn, ndip=None) -> None:
    """conf.dat as print_conf writes it: the box line in iostream's default
    format, then per particle r, p, O (row-major), l, ' | ', the mass, per
    dipole its lab position, direction and moment with ' . ', and the
    cluster label, all fixed to 12 decimals; then 'xi stored-normal' of the
    two thermostats.  dip: per particle (nd, 5) body-frame rows; ndip: how
    many of them each particle has (its species' count; default all).  The
    lab dipoles are computed for all particles at once with the operations
    of dipoles_lab, in its order."""
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    n = len(r)
    p = np.asarray(p, dtype=np.float64).reshape(n, 3)
    O = np.asarray(O, dtype=np.float64).reshape(n, 3, 3)
    l = np.asarray(l, dtype=np.float64).reshape(n, 3)
    mass = np.asarray(mass, dtype=np.float64).reshape(n)
    clust = np.asarray(clust).reshape(n)
    dip = np.asarray(dip, dtype=np.float64).reshape(n, -1, 5) if n else np.zeros((0, 0, 5))
    ndip = np.full(n, dip.shape[1], dtype=np.int64) if ndip is None else np.asarray(ndip).reshape(n)
    lines = [None] * n
    for k in np.unique(ndip):
        idx = np.nonzero(ndip == k)[0]
        cols = [r[idx], p[idx], O[idx].reshape(-1, 9), l[idx], mass[idx, None]]
        for w in range(int(k)):
            d = dip[idx, w]
            pos = r[idx] + d[:, 0:1] * O[idx, 2, :]
            ori = np.zeros((len(idx), 3))
            ori = ori + O[idx, 0, :] * d[:, 1:2]
            ori = ori + O[idx, 1, :] * d[:, 2:3]
            ori = ori + O[idx, 2, :] * d[:, 3:4]
            cols += [pos, ori, d[:, 4:5]]
        vals = np.concatenate(cols, axis=1)
        fmt = " ".join(["%.12f"] * 18) + "  | %.12f " + "%.12f %.12f %.12f %.12f %.12f %.12f %.12f . " * int(k)
        for q, i in enumerate(idx):
            lines[i] = fmt % tuple(vals[q]) + str(int(clust[i])) + "\n"
    out = [f"{g6(box[0])} {g6(box[1])} {g6(box[2])}\n"] + lines
    for k in range(2):
        out.append(f"{f12(xi[k])} {f12(strn[k])}\n")
    with open(path, "w") as f:
        f.write("".join(out))


def read_conf(path: str, n_part, nd_part):
    """conf.dat as chrg_conf reads it: box, then per particle r, p, O, l,
    the mass after '|', the dipole tokens (skipped: they follow from the
    state), the cluster label; then xi and the stored normal of each
    thermostat.  n_part, nd_part: particles and dipoles per species."""
    toks = open(path).read().split()
    k = 0
    box = np.array([float(t) for t in toks[0:3]])
    k = 3
    n = int(sum(n_part))
    r, p, l = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
    O = np.zeros((n, 3, 3))
    mass = np.zeros(n)
    clust = np.zeros(n, dtype=np.int64)
    i = 0
    for ns, nd in zip(n_part, nd_part):
        for _ in range(int(ns)):
            v = [float(t) for t in toks[k:k + 18]]
            r[i], p[i] = v[0:3], v[3:6]
            O[i] = np.array(v[6:15]).reshape(3, 3)
            l[i] = v[15:18]
            mass[i] = float(toks[k + 19])
            k += 20 + 8 * int(nd)
            clust[i] = int(toks[k])
            k += 1
            i += 1
    xi = np.array([float(toks[k]), float(toks[k + 2])])
    strn = np.array([float(toks[k + 1]), float(toks[k + 3])])
    return dict(box=box, r=r, p=p, O=O, l=l, mass=mass, clust=clust, xi=xi, strn=strn)


def write_ini_pos(path: str, r, box) -> None:
    """iniPos.dat as ini_pos writes it (v25/functions.cpp:584-597): per rod
    its position, zero momentum, the identity orientation and zero angular
    momentum with a trailing 1, then the box -- iostream's default format."""
    out = []
    for v in np.asarray(r, dtype=np.float64).reshape(-1, 3):
        out.append(f"{g6(v[0])} {g6(v[1])} {g6(v[2])} 0 0 0 1 0 0 0 1 0 0 0 1  0 0 0 1\n")
    out.append(f"{g6(box[0])} {g6(box[1])} {g6(box[2])}\n")
    with open(path, "w") as f:
        f.write("".join(out))


def write_comp_conf(path: str, r) -> None:
    """compConf.dat (savec_list): the centres at the last list build."""
    with open(path, "w") as f:
        for v in np.asarray(r, dtype=np.float64).reshape(-1, 3):
            f.write(f"{f12(v[0])} {f12(v[1])} {f12(v[2])}\n")


# ---------------------------------------------------------------------------
# generator states (gsl_rng_fwrite of GSL's mt19937)
# ---------------------------------------------------------------------------
def write_mt_state(path: str, mt, mti: int) -> None:
    """GSL's mt19937 state as gsl_rng_fwrite stores it on an LP64 host: 624
    unsigned longs, the int position, padding to 8 bytes (5000 bytes; the
    padding is zero here, where the reference's file holds whatever its
    memory held)."""
    words = [int(x) & 0xffffffff for x in np.asarray(mt).reshape(-1)]
    assert len(words) == 624
    with open(path, "wb") as f:
        f.write(struct.pack("<624Qi4x", *words, int(mti)))


def read_mt_state(path: str):
    """(mt[624] as uint32, position) from a ran_state file: 5000 bytes (LP64,
    the reference's own hosts) or 2500 (32-bit unsigned long)."""
    data = open(path, "rb").read()
    if len(data) == 5000:
        v = struct.unpack("<624Qi4x", data)
    elif len(data) == 2500:
        v = struct.unpack("<624Ii", data)
    else:
        raise ValueError(f"{path}: {len(data)} bytes is not an mt19937 state")
    mt = np.array([x & 0xffffffff for x in v[:624]], dtype=np.uint32)
    return mt, int(v[624])


# ---------------------------------------------------------------------------
# accumulators and counters.dat
# ---------------------------------------------------------------------------
SCALARS = ("K", "U", "P", "Uss", "Pss", "UdipR", "PdipR", "UdipK", "PdipK", "Uext")
TENSORS = ("PT", "PTss", "PTdipR", "PTdipK", "PTkin")


class Accumulator:
    """The reference's accumulator (v25/classes.hpp:185-290,
    v25/classes.cpp:369-500): the per-step thermodynamic values and their
    running sums.  += keeps the reference's behaviour of ASSIGNING Uext
    (v25/classes.cpp:436), so counters.dat and the averages it prints carry
    the same numbers."""

    def __init__(self):
        for k in SCALARS:
            setattr(self, k, 0.0)
        for k in TENSORS:
            setattr(self, k, np.zeros((3, 3)))
        self.G1 = 0.0
        self.G2 = 0.0

    def __iadd__(self, o: "Accumulator"):
        for k in SCALARS:
            if k == "Uext":
                self.Uext = o.Uext
            else:
                setattr(self, k, getattr(self, k) + getattr(o, k))
        for k in TENSORS:
            setattr(self, k, getattr(self, k) + getattr(o, k))
        self.G1 += o.G1
        self.G2 += o.G2
        return self

    def __mul__(self, o: "Accumulator") -> "Accumulator":
        r = Accumulator()
        for k in SCALARS:
            setattr(r, k, getattr(self, k) * getattr(o, k))
        for k in TENSORS:
            setattr(r, k, getattr(self, k) * getattr(o, k))
        r.G1 = self.G1 * o.G1
        r.G2 = self.G2 * o.G2
        return r


def write_counters(path: str, Time: float, cont: int, Ntcf: int, Ntcv: int, mcont: int, AcT: Accumulator,
                   AcTsq: Accumulator, npc=None) -> None:
    """counters.dat (save_cont): the run's clock and counters, then each
    accumulated value next to its accumulated square, the tensors row by
    row, all fixed to 12 decimals.  npc: the later driver's two
    polymerisation counters (clusterings, particles in clusters of two or
    more; v25/v251/functions.cpp:2294), written last."""
    v = [f12(Time), str(int(cont)), str(int(Ntcf)), str(int(Ntcv)), str(int(mcont))]
    for k in SCALARS:
        v += [f12(getattr(AcT, k)), f12(getattr(AcTsq, k))]
    for k in TENSORS:
        v += [f12(x) for x in getattr(AcT, k).ravel()]
        v += [f12(x) for x in getattr(AcTsq, k).ravel()]
    v += [f12(AcT.G1), f12(AcTsq.G1), f12(AcT.G2), f12(AcTsq.G2)]
    if npc is not None:
        v += [str(int(npc[0])), str(int(npc[1]))]
    with open(path, "w") as f:
        f.write(" ".join(v) + " \n")


def read_counters(path: str, npc: bool = False):
    """counters.dat (chrg_cont): (Time, cont, Ntcf, Ntcv, mcont, AcT, AcTsq),
    and the two polymerisation counters last when npc (the later driver)."""
    t = open(path).read().split()
    extra = None
    if npc:
        extra = [int(t[-2]), int(t[-1])]
        t = t[:-2]
    Time, cont, Ntcf, Ntcv, mcont = float(t[0]), int(t[1]), int(t[2]), int(t[3]), int(t[4])
    vals = [float(x) for x in t[5:]]
    AcT, AcTsq = Accumulator(), Accumulator()
    k = 0
    for name in SCALARS:
        setattr(AcT, name, vals[k])
        setattr(AcTsq, name, vals[k + 1])
        k += 2
    for name in TENSORS:
        setattr(AcT, name, np.array(vals[k:k + 9]).reshape(3, 3))
        setattr(AcTsq, name, np.array(vals[k + 9:k + 18]).reshape(3, 3))
        k += 18
    AcT.G1, AcTsq.G1, AcT.G2, AcTsq.G2 = vals[k:k + 4]
    if npc:
        return Time, cont, Ntcf, Ntcv, mcont, AcT, AcTsq, extra
    return Time, cont, Ntcf, Ntcv, mcont, AcT, AcTsq


# ---------------------------------------------------------------------------
# output.dat and the other per-step files
# ---------------------------------------------------------------------------
def output_line(Time: float, t_elap: float, t_cpu: float, var: Accumulator, Mom) -> str:
    """One output.dat line (print_out): 'Time. wall cpu | K U P Uss Pss
    UdipR PdipR UdipK PdipK |P|^2 |L|^2', fixed to 12 decimals."""
    vals = [var.K, var.U, var.P, var.Uss, var.Pss, var.UdipR, var.PdipR, var.UdipK, var.PdipK,
            Mom[0] * Mom[0] + Mom[1] * Mom[1] + Mom[2] * Mom[2], Mom[3] * Mom[3] + Mom[4] * Mom[4] + Mom[5] * Mom[5]]
    return f"{f12(Time)}. {f12(t_elap)} {f12(t_cpu)} | " + " ".join(f12(v) for v in vals) + "\n"


def ptens_line(time: float, HF, PT) -> str:
    """ptens.dat (print_ptens): the time in the default format, then the
    Helfand moment sum r_i p_j and the pressure tensor, fixed 12."""
    return g6(time) + " " + "".join(f12(x) + " " for x in np.asarray(HF).ravel()) + \
        "".join(f12(x) + " " for x in np.asarray(PT).ravel()) + "\n"


def magmom_line(time: float, M) -> str:
    """magmom.dat (print_magmom): the time, then M fixed 12."""
    return g6(time) + " " + "".join(f12(x) + " " for x in M) + "\n"


def write_pos_vel(path: str, blocks, Dt: float) -> None:
    """pos_vel_N.dat (pos_vel): per listed particle 'r v | u omega', then the
    sampling interval.  blocks: rows (r[3], v[3], u[3], omega[3])."""
    with open(path, "w") as f:
        for r, v, u, w in blocks:
            f.write(" ".join(f12(x) for x in r) + " " + " ".join(f12(x) for x in v) + " | ")
            f.write(" ".join(f12(x) for x in u) + " " + " ".join(f12(x) for x in w) + "\n")
        f.write(f12(Dt) + "\n")


def write_correlation(path: str, hist, counts, Lmin: float, bar_w: float, cor_cont: float) -> None:
    """correlation.dat (nor_correl): per bin 'cor_cont norm pos & ', then the
    four normalised functions of each species ('| ' after each) and of each
    species pair.  The stream's fixed flag, once set, stays: cor_cont is in
    the default format on the first line and fixed to 8 decimals after."""
    from .lib import normalize_correlations

    counts = list(counts)
    nc = len(counts)
    h = np.asarray(hist, dtype=np.float64).reshape(nc + nc * (nc - 1) // 2, 4, -1)
    box = (Lmin, Lmin, Lmin)
    pos, norm, g = normalize_correlations(h, counts, box, bar_w, cor_cont)
    out = []
    for b in range(h.shape[2]):
        cc = g6(cor_cont) if b == 0 else "%.8f" % cor_cont
        line = f"{cc} {'%.8f' % norm[b]} {'%.4f' % pos[b]} & "
        for k in range(nc):
            if counts[k] > 1:
                line += "".join("%.8f " % g[k, f, b] for f in range(4))
            else:
                line += "0 "
            line += "| "
        for q in range(nc, h.shape[0]):
            line += "".join("%.8f " % g[q, f, b] for f in range(4))
            line += "| "
        out.append(line + "\n")
    with open(path, "w") as f:
        f.write("".join(out))


def read_correlation(path: str, counts, nbins: int):
    """correlation.dat (chrg_correl): (cor_cont, hist) with the histograms
    rebuilt from the normalised values as the reference rebuilds them."""
    counts = list(counts)
    nc = len(counts)
    nblk = nc + nc * (nc - 1) // 2
    hist = np.zeros((nblk, 4, nbins))
    t = open(path).read().split()
    k = 0
    cor_cont = 0.0
    div = (1.0, 3.0, 1.5, 5.0)
    for b in range(nbins):
        cor_cont, norm, _pos = float(t[k]), float(t[k + 1]), float(t[k + 2])
        k += 4
        nnorm = norm * cor_cont
        for s in range(nc):
            nn = counts[s]
            for f in range(4):
                hist[s, f, b] = float(t[k]) * nnorm * nn * (nn - 1) / div[f]
                k += 1
            k += 1
        q = nc
        for m in range(nc - 1):
            for n in range(m + 1, nc):
                for f in range(4):
                    hist[q, f, b] = float(t[k]) * nnorm * counts[n] * counts[m] / div[f]
                    k += 1
                k += 1
                q += 1
    return cor_cont, hist


def final_report(Time, AcT: Accumulator, AcTsq: Accumulator, cont: int, p: RunInput, box, pol_deg=None) -> str:
    """The closing block print_final appends to output.dat: run parameters,
    then each average with its fluctuation sqrt(<x^2> - <x>^2), in
    iostream's default format; the later driver adds the degree of
    polymerisation (v25/v251/functions.cpp:2876)."""
    def av(x, xsq):
        a = x / cont
        return a, math.sqrt(xsq / cont - a * a) if xsq / cont - a * a >= 0 else float("nan")

    o = []
    V = box[0] * box[1] * box[2]
    o.append("NVT ensemble\n")
    o.append(f"Temperature: {g6(p.temp)}\n")
    o.append(f"Density: {g6(p.n_total / V)}\n")
    o.append(f"Volume (Lx,Ly,Lz): {g6(box[0])} x {g6(box[1])} x {g6(box[2])} = {g6(V)}\n")
    o.append(f"Elapsed time: {g6(Time)}\n")
    o.append("Component | No. of particles | mass | L | D | Vol. frac.\n")
    for n in range(p.n_comp):
        rad = p.diameter[n] / 2
        NN = p.n_part[n]
        vf = NN * math.pi * (4. * rad / 3 + p.length[n]) * rad * rad / V
        o.append(f"{n} | {NN} | {g6(p.mass[n])} | {g6(p.length[n])} | {g6(p.diameter[n])} | {g6(vf)}\n")
    o.append("Dipoles: (position ; orientation ; dip.moment)\n")
    for n in range(p.n_comp):
        o.append(f"species {n}\n")
        for w in np.asarray(p.dip[n]).reshape(-1, 5):
            o.append(f"{g6(w[0])} ; {g6(w[1])} {g6(w[2])} {g6(w[3])} ; {g6(w[4])}\n")
    o.append(f"External field: ({g6(p.B[0])},{g6(p.B[1])},{g6(p.B[2])})\n")
    o.append(f"Thermostat mass: {g6(p.Q)} Thermostat shear rate: {g6(p.gamma)}\n")
    o.append("------------------\n")
    s = {k: av(getattr(AcT, k), getattr(AcTsq, k)) for k in SCALARS}
    pm = lambda k: f"{g6(s[k][0])}+/-{g6(s[k][1])}"  # noqa: E731
    o.append(f"Av. kinetic energy: {pm('K')}\n")
    o.append(f"Av. potential energy: {pm('U')}\n")
    o.append(f"Av. soft sphere en.: {pm('Uss')} Av. dipolarR en.: {pm('UdipR')} Av. dipolarK en.: {pm('UdipK')}\n")
    o.append(f"Av. Ext.Field en.: {pm('Uext')}\n")
    o.append(f"Av. pressure: {pm('P')}\n")
    o.append(f"Av. soft sphere pres.: {pm('Pss')} Av. dipolarR pres.: {pm('PdipR')} "
             f"Av. dipolarK pres.: {pm('PdipK')}\n")
    for title, k in (("Av. Pressure tensor: ", "PT"), ("kinetic part: ", "PTkin"), ("soft core part: ", "PTss"),
                     ("real dip part: ", "PTdipR"), ("reciprocal dip part: ", "PTdipK")):
        o.append(title + "\n")
        a, q = getattr(AcT, k), getattr(AcTsq, k)
        for i in range(3):
            cells = []
            for j in range(3):
                m, fl = av(a[i][j], q[i][j])
                cells.append(f"{g6(m)}+/-{g6(fl)}")
            o.append("| " + " ".join(cells) + " |\n")
    g1, fg1 = av(AcT.G1, AcTsq.G1)
    g2, fg2 = av(AcT.G2, AcTsq.G2)
    o.append("Average G1(P) parameter:\n")
    o.append(f"{g6(g1)} +/- {g6(fg1)}\n")
    o.append("Average G2(S) mayer-saupe parameter:\n")
    o.append(f"{g6(g2)} +/- {g6(fg2)}\n")
    if pol_deg is not None:
        o.append(f"Polymerization degree: {g6(pol_deg)}\n")
    return "".join(o)


def append(path: str, text: str) -> None:
    with open(path, "a") as f:
        f.write(text)


def ensure_dir(path: str) -> None:
    os.makedirs(path, exist_ok=True)
