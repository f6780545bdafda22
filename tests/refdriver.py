"""Runs the reference's own driver (oracle/_ref/DSCmd_v25, built from the
reference's unmodified sources) from a state we write, as a restart
(signal = 1): input.txt, conf.dat and the thermostats' generator states are
written in the reference's formats (v25/functions.cpp:10-87,1181-1296,
v25/classes.cpp:344-367), the driver runs, and its output.dat and final
conf.dat are parsed back.  Test infrastructure."""
from __future__ import annotations

import os
import struct
import subprocess

import numpy as np

INPUT = """No. of steps=\t\t{steps}
Steps before average=\t0
Signal=\t\t\t1
No. of components=\t1
No. of Particles=\t{n}
Lengths=\t\t{L}
Diameters=\t\t{D}
masses=\t\t  \t{m}
Ext Mag.Field=          {B0} {B1} {B2}
Density=\t\t{dens}
Temperature=\t\t{T}
Thermostat"mass"=\t{Q}
Thermostat"shearRate"=\t{gamma}
Lx, Ly asp.rat. to Lz=  1 1
Time step size=\t\t{dt}
Cutoff dist(SRange)=\t{sr_cut}
No. of Kvectors=        {K}
Convergence param(a)=   {alpha}
Histogram bar width=\t0.05
corr. sum freq.=\t{big}
DiffCorr. frequency=    {big}
ViscCorr. frequency=    {big}
clustering frequency=\t{cl_fr}
proximity dist.=\t{min_s}
Printing frequency=\t1

dipoles:(No.of.dipoles)
(position ; orientation ; dip.moment)
species1: {nd}
{dips}species2: 0
species3: 0
species4: 0
species5: 0
"""


def mt_state_bytes(seed: int) -> bytes:
    """A freshly seeded MT19937 state in the layout the reference's
    generator files use (624 unsigned longs, an int, padding)."""
    s = seed & 0xffffffff or 4357
    mt = [s]
    for i in range(1, 624):
        mt.append((1812433253 * (mt[-1] ^ (mt[-1] >> 30)) + i) & 0xffffffff)
    return struct.pack("<624Qi4x", *mt, 624)


def write_run(d, *, r, p, O, l, L, D, m, dip, box, xi, strn, steps, T, Q, gamma, dt, sr_cut, K, alpha, B,
              cl_fr, min_s):
    n = len(r)
    f_ = lambda v: repr(float(v))  # noqa: E731  (plain digits, never numpy's repr)
    dips = "".join(f"{f_(w[0])} ; {f_(w[1])} {f_(w[2])} {f_(w[3])} ; {f_(w[4])}\n" for w in dip)
    with open(os.path.join(d, "input.txt"), "w") as f:
        f.write(INPUT.format(steps=steps, n=n, L=f_(L), D=f_(D), m=f_(m), B0=f_(B[0]), B1=f_(B[1]), B2=f_(B[2]),
                             dens=f_(n / np.prod(box)), T=f_(T), Q=f_(Q), gamma=f_(gamma), dt=f_(dt),
                             sr_cut=f_(sr_cut), K=int(K), alpha=f_(alpha), big=10 ** 8, cl_fr=int(cl_fr),
                             min_s=f_(min_s), nd=len(dip), dips=dips))
    with open(os.path.join(d, "conf.dat"), "w") as f:
        f.write(f"{f_(box[0])} {f_(box[1])} {f_(box[2])}\n")
        for i in range(n):
            vals = list(r[i]) + list(p[i]) + list(O[i].ravel()) + list(l[i])
            f.write(" ".join(repr(float(v)) for v in vals))
            f.write(f"  | {f_(m)} ")
            f.write("0 0 0 0 0 0 0 . " * len(dip))
            f.write("0\n")
        for k in range(2):
            f.write(f"{f_(xi[k])} {f_(strn[k])}\n")
    for k, seed in enumerate((1, 2)):
        with open(os.path.join(d, f"ran_state{k}F.dat"), "wb") as f:
            f.write(mt_state_bytes(seed))


def run(d, binary, timeout=600):
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.run([binary], cwd=d, env=env, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL,
                   timeout=timeout, check=False)


def read_output(d):
    """Per-step rows of output.dat: K U P Uss Pss UdipR PdipR UdipK PdipK |P|^2 |L|^2."""
    rows = []
    with open(os.path.join(d, "output.dat")) as f:
        for line in f:
            if "|" not in line or not line[:1].isdigit() or not line.split()[0].endswith("."):
                continue
            v = line.split("|")[1].split()
            if len(v) == 11:
                rows.append([float(x) for x in v])
    return np.array(rows)


def read_conf(d, n, nd):
    toks = open(os.path.join(d, "conf.dat")).read().split()
    box = np.array([float(t) for t in toks[:3]])
    k = 3
    out = dict(r=np.zeros((n, 3)), p=np.zeros((n, 3)), O=np.zeros((n, 3, 3)), l=np.zeros((n, 3)),
               clust=np.zeros(n, np.int64))
    for i in range(n):
        v = [float(t) for t in toks[k:k + 18]]
        out["r"][i], out["p"][i] = v[0:3], v[3:6]
        out["O"][i] = np.array(v[6:15]).reshape(3, 3)
        out["l"][i] = v[15:18]
        k += 18 + 2 + 8 * nd
        out["clust"][i] = int(toks[k])
        k += 1
    out["xi"] = np.array([float(toks[k]), float(toks[k + 2])])
    out["box"] = box
    return out
