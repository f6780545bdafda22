"""Seeded synthetic systems of polydisperse dipolar spherocylinders.

The reference starts from a lattice plus 1000 cluster pivots
(v25/functions.cpp:491-1156, v25/main.cpp:215-239); the workloads here are
instead the seeded random constructions the benchmark configurations name:
random non-overlapping placement by rejection on the segment distance,
orientations uniform on the sphere, Maxwell-Boltzmann momenta and angular
momenta at temperature T with the total momentum removed (the reference
refuses to start otherwise, v25/main.cpp:356-373).

Conventions, as in the reference:
* orientation O: rows are the body axes in the lab frame, row 2 is the rod
  axis (v25/classes.hpp:74, v25/classes.cpp:123-124);
* dipoles per particle: (offset along the axis, body-frame direction, moment)
  (v25/classes.cpp:148-173); all workloads use one axial centred dipole;
* inertia from the particle's shape and mass (v25/classes.cpp:175-185);
* masses are 1 (the benchmark configurations do not give masses).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SPHERO_VOL = lambda L, D: math.pi * D * D * L / 4.0 + math.pi * D ** 3 / 6.0  # noqa: E731


def inertia(L, D, m):
    """Principal moments of a uniform spherocylinder, as Spherocyl::set_inertia
    (v25/classes.cpp:175-185) computes them."""
    L = np.asarray(L, dtype=np.float64)
    D = np.asarray(D, dtype=np.float64)
    m = np.asarray(m, dtype=np.float64)
    R = D / 2
    Rsq = R * R
    Rft = Rsq * Rsq
    Lsq = L * L
    vol = math.pi * Rsq * (L + 3.0 * R / 4)
    mdens = m / vol
    I0 = mdens * math.pi * (Lsq * L * Rsq / 12 + Lsq * Rsq * R / 3 + L * Rft / 4 + 8.0 * Rft * R / 15)
    I2 = mdens * math.pi * (L * Rft / 2 + 8.0 * Rft * R / 15)
    return np.stack([I0, I0, I2], axis=-1)


def segment_distance_sq(p1, d1, p2, d2):
    """Squared distance between segments p1 + s d1 and p2 + t d2, s, t in
    [0, 1], vectorised over the second argument.  Closest points of two
    segments as in Ericson, Real-Time Collision Detection, sec. 5.1.9; used
    only to reject overlapping placements."""
    r = p1 - p2
    a = float(d1 @ d1)
    e = np.einsum("ij,ij->i", d2, d2)
    f = np.einsum("ij,ij->i", d2, r)
    c = r @ d1
    b = d2 @ d1
    denom = a * e - b * b
    s = np.where(denom > 1e-12, np.clip((b * f - c * e) / np.where(denom > 1e-12, denom, 1.0), 0.0, 1.0), 0.0)
    t = (b * s + f) / e
    t_lo = t < 0
    t_hi = t > 1
    s = np.where(t_lo, np.clip(-c / a, 0.0, 1.0), s)
    s = np.where(t_hi, np.clip((b - c) / a, 0.0, 1.0), s)
    t = np.clip(t, 0.0, 1.0)
    c1 = p1 + s[:, None] * d1
    c2 = p2 + t[:, None] * d2
    dd = c1 - c2
    return np.einsum("ij,ij->i", dd, dd)


def random_rotations(rng, n):
    """n orientation matrices whose row 2 (the rod axis) is uniform on S^2."""
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    a = rng.normal(size=(n, 3))
    a -= (a * u).sum(1, keepdims=True) * u
    a /= np.linalg.norm(a, axis=1, keepdims=True)
    b = np.cross(u, a)
    return np.stack([a, b, u], axis=1)  # rows: body x, body y, body z (= axis)


def place_rods(rng, lengths, dia, box, min_gap=0.0, max_tries=200000):
    """Random non-overlapping placement (segment distance >= (D_i+D_j)/2 + gap)
    by sequential rejection with a cell grid.  Returns positions and
    orientation matrices."""
    n = len(lengths)
    box = np.asarray(box, dtype=np.float64)
    reach = float(lengths.max() + dia.max() + min_gap)
    ncell = np.maximum(1, np.floor(box / reach).astype(int))
    cell = box / ncell
    grid: dict[tuple, list] = {}
    pos = np.zeros((n, 3))
    O = np.zeros((n, 3, 3))
    tries = 0
    for i in range(n):
        while True:
            tries += 1
            if tries > max_tries + 50 * n:
                raise RuntimeError("placement failed: packing fraction too high for rejection")
            r = rng.uniform(0, 1, 3) * box
            o = random_rotations(rng, 1)[0]
            c = tuple((np.floor(r / cell).astype(int)) % ncell)
            cand = []
            rng3 = [range(-1, 2) if ncell[a] >= 3 else range(ncell[a]) for a in range(3)]
            seen = set()
            for dx in rng3[0]:
                for dy in rng3[1]:
                    for dz in rng3[2]:
                        if ncell[0] >= 3:
                            kx = (c[0] + dx) % ncell[0]
                        else:
                            kx = dx
                        ky = (c[1] + dy) % ncell[1] if ncell[1] >= 3 else dy
                        kz = (c[2] + dz) % ncell[2] if ncell[2] >= 3 else dz
                        key = (kx, ky, kz)
                        if key in seen:
                            continue
                        seen.add(key)
                        cand.extend(grid.get(key, ()))
            ok = True
            if cand:
                j = np.asarray(cand)
                rij = r - pos[j]
                rij -= box * np.floor(rij / box + 0.5)
                # segment i from -L/2 to L/2 around 0; segments j around -rij
                di = lengths[i] * o[2]
                dj = lengths[j, None] * O[j, 2]
                p1 = -0.5 * di
                p2 = -rij - 0.5 * dj
                d2 = segment_distance_sq(p1, di, p2, dj)
                lim = (0.5 * (dia[i] + dia[j]) + min_gap) ** 2
                ok = bool(np.all(d2 >= lim))
            if ok:
                pos[i] = r
                O[i] = o
                grid.setdefault(c, []).append(i)
                break
    return pos, O


@dataclass
class SystemSpec:
    """Everything one MD system needs besides its particle state."""

    n: int
    box: np.ndarray
    alpha: float
    K_max: int
    ksq_max: int
    temp: float = 1.0
    Q: float = 1.0
    gamma: float = 0.0
    dt: float = 1e-3
    B: np.ndarray = field(default_factory=lambda: np.zeros(3))
    sr_cut: float = 0.0
    xi0: float = 0.0
    min_s: float = 0.1
    cl_fr: int = 0
    steps: int = 1000
    label: str = ""
    rc_real: float = 0.0  # real-space cutoff: 0 = all minimum-image pairs (the reference)
    cl_energy: float = 0.0  # cluster bonds by pair energy below -cl_energy kT; 0 = the reference's test


@dataclass
class SystemState:
    """Particle state (SoA, FP64)."""

    r: np.ndarray
    p: np.ndarray
    O: np.ndarray
    l: np.ndarray
    length: np.ndarray
    dia: np.ndarray
    mass: np.ndarray
    dip: np.ndarray  # (n, nd, 5)

    @property
    def n(self) -> int:
        return len(self.length)

    def copy(self) -> "SystemState":
        return SystemState(*(np.array(getattr(self, k), copy=True) for k in
                             ("r", "p", "O", "l", "length", "dia", "mass", "dip")))


def maxwell_boltzmann(rng, mass, I, O, temp):
    n = len(mass)
    p = rng.normal(size=(n, 3)) * np.sqrt(mass * temp)[:, None]
    p -= p.mean(axis=0, keepdims=True)
    lb = rng.normal(size=(n, 3)) * np.sqrt(I * temp)
    l = np.einsum("nab,na->nb", O, lb)  # lab = O^T l_body
    return p, l


def make_system(*, n, phi, lengths, mu, temp=1.0, seed=0, dia=None, mass=None,
                min_gap=0.0, aspect=(1.0, 1.0)):
    """Seeded random system: n rods with the given lengths (array) and dipole
    moments (array, axial centred), packing fraction phi, temperature temp."""
    rng = np.random.default_rng(seed)
    lengths = np.asarray(lengths, dtype=np.float64)
    dia = np.ones(n) if dia is None else np.asarray(dia, dtype=np.float64)
    mass = np.ones(n) if mass is None else np.asarray(mass, dtype=np.float64)
    vol = np.pi * dia ** 2 * lengths / 4 + np.pi * dia ** 3 / 6
    V = vol.sum() / phi
    Lz = (V / (aspect[0] * aspect[1])) ** (1.0 / 3.0)
    box = np.array([aspect[0] * Lz, aspect[1] * Lz, Lz])
    from .lib import place_rods as _place

    r, O = _place(lengths, dia, box, seed=int(rng.integers(1 << 62)), gap=min_gap)
    I = inertia(lengths, dia, mass)
    p, l = maxwell_boltzmann(rng, mass, I, O, temp)
    dip = np.zeros((n, 1, 5))
    dip[:, 0, 3] = 1.0
    dip[:, 0, 4] = np.asarray(mu, dtype=np.float64)
    return SystemState(r, p, O, l, lengths, dia, mass, dip), box


# ---------------------------------------------------------------------------
# The benchmark workloads (seeded synthetic stand-ins for the configurations)
# ---------------------------------------------------------------------------

def _kmax_for(ksq):
    return int(math.isqrt(ksq)) + 1


def plain_c0(seed=0, n=256):
    """N=256, phi=0.10, L ~ N(3, 0.3) clipped to [2, 4], mu^2 = 2 axial,
    alpha = 5.6/L_box, |n|^2 <= 27, Q = 1, dt = 1e-3, 1000 steps."""
    rng = np.random.default_rng(10_000 + seed)
    lengths = np.clip(rng.normal(3.0, 0.3, n), 2.0, 4.0)
    st, box = make_system(n=n, phi=0.10, lengths=lengths, mu=np.full(n, math.sqrt(2.0)), seed=seed)
    spec = SystemSpec(n=n, box=box, alpha=5.6 / box[0], K_max=_kmax_for(27), ksq_max=27,
                      steps=1000, label="plain_n256_phi0.10")
    return spec, st


def plain_c1(seed=1, n=4096):
    """N=4096, phi=0.20, L ~ U[2, 5], mu proportional to volume with
    <mu^2> = 3, alpha = 7/L_box, |n|^2 <= 64, 5000 steps."""
    rng = np.random.default_rng(20_000 + seed)
    lengths = rng.uniform(2.0, 5.0, n)
    vol = np.pi * lengths / 4 + np.pi / 6
    mu = vol * math.sqrt(3.0 / np.mean(vol ** 2))
    st, box = make_system(n=n, phi=0.20, lengths=lengths, mu=mu, seed=seed)
    spec = SystemSpec(n=n, box=box, alpha=7.0 / box[0], K_max=_kmax_for(64), ksq_max=64,
                      steps=5000, label="plain_n4096_phi0.20")
    return spec, st


def plain_c2(seed=2, n=32768):
    """N=32768, phi=0.15, mu^2 = 5, field along z with mu B / kT = 2,
    L ~ N(3, 0.5), |n|^2 <= 100, alpha = 6/L_box (not given; chosen),
    clusters every 100 steps, 20000 steps."""
    rng = np.random.default_rng(30_000 + seed)
    lengths = np.clip(rng.normal(3.0, 0.5, n), 1.0, None)
    mu = math.sqrt(5.0)
    st, box = make_system(n=n, phi=0.15, lengths=lengths, mu=np.full(n, mu), seed=seed)
    spec = SystemSpec(n=n, box=box, alpha=6.0 / box[0], K_max=_kmax_for(100), ksq_max=100,
                      B=np.array([0.0, 0.0, 2.0 / mu]), cl_fr=100, steps=20000,
                      label="plain_n32768_phi0.15")
    return spec, st


def replica_mix_specs(n_systems=256, seed=3, n_lo=128, n_hi=2048):
    """Draw the 256-replica mix parameters: N log-uniform in [128, 2048],
    phi U[0.05, 0.25], mu^2 U[0.5, 4], T U[0.8, 1.5], L U[2, 4],
    alpha = 6/L_box, |n|^2 <= 36, 2000 steps."""
    rng = np.random.default_rng(40_000 + seed)
    out = []
    for k in range(n_systems):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        out.append(dict(n=n, phi=float(rng.uniform(0.05, 0.25)), mu2=float(rng.uniform(0.5, 4.0)),
                        T=float(rng.uniform(0.8, 1.5)), seed=int(rng.integers(1 << 30))))
    return out


def replica_system(d, ksq=36, steps=2000):
    rng = np.random.default_rng(d["seed"])
    n = d["n"]
    lengths = rng.uniform(2.0, 4.0, n)
    st, box = make_system(n=n, phi=d["phi"], lengths=lengths, mu=np.full(n, math.sqrt(d["mu2"])),
                          temp=d["T"], seed=d["seed"] + 1)
    spec = SystemSpec(n=n, box=box, alpha=6.0 / box[0], K_max=_kmax_for(ksq), ksq_max=ksq,
                      temp=d["T"], steps=steps, label=f"replica_n{n}")
    return spec, st


def serving_job(seed, ksq=36):
    """One serving job: N log-uniform [64, 8192], steps U[500, 5000],
    phi U[.05, .25], mu^2 U[.5, 5], T U[.8, 1.5], L ~ N(3, 0.3)."""
    rng = np.random.default_rng(50_000 + seed)
    n = int(round(math.exp(rng.uniform(math.log(64), math.log(8192)))))
    steps = int(rng.integers(500, 5001))
    phi = float(rng.uniform(0.05, 0.25))
    mu2 = float(rng.uniform(0.5, 5.0))
    T = float(rng.uniform(0.8, 1.5))
    lengths = np.clip(rng.normal(3.0, 0.3, n), 1.5, 4.5)
    st, box = make_system(n=n, phi=phi, lengths=lengths, mu=np.full(n, math.sqrt(mu2)), temp=T,
                          seed=seed + 7)
    spec = SystemSpec(n=n, box=box, alpha=6.0 / box[0], K_max=_kmax_for(ksq), ksq_max=ksq, temp=T,
                      steps=steps, label=f"job{seed}_n{n}")
    return spec, st
