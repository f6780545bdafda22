"""mdSpherocyl's run loop (v25/main.cpp) on the GB300 library.

    python -m mdspherocyl_gb300.driver [workdir] [--device N] [--variant v25|v251]

Reads input.txt in workdir and runs it as the reference's executable does:
the same restart modes, the same per-step bookkeeping and the same files,
written in the reference's formats (mdspherocyl_gb300/files.py), with every
step taken on the GPU by mdsc_step_trace.

  signal 1  restart from conf.dat and the thermostats' generator states
            (ran_state0F.dat, ran_state1F.dat); averages start afresh
  signal 2  the same, continuing counters.dat and correlation.dat
  signal 0  a new configuration: the reference's lattice on the GPU
            (mdsc_lattice, ini_pos of v25/functions.cpp:491-675, written to
            iniPos.dat as the reference writes it) with Maxwell-Boltzmann
            momenta of zero sum (mdsc_thermalize).  The reference then
            shuffles the lattice with 1000 cluster moves (GCAmix,
            :3328-3409) and draws its momenta with ini_mom from its run
            generator; neither is restated, so a signal-0 run starts from
            the reference's lattice with other momenta.

Per step (v25/main.cpp:520-818): the thermodynamic values of the step
(energies per particle, pressures, pressure tensors), then past the
equilibration steps the correlation histograms every corrf steps, the order
parameters, the pos_vel dumps every tcfd steps, ptens.dat and magmom.dat
every tcfv steps and the running sums; every iprint steps conf.dat, the
generator states, counters.dat, correlation.dat and a line of output.dat;
at the end the averages block of output.dat and time.dat (the reference's
per-function lines, from the GPU kernels' times).  The reference's
neighbour-list bookkeeping file compConf.dat is written once, at the start:
this library keeps its own list state on the GPU.

--variant v251 runs the reference's later driver (v25/v251/main.cpp): the
thermostats start at xi = 1 (v25/v251/classes.hpp:154), each clustering adds
to the degree-of-polymerisation counters (clusterings; particles in clusters
of two or more, v25/v251/functions.cpp:3249-3256), which counters.dat
carries and the closing report divides.
"""
from __future__ import annotations

import argparse
import math
import os
import sys
import time

import numpy as np

from . import files as F
from . import lib as L
from .systems import SystemSpec, SystemState, inertia

MX_TCF = 25  # particles per species in the time-correlation dumps (v25/main.cpp:29)
OVERLAP = 4  # MDSC_ERR_OVERLAP


class RunError(RuntimeError):
    """A condition on which the reference writes Error.dat and stops."""


def layout(p: F.RunInput):
    """Per-particle shapes and dipole tables from the per-species input:
    species in order, each a contiguous block (calc_II numbering).  Species
    with fewer dipoles than the most are padded with zero moments, which add
    nothing to any sum."""
    nd = max([len(d) for d in p.dip] + [0])
    n = p.n_total
    length, dia, mass = np.zeros(n), np.zeros(n), np.zeros(n)
    dip = np.zeros((n, max(nd, 1), 5))
    dip[:, :, 3] = 1.0
    nd_part = []
    i = 0
    for s in range(p.n_comp):
        k = int(p.n_part[s])
        length[i:i + k], dia[i:i + k], mass[i:i + k] = p.length[s], p.diameter[s], p.mass[s]
        d = np.asarray(p.dip[s], dtype=np.float64).reshape(-1, 5)
        dip[i:i + k, :len(d)] = d
        nd_part.append(len(d))
        i += k
    return length, dia, mass, dip[:, :max(nd, 1)] if nd > 0 else dip[:, :0], nd, nd_part


def check_input(p: F.RunInput) -> None:
    """The reference's checks before it starts (v25/main.cpp:97-118)."""
    for n in range(p.n_comp):
        if p.n_part[n] < 1:
            raise RunError("No. of particles per species must be >= 1")
    for n in range(p.n_comp):
        for i, w in enumerate(np.asarray(p.dip[n]).reshape(-1, 5)):
            if abs(w[0]) >= (p.length[n] + p.diameter[n]) / 2 - 0.01:
                raise RunError(f"dipole {i} of species {n} is ouside the core!")


def new_box(p: F.RunInput):
    """Signal 0: the box from the density and aspect ratios (v25/main.cpp:216-219)."""
    Lz = (p.n_total / (p.ArLx * p.ArLy * p.dens)) ** (1.0 / 3)
    return np.array([p.ArLx * Lz, p.ArLy * Lz, Lz])


class Driver:
    def __init__(self, workdir: str = ".", device: int = 0, out=sys.stdout, variant: str = "v25",
                 rc_real: float = 0.0, ksq_max: int = 0, cl_energy: float = 0.0):
        """rc_real, ksq_max and cl_energy are this library's knobs, not
        input.txt's (which keeps the reference's layout): a real-space
        cutoff, a spherical k-set |n|^2 <= ksq_max, clusters by pair energy
        below -cl_energy kT.  Their defaults are the reference's behaviour."""
        if variant not in ("v25", "v251"):
            raise ValueError(f"unknown driver variant {variant}")
        self.d = workdir
        self.device = device
        self.out = out
        self.v251 = variant == "v251"
        self.rc_real, self.ksq_max, self.cl_energy = float(rc_real), int(ksq_max), float(cl_energy)
        self._cor_s = 0.0  # host seconds in the correlation calls

    def path(self, name: str) -> str:
        return os.path.join(self.d, name)

    def error(self, msg: str) -> None:
        F.append(self.path("Error.dat"), msg + "\n")

    # ------------------------------------------------------------------
    def run(self) -> int:
        open(self.path("Error.dat"), "w").close()
        try:
            return self._run()
        except RunError as e:
            self.error(str(e))
            return 1

    def _run(self) -> int:
        p = F.read_input(self.path("input.txt"))
        check_input(p)
        n = p.n_total
        length, dia, mass, dip, nd, nd_part = layout(p)
        dmax = max(p.length[k] + p.diameter[k] for k in range(p.n_comp))
        dmin = min(p.diameter)
        Time, cont, Ntcf, Ntcv, mcont = 0.0, 0, 0, 0, 0
        AcT, AcTsq = F.Accumulator(), F.Accumulator()
        cor_cont = 0.0
        # the thermostats' starting xi: 0 in v25, 1 in v251 (Thermostat())
        xi, strn = (np.ones(2) if self.v251 else np.zeros(2)), np.zeros(2)
        self._npc = [0, 0]
        rng_state = [None, None]
        clust = np.zeros(n, dtype=np.int32)
        hist = None
        if p.signal == 0:
            # positions and momenta are made on the GPU once the batch exists
            box = new_box(p)
            r, pm, l = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
            O = np.tile(np.eye(3), (n, 1, 1))
        elif p.signal in (1, 2):
            if p.signal == 2:
                if not os.path.exists(self.path("counters.dat")):
                    raise RunError("problem opening counters.dat for reading")
                got = F.read_counters(self.path("counters.dat"), npc=self.v251)
                Time, cont, Ntcf, Ntcv, mcont, AcT, AcTsq = got[:7]
                if self.v251:
                    self._npc = list(got[7])
            if not os.path.exists(self.path("conf.dat")):
                raise RunError("problem opening conf.dat for reading")
            c = F.read_conf(self.path("conf.dat"), p.n_part, nd_part)
            # the masses come from input.txt: set_mass(mass[n]) follows chrg_conf (v25/main.cpp:272-278)
            box, r, pm, O, l = c["box"], c["r"], c["p"], c["O"], c["l"]
            xi, strn, clust = c["xi"], c["strn"], c["clust"].astype(np.int32)
            for k in range(2):
                f = self.path(f"ran_state{k}F.dat")
                if not os.path.exists(f):
                    raise RunError(f"problem reading ran_state{k}.dat")
                rng_state[k] = F.read_mt_state(f)
        else:
            raise RunError("signal must be 0, 1 or 2!")
        Lmin = float(min(box))
        nbins = int(math.floor(math.sqrt(3.0) * Lmin / (2.0 * p.bar_w)))
        nblk = p.n_comp + p.n_comp * (p.n_comp - 1) // 2
        hist = np.zeros((nblk, 4, nbins))
        if p.signal == 2:
            if os.path.exists(self.path("correlation.dat")):
                cor_cont, hist = F.read_correlation(self.path("correlation.dat"), p.n_part, nbins)
            else:
                self.error("problem opening correlation.dat for reading\nstarting correlation.dat from scratch!")
                cor_cont = 0.0
        # the total momentum check, as written (ptot[2] twice, v25/main.cpp:366)
        ptot = pm.sum(axis=0)
        if ptot[0] > 1e-8 or ptot[2] > 1e-8 or ptot[2] > 1e-8:
            raise RunError(f"Total momentum is not zero! : {F.g6(ptot[0])} , {F.g6(ptot[1])} , {F.g6(ptot[2])}")
        V = float(box[0] * box[1] * box[2])
        sr_cut = p.sr_cut if p.sr_cut != 0 else Lmin / 2 - dmin
        if sr_cut > Lmin / 2:
            raise RunError(f"sr_cut must be less than L/2-dmax: {F.g6(Lmin / 2 - dmin)}")
        if sr_cut < dmax + 0.5:
            raise RunError(f"sr_cut must be >= the largest dimension  + 0.5.and {F.g6(sr_cut)} < {F.g6(dmax + 0.5)}")
        if Lmin > 200:
            raise RunError(f"Tab is not large enough. Lmin={F.g6(Lmin)} > 200")

        spec = SystemSpec(n=n, box=box, alpha=p.alpha, K_max=p.K_max, ksq_max=self.ksq_max, temp=p.temp, Q=p.Q,
                          gamma=p.gamma, dt=p.Dt, B=np.asarray(p.B, dtype=np.float64), sr_cut=sr_cut, xi0=0.0,
                          min_s=p.min_s, cl_fr=p.cl_fr, rc_real=self.rc_real, cl_energy=self.cl_energy)
        st = SystemState(r, pm, O, l, length, dia, mass, dip)
        self._mass = mass
        # each particle's own dipoles (its species'): print_conf writes no padding
        self._ndip = np.repeat(np.asarray(nd_part, dtype=np.int64), p.n_part)
        bt = L.Batch([spec], None, device=self.device, descs=[L.desc_from_spec(spec, nd)])
        try:
            return self._loop(p, bt, st, clust, xi, strn, rng_state, box, V, Lmin, nbins, hist, cor_cont, Time,
                              cont, Ntcf, Ntcv, mcont, AcT, AcTsq, length, dia, mass, dip, nd_part)
        finally:
            bt.close()

    # ------------------------------------------------------------------
    def _loop(self, p, bt, st, clust, xi, strn, rng_state, box, V, Lmin, nbins, hist, cor_cont, Time, cont,
              Ntcf, Ntcv, mcont, AcT, AcTsq, length, dia, mass, dip, nd_part) -> int:
        n = p.n_total
        bt.upload(0, st, clust=clust)
        r_start = st.r
        if p.signal == 0:
            nov = bt.lattice(0, p.n_part)
            d0 = bt.download(0)
            F.write_ini_pos(self.path("iniPos.dat"), d0["r"], box)
            r_start = d0["r"]
            if nov:
                self.error("initial conf. overlap")
            bt.thermalize(0, p.temp, seed=1)
        bt.set_thermostat(0, xi, strn)
        for k in range(2):
            if rng_state[k] is not None:
                bt.set_rng(0, k, *rng_state[k])
        if p.n_comp > 1:
            bt.set_species(0, p.n_part)
        if p.signal == 0:
            self._print_conf(bt, box, dip)
        F.write_comp_conf(self.path("compConf.dat"), r_start)
        # the initial forces: force_sc's overlap check before the loop
        try:
            obs0 = bt.observe()[0]
        except L.MdscError as e:
            if e.code == OVERLAP:
                raise RunError("initial overlap!") from e
            raise
        Uself = obs0["U_self"] / n
        var = F.Accumulator()
        np_tc = [min(int(k), MX_TCF) for k in p.n_part]
        I = inertia(length, dia, mass)
        total = p.pre_steps + p.Nsteps
        t_wall0, t_cpu0 = time.perf_counter(), time.process_time()
        step = 0
        while step < total:
            # steps up to the next one that needs more than its observables
            nxt = step
            while nxt < total - 1 and not self._event(p, nxt):
                nxt += 1
            try:
                trace = bt.step_trace(nxt - step + 1)
            except L.MdscError as e:
                if e.code == OVERLAP:  # force_sc's false (v25/main.cpp:591-597)
                    self._print_conf(bt, box, dip)
                    raise RunError("overlap!") from e
                raise
            for k, ob in enumerate(trace):
                s = step + k
                o = ob[0]
                # the top of the reference's step (v25/main.cpp:522-528)
                if s == p.pre_steps and p.signal in (0, 1):
                    Time = 0.0
                if Time == 0.0:
                    for fn in ("ptens.dat", "magmom.dat"):
                        if os.path.exists(self.path(fn)):
                            os.remove(self.path(fn))
                print(F.g6(Time), file=self.out)
                self._set_var(var, o, n, V, p.dens, Uself)
                Time += p.Dt
                if self.v251 and p.cl_fr > 0 and math.fmod(float(s), p.cl_fr) == 0:
                    # this step clustered (the last of its chunk): the degree of polymerisation
                    lab = bt.download(0)["clust"]
                    sizes = np.bincount(lab[lab >= 0])
                    self._npc[0] += 1
                    self._npc[1] += int(sizes[sizes > 1].sum())
                if s >= p.pre_steps:
                    if p.corrf > 0 and math.fmod(float(np.float32(s)), p.corrf) == 0:
                        t_c = time.perf_counter()
                        hist = bt.correlations(p.bar_w, [hist])[0]
                        self._cor_s += time.perf_counter() - t_c
                        cor_cont += 1.0 / V
                    var.G1, var.G2 = o["G1"], o["G2"]
                    if p.tcfd > 0 and math.fmod(float(np.float32(s)), p.tcfd) == 0:
                        self._pos_vel(bt, np_tc, p, I, mass, Ntcf)
                        Ntcf += 1
                    if p.tcfv > 0 and math.fmod(float(np.float32(s)), p.tcfv) == 0:
                        d = bt.download(0)
                        HF = np.einsum("ni,nj->ij", d["r"], d["p"])
                        F.append(self.path("ptens.dat"), F.ptens_line(Time, HF, var.PT))
                        Ntcv += 1
                        # the moment from FP64 sums (the step's own M is summed from
                        # the FP32 dipole vectors, ~1e-7 of each moment)
                        M = bt.order_params()[2][0]
                        F.append(self.path("magmom.dat"), F.magmom_line(Time, M))
                        mcont += 1
                    AcT += var
                    AcTsq += var * var
                    cont += 1
                if math.fmod(float(s), p.iprint) == 0:
                    d = self._print_conf(bt, box, dip)
                    F.write_counters(self.path("counters.dat"), Time, cont, Ntcf, Ntcv, mcont, AcT, AcTsq,
                                     npc=self._npc if self.v251 else None)
                    if s >= p.pre_steps and p.corrf > 0 and math.fmod(float(np.float32(s)), p.corrf) == 0:
                        F.write_correlation(self.path("correlation.dat"), hist, p.n_part, Lmin, p.bar_w, cor_cont)
                    # total momentum and angular momentum (v25/main.cpp:788-800)
                    Mom = list(d["p"].sum(axis=0)) + list(d["l"].sum(axis=0))
                    t_wall, t_cpu = time.perf_counter(), time.process_time()
                    # microseconds as integers, divided as the reference divides them
                    te = (int((t_wall - t_wall0) * 1e6) // p.iprint) * 1e-6
                    tc = (int((t_cpu - t_cpu0) * 1e6) / p.iprint) * 1e-6
                    F.append(self.path("output.dat"), F.output_line(Time, te, tc, var, Mom))
                    t_wall0, t_cpu0 = t_wall, t_cpu
            step = nxt + 1
        self._write_time(bt, p, V, cor_cont)
        if cont > 0:
            pol = None
            if self.v251:
                num, den = float(self._npc[1]), float(n * self._npc[0])
                pol = num / den if den != 0 else (float("nan") if num == 0 else float("inf"))
            F.append(self.path("output.dat"), F.final_report(Time, AcT, AcTsq, cont, p, box, pol_deg=pol))
        return 0

    def _write_time(self, bt, p, V: float, cor_cont: float) -> None:
        """time.dat in the reference's layout (v25/main.cpp:825-838; the later
        driver adds the two Ewald lines, v25/v251/main.cpp:826-840): seconds
        per step of each function's GPU kernels, timed with CUDA events on a
        copy of the final state (the run's own state is not advanced), and
        the correlation calls' host time divided as the reference divides
        it.  The cpu column is the host's share, which the GPU work leaves at
        about zero."""
        ms = {}
        try:
            with L.Batch([None], None, device=self.device, descs=[bt._descs[0]]) as sc:
                sc.transfer_from(0, bt, 0)
                ms = sc.profile(5)
        except L.MdscError:
            pass
        t = lambda *names: sum(ms.get(x, 0.0) for x in names) * 1e-3  # noqa: E731
        rows = [("X move time", t("integrate_first")), ("Force_ss time", t("list_build", "wca"))]
        if self.v251:
            rows += [("Force_dipR time", t("real_pairs", "real_sum", "near_pass_real")),
                     ("Force_dipK time", t("kspace_sum", "kspace_combine", "kspace_gather"))]
        rows.append(("P move time", t("finalize", "reduce_obs")))
        cor = self._cor_s / (V * cor_cont) if cor_cont > 0 else 0.0
        rows.append(("correl. time", cor))
        with open(self.path("time.dat"), "w") as f:
            for name, sec in rows:
                f.write(f"{name}. elap: {F.g6(sec)} cpu: 0\n")

    def _event(self, p, s: int) -> bool:
        """A step after which the loop needs more than the step's observables."""
        if math.fmod(float(s), p.iprint) == 0:
            return True
        if self.v251 and p.cl_fr > 0 and math.fmod(float(s), p.cl_fr) == 0:
            return True
        if s >= p.pre_steps:
            for fr in (p.corrf, p.tcfd, p.tcfv):
                if fr > 0 and math.fmod(float(np.float32(s)), fr) == 0:
                    return True
        return False

    @staticmethod
    def _set_var(var, o, n, V, dens, Uself) -> None:
        """The step's thermodynamic values (v25/main.cpp:618-650)."""
        WdipR, WdipK = 3 * o["U_dipR"], 3 * o["U_dipK"]
        var.K = (o["K"][0] + o["K"][1]) / n
        var.Uss, var.UdipR, var.UdipK, var.Uext = o["U_ss"] / n, o["U_dipR"] / n, o["U_dipK"] / n, o["U_ext"] / n
        var.U = Uself + var.Uss + var.UdipR + var.UdipK + var.Uext
        var.Pss = o["W_ss"] / (3 * V)
        var.PdipR = WdipR / (3 * V)
        var.PdipK = WdipK / (3 * V)
        ctemp = var.K / 3
        var.P = ctemp * dens + var.Pss + var.PdipR + var.PdipK
        var.PTkin = np.array(o["PT_kin"]).reshape(3, 3) / V
        var.PTss = np.array(o["PT_ss"]).reshape(3, 3) / V
        var.PTdipR = np.array(o["PT_dipR"]).reshape(3, 3) / V
        var.PTdipK = np.array(o["PT_dipK"]).reshape(3, 3) / V
        var.PT = var.PTkin + var.PTss + var.PTdipR + var.PTdipK

    def _print_conf(self, bt, box, dip) -> None:
        """conf.dat and the generator states, as print_conf(..., fin = true)."""
        d = bt.download(0)
        xi, strn = bt.get_thermostat(0)
        F.write_conf(self.path("conf.dat"), box, d["r"], d["p"], d["O"], d["l"], self._mass, dip, d["clust"], xi,
                     strn, ndip=self._ndip)
        for k in range(2):
            mt, mti = bt.get_rng(0, k)
            F.write_mt_state(self.path(f"ran_state{k}F.dat"), mt, mti)
        return d

    def _pos_vel(self, bt, np_tc, p, I, mass, num) -> None:
        """pos_vel/pos_vel_<num>.dat (v25/functions.cpp:2602-2643): centre,
        velocity, axis and angular velocity O^T I^-1 O l of the first
        np_tc particles of each species."""
        d = bt.download(0)
        rows = []
        i0 = 0
        for s in range(p.n_comp):
            m = mass[i0]
            for i in range(i0, i0 + np_tc[s]):
                O = d["O"][i]
                Ib = O.T @ np.diag(1.0 / I[i]) @ O
                rows.append((d["r"][i], d["p"][i] / m, O[2], Ib @ d["l"][i]))
            i0 += int(p.n_part[s])
        F.ensure_dir(self.path("pos_vel"))
        F.write_pos_vel(self.path(os.path.join("pos_vel", f"pos_vel_{num}.dat")), rows, p.Dt * p.tcfd)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("workdir", nargs="?", default=".")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--variant", choices=("v25", "v251"), default="v25")
    ap.add_argument("--real-cutoff", type=float, default=0.0,
                    help="real-space cutoff (the reference's table zeroed beyond it); 0: all pairs")
    ap.add_argument("--ksq-max", type=int, default=0, help="keep |n|^2 <= this of the k cube; 0: the whole cube")
    ap.add_argument("--cluster-energy", type=float, default=0.0,
                    help="clusters by pair energy below -this kT; 0: the reference's geometric test")
    a = ap.parse_args(argv)
    return Driver(a.workdir, a.device, variant=a.variant, rc_real=a.real_cutoff, ksq_max=a.ksq_max,
                  cl_energy=a.cluster_energy).run()


if __name__ == "__main__":
    sys.exit(main())
