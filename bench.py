#!/usr/bin/env python
"""Benchmark of the GB300 MD step on the 256-replica mix.

Workload (default "replica_mix"): 256 independent dipolar-spherocylinder
systems, N log-uniform in [128, 2048] (182,573 particles in all), packing
fraction U[0.05, 0.25], mu^2 U[0.5, 4], T U[0.8, 1.5], lengths U[2, 4],
alpha = 6/L_box, |n|^2 <= 36, real space over all minimum-image pairs,
Nose thermostat Q = 1, dt = 1e-3; seeded synthetic configurations.  One
"step" advances every system by one MD step in one CUDA-graph launch.

Metric: aggregate particle-steps/s.  `value` is device-timed with the
state resident in HBM (CUDA events around each step, L2 flushed between
steps); `e2e` goes through the C ABI with host buffers: every step uploads
the packed state (r, p, O, l, F, T) from pinned memory, steps once and
downloads the observables and the whole updated state again.  The roofline
of the dominant kernel (real_pairs, FP32-bound) is taken against the FP32
multiply-add peak measured on the same device (mdsc_fp32_peak).

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]
                  [--workload replica_mix|c0|c1|c2]

--workload c0/c1/c2 runs one system of the single-system configurations
instead (N = 256, 4096, 32768; c2 clusters every 100 steps by pair energy,
timed beside the steps).

--impl reference times the reference's CPU routines (the C restatement in
oracle/, all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "particle-steps/s batched/served vs plain GPU at <=1e-5 force err; job p50/p99"
UNIT = "particle-steps/s"
# real-space Ewald pair: FLOP per dipole pair of the tile kernel
# (minimum image 9, r^2 5, rsqrt 1, erfc + exp ~30, A B C 12, table
# correction 15, three dot products 15, energy 4, force 21, torques 36,
# pressure tensor 18, accumulation 13 -> ~180, the figure of the survey)
FLOP_PER_PAIR = 180.0
# DRAM bytes (read + write) per dipole pair of real_pairs_kernel from one
# cold-cache ncu capture: 3.751 MB + 0.003 MB over the 47,281,855 pairs of the
# 128-replica mix (profiles/real_pairs_replica_mix128.md, the analytic form).
# The kernel reads each tile's dipoles and writes its partial slots, so its
# traffic scales with the work a launch processes.
REAL_PAIRS_DRAM_BYTES_PER_PAIR = 3.754e6 / 47_281_855


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate_ranks(sums, maxes, device="cpu"):
    """Whole-job figures over the ranks of the process group: each entry of
    `sums` added over ranks (particles, work), each entry of `maxes` the
    maximum over ranks (times).  One rank: returned unchanged."""
    import torch
    import torch.distributed as dist

    sums, maxes = [float(x) for x in sums], [float(x) for x in maxes]
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return sums, maxes
    a = torch.tensor(sums, dtype=torch.float64, device=device)
    b = torch.tensor(maxes, dtype=torch.float64, device=device)
    dist.all_reduce(a, op=dist.ReduceOp.SUM)
    dist.all_reduce(b, op=dist.ReduceOp.MAX)
    return a.tolist(), b.tolist()


def build_mix(seed: int, nsys: int):
    from mdspherocyl_gb300 import systems as S

    ds = S.replica_mix_specs(n_systems=nsys, seed=seed)
    return [S.replica_system(d) for d in ds], ds


# the single-system configurations: builder, description, energy-criterion
# cluster threshold (kT) or None
SINGLE = {
    "c0": ("plain_c0", "N=256, phi=0.10, L ~ N(3, 0.3), mu^2=2 axial, alpha=5.6/L_box, |n|^2<=27", None),
    "c1": ("plain_c1", "N=4096, phi=0.20, L ~ U[2, 5], mu ~ volume with <mu^2>=3, alpha=7/L_box, |n|^2<=64", None),
    "c2": ("plain_c2", "N=32768, phi=0.15, mu^2=5, field mu B/kT=2 along z, L ~ N(3, 0.5), alpha=6/L_box, "
                       "|n|^2<=100, clusters every 100 steps by pair energy < -1.5 kT", 1.5),
}


def build_workload(args, rank: int = 0):
    """[(spec, state)] of the workload and its config entries."""
    if args.workload == "replica_mix":
        states, _ = build_mix(args.seed + 1000 * rank, args.systems)
        return states, {"workload": "replica_mix", "ksq_max": 36, "alpha": "6/L_box"}
    from mdspherocyl_gb300 import systems as S

    fn, desc, _ = SINGLE[args.workload]
    spec, st = getattr(S, fn)(seed=args.seed + 1000 * rank)
    spec.rc_real = 0.5 * float(min(spec.box)) if args.real_cutoff == "half" else float(args.real_cutoff)
    args.rc_value = spec.rc_real
    return [(spec, st)], {"workload": f"plain_{args.workload}", "description": desc, "ksq_max": spec.ksq_max,
                          "alpha": float(spec.alpha), "box": float(spec.box[0])}


def real_space(args) -> str:
    rc = getattr(args, "rc_value", 0.0)
    if args.workload != "replica_mix" and rc > 0:
        return f"cutoff {rc:.4g}: the reference's table zeroed beyond it, over a neighbour list (rc_real)"
    return "all minimum-image pairs"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(states, threads: int, budget_s: float = 20.0, stride: int = 16, keep: dict | None = None):
    """Times the oracle's MD step (the reference's routines restated in C,
    OpenMP over `threads` host threads) on every `stride`-th system of the
    mix -- a sample that spans the mix's N distribution -- one step each,
    until `budget_s` is spent.  Returns particle-steps/s and the sample.
    With `keep`, each stepped system's results (observables, F, T, r, p)
    are stored there by system index: the oracle's answers for the parity
    block."""
    import oracle

    orc = oracle.Oracle()
    orc.set_threads(threads)
    done_p, t_tot, used = 0, 0.0, []
    for k in range(0, len(states), stride):
        spec, st = states[k]
        o = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, spec.box)
        md = oracle.MDOracle(orc, o, dt=spec.dt, temp=spec.temp, Q=spec.Q, gamma=spec.gamma, xi0=spec.xi0,
                             sr_cut=3.0, K_max=spec.K_max, ksq_max=spec.ksq_max, alpha=spec.alpha, B=spec.B,
                             rc_real=spec.rc_real)
        t0 = time.perf_counter()
        md.step()
        t_tot += time.perf_counter() - t0
        done_p += spec.n
        used.append(spec.n)
        if keep is not None:
            keep[k] = {"obs": md.obs(), "F": o.F.copy(), "T": o.T.copy(), "r": o.r.copy(), "p": o.p.copy()}
        md.close()
        if t_tot > budget_s:
            break
    return done_p / t_tot, used, t_tot


# ---- parity of the GPU path against the oracle (the CPU leg's checker) ----
# bars: Ewald forces and torques RMS relative 1e-5; total energy of a step
# 1e-7; U alone 1e-6; pressure tensor RMS relative 1e-5; WCA (FP64) 1e-12;
# cluster labels identical
BARS = {"rms_F": 1e-5, "rms_T": 1e-5, "rel_E": 1e-7, "rel_U": 1e-6, "rms_PT": 1e-5}


def _rms_rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    den = float(np.sqrt(np.mean(b ** 2)))
    return float(np.sqrt(np.mean((a - b) ** 2)) / den) if den > 0 else float(np.abs(a).max())


def _step_errors(gobs, gstate, oobs, ostate):
    """Errors of one GPU step against the oracle's step of the same system."""
    Ug = gobs["U_ss"] + gobs["U_dipR"] + gobs["U_dipK"] + gobs["U_ext"] + gobs["U_self"]
    Uo = oobs["Uss"] + oobs["UdipR"] + oobs["UdipK"] + oobs["Uext"] + oobs["Uself"]
    Kg, Ko = float(np.sum(gobs["K"])), float(np.sum(oobs["K"]))
    PTg = sum(np.asarray(gobs[k]).reshape(3, 3) for k in ("PT_kin", "PT_ss", "PT_dipR", "PT_dipK"))
    PTo = oobs["PTkin"] + oobs["PTss"] + oobs["PTdipR"] + oobs["PTdipK"]
    return {"rms_F": _rms_rel(gstate["F"], ostate["F"]), "rms_T": _rms_rel(gstate["T"], ostate["T"]),
            "rel_E": abs((Kg + Ug) - (Ko + Uo)) / abs(Ko + Uo), "rel_U": abs(Ug - Uo) / abs(Uo),
            "rms_PT": _rms_rel(PTg, PTo), "max_dr": float(np.abs(gstate["r"] - ostate["r"]).max())}


def _worst(rows):
    w = {k: max(r[k] for r in rows) for k in rows[0]}
    w["within_bars"] = all(w[k] <= v for k, v in BARS.items() if k in w)
    return w


def parity_block(mix_first, mix_oracle, device: int, threads: int, with_c2: bool = True) -> dict:
    """One step of c0 (N=256) and c1 (N=4096) from their seeded states, the
    sampled systems of the mix (c3, stepped inside the full batch), and one
    evaluation of every force term of c2 (N=32768) with its geometric
    cluster labels: GPU against the oracle."""
    import oracle
    from mdspherocyl_gb300 import lib as L
    from mdspherocyl_gb300 import systems as S

    orc = oracle.Oracle()
    orc.set_threads(threads)
    out = {"bars": BARS}
    rows = [_step_errors(mix_first[k][0], mix_first[k][1], mix_oracle[k]["obs"], mix_oracle[k])
            for k in sorted(mix_oracle) if k in mix_first]
    if rows:
        out["c3"] = {"systems": len(rows), "what": "every 16th system of the mix, one step inside the full batch",
                     **_worst(rows)}
    for name, fn in (("c0", "plain_c0"), ("c1", "plain_c1")):
        spec, st = getattr(S, fn)(seed=3)
        with L.Batch([spec], [st], device=device) as b1:
            gobs = b1.step(1)[0]
            gst = b1.download(0)
        o = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, spec.box)
        md = oracle.MDOracle(orc, o, dt=spec.dt, temp=spec.temp, Q=spec.Q, gamma=spec.gamma, xi0=spec.xi0,
                             sr_cut=3.0, K_max=spec.K_max, ksq_max=spec.ksq_max, alpha=spec.alpha, B=spec.B)
        md.step()
        e = _step_errors(gobs, gst, md.obs(), {"F": o.F, "T": o.T, "r": o.r})
        md.close()
        out[name] = {"n": spec.n, "what": "one step from the seeded state", **e,
                     "within_bars": all(e[k] <= v for k, v in BARS.items())}
    if with_c2:
        spec, st = S.plain_c2(seed=3)
        c2 = {"n": spec.n, "what": "one evaluation of each force term; geometric cluster labels"}
        with L.Batch([spec], [st], device=device) as b1:
            for name, call, ofn in (
                ("sc", b1.force_sc, lambda s: orc.force_sc(s, 3.0, 3.5)[1:]),
                ("dipR", b1.force_dipR, lambda s: orc.force_dipR(s, spec.alpha)),
                ("dipK", b1.force_dipK, lambda s: orc.force_dipK(s, spec.K_max, spec.alpha, spec.ksq_max)),
            ):
                b1.zero_forces()
                res = call()
                d = b1.download(0)
                so = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, spec.box)
                ores = ofn(so)
                c2[name] = {"rms_F": _rms_rel(d["F"], so.F), "rms_T": _rms_rel(d["T"], so.T),
                            "rel_U": abs(res[0][0] - ores[0]) / abs(ores[0]), "rms_PT": _rms_rel(res[-1][0], ores[-1])}
            lab, nc = b1.clust_conf(0)
        so = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, spec.box)
        lo, nco, _ = orc.clust_conf(so, float(spec.min_s), seed=1, skip=0)
        c2["labels_equal"] = bool(np.array_equal(lab, lo)) and nc == nco
        c2["clusters"] = int(nc)
        c2["within_bars"] = (c2["labels_equal"] and max(c2["sc"][k] for k in ("rms_F", "rms_T", "rel_U")) <= 1e-12
                             and all(c2[t][k] <= 1e-5 for t in ("dipR", "dipK") for k in ("rms_F", "rms_T", "rel_U",
                                                                                         "rms_PT")))
        out["c2"] = c2
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    states, cfg = build_workload(args)
    single = args.workload != "replica_mix"
    if single:
        # one system: one full-size step is the bounded sample
        v, used, tt = cpu_sample(states, threads, budget_s=args.cpu_budget, stride=1)
        value, ms_step = v, 1e3 * tt
        sample = (f"oracle MD step (reference routines restated in C, OpenMP) on the whole system (N={used[0]}), "
                  f"one step")
    else:
        # every 16th system of the mix, each built once (untimed); every timed step
        # is one MD step of one of them, round robin, so K steps cost about K / 16
        # sample steps; the rate is all particles stepped over all the time taken
        import oracle

        orc = oracle.Oracle()
        orc.set_threads(threads)
        mds, ns = [], []
        for k in range(0, len(states), 16):
            spec, st = states[k]
            o = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, spec.box)
            mds.append(oracle.MDOracle(orc, o, dt=spec.dt, temp=spec.temp, Q=spec.Q, gamma=spec.gamma,
                                       xi0=spec.xi0, sr_cut=3.0, K_max=spec.K_max, ksq_max=spec.ksq_max,
                                       alpha=spec.alpha, B=spec.B, rc_real=spec.rc_real))
            ns.append(spec.n)
        for it in range(args.warmup):
            mds[it % len(mds)].step()
        done_p, tt = 0, 0.0
        for it in range(args.steps):
            k = (args.warmup + it) % len(mds)
            t0 = time.perf_counter()
            mds[k].step()
            tt += time.perf_counter() - t0
            done_p += ns[k]
        for md in mds:
            md.close()
        value, ms_step = done_p / tt, 1e3 * tt / max(args.steps, 1)
        sample = (f"oracle MD step (reference routines restated in C, OpenMP) on every 16th system of the mix "
                  f"({len(mds)} systems, N={min(ns)}..{max(ns)}), each built once; one system's step per timed "
                  f"step, round robin")
    cfg.update({"systems": len(states), "particles": int(sum(s.n for s, _ in states)),
                "real_space": real_space(args)})
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": cfg,
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def run_serving(args, device: int, jobs_n: int, rate: float, seed_off: int = 0) -> dict:
    """Poisson stream of jobs (one system each) through the continuous-
    batching server; job configurations are generated before the clock
    starts (they are the clients' inputs)."""
    import multiprocessing as mp

    from mdspherocyl_gb300 import serve
    from mdspherocyl_gb300 import systems as S

    arr = serve.poisson_arrivals(jobs_n, rate, seed=args.seed + 7 + seed_off)
    t0 = time.time()
    ids = [seed_off * 100_000 + k for k in range(jobs_n)]
    with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
        made = pool.map(S.serving_job, ids, chunksize=1)
    log(f"serving: {jobs_n} jobs generated in {time.time() - t0:.1f}s")
    jobs = [serve.Job(k, spec, st, spec.steps, arrival=float(arr[k])) for k, (spec, st) in enumerate(made)]
    srv = serve.Server(hbm_budget_bytes=120e9, tick_steps=args.tick, device=device)
    t0 = time.perf_counter()
    stats = srv.run(jobs)
    wall = time.perf_counter() - t0
    out = serve.summarize(stats, wall, jobs)
    out.update({"rate_per_s": rate, "hbm_budget_bytes": 120e9, "tick_steps": args.tick,
                "jobs_spec": "N log-U[64,8192], steps U[500,5000], phi U[.05,.25], mu^2 U[.5,5], T U[.8,1.5], "
                             "L ~ N(3, 0.3); alpha = 6/L_box, |n|^2 <= 36"})
    return out


def run_ours(args):
    ws, rank, local = dist_env()
    import torch

    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    device = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(device)
    from mdspherocyl_gb300 import lib as L

    t0 = time.time()
    states, cfg = build_workload(args, rank)
    single = args.workload != "replica_mix"
    specs = [s for s, _ in states]
    sts = [st for _, st in states]
    ntot = int(sum(s.n for s in specs))
    log(f"[rank {rank}] workload built in {time.time() - t0:.1f}s: {len(specs)} systems, {ntot} particles")
    bt = L.Batch(specs, sts, device=device)
    u_bond = SINGLE[args.workload][2] if single else None
    if u_bond:
        bt.set_cluster_energy(0, u_bond)
    stream = torch.cuda.ExternalStream(bt.lib.mdsc_stream(bt.h), device=device)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{device}")

    # ---- the first step of the sampled systems, kept for the parity block ----
    mix_first = {}
    if not single and not args.no_cpu and not args.no_parity and ws == 1:
        first = bt.step(1)
        mix_first = {k: (first[k], bt.download(k)) for k in range(0, len(specs), 16)}

    # ---- device-resident throughput ----
    bt.step(max(args.warmup, 3))
    torch.cuda.synchronize()
    clk = ClockSampler(device)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk.start()
    ms = []
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()  # L2 (129 MB) flushed between timed steps, outside the timed region
        code = bt.lib.mdsc_step(bt.h, 1, None)  # CUDA events on the library's stream around the step
        if code != 0:
            raise L.MdscError(code, "mdsc_step", bt._err())
        ms.append(bt.lib.mdsc_last_device_ms(bt.h))
    torch.cuda.synchronize()
    clocks = clk.stop()
    t_dev = sum(ms) / 1e3
    # every rank runs its own mix (different seeds, so different particle
    # counts): whole-job particles summed, time the slowest rank's
    (ntot_all,), (t_dev,) = aggregate_ranks([ntot], [t_dev], device=f"cuda:{device}")
    value = ntot_all * args.steps / t_dev
    obs = bt.observe()
    # kernels per graph-launched step, as captured for the timed steps (a
    # later mdsc_set_list_cells drops the graphs and the count with them),
    # + the per-call reset of the noise row
    launches = bt.launches_per_step + 1
    st_ok = all(o["status"] == 0 for o in obs)
    clustering = None
    if single and specs[0].cl_fr > 0:
        # the clusterings the step runs every cl_fr steps are outside the
        # device-timed graph launches: timed here, host clock around a
        # synchronous mdsc_clust_conf (bonds, union-find, label replay)
        bt.clust_conf(0)
        tc = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, ncl = bt.clust_conf(0)
            tc.append(time.perf_counter() - t0)
        c_ms = 1e3 * statistics.median(tc)
        per_step = c_ms / specs[0].cl_fr
        clustering = {"every": specs[0].cl_fr, "criterion": f"pair energy < -{u_bond} kT" if u_bond else "geometric",
                      "ms_per_clustering": c_ms, "clusters": ncl,
                      "value_with_clustering": ntot * args.steps / (t_dev + args.steps * per_step / 1e3)}

    # ---- the plain path: one system per launch sequence, one after another ----
    plain = None
    if not args.no_plain and ws == 1 and not single:  # the batched-vs-plain ratio: a one-GPU, mix figure
        singles = [L.Batch([sp], [st], device=device) for sp, st in zip(specs, sts)]
        for b1 in singles:
            b1.step(2)
        dev_ms, t0 = 0.0, time.perf_counter()
        for _ in range(args.plain_steps):
            for b1 in singles:
                code = b1.lib.mdsc_step(b1.h, 1, None)
                if code != 0:
                    raise L.MdscError(code, "mdsc_step (plain)", b1._err())
                dev_ms += b1.lib.mdsc_last_device_ms(b1.h)
        wall = time.perf_counter() - t0
        for b1 in singles:
            b1.close()
        pv_dev = ntot * args.plain_steps / (dev_ms / 1e3)
        pv_wall = ntot * args.plain_steps / wall
        plain = {"value_device": pv_dev, "value_wall": pv_wall, "unit": UNIT, "steps": args.plain_steps,
                 "how": "each system its own handle and launch sequence, stepped one after another",
                 "batched_over_plain_device": value / pv_dev, "batched_over_plain_wall": value / pv_wall}

    # ---- kernel times (events per kernel, serialised) ----
    tun = bt.tuning()
    tuning = {k: tun[k] for k in ("rp_warps", "rsum_threads", "wca_blocks", "kg_scalar")}
    tuning["chosen_by"] = "autotuner (mdsc_autotune)" if tun["tuned"] else "defaults"
    prof = bt.profile(max(2, min(5, args.steps)))
    pairs = sum(s.n * (s.n - 1) // 2 for s in specs)
    # with a real-space cutoff the tiles do not run (real_cut does, over the
    # neighbour list): no all-pairs roofline
    cutoff = single and getattr(args, "rc_value", 0.0) > 0
    rp_ms = prof.get("real_pairs", float("nan"))
    achieved = FLOP_PER_PAIR * pairs / (rp_ms * 1e-3) / 1e12 if not cutoff else float("nan")
    # the FP32 multiply-add peak of this device, measured (mdsc_fp32_peak),
    # with the SM clock sampled while the probe runs
    pclk = ClockSampler(device)
    pclk.start()
    probe = L.fp32_peak(device, reps=5)
    probe_clocks = pclk.stop()
    fp32_peak = max(probe["ffma_tflops"], probe["ffma2_tflops"])

    # ---- end to end through the C ABI with host buffers ----
    nd = sts[0].dip.shape[1]
    pin = lambda *shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()  # noqa: E731
    h = {k: pin(ntot, 3) for k in ("r", "p", "l", "F", "T")}
    h["O"] = pin(ntot, 3, 3)
    bt.download_all(h["r"], h["p"], h["O"], h["l"], h["F"], h["T"])
    # every step: the step's input (the whole state of every system) from
    # pinned host memory, the step, and the step's result read back: every
    # system's observables (energies, pressure tensors, thermostat, status)
    # and the whole updated state (r, p, O, l, F, T), as a caller of the
    # reference's per-function boundary needs it
    obs_buf = (L.Observables * len(specs))()
    bytes_state = sum(v.nbytes for v in h.values())
    bytes_obs = ctypes.sizeof(obs_buf)

    def e2e_step(state_back: bool):
        # mdsc_step_io: the state up, one step, the observables and (state_back)
        # the updated state down into the same host arrays
        bt.step_io(h, 1, h if state_back else None, obs_buf)

    def e2e_rate(state_back: bool):
        for _ in range(2):
            e2e_step(state_back)
        nst = max(3, min(args.steps, 20))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(nst):
            e2e_step(state_back)
        torch.cuda.synchronize()
        tt = time.perf_counter() - t0
        (_,), (tt,) = aggregate_ranks([0], [tt], device=f"cuda:{device}")
        return ntot_all * nst / tt

    e2e = e2e_rate(True)
    e2e_obs_only = e2e_rate(False)

    # ---- a forced list rebuild of every system (mdsc_neigh_list: positions
    # to working copies, the build, a synchronize), on cells and over all
    # pairs: the two give the same lists ----
    def rebuild_ms(cells: bool) -> float:
        bt.set_list_cells(cells)
        bt.neigh_list()
        ts = []
        for _ in range(5):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            bt.neigh_list()
            ts.append(1e3 * (time.perf_counter() - t0))
        return statistics.median(ts)

    list_build = {"cells_ms": rebuild_ms(True), "all_pairs_ms": rebuild_ms(False),
                  "how": "host clock around mdsc_neigh_list (every system rebuilt, then a synchronize), median of 5"}
    bt.set_list_cells(True)

    # ---- the step graph's own cost: the same graph with every system held
    # at its step limit, so every kernel returns at once (launch, fork/join
    # and block-scheduling overhead per step) ----
    cur = [o["step"] for o in bt.observe()]
    for k in range(len(specs)):
        bt.set_step_limit(k, cur[k])
    bt.step(5)
    ov = []
    for _ in range(3):
        bt.lib.mdsc_step(bt.h, 50, None)
        ov.append(bt.lib.mdsc_last_device_ms(bt.h) / 50)
    for k in range(len(specs)):
        bt.set_step_limit(k, 0)
    graph_overhead = {"us_per_step": 1e3 * statistics.median(ov), "launches_per_step": launches,
                      "how": "device time of 50 graph launches with every system at its step limit, median of 3"}
    bt.close()
    serving = None
    if args.jobs > 0 and ws == 1 and not single:
        # the configured stream (2000 jobs at 40/s), then a rate the GPU sustains
        serving = run_serving(args, device, args.jobs, args.rate)
        if args.stable_jobs > 0:
            serving["at_sustainable_rate"] = run_serving(args, device, args.stable_jobs, args.stable_rate, seed_off=1)

    out = None
    if rank == 0:
        cpu = None
        if not args.no_cpu and ws == 1:
            threads = os.cpu_count() or 1
            mix_oracle = {}
            v, used, tt = cpu_sample(states, threads, budget_s=args.cpu_budget, stride=1 if single else 16,
                                     keep=mix_oracle)
            cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": (f"oracle MD step (reference routines restated in C, OpenMP, {threads} threads) "
                              f"on every 16th system of the mix ({len(used)} systems, N={min(used)}..{max(used)}, "
                              f"{sum(used)} particles), one step each, {tt:.1f}s") if not single else
                             (f"oracle MD step (reference routines restated in C, OpenMP, {threads} threads) "
                              f"on the whole system (N={used[0]}), one step, {tt:.1f}s")}
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair/k-space arithmetic, f64 state and sums",
            "data": "synthetic",
            "config": {**cfg, "systems": len(specs) * ws, "particles": int(ntot_all),
                       "particles_rank0": ntot,
                       "N_range": [min(s.n for s in specs), max(s.n for s in specs)],
                       "real_space": real_space(args), "dt": 1e-3,
                       "l2": "flushed between timed steps (256 MB write)", "parallelism": f"replicas x{ws}",
                       "graph": "one CUDA graph per step", "launch_mappings": tuning},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": bytes_state,
                    "d2h_bytes_per_step": bytes_state + bytes_obs,
                    "how": "C ABI (mdsc_step_io), pinned host buffers: the whole state up, one step, observables "
                           "and the whole updated state (r, p, O, l, F, T) down, every step; r and O travel while "
                           "the step's forces are computed",
                    "observables_only": {"value": e2e_obs_only, "d2h_bytes_per_step": bytes_obs}},
            "gpu_launches": launches * args.steps,
            "roofline": None if cutoff else {
                "bound": "fp32", "kernel": "real_pairs", "achieved": achieved, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                "traffic": REAL_PAIRS_DRAM_BYTES_PER_PAIR * pairs,
                "traffic_unit": "bytes per launch (ncu dram read+write, scaled by pairs)",
                "peak_source": ("measured: mdsc_fp32_peak (independent FFMA / FFMA2 chains on every SM, "
                                "CUDA events, best of 5), the larger of the two forms, of measured"),
                "peak_probe": {**probe, "clocks": probe_clocks},
                "flop_per_pair": FLOP_PER_PAIR, "pairs_per_launch": pairs,
                "kernel_ms": rp_ms},
            "kernel_ms": prof,
            "list_build": list_build,
            "graph_overhead": graph_overhead,
            "plain_gpu": plain,
            "serving": serving,
            "clustering": clustering,
            "clocks": clocks,
            "status_ok": st_ok,
        }
        if cpu is not None:
            out["cpu_baseline"] = cpu
            if not args.no_parity and not single:
                t0 = time.perf_counter()
                par = parity_block(mix_first, mix_oracle, device, threads, with_c2=not args.no_parity_c2)
                par["seconds"] = time.perf_counter() - t0
                out["parity"] = par
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--systems", type=int, default=256)
    ap.add_argument("--workload", default="replica_mix", choices=["replica_mix", *SINGLE],
                    help="replica_mix: the 256-system mix (the headline); c0/c1/c2: one system of that config")
    ap.add_argument("--real-cutoff", default="0",
                    help="c0/c1/c2: real-space cutoff, a length or 'half' (L_box/2); 0 = all pairs, the "
                         "reference (config 0 states L_box/2, config 1 3.5)")
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the parity block of the CPU leg")
    ap.add_argument("--no-parity-c2", action="store_true", help="parity block without the N=32768 evaluation")
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--jobs", type=int, default=2000, help="serving leg: jobs (0 = skip)")
    ap.add_argument("--rate", type=float, default=40.0, help="serving leg: arrivals per second")
    ap.add_argument("--stable-jobs", type=int, default=400,
                    help="serving leg: jobs of a second stream at a rate the GPU sustains (0 = skip)")
    ap.add_argument("--stable-rate", type=float, default=10.0, help="arrivals per second of that stream")
    ap.add_argument("--tick", type=int, default=50, help="serving leg: steps between admissions")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
