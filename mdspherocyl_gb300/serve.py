"""Continuous-batching job server for the GB300 MD step.

Jobs (one system each, with a number of steps) arrive over time.  The
server keeps every running system resident on the GPU in one batch and
advances the whole batch by a tick of steps, one CUDA-graph launch per step.
Each system carries a step limit (mdsc_set_step_limit): a job whose steps
run out within a tick stops at exactly its step count and costs nothing for
the rest of the tick, so ticks are never shortened for one job.

Membership changes at tick boundaries.  The next batch is planned before a
tick starts -- the jobs that will still be running after it (known from
their step counts) plus the waiting jobs that fit -- and a worker thread
builds it while the GPU runs the tick: the allocation, the new jobs'
uploads and step limits.  When the tick ends the running systems move into
it on the GPU (mdsc_transfer_many, one kernel, no host round trip) and the
next tick starts; the GPU waits only for those copies.  Admission is by an
HBM budget: the planned batch must fit it (during a repack the old and the
new batch are both resident).  A batch's device bytes are a sum over its
systems (every array is per system, per particle, per tile or per k), so the
server sums each job's own mdsc_estimate_bytes, taken once when the job is
first considered: never below the batch's estimate (each job's share carries
its own alignment) and within 1% of it on the 256-replica mix, with no
layout of the whole batch inside the tick loop.

A job's result is independent of the jobs it shares the GPU with: every
kernel works per system and sums in a fixed order, so a system gives the
same bits alone and in any mix (tests/test_serve.py).  A system that reports
an error (the reference's overlap abort, a NaN, a full list) fails its own
job, which leaves at the end of that tick; the others run on undisturbed.
"""
from __future__ import annotations

import json
import time
from collections import deque
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from . import lib as L
from .systems import SystemSpec, SystemState


@dataclass
class Job:
    jid: int
    spec: SystemSpec
    state: SystemState
    steps: int
    arrival: float = 0.0
    # filled in by the server
    start: float | None = None
    finish: float | None = None
    done: int = 0
    result: dict | None = None
    obs: dict | None = None
    error: str | None = None  # the status of a system that failed (overlap, NaN, ...)
    nbytes: int | None = None  # its device bytes alone (mdsc_estimate_bytes), once

    @property
    def n(self) -> int:
        return self.spec.n

    def record(self) -> dict:
        """One line of the server's job log."""
        rej = isinstance(self.obs, dict) and str(self.obs.get("status", "")).startswith("rejected")
        return {"job": self.jid, "n": self.n, "steps": self.steps, "done": self.done, "arrival": self.arrival,
                "start": self.start, "finish": self.finish,
                "latency": None if self.finish is None else self.finish - self.arrival,
                "error": self.obs["status"] if rej else self.error}


@dataclass
class ServerStats:
    completed: list = field(default_factory=list)
    ticks: int = 0
    repacks: int = 0
    particle_steps: int = 0
    gpu_ms: float = 0.0
    max_running: int = 0
    # per tick: seconds since the start, jobs waiting, jobs running,
    # particles running, the tick's device ms and wall ms, repacked after it
    trace: list = field(default_factory=list)

    def latencies(self):
        return np.array([j.finish - j.arrival for j in self.completed])


class Server:
    def __init__(self, hbm_budget_bytes: float = 120e9, tick_steps: int = 50, max_systems: int = 512,
                 device: int = 0, keep_results: bool = False, clock=time.perf_counter, log=None,
                 pipeline: bool = True):
        """log: a writable text stream; every finished (or rejected) job adds
        one JSON line to it (Job.record).  pipeline: build the next batch on
        a worker thread while the GPU runs the current tick."""
        self.budget = float(hbm_budget_bytes)
        self.tick = int(tick_steps)
        self.max_systems = int(max_systems)
        self.device = device
        self.keep_results = keep_results
        self.clock = clock
        self.waiting: deque[Job] = deque()
        self.running: list[Job] = []
        self.batch: L.Batch | None = None
        self.stats = ServerStats()
        self.log = log
        self.pool = ThreadPoolExecutor(max_workers=1) if pipeline else None
        self._t0 = 0.0

    def _complete(self, job: Job) -> None:
        self.stats.completed.append(job)
        if self.log is not None:
            self.log.write(json.dumps(job.record()) + "\n")

    # -- admission --------------------------------------------------------
    def submit(self, job: Job) -> None:
        self.waiting.append(job)

    def _desc(self, job: Job):
        return L.desc_from_spec(job.spec, job.state.dip.shape[1])

    def _fits(self, jobs) -> bool:
        if len(jobs) > self.max_systems:
            return False
        for j in jobs:
            if j.nbytes is None:
                j.nbytes = L.estimate_bytes([self._desc(j)])
        need = sum(j.nbytes for j in jobs)
        if any(getattr(j.spec, "cl_energy", 0.0) > 0 for j in jobs):
            need += 260 * sum(j.n for j in jobs)  # the energy criterion's candidate lists (mdsc_set_cluster_energy)
        return need <= self.budget

    def _admit(self, keep: list[Job], now: float) -> list[Job]:
        """Waiting jobs (arrived by now) that fit beside `keep`, in arrival order."""
        new = []
        while self.waiting and self.waiting[0].arrival <= now:
            head = self.waiting[0]
            if self._fits(keep + new + [head]):
                head.start = now
                new.append(self.waiting.popleft())
            elif not keep and not new:
                # larger than the whole budget on its own: it can never run
                head.finish = now
                head.obs = {"status": "rejected: exceeds the HBM budget"}
                self._complete(self.waiting.popleft())
            else:
                break
        return new

    # -- batches ------------------------------------------------------------
    def _build(self, members: list[Job], fresh: list[Job]) -> L.Batch:
        """A batch for `members`; the fresh ones uploaded with their step
        limits (the others arrive by transfer).  Runs on the worker thread."""
        ids = {id(j) for j in fresh}
        nb = L.Batch([j.spec for j in members], None, device=self.device, descs=[self._desc(j) for j in members])
        for k, j in enumerate(members):
            if id(j) in ids:
                nb.upload(k, j.state)
                nb.set_step_limit(k, j.steps)
        return nb

    def _switch(self, nb: L.Batch | None, members: list[Job]) -> None:
        """Move the running members into nb on the GPU, retire the old batch."""
        old, old_index = self.batch, {id(j): k for k, j in enumerate(self.running)}
        if nb is not None and old is not None:
            pairs = [(k, old_index[id(j)]) for k, j in enumerate(members) if id(j) in old_index]
            if pairs:
                nb.transfer_many(old, pairs)
        if old is not None:
            old.close()
        self.batch, self.running = nb, (members if nb is not None else [])
        self.stats.repacks += 1

    # -- one tick -----------------------------------------------------------
    def _finish(self, jobs: list[Job], now: float) -> None:
        slot = {id(j): k for k, j in enumerate(self.running)}
        for j in jobs:
            if self.keep_results and self.batch is not None:
                j.result = self.batch.download(slot[id(j)])
            j.finish = now
            self._complete(j)

    def tick_once(self) -> bool:
        """Plan, advance, retire, switch.  Returns False when nothing runs."""
        now = self.clock()
        if self.batch is None:
            new = self._admit([], now)
            if not new:
                return False
            self._switch(self._build(new, new), new)
        # the plan for after this tick: who keeps running, who joins
        keep = [j for j in self.running if j.done + self.tick < j.steps and not j.error]
        new = self._admit(keep, now)
        change = bool(new) or len(keep) != len(self.running)
        members = keep + new
        fut = None
        if change and members and self.pool is not None:
            fut = self.pool.submit(self._build, members, new)
        # the tick
        t_wall = self.clock()
        arr = (L.Observables * len(self.running))()
        code = self.batch.lib.mdsc_step(self.batch.h, self.tick, arr)
        dev_ms = self.batch.lib.mdsc_last_device_ms(self.batch.h)
        failed = []
        if code != 0:
            # a system's own error fails its job only; anything else is the server's
            bad = [k for k, o in enumerate(arr) if o.status != 0]
            if not bad:
                if fut is not None:
                    fut.result().close()
                raise L.MdscError(code, "mdsc_step", self.batch._err())
            for k in bad:
                self.running[k].error = L.STATUS.get(arr[k].status, str(arr[k].status))
                failed.append(self.running[k])
        steps_taken = 0
        for j, o in zip(self.running, arr):
            steps_taken += (int(o.step) - j.done) * j.n
            j.done = int(o.step)
            if j.done >= j.steps or j.error:
                j.obs = o.as_dict()  # a finished job's last observables
        self.stats.gpu_ms += dev_ms
        self.stats.ticks += 1
        self.stats.particle_steps += steps_taken
        self.stats.max_running = max(self.stats.max_running, len(self.running))
        now = self.clock()
        self._finish([j for j in self.running if j.done >= j.steps or j.error], now)
        if failed:
            # a job failed within the tick: plan again without it
            if fut is not None:
                fut.result().close()
                fut = None
            members = [j for j in members if not j.error]
            change = True
        if change:
            if fut is not None:
                nb = fut.result()
            else:
                running = {id(j) for j in self.running}
                fresh = [j for j in members if id(j) not in running]
                nb = self._build(members, fresh) if members else None
            self._switch(nb, members)
        self.stats.trace.append((round(now - self._t0, 4), len(self.waiting), len(self.running),
                                 sum(j.n for j in self.running), round(dev_ms, 3),
                                 round(1e3 * (now - t_wall), 3), int(change)))
        return True

    def run(self, jobs: list[Job], t0: float | None = None) -> ServerStats:
        """Serve jobs whose `arrival` times are seconds after t0 (now by
        default); returns when every job has completed."""
        t0 = self.clock() if t0 is None else t0
        self._t0 = t0
        pending = deque(sorted(jobs, key=lambda j: j.arrival))
        for j in pending:
            j.arrival += t0
        total = len(pending)
        while len(self.stats.completed) < total:
            now = self.clock()
            while pending and pending[0].arrival <= now:
                self.submit(pending.popleft())
            busy = self.tick_once()
            if not busy and not self.waiting and pending:
                time.sleep(max(0.0, min(0.01, pending[0].arrival - self.clock())))
        if self.batch is not None:
            self.batch.close()
            self.batch = None
        if self.pool is not None:
            self.pool.shutdown(wait=True)
        return self.stats


def poisson_arrivals(n_jobs: int, rate: float, seed: int) -> np.ndarray:
    """Arrival times (s) of a Poisson stream of rate `rate` per second."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, n_jobs))


def summarize(stats: ServerStats, wall_s: float, jobs: list[Job] | None = None) -> dict:
    lat = stats.latencies()
    out = {
        "jobs": len(stats.completed),
        "failed": sum(1 for j in stats.completed if j.error),
        "p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
        "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
        "mean_latency_s": float(lat.mean()) if len(lat) else None,
        "particle_steps_per_s": stats.particle_steps / wall_s if wall_s > 0 else None,
        "particle_steps": stats.particle_steps,
        "wall_s": wall_s,
        "gpu_busy_s": stats.gpu_ms / 1e3,
        "gpu_busy_frac": stats.gpu_ms / 1e3 / wall_s if wall_s > 0 else None,
        "ticks": stats.ticks,
        "repacks": stats.repacks,
        "max_running": stats.max_running,
    }
    if jobs:
        arr = np.array([j.arrival for j in jobs])
        span = float(arr.max() - arr.min()) if len(arr) > 1 else 0.0
        work = float(sum(j.n * j.steps for j in jobs))
        waits = np.array([j.start - j.arrival for j in jobs if j.start is not None])
        out["offered_particle_steps_per_s"] = work / span if span > 0 else None
        out["arrival_span_s"] = span
        out["p50_queue_wait_s"] = float(np.percentile(waits, 50)) if len(waits) else None
        out["p99_queue_wait_s"] = float(np.percentile(waits, 99)) if len(waits) else None
    if stats.trace:
        tr = np.array(stats.trace, dtype=np.float64)
        out["queue"] = {"max_waiting": int(tr[:, 1].max()), "max_running": int(tr[:, 2].max()),
                        "mean_running_particles": float(tr[:, 3].mean())}
        # ticks: the GPU's time and the host's, and what a repack added
        out["tick"] = {"mean_device_ms": float(tr[:, 4].mean()), "mean_wall_ms": float(tr[:, 5].mean()),
                       "mean_wall_ms_with_repack": float(tr[tr[:, 6] == 1, 5].mean()) if (tr[:, 6] == 1).any()
                       else None,
                       "mean_wall_ms_without": float(tr[tr[:, 6] == 0, 5].mean()) if (tr[:, 6] == 0).any() else None}
        # the queue over time: (seconds, waiting, running, running particles)
        # about every 5 s
        pts, nxt = [], 0.0
        for row in stats.trace:
            if row[0] >= nxt:
                pts.append([round(row[0], 2), int(row[1]), int(row[2]), int(row[3])])
                nxt = row[0] + 5.0
        out["queue_over_time"] = pts
    return out
