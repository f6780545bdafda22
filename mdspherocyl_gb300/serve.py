"""Continuous-batching job server for the GB300 MD step.

Jobs (one system each, with a number of steps) arrive over time.  The
server keeps every running system resident on the GPU in one batch, advances
the whole batch by a tick of steps with one CUDA-graph launch per step, and
at every tick boundary retires finished jobs and admits waiting ones as
slots and memory allow.  When the membership changes it builds a new batch
and moves the running systems into it on the GPU (mdsc_transfer), so no
running state returns to the host.  Admission is by an HBM budget:
mdsc_estimate_bytes of the would-be batch must fit it.

A job's result is independent of the jobs it shares the GPU with: every
kernel works per system and sums in a fixed order, so a system gives the
same bits alone and in any mix (tests/test_serve.py).  A system that reports
an error (the reference's overlap abort, a NaN, a full list) fails its own
job, which leaves at the next tick; the others run on undisturbed.
"""
from __future__ import annotations

import json
import time
from collections import deque
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

    def latencies(self):
        return np.array([j.finish - j.arrival for j in self.completed])


class Server:
    def __init__(self, hbm_budget_bytes: float = 120e9, tick_steps: int = 50, max_systems: int = 512,
                 device: int = 0, keep_results: bool = False, clock=time.perf_counter, log=None):
        """log: a writable text stream; every finished (or rejected) job adds
        one JSON line to it (Job.record)."""
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
        need = L.estimate_bytes([self._desc(j) for j in jobs])
        if any(getattr(j.spec, "cl_energy", 0.0) > 0 for j in jobs):
            need += 260 * sum(j.n for j in jobs)  # the energy criterion's candidate lists (mdsc_set_cluster_energy)
        return need <= self.budget

    # -- one tick -----------------------------------------------------------
    def _repack(self, keep: list[Job], new: list[Job]) -> None:
        members = keep + new
        old, old_index = self.batch, {id(j): k for k, j in enumerate(self.running)}
        if not members:
            if old is not None:
                old.close()
            self.batch, self.running = None, []
            return
        descs = [self._desc(j) for j in members]
        nb = L.Batch([j.spec for j in members], None, device=self.device, descs=descs)
        for k, j in enumerate(members):
            if id(j) in old_index:
                nb.transfer_from(k, old, old_index[id(j)])
            else:
                nb.upload(k, j.state)
        if old is not None:
            old.close()
        self.batch, self.running = nb, members
        self.stats.repacks += 1

    def tick_once(self) -> bool:
        """Retire, admit, advance.  Returns False when nothing is running."""
        now = self.clock()
        finished = [j for j in self.running if j.done >= j.steps or j.error]
        keep = [j for j in self.running if j.done < j.steps and not j.error]
        for j in finished:
            k = self.running.index(j)
            if self.keep_results:
                j.result = self.batch.download(k)
            j.finish = now
            self._complete(j)
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
        if finished or new:
            self._repack(keep, new)
        if not self.running:
            return False
        steps = min(self.tick, min(j.steps - j.done for j in self.running))
        arr = (L.Observables * len(self.running))()
        code = self.batch.lib.mdsc_step(self.batch.h, steps, arr)
        obs = [o.as_dict() for o in arr]
        if code != 0:
            # a system's own error fails its job only; anything else is the server's
            bad = [k for k, o in enumerate(obs) if o["status"] != 0]
            if not bad:
                raise L.MdscError(code, "mdsc_step", self.batch._err())
            for k in bad:
                self.running[k].error = L.STATUS.get(obs[k]["status"], str(obs[k]["status"]))
        self.stats.gpu_ms += self.batch.lib.mdsc_last_device_ms(self.batch.h)
        for j, o in zip(self.running, obs):
            j.done += steps
            j.obs = o
        self.stats.ticks += 1
        self.stats.particle_steps += steps * sum(j.n for j in self.running)
        self.stats.max_running = max(self.stats.max_running, len(self.running))
        return True

    def run(self, jobs: list[Job], t0: float | None = None) -> ServerStats:
        """Serve jobs whose `arrival` times are seconds after t0 (now by
        default); returns when every job has completed."""
        t0 = self.clock() if t0 is None else t0
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
        return self.stats


def poisson_arrivals(n_jobs: int, rate: float, seed: int) -> np.ndarray:
    """Arrival times (s) of a Poisson stream of rate `rate` per second."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, n_jobs))


def summarize(stats: ServerStats, wall_s: float) -> dict:
    lat = stats.latencies()
    return {
        "jobs": len(stats.completed),
        "failed": sum(1 for j in stats.completed if j.error),
        "p50_latency_s": float(np.percentile(lat, 50)) if len(lat) else None,
        "p99_latency_s": float(np.percentile(lat, 99)) if len(lat) else None,
        "mean_latency_s": float(lat.mean()) if len(lat) else None,
        "particle_steps_per_s": stats.particle_steps / wall_s if wall_s > 0 else None,
        "particle_steps": stats.particle_steps,
        "wall_s": wall_s,
        "gpu_busy_s": stats.gpu_ms / 1e3,
        "ticks": stats.ticks,
        "repacks": stats.repacks,
        "max_running": stats.max_running,
    }
