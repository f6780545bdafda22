"""Continuous batching: jobs arriving while others run are admitted as
slots free up, moved between batches on the GPU, and every job's result is
bit-identical to the same job run alone."""
import time

import numpy as np
import pytest

from mdspherocyl_gb300 import lib as L
from mdspherocyl_gb300 import serve
from mdspherocyl_gb300 import systems as S

pytestmark = pytest.mark.gpu


def _jobs():
    rs = np.random.default_rng(5)
    jobs = []
    for k, (n, steps) in enumerate(((70, 33), (150, 57), (96, 21), (260, 44), (64, 70), (120, 12))):
        st, box = S.make_system(n=n, phi=float(rs.uniform(0.05, 0.2)), lengths=np.clip(rs.normal(3, 0.3, n), 2, 4),
                                mu=np.full(n, float(rs.uniform(0.7, 2.0))), seed=200 + k, temp=1.1)
        spec = S.SystemSpec(n=n, box=box, alpha=6.0 / box[0], K_max=7, ksq_max=36, temp=1.1,
                            gamma=0.7 if k % 2 else 0.0, cl_fr=10 if k == 1 else 0,
                            B=np.array([0.0, 0.1 * k, 0.0]))
        jobs.append(serve.Job(k, spec, st, steps, arrival=0.01 * k))
    return jobs


def test_each_job_alone_equals_in_the_mix():
    alone = {}
    for j in _jobs():
        with L.Batch([j.spec], [j.state]) as bt:
            bt.step(j.steps)
            alone[j.jid] = bt.download(0)
    srv = serve.Server(tick_steps=9, keep_results=True)
    stats = srv.run(_jobs())
    assert len(stats.completed) == 6
    assert stats.repacks >= 3
    for j in stats.completed:
        assert j.done == j.steps
        for f in ("r", "p", "O", "l", "F", "T", "clust"):
            assert np.array_equal(j.result[f], alone[j.jid][f]), (j.jid, f)


def test_budget_admission_serialises_jobs():
    import io
    import json

    jobs = _jobs()[:3]
    one = max(L.estimate_bytes([L.desc_from_spec(j.spec, 1)]) for j in jobs)
    log = io.StringIO()
    srv = serve.Server(hbm_budget_bytes=one * 1.01, tick_steps=10, log=log)
    stats = srv.run(jobs)
    assert len(stats.completed) == 3 and stats.max_running == 1
    lat = stats.latencies()
    assert np.all(lat > 0)
    # one JSON line per job: its size, steps, times and error
    recs = [json.loads(x) for x in log.getvalue().splitlines()]
    assert sorted(r["job"] for r in recs) == [j.jid for j in jobs]
    for r in recs:
        assert r["done"] == r["steps"] and r["error"] is None and r["finish"] >= r["start"] >= r["arrival"]


def test_a_failing_job_leaves_alone():
    """One job starts with two rods on top of each other: the reference's
    overlap abort fails that job (status MDSC_ERR_OVERLAP); every other job
    finishes with the bits it has alone."""
    jobs = _jobs()
    bad = jobs[2]
    bad.state = bad.state.copy()
    bad.state.r[1] = bad.state.r[0] + np.array([0.05, 0.0, 0.0])
    bad.state.O[1] = bad.state.O[0]
    alone = {}
    for j in _jobs():
        if j.jid == bad.jid:
            continue
        with L.Batch([j.spec], [j.state]) as bt:
            bt.step(j.steps)
            alone[j.jid] = bt.download(0)
    srv = serve.Server(tick_steps=9, keep_results=True)
    stats = srv.run(jobs)
    assert len(stats.completed) == 6
    failed = [j for j in stats.completed if j.error]
    assert [j.jid for j in failed] == [bad.jid] and failed[0].error == "MDSC_ERR_OVERLAP"
    for j in stats.completed:
        if j.jid == bad.jid:
            continue
        assert j.done == j.steps and j.error is None
        for f in ("r", "p", "O", "l", "F", "T", "clust"):
            assert np.array_equal(j.result[f], alone[j.jid][f]), (j.jid, f)
    assert serve.summarize(stats, 1.0)["failed"] == 1


def test_cutoff_and_energy_cluster_jobs_as_alone():
    """Jobs with a real-space cutoff and jobs clustered by pair energy, beside
    plain ones, moved between batches as the server repacks: each ends with
    the bits (and the cluster labels) it has alone."""
    rs = np.random.default_rng(9)
    jobs = []
    for k, (n, steps, rc, ce, fr) in enumerate(((300, 31, 4.0, 1.2, 5), (200, 40, 0.0, 0.0, 0), (260, 27, 0.0, 1.5, 7),
                                                (150, 35, 3.0, 0.0, 0), (120, 22, 0.0, 0.0, 4))):
        st, box = S.make_system(n=n, phi=float(rs.uniform(0.1, 0.25)), lengths=rs.uniform(2, 3.5, n),
                                mu=np.full(n, float(rs.uniform(1.5, 2.5))), seed=300 + k, temp=1.0)
        spec = S.SystemSpec(n=n, box=box, alpha=7.0 / box[0], K_max=6, ksq_max=0, rc_real=rc, cl_energy=ce, cl_fr=fr)
        jobs.append(serve.Job(k, spec, st, steps, arrival=0.01 * k))
    alone = {}
    for j in jobs:
        with L.Batch([j.spec], [j.state]) as bt:
            bt.step(j.steps)
            alone[j.jid] = bt.download(0)
    srv = serve.Server(tick_steps=9, keep_results=True)
    stats = srv.run(jobs)
    assert len(stats.completed) == 5 and stats.repacks >= 3
    for j in stats.completed:
        assert j.done == j.steps and j.error is None
        for f in ("r", "p", "O", "l", "F", "T", "clust"):
            assert np.array_equal(j.result[f], alone[j.jid][f]), (j.jid, f)


def test_step_limits_stop_systems_exactly():
    """mdsc_set_step_limit: in one batch stepped 20 steps, systems limited
    to 5 and 12 steps stop there (their step counts, states and observables
    those of 5 and 12 steps alone, bit for bit) while the third takes all 20;
    the limited ones cost no steps afterwards."""
    jobs = _jobs()[:3]
    limits = (5, 12, 0)
    alone = []
    for j, lim in zip(jobs, limits):
        with L.Batch([j.spec], [j.state]) as bt:
            o = bt.step(lim or 20)[0]
            alone.append((o, bt.download(0)))
    with L.Batch([j.spec for j in jobs], [j.state for j in jobs]) as bt:
        for k, lim in enumerate(limits):
            bt.set_step_limit(k, lim)
        obs = bt.step(20)
        for k, lim in enumerate(limits):
            assert obs[k]["step"] == (lim or 20)
            d = bt.download(k)
            for f in ("r", "p", "O", "l", "F", "T"):
                assert np.array_equal(d[f], alone[k][1][f]), (k, f)
            for key in ("U_dipR", "U_dipK", "U_ss", "K", "xi"):
                assert np.array_equal(np.asarray(obs[k][key]), np.asarray(alone[k][0][key])), (k, key)
