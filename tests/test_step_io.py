"""mdsc_step_io (state up, steps, state down in one call, the positions and
orientations downloaded while the last step's forces are computed) gives the
bits of mdsc_upload_all + mdsc_step + mdsc_download_all, with pageable and
with pinned host arrays, and with a system held at its step limit."""
import numpy as np
import pytest

from mdspherocyl_gb300 import lib as L
from mdspherocyl_gb300 import systems as S

pytestmark = pytest.mark.gpu


def _mix():
    rs = np.random.default_rng(4)
    out = []
    for k, n in enumerate((150, 330, 220, 90)):
        st, box = S.make_system(n=n, phi=float(rs.uniform(0.08, 0.2)), lengths=rs.uniform(2, 4, n),
                                mu=np.full(n, 1.3), seed=900 + k, temp=1.1)
        spec = S.SystemSpec(n=n, box=box, alpha=6.0 / box[0], K_max=7, ksq_max=36, temp=1.1,
                            gamma=0.5 * (k % 2))
        out.append((spec, st))
    return out


def _arrays(bt):
    n = sum(s.n for s, _ in _mix())
    h = {k: np.zeros((n, 3)) for k in "rplFT"}
    h["O"] = np.zeros((n, 3, 3))
    bt.download_all(h["r"], h["p"], h["O"], h["l"], h["F"], h["T"])
    return h


def _pinned_like(arrs):
    import torch

    out = {}
    for k, v in arrs.items():
        t = torch.empty(v.shape, dtype=torch.float64, pin_memory=True).numpy()
        t[...] = v
        out[k] = t
    return out


@pytest.mark.parametrize("nsteps", [1, 3])
@pytest.mark.parametrize("pinned", [False, True])
def test_step_io_equals_upload_step_download(nsteps, pinned):
    systems = _mix()
    specs, states = [s for s, _ in systems], [t for _, t in systems]
    with L.Batch(specs, states) as a, L.Batch(specs, states) as b:
        a.step(2)
        b.step(2)
        for bt in (a, b):  # one system stops inside the second call
            bt.set_step_limit(2, 2 + nsteps + 1)
        ha = _arrays(a)
        hb = {k: v.copy() for k, v in ha.items()}
        if pinned:
            hb = _pinned_like(hb)
        for _ in range(3):  # the host owns the state between calls
            a.upload_all(ha["r"], ha["p"], ha["O"], ha["l"], ha["F"], ha["T"])
            oa = a.step(nsteps)
            a.download_all(ha["r"], ha["p"], ha["O"], ha["l"], ha["F"], ha["T"])
            obs = (L.Observables * len(specs))()
            b.step_io(hb, nsteps, hb, obs)
            ob = [o.as_dict() for o in obs]
            for k in "rpOlFT":
                assert np.array_equal(ha[k], hb[k]), k
            for x, y in zip(oa, ob):
                for key in ("U_ss", "U_dipR", "U_dipK", "K", "step"):
                    assert np.array_equal(np.asarray(x[key]), np.asarray(y[key])), key


def test_step_io_without_state_or_steps():
    """nsteps = 0 moves the state only; no `in` steps the device state; no
    `out` leaves the host arrays alone."""
    systems = _mix()
    specs, states = [s for s, _ in systems], [t for _, t in systems]
    with L.Batch(specs, states) as a, L.Batch(specs, states) as b:
        a.step(2)
        b.step(2)
        h = _arrays(a)
        g = {k: np.full_like(v, np.nan) for k, v in h.items()}
        b.step_io(h, 0, g)  # up and down, no step
        for k in "rpOlFT":
            assert np.array_equal(g[k], h[k]), k
        a.step(3)
        b.step_io(None, 3, None)  # three steps of the device state
        b.step_io(None, 0, g)
        ref = _arrays(a)
        for k in "rpOlFT":
            assert np.array_equal(g[k], ref[k]), k
        keep = {k: v.copy() for k, v in g.items()}
        b.step_io(None, 1, None)  # no `out`: the host arrays are not written
        for k in "rpOlFT":
            assert np.array_equal(g[k], keep[k]), k
