"""Autotuner (mdsc_autotune / mdsc_set_tuning): every launch mapping it can
choose gives bit-identical results, and a tuning run reports its timings
and picks from the candidate sets."""
import numpy as np
import pytest

from mdspherocyl_gb300 import lib as L
from mdspherocyl_gb300 import systems as S

pytestmark = pytest.mark.gpu

MAPPINGS = [  # (tiles per block, strip-sum threads, WCA evaluation blocks, gather form)
    (1, 256, 152 * 8, 0),
    (4, 512, 152 * 2, 1),
    (2, 128, 152 * 16, 1),
    (4, 128, 152, 0),
]


def _mix():
    rs = np.random.default_rng(5)
    out = []
    for k, n in enumerate((90, 260, 180)):
        st, box = S.make_system(n=n, phi=float(rs.uniform(0.08, 0.2)), lengths=rs.uniform(2, 4, n),
                                mu=np.full(n, 1.4), seed=300 + k, temp=1.1)
        spec = S.SystemSpec(n=n, box=box, alpha=6.0 / box[0], K_max=7, ksq_max=36, temp=1.1,
                            gamma=0.5 * (k % 2))
        out.append((spec, st))
    return out


def test_every_mapping_gives_the_same_bits():
    systems = _mix()
    ref = None
    for m in MAPPINGS:
        with L.Batch([s for s, _ in systems], [t for _, t in systems]) as bt:
            bt.set_tuning(*m)
            obs = bt.step(10)
            got = ([bt.download(k) for k in range(len(systems))], obs)
            assert bt.tuning()["rp_warps"] == m[0]
        if ref is None:
            ref = got
            continue
        for k in range(len(systems)):
            for f in ("r", "p", "O", "l", "F", "T"):
                assert np.array_equal(got[0][k][f], ref[0][k][f]), (m, k, f)
            for key in ("U_ss", "U_dipR", "U_dipK", "K", "PT_dipR", "PT_dipK", "PT_kin", "xi"):
                assert np.array_equal(np.asarray(got[1][k][key]), np.asarray(ref[1][k][key])), (m, k, key)


def test_autotune_picks_from_the_candidates():
    systems = _mix()
    with L.Batch([s for s, _ in systems], [t for _, t in systems]) as bt:
        t = bt.autotune(force=True)
        assert t["tuned"]
        assert t["rp_warps"] in (1, 2, 4)
        assert t["rsum_threads"] in (128, 256, 512)
        assert t["wca_blocks"] in (152 * 2, 152 * 4, 152 * 8, 152 * 16)
        assert t["kg_scalar"] in (0, 1)
        for name in ("rp_warps=", "rsum_threads=", "wca_blocks=", "kg_scalar="):
            assert name in t["log"]
        obs = bt.step(3)
        assert all(o["status"] == 0 for o in obs)


def test_set_tuning_rejects_bad_values():
    systems = _mix()[:1]
    with L.Batch([s for s, _ in systems], [t for _, t in systems]) as bt:
        with pytest.raises(Exception):
            bt.set_tuning(3, 256, 1216, 0)
