"""The fixed per-rod capacities (64 Verlet-list partners, 16 WCA contact
candidates of higher index, 256 neighbour-pass entries) hold over the
densest systems the workloads draw, and a system beyond them is reported
(MDSC_ERR_LIST_OVERFLOW) instead of computed with a list cut short."""
import numpy as np
import pytest

from mdspherocyl_gb300 import lib as L
from mdspherocyl_gb300 import systems as S

pytestmark = pytest.mark.gpu


def test_densest_workload_systems_stay_within_the_caps():
    rs = np.random.default_rng(77)
    systems = []
    # the mix's densest corner (phi 0.25, short and long rods), config 1's
    # (phi 0.20, lengths up to 5), a serving job's (phi 0.25, L ~ N(3, 0.3)),
    # and config 1 with its 3.5 real-space cutoff
    for k, (n, phi, lo, hi, rc) in enumerate(((2048, 0.25, 2.0, 4.0, 0.0), (4096, 0.20, 2.0, 5.0, 0.0),
                                              (3000, 0.25, 2.4, 3.6, 0.0), (4096, 0.20, 2.0, 5.0, 3.5))):
        st, box = S.make_system(n=n, phi=phi, lengths=rs.uniform(lo, hi, n), mu=np.full(n, 1.5), seed=900 + k)
        spec = S.SystemSpec(n=n, box=box, alpha=7.0 / box[0], K_max=5, ksq_max=16, rc_real=rc)
        systems.append((spec, st))
    with L.Batch([s for s, _ in systems], [t for _, t in systems]) as bt:
        obs = bt.step(30)
    assert all(o["status"] == 0 for o in obs)


def test_a_list_beyond_its_capacity_is_reported():
    """Parallel rods of length 2 on a tight lattice (packing fraction 0.6)
    with a proximity distance of 2 for the clusters: the Verlet-list radius
    then holds well over 64 partners per rod."""
    nx, ny, nz = 8, 8, 4
    dx, dz = 1.05, 3.1
    r = np.array([[(i + 0.5) * dx, (j + 0.5) * dx, (k + 0.5) * dz] for k in range(nz) for j in range(ny)
                  for i in range(nx)])
    n = len(r)
    box = np.array([nx * dx, ny * dx, nz * dz])
    O = np.stack([np.eye(3)] * n)
    dip = np.zeros((n, 1, 5))
    dip[:, 0, 3] = 1.0
    dip[:, 0, 4] = 1.0
    st = S.SystemState(r, np.zeros((n, 3)), O, np.zeros((n, 3)), np.full(n, 2.0), np.ones(n), np.ones(n), dip)
    spec = S.SystemSpec(n=n, box=box, alpha=6.0 / box.min(), K_max=4, ksq_max=0, min_s=2.0)
    with L.Batch([spec], [st]) as bt:
        with pytest.raises(L.MdscError) as e:
            bt.step(1)
        assert L.STATUS[e.value.code] == "MDSC_ERR_LIST_OVERFLOW"
