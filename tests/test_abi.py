"""The C ABI without a GPU: the library builds, loads and exports every
entry point include/mdsc.h declares; host-side routines behave."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle
from conftest import ROOT
from mdspherocyl_gb300 import build as B
from mdspherocyl_gb300 import lib as L
from mdspherocyl_gb300 import systems as S


def declared_entry_points():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(mdsc_[A-Za-z_0-9]+)\s*\(", src))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    path = B.build()
    lib = ctypes.CDLL(path)
    names = declared_entry_points()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(L.EXPORTS)


def test_ctypes_structures_match_the_library():
    """The Python layouts of mdsc_system_desc, mdsc_host_state,
    mdsc_observables and mdsc_view have the library's sizes."""
    lib = ctypes.CDLL(B.build())
    lib.mdsc_abi_sizes.restype = None
    sz = [ctypes.c_size_t(0) for _ in range(4)]
    lib.mdsc_abi_sizes(*[ctypes.byref(x) for x in sz])
    assert [x.value for x in sz] == [ctypes.sizeof(t) for t in (L.SystemDesc, L.HostState, L.Observables, L.View)]


def test_estimate_bytes_without_gpu():
    spec, st = S.plain_c0(seed=0, n=64)
    d = L.desc_from_spec(spec, 1)
    nb = L.estimate_bytes([d])
    assert nb > 64 * 200
    assert L.estimate_bytes([d, d]) > nb


def test_estimate_bytes_sum_of_jobs_bounds_the_batch():
    """The server admits against the sum of its jobs' own estimates: that sum
    must never be below the batch's estimate, and close to it."""
    jobs = [S.serving_job(k) for k in range(24)]
    descs = [L.desc_from_spec(spec, 1) for spec, _ in jobs]
    batch = L.estimate_bytes(descs)
    singles = sum(L.estimate_bytes([d]) for d in descs)
    assert batch <= singles <= 1.02 * batch


def test_estimate_bytes_counts_the_cutoff_lists_and_gather_parts():
    """The HBM a batch needs (what the server admits against) includes the
    real-space neighbour lists of a cutoff system (256 ints per rod) and the
    partial sums of a split k-space gather (N >= 4096, one dipole)."""
    spec, st = S.plain_c0(seed=0, n=512)
    d0 = L.desc_from_spec(spec, 1)
    spec.rc_real = 3.0
    d1 = L.desc_from_spec(spec, 1)
    b0, b1 = L.estimate_bytes([d0]), L.estimate_bytes([d1])
    # the lists (512 x 256 ints) less the all-pairs tiles' partials it drops (8 x 8 tiles x 6 x 64 floats)
    assert b1 - b0 >= 512 * 256 * 4 - 8 * 8 * 6 * 64 * 4 - 64 * 1024
    big, _ = S.plain_c1(seed=0, n=4096)
    d2 = L.desc_from_spec(big, 1)
    d3 = L.desc_from_spec(big, 1)
    d3.n = 4095  # below the split: one part per particle block
    # 32 particle blocks, at least 2 parts each, kPartBlock x 12 floats a part
    assert L.estimate_bytes([d2]) - L.estimate_bytes([d3]) >= 32 * 2 * 128 * 12 * 4


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="a GPU is visible")
def test_create_without_gpu_fails_cleanly():
    spec, st = S.plain_c0(seed=0, n=32)
    with pytest.raises(L.MdscError) as e:
        L.Batch([spec], [st])
    assert e.value.code in (2, 8)


def test_place_rods_non_overlapping_and_seeded(orc):
    rng = np.random.default_rng(1)
    n = 150
    ln = rng.uniform(2, 4, n)
    d = np.ones(n)
    box = np.full(3, ((np.pi * ln / 4 + np.pi / 6).sum() / 0.2) ** (1 / 3))
    r1, O1 = L.place_rods(ln, d, box, seed=5)
    r2, O2 = L.place_rods(ln, d, box, seed=5)
    assert np.array_equal(r1, r2) and np.array_equal(O1, O2)
    assert np.allclose(np.einsum("nij,nkj->nik", O1, O1), np.eye(3), atol=1e-12)
    assert np.allclose(np.linalg.det(O1), 1.0)
    s = oracle.System(r1, np.zeros((n, 3)), O1, np.zeros((n, 3)), ln, d, np.ones(n), np.zeros((n, 1, 5)), box)
    for i in range(n):
        for j in range(i + 1, n):
            dsq, _, _ = orc.seg_dist(s, i, j)
            assert dsq >= 1.0 - 1e-9, (i, j, dsq)


def test_generated_systems_follow_the_workload_spec():
    spec, st = S.plain_c0(seed=3)
    assert st.n == 256 and spec.ksq_max == 27 and spec.K_max == 6
    assert np.isclose(spec.alpha * spec.box[0], 5.6)
    vol = np.pi * st.length / 4 + np.pi / 6
    assert np.isclose(vol.sum() / np.prod(spec.box), 0.10)
    assert st.length.min() >= 2.0 and st.length.max() <= 4.0
    assert np.allclose(st.dip[:, 0, 4] ** 2, 2.0)
    assert np.abs(st.p.sum(0)).max() < 1e-10
    mix = S.replica_mix_specs()
    ns = np.array([d["n"] for d in mix])
    assert len(mix) == 256 and ns.min() >= 128 and ns.max() <= 2048


def test_k_half_space_equals_reference_cube():
    """The distinct +-k representatives with weight 2 Kvec/V (what the GPU
    path sums over) give the same sum as the reference's cube loop with its
    four sign patterns and 1/2, 1/4 weights (v25/functions.cpp:1725-1744,
    1845-1850) for any f with f(k) = f(-k)."""
    rng = np.random.default_rng(2)
    coef = rng.normal(size=6)

    def f(kx, ky, kz):  # even in k, otherwise arbitrary
        return np.cos(coef[0] * kx + coef[1] * ky + coef[2] * kz) + np.cos(coef[3] * kx - coef[4] * ky + coef[5] * kz)

    for K in (3, 5, 6):
        ref = 0.0
        for nz in range(K):
            for ny in range(K):
                for nx in range(K):
                    if nx == ny == nz == 0:
                        continue
                    s = sum(f(sx * nx, sy * ny, nz) for sx, sy in ((1, 1), (-1, 1), (1, -1), (-1, -1)))
                    if (nx == 0 and ny == 0) or (nx == 0 and nz == 0) or (ny == 0 and nz == 0):
                        s /= 4
                    elif (nz == 0 and nx != 0 and ny != 0) or (ny == 0 and nz != 0 and nx != 0) or \
                            (nx == 0 and ny != 0 and nz != 0):
                        s /= 2
                    ref += s
        ours = 0.0
        for nz in range(K):
            for ny in range(-(K - 1), K):
                for nx in range(-(K - 1), K):
                    if nz > 0 or (nz == 0 and ny > 0) or (nz == 0 and ny == 0 and nx > 0):
                        ours += f(nx, ny, nz)
        assert abs(ours - ref) < 1e-9 * max(1.0, abs(ref))


def test_gsl_generator_files_have_the_reference_layout():
    import refdriver

    assert len(refdriver.mt_state_bytes(1)) == 5000
