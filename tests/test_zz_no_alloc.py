"""mdsc_force_dipR_noalloc: the real-space Ewald forces for callers that
cannot allocate GPU memory (a host with a fixed device-memory budget, a
real-time loop, a plugin whose host owns every buffer).  Its results must
match the regular entry point, mdsc_force_dipR, on two calls in a row --
the second call reuses the fixed scratch array the first one left behind.

This file is collected last so that a run which stops at the first failure
has already run every other test."""
import ctypes

import numpy as np
import pytest

from conftest import rms_rel
from mdspherocyl_gb300 import lib as L
from mdspherocyl_gb300 import systems as S

pytestmark = pytest.mark.gpu

TOL_F = 1e-5  # the tolerance the other GPU tests hold the Ewald forces to


def _regular(spec, st):
    """The regular entry point's answer (mdsc_force_dipR on its own batch)."""
    with L.Batch([spec], [st]) as bt:
        bt.zero_forces()
        U_ref, PT_ref = bt.force_dipR()
        ref = bt.download(0)
    return ref["F"], ref["T"], U_ref[0], PT_ref[0]


def test_noalloc_matches_force_dipR_on_two_calls():
    """Two calls in a row on different systems: first the largest the fixed
    scratch holds (4096 dipoles, 64 strips, 2080 tiles: every byte of the
    array in use), then a smaller one with other positions, moments and box.
    A second call that read partials, energies or tiles the first left
    behind would differ from its own regular answer."""
    import torch

    lib = L.load()
    cases = [S.plain_c0(seed=9, n=4096), S.plain_c0(seed=21, n=700)]
    assert cases[0][1].n == 4096 and not np.allclose(cases[0][0].box, cases[1][0].box)
    refs = [_regular(spec, st) for spec, st in cases]
    dev = torch.device("cuda:0")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for (spec, st), (F_ref, T_ref, U_ref, PT_ref) in zip(cases, refs):
        n = st.n
        pos = torch.tensor(st.r, dtype=torch.float64, device=dev)
        mom = torch.tensor(st.dip[:, 0, 4:5] * st.O[:, 2, :], dtype=torch.float64, device=dev)
        F = torch.full((n, 3), float("nan"), dtype=torch.float64, device=dev)
        T = torch.full((n, 3), float("nan"), dtype=torch.float64, device=dev)
        UPT = torch.full((10,), float("nan"), dtype=torch.float64, device=dev)
        box = (ctypes.c_double * 3)(*[float(x) for x in spec.box])
        code = lib.mdsc_force_dipR_noalloc(n, ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(mom.data_ptr()),
                                           ctypes.cast(box, ctypes.POINTER(ctypes.c_double)), float(spec.alpha),
                                           ctypes.c_void_p(F.data_ptr()), ctypes.c_void_p(T.data_ptr()),
                                           ctypes.c_void_p(UPT.data_ptr()), stream)
        torch.cuda.synchronize()
        assert code == 0, L.STATUS.get(code, code)
        f, t, upt = F.cpu().numpy(), T.cpu().numpy(), UPT.cpu().numpy()
        assert rms_rel(f, F_ref) < TOL_F, (n, rms_rel(f, F_ref))
        assert rms_rel(t, T_ref) < TOL_F, (n, rms_rel(t, T_ref))
        assert abs(upt[0] - U_ref) < TOL_F * max(1.0, abs(U_ref)), (n, upt[0], U_ref)
        assert rms_rel(upt[1:].reshape(3, 3), PT_ref) < TOL_F, n


def test_noalloc_rejects_more_dipoles_than_its_scratch_holds():
    lib = L.load()
    box = (ctypes.c_double * 3)(20.0, 20.0, 20.0)
    one = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    code = lib.mdsc_force_dipR_noalloc(4097, one, one, ctypes.cast(box, ctypes.POINTER(ctypes.c_double)), 0.5,
                                       one, one, one, None)
    assert L.STATUS[code] == "MDSC_ERR_TOO_LARGE"
