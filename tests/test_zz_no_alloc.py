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


def test_noalloc_matches_force_dipR_on_two_calls():
    import torch

    lib = L.load()
    spec, st = S.plain_c0(seed=9, n=300)
    with L.Batch([spec], [st]) as bt:
        bt.zero_forces()
        U_ref, PT_ref = bt.force_dipR()
        ref = bt.download(0)
    n = st.n
    dev = torch.device("cuda:0")
    pos = torch.tensor(st.r, dtype=torch.float64, device=dev)
    mom = torch.tensor(st.dip[:, 0, 4:5] * st.O[:, 2, :], dtype=torch.float64, device=dev)
    F = torch.empty((n, 3), dtype=torch.float64, device=dev)
    T = torch.empty((n, 3), dtype=torch.float64, device=dev)
    UPT = torch.empty(10, dtype=torch.float64, device=dev)
    box = (ctypes.c_double * 3)(*[float(x) for x in spec.box])
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        F.fill_(float("nan"))
        T.fill_(float("nan"))
        UPT.fill_(float("nan"))
        code = lib.mdsc_force_dipR_noalloc(n, ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(mom.data_ptr()),
                                           ctypes.cast(box, ctypes.POINTER(ctypes.c_double)), float(spec.alpha),
                                           ctypes.c_void_p(F.data_ptr()), ctypes.c_void_p(T.data_ptr()),
                                           ctypes.c_void_p(UPT.data_ptr()), stream)
        torch.cuda.synchronize()
        assert code == 0, L.STATUS.get(code, code)
        f, t, upt = F.cpu().numpy(), T.cpu().numpy(), UPT.cpu().numpy()
        assert rms_rel(f, ref["F"]) < TOL_F
        assert rms_rel(t, ref["T"]) < TOL_F
        assert abs(upt[0] - U_ref[0]) < TOL_F * max(1.0, abs(U_ref[0]))
        assert rms_rel(upt[1:].reshape(3, 3), PT_ref[0]) < TOL_F


def test_noalloc_rejects_more_dipoles_than_its_scratch_holds():
    lib = L.load()
    box = (ctypes.c_double * 3)(20.0, 20.0, 20.0)
    one = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    code = lib.mdsc_force_dipR_noalloc(4097, one, one, ctypes.cast(box, ctypes.POINTER(ctypes.c_double)), 0.5,
                                       one, one, one, None)
    assert L.STATUS[code] == "MDSC_ERR_TOO_LARGE"
