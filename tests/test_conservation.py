"""The conserved quantity of the reference's Nose-Hoover integrator, which
the reference itself does not compute: with a deterministic thermostat
(gamma = 0),

    H = K_t + K_r + U + Q (xi_t^2 + xi_r^2) / 2 + 3 N T (eta_t + eta_r),
    eta = integral of xi dt   (trapezoid over the per-step xi),

stays put while K and U exchange energy.  Checked on the oracle's
restatement of the driver step (CPU) and on the GPU step's per-step trace
(mdsc_step_trace): H moves by a small fraction of the kinetic energy's own
fluctuation."""
import numpy as np
import pytest

import oracle
from mdspherocyl_gb300 import systems as S


def _H(K, U, xi, eta, Q, n, T):
    return K + U + 0.5 * Q * (xi ** 2).sum() + 3 * n * T * eta.sum()


def test_oracle_step_conserves_H():
    spec, st = S.plain_c0(seed=3, n=48)
    orc = oracle.Oracle()
    o = oracle.System(st.r, st.p, st.O, st.l, st.length, st.dia, st.mass, st.dip, spec.box)
    dt, T, Q = 1e-3, 1.0, 1.0
    md = oracle.MDOracle(orc, o, dt=dt, temp=T, Q=Q, gamma=0.0, xi0=0.0, sr_cut=3.0, K_max=spec.K_max,
                         ksq_max=spec.ksq_max, alpha=spec.alpha, B=np.zeros(3))
    eta, xprev = np.zeros(2), np.zeros(2)
    H, K = [], []
    for _ in range(800):
        assert md.step()
        ob = md.obs()
        eta += 0.5 * dt * (xprev + ob["xi"])
        xprev = ob["xi"].copy()
        U = ob["Uss"] + ob["UdipR"] + ob["UdipK"] + ob["Uext"] + ob["Uself"]
        K.append(ob["K"].sum())
        H.append(_H(K[-1], U, ob["xi"], eta, Q, 48, T))
    H, K = np.array(H), np.array(K)
    assert np.ptp(H) < 2e-3 * K.std()


@pytest.mark.gpu
def test_gpu_step_conserves_H():
    from mdspherocyl_gb300 import lib as L

    spec, st = S.plain_c0(seed=4, n=256)
    spec.gamma, spec.Q = 0.0, 1.0
    dt, T, Q, n = spec.dt, spec.temp, spec.Q, 256
    with L.Batch([spec], [st]) as bt:
        trace = bt.step_trace(3000)
    eta, xprev = np.zeros(2), np.zeros(2)
    H, K = [], []
    for ob in trace:
        o = ob[0]
        xi = np.array(o["xi"])
        eta += 0.5 * dt * (xprev + xi)
        xprev = xi
        U = o["U_ss"] + o["U_dipR"] + o["U_dipK"] + o["U_ext"] + o["U_self"]
        K.append(sum(o["K"]))
        H.append(_H(K[-1], U, xi, eta, Q, n, T))
    H, K = np.array(H), np.array(K)
    assert np.ptp(H) < 2e-3 * K.std(), (np.ptp(H), K.std())
