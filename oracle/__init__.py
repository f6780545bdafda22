"""CPU oracle for the MD-step path -- TEST INFRASTRUCTURE ONLY.

Two implementations of the reference's FP64 routines live here:

* ``mdsc_oracle.c`` -- a plain-C restatement of the reference routines (each
  function cites the reference file:line it follows).  Built by
  :func:`build_oracle` into ``oracle/_build/libmdsc_oracle.so``.
* ``_ref/libmdsc_ref.so`` -- the reference's own, unmodified sources compiled
  by ``oracle/build_ref.sh`` around a thin harness (``ref_harness.cpp``).  It
  exists only where the reference sources are present; it pins the
  restatement.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may use this package, and only as the checker or as the timed
CPU baseline.  The GPU product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_int, c_ulong, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD, "libmdsc_oracle.so")
REF_SO = os.path.join(REF_DIR, "libmdsc_ref.so")
# the same sources without OpenMP, for systems below 16 particles per thread
REF_SERIAL_SO = os.path.join(REF_DIR, "libmdsc_ref_serial.so")

_dp = POINTER(c_double)
_ip = POINTER(c_int)


class CState(ctypes.Structure):
    """Mirror of mdsc_oracle_state / mdsc_ref_state."""

    _fields_ = [
        ("n", c_int), ("nd", c_int), ("L", c_double * 3),
        ("r", _dp), ("p", _dp), ("O", _dp), ("l", _dp), ("F", _dp), ("T", _dp),
        ("len", _dp), ("dia", _dp), ("mass", _dp), ("dip", _dp), ("clust", _ip),
    ]


class System:
    """One system of spherocylinders as structure-of-arrays (FP64)."""

    FIELDS = ("r", "p", "O", "l", "F", "T", "len", "dia", "mass", "dip")

    def __init__(self, r, p, O, l, length, dia, mass, dip, L, F=None, T=None, clust=None):
        n = len(length)

        def own(x, shape, dtype=np.float64):
            # always a private, contiguous copy: the C routines write in place
            return np.array(x, dtype=dtype, copy=True, order="C").reshape(shape)

        self.r = own(r, (n, 3))
        self.p = own(p, (n, 3))
        self.O = own(O, (n, 3, 3))
        self.l = own(l, (n, 3))
        self.len = own(length, (n,))
        self.dia = own(dia, (n,))
        self.mass = own(mass, (n,))
        self.dip = own(dip, (n, -1, 5))
        self.F = np.zeros((n, 3)) if F is None else own(F, (n, 3))
        self.T = np.zeros((n, 3)) if T is None else own(T, (n, 3))
        self.clust = np.zeros(n, dtype=np.int32) if clust is None else own(clust, (n,), np.int32)
        self.L = np.array(L, dtype=np.float64).reshape(3)

    @property
    def n(self) -> int:
        return len(self.len)

    @property
    def nd(self) -> int:
        return self.dip.shape[1]

    def copy(self) -> "System":
        return System(self.r.copy(), self.p.copy(), self.O.copy(), self.l.copy(), self.len.copy(),
                      self.dia.copy(), self.mass.copy(), self.dip.copy(), self.L.copy(),
                      self.F.copy(), self.T.copy(), self.clust.copy())

    def cstate(self) -> CState:
        s = CState()
        s.n, s.nd = self.n, self.nd
        for a in range(3):
            s.L[a] = float(self.L[a])
        for name in ("r", "p", "O", "l", "F", "T", "len", "dia", "mass", "dip"):
            arr = getattr(self, name)
            assert arr.flags.c_contiguous and arr.dtype == np.float64
            setattr(s, name, arr.ctypes.data_as(_dp))
        s.clust = self.clust.ctypes.data_as(_ip)
        return s


def _cc():
    return os.environ.get("CC", "gcc")


def build_oracle(force: bool = False) -> str:
    """Compile the C restatement into oracle/_build/libmdsc_oracle.so."""
    src = os.path.join(HERE, "mdsc_oracle.c")
    deps = [src, os.path.join(HERE, "mdsc_oracle.h"), os.path.join(HERE, "mt19937.h")]
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= max(os.path.getmtime(d) for d in deps)):
        return ORACLE_SO
    os.makedirs(BUILD, exist_ok=True)
    tmp = ORACLE_SO + f".tmp{os.getpid()}"
    cmd = [_cc(), "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=gnu99",
           "-o", tmp, src, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_root() -> str:
    """Where the reference's sources lie: MDSC_REFERENCE, else the default of
    the build recipe (build_ref.sh --where)."""
    env = os.environ.get("MDSC_REFERENCE")
    if env:
        return env
    out = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), "--where"], capture_output=True, text=True)
    return out.stdout.strip()


def reference_present() -> bool:
    root = reference_root()
    return bool(root) and os.path.isdir(os.path.join(root, "v25"))


def build_ref() -> str | None:
    """Build oracle/_ref from the reference sources when they are present."""
    script = os.path.join(HERE, "build_ref.sh")
    if not reference_present():
        return None
    subprocess.check_call(["bash", script])
    return REF_SO if os.path.exists(REF_SO) else None


def _bind(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


_SP = POINTER(CState)


class Oracle:
    """ctypes front-end of the C restatement (mdsc_oracle.c)."""

    def __init__(self, path: str | None = None):
        path = path or build_oracle()
        self.lib = lib = ctypes.CDLL(path)
        self._seg = _bind(lib, "mdsc_or_seg_dist", c_double, [_SP, c_int, c_int, _dp, _dp, _dp])
        self._nl = _bind(lib, "mdsc_or_neigh_list", c_int, [_SP, c_double, _ip, _ip, c_int])
        self._sc = _bind(lib, "mdsc_or_force_sc", c_int, [_SP, c_double, c_double, _dp, _dp, _dp])
        self._tab = _bind(lib, "mdsc_or_tabul", None, [c_double, _dp])
        self._dipR = _bind(lib, "mdsc_or_force_dipR", None, [_SP, _dp, _dp, _dp])
        self._mask = _bind(lib, "mdsc_or_mask_table", None, [_dp, c_double])
        self._wave = _bind(lib, "mdsc_or_wave_v", None, [_dp, _dp, c_double, c_int, c_int])
        self._dipK = _bind(lib, "mdsc_or_force_dipK", None, [_SP, c_int, c_double, _dp, _dp, _dp])
        self._ext = _bind(lib, "mdsc_or_ext_field", None, [_SP, _dp, _dp])
        self._self = _bind(lib, "mdsc_or_self_ener", c_double, [_SP])
        self._mx = _bind(lib, "mdsc_or_moveX", None, [_SP, c_double])
        self._mp = _bind(lib, "mdsc_or_moveP", None, [_SP, _dp, c_double, c_int, _dp, _dp])
        self._ren = _bind(lib, "mdsc_or_renorm", None, [_SP])
        self._thr = _bind(lib, "mdsc_or_set_threads", None, [c_int])
        self._inertia = _bind(lib, "mdsc_or_inertia", None, [c_double, c_double, c_double, _dp])
        self._rng_new = _bind(lib, "mdsc_or_rng_new", c_void_p, [c_ulong])
        self._rng_u = _bind(lib, "mdsc_or_rng_uniform", c_double, [c_void_p])
        self._rng_free = _bind(lib, "mdsc_or_rng_free", None, [c_void_p])
        self._cl = _bind(lib, "mdsc_or_clust_conf_rng", c_int, [_SP, c_double, c_void_p])
        self._cle = _bind(lib, "mdsc_or_clust_energy_rng", c_int, [_SP, c_double, c_void_p])
        self._pe = _bind(lib, "mdsc_or_pair_energy", c_double, [_SP, c_int, c_int])
        self._corr = _bind(lib, "mdsc_or_acc_correl", None, [_SP, c_double, c_int, _dp])
        self._corr_sp = _bind(lib, "mdsc_or_acc_correl_species", None, [_SP, c_int, _ip, c_double, c_int, _dp])
        self._oo = _bind(lib, "mdsc_or_oo_params", None, [_SP, _dp, _dp, _dp])
        self._tabcache: dict[float, np.ndarray] = {}

    def clust_conf(self, sysm: System, min_s: float, seed: int = 1, skip: int = 0):
        """clust_conf labels with an MT19937 seeded `seed`, advanced `skip`
        draws; returns (labels, number of clusters, the next draw)."""
        rng = self._rng_new(seed)
        try:
            for _ in range(skip):
                self._rng_u(rng)
            cs = sysm.cstate()
            nc = self._cl(ctypes.byref(cs), min_s, rng)
            nxt = self._rng_u(rng)
        finally:
            self._rng_free(rng)
        return sysm.clust.copy(), nc, nxt

    def pair_energy(self, sysm: System, a: int, b: int) -> float:
        """The energy criterion's pair energy (WCA + bare dipole-dipole) of
        particles a < b."""
        cs = sysm.cstate()
        return self._pe(ctypes.byref(cs), int(a), int(b))

    def clust_energy(self, sysm: System, u_bond: float, seed: int = 1, skip: int = 0):
        """clust_conf's labelling over the energy criterion: bonds where the
        pair energy is below -u_bond; returns (labels, clusters, next draw)."""
        rng = self._rng_new(seed)
        try:
            for _ in range(skip):
                self._rng_u(rng)
            cs = sysm.cstate()
            nc = self._cle(ctypes.byref(cs), u_bond, rng)
            nxt = self._rng_u(rng)
        finally:
            self._rng_free(rng)
        return sysm.clust.copy(), nc, nxt

    def acc_correl(self, sysm: System, bar_w: float, nbins: int, hist=None):
        """acc_correl (one species): the pair histograms 000, 110, 112, 220
        of this state, added to hist (4 x nbins)."""
        h = np.zeros((4, nbins)) if hist is None else hist
        cs = sysm.cstate()
        self._corr(ctypes.byref(cs), bar_w, nbins, h.ctypes.data_as(_dp))
        return h

    def acc_correl_species(self, sysm: System, counts, bar_w: float, nbins: int, hist=None):
        """acc_correl with species of counts[k] contiguous particles: the
        species blocks, then the species-pair blocks, each (4, nbins)."""
        nsp = len(counts)
        h = np.zeros((nsp + nsp * (nsp - 1) // 2, 4, nbins)) if hist is None else hist
        c = np.ascontiguousarray(counts, dtype=np.int32)
        cs = sysm.cstate()
        self._corr_sp(ctypes.byref(cs), nsp, c.ctypes.data_as(_ip), bar_w, nbins, h.ctypes.data_as(_dp))
        return h

    def oo_params(self, sysm: System):
        """oo_params: G1, G2 and the total dipole moment M."""
        G1, G2 = c_double(0), c_double(0)
        M = np.zeros(3)
        cs = sysm.cstate()
        self._oo(ctypes.byref(cs), ctypes.byref(G1), ctypes.byref(G2), M.ctypes.data_as(_dp))
        return G1.value, G2.value, M

    def set_threads(self, n: int) -> None:
        self._thr(int(n))

    def inertia(self, L, D, m):
        out = np.zeros(3)
        self._inertia(L, D, m, out.ctypes.data_as(_dp))
        return out

    def seg_dist(self, sysm: System, i: int, j: int, rij=None):
        if rij is None:
            rij = sysm.r[i] - sysm.r[j]
            rij = rij - sysm.L * np.floor(rij / sysm.L + 0.5)
        rij = np.ascontiguousarray(rij, dtype=np.float64)
        d = np.zeros(3)
        st = np.zeros(2)
        cs = sysm.cstate()
        dsq = self._seg(ctypes.byref(cs), i, j, rij.ctypes.data_as(_dp), d.ctypes.data_as(_dp),
                        st.ctypes.data_as(_dp))
        return dsq, d, st

    def neigh_list(self, sysm: System, r_list: float):
        n = sysm.n
        counts = np.zeros(n, np.int32)
        cap = 64 * n + 64
        idx = np.zeros(cap, np.int32)
        cs = sysm.cstate()
        tot = self._nl(ctypes.byref(cs), r_list, counts.ctypes.data_as(_ip), idx.ctypes.data_as(_ip), cap)
        if tot > cap:
            idx = np.zeros(tot, np.int32)
            self._nl(ctypes.byref(cs), r_list, counts.ctypes.data_as(_ip), idx.ctypes.data_as(_ip), tot)
        return counts, idx[:tot]

    def force_sc(self, sysm: System, r_cut: float, r_list: float):
        U, W = c_double(0), c_double(0)
        PT = np.zeros(9)
        cs = sysm.cstate()
        ok = self._sc(ctypes.byref(cs), r_cut, r_list, ctypes.byref(U), ctypes.byref(W), PT.ctypes.data_as(_dp))
        return bool(ok), U.value, W.value, PT.reshape(3, 3)

    def tabul(self, alpha: float) -> np.ndarray:
        key = float(alpha)
        if key not in self._tabcache:
            tab = np.zeros((32768, 3))
            self._tab(alpha, tab.ctypes.data_as(_dp))
            self._tabcache[key] = tab
        return self._tabcache[key]

    def force_dipR(self, sysm: System, alpha: float, rc: float = 0.0):
        """force_dipR; rc > 0: with tabul's table zeroed beyond rc (entry k
        holds r = 0.5 * 200.2 * (k + 1) / 32768), the real-space cutoff of
        the library's rc_real."""
        tab = self.tabul(alpha)
        if rc > 0:
            tab = tab.copy()
            self._mask(tab.ctypes.data_as(_dp), rc)
        U = c_double(0)
        PT = np.zeros(9)
        cs = sysm.cstate()
        self._dipR(ctypes.byref(cs), tab.ctypes.data_as(_dp), ctypes.byref(U), PT.ctypes.data_as(_dp))
        return U.value, PT.reshape(3, 3)

    def wave_v(self, L, alpha: float, K_max: int, ksq_max: int = 0) -> np.ndarray:
        kv = np.zeros((K_max + 1) ** 3)
        Lc = np.ascontiguousarray(L, dtype=np.float64)
        self._wave(kv.ctypes.data_as(_dp), Lc.ctypes.data_as(_dp), alpha, K_max, ksq_max)
        return kv

    def force_dipK(self, sysm: System, K_max: int, alpha: float, ksq_max: int = 0):
        kv = self.wave_v(sysm.L, alpha, K_max, ksq_max)
        U = c_double(0)
        PT = np.zeros(9)
        cs = sysm.cstate()
        self._dipK(ctypes.byref(cs), K_max, alpha, kv.ctypes.data_as(_dp), ctypes.byref(U),
                   PT.ctypes.data_as(_dp))
        return U.value, PT.reshape(3, 3)

    def ext_field(self, sysm: System, B):
        U = c_double(0)
        Bc = np.ascontiguousarray(B, dtype=np.float64)
        cs = sysm.cstate()
        self._ext(ctypes.byref(cs), Bc.ctypes.data_as(_dp), ctypes.byref(U))
        return U.value

    def self_ener(self, sysm: System) -> float:
        cs = sysm.cstate()
        return self._self(ctypes.byref(cs))

    def moveX(self, sysm: System, dt: float) -> None:
        cs = sysm.cstate()
        self._mx(ctypes.byref(cs), dt)

    def moveP(self, sysm: System, xi, dt: float, last: bool):
        xi_c = np.ascontiguousarray(xi, dtype=np.float64)
        K = np.zeros(2)
        PT = np.zeros(9)
        cs = sysm.cstate()
        self._mp(ctypes.byref(cs), xi_c.ctypes.data_as(_dp), dt, int(last), K.ctypes.data_as(_dp),
                 PT.ctypes.data_as(_dp))
        return K, PT.reshape(3, 3)

    def renorm(self, sysm: System) -> None:
        cs = sysm.cstate()
        self._ren(ctypes.byref(cs))


class MDOracle:
    """The reference driver's step loop (mdsc_or_md_*) on one system."""

    class _MD(ctypes.Structure):
        pass

    def __init__(self, oracle: Oracle, sysm: System, *, dt, temp, Q, gamma, xi0, sr_cut, K_max,
                 ksq_max, alpha, B, cl_fr=0, min_s=0.1, rc_real=0.0):
        lib = oracle.lib
        self.lib = lib
        self.sys = sysm
        # opaque storage: sizeof(mdsc_or_md) is well under 64 KB
        self._buf = ctypes.create_string_buffer(65536)
        self._cs = sysm.cstate()
        init = _bind(lib, "mdsc_or_md_init", c_int,
                     [c_void_p, _SP, c_double, c_double, c_double, c_double, c_double, c_double,
                      c_int, c_int, c_double, _dp, c_int, c_double])
        self._step = _bind(lib, "mdsc_or_md_step", c_int, [c_void_p, _SP])
        self._free = _bind(lib, "mdsc_or_md_free", None, [c_void_p])
        self._obs = _bind(lib, "mdsc_or_md_obs", None, [c_void_p, _dp])
        self._setth = _bind(lib, "mdsc_or_md_set_thermo", None, [c_void_p, _dp, _dp])
        Bc = np.ascontiguousarray(B, dtype=np.float64)
        ok = init(self._buf, ctypes.byref(self._cs), dt, temp, Q, gamma, xi0, sr_cut, K_max,
                  ksq_max, alpha, Bc.ctypes.data_as(_dp), cl_fr, min_s)
        if not ok:
            raise RuntimeError("initial overlap")
        if rc_real > 0 and not _bind(lib, "mdsc_or_md_mask_table", c_int, [c_void_p, _SP, c_double])(
                self._buf, ctypes.byref(self._cs), rc_real):
            raise RuntimeError("initial overlap")

    def step(self) -> bool:
        return bool(self._step(self._buf, ctypes.byref(self._cs)))

    def set_thermostat(self, xi, strn) -> None:
        x = np.ascontiguousarray(xi, dtype=np.float64)
        s = np.ascontiguousarray(strn, dtype=np.float64)
        self._setth(self._buf, x.ctypes.data_as(_dp), s.ctypes.data_as(_dp))

    def obs(self) -> dict:
        o = np.zeros(48)
        self._obs(self._buf, o.ctypes.data_as(_dp))
        return dict(K=o[0:2].copy(), Uss=o[2], Wss=o[3], UdipR=o[4], UdipK=o[5], Uext=o[6], Uself=o[7],
                    xi=o[8:10].copy(), step=int(o[10]), list_builds=int(o[11]), PTkin=o[12:21].reshape(3, 3),
                    PTss=o[21:30].reshape(3, 3), PTdipR=o[30:39].reshape(3, 3), PTdipK=o[39:48].reshape(3, 3))

    def close(self):
        if self._buf is not None:
            self._free(self._buf)
            self._buf = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ref:
    """ctypes front-end of the reference's own routines (oracle/_ref)."""

    def __init__(self, path: str = REF_SO, threads: int = 1):
        self.lib = lib = ctypes.CDLL(path)
        _bind(lib, "mdsc_ref_set_threads", None, [c_int])(int(threads))
        self._seg = _bind(lib, "mdsc_ref_seg_dist", c_double, [_SP, c_int, c_int, _dp, _dp])
        self._nl = _bind(lib, "mdsc_ref_neigh_list", c_int, [_SP, c_double, _ip, _ip, c_int])
        self._sc = _bind(lib, "mdsc_ref_force_sc", c_int, [_SP, c_double, c_double, _dp, _dp, _dp])
        self._tab = _bind(lib, "mdsc_ref_tabul", None, [c_double, _dp])
        self._dipR = _bind(lib, "mdsc_ref_force_dipR", None, [_SP, c_double, _dp, _dp])
        self._dipRc = _bind(lib, "mdsc_ref_force_dipR_cut", None, [_SP, c_double, c_double, _dp, _dp])
        self._dipK = _bind(lib, "mdsc_ref_force_dipK", None, [_SP, c_int, c_double, c_int, _dp, _dp])
        self._ext = _bind(lib, "mdsc_ref_ext_field", None, [_SP, _dp, _dp])
        self._self = _bind(lib, "mdsc_ref_self_ener", c_double, [_SP])
        self._mx = _bind(lib, "mdsc_ref_moveX", None, [_SP, c_double])
        self._mp = _bind(lib, "mdsc_ref_moveP", None, [_SP, _dp, c_double, c_int, _dp, _dp])
        self._ren = _bind(lib, "mdsc_ref_renorm", None, [_SP])
        self._rng_new = _bind(lib, "mdsc_ref_rng_new", c_void_p, [c_ulong])
        self._rng_u = _bind(lib, "mdsc_ref_rng_uniform", c_double, [c_void_p])
        self._rng_free = _bind(lib, "mdsc_ref_rng_free", None, [c_void_p])
        self._cl = _bind(lib, "mdsc_ref_clust_conf", None, [_SP, c_double, c_void_p])
        self._corr = _bind(lib, "mdsc_ref_acc_correl", None, [_SP, c_double, c_int, _dp])
        self._corr_sp = _bind(lib, "mdsc_ref_acc_correl_species", None, [_SP, c_int, _ip, c_double, c_int, _dp])
        self._oo = _bind(lib, "mdsc_ref_oo_params", None, [_SP, _dp, _dp, _dp])
        self._mt = _bind(lib, "mdsc_ref_moveTher", None,
                         [_dp, _dp, c_double, c_double, c_void_p, c_void_p, c_double, c_double, _dp,
                          c_double, c_int])

    def seg_dist(self, sysm, i, j):
        d = np.zeros(3)
        st = np.zeros(2)
        cs = sysm.cstate()
        dsq = self._seg(ctypes.byref(cs), i, j, d.ctypes.data_as(_dp), st.ctypes.data_as(_dp))
        return dsq, d, st

    def acc_correl(self, sysm, bar_w, nbins, hist=None):
        h = np.zeros((4, nbins)) if hist is None else hist
        cs = sysm.cstate()
        self._corr(ctypes.byref(cs), bar_w, nbins, h.ctypes.data_as(_dp))
        return h

    def acc_correl_species(self, sysm, counts, bar_w, nbins, hist=None):
        nsp = len(counts)
        h = np.zeros((nsp + nsp * (nsp - 1) // 2, 4, nbins)) if hist is None else hist
        c = np.ascontiguousarray(counts, dtype=np.int32)
        cs = sysm.cstate()
        self._corr_sp(ctypes.byref(cs), nsp, c.ctypes.data_as(_ip), bar_w, nbins, h.ctypes.data_as(_dp))
        return h

    def oo_params(self, sysm):
        G1, G2 = c_double(0), c_double(0)
        M = np.zeros(3)
        cs = sysm.cstate()
        self._oo(ctypes.byref(cs), ctypes.byref(G1), ctypes.byref(G2), M.ctypes.data_as(_dp))
        return G1.value, G2.value, M

    def neigh_list(self, sysm, r_list):
        n = sysm.n
        counts = np.zeros(n, np.int32)
        cap = 64 * n + 64
        idx = np.zeros(cap, np.int32)
        cs = sysm.cstate()
        tot = self._nl(ctypes.byref(cs), r_list, counts.ctypes.data_as(_ip), idx.ctypes.data_as(_ip), cap)
        if tot > cap:
            idx = np.zeros(tot, np.int32)
            self._nl(ctypes.byref(cs), r_list, counts.ctypes.data_as(_ip), idx.ctypes.data_as(_ip), tot)
        return counts, idx[:tot]

    def force_sc(self, sysm, r_cut, r_list):
        U, W = c_double(0), c_double(0)
        PT = np.zeros(9)
        cs = sysm.cstate()
        ok = self._sc(ctypes.byref(cs), r_cut, r_list, ctypes.byref(U), ctypes.byref(W), PT.ctypes.data_as(_dp))
        return bool(ok), U.value, W.value, PT.reshape(3, 3)

    def tabul(self, alpha):
        tab = np.zeros((32768, 3))
        self._tab(alpha, tab.ctypes.data_as(_dp))
        return tab

    def force_dipR(self, sysm, alpha, rc=0.0):
        U = c_double(0)
        PT = np.zeros(9)
        cs = sysm.cstate()
        if rc > 0:
            self._dipRc(ctypes.byref(cs), alpha, rc, ctypes.byref(U), PT.ctypes.data_as(_dp))
        else:
            self._dipR(ctypes.byref(cs), alpha, ctypes.byref(U), PT.ctypes.data_as(_dp))
        return U.value, PT.reshape(3, 3)

    def force_dipK(self, sysm, K_max, alpha, ksq_max=0):
        U = c_double(0)
        PT = np.zeros(9)
        cs = sysm.cstate()
        self._dipK(ctypes.byref(cs), K_max, alpha, ksq_max, ctypes.byref(U), PT.ctypes.data_as(_dp))
        return U.value, PT.reshape(3, 3)

    def ext_field(self, sysm, B):
        U = c_double(0)
        Bc = np.ascontiguousarray(B, dtype=np.float64)
        cs = sysm.cstate()
        self._ext(ctypes.byref(cs), Bc.ctypes.data_as(_dp), ctypes.byref(U))
        return U.value

    def self_ener(self, sysm):
        cs = sysm.cstate()
        return self._self(ctypes.byref(cs))

    def moveX(self, sysm, dt):
        cs = sysm.cstate()
        self._mx(ctypes.byref(cs), dt)

    def moveP(self, sysm, xi, dt, last):
        xi_c = np.ascontiguousarray(xi, dtype=np.float64)
        K = np.zeros(2)
        PT = np.zeros(9)
        cs = sysm.cstate()
        self._mp(ctypes.byref(cs), xi_c.ctypes.data_as(_dp), dt, int(last), K.ctypes.data_as(_dp),
                 PT.ctypes.data_as(_dp))
        return K, PT.reshape(3, 3)

    def renorm(self, sysm):
        cs = sysm.cstate()
        self._ren(ctypes.byref(cs))

    def clust_conf(self, sysm, min_s, seed=1, skip=0):
        """Labels from clust_conf with a generator seeded `seed` and advanced
        by `skip` draws; returns the next draw too, to pin stream position."""
        rng = self._rng_new(seed)
        try:
            for _ in range(skip):
                self._rng_u(rng)
            cs = sysm.cstate()
            self._cl(ctypes.byref(cs), min_s, rng)
            nxt = self._rng_u(rng)
        finally:
            self._rng_free(rng)
        return sysm.clust.copy(), nxt
