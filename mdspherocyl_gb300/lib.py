"""ctypes binding of the C ABI (include/mdsc.h) and a thin Python front-end.

The library is the in-tree build mdspherocyl_gb300/_lib/libmdsc.so.  There
is no fallback: if it cannot be built or loaded, or no GPU is visible,
every call raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_longlong, c_size_t, c_ulong, c_void_p

import numpy as np

from . import build as _build
from .systems import SystemSpec, SystemState

_dp = POINTER(c_double)
_ip = POINTER(c_int)

MAX_DIPOLES = 4

STATUS = {
    0: "MDSC_OK", 1: "MDSC_ERR_BAD_ARG", 2: "MDSC_ERR_CUDA", 3: "MDSC_ERR_OOM",
    4: "MDSC_ERR_OVERLAP", 5: "MDSC_ERR_NAN", 6: "MDSC_ERR_TABLE_RANGE",
    7: "MDSC_ERR_LIST_OVERFLOW", 8: "MDSC_ERR_NO_DEVICE", 9: "MDSC_ERR_TOO_LARGE",
    10: "MDSC_ERR_STATE",
}

# every entry point include/mdsc.h declares
EXPORTS = [
    "mdsc_create", "mdsc_destroy", "mdsc_num_systems", "mdsc_device_bytes", "mdsc_estimate_bytes",
    "mdsc_last_error", "mdsc_upload", "mdsc_download", "mdsc_upload_all", "mdsc_download_all",
    "mdsc_set_thermostat", "mdsc_zero_forces", "mdsc_force_sc", "mdsc_force_dipR",
    "mdsc_force_dipK", "mdsc_ext_field", "mdsc_self_ener", "mdsc_moveX", "mdsc_moveP",
    "mdsc_renorm", "mdsc_neigh_list", "mdsc_check_list", "mdsc_clust_conf", "mdsc_set_cluster_energy",
    "mdsc_abi_sizes",
    "mdsc_step", "mdsc_step_io",
    "mdsc_observe", "mdsc_launches_per_step", "mdsc_stream", "mdsc_profile_steps",
    "mdsc_place_rods", "mdsc_last_device_ms", "mdsc_force_dipR_noalloc", "mdsc_transfer",
    "mdsc_autotune", "mdsc_tuning", "mdsc_set_tuning", "mdsc_correlation_bins", "mdsc_correlations",
    "mdsc_order_params", "mdsc_step_trace", "mdsc_get_rng", "mdsc_set_rng", "mdsc_set_species",
    "mdsc_correlation_size", "mdsc_get_thermostat", "mdsc_render", "mdsc_lattice", "mdsc_thermalize",
    "mdsc_fp32_peak", "mdsc_set_list_cells", "mdsc_transfer_many", "mdsc_set_step_limit",
]


class SystemDesc(ctypes.Structure):
    _fields_ = [
        ("n", c_int), ("nd", c_int), ("box", c_double * 3), ("alpha", c_double),
        ("K_max", c_int), ("ksq_max", c_int), ("sr_cut", c_double), ("dt", c_double),
        ("temp", c_double), ("Q", c_double), ("gamma", c_double), ("xi0", c_double),
        ("B", c_double * 3), ("min_s", c_double), ("cl_fr", c_int),
        ("thermo_seed", c_ulong * 2), ("cluster_seed", c_ulong), ("cluster_skip", c_ulong),
        ("rc_real", c_double),
    ]


class HostState(ctypes.Structure):
    _fields_ = [
        ("r", _dp), ("p", _dp), ("O", _dp), ("l", _dp), ("F", _dp), ("T", _dp),
        ("len", _dp), ("dia", _dp), ("mass", _dp), ("dip", _dp), ("clust", _ip),
    ]


class Observables(ctypes.Structure):
    _fields_ = [
        ("K", c_double * 2), ("U_ss", c_double), ("W_ss", c_double), ("U_dipR", c_double),
        ("U_dipK", c_double), ("U_ext", c_double), ("U_self", c_double),
        ("PT_kin", c_double * 9), ("PT_ss", c_double * 9), ("PT_dipR", c_double * 9),
        ("PT_dipK", c_double * 9), ("xi", c_double * 2), ("step", c_longlong),
        ("status", c_int), ("n_clusters", c_int), ("list_builds", c_int), ("pad", c_int),
        ("G1", c_double), ("G2", c_double), ("M", c_double * 3),
    ]

    def as_dict(self) -> dict:
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if hasattr(v, "__len__") else v
        return d


class View(ctypes.Structure):
    """mdsc_view: what mdsc_render draws and from where (the reference
    viewer's controls and defaults, v25/graphic.cpp:24-41)."""

    _fields_ = [
        ("width", c_int), ("height", c_int), ("theta", c_double), ("phi", c_double), ("dist", c_double),
        ("ref", c_double * 3), ("shift", c_double * 3), ("dipoles", c_int), ("images", c_int), ("box", c_int),
        ("cluster", c_int),
    ]

    @classmethod
    def make(cls, width=480, height=480, theta=0.1, phi=0.0, dist=15.0, ref=(0, 0, 0), shift=(0, 0, 0),
             dipoles=True, images=False, box=True, cluster=-1) -> "View":
        v = cls()
        v.width, v.height, v.theta, v.phi, v.dist = int(width), int(height), float(theta), float(phi), float(dist)
        for a in range(3):
            v.ref[a], v.shift[a] = float(ref[a]), float(shift[a])
        v.dipoles, v.images, v.box, v.cluster = int(bool(dipoles)), int(bool(images)), int(bool(box)), int(cluster)
        return v


def write_ppm(path: str, rgb) -> None:
    """A binary PPM (P6) of an (height, width, 3) uint8 image."""
    a = np.ascontiguousarray(rgb, dtype=np.uint8)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (a.shape[1], a.shape[0]))
        f.write(a.tobytes())


def read_ppm(path: str):
    """The (height, width, 3) uint8 image of a binary PPM written by write_ppm."""
    data = open(path, "rb").read()
    parts = data.split(b"\n", 3)
    assert parts[0] == b"P6" and parts[2] == b"255"
    w, h = (int(x) for x in parts[1].split())
    return np.frombuffer(parts[3], dtype=np.uint8, count=w * h * 3).reshape(h, w, 3)


class MdscError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        super().__init__(f"{where}: {STATUS.get(code, code)} {detail}".strip())


_LIB = None


def load(build: bool = True) -> ctypes.CDLL:
    """Load libmdsc.so (building it first if needed)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"libmdsc.so not found at {path}")
    lib = ctypes.CDLL(path)
    P = POINTER
    sig = {
        "mdsc_create": (c_int, [P(SystemDesc), c_int, c_int, P(c_void_p)]),
        "mdsc_destroy": (c_int, [c_void_p]),
        "mdsc_num_systems": (c_int, [c_void_p]),
        "mdsc_device_bytes": (c_size_t, [c_void_p]),
        "mdsc_estimate_bytes": (c_size_t, [P(SystemDesc), c_int]),
        "mdsc_last_error": (c_int, [c_void_p, c_char_p, c_size_t]),
        "mdsc_upload": (c_int, [c_void_p, c_int, P(HostState)]),
        "mdsc_download": (c_int, [c_void_p, c_int, P(HostState)]),
        "mdsc_upload_all": (c_int, [c_void_p, P(HostState)]),
        "mdsc_download_all": (c_int, [c_void_p, P(HostState)]),
        "mdsc_set_thermostat": (c_int, [c_void_p, c_int, _dp, _dp]),
        "mdsc_zero_forces": (c_int, [c_void_p]),
        "mdsc_force_sc": (c_int, [c_void_p, _dp, _dp, _dp]),
        "mdsc_force_dipR": (c_int, [c_void_p, _dp, _dp]),
        "mdsc_force_dipK": (c_int, [c_void_p, _dp, _dp]),
        "mdsc_ext_field": (c_int, [c_void_p, _dp]),
        "mdsc_self_ener": (c_int, [c_void_p, _dp]),
        "mdsc_moveX": (c_int, [c_void_p]),
        "mdsc_moveP": (c_int, [c_void_p, _dp, c_int, _dp, _dp]),
        "mdsc_renorm": (c_int, [c_void_p]),
        "mdsc_neigh_list": (c_int, [c_void_p]),
        "mdsc_check_list": (c_int, [c_void_p, _ip]),
        "mdsc_clust_conf": (c_int, [c_void_p, c_int, _ip, _ip]),
        "mdsc_set_cluster_energy": (c_int, [c_void_p, c_int, c_double]),
        "mdsc_abi_sizes": (None, [P(c_size_t), P(c_size_t), P(c_size_t), P(c_size_t)]),
        "mdsc_step": (c_int, [c_void_p, c_int, P(Observables)]),
        "mdsc_step_io": (c_int, [c_void_p, P(HostState), c_int, P(HostState), P(Observables)]),
        "mdsc_observe": (c_int, [c_void_p, P(Observables)]),
        "mdsc_launches_per_step": (c_int, [c_void_p]),
        "mdsc_stream": (c_void_p, [c_void_p]),
        "mdsc_last_device_ms": (c_double, [c_void_p]),
        "mdsc_transfer": (c_int, [c_void_p, c_int, c_void_p, c_int]),
        "mdsc_autotune": (c_int, [c_void_p, c_int]),
        "mdsc_tuning": (c_int, [c_void_p, _ip, c_char_p, c_size_t]),
        "mdsc_set_tuning": (c_int, [c_void_p, _ip]),
        "mdsc_correlation_bins": (c_int, [c_void_p, c_int, c_double]),
        "mdsc_correlations": (c_int, [c_void_p, c_double, _dp]),
        "mdsc_set_species": (c_int, [c_void_p, c_int, c_int, _ip]),
        "mdsc_get_thermostat": (c_int, [c_void_p, c_int, _dp, _dp]),
        "mdsc_render": (c_int, [c_void_p, c_int, P(View), c_void_p]),
        "mdsc_lattice": (c_int, [c_void_p, c_int, c_int, _ip, _ip]),
        "mdsc_thermalize": (c_int, [c_void_p, c_int, c_double, ctypes.c_ulonglong]),
        "mdsc_correlation_size": (c_int, [c_void_p, c_int, c_double]),
        "mdsc_order_params": (c_int, [c_void_p, _dp, _dp, _dp]),
        "mdsc_step_trace": (c_int, [c_void_p, c_int, P(Observables)]),
        "mdsc_get_rng": (c_int, [c_void_p, c_int, c_int, P(ctypes.c_uint32), _ip]),
        "mdsc_set_rng": (c_int, [c_void_p, c_int, c_int, P(ctypes.c_uint32), c_int]),
        "mdsc_force_dipR_noalloc": (c_int, [c_int, c_void_p, c_void_p, _dp, c_double, c_void_p, c_void_p,
                                            c_void_p, c_void_p]),
        "mdsc_profile_steps": (c_int, [c_void_p, c_int, c_int, c_char_p, c_size_t, _dp, _ip]),
        "mdsc_place_rods": (c_int, [c_int, _dp, _dp, _dp, ctypes.c_ulonglong, c_double, c_int, _dp, _dp]),
        "mdsc_fp32_peak": (c_int, [c_int, c_int, _dp, _dp, _dp, _ip]),
        "mdsc_set_list_cells": (c_int, [c_void_p, c_int]),
        "mdsc_transfer_many": (c_int, [c_void_p, c_void_p, _ip, _ip, c_int]),
        "mdsc_set_step_limit": (c_int, [c_void_p, c_int, c_longlong]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def desc_from_spec(spec: SystemSpec, nd: int) -> SystemDesc:
    d = SystemDesc()
    d.n, d.nd = int(spec.n), int(nd)
    for a in range(3):
        d.box[a] = float(spec.box[a])
        d.B[a] = float(spec.B[a])
    d.alpha = float(spec.alpha)
    d.K_max, d.ksq_max = int(spec.K_max), int(spec.ksq_max)
    d.sr_cut = float(spec.sr_cut)
    d.dt, d.temp, d.Q, d.gamma, d.xi0 = (float(spec.dt), float(spec.temp), float(spec.Q),
                                          float(spec.gamma), float(spec.xi0))
    d.min_s = float(spec.min_s)
    d.cl_fr = int(spec.cl_fr)
    d.thermo_seed[0], d.thermo_seed[1] = 1, 2
    d.cluster_seed, d.cluster_skip = 1, 0
    d.rc_real = float(getattr(spec, "rc_real", 0.0))
    return d


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


class Batch:
    """One handle of the library: nsys independent systems resident on the GPU.

    Mirrors the reference's hot-path functions (force_sc, force_dipR,
    force_dipK, ext_field, self_ener, moveX, moveP, renorm, neigh_list,
    check_list, clust_conf) and adds the fused, graph-captured step.
    """

    def __init__(self, specs, states=None, device: int = 0, descs=None):
        self.lib = load()
        self.specs = list(specs)
        if descs is None:
            nds = [states[k].dip.shape[1] if states is not None else 1 for k in range(len(self.specs))]
            descs = [desc_from_spec(s, nd) for s, nd in zip(self.specs, nds)]
        self.nsys = len(descs)
        self._descs = (SystemDesc * self.nsys)(*descs)
        h = c_void_p()
        self._check(self.lib.mdsc_create(self._descs, self.nsys, device, ctypes.byref(h)), "mdsc_create")
        self.h = h
        self.n = [d.n for d in descs]
        self.nd = [d.nd for d in descs]
        for k, spec in enumerate(self.specs):
            if spec is not None and getattr(spec, "cl_energy", 0.0) > 0:
                self.set_cluster_energy(k, spec.cl_energy)
        if states is not None:
            for k, st in enumerate(states):
                self.upload(k, st)

    # -- plumbing --
    def _err(self) -> str:
        if not getattr(self, "h", None):
            return ""
        buf = ctypes.create_string_buffer(512)
        self.lib.mdsc_last_error(self.h, buf, 512)
        return buf.value.decode(errors="replace")

    def _check(self, code: int, where: str) -> None:
        if code != 0:
            raise MdscError(code, where, self._err())

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.mdsc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def device_bytes(self) -> int:
        return int(self.lib.mdsc_device_bytes(self.h))

    @property
    def launches_per_step(self) -> int:
        return int(self.lib.mdsc_launches_per_step(self.h))

    # -- state --
    @staticmethod
    def _hoststate(r, p, O, l, F=None, T=None, length=None, dia=None, mass=None, dip=None, clust=None):
        hs = HostState()
        hs.r, hs.p, hs.O, hs.l = _ptr(r), _ptr(p), _ptr(O), _ptr(l)
        hs.F, hs.T = _ptr(F), _ptr(T)
        hs.len, hs.dia, hs.mass, hs.dip = _ptr(length), _ptr(dia), _ptr(mass), _ptr(dip)
        hs.clust = None if clust is None else clust.ctypes.data_as(_ip)
        return hs

    def upload(self, k: int, st: SystemState, F=None, T=None, clust=None) -> None:
        c = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
        arrs = dict(r=c(st.r), p=c(st.p), O=c(st.O), l=c(st.l), length=c(st.length), dia=c(st.dia),
                    mass=c(st.mass), dip=c(st.dip), F=None if F is None else c(F),
                    T=None if T is None else c(T),
                    clust=None if clust is None else np.ascontiguousarray(clust, dtype=np.int32))
        hs = self._hoststate(**arrs)
        self._check(self.lib.mdsc_upload(self.h, k, ctypes.byref(hs)), "mdsc_upload")

    def download(self, k: int, template: SystemState | None = None) -> dict:
        n = self.n[k]
        out = dict(r=np.zeros((n, 3)), p=np.zeros((n, 3)), O=np.zeros((n, 3, 3)), l=np.zeros((n, 3)),
                   F=np.zeros((n, 3)), T=np.zeros((n, 3)), clust=np.zeros(n, np.int32))
        hs = self._hoststate(out["r"], out["p"], out["O"], out["l"], out["F"], out["T"], clust=out["clust"])
        self._check(self.lib.mdsc_download(self.h, k, ctypes.byref(hs)), "mdsc_download")
        return out

    def upload_all(self, r, p, O, l, F=None, T=None, length=None, dia=None, mass=None, dip=None) -> None:
        hs = self._hoststate(r, p, O, l, F, T, length, dia, mass, dip)
        self._check(self.lib.mdsc_upload_all(self.h, ctypes.byref(hs)), "mdsc_upload_all")

    def download_all(self, r, p, O, l, F=None, T=None) -> None:
        hs = self._hoststate(r, p, O, l, F, T)
        self._check(self.lib.mdsc_download_all(self.h, ctypes.byref(hs)), "mdsc_download_all")

    def step_io(self, state_in: dict | None, nsteps: int, state_out: dict | None, obs=None) -> None:
        """mdsc_step_io: upload state_in (arrays r, p, O, l, F, T for the
        whole batch; None keeps the device state), take nsteps steps and
        download into state_out (None: nothing); obs: an Observables array
        of nsys entries or None."""
        hi = None if state_in is None else ctypes.byref(self._hoststate(*(state_in.get(k) for k in "rpOlFT")))
        ho = None if state_out is None else ctypes.byref(self._hoststate(*(state_out.get(k) for k in "rpOlFT")))
        self._check(self.lib.mdsc_step_io(self.h, hi, int(nsteps), ho, obs), "mdsc_step_io")

    def set_thermostat(self, k: int, xi, strn=None) -> None:
        x = np.ascontiguousarray(xi, dtype=np.float64)
        s = None if strn is None else np.ascontiguousarray(strn, dtype=np.float64)
        self._check(self.lib.mdsc_set_thermostat(self.h, k, _ptr(x), _ptr(s)), "mdsc_set_thermostat")

    # -- the reference's functions --
    def get_thermostat(self, k: int):
        """(xi[2], stored normal[2]) of system k."""
        xi, strn = np.zeros(2), np.zeros(2)
        self._check(self.lib.mdsc_get_thermostat(self.h, k, _ptr(xi), _ptr(strn)), "mdsc_get_thermostat")
        return xi, strn

    def zero_forces(self):
        self._check(self.lib.mdsc_zero_forces(self.h), "mdsc_zero_forces")

    def force_sc(self):
        U, W, PT = np.zeros(self.nsys), np.zeros(self.nsys), np.zeros((self.nsys, 9))
        code = self.lib.mdsc_force_sc(self.h, _ptr(U), _ptr(W), _ptr(PT))
        self._check(code, "mdsc_force_sc")
        return U, W, PT.reshape(self.nsys, 3, 3)

    def force_dipR(self):
        U, PT = np.zeros(self.nsys), np.zeros((self.nsys, 9))
        self._check(self.lib.mdsc_force_dipR(self.h, _ptr(U), _ptr(PT)), "mdsc_force_dipR")
        return U, PT.reshape(self.nsys, 3, 3)

    def force_dipK(self):
        U, PT = np.zeros(self.nsys), np.zeros((self.nsys, 9))
        self._check(self.lib.mdsc_force_dipK(self.h, _ptr(U), _ptr(PT)), "mdsc_force_dipK")
        return U, PT.reshape(self.nsys, 3, 3)

    def ext_field(self):
        U = np.zeros(self.nsys)
        self._check(self.lib.mdsc_ext_field(self.h, _ptr(U)), "mdsc_ext_field")
        return U

    def self_ener(self):
        U = np.zeros(self.nsys)
        self._check(self.lib.mdsc_self_ener(self.h, _ptr(U)), "mdsc_self_ener")
        return U

    def moveX(self):
        self._check(self.lib.mdsc_moveX(self.h), "mdsc_moveX")

    def moveP(self, xi, last: bool):
        x = np.ascontiguousarray(np.broadcast_to(np.asarray(xi, dtype=np.float64), (self.nsys, 2)))
        K, PT = np.zeros((self.nsys, 2)), np.zeros((self.nsys, 9))
        self._check(self.lib.mdsc_moveP(self.h, _ptr(x), int(last), _ptr(K), _ptr(PT)), "mdsc_moveP")
        return K, PT.reshape(self.nsys, 3, 3)

    def renorm(self):
        self._check(self.lib.mdsc_renorm(self.h), "mdsc_renorm")

    def neigh_list(self):
        self._check(self.lib.mdsc_neigh_list(self.h), "mdsc_neigh_list")

    def check_list(self):
        out = np.zeros(self.nsys, np.int32)
        self._check(self.lib.mdsc_check_list(self.h, out.ctypes.data_as(_ip)), "mdsc_check_list")
        return out.astype(bool)

    def clust_conf(self, k: int):
        lab = np.zeros(self.n[k], np.int32)
        nc = c_int(0)
        self._check(self.lib.mdsc_clust_conf(self.h, k, lab.ctypes.data_as(_ip), ctypes.byref(nc)),
                    "mdsc_clust_conf")
        return lab, nc.value

    def set_cluster_energy(self, k: int, u_bond_kT: float) -> None:
        """System k's cluster bonds: U_pair < -u_bond_kT * T (pair energy =
        WCA + bare dipole-dipole), or the reference's geometric test for 0."""
        self._check(self.lib.mdsc_set_cluster_energy(self.h, k, float(u_bond_kT)), "mdsc_set_cluster_energy")

    # -- observables outside the step --
    def correlation_bins(self, k: int, bar_w: float) -> int:
        return int(self.lib.mdsc_correlation_bins(self.h, k, float(bar_w)))

    def set_species(self, k: int, counts) -> None:
        """Species of system k: contiguous blocks of counts[c] particles."""
        c = np.ascontiguousarray(counts, dtype=np.int32)
        self._check(self.lib.mdsc_set_species(self.h, k, len(c), c.ctypes.data_as(_ip)), "mdsc_set_species")
        self._nsp = getattr(self, "_nsp", [1] * self.nsys)
        self._nsp[k] = len(c)

    def correlations(self, bar_w: float, hist=None):
        """acc_correl on the GPU: per system an array (blocks, 4, nbins) --
        its species blocks (Hista), then its species-pair blocks (Histe) --
        of the 000, 110, 112 and 220 pair sums.  hist (a list of such
        arrays, e.g. the last call's result) is added to, as the reference
        accumulates."""
        nsp = getattr(self, "_nsp", [1] * self.nsys)
        nb = [self.correlation_bins(k, bar_w) for k in range(self.nsys)]
        nblk = [c + c * (c - 1) // 2 for c in nsp]
        size = [self.lib.mdsc_correlation_size(self.h, k, float(bar_w)) for k in range(self.nsys)]
        assert all(size[k] == nblk[k] * 4 * nb[k] for k in range(self.nsys))
        off = np.cumsum([0] + size)
        flat = np.zeros(int(off[-1]))
        if hist is not None:
            for k in range(self.nsys):
                flat[off[k]:off[k + 1]] = np.asarray(hist[k], dtype=np.float64).reshape(-1)
        self._check(self.lib.mdsc_correlations(self.h, float(bar_w), _ptr(flat)), "mdsc_correlations")
        return [flat[off[k]:off[k + 1]].reshape(nblk[k], 4, nb[k]) for k in range(self.nsys)]

    def order_params(self):
        """oo_params on the GPU: G1 (nsys,), G2 (nsys,), M (nsys, 3)."""
        G1, G2, M = np.zeros(self.nsys), np.zeros(self.nsys), np.zeros((self.nsys, 3))
        self._check(self.lib.mdsc_order_params(self.h, _ptr(G1), _ptr(G2), _ptr(M)), "mdsc_order_params")
        return G1, G2, M

    def lattice(self, k: int, counts) -> int:
        """The reference's lattice for system k (mdsc_lattice); returns the
        overlapping pairs its closing test finds."""
        c = np.ascontiguousarray(counts, dtype=np.int32)
        nov = c_int(0)
        self._check(self.lib.mdsc_lattice(self.h, k, len(c), c.ctypes.data_as(_ip), ctypes.byref(nov)),
                    "mdsc_lattice")
        return nov.value

    def thermalize(self, k: int, temp: float, seed: int = 1) -> None:
        self._check(self.lib.mdsc_thermalize(self.h, k, float(temp), int(seed)), "mdsc_thermalize")

    def render(self, k: int, view: "View | None" = None, **kw):
        """A picture of system k (mdsc_render): (height, width, 3) uint8."""
        v = view if view is not None else View.make(**kw)
        img = np.zeros((v.height, v.width, 3), dtype=np.uint8)
        self._check(self.lib.mdsc_render(self.h, k, ctypes.byref(v), img.ctypes.data_as(c_void_p)), "mdsc_render")
        return img

    def transfer_from(self, k: int, src: "Batch", ks: int) -> None:
        """Move system ks of src into slot k of this batch, on the GPU."""
        self._check(self.lib.mdsc_transfer(self.h, k, src.h, ks), "mdsc_transfer")

    # -- fused step --
    def step(self, nsteps: int = 1):
        obs = (Observables * self.nsys)()
        self._check(self.lib.mdsc_step(self.h, int(nsteps), obs), "mdsc_step")
        return [o.as_dict() for o in obs]

    def step_trace(self, nsteps: int):
        """nsteps steps; every step's observables, [step][system] dicts."""
        tr = (Observables * (max(nsteps, 0) * self.nsys))()
        self._check(self.lib.mdsc_step_trace(self.h, int(nsteps), tr), "mdsc_step_trace")
        return [[tr[k * self.nsys + s].as_dict() for s in range(self.nsys)] for k in range(nsteps)]

    def get_rng(self, k: int, which: int):
        """MT19937 state (624 words, position) of generator `which` of system k."""
        mt = np.zeros(624, dtype=np.uint32)
        mti = c_int(0)
        self._check(self.lib.mdsc_get_rng(self.h, k, which, mt.ctypes.data_as(POINTER(ctypes.c_uint32)),
                                          ctypes.byref(mti)), "mdsc_get_rng")
        return mt, mti.value

    def set_rng(self, k: int, which: int, mt, mti: int) -> None:
        a = np.ascontiguousarray(mt, dtype=np.uint32)
        self._check(self.lib.mdsc_set_rng(self.h, k, which, a.ctypes.data_as(POINTER(ctypes.c_uint32)), int(mti)),
                    "mdsc_set_rng")

    def observe(self):
        obs = (Observables * self.nsys)()
        self._check(self.lib.mdsc_observe(self.h, obs), "mdsc_observe")
        return [o.as_dict() for o in obs]

    def autotune(self, force: bool = False) -> dict:
        """Choose the launch mappings now (mdsc_autotune) and return them."""
        self._check(self.lib.mdsc_autotune(self.h, int(force)), "mdsc_autotune")
        return self.tuning()

    def set_tuning(self, rp_warps: int, rsum_threads: int, wca_blocks: int, kg_scalar: int) -> None:
        """Pin the launch mappings (mdsc_set_tuning) instead of tuning them."""
        v = np.array([rp_warps, rsum_threads, wca_blocks, kg_scalar], dtype=np.int32)
        self._check(self.lib.mdsc_set_tuning(self.h, v.ctypes.data_as(_ip)), "mdsc_set_tuning")

    def transfer_many(self, src: "Batch", pairs) -> None:
        """Slots (k, ks) of this batch from src, all at once (mdsc_transfer_many)."""
        d = np.ascontiguousarray([p[0] for p in pairs], dtype=np.int32)
        q = np.ascontiguousarray([p[1] for p in pairs], dtype=np.int32)
        self._check(self.lib.mdsc_transfer_many(self.h, src.h, d.ctypes.data_as(_ip), q.ctypes.data_as(_ip), len(d)),
                    "mdsc_transfer_many")

    def set_step_limit(self, k: int, limit: int) -> None:
        """System k stops taking steps at step count `limit` (<= 0: no limit)."""
        self._check(self.lib.mdsc_set_step_limit(self.h, k, int(limit)), "mdsc_set_step_limit")

    def set_list_cells(self, on: bool) -> None:
        """List builds on cells (the default) or over all pairs; same lists."""
        self._check(self.lib.mdsc_set_list_cells(self.h, int(bool(on))), "mdsc_set_list_cells")

    def tuning(self) -> dict:
        """The launch mappings in use and the last tuning's timings."""
        v = np.zeros(5, dtype=np.int32)
        buf = ctypes.create_string_buffer(4096)
        self._check(self.lib.mdsc_tuning(self.h, v.ctypes.data_as(_ip), buf, 4096), "mdsc_tuning")
        return {"rp_warps": int(v[0]), "rsum_threads": int(v[1]), "wca_blocks": int(v[2]),
                "kg_scalar": int(v[3]), "tuned": bool(v[4]), "log": buf.value.decode()}

    def profile(self, nsteps: int):
        nmax, stride = 16, 32
        names = ctypes.create_string_buffer(nmax * stride)
        ms = np.zeros(nmax)
        nk = c_int(0)
        self._check(self.lib.mdsc_profile_steps(self.h, nsteps, nmax, names, stride, _ptr(ms),
                                                ctypes.byref(nk)), "mdsc_profile_steps")
        out = {}
        for k in range(nk.value):
            nm = names.raw[k * stride:(k + 1) * stride].split(b"\0")[0].decode()
            out[nm] = float(ms[k])
        return out


def normalize_correlations(hist, counts, box, bar_w: float, cor_cont: float = 1.0):
    """nor_correl (v25/functions.cpp:2472-2540): the bin centres, the shell
    volumes and the normalised 000, 110, 112, 220 functions (factors 1, 3,
    3/2, 5) of every block of hist (blocks, 4, nbins) as mdsc_correlations
    lays them out -- a species block over norm * cor_cont * N (N - 1) (zero
    for a species of one particle), a species-pair block over
    norm * cor_cont * N_m N_n -- as arrays instead of the reference's
    correlation.dat.  cor_cont: the accumulated configurations weighted as
    the driver weights them (1 / V each, v25/main.cpp:716)."""
    counts = list(counts)
    nc = len(counts)
    h = np.asarray(hist, dtype=np.float64).reshape(nc + nc * (nc - 1) // 2, 4, -1)
    Lmin = float(min(box))
    pos = (np.arange(h.shape[2]) + 0.5) * bar_w
    shell = 4.0 * np.pi * pos * pos * (3.0 * Lmin / (2.0 * pos) - 2.0) * bar_w
    sphere = 4.0 * np.pi * (pos * pos * bar_w + bar_w ** 3 / 12.0)
    norm = np.where((pos >= Lmin / 2.0) & (pos <= Lmin / np.sqrt(2.0)), shell, sphere)
    fac = np.array([1.0, 3.0, 1.5, 5.0])[:, None]
    g = np.zeros_like(h)
    for k in range(nc):
        if counts[k] > 1:
            g[k] = fac * h[k] / (norm * cor_cont * counts[k] * (counts[k] - 1))
    q = nc
    for m in range(nc - 1):
        for n in range(m + 1, nc):
            g[q] = fac * h[q] / (norm * cor_cont * counts[n] * counts[m])
            q += 1
    return pos, norm, g


def place_rods(lengths, dia, box, seed: int, gap: float = 0.0):
    """Seeded non-overlapping placement (host routine of the library)."""
    lib = load()
    n = len(lengths)
    ln = np.ascontiguousarray(lengths, dtype=np.float64)
    dd = np.ascontiguousarray(dia, dtype=np.float64)
    bx = np.ascontiguousarray(box, dtype=np.float64)
    r = np.zeros((n, 3))
    O = np.zeros((n, 3, 3))
    code = lib.mdsc_place_rods(n, _ptr(ln), _ptr(dd), _ptr(bx), int(seed) & ((1 << 64) - 1), float(gap),
                               2000000, _ptr(r), _ptr(O))
    if code != 0:
        raise MdscError(code, "mdsc_place_rods")
    return r, O


def estimate_bytes(descs) -> int:
    lib = load()
    arr = (SystemDesc * len(descs))(*descs)
    return int(lib.mdsc_estimate_bytes(arr, len(descs)))


def fp32_peak(device: int = 0, reps: int = 5) -> dict:
    """Measured FP32 multiply-add throughput of the device (mdsc_fp32_peak):
    TFLOP/s of the scalar and paired forms and the best paired launch's ms."""
    lib = load()
    a, b, ms = c_double(), c_double(), c_double()
    sms = c_int()
    code = lib.mdsc_fp32_peak(device, reps, ctypes.byref(a), ctypes.byref(b), ctypes.byref(ms), ctypes.byref(sms))
    if code != 0:
        raise MdscError(code, "mdsc_fp32_peak", "")
    return {"ffma_tflops": a.value, "ffma2_tflops": b.value, "launch_ms": ms.value, "sms": sms.value}
