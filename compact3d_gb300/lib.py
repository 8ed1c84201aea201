"""ctypes binding of libc3d.so and a Python mirror of the reference's step interface.

The reference exposes no library API: the driver calls ``GETUP(U,P,HH,SS,NTIME,PRESG,
PRESG3,SGSVIS)`` (compact3d.f:879) and the diagnostics ``DIVCHECK``, ``CFL``, ``CHKMF``
and ``WALLSS`` with Fortran arrays.  ``Channel`` offers the same calls with numpy arrays in
the same Fortran layouts, implemented by the CUDA library through its C-ABI.

There is no CPU fallback: if libc3d.so cannot be loaded, or no CUDA device is present,
the calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .grid import C3D_FP64, C3D_MIXED, Grid, c3d_grid

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libc3d.so")

C3D_OK = 0
ERRORS = {-1: "EINVAL", -2: "ECUDA", -3: "ENOMEM", -4: "ENOTCONV", -5: "ENONFINITE",
          -6: "ESTATE", -7: "ENODEV", -8: "EIO"}

# Every function declared in include/c3d.h, with its ctypes signature.
_vp, _ip, _dp = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)


class c3d_diag(ctypes.Structure):
    _fields_ = [("divmax", ctypes.c_double), ("cflm", ctypes.c_double),
                ("flow1", ctypes.c_double), ("flow3", ctypes.c_double),
                ("wsm", ctypes.c_double * 3), ("nonfinite", ctypes.c_int)]


SIGNATURES = {
    "c3d_error_string": (ctypes.c_char_p, [_ip]),
    "c3d_last_error": (ctypes.c_char_p, []),
    "c3d_version": (_ip, []),
    "c3d_set_device": (_ip, [_ip]),
    "c3d_create": (_ip, [ctypes.POINTER(c3d_grid), ctypes.POINTER(_vp)]),
    "c3d_destroy": (_ip, [_vp]),
    "c3d_upload": (_ip, [_vp, _dp, _dp, _dp, _dp]),
    "c3d_download": (_ip, [_vp, _dp, _dp, _dp, _dp]),
    "c3d_upload_wall": (_ip, [_vp, _dp, _dp]),
    "c3d_download_wall": (_ip, [_vp, _dp, _dp]),
    "c3d_set_wsm": (_ip, [_vp, _dp]),
    "c3d_get_wsm": (_ip, [_vp, _dp]),
    "c3d_set_wall_iter_cap": (_ip, [_vp, _ip]),
    "c3d_autotune": (_ip, [_vp, ctypes.POINTER(_ip)]),
    "c3d_get_schedule": (_ip, [_vp, ctypes.POINTER(_ip)]),
    "c3d_set_schedule": (_ip, [_vp, ctypes.POINTER(_ip)]),
    "c3d_op_set": (_ip, [_vp, _dp]),
    "c3d_op_apply": (_ip, [_vp, _ip, _ip]),
    "c3d_op_get": (_ip, [_vp, _dp]),
    "c3d_plane_stats": (_ip, [_vp, _dp]),
    "c3d_plane_spectra": (_ip, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "c3d_plane_quadrants": (_ip, [_vp, _dp, _dp]),
    "c3d_wall_spectrum": (_ip, [_vp, ctypes.c_double, _dp]),
    "c3d_set_cflmax": (_ip, [_vp, ctypes.c_double]),
    "c3d_particles_advance": (_ip, [_vp, _ip, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.POINTER(ctypes.c_int)]),
    "c3d_particles_source": (_ip, [_vp, _ip, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp, _dp, _dp]),
    "c3d_corr3d": (_ip, [_vp, _dp]),
    "c3d_checkpoint_write": (_ip, [_vp, ctypes.c_char_p, _ip, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    "c3d_checkpoint_read": (_ip, [_vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), _dp, _dp, _dp]),
    "c3d_step": (_ip, [_vp, _ip, ctypes.c_double, _dp, _dp]),
    "c3d_diagnose": (_ip, [_vp, ctypes.POINTER(c3d_diag)]),
    "c3d_getup": (_ip, [_vp, _dp, _dp, _dp, _dp, _ip, ctypes.c_double, _dp, _dp]),
    "c3d_project": (_ip, [_vp]),
    "c3d_host_register": (_ip, [_vp, ctypes.c_size_t]),
    "c3d_host_unregister": (_ip, [_vp]),
    "c3d_host_alloc": (_ip, [ctypes.c_size_t, ctypes.POINTER(_vp)]),
    "c3d_host_free": (_ip, [_vp]),
    "c3d_sync": (_ip, [_vp]),
    "c3d_pipe_wait_selftest": (_ip, [_vp, ctypes.c_double]),
    "c3d_last_step_stats": (_ip, [_vp, _dp, ctypes.POINTER(_ip)]),
    "c3d_step_async": (_ip, [_vp, _ip, ctypes.c_double]),
    "c3d_set_presg": (_ip, [_vp, ctypes.c_double, ctypes.c_double]),
    "c3d_get_presg": (_ip, [_vp, _dp, _dp]),
    "c3d_timer_start": (_ip, [_vp]),
    "c3d_timer_stop": (_ip, [_vp, _dp]),
    "c3d_profile": (_ip, [_vp, _ip]),
    "c3d_profile_count": (_ip, [_vp]),
    "c3d_profile_get": (_ip, [_vp, _ip, ctypes.POINTER(ctypes.c_char_p), _dp, ctypes.POINTER(_ip), _dp]),
    "c3d_divcheck_noalloc": (_ip, [ctypes.POINTER(c3d_grid), _dp, _dp]),
    "c3d_batch_create": (_ip, [_ip, ctypes.POINTER(c3d_grid), ctypes.POINTER(_vp)]),
    "c3d_batch_destroy": (_ip, [_vp]),
    "c3d_batch_channel": (_ip, [_vp, _ip, ctypes.POINTER(_vp)]),
    "c3d_batch_step": (_ip, [_vp, _ip, _dp, _dp, _dp]),
    "c3d_batch_sync": (_ip, [_vp]),
    "c3d_batch_set_form": (_ip, [_vp, _ip]),
    "c3d_batch_get_form": (_ip, [_vp, ctypes.POINTER(_ip)]),
    "c3d_batch_set_groups": (_ip, [_vp, _ip]),
    "c3d_batch_set_z_segments": (_ip, [_vp, _vp]),
    "c3d_batch_set_x_warps": (_ip, [_vp, _ip]),
    "c3d_batch_set_concurrent": (_ip, [_vp, _ip]),
    "c3d_batch_last_step_stats": (_ip, [_vp, _dp, ctypes.POINTER(_ip)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libc3d.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing; run __graft_entry__.build() or "
                               "python -m compact3d_gb300.build")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


# Operators of c3d_op_apply (include/c3d.h)
C3D_SCHEDULE_LEN = 16   # ints of a launch schedule (include/c3d.h)
OPS = {"DX1": 1, "DX2": 2, "IX": 3, "DZ1": 4, "DZ2": 5, "IZ": 6, "DY1": 7, "DY2": 8, "POISSON": 9}


class C3DError(RuntimeError):
    def __init__(self, code: int, where: str):
        L = load()
        msg = L.c3d_last_error().decode(errors="replace")
        super().__init__(f"{where}: {ERRORS.get(code, code)} ({msg})")
        self.code = code


def check(code: int, where: str):
    if code != C3D_OK:
        raise C3DError(code, where)


def _p(a):
    if a is None:
        return None
    if a.dtype != np.float64 or not (a.flags.f_contiguous or a.ndim == 1):
        raise TypeError("arrays must be float64 in Fortran order")
    return a.ctypes.data_as(_dp)


class Channel:
    """One channel on the GPU; arrays use the reference's Fortran layouts."""

    def __init__(self, grid: Grid, precision: int | None = None):
        self.grid = grid
        self.precision = grid.precision if precision is None else precision
        self._gs = grid.struct(self.precision)
        h = _vp()
        check(load().c3d_create(ctypes.byref(self._gs), ctypes.byref(h)), "c3d_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None) and not getattr(self, "_owned_by_batch", False):
            load().c3d_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, U, P, HH):
        check(load().c3d_upload(self.h, _p(U), _p(P), _p(HH), None), "c3d_upload")

    def download(self, U=None, P=None, HH=None):
        g = self.grid
        U = g.zeros_u() if U is None else U
        P = g.zeros_p() if P is None else P
        HH = g.zeros_u() if HH is None else HH
        check(load().c3d_download(self.h, _p(U), _p(P), _p(HH), None), "c3d_download")
        return U, P, HH

    # ---- LES (FILES != 0) ----
    def download_sgsvis(self):
        """SGSVIS(0:M1,0:M2,0:M3) of the last step (periodic ghost columns filled)."""
        S = self.grid.zeros_s()
        check(load().c3d_download(self.h, None, None, None, _p(S)), "c3d_download")
        return S

    def upload_wall(self, tauw=None, taub=None):
        check(load().c3d_upload_wall(self.h, _p(tauw), _p(taub)), "c3d_upload_wall")

    def download_wall(self):
        g = self.grid
        tw = np.zeros(g.shape_tau(), order="F")
        tb = np.zeros(g.shape_tau(), order="F")
        check(load().c3d_download_wall(self.h, _p(tw), _p(tb)), "c3d_download_wall")
        return tw, tb

    def set_wsm(self, wsm):
        w = np.ascontiguousarray(wsm, dtype=np.float64)
        check(load().c3d_set_wsm(self.h, _p(w)), "c3d_set_wsm")

    def get_wsm(self):
        w = np.zeros(3)
        check(load().c3d_get_wsm(self.h, _p(w)), "c3d_get_wsm")
        return w

    # ---- launch schedule ----
    SCHEDULE_KEYS = ("z_segment_zA", "z_segment_zB", "z_segment_zC", "z_segment_zD", "z_segment_zE",
                     "x_rows_per_block", "fft_z_tile", "fft_x_plan", "fft_z_plan", "z_split_zA",
                     "x_split_xA", "x_bulk_stages", "x_stage_xA", "ycn_tile", "x_row_lanes", "concurrent_pieces")

    def autotune(self) -> dict:
        sch = (_ip * C3D_SCHEDULE_LEN)()
        check(load().c3d_autotune(self.h, sch), "c3d_autotune")
        return dict(zip(self.SCHEDULE_KEYS, sch[:]))

    def get_schedule(self) -> dict:
        sch = (_ip * C3D_SCHEDULE_LEN)()
        check(load().c3d_get_schedule(self.h, sch), "c3d_get_schedule")
        return dict(zip(self.SCHEDULE_KEYS, sch[:]))

    def set_schedule(self, sched: dict):
        sch = (_ip * C3D_SCHEDULE_LEN)(*[int(sched.get(k, 0)) for k in self.SCHEDULE_KEYS])
        check(load().c3d_set_schedule(self.h, sch), "c3d_set_schedule")

    # ---- ENERGY's plane statistics ----
    STAT_NAMES = ("u", "v", "w", "p", "wx", "wy", "wz", "uu", "vv", "ww", "uv", "uw", "vw", "pp", "pv",
                  "wxwx", "wywy", "wzwz", "uuv", "vww", "skew_u", "skew_v", "skew_w", "flat_u", "flat_v",
                  "flat_w", "dudy", "dvdy", "dwdy")

    def plane_stats(self):
        """(N2M, 29) array of ENERGY's plane statistics; columns as STAT_NAMES."""
        out = np.zeros(self.grid.n2m * 29)
        check(load().c3d_plane_stats(self.h, _p(out)), "c3d_plane_stats")
        return out.reshape(self.grid.n2m, 29)

    def plane_spectra(self, vmo=None):
        """ENERGY's spectra and two-point correlations: dict of Fortran (N, N2M, 3) arrays
        xspec, zspec, rxx, rzz, rxy; vmo (N2M, 3) is the mean the spectra subtract (None:
        the instantaneous plane means)."""
        g = self.grid
        out = {k: np.zeros((n, g.n2m, 3), order="F") for k, n in
               (("xspec", g.n1m), ("zspec", g.n3m), ("rxx", g.n1m), ("rzz", g.n3m), ("rxy", g.n1m))}
        v = None if vmo is None else np.asfortranarray(vmo, dtype=np.float64)
        check(load().c3d_plane_spectra(self.h, _p(v), *(_p(out[k].reshape(-1, order="F")) for k in
                                                        ("xspec", "zspec", "rxx", "rzz", "rxy"))),
              "c3d_plane_spectra")
        return out

    def plane_quadrants(self, vmp=None):
        """ENERGY's quadrant analysis: (N2M, 8) array, Q(J,1..4) then QP(J,1..4); vmp
        (N2M, 2) or None (the reference's never-assigned VMP, zero)."""
        out = np.zeros(self.grid.n2m * 8)
        v = None if vmp is None else np.asfortranarray(vmp, dtype=np.float64)
        check(load().c3d_plane_quadrants(self.h, _p(v), _p(out)), "c3d_plane_quadrants")
        return out.reshape(self.grid.n2m, 8)

    def particles_advance(self, par, dt, diam=0.0002, dens=2220.0, hhh=0.05):
        """One particle step on the device: par (N, 6) x, y, z, u, v, w -> (par, impact)."""
        p = np.ascontiguousarray(par, dtype=np.float64).copy()
        imp = np.zeros(len(p), dtype=np.int32)
        check(load().c3d_particles_advance(self.h, len(p), _p(p.reshape(-1)), diam, dens, hhh, dt,
                                           imp.ctypes.data_as(ctypes.POINTER(ctypes.c_int))), "c3d_particles_advance")
        return p, imp

    def particles_source(self, par, diam=0.0002, dens=2220.0, hhh=0.05):
        """SOURCE_PAR's terms for par (N, 6): three Fortran (0:N1,0:N2,0:N3) arrays."""
        p = np.ascontiguousarray(par, dtype=np.float64)
        out = [self.grid.zeros_s() for _ in range(3)]
        check(load().c3d_particles_source(self.h, len(p), _p(p.reshape(-1)), diam, dens, hhh, *(_p(o) for o in out)),
              "c3d_particles_source")
        return out

    def set_cflmax(self, cflmax: float):
        check(load().c3d_set_cflmax(self.h, float(cflmax)), "c3d_set_cflmax")

    def wall_spectrum(self, utau: float):
        """SPECTAUW(1:N1M, 1:N3M, 1) of the bottom wall's TAUW about utau^2."""
        out = np.zeros((self.grid.n1m, self.grid.n3m), order="F")
        check(load().c3d_wall_spectrum(self.h, float(utau), _p(out)), "c3d_wall_spectrum")
        return out

    def corr3d(self):
        """RXYZ(1:N1M, 1:N2M, 1:N3M, 3)."""
        g = self.grid
        out = np.zeros((g.n1m, g.n2m, g.n3m, 3), order="F")
        check(load().c3d_corr3d(self.h, _p(out)), "c3d_corr3d")
        return out

    # ---- checkpoint (CWRITE / READUP in a format that round-trips) ----
    def checkpoint_write(self, path, ntime: int, time: float, presg: float, presg3: float):
        check(load().c3d_checkpoint_write(self.h, str(path).encode(), int(ntime), float(time), float(presg),
                                          float(presg3)), "c3d_checkpoint_write")

    def checkpoint_read(self, path):
        """Loads the state of a checkpoint; returns (ntime, time, presg, presg3)."""
        nt = ctypes.c_int(0)
        t, a, b = ((ctypes.c_double * 1)() for _ in range(3))
        check(load().c3d_checkpoint_read(self.h, str(path).encode(), ctypes.byref(nt), t, a, b),
              "c3d_checkpoint_read")
        return nt.value, t[0], a[0], b[0]

    # ---- operators one at a time ----
    def op_set(self, F):
        check(load().c3d_op_set(self.h, _p(F)), "c3d_op_set")

    def op_apply(self, op: int, count: int = 1):
        check(load().c3d_op_apply(self.h, int(op), int(count)), "c3d_op_apply")

    def op_get(self):
        F = self.grid.zeros_s()
        check(load().c3d_op_get(self.h, _p(F)), "c3d_op_get")
        return F

    def operator(self, op: int, F):
        """One operator on a host field F(0:M1,0:M2,0:M3); returns the result."""
        self.op_set(F)
        self.op_apply(op, 1)
        return self.op_get()

    def set_wall_iter_cap(self, cap: int):
        check(load().c3d_set_wall_iter_cap(self.h, int(cap)), "c3d_set_wall_iter_cap")

    def step(self, ntime: int, dt: float, presg: float, presg3: float):
        """GETUP on the device-resident state; returns the new (PRESG, PRESG3)."""
        a = (ctypes.c_double * 1)(presg)
        b = (ctypes.c_double * 1)(presg3)
        check(load().c3d_step(self.h, ntime, dt, a, b), "c3d_step")
        return a[0], b[0]

    def getup(self, U, P, HH, ntime: int, dt: float, presg: float, presg3: float, sgsvis=None):
        """GETUP(U,P,HH,SS,NTIME,PRESG,PRESG3,SGSVIS) with host arrays updated in place."""
        a = (ctypes.c_double * 1)(presg)
        b = (ctypes.c_double * 1)(presg3)
        check(load().c3d_getup(self.h, _p(U), _p(P), _p(HH), _p(sgsvis), ntime, dt, a, b), "c3d_getup")
        return a[0], b[0]

    def project(self):
        check(load().c3d_project(self.h), "c3d_project")

    def diagnose(self) -> dict:
        d = c3d_diag()
        rc = load().c3d_diagnose(self.h, ctypes.byref(d))
        if rc not in (C3D_OK, -5):
            check(rc, "c3d_diagnose")
        return dict(divmax=d.divmax, cflm=d.cflm, flow1=d.flow1, flow3=d.flow3,
                    wsm=np.array(d.wsm[:]), nonfinite=bool(d.nonfinite))

    def sync(self):
        check(load().c3d_sync(self.h), "c3d_sync")

    def step_async(self, ntime: int, dt: float):
        check(load().c3d_step_async(self.h, ntime, dt), "c3d_step_async")

    def set_presg(self, presg: float, presg3: float):
        check(load().c3d_set_presg(self.h, presg, presg3), "c3d_set_presg")

    def get_presg(self):
        a = (ctypes.c_double * 1)()
        b = (ctypes.c_double * 1)()
        check(load().c3d_get_presg(self.h, a, b), "c3d_get_presg")
        return a[0], b[0]

    def timer_start(self):
        check(load().c3d_timer_start(self.h), "c3d_timer_start")

    def timer_stop(self) -> float:
        ms = (ctypes.c_double * 1)()
        check(load().c3d_timer_stop(self.h, ms), "c3d_timer_stop")
        return ms[0]

    def profile(self, enable: bool = True):
        check(load().c3d_profile(self.h, int(enable)), "c3d_profile")

    def profile_read(self) -> list[dict]:
        L = load()
        out = []
        for i in range(L.c3d_profile_count(self.h)):
            nm = ctypes.c_char_p()
            ms = (ctypes.c_double * 1)()
            n = (ctypes.c_int * 1)()
            b = (ctypes.c_double * 1)()
            check(L.c3d_profile_get(self.h, i, ctypes.byref(nm), ms, n, b), "c3d_profile_get")
            out.append(dict(name=nm.value.decode(), ms=ms[0], launches=n[0], bytes=b[0]))
        return out

    def last_step_stats(self):
        ms = (ctypes.c_double * 1)()
        n = (ctypes.c_int * 1)()
        check(load().c3d_last_step_stats(self.h, ms, n), "c3d_last_step_stats")
        return ms[0], n[0]


class Batch:
    """An ensemble of independent channels stepped together as one CUDA graph."""

    def __init__(self, grids, precision: int | None = None):
        self.grids = list(grids)
        self._gs = (c3d_grid * len(self.grids))()
        for i, g in enumerate(self.grids):
            self._gs[i] = g.struct(g.precision if precision is None else precision)
        h = _vp()
        check(load().c3d_batch_create(len(self.grids), self._gs, ctypes.byref(h)), "c3d_batch_create")
        self.h = h
        self.channels = []
        for i, g in enumerate(self.grids):
            c = _vp()
            check(load().c3d_batch_channel(self.h, i, ctypes.byref(c)), "c3d_batch_channel")
            ch = Channel.__new__(Channel)
            ch.grid, ch.precision, ch.h = g, g.precision if precision is None else precision, c
            ch._owned_by_batch = True
            self.channels.append(ch)

    def close(self):
        if getattr(self, "h", None):
            for ch in self.channels:
                ch.h = None
            load().c3d_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, ntime: int, dt, presg, presg3):
        n = len(self.grids)
        dta = (ctypes.c_double * n)(*dt)
        a = (ctypes.c_double * n)(*presg)
        b = (ctypes.c_double * n)(*presg3)
        check(load().c3d_batch_step(self.h, ntime, dta, a, b), "c3d_batch_step")
        return list(a), list(b)

    def last_step_stats(self):
        ms = (ctypes.c_double * 1)()
        n = (ctypes.c_int * 1)()
        check(load().c3d_batch_last_step_stats(self.h, ms, n), "c3d_batch_last_step_stats")
        return ms[0], n[0]

    FORMS = {"streams": 0, "worklist": 1}

    def set_form(self, form: str):
        """'worklist' (one launch per pass over all channels; DNS channels of one
        precision) or 'streams' (each channel's step on its own stream)."""
        check(load().c3d_batch_set_form(self.h, self.FORMS[form]), "c3d_batch_set_form")

    def set_groups(self, groups: int):
        """Work-list form: the channels in `groups` groups, each on its own stream."""
        check(load().c3d_batch_set_groups(self.h, int(groups)), "c3d_batch_set_groups")

    def set_z_segments(self, seg):
        """Work-list form: segment length (8, 16 or 32) of the z passes zA..zE."""
        a = (ctypes.c_int * 5)(*[int(x) for x in seg])
        check(load().c3d_batch_set_z_segments(self.h, a), "c3d_batch_set_z_segments")

    def set_x_warps(self, warps: int):
        """Work-list form: warps per block of the x passes (2, 4 or 8)."""
        check(load().c3d_batch_set_x_warps(self.h, int(warps)), "c3d_batch_set_x_warps")

    def set_concurrent(self, on: int):
        """Work-list form: the pieces of the explicit passes as concurrent branches."""
        check(load().c3d_batch_set_concurrent(self.h, int(on)), "c3d_batch_set_concurrent")

    def get_form(self) -> str:
        f = (ctypes.c_int * 1)()
        check(load().c3d_batch_get_form(self.h, f), "c3d_batch_get_form")
        return {v: k for k, v in self.FORMS.items()}[f[0]]


class TimeAverage:
    """TAVER (compact3d.f:10755-11060): running means of statistics tables over the samples
    NAVG = 1, 2, ...: the first sample is copied, later ones enter as
    XO = (XO (NAVG - 1) + X) / NAVG, in that operation order.  Tables are numpy arrays
    (plane_stats, plane_spectra's tables, plane_quadrants, wall stresses, ...) keyed by
    name; every sample must carry the same keys."""

    def __init__(self):
        self.navg = 0
        self.mean = {}

    def add(self, **tables):
        self.navg += 1
        if self.navg == 1:
            self.mean = {k: np.array(v, dtype=np.float64, copy=True) for k, v in tables.items()}
        else:
            if set(tables) != set(self.mean):
                raise ValueError("TimeAverage: a sample's tables differ from the first sample's")
            n = float(self.navg)
            for k, v in tables.items():
                self.mean[k] = (self.mean[k] * (n - 1.0) + np.asarray(v, dtype=np.float64)) / n
        return self.mean


_host_arrays = {}


def host_array(shape, dtype=np.float64) -> np.ndarray:
    """A Fortran-order array in page-locked host memory from c3d_host_alloc (transfers at
    the host link's rate); release it with host_free."""
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    p = _vp()
    check(load().c3d_host_alloc(n, ctypes.byref(p)), "c3d_host_alloc")
    buf = (ctypes.c_char * n).from_address(p.value)
    a = np.ndarray(shape, dtype=dtype, buffer=buf, order="F")
    _host_arrays[a.ctypes.data] = p.value
    return a


def host_free(a: np.ndarray):
    p = _host_arrays.pop(a.ctypes.data)
    check(load().c3d_host_free(p), "c3d_host_free")


def host_register(a: np.ndarray):
    check(load().c3d_host_register(a.ctypes.data, a.nbytes), "c3d_host_register")


def host_unregister(a: np.ndarray):
    check(load().c3d_host_unregister(a.ctypes.data), "c3d_host_unregister")


__all__ = ["Channel", "Batch", "load", "C3DError", "host_register", "host_unregister", "host_array", "host_free", "C3D_FP64",
           "C3D_MIXED", "SIGNATURES"]
