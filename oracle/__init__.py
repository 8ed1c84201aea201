"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the FP64 CPU oracle (c3d_oracle.cpp).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use this
module, as the checker; the product path never imports it.  Parity of the oracle is
unpinned (the reference ships no golden vectors and cannot be built here); it is checked
against known answers in tests/test_oracle.py.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "libc3d_oracle.so")
SRC = os.path.join(HERE, "c3d_oracle.cpp")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (-O3 -fopenmp -ffp-contract=off)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["g++", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17",
               "-o", LIB + ".tmp", SRC]
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
        L.orc_create.restype = vp
        L.orc_create.argtypes = [vp]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_threads.argtypes = [ip]
        L.orc_max_threads.restype = ip
        L.orc_getup.restype = ip
        L.orc_getup.argtypes = [vp, dp, dp, dp, dp, ip, ctypes.c_double, dp, dp]
        L.orc_project.argtypes = [vp, dp]
        L.orc_bcond.argtypes = [vp, dp]
        L.orc_getdp.argtypes = [vp, dp, dp]
        L.orc_rhsdp.argtypes = [vp, dp, ctypes.c_double, dp]
        L.orc_divcheck.restype = ctypes.c_double
        L.orc_divcheck.argtypes = [vp, dp]
        L.orc_cfl.restype = ctypes.c_double
        L.orc_cfl.argtypes = [vp, dp]
        L.orc_chkmf.argtypes = [vp, dp, dp, dp]
        L.orc_wallss.argtypes = [vp, dp, dp]
        L.orc_plane_stats.argtypes = [vp, dp, dp, dp]
        L.orc_set_wall.argtypes = [vp, dp, dp, ip]
        L.orc_get_wall.argtypes = [vp, dp, dp, dp]
        L.orc_set_wsm.argtypes = [vp, dp]
        L.orc_set_wall_iter_cap.argtypes = [vp, ip]
        L.orc_sgs.restype = ip
        L.orc_sgs.argtypes = [vp, dp, dp, dp]
        L.orc_wallmodel.restype = ip
        L.orc_sgs_rhs.restype = ip
        L.orc_operator.restype = ip
        L.orc_operator.argtypes = [vp, ip, dp, dp]
        L.orc_sgs_rhs.argtypes = [vp, dp, dp, dp]
        L.orc_wallmodel.argtypes = [vp, dp]
        L.orc_dqrrt.restype = ip
        L.orc_dqrrt.argtypes = [dp, ip, ctypes.c_double, dp, dp, dp]
        L.orc_get_beta.argtypes = [vp, dp]
        L.orc_filter.argtypes = [vp, ip, dp, ip]
        L.orc_plane_spectra.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_plane_quadrants.argtypes = [vp, dp, dp, dp]
        L.orc_wall_spectrum.argtypes = [vp, ctypes.c_double, dp]
        L.orc_set_cflmax.argtypes = [vp, ctypes.c_double]
        L.orc_particles_advance.argtypes = [vp, dp, ip, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
        L.orc_particles_source.argtypes = [vp, dp, ip, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                           dp, dp, dp]
        L.orc_iwm_slots.restype = ip
        L.orc_get_iwm.argtypes = [vp, dp]
        L.orc_corr3d.argtypes = [vp, dp, dp]
        for f in ("orc_ctdma11", "orc_ctdma_recip"):
            getattr(L, f).argtypes = [ip, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp, dp]
        L.orc_tdmap.argtypes = [ip, dp, dp, dp, dp, dp]
        L.orc_fft.argtypes = [ip, dp, ip]
        L.orc_dft2d.argtypes = [ip, ip, dp, ip]
        L.orc_poisson_metrics.argtypes = [vp, dp, dp, dp, dp, dp]
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim == 1), "Fortran float64 array"
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """One channel in the CPU oracle; arrays are Fortran-layout numpy float64."""

    def __init__(self, grid, threads: int | None = None):
        self.grid = grid
        self._gs = grid.struct()
        self.h = lib().orc_create(ctypes.byref(self._gs))
        if not self.h:
            raise ValueError("oracle rejected the grid")
        if threads:
            lib().orc_set_threads(threads)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def getup(self, U, P, HH, ntime, dt, presg, presg3, sgsvis=None):
        a = (ctypes.c_double * 1)(presg)
        b = (ctypes.c_double * 1)(presg3)
        rc = lib().orc_getup(self.h, _p(U), _p(P), _p(HH), _p(sgsvis), ntime, dt, a, b)
        if rc != 0:
            raise RuntimeError(f"orc_getup failed: {rc}")
        return a[0], b[0]

    def project(self, U):
        lib().orc_project(self.h, _p(U))

    def bcond(self, U):
        lib().orc_bcond(self.h, _p(U))

    def getdp(self, RDP):
        DP = np.zeros_like(RDP, order="F")
        lib().orc_getdp(self.h, _p(RDP), _p(DP))
        return DP

    def rhsdp(self, UH, dt):
        RDP = self.grid.zeros_p()
        lib().orc_rhsdp(self.h, _p(UH), dt, _p(RDP))
        return RDP

    def divcheck(self, U):
        return lib().orc_divcheck(self.h, _p(U))

    def cfl(self, U):
        return lib().orc_cfl(self.h, _p(U))

    def chkmf(self, U):
        f1 = (ctypes.c_double * 1)()
        f3 = (ctypes.c_double * 1)()
        lib().orc_chkmf(self.h, _p(U), f1, f3)
        return f1[0], f3[0]

    def wallss(self, U):
        w = (ctypes.c_double * 3)()
        lib().orc_wallss(self.h, _p(U), w)
        return np.array(w[:])

    def plane_stats(self, U, P):
        """ENERGY's plane statistics (N2M, 29); columns as c3d_plane_stats."""
        out = np.zeros(self.grid.n2m * 29)
        lib().orc_plane_stats(self.h, _p(U), _p(P), _p(out))
        return out.reshape(self.grid.n2m, 29)

    def plane_spectra(self, U, vmo=None):
        """ENERGY's spectra and correlations: dict of Fortran (N, N2M, 3) arrays xspec,
        zspec (N1M / N3M wavenumbers), rxx, rzz, rxy; vmo (N2M, 3) or None."""
        g = self.grid
        out = {k: np.zeros((n, g.n2m, 3), order="F") for k, n in
               (("xspec", g.n1m), ("zspec", g.n3m), ("rxx", g.n1m), ("rzz", g.n3m), ("rxy", g.n1m))}
        v = None if vmo is None else np.asfortranarray(vmo, dtype=np.float64)
        lib().orc_plane_spectra(self.h, _p(U), _p(v), *(_p(out[k]) for k in ("xspec", "zspec", "rxx", "rzz", "rxy")))
        return out

    def plane_quadrants(self, U, vmp=None):
        """ENERGY's quadrant analysis: (N2M, 8), Q(J,1..4) then QP(J,1..4)."""
        out = np.zeros(self.grid.n2m * 8)
        v = None if vmp is None else np.asfortranarray(vmp, dtype=np.float64)
        lib().orc_plane_quadrants(self.h, _p(U), _p(v), _p(out))
        return out.reshape(self.grid.n2m, 8)

    def wall_spectrum(self, utau):
        """SPECTAUW(1:N1M, 1:N3M, 1) of the oracle's current bottom-wall TAUW."""
        out = np.zeros((self.grid.n1m, self.grid.n3m), order="F")
        lib().orc_wall_spectrum(self.h, float(utau), _p(out.reshape(-1, order="F")))
        return out

    def corr3d(self, U):
        """RXYZ(1:N1M, 1:N2M, 1:N3M, 3)."""
        g = self.grid
        out = np.zeros((g.n1m, g.n2m, g.n3m, 3), order="F")
        lib().orc_corr3d(self.h, _p(U), _p(out.reshape(-1, order="F")))
        return out

    def set_cflmax(self, cflmax):
        lib().orc_set_cflmax(self.h, float(cflmax))

    def get_iwm(self):
        """WALLMODEL_IWMLES_SMOOTH's per-point state, (slots, N3M, N1M)."""
        g = self.grid
        out = np.zeros(lib().orc_iwm_slots() * g.n1m * g.n3m)
        lib().orc_get_iwm(self.h, _p(out))
        return out.reshape(-1, g.n3m, g.n1m)

    def particles_advance(self, U, par, dt, diam=0.0002, dens=2220.0, hhh=0.05):
        """One CALC_UX_4RK + BC_PAR step of particles par (N, 6): returns (par, impact)."""
        p = np.ascontiguousarray(par, dtype=np.float64).copy()
        imp = np.zeros(len(p), dtype=np.int32)
        lib().orc_particles_advance(self.h, _p(U), len(p), _p(p.reshape(-1)), diam, dens, hhh, dt,
                                    imp.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        return p, imp

    def particles_source(self, U, par, diam=0.0002, dens=2220.0, hhh=0.05):
        """SOURCE_PAR's terms: (RUH1, RUH2, RUH3), each a Fortran (0:M1,0:M2,0:M3) array."""
        p = np.ascontiguousarray(par, dtype=np.float64)
        out = [self.grid.zeros_s() for _ in range(3)]
        lib().orc_particles_source(self.h, _p(U), len(p), _p(p.reshape(-1)), diam, dens, hhh, *(_p(o) for o in out))
        return out

    def diagnose(self, U):
        f1, f3 = self.chkmf(U)
        return dict(divmax=self.divcheck(U), cflm=self.cfl(U), flow1=f1, flow3=f3,
                    wsm=self.wallss(U))

    # ---- LES: SGS models and the wall model (FILES != 0) ----
    def sgs(self, U):
        """SGSDY / SGSCS on U: returns (SGSVIS(0:M1,0:M2,0:M3), SMAGC(1:N2M))."""
        g = self.grid
        S = g.zeros_s()
        sm = np.zeros(g.n2m)
        rc = lib().orc_sgs(self.h, _p(U), _p(S), _p(sm))
        if rc != 0:
            raise RuntimeError(f"orc_sgs failed: {rc}")
        return S, sm

    def sgs_rhs(self, U, sgsvis):
        """The SGS-flux terms RHS1/2/3 subtract from HH, for a given SGSVIS."""
        HH = self.grid.zeros_u()
        lib().orc_sgs_rhs(self.h, _p(U), _p(sgsvis), _p(HH))
        return HH

    def operator(self, op: int, F):
        """The operator `op` (C3D_OP_* numbering) on F(0:M1,0:M2,0:M3)."""
        X = self.grid.zeros_s()
        rc = lib().orc_operator(self.h, int(op), _p(np.asfortranarray(F)), _p(X))
        if rc != 0:
            raise RuntimeError(f"orc_operator failed: {rc}")
        return X

    def wallmodel(self, U):
        """The grid's wall model (WMODEL 1: WALLMODEL_INSTANT, 3: MARUSIC1, 4:
        WALLMODEL_WERNER, 5: PIOMELLI) on U; returns the status (0, -4 if an INSTANT point
        hit the iteration cap, -1 if a shifted point found no cell)."""
        return lib().orc_wallmodel(self.h, _p(U))

    def get_beta(self):
        """SGSSD's scale-dependence BETA(1:N2M) of the last SGS evaluation (unclipped)."""
        b = np.zeros(self.grid.n2m)
        lib().orc_get_beta(self.h, _p(b))
        return b

    def filter(self, F, four=False):
        """FILTER (or FILTER4) of fields F (n, N3M, N1M) (x fastest); returns a copy."""
        F = np.ascontiguousarray(F, dtype=np.float64).copy()
        lib().orc_filter(self.h, int(four), _p(F.reshape(-1)), F.shape[0])
        return F

    def set_wall(self, tauw=None, taub=None, ifwall=0):
        lib().orc_set_wall(self.h, _p(tauw), _p(taub), ifwall)

    def get_wall(self):
        g = self.grid
        tw = np.zeros(g.shape_tau(), order="F")
        tb = np.zeros(g.shape_tau(), order="F")
        w = np.zeros(3)
        lib().orc_get_wall(self.h, _p(tw), _p(tb), _p(w))
        return tw, tb, w

    def set_wsm(self, wsm):
        w = np.ascontiguousarray(wsm, dtype=np.float64)
        lib().orc_set_wsm(self.h, _p(w))

    def set_wall_iter_cap(self, cap: int):
        lib().orc_set_wall_iter_cap(self.h, int(cap))

    def poisson_metrics(self):
        g = self.grid
        ak1 = np.zeros(g.n1m)
        ak3 = np.zeros(g.n3m // 2 + 1)
        pm, pc, pp = (np.zeros(g.n2m) for _ in range(3))
        lib().orc_poisson_metrics(self.h, _p(ak1), _p(ak3), _p(pm), _p(pc), _p(pp))
        return ak1, ak3, pm, pc, pp


def ctdma11(d, a, b, c):
    d = np.ascontiguousarray(d, dtype=np.float64)
    x = np.zeros_like(d)
    lib().orc_ctdma11(len(d), a, b, c, _p(d), _p(x))
    return x


def ctdma_recip(d, a, b, c):
    d = np.ascontiguousarray(d, dtype=np.float64)
    x = np.zeros_like(d)
    lib().orc_ctdma_recip(len(d), a, b, c, _p(d), _p(x))
    return x


def tdmap(a, b, c, r):
    a, b, c, r = (np.ascontiguousarray(v, dtype=np.float64) for v in (a, b, c, r))
    x = np.zeros_like(r)
    lib().orc_tdmap(len(r), _p(a), _p(b), _p(c), _p(r), _p(x))
    return x


def fft(z, sign=-1):
    z = np.ascontiguousarray(z, dtype=np.complex128).copy()
    lib().orc_fft(len(z), z.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), sign)
    return z


def dft2d(z, sign=-1):
    """z: Fortran-order complex array (n1, n3)."""
    z = np.asfortranarray(z, dtype=np.complex128).copy(order="F")
    n1, n3 = z.shape
    lib().orc_dft2d(n1, n3, z.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), sign)
    return z


def dqrrt(pa, eps=1.0e-5):
    """DQRRT/CHHQR: (BETA, eigenvalues as complex, ok) for x^n + pa[0] x^(n-1) + ... + pa[n-1]."""
    pa = np.ascontiguousarray(pa, dtype=np.float64)
    n = len(pa)
    wr, wi = np.zeros(n), np.zeros(n)
    beta = (ctypes.c_double * 1)()
    ok = lib().orc_dqrrt(_p(pa), n, eps, beta, _p(wr), _p(wi))
    return beta[0], wr + 1j * wi, ok


def set_threads(n: int):
    lib().orc_set_threads(n)


def max_threads() -> int:
    return lib().orc_max_threads()
