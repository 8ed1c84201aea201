"""TEST INFRASTRUCTURE ONLY: the reference's own Fortran routines, translated to C by
``oracle/f77c.py`` and compiled with gcc, driven through ctypes.

No Fortran compiler exists on this machine or on the GPU machine, so the reference's
GETUP (compact3d.f:879-960) and everything it calls, MESH, INDICES, INIWAVE and the
per-step diagnostics run here as a mechanical C translation of compact3d.f (an ``-r8``
build: REAL is 8 bytes).  FFTW, which GETDP calls and which the reference neither vendors
nor pins, is replaced by ``oracle/fftw_shim.c`` (the DFT FFTW documents, summed
directly).  The reference's extents are compile-time PARAMETERs (PARAM.H), so one
library is built per grid: ``oracle/_ref/ref_<M1>_<M2>_<M3>.{c,json,so}``.

The translation needs the reference source (``C3D_REFERENCE_DIR``, default the
reference checkout); where it is absent, a translation made earlier is compiled if it is
there, and ``available()`` is False otherwise.  Only tests use this module, as a checker
of the oracle restatement and of the fixtures under tests/golden/.
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_DIR = os.environ.get("C3D_REFERENCE_DIR", "/root/reference")
SOURCE = os.path.join(REF_DIR, "compact3d.f")
ROOTS = ["GETUP", "DIVCHECK", "CFL", "CHKMF", "WALLSS", "MESH", "INDICES", "INIWAVE"]
CT = {"R": ctypes.c_double, "I": ctypes.c_int, "I8": ctypes.c_longlong, "L": ctypes.c_int, "F": ctypes.c_float}
NP = {"R": np.float64, "I": np.int32, "I8": np.int64, "L": np.int32, "F": np.float32, "C": np.complex128}


def _paths(m1, m2, m3, omp=False):
    base = os.path.join(OUT, f"ref{'_omp' if omp else ''}_{m1}_{m2}_{m3}")
    return base + ".c", base + ".json", base + ".so"


def available(m1: int = 17, m2: int = 17, m3: int = 17, omp: bool = False) -> bool:
    c, j, _ = _paths(m1, m2, m3, omp)
    return os.path.exists(SOURCE) or (os.path.exists(c) and os.path.exists(j))


def build(m1: int, m2: int, m3: int, omp: bool = False) -> str:
    """Translate (when the reference source is here) and compile the library for
    PARAMETER (M1=m1, M2=m2, M3=m3).  With `omp` the reference's !$OMP PARALLEL DO
    directives become OpenMP loops (locals per call, as a recursive build has them) and
    the library is compiled with -fopenmp: the reference's own OpenMP CPU path, for
    timing; without, one thread, locals kept between calls (the tests' form)."""
    from . import f77c
    os.makedirs(OUT, exist_ok=True)
    c, j, so = _paths(m1, m2, m3, omp)
    shim = os.path.join(HERE, "fftw_shim.c")
    if os.path.exists(SOURCE):
        deps = [SOURCE, os.path.join(HERE, "f77c.py")]
        if not os.path.exists(c) or any(os.path.getmtime(d) > os.path.getmtime(c) for d in deps):
            f77c.translate(SOURCE, c + ".tmp.c", m1, m2, m3, ROOTS, omp=omp)
            os.replace(c + ".tmp.c", c)
            os.replace(c + ".tmp.json", j)
    if not os.path.exists(c):
        raise FileNotFoundError(f"no reference source ({SOURCE}) and no earlier translation ({c})")
    if not os.path.exists(so) or any(os.path.getmtime(d) > os.path.getmtime(so) for d in (c, shim)):
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=gnu11", "-w"]
        if omp:
            cmd.append("-fopenmp")
        subprocess.check_call(cmd + ["-o", so + ".tmp", c, shim, "-lm"])
        os.replace(so + ".tmp", so)
    return so


# PARAMETER extents of the grids the tests compare on (tiny16 and the les16 fixture, small32,
# the les32 grids)
TEST_EXTENTS = [(17, 17, 17), (33, 25, 49), (33, 17, 33)]


# PARAMETER extents of the benchmark's reference arm (channel384), built with OpenMP
ARM_EXTENTS = [(385, 257, 385)]


def build_for_tests():
    """Builds the libraries of TEST_EXTENTS and, with OpenMP, of ARM_EXTENTS (in parallel)
    where the reference source or an earlier translation is present; returns the paths."""
    import concurrent.futures as cf
    todo = [(m, False) for m in TEST_EXTENTS if available(*m)]
    todo += [(m, True) for m in ARM_EXTENTS if available(*m, omp=True)]
    with cf.ThreadPoolExecutor(max_workers=max(1, len(todo))) as ex:
        return list(ex.map(lambda t: build(*t[0], omp=t[1]), todo))


def _dp(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class RefChannel:
    """The reference's COMMON state for one grid and its GETUP and diagnostics.

    The mesh metrics come from ``grid.arrays`` (the same values the oracle and the GPU
    library are given), so grids with any stretching can be compared; ``reference_mesh``
    runs the reference's own MESH instead (CKS = 2.5 as compact3d.f hard-codes it)."""

    def __init__(self, grid, reference_mesh: bool = False, omp: bool = False):
        self.g = g = grid
        self.m = (g.n1, g.n2, g.n3)
        self.omp = omp
        self._runner = None
        if omp:
            # the OpenMP build keeps its per-call arrays on the stack, as a recursive Fortran
            # build does: its calls run on a thread with a 1 GiB stack, its worker threads get
            # OMP_STACKSIZE (effective when the OpenMP runtime has not started yet)
            os.environ.setdefault("OMP_STACKSIZE", "64M")
            import concurrent.futures as cf
            import threading
            old = threading.stack_size()
            threading.stack_size(1 << 30)
            try:
                self._runner = cf.ThreadPoolExecutor(max_workers=1)
                self._runner.submit(lambda: None).result()
            finally:
                threading.stack_size(old)
        so = build(*self.m, omp=omp)
        self.lib = ctypes.CDLL(so)
        self.layout = json.load(open(_paths(*self.m, omp)[1]))["layout"]
        self.set("DIM", N1=g.n1, N2=g.n2, N3=g.n3, N1M=g.n1m, N2M=g.n2m, N3M=g.n3m)
        self.set("SIZE", ALX=g.alx, ALY=2.0 if g.aly > 1.5 else 1.0, ALZ=g.alz)
        self.set("PARA", RE=g.re)
        self.set("FINOUT", FILES=float(g.files))
        self.set("WALLMODEL", WMODEL=float(g.wmodel))
        self.set("ROUGHNESS", Y0=g.y0)
        self.set("TSTEP", CFLMAX=1.0)
        self.lib.f77_MESH()            # MESH02 (cell faces and centres), MESH1, and the y grid at CKS = 2.5
        if not reference_mesh:
            a = g.arrays
            self.view("MESH2", "Y")[:] = a["y"]
            dy = self.view("MESH3", "DY")
            dy[:] = a["dy"]
            for nm in ("H", "HM", "HC", "HP"):
                self.view("MESH3", nm)[:] = a[nm.lower()]
            for nm in ("DYM", "DYC", "DYP"):
                self.view("MESH4", nm)[:] = a[nm.lower()]
            self.set("SIZE", ALY=a["aly"], VOL=a["vol"])
            y = a["y"]
            self.view("MESH02", "YG")[1:] = y[1:]
            yc = self.view("MESH02", "YC")
            yc[1:g.n2m + 1] = 0.5 * (y[2:g.n2 + 1] + y[1:g.n2])
            yc[g.n2] = y[g.n2]
        self.lib.f77_INDICES()
        self.lib.f77_INIWAVE()

    # ---- COMMON access ----
    def _var(self, block, name):
        for v in self.layout[block]["vars"]:
            if v["name"] == name:
                return v
        raise KeyError(f"/{block}/ {name}")

    def view(self, block, name):
        """A numpy view of a COMMON variable (Fortran order, its declared bounds)."""
        v = self._var(block, name)
        base = ctypes.c_void_p.in_dll(self.lib, f"f77c_{block}").value   # the block's memory
        shape = tuple(hi - lo + 1 for lo, hi in v["dims"]) or (1,)
        n = int(np.prod(shape))
        dt = np.dtype(NP[v["type"]])
        buf = (ctypes.c_ubyte * (n * dt.itemsize)).from_address(base + v["offset"])
        return np.ndarray(shape, dtype=dt, buffer=buf, order="F")

    def set(self, block, **vals):
        for k, x in vals.items():
            self.view(block, k)[...] = x

    def get(self, block, name):
        a = self.view(block, name)
        return a.copy() if a.size > 1 else a.reshape(-1)[0].item()

    # ---- the reference's routines ----
    def getup(self, U, P, HH, ntime, dt, presg, presg3, sgsvis=None):
        g = self.g
        for a in (U, P, HH):
            assert a.dtype == np.float64 and a.flags.f_contiguous
        self.set("TSTEP", DT=dt)
        if not hasattr(self, "_ss"):
            self._ss = g.zeros_u()
        S = sgsvis if sgsvis is not None else g.zeros_s()
        pg = ctypes.c_double(presg)
        pg3 = ctypes.c_double(presg3)
        nt = ctypes.c_int(ntime)
        if g.wmodel == 0:
            # MAIN calls WALLSS before GETUP when there is no wall model (compact3d.f:125):
            # the SGS models' van Driest damping reads its WSM
            t = ctypes.c_double(0.0)
            if self._runner is not None:
                self._runner.submit(self.lib.f77_WALLSS, _dp(U), _dp(P), ctypes.byref(t)).result()
            else:
                self.lib.f77_WALLSS(_dp(U), _dp(P), ctypes.byref(t))
        args = (_dp(U), _dp(P), _dp(HH), _dp(self._ss), ctypes.byref(nt), ctypes.byref(pg), ctypes.byref(pg3), _dp(S))
        if self._runner is not None:
            self._runner.submit(self.lib.f77_GETUP, *args).result()
        else:
            self.lib.f77_GETUP(*args)
        return pg.value, pg3.value

    def divcheck(self, U):
        t = ctypes.c_double(0.0)
        d = ctypes.c_double(0.0)
        n = ctypes.c_int(1)
        self.lib.f77_DIVCHECK(_dp(U), ctypes.byref(t), ctypes.byref(d), ctypes.byref(n))
        return d.value

    def cfl(self, U):
        c = ctypes.c_double(0.0)
        self.lib.f77_CFL(_dp(U), ctypes.byref(c))
        return c.value

    def chkmf(self, U):
        t = ctypes.c_double(0.0)
        self.lib.f77_CHKMF(_dp(U), ctypes.byref(t))
        return self.get("FLOWRATE", "FLOW1"), self.get("FLOWRATE", "FLOW3")

    def wallss(self, U, P):
        t = ctypes.c_double(0.0)
        self.lib.f77_WALLSS(_dp(U), _dp(P), ctypes.byref(t))
        return self.view("WSMEM", "WSM").copy()

    def mesh(self):
        """The reference MESH's metrics in the layout of compact3d_gb300.grid.mesh."""
        g = self.g
        out = dict(y=self.view("MESH2", "Y").copy(), dy=self.view("MESH3", "DY").copy())
        for nm in ("H", "HM", "HC", "HP"):
            out[nm.lower()] = self.view("MESH3", nm).copy()[:g.n2]
        for nm in ("DYM", "DYC", "DYP"):
            out[nm.lower()] = self.view("MESH4", nm).copy()[:g.n2]
        out["aly"] = self.get("SIZE", "ALY")
        out["vol"] = self.get("SIZE", "VOL")
        out["dx1"] = self.get("MESH1", "DX1")
        out["dx3"] = self.get("MESH1", "DX3")
        return out

    def poisson_metrics(self):
        g = self.g
        return dict(ak1=self.view("WAVK13", "AK1").copy()[:g.n1m], ak3=self.view("WAVK13", "AK3").copy()[:g.n3m // 2 + 1],
                    pmj=self.view("METPOI", "PMJ").copy()[:g.n2m], pcj=self.view("METPOI", "PCJ").copy()[:g.n2m],
                    ppj=self.view("METPOI", "PPJ").copy()[:g.n2m])

    # LES state
    def set_wall(self, tauw, taub):
        self.view("TAUXYZ", "TAUW")[...] = tauw
        self.view("TAUXYZ", "TAUB")[...] = taub

    def get_wall(self):
        return self.view("TAUXYZ", "TAUW").copy(), self.view("TAUXYZ", "TAUB").copy(), self.view("WSMEM", "WSM").copy()

    def set_wsm(self, wsm):
        self.view("WSMEM", "WSM")[...] = wsm
