"""Grid construction for the C-ABI: the driver-side MESH/INDICES metrics.

The Fortran driver computes the wall-normal grid and its finite-difference metrics in
MESH (compact3d.f:302-443) and hands them to the GPU step through ``c3d_grid``.  This
module restates MESH in numpy so that tests, the bench and Python users can build the
same arrays.  The only generalisation is the stretching parameter: the reference
hard-codes ``CKS=2.5`` (compact3d.f:338); here it is the ``cks`` argument (default 2.5).

Named workloads (``WORKLOADS``) carry the channel geometries used by the tests and the
bench: cell counts, domain, stretching, Reynolds number ``RE = 1/nu`` (the reference's
laminar-centreline scaling, so ``Re_bulk = 4/3 RE``) and time step.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

C3D_FP64 = 0
C3D_MIXED = 1
C3D_MIXED_IR = 2


class c3d_grid(ctypes.Structure):
    """ctypes mirror of ``struct c3d_grid`` in include/c3d.h."""

    _fields_ = [
        ("n1", ctypes.c_int), ("n2", ctypes.c_int), ("n3", ctypes.c_int),
        ("alx", ctypes.c_double), ("aly", ctypes.c_double), ("alz", ctypes.c_double),
        ("vol", ctypes.c_double),
        ("dx1", ctypes.c_double), ("dx3", ctypes.c_double),
        ("re", ctypes.c_double),
        ("y", ctypes.POINTER(ctypes.c_double)),
        ("dy", ctypes.POINTER(ctypes.c_double)),
        ("h", ctypes.POINTER(ctypes.c_double)),
        ("hm", ctypes.POINTER(ctypes.c_double)),
        ("hc", ctypes.POINTER(ctypes.c_double)),
        ("hp", ctypes.POINTER(ctypes.c_double)),
        ("dym", ctypes.POINTER(ctypes.c_double)),
        ("dyc", ctypes.POINTER(ctypes.c_double)),
        ("dyp", ctypes.POINTER(ctypes.c_double)),
        ("files", ctypes.c_int),
        ("wmodel", ctypes.c_int),
        ("precision", ctypes.c_int),
    ]


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


@dataclass
class Grid:
    """A channel grid: extents, domain and the MESH metrics (all float64)."""

    n1m: int
    n2m: int
    n3m: int
    alx: float
    aly: float
    alz: float
    re: float
    cks: float = 2.5
    wmodel: int = 0
    files: int = 0
    y0: float = 0.0
    precision: int = C3D_FP64
    arrays: dict = field(default_factory=dict, repr=False)

    def __post_init__(self):
        self.arrays = mesh(self.n1m + 1, self.n2m + 1, self.n3m + 1, self.alx, self.aly,
                           self.alz, self.cks, self.wmodel, self.y0)
        self.aly = self.arrays["aly"]
        self._struct = None

    # Fortran extents M1=N1, M2=N2, M3=N3
    @property
    def n1(self):
        return self.n1m + 1

    @property
    def n2(self):
        return self.n2m + 1

    @property
    def n3(self):
        return self.n3m + 1

    @property
    def points(self) -> int:
        """Grid points advanced per step (N1M*N2M*N3M)."""
        return self.n1m * self.n2m * self.n3m

    def struct(self, precision: int | None = None) -> c3d_grid:
        a = self.arrays
        g = c3d_grid()
        g.n1, g.n2, g.n3 = self.n1, self.n2, self.n3
        g.alx, g.aly, g.alz = self.alx, a["aly"], self.alz
        g.vol = a["vol"]
        g.dx1, g.dx3 = a["dx1"], a["dx3"]
        g.re = self.re
        for name in ("y", "dy", "h", "hm", "hc", "hp", "dym", "dyc", "dyp"):
            setattr(g, name, _dptr(a[name]))
        g.files = self.files
        g.wmodel = self.wmodel
        g.precision = self.precision if precision is None else precision
        self._struct = g   # keep alive with the arrays it points to
        return g

    # Fortran array shapes (column-major)
    def shape_u(self):
        return (self.n1 + 1, self.n2 + 1, self.n3 + 1, 3)

    def shape_p(self):
        return (self.n1, self.n2, self.n3)

    def shape_s(self):
        return (self.n1 + 1, self.n2 + 1, self.n3 + 1)

    def shape_tau(self):
        return (self.n1 + 1, self.n3 + 1, 2)

    def zeros_u(self):
        return np.zeros(self.shape_u(), dtype=np.float64, order="F")

    def zeros_p(self):
        return np.zeros(self.shape_p(), dtype=np.float64, order="F")

    def zeros_s(self):
        return np.zeros(self.shape_s(), dtype=np.float64, order="F")


def mesh(n1: int, n2: int, n3: int, alx: float, aly: float, alz: float,
         cks: float = 2.5, wmodel: int = 0, y0: float = 0.0) -> dict:
    """MESH (compact3d.f:302-443) for points N1, N2, N3.

    Returns Y(0:N2) and DY(0:N2) as length-(N2+1) arrays indexed like Fortran, and
    H, HM, HC, HP, DYM, DYC, DYP(1:N2) as length-N2 arrays (Fortran J at index J-1).
    Entries the reference never assigns (DY(0), DY(N2), HP(N2), ...) are zero, as in a
    zero-initialised COMMON block.
    """
    n1m, n2m, n3m = n1 - 1, n2 - 1, n3 - 1
    Y = np.zeros(n2 + 1)
    Y[0] = 0.0 if wmodel == 0 else y0
    for J in range(1, n2 + 1):
        if wmodel == 0:
            if aly == 2.0:
                Y[J] = 1 - math.tanh(cks * (1 - aly * (J - 1) / (n2 - 1))) / math.tanh(cks)
            else:
                Y[J] = 1 - math.tanh(cks * (1 - 2.0 * aly * (J - 1) / (2 * n2 - 1))) / math.tanh(cks)
        else:
            Y[J] = (aly - y0) * (J - 1) / (n2 - 1) + y0
    aly = Y[n2]
    vol = alx * aly * alz
    dx1 = float(n1m) / alx
    dx3 = float(n3m) / alz
    DY = np.zeros(n2 + 1)
    H = np.zeros(n2 + 1)
    HP = np.zeros(n2 + 1)
    HC = np.zeros(n2 + 1)
    HM = np.zeros(n2 + 1)
    DYP = np.zeros(n2 + 1)
    DYC = np.zeros(n2 + 1)
    DYM = np.zeros(n2 + 1)
    DY[1] = Y[2]
    for J in range(2, n2m + 1):
        DY[J] = Y[J + 1] - Y[J]
        H[J] = 0.5 * (DY[J] + DY[J - 1])
    H[1] = 0.5 * DY[1]
    H[n2] = 0.5 * DY[n2m]
    for J in range(2, n2m):
        HP[J] = 1.0 / H[J + 1] / DY[J]
        HC[J] = (H[J + 1] + H[J]) / H[J + 1] / H[J] / DY[J]
        HM[J] = 1.0 / H[J] / DY[J]
    HP[1] = 4.0 * H[1] / H[2] / (H[1] + H[2]) / DY[1]
    HC[1] = 4.0 / H[2] / DY[1]
    HM[1] = 4.0 / (H[1] + H[2]) / DY[1]
    HP[n2m] = 4.0 / (H[n2m] + H[n2]) / DY[n2m]
    HC[n2m] = 4.0 / H[n2m] / DY[n2m]
    HM[n2m] = 4.0 * H[n2] / H[n2m] / (H[n2m] + H[n2]) / DY[n2m]
    if wmodel != 0:
        HP[1] = 1.0 / H[2] / DY[1]
        HC[1] = 1.0 / H[2] / DY[1]
        HM[1] = 0.0
        HP[n2m] = 0.0
        HC[n2m] = 1.0 / H[n2m] / DY[n2m]
        HM[n2m] = 1.0 / H[n2m] / DY[n2m]
    for J in range(2, n2m + 1):
        DYP[J] = 1.0 / H[J] / DY[J]
        DYC[J] = 1.0 / H[J] * (1.0 / DY[J] + 1.0 / DY[J - 1])
        DYM[J] = 1.0 / H[J] / DY[J - 1]
    one = lambda a: np.ascontiguousarray(a[1:n2 + 1])
    return dict(y=Y, dy=DY, h=one(H), hm=one(HM), hc=one(HC), hp=one(HP),
                dym=one(DYM), dyc=one(DYC), dyp=one(DYP), aly=float(aly), vol=float(vol),
                dx1=dx1, dx3=dx3)


def re_from_retau(ret: float) -> float:
    """RE (=1/nu, laminar-centreline scaling) for a target Re_tau from the reference's
    own estimate RET = 0.09*RE**0.88 (compact3d.f:618)."""
    return (ret / 0.09) ** (1.0 / 0.88)


PI = math.pi

# Channel workloads.  Cells are N1M x N2M x N3M; Re_bulk(2h) = 4/3 RE (the laminar bulk
# velocity of the unit-centreline profile is 2/3).
WORKLOADS = {
    # 64 x 65 x 64 points, 4pi x 2 x 4/3 pi, beta=2.0, Re_bulk=5600 -> RE=4200, dt=0.002
    "channel64": dict(n1m=64, n2m=64, n3m=64, alx=4 * PI, aly=2.0, alz=4 * PI / 3, cks=2.0,
                      re=4200.0, dt=0.002),
    # 256 x 193 x 256 points (operator workload), same domain and stretching
    "field256": dict(n1m=256, n2m=192, n3m=256, alx=4 * PI, aly=2.0, alz=4 * PI / 3, cks=2.0,
                     re=4200.0, dt=0.002),
    # 384 x 257 x 384 points, 2pi x 2 x pi, beta=2.2, Re_bulk=20000 -> RE=15000, dt=0.001
    "channel384": dict(n1m=384, n2m=256, n3m=384, alx=2 * PI, aly=2.0, alz=PI, cks=2.2,
                       re=15000.0, dt=0.001),
    # wall-modelled LES: 128 x 65 x 128 points, 8pi x 2 x 3pi, uniform y (wall model)
    "les128": dict(n1m=128, n2m=64, n3m=128, alx=8 * PI, aly=2.0, alz=3 * PI, cks=1.0,
                   re=round(re_from_retau(2000.0), 1), dt=0.005, wmodel=1, files=2),
    # small wall-modelled LES grids for parity tests (Smagorinsky and dynamic)
    "les32cs": dict(n1m=32, n2m=16, n3m=32, alx=8 * PI, aly=2.0, alz=3 * PI, cks=1.0,
                    re=round(re_from_retau(2000.0), 1), dt=0.002, wmodel=1, files=2),
    "les32dy": dict(n1m=32, n2m=16, n3m=32, alx=8 * PI, aly=2.0, alz=3 * PI, cks=1.0,
                    re=round(re_from_retau(2000.0), 1), dt=0.002, wmodel=1, files=1),
    # small grids for parity tests
    "tiny16": dict(n1m=16, n2m=16, n3m=16, alx=2 * PI, aly=2.0, alz=PI, cks=2.0,
                   re=1000.0, dt=0.002),
    "small32": dict(n1m=32, n2m=24, n3m=48, alx=2 * PI, aly=2.0, alz=PI, cks=2.0,
                    re=2000.0, dt=0.002),
}


def make_grid(name: str, precision: int = C3D_FP64, **over) -> tuple[Grid, float]:
    """Grid and dt of a named workload; keyword overrides replace its entries."""
    w = dict(WORKLOADS[name])
    w.update(over)
    dt = w.pop("dt")
    g = Grid(n1m=w["n1m"], n2m=w["n2m"], n3m=w["n3m"], alx=w["alx"], aly=w["aly"],
             alz=w["alz"], re=w["re"], cks=w.get("cks", 2.5), wmodel=w.get("wmodel", 0),
             files=w.get("files", 0), precision=precision, y0=w.get("y0", 0.0))
    return g, dt
