"""Problem description (the reference's grid + inputs module state) and synthetic workloads.

A :class:`Problem` holds what the reference keeps in ``inputs`` and ``globe_data`` for one grid:
per-cell material properties (``heatblock``, src/heatflow/mod_constructions.f90:25-31), the
boundary block and the time-stepping flags (src/heatflow/mod_inputs.f90:80-107).  Arrays are in
cell order I = ix + nx*(iy + ny*iz), x fastest.

The workload builders reproduce the synthetic inputs used for parity and measurement (seeded
numpy generators; no external data).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import abi


@dataclass
class Problem:
    nx: int
    ny: int
    nz: int
    lx: float
    ly: float
    lz: float
    kappa: np.ndarray
    rho: np.ndarray
    heat_capacity: np.ndarray
    tau: np.ndarray
    em: Optional[np.ndarray] = None
    iheater: Optional[np.ndarray] = None
    power: Optional[np.ndarray] = None
    power_in: float = 0.0
    freq: float = 1.0
    time_step: float = 1.0
    heated_steps: int = 0
    icattaneo: int = 1
    isteady: int = 0
    periodic: Sequence[int] = (0, 0, 0)
    cg_face: Sequence[int] = (0, 0, 0, 0, 0, 0)
    kappa_bound: Sequence[float] = (0.0,) * 6
    t_bath_face: Sequence[float] = (0.0,) * 6
    t_bath: float = 0.0
    t_bath_cg: float = 0.0
    br: float = 1.0
    qdens_mode: int = abi.HF_QDENS_HEATED_VOLUME
    t_system: float = 300.0          # initial temperature (initial_evolve, mod_init_evolve.f90:47)
    _keep: list = field(default_factory=list, repr=False)

    @property
    def ncells(self) -> int:
        return self.nx * self.ny * self.nz

    def __post_init__(self):
        n = self.ncells
        for name in ("kappa", "rho", "heat_capacity", "tau"):
            a = np.ascontiguousarray(np.broadcast_to(np.asarray(getattr(self, name), np.float64), (n,)))
            setattr(self, name, a)
        if self.em is not None:
            self.em = np.ascontiguousarray(np.broadcast_to(np.asarray(self.em, np.float64), (n,)))
        if self.iheater is not None:
            self.iheater = np.ascontiguousarray(np.broadcast_to(np.asarray(self.iheater, np.int64), (n,)))
        if self.power is not None:
            self.power = np.ascontiguousarray(np.broadcast_to(np.asarray(self.power, np.float64), (n,)))

    def to_c(self) -> abi.HfProblem:
        """Fill an hf_problem; the arrays stay owned by this object."""
        def dp(a):
            return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))

        def ip(a):
            return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int64))

        p = abi.HfProblem()
        p.nx, p.ny, p.nz = self.nx, self.ny, self.nz
        p.lx, p.ly, p.lz = self.lx, self.ly, self.lz
        p.kappa, p.rho, p.heat_capacity, p.tau = dp(self.kappa), dp(self.rho), dp(self.heat_capacity), dp(self.tau)
        p.em, p.iheater, p.power = dp(self.em), ip(self.iheater), dp(self.power)
        p.power_in, p.freq, p.time_step = self.power_in, self.freq, self.time_step
        p.heated_steps = int(self.heated_steps)
        p.icattaneo, p.isteady = int(self.icattaneo), int(self.isteady)
        for a in range(3):
            p.periodic[a] = int(self.periodic[a])
        for f in range(6):
            p.cg_face[f] = int(self.cg_face[f])
            p.kappa_bound[f] = float(self.kappa_bound[f])
            p.t_bath_face[f] = float(self.t_bath_face[f])
        p.t_bath, p.t_bath_cg, p.br = self.t_bath, self.t_bath_cg, self.br
        p.qdens_mode = int(self.qdens_mode)
        return p

    def initial_state(self):
        t = np.full(self.ncells, self.t_system, dtype=np.float64)
        return t.copy(), t.copy()


# ---------------------------------------------------------------------------------------------
# Materials used by the synthetic workloads
SILICON = dict(kappa=149.0, rho=2329.0, heat_capacity=710.0, tau=1e-12)
POLYMER = dict(kappa=0.2, rho=1190.0, heat_capacity=1200.0, tau=1e-12)


def _dirichlet(p_kappa_bound: float, t: float = 300.0):
    return dict(kappa_bound=(p_kappa_bound,) * 6, t_bath_face=(t,) * 6, t_bath=t)


def point_source_cube(n: int = 20, *, icattaneo: int = 1, power_in: float = 1e-6,
                      dx: float = 1e-9, dt: float = 1e-13) -> Problem:
    """Plain Cattaneo cube: one silicon-like material, 300 K Dirichlet on all faces, constant
    point source at the centre cell (n//2 in every axis, 0-based), dt = 1e-13 s."""
    N = n ** 3
    ih = np.zeros(N, np.int64)
    c = n // 2 - 1 if n % 2 == 0 else n // 2   # 1-based centre (10,10,10) of a 20^3 grid
    ih[c + n * (c + n * c)] = 1
    return Problem(nx=n, ny=n, nz=n, lx=n * dx, ly=n * dx, lz=n * dx,
                   kappa=SILICON["kappa"], rho=SILICON["rho"], heat_capacity=SILICON["heat_capacity"],
                   tau=SILICON["tau"], em=0.0, iheater=ih, power_in=power_in, time_step=dt,
                   icattaneo=icattaneo, **_dirichlet(149.0))


def layered_slab(n: int = 128, *, icattaneo: int = 1, layer: int = 16, peak: float = 1e-5,
                 sigma: float = 5.0, dx: float = 1e-9, dt: float = 1e-13,
                 nz: Optional[int] = None) -> Problem:
    """Two-material layered slab: z-layers alternating every `layer` cells between silicon-like
    (kappa 149) and polymer-like (kappa 0.2, rho 1190, c 1200) material, Dirichlet 300 K on all
    faces (boundary kappa 149), Gaussian heating over the top face (iz = nz-1): per-cell power
    peak*exp(-r^2/(2 sigma^2)) around the face centre, each cell's own volume as density."""
    nz = n if nz is None else nz
    nx = ny = n
    N = nx * ny * nz
    iz = np.repeat(np.arange(nz), nx * ny)
    poly = (iz // layer) % 2 == 1
    kappa = np.where(poly, POLYMER["kappa"], SILICON["kappa"])
    rho = np.where(poly, POLYMER["rho"], SILICON["rho"])
    hc = np.where(poly, POLYMER["heat_capacity"], SILICON["heat_capacity"])
    tau = np.full(N, 1e-12)
    ix = np.tile(np.arange(nx), ny * nz)
    iy = np.tile(np.repeat(np.arange(ny), nx), nz)
    r2 = (ix - (nx - 1) / 2.0) ** 2 + (iy - (ny - 1) / 2.0) ** 2
    top = iz == nz - 1
    power = np.where(top, peak * np.exp(-r2 / (2 * sigma * sigma)), 0.0)
    ih = np.where(top, 1, 0).astype(np.int64)
    return Problem(nx=nx, ny=ny, nz=nz, lx=nx * dx, ly=ny * dx, lz=nz * dx,
                   kappa=kappa, rho=rho, heat_capacity=hc, tau=tau, em=0.0, iheater=ih,
                   power=power, time_step=dt, icattaneo=icattaneo,
                   qdens_mode=abi.HF_QDENS_CELL_VOLUME, **_dirichlet(149.0))


def random_instance(rng: np.random.Generator, *, lo: int = 16, hi: int = 96, dx: float = 1e-9,
                    dt: float = 1e-13) -> Problem:
    """One instance of the batched sweep: edges U{lo..hi} per axis, kappa lognormal (median 50,
    sigma 1.0), rho*c U[1e6, 3e6] (c = 1000), tau 1e-12, 1-4 point sources of U[1e-7, 1e-5] W,
    Dirichlet 300 K (boundary kappa 50)."""
    nx, ny, nz = (int(v) for v in rng.integers(lo, hi + 1, size=3))
    N = nx * ny * nz
    kappa = np.exp(np.log(50.0) + 1.0 * rng.standard_normal(N))
    rhoc = rng.uniform(1e6, 3e6, size=N)
    ns = int(rng.integers(1, 5))
    cells = rng.choice(N, size=ns, replace=False)
    power = np.zeros(N)
    power[cells] = rng.uniform(1e-7, 1e-5, size=ns)
    ih = np.zeros(N, np.int64)
    ih[cells] = 1
    return Problem(nx=nx, ny=ny, nz=nz, lx=nx * dx, ly=ny * dx, lz=nz * dx, kappa=kappa,
                   rho=rhoc / 1000.0, heat_capacity=1000.0, tau=1e-12, em=0.0, iheater=ih,
                   power=power, time_step=dt, icattaneo=1, qdens_mode=abi.HF_QDENS_CELL_VOLUME,
                   **_dirichlet(50.0))


def batched_sweep(count: int = 256, seed: int = 0, **kw) -> list[Problem]:
    rng = np.random.default_rng(seed)
    return [random_instance(rng, **kw) for _ in range(count)]


def inclusions(n: int = 512, *, frac: float = 0.05, rmin: int = 3, rmax: int = 10, seed: int = 0,
               heated_layers: int = 8, power_per_cell: float = 1e-9, dx: float = 1e-9,
               dt: float = 1e-13) -> Problem:
    """Large single grid with random spherical polymer inclusions (radius U{rmin..rmax}) in a
    silicon-like matrix until `frac` of the cells are polymer; periodic x/y, Dirichlet z;
    heater case 1 on the bottom `heated_layers` layers with the reference's total-power
    semantics (power_in = power_per_cell * heated cells, divided by the heated volume)."""
    rng = np.random.default_rng(seed)
    poly = np.zeros((n, n, n), dtype=bool)   # [z][y][x]
    target = frac * n ** 3
    count = 0
    while count < target:
        r = int(rng.integers(rmin, rmax + 1))
        cz, cy, cx = (int(v) for v in rng.integers(0, n, size=3))
        zs, ys, xs = np.ogrid[-r:r + 1, -r:r + 1, -r:r + 1]
        ball = zs * zs + ys * ys + xs * xs <= r * r
        z0, y0, x0 = cz - r, cy - r, cx - r
        zi = np.arange(z0, z0 + 2 * r + 1)
        keep_z = (zi >= 0) & (zi < n)
        yi = (np.arange(y0, y0 + 2 * r + 1)) % n
        xi = (np.arange(x0, x0 + 2 * r + 1)) % n
        sub = poly[np.ix_(zi[keep_z], yi, xi)]
        new = sub | ball[keep_z]
        count += int(new.sum() - sub.sum())
        poly[np.ix_(zi[keep_z], yi, xi)] = new
    poly = poly.reshape(-1)
    kappa = np.where(poly, POLYMER["kappa"], SILICON["kappa"])
    rho = np.where(poly, POLYMER["rho"], SILICON["rho"])
    hc = np.where(poly, POLYMER["heat_capacity"], SILICON["heat_capacity"])
    ih = np.zeros(n ** 3, np.int64)
    ih[: heated_layers * n * n] = 1
    nheated = heated_layers * n * n
    return Problem(nx=n, ny=n, nz=n, lx=n * dx, ly=n * dx, lz=n * dx, kappa=kappa, rho=rho,
                   heat_capacity=hc, tau=1e-12, em=0.0, iheater=ih,
                   power_in=power_per_cell * nheated, time_step=dt, icattaneo=1,
                   periodic=(1, 1, 0), **_dirichlet(149.0))
