"""Synthetic workloads of the SCALE-DG nonhydrostatic 3D dynamics step.

Each case is a flat cube domain (periodic in x and y, slip lids at bottom and top) with
a horizontally homogeneous hydrostatic base state and a potential-temperature
perturbation, built the way the reference's initial-condition code builds them:

* base states: ``constT`` / ``constPT`` / ``constBVFreq``
  (FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_hydrostatic.F90:86-230);
* DDENS/DRHOT from a potential-temperature perturbation at fixed hydrostatic pressure
  (model/atm_nonhydro3d/test/case/density_current/mod_user.F90:242-249);
* cosine-bell bubble 0.5 (1 + cos(pi r)) inside r <= 1
  (model/atm_nonhydro3d/src/preprocess/mod_mkinit_util.F90:139-152).  The reference
  L2-projects the bell from an order-11 element; here it is sampled at the nodes.

Fields are numpy float64 arrays of shape (Ne, Np) in C order (== FElib's column-major
(Np, Ne)); element ke = ex + NeX*ey + NeX*NeY*ez, node n = i + N1*j + N1^2*k.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

import numpy as np

from .element import lgl_nodes

GRAV = 9.80616
RDRY = 287.04
CPDRY = 1004.64
CVDRY = CPDRY - RDRY
PRES00 = 1.0e5


@dataclass
class Case:
    name: str
    porder: int
    NeX: int
    NeY: int
    NeZ: int
    dom: tuple  # (xmin, xmax, ymin, ymax, zmin, zmax)
    eqs: str  # "HEVE" | "HEVI"
    dt: float
    nsteps: int
    base: str = "constT"  # constT | constPT | constBVFreq
    T0: float = 300.0
    psfc: float = PRES00
    bvf: float = 0.0
    u0: float = 0.0
    bubble: dict = field(default_factory=dict)  # amp, rx, ry, rz, xc, yc, zc
    noise: dict = field(default_factory=dict)  # amp, zmax, seed
    filter_on: bool = True
    newton_tol: float = 1e-10
    grav: float = GRAV
    v0: float = 0.0
    tracer: dict = field(default_factory=dict)  # cosine-bell tracer: qmax, rx, ry, rz, xc, yc, zc

    @property
    def N1(self):
        return self.porder + 1

    @property
    def Np(self):
        return self.N1 ** 3

    @property
    def Ne(self):
        return self.NeX * self.NeY * self.NeZ

    @property
    def dofs(self):
        return 5 * self.Np * self.Ne

    def scaled(self, NeX=None, NeY=None, NeZ=None, porder=None, keep_extent=False):
        """Same physics on a different element count (domain extents scale with the count
        unless ``keep_extent``), for parity tests at sizes the oracle finishes quickly."""
        NeX = NeX or self.NeX
        NeY = NeY or self.NeY
        NeZ = NeZ or self.NeZ
        xmin, xmax, ymin, ymax, zmin, zmax = self.dom
        if not keep_extent:
            xmax = xmin + (xmax - xmin) * NeX / self.NeX
            ymax = ymin + (ymax - ymin) * NeY / self.NeY
            zmax = zmin + (zmax - zmin) * NeZ / self.NeZ
        b = dict(self.bubble)
        if b and not keep_extent:
            b["xc"] = 0.5 * (xmin + xmax)
            b["yc"] = 0.5 * (ymin + ymax)
        tr = dict(self.tracer)
        if tr and not keep_extent:  # keep the tracer's position and size relative to the domain
            fx, fy, fz = NeX / self.NeX, NeY / self.NeY, NeZ / self.NeZ
            tr.update(xc=xmin + (tr["xc"] - xmin) * fx, yc=ymin + (tr["yc"] - ymin) * fy,
                      zc=zmin + (tr["zc"] - zmin) * fz, rx=tr["rx"] * fx, ry=tr["ry"] * fy, rz=tr["rz"] * fz)
        return replace(self, NeX=NeX, NeY=NeY, NeZ=NeZ, porder=porder or self.porder,
                       dom=(xmin, xmax, ymin, ymax, zmin, zmax), bubble=b, tracer=tr)


def C1():
    """p=3, 8x8x8 over 1 km^3, constT 300 K, +2 K bubble r=250 m at z=350 m, HEVE SSP-RK3."""
    return Case("C1_p3_8x8x8_heve", 3, 8, 8, 8, (0.0, 1000.0, 0.0, 1000.0, 0.0, 1000.0), "HEVE",
                dt=0.05, nsteps=100, base="constT",
                bubble=dict(amp=2.0, rx=250.0, ry=250.0, rz=250.0, xc=500.0, yc=500.0, zc=350.0))


def C2():
    """p=7, 32x32x8 over 25.6x25.6x6.4 km, constT 300 K, -15 K density current, u=10 m/s, HEVI."""
    return Case("C2_p7_32x32x8_hevi", 7, 32, 32, 8, (0.0, 25600.0, 0.0, 25600.0, 0.0, 6400.0), "HEVI",
                dt=0.5, nsteps=200, base="constT", u0=10.0,
                bubble=dict(amp=-15.0, rx=4000.0, ry=4000.0, rz=2000.0, xc=12800.0, yc=12800.0, zc=3000.0))


def C3():
    """C1 numerics in the precision form (FP32 on deviations, 3xTF32 contractions), 1 hour."""
    c = C1()
    return replace(c, name="C3_p3_8x8x8_mixed_1h", nsteps=int(round(3600.0 / c.dt)))


def C5():
    """p=7, 128x128x16 over 12.8x12.8x3.2 km, constBVFreq N=0.01, +-0.1 K noise below 500 m, u=5."""
    return Case("C5_p7_128x128x16_hevi", 7, 128, 128, 16, (0.0, 12800.0, 0.0, 12800.0, 0.0, 3200.0), "HEVI",
                dt=0.5, nsteps=720, base="constBVFreq", bvf=0.01, T0=300.0, u0=5.0,
                noise=dict(amp=0.1, zmax=500.0, seed=0))


def T1():
    """Tracer advection test (model/atm_nonhydro3d/test/case/tracer_advection/{init,run}.conf):
    p=3, 20x20x5 elements over 60x60x20 km, constPT 300 K base state with g = 0 (uniform density),
    uniform wind (u, v) = (-35, -40) m/s, cosine-bell tracer of peak 1 and radii 10 km at
    (12, 12, 5) km; tracer SSP-RK3, dt = 2 s, 900 s; no modal filter; FCT + TMAR on."""
    return Case("T1_p3_20x20x5_trcadv", 3, 20, 20, 5, (0.0, 60000.0, 0.0, 60000.0, 0.0, 20000.0), "HEVE",
                dt=2.0, nsteps=450, base="constPT", T0=300.0, psfc=101325.0, grav=0.0, u0=-35.0, v0=-40.0,
                filter_on=False,
                tracer=dict(qmax=1.0, rx=10000.0, ry=10000.0, rz=10000.0, xc=12000.0, yc=12000.0, zc=5000.0))


CASES = {"C1": C1, "C2": C2, "C3": C3, "C5": C5, "T1": T1}


def node_coords(case: Case):
    x1, _ = lgl_nodes(case.porder)
    N1 = case.N1
    xmin, xmax, ymin, ymax, zmin, zmax = case.dom
    dx, dy, dz = (xmax - xmin) / case.NeX, (ymax - ymin) / case.NeY, (zmax - zmin) / case.NeZ
    r = 0.5 * (x1 + 1.0)
    ex = np.arange(case.NeX)
    ey = np.arange(case.NeY)
    ez = np.arange(case.NeZ)
    # (ez, ey, ex, k, j, i)
    X = xmin + (ex[None, None, :, None, None, None] + r[None, None, None, None, None, :]) * dx
    Y = ymin + (ey[None, :, None, None, None, None] + r[None, None, None, None, :, None]) * dy
    Z = zmin + (ez[:, None, None, None, None, None] + r[None, None, None, :, None, None]) * dz
    shp = (case.NeZ, case.NeY, case.NeX, N1, N1, N1)
    X, Y, Z = (np.broadcast_to(a, shp).reshape(case.Ne, case.Np) for a in (X, Y, Z))
    return X.copy(), Y.copy(), Z.copy()


def base_state(case: Case, z):
    """(DENS_hyd, PRES_hyd, PT_hyd) at heights z."""
    rovcp = RDRY / CPDRY
    if case.base == "constT":
        H0 = RDRY * case.T0 / case.grav
        pres = case.psfc * np.exp(-z / H0)
        dens = pres / (RDRY * case.T0)
        pt = case.T0 * (PRES00 / pres) ** rovcp
    elif case.base == "constPT":
        exner_sfc = (case.psfc / PRES00) ** rovcp
        exner = exner_sfc - case.grav / (CPDRY * case.T0) * z
        pres = PRES00 * exner ** (CPDRY / RDRY)
        dens = pres / (RDRY * exner * case.T0)
        pt = np.full_like(z, case.T0)
    elif case.base == "constBVFreq":
        exner_sfc = (case.psfc / PRES00) ** rovcp
        pt = case.T0 * np.exp(case.bvf ** 2 / case.grav * z)
        exner = exner_sfc + case.grav ** 2 / (CPDRY * case.bvf ** 2) * (1.0 / pt - 1.0 / case.T0)
        pres = PRES00 * exner ** (CPDRY / RDRY)
        dens = pres / (RDRY * exner * pt)
    else:
        raise ValueError(case.base)
    return dens, pres, pt


def initial_state(case: Case, seed=None):
    """Returns (q, base) with q = [DDENS, MOMX, MOMY, MOMZ, DRHOT] and
    base = dict(dens_hyd, pres_hyd, therm_hyd, pt_hyd, x, y, z)."""
    x, y, z = node_coords(case)
    dens_hyd, pres_hyd, pt_hyd = base_state(case, z)
    dth = np.zeros_like(z)
    if case.bubble:
        b = case.bubble
        r = np.sqrt(((x - b["xc"]) / b["rx"]) ** 2 + ((y - b["yc"]) / b["ry"]) ** 2 + ((z - b["zc"]) / b["rz"]) ** 2)
        dth += np.where(r <= 1.0, b["amp"] * 0.5 * (1.0 + np.cos(np.pi * np.minimum(r, 1.0))), 0.0)
    if case.noise:
        nz = case.noise
        rng = np.random.default_rng(nz.get("seed", 0) if seed is None else seed)
        dth += np.where(z < nz["zmax"], rng.uniform(-nz["amp"], nz["amp"], size=z.shape), 0.0)
    pt = pt_hyd + dth
    rovcp = RDRY / CPDRY
    dens = pres_hyd / (RDRY * pt * (pres_hyd / PRES00) ** rovcp)
    therm_hyd = PRES00 / RDRY * (pres_hyd / PRES00) ** (CVDRY / CPDRY)
    ddens = dens - dens_hyd
    drhot = dens * pt - therm_hyd
    momx = dens * case.u0
    momy = dens * case.v0
    momz = np.zeros_like(z)
    q = [ddens, momx, momy, momz, drhot]
    base = dict(dens_hyd=dens_hyd, pres_hyd=pres_hyd, therm_hyd=therm_hyd, pt_hyd=pt_hyd, x=x, y=y, z=z)
    return q, base


def tracer_state(case: Case):
    """Initial tracer mixing ratio of a case with a ``tracer`` bell: qmax (0.5 (1 + cos(pi r)))
    inside r <= 1 (mkinitutil_calc_cosinebell, exponent 1), sampled at the nodes."""
    x, y, z = node_coords(case)
    tr = case.tracer
    r = np.sqrt(((x - tr["xc"]) / tr["rx"]) ** 2 + ((y - tr["yc"]) / tr["ry"]) ** 2 + ((z - tr["zc"]) / tr["rz"]) ** 2)
    return np.where(r <= 1.0, tr["qmax"] * 0.5 * (1.0 + np.cos(np.pi * np.minimum(r, 1.0))), 0.0)
