"""Analytic known answers for the dynamics step: states whose evolution is known without running
any implementation, and the measurements that compare a run with them.

Shared by the CPU tests of the oracle (tests/test_oracle_physics.py) and their GPU twins
(tests/test_gpu_physics.py), which put the CUDA path through the same checks.  Everything here is
numpy; nothing calls the oracle or the library.

* Discrete hydrostatic balance.  DPRES is a polynomial of degree p in z over the whole column
  (continuous across elements, so it has no face jumps) and DDENS = -dDPRES/dz / g, of degree
  p - 1, which the vertical truncation VPOrdM1 in the gravity term keeps.  The pressure gradient
  and gravity then cancel node by node and the DG tendency is zero to roundoff: FElib's
  deviation form (-dDPRES/dz - g VFilterPM1(DDENS), rhot_heve.F90:292-489, with the VPOrdM1
  truncation of scale_element_operation_tensorprod3D.F90:5560-5563) is built for exactly this
  balance.  A pure degree-p vertical mode added to DDENS exerts no gravity force at all (VPOrdM1
  removes it), so the state stays steady with it.
* Lamb wave.  In an isothermal atmosphere under gravity, p' = eps P_s exp(-z/(gamma H)) cos(kx)
  with rho' = p'/c^2, u' = p'/(rho_0 c) and w' = 0 is an exact solution of the linearised
  compressible equations that travels at c = sqrt(gamma R T) (hydrostatic in the vertical,
  acoustic in the horizontal; it satisfies the slip lids because w' = 0).
* Vertical acoustic mode.  Without gravity (uniform base state), p' = eps P cos(mz) cos(wt),
  rho_0 w' = (eps P / c) sin(mz) sin(wt) with m = pi/Z and w = c m: the standing mode between
  the two slip lids, the one HEVI treats implicitly.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np

from fedg import cases
from fedg.element import legendre, lgl_nodes

GAMMA = cases.CPDRY / cases.CVDRY


def quad_weights(case):
    """(Ne, Np) LGL quadrature weights of the flat cube: J w_i w_j w_k, J = dx dy dz / 8."""
    _, w = lgl_nodes(case.porder)
    xmin, xmax, ymin, ymax, zmin, zmax = case.dom
    J = (xmax - xmin) / case.NeX * (ymax - ymin) / case.NeY * (zmax - zmin) / case.NeZ / 8.0
    w3 = (w[:, None, None] * w[None, :, None] * w[None, None, :]).reshape(-1)  # (k, j, i) -> node i + N1 j + N1^2 k
    return np.broadcast_to(J * w3, (case.Ne, case.Np)).copy()


def rhot_of_pres(p):
    """RHOT of the dry equation of state PRES = P00 (Rd RHOT / P00)^(cp/cv)."""
    return cases.PRES00 / cases.RDRY * (p / cases.PRES00) ** (cases.CVDRY / cases.CPDRY)


def pres_of_rhot(rhot):
    return cases.PRES00 * (cases.RDRY * rhot / cases.PRES00) ** GAMMA


def dpres(q, b):
    """DPRES of a state from its DRHOT, by the equation of state (numpy, FP64)."""
    return pres_of_rhot(b["therm_hyd"] + q[4]) - b["pres_hyd"]


def base_only(case):
    """The case's hydrostatic base state with no perturbation and no wind."""
    return cases.initial_state(replace(case, bubble={}, noise={}, u0=0.0, v0=0.0))[1]


# ------------------------------------------------------------------------------------------------
def hydrostatic_state(case, seed=0, amp=30.0, U=0.0, extra=True):
    """Deviation state in discrete hydrostatic balance (module docstring).  Returns (q, b, info)
    with info['gterm'] = g max|DDENS_bal|, the size of the balanced gravity term."""
    b = base_only(case)
    rng = np.random.default_rng(seed)
    z = b["z"]
    zmin, zmax = case.dom[4], case.dom[5]
    H = zmax - zmin
    zt = (z - zmin) / H
    c = rng.uniform(-1.0, 1.0, case.porder)
    dp = amp * sum(c[n - 1] * zt ** n for n in range(1, case.porder + 1))
    dpdz = amp / H * sum(n * c[n - 1] * zt ** (n - 1) for n in range(1, case.porder + 1))
    ddens_bal = -dpdz / case.grav
    ddens = ddens_bal.copy()
    if extra:
        # a pure degree-p vertical Legendre mode in each element, horizontally uniform (so a uniform
        # wind advects nothing), 1e-2 of the balanced density deviation.  P_p(1) = 1 and
        # P_p(-1) = (-1)^p, so the amplitude alternates in sign from element to element for odd p
        # (constant for even p): the field is continuous across the vertical faces and the Rusanov
        # dissipation sees no jump.
        x1, _ = lgl_nodes(case.porder)
        N1 = case.N1
        kidx = np.arange(case.Np) // (N1 * N1)
        ez = np.arange(case.Ne) // (case.NeX * case.NeY)
        a = rng.uniform(0.5, 1.0) * (-1.0 if case.porder % 2 else 1.0) ** ez
        ddens += 1e-2 * np.max(np.abs(ddens_bal)) * a[:, None] * legendre(case.porder, x1[kidx])[None, :]
    drhot = rhot_of_pres(b["pres_hyd"] + dp) - b["therm_hyd"]
    dens = b["dens_hyd"] + ddens
    q = [ddens, dens * U, np.zeros_like(z), np.zeros_like(z), drhot]
    return q, b, dict(gterm=case.grav * float(np.max(np.abs(ddens_bal))), dpres=dp)


def hydro_case(porder=3, NeZ=4, **kw):
    """Small flat-cube mesh for the balance tests: isothermal 300 K base state, 2x2 columns."""
    if porder == 3:
        c = cases.C1().scaled(2, 2, NeZ)
    else:
        c = cases.C2().scaled(2, 2, NeZ, porder=porder)
    return replace(c, bubble={}, noise={}, u0=0.0, **kw)


# ------------------------------------------------------------------------------------------------
def lamb_case(porder=3, NeX=8, NeZ=4, Lx=20000.0, Ztop=10000.0, eqs="HEVE"):
    c = cases.C1()
    return replace(c, name="lamb", porder=porder, NeX=NeX, NeY=1, NeZ=NeZ, dom=(0.0, Lx, 0.0, Lx / NeX, 0.0, Ztop),
                   eqs=eqs, bubble={}, noise={}, u0=0.0, base="constT", T0=300.0, filter_on=False)


def lamb_speed(case):
    return float(np.sqrt(GAMMA * cases.RDRY * case.T0))


def lamb_state(case, eps=1e-7):
    b = base_only(case)
    c = lamb_speed(case)
    H = cases.RDRY * case.T0 / case.grav
    k = 2.0 * np.pi / (case.dom[1] - case.dom[0])
    x, z = b["x"], b["z"]
    pp = eps * case.psfc * np.exp(-z / (GAMMA * H)) * np.cos(k * x)
    rho = pp / c ** 2
    u = pp / (b["dens_hyd"] * c)
    drhot = rhot_of_pres(b["pres_hyd"] + pp) - b["therm_hyd"]
    q = [rho, b["dens_hyd"] * u, np.zeros_like(z), np.zeros_like(z), drhot]
    return q, b


def lamb_phase(case, q, b):
    """Phase of the wave's exp(ikx) component of DPRES (radians, in (-pi, pi])."""
    k = 2.0 * np.pi / (case.dom[1] - case.dom[0])
    W = quad_weights(case)
    A = np.sum(W * dpres(q, b) * np.exp(-1j * k * b["x"]))
    return float(np.angle(A)), float(np.abs(A))


# ------------------------------------------------------------------------------------------------
def vacoustic_case(porder=3, NeZ=4, Ztop=10000.0, eqs="HEVE"):
    """Single column of elements, no gravity: a uniform 300 K atmosphere at 1e5 Pa between lids."""
    c = cases.C1()
    return replace(c, name="vacoustic", porder=porder, NeX=1, NeY=1, NeZ=NeZ,
                   dom=(0.0, 1000.0, 0.0, 1000.0, 0.0, Ztop), eqs=eqs, bubble={}, noise={}, u0=0.0,
                   base="constPT", T0=300.0, psfc=cases.PRES00, grav=0.0, filter_on=False)


def vacoustic_omega(case):
    c = float(np.sqrt(GAMMA * cases.RDRY * case.T0))
    return c * np.pi / (case.dom[5] - case.dom[4]), c


def vacoustic_state(case, eps=1e-7):
    b = base_only(case)
    _, c = vacoustic_omega(case)
    m = np.pi / (case.dom[5] - case.dom[4])
    pp = eps * case.psfc * np.cos(m * (b["z"] - case.dom[4]))
    drhot = rhot_of_pres(b["pres_hyd"] + pp) - b["therm_hyd"]
    z0 = np.zeros_like(pp)
    return [pp / c ** 2, z0, z0.copy(), z0.copy(), drhot], b


def vacoustic_phase(case, q, b):
    """w t of the standing mode: atan2(c <MOMZ, sin mz>, <DPRES, cos mz>)."""
    _, c = vacoustic_omega(case)
    m = np.pi / (case.dom[5] - case.dom[4])
    W = quad_weights(case)
    zz = b["z"] - case.dom[4]
    a = np.sum(W * dpres(q, b) * np.cos(m * zz))
    s = np.sum(W * q[3] * np.sin(m * zz))
    return float(np.arctan2(c * s, a)), float(np.hypot(c * s, a))


# ------------------------------------------------------------------------------------------------
def integrals(case, q, b=None):
    """LGL integrals of DDENS, MOMX, MOMY and DRHOT, which periodic sides and slip lids conserve, and
    the scales their changes are measured against: the L1 norms of DDENS and DRHOT, and for MOMX and
    MOMY the L1 norm of the horizontal momentum vector (so that a component with no mean is not
    measured against its own small norm).  With the base state b, the scales are the totals instead:
    total mass, total horizontal momentum, total RHOT."""
    W = quad_weights(case)
    I = np.array([np.sum(W * q[v]) for v in (0, 1, 2, 4)])
    hm = np.sum(W * np.hypot(q[1], q[2]))
    if b is None:
        A = np.array([np.sum(W * np.abs(q[0])), hm, hm, np.sum(W * np.abs(q[4]))])
    else:
        A = np.array([np.sum(W * (b["dens_hyd"] + q[0])), hm, hm, np.sum(W * (b["therm_hyd"] + q[4]))])
    return I, A


class ColumnIndex:
    """Maps a column-local unknown (variable, level) to the global nodes of every column."""

    def __init__(self, case):
        N1, NF = case.N1, case.N1 * case.N1
        self.case = case
        self.L = case.NeZ * N1
        nxy = case.NeX * case.NeY
        ncol = nxy * NF
        col = np.arange(ncol)
        ij, exy = col % NF, col // NF
        # level l = ez N1 + k of column (exy, ij): element exy + nxy ez, node ij + NF k
        lv = np.arange(self.L)
        ez, k = lv // N1, lv % N1
        self.elem = exy[:, None] + nxy * ez[None, :]  # (ncol, L)
        self.node = ij[:, None] + NF * k[None, :]
        self.ncol = ncol

    def gather(self, f):
        return f[self.elem, self.node]  # (ncol, L)

    def scatter(self, f, vals):
        f[self.elem, self.node] = vals


def newton_step_fd(case, op, qs, z0, impl_fac, scales, h_rel=1e-6):
    """One Newton step of F(P) = P - q* - impl_fac A(P) from P = z0, with the Jacobian of A taken by
    central differences of op(P, z0), the operator with its Rusanov speed frozen at z0.  Every column
    is independent, so one evaluation perturbs the same (variable, level) in all columns at once;
    scales[v] is the size of variable v (the step is h_rel x scale).  Returns the new iterate."""
    ci = ColumnIndex(case)
    L, nc = ci.L, ci.ncol
    nu = 5 * L

    def F(P):
        A = op(P, z0)
        return np.concatenate([ci.gather(P[v] - qs[v] - impl_fac * A[v]) for v in range(5)], axis=1)  # (nc, 5L)

    F0 = F(z0)
    J = np.zeros((nc, nu, nu))
    for v in range(5):
        h = h_rel * scales[v]
        for l in range(L):
            Pp = [a.copy() for a in z0]
            Pm = [a.copy() for a in z0]
            e = np.zeros((nc, L))
            e[:, l] = h
            ci.scatter(Pp[v], ci.gather(Pp[v]) + e)
            ci.scatter(Pm[v], ci.gather(Pm[v]) - e)
            J[:, :, v * L + l] = (F(Pp) - F(Pm)) / (2.0 * h)
    d = np.linalg.solve(J, -F0[:, :, None])[:, :, 0]
    out = [a.copy() for a in z0]
    for v in range(5):
        ci.scatter(out[v], ci.gather(z0[v]) + d[:, v * L:(v + 1) * L])
    return out
