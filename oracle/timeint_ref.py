"""numpy restatement of FElib's ``timeint_rk`` stage arithmetic (test infrastructure only).

Follows FElib/src/common/scale_timeint_rk.F90:
  * ``store_var0``      -- the driver's StoreVar0 (copy q -> var0)
  * ``store_implicit``  -- rk_storeimpl_general2D, :2510-2565
  * ``advance``         -- rk_advance_general2D, :2201-2360 (IMEX and explicit general forms)
                           rk_advance_low_storage2D, :1182-1278 (Shu-Osher low-storage form)
and the tables of FElib/src/common/scale_timeint_rk_butcher_tab.F90:200-274.
"""
from __future__ import annotations

import numpy as np

SQ2 = np.sqrt(2.0)


def tables(name: str):
    if name == "IMEX_ARK232":
        alp = (3.0 + 2.0 * SQ2) / 6.0
        gam = 1.0 - 1.0 / SQ2
        dl = 1.0 / (2.0 * SQ2)
        a_ex = np.zeros((3, 3))
        a_im = np.zeros((3, 3))
        a_ex[1, 0] = 2.0 * gam
        a_ex[2, :] = (1.0 - alp, alp, 0.0)
        a_im[1, :] = (gam, gam, 0.0)
        a_im[2, :] = (dl, dl, gam)
        b = np.array([dl, dl, gam])
        return dict(kind="imex", nstage=3, a_ex=a_ex, a_im=a_im, b_ex=b, b_im=b.copy())
    if name == "ERK_SSP_3s3o":
        sig = np.zeros((4, 3))
        gmm = np.zeros((4, 3))
        sig[1, 0] = 1.0
        sig[2, 0:2] = (0.75, 0.25)
        sig[3, 0:3] = (1.0 / 3.0, 0.0, 2.0 / 3.0)
        gmm[1, 0] = 1.0
        gmm[2, 1] = 0.25
        gmm[3, 2] = 2.0 / 3.0
        # stage nodes of the equivalent Butcher form (a21 = 1, a31 = a32 = 1/4)
        c = np.array([0.0, 1.0, 0.5])
        return dict(kind="lowstorage", nstage=3, sig=sig, gam=gmm, c=c)
    raise ValueError(name)


class TimeIntRK:
    """Holds var0 / varTmp and the tendency buffers of one scheme, like FElib's type."""

    def __init__(self, name: str, dt: float, shape):
        self.t = tables(name)
        self.dt = dt
        self.nstage = self.t["nstage"]
        self.var0 = np.zeros(shape)
        self.varTmp = np.zeros(shape)
        self.tend_ex = np.zeros((self.nstage,) + tuple(shape))
        self.tend_im = np.zeros((self.nstage,) + tuple(shape))

    def implicit_diagfac(self, s: int) -> float:  # Get_implicit_diagfac, :304-317 (s is 1-based)
        if self.t["kind"] != "imex":
            return 0.0
        return self.t["a_im"][s - 1, s - 1] * self.dt

    def store_var0(self, q):
        self.var0[...] = q

    def store_implicit(self, s: int, q):
        if self.t["kind"] != "imex":
            return
        if s == 1:
            self.var0[...] = q
            self.varTmp[...] = q
        q += self.dt * self.t["a_im"][s - 1, s - 1] * self.tend_im[s - 1]

    def advance(self, s: int, q):
        t, dt = self.t, self.dt
        if t["kind"] == "lowstorage":
            sig, gam, ns = t["sig"], t["gam"], self.nstage
            sig_ss, gam_ss = sig[s, s - 1], dt * gam[s, s - 1]
            if s == ns:
                q[...] = self.varTmp + sig_ss * q + gam_ss * self.tend_ex[0]
                return
            if s == 1:
                self.var0[...] = q
                self.varTmp[...] = 0.0
            sig_ns, gam_ns = sig[ns, s - 1], dt * gam[ns, s - 1]
            if abs(sig_ns) > 1e-16 or abs(gam_ns) > 1e-16:
                self.varTmp += sig_ns * q + gam_ns * self.tend_ex[0]
            q[...] = (1.0 - sig_ss) * self.var0 + sig_ss * q + gam_ss * self.tend_ex[0]
            return
        ns = self.nstage
        if s == ns:
            q[...] = self.varTmp + t["b_ex"][s - 1] * dt * self.tend_ex[s - 1] + t["b_im"][s - 1] * dt * self.tend_im[s - 1]
            return
        q[...] = self.var0
        self.varTmp += t["b_ex"][s - 1] * dt * self.tend_ex[s - 1] + t["b_im"][s - 1] * dt * self.tend_im[s - 1]
        for j in range(1, s + 1):
            q += t["a_ex"][s, j - 1] * dt * self.tend_ex[j - 1] + t["a_im"][s, j - 1] * dt * self.tend_im[j - 1]


def damped_oscillator_error(name: str, dt: float, end_time: float = 1.0, omg=2.0 * np.pi, r=0.1):
    """The IMEX/explicit oscillator of FElib/test/common/timeint_rk/test_timeint_rk.f90:173-282:
    u' = omg v - r u (explicit damping), v' = -omg u (rotation implicit when the scheme is IMEX).
    Returns the max error of u against the closed form over the run."""
    tint = TimeIntRK(name, dt, (2,))
    q = np.array([1.0, 0.0])
    omgg = np.sqrt(omg ** 2 - r ** 2 / 4.0)
    nstep = int(round(end_time / dt))
    err = 0.0
    imex = tint.t["kind"] == "imex"
    for n in range(1, nstep + 1):
        for s in range(1, tint.nstage + 1):
            buf = s - 1 if tint.t["kind"] == "imex" else 0
            if imex:
                fac = tint.implicit_diagfac(s)
                coef = fac * omg
                if abs(fac) > 0:
                    ui = (q[0] + coef * q[1]) / (1.0 + coef ** 2)
                    vi = (q[1] - coef * q[0]) / (1.0 + coef ** 2)
                    tint.tend_im[buf] = [(ui - q[0]) / fac, (vi - q[1]) / fac]
                else:
                    tint.tend_im[buf] = [omg * q[1], -omg * q[0]]
                tint.store_implicit(s, q)
                tint.tend_ex[buf] = [-r * q[0], 0.0]
            else:
                tint.tend_ex[buf] = [omg * q[1] - r * q[0], -omg * q[0]]
            tint.advance(s, q)
        t = n * dt
        ans = (np.cos(omgg * t) - r / (2.0 * omgg) * np.sin(omgg * t)) * np.exp(-0.5 * r * t)
        err = max(err, abs(q[0] - ans))
    return err
