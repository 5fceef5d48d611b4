"""ctypes wrapper of the FP64 CPU oracle (``fedg_oracle.cpp``).

Test infrastructure only: the checker used by ``tests/``, ``__graft_entry__.smoke()``
and the ``cpu_baseline`` leg of ``bench.py``.  The product path never imports this.

Every routine follows FElib (ywkawai/FE-Project); the per-function citations are in
``fedg_oracle.cpp``.  Fields are numpy float64 arrays of shape ``(Ne, Np)`` in C order,
which is the same memory as FElib's column-major ``(Np, Ne)``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfedg_oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)


class OrcDesc(ctypes.Structure):
    _fields_ = [
        ("porder", ctypes.c_int),
        ("NeX", ctypes.c_int), ("NeY", ctypes.c_int), ("NeZ", ctypes.c_int),
        ("xmin", ctypes.c_double), ("xmax", ctypes.c_double),
        ("ymin", ctypes.c_double), ("ymax", ctypes.c_double),
        ("zmin", ctypes.c_double), ("zmax", ctypes.c_double),
        ("grav", ctypes.c_double), ("rdry", ctypes.c_double), ("cpdry", ctypes.c_double),
        ("cvdry", ctypes.c_double), ("pres00", ctypes.c_double),
        ("coriolis_f", ctypes.c_double),
        ("filter_on", ctypes.c_int),
        ("mf_etac", ctypes.c_double), ("mf_alpha", ctypes.c_double), ("mf_order", ctypes.c_int),
        ("newton_cref", ctypes.c_double),
    ]


# void (*)(void* user, int stage, const double* const* q, const double* dpres)
HALO_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.POINTER(ctypes.c_double)),
                           ctypes.POINTER(ctypes.c_double))


def build() -> str:
    """Compile the oracle with its Makefile (gcc + OpenMP); returns the .so path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
        os.path.join(_HERE, "fedg_oracle.cpp")
    ):
        build()
    lib = ctypes.CDLL(_LIB_PATH)
    lib.orc_create.restype = ctypes.c_void_p
    lib.orc_create.argtypes = [ctypes.POINTER(OrcDesc)]
    lib.orc_destroy.argtypes = [ctypes.c_void_p]
    lib.orc_set_halo.argtypes = [ctypes.c_void_p, ctypes.POINTER(_dp), HALO_CB, ctypes.c_void_p]
    lib.orc_num_threads.restype = ctypes.c_int
    lib.orc_set_num_threads.argtypes = [ctypes.c_int]
    lib.orc_get_1d.argtypes = [ctypes.c_void_p] + [_dp] * 8
    lib.orc_node_coords.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
    lib.orc_set_base_state.argtypes = [ctypes.c_void_p, _dp, _dp]
    lib.orc_get_therm_hyd.argtypes = [ctypes.c_void_p, _dp]
    lib.orc_drhot2pres.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
    pp = ctypes.POINTER(_dp)
    lib.orc_cal_tend.argtypes = [ctypes.c_void_p, ctypes.c_int, pp, _dp, pp]
    lib.orc_cal_vi.restype = ctypes.c_long
    lib.orc_cal_vi.argtypes = [ctypes.c_void_p, pp, pp, ctypes.c_double, ctypes.c_double,
                               ctypes.c_int, ctypes.c_double, pp, ctypes.POINTER(ctypes.c_int)]
    lib.orc_modalfilter.argtypes = [ctypes.c_void_p, pp]
    lib.orc_vi_operator.argtypes = [ctypes.c_void_p, pp, pp, pp]
    lib.orc_step_heve.argtypes = [ctypes.c_void_p, pp, ctypes.c_double, ctypes.c_int]
    lib.orc_step_hevi.restype = ctypes.c_long
    lib.orc_step_hevi.argtypes = [ctypes.c_void_p, pp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_double, _dp]
    lib.orc_trc_alphdens_advtest.argtypes = [ctypes.c_void_p] + [_dp] * 6
    lib.orc_trc_save_massflux.argtypes = [ctypes.c_void_p, ctypes.c_int, pp, _dp, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_int, pp, _dp, _dp]
    lib.orc_trc_fct_coef.argtypes = [ctypes.c_void_p, _dp, pp, _dp, _dp, _dp, _dp, _dp, ctypes.c_double,
                                     ctypes.c_double, _dp]
    lib.orc_trc_cal_tend.argtypes = [ctypes.c_void_p, _dp, pp, _dp, _dp, _dp, _dp, _dp]
    lib.orc_trc_tmar.argtypes = [ctypes.c_void_p, _dp, _dp]
    lib.orc_trc_filter.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_int]
    lib.orc_trc_step.argtypes = [ctypes.c_void_p, _dp, pp, _dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_int, _dp, _dp,
                                 _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int]
    lib.orc_set_trc_flux.argtypes = [ctypes.c_void_p, pp]
    lib.orc_set_sponge.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    lib.orc_numdiff_apply.argtypes = [ctypes.c_void_p, pp, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double]
    lib.orc_sponge_add_tend.argtypes = [ctypes.c_void_p, pp, pp, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    _lib = lib
    return lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def _optr(a):
    """pointer of an optional array (None -> NULL)"""
    return None if a is None else _ptr(a)


def _c64(a):
    return None if a is None else np.ascontiguousarray(a, np.float64)


def _pp(arrs):
    arr = (_dp * len(arrs))(*[_ptr(a) for a in arrs])
    return ctypes.cast(arr, ctypes.POINTER(_dp)), arrs


def set_num_threads(n: int) -> None:
    _load().orc_set_num_threads(int(n))


def num_threads() -> int:
    return int(_load().orc_num_threads())


class Oracle:
    """FP64 CPU restatement of FElib's nonhydro3d HEVE/HEVI dynamics on a flat cube domain."""

    def __init__(self, porder, NeX, NeY, NeZ, dom, *, grav=9.80616, rdry=287.04, cpdry=1004.64,
                 cvdry=717.6, pres00=1.0e5, coriolis_f=0.0, filter_on=True, mf_etac=2.0 / 3.0,
                 mf_alpha=36.0, mf_order=16, newton_cref=340.0):
        lib = _load()
        xmin, xmax, ymin, ymax, zmin, zmax = dom
        d = OrcDesc(porder, NeX, NeY, NeZ, xmin, xmax, ymin, ymax, zmin, zmax, grav, rdry, cpdry,
                    cvdry, pres00, coriolis_f, int(filter_on), mf_etac, mf_alpha, mf_order, newton_cref)
        self._h = lib.orc_create(ctypes.byref(d))
        if not self._h:
            raise ValueError("oracle: invalid descriptor")
        self.lib = lib
        self.N1 = porder + 1
        self.Np = self.N1 ** 3
        self.Ne = NeX * NeY * NeZ
        self.shape = (self.Ne, self.Np)
        self.NeX, self.NeY, self.NeZ = NeX, NeY, NeZ

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self.lib.orc_destroy(h)
            self._h = None

    def operators_1d(self):
        n = self.N1
        x, w = np.zeros(n), np.zeros(n)
        D, Mi, F, T, V, iV = (np.zeros((n, n)) for _ in range(6))
        self.lib.orc_get_1d(self._h, _ptr(x), _ptr(w), _ptr(D), _ptr(Mi), _ptr(F), _ptr(T), _ptr(V), _ptr(iV))
        return dict(x=x, w=w, D=D, Minv=Mi, F=F, T=T, V=V, invV=iV)

    def coords(self):
        x, y, z = (np.zeros(self.shape) for _ in range(3))
        self.lib.orc_node_coords(self._h, _ptr(x), _ptr(y), _ptr(z))
        return x, y, z

    def set_base_state(self, dens_hyd, pres_hyd):
        self.lib.orc_set_base_state(self._h, _ptr(np.ascontiguousarray(dens_hyd, np.float64)),
                                    _ptr(np.ascontiguousarray(pres_hyd, np.float64)))

    def therm_hyd(self):
        out = np.zeros(self.shape)
        self.lib.orc_get_therm_hyd(self._h, _ptr(out))
        return out

    def drhot2pres(self, drhot):
        pres, dpres = np.zeros(self.shape), np.zeros(self.shape)
        self.lib.orc_drhot2pres(self._h, _ptr(np.ascontiguousarray(drhot)), _ptr(pres), _ptr(dpres))
        return pres, dpres

    def cal_tend(self, q, hevi, dpres=None):
        """q: list of 5 arrays (DDENS, MOMX, MOMY, MOMZ, DRHOT) -> 5 tendencies."""
        qs = [np.ascontiguousarray(a, np.float64) for a in q]
        out = [np.zeros(self.shape) for _ in range(5)]
        pq, _k1 = _pp(qs)
        po, _k2 = _pp(out)
        dp = _ptr(np.ascontiguousarray(dpres, np.float64)) if dpres is not None else None
        self.lib.orc_cal_tend(self._h, int(hevi), pq, dp, po)
        return out

    def cal_vi(self, q, q0, impl_fac, dt, max_iter=1, tol=0.0, want_iters=False):
        qs = [np.ascontiguousarray(a, np.float64) for a in q]
        q0s = [np.ascontiguousarray(a, np.float64) for a in q0]
        out = [np.zeros(self.shape) for _ in range(5)]
        ncol = self.NeX * self.NeY * self.N1 * self.N1
        its = np.zeros(ncol, np.int32)
        pq, _k1 = _pp(qs)
        pz, _k2 = _pp(q0s)
        po, _k3 = _pp(out)
        nfail = self.lib.orc_cal_vi(self._h, pq, pz, float(impl_fac), float(dt), int(max_iter), float(tol), po,
                                    its.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        if want_iters:
            return out, int(nfail), its
        return out

    def vi_operator(self, P, q0):
        """The implicit (vertical) operator A(P) of cal_vi on every column, with its Rusanov speed
        frozen at q0: the operator whose Newton solve cal_vi performs."""
        ps = [np.ascontiguousarray(a, np.float64) for a in P]
        q0s = [np.ascontiguousarray(a, np.float64) for a in q0]
        out = [np.zeros(self.shape) for _ in range(5)]
        pp_, _k1 = _pp(ps)
        pz, _k2 = _pp(q0s)
        po, _k3 = _pp(out)
        self.lib.orc_vi_operator(self._h, pp_, pz, po)
        return out

    def modalfilter(self, q):
        qs = [np.ascontiguousarray(a, np.float64).copy() for a in q]
        pq, _k = _pp(qs)
        self.lib.orc_modalfilter(self._h, pq)
        return qs

    def step_heve(self, q, dt, nsteps):
        qs = [np.ascontiguousarray(a, np.float64).copy() for a in q]
        pq, _k = _pp(qs)
        self.lib.orc_step_heve(self._h, pq, float(dt), int(nsteps))
        return qs

    def step_hevi(self, q, dt, nsteps, max_iter=1, tol=0.0):
        qs = [np.ascontiguousarray(a, np.float64).copy() for a in q]
        pq, _k = _pp(qs)
        mi = ctypes.c_double(0.0)
        nfail = self.lib.orc_step_hevi(self._h, pq, float(dt), int(nsteps), int(max_iter), float(tol),
                                       ctypes.byref(mi))
        return qs, int(nfail), float(mi.value)

    # ---- part of a domain decomposed along x and/or y (scale_meshfieldcomm_base.F90:340-470) ----
    def halo_pack(self, q, dpres, sides=(0, 1)):
        """The boundary face layers of this part, {side: [6 fields][boundary elements * N1*N1]} for the
        halo sides (0 x-, 1 x+, 2 y-, 3 y+): side 0 the nodes (0, a, b) of the elements ex = 0, side 1
        the nodes (N, a, b) of ex = NeX-1 (elements in the order ey + NeY ez), sides 2 and 3 the nodes
        (a, 0, b) of ey = 0 and (a, N, b) of ey = NeY-1 (order ex + NeX ez); face node a + N1 b; fields
        DDENS, MOMX, MOMY, MOMZ, DRHOT, DPRES (the library's buffer layout)."""
        N1 = self.N1
        out = {}
        fields = [np.asarray(a, np.float64).reshape(self.NeZ, self.NeY, self.NeX, N1, N1, N1)  # ez ey ex k j i
                  for a in list(q) + [dpres]]
        for sd in sides:
            if sd < 2:
                ex, i = (0, 0) if sd == 0 else (self.NeX - 1, N1 - 1)
                out[sd] = np.stack([x[:, :, ex, :, :, i].reshape(-1) for x in fields])  # (ez, ey, b, a)
            else:
                ey, j = (0, 0) if sd == 2 else (self.NeY - 1, N1 - 1)
                out[sd] = np.stack([x[:, ey, :, :, j, :].reshape(-1) for x in fields])  # (ez, ex, b, a)
        return out

    def set_halo(self, exchange, sides=(0, 1)):
        """Makes this oracle one part of a decomposed domain with halo exchanges on `sides`: before
        every tendency of step_hevi/step_heve, exchange(stage, send, recv) gets the packed layers (send,
        as halo_pack) and must fill recv[opposite side] of each neighbour's layer in place: recv[0] with
        the x- neighbour's send[1], recv[1] with the x+ neighbour's send[0], recv[2] and recv[3] the
        same in y."""
        n = self.Np * self.Ne
        Nfp = self.N1 * self.N1
        self._hrecv = {sd: np.zeros((6, (self.NeY if sd < 2 else self.NeX) * self.NeZ * Nfp)) for sd in sides}
        self.halo_errors = []

        def cb(_user, stage, qpp, dpp):
            try:
                q = [np.ctypeslib.as_array(qpp[v], shape=(n,)) for v in range(5)]
                dp = np.ctypeslib.as_array(dpp, shape=(n,))
                exchange(int(stage), self.halo_pack(q, dp, sides), self._hrecv)
            except Exception as e:  # a ctypes callback cannot raise into C
                self.halo_errors.append(e)

        self._halo_cb = HALO_CB(cb)
        self._hptrs = (_dp * 4)(*[_ptr(self._hrecv[sd]) if sd in self._hrecv else None for sd in range(4)])
        self.lib.orc_set_halo(self._h, self._hptrs, self._halo_cb, None)

    # ---- tracer advection (trcadvect3d_heve.F90, driver_trcadv3d.F90) ----
    # Face-node arrays (alph_dens) have shape (Ne, 6, N1*N1): FElib's (NfpTot, Ne).

    @property
    def face_shape(self):
        return (self.Ne, 6, self.N1 * self.N1)

    def trc_alphdens_advtest(self, ddens, momx, momy, momz):
        aM, aP = np.zeros(self.face_shape), np.zeros(self.face_shape)
        a = [_c64(x) for x in (ddens, momx, momy, momz)]
        self.lib.orc_trc_alphdens_advtest(self._h, *[_ptr(x) for x in a], _ptr(aM), _ptr(aP))
        return aM, aP

    def trc_save_massflux(self, rkstage, q, w_h, w_v, is_hevi, mflx, aM, aP, dpres=None):
        """Updates mflx (3 arrays) and aM, aP in place (stage 1 resets them)."""
        qs = [_c64(x) for x in q]
        pq, _k1 = _pp(qs)
        pm, _k2 = _pp(mflx)
        dp = _c64(dpres)
        self.lib.orc_trc_save_massflux(self._h, int(rkstage), pq, _optr(dp), float(w_h), float(w_v), int(is_hevi),
                                       pm, _ptr(aM), _ptr(aP))

    def trc_fct_coef(self, Q, mflx, aM, aP, ddens, ddens0, c_ssm1, dt, rhoq_tp=None):
        fct = np.zeros(self.shape)
        ms = [_c64(x) for x in mflx]
        pm, _k = _pp(ms)
        rq = _c64(rhoq_tp)
        self.lib.orc_trc_fct_coef(self._h, _ptr(_c64(Q)), pm, _optr(rq), _ptr(_c64(aM)), _ptr(_c64(aP)),
                                  _ptr(_c64(ddens)), _ptr(_c64(ddens0)), float(c_ssm1), float(dt), _ptr(fct))
        return fct

    def trc_cal_tend(self, Q, mflx, aM, aP, fct, rhoq_tp=None):
        out = np.zeros(self.shape)
        ms = [_c64(x) for x in mflx]
        pm, _k = _pp(ms)
        rq = _c64(rhoq_tp)
        self.lib.orc_trc_cal_tend(self._h, _ptr(_c64(Q)), pm, _ptr(_c64(aM)), _ptr(_c64(aP)), _ptr(_c64(fct)),
                                  _optr(rq), _ptr(out))
        return out

    def trc_tmar(self, Q, ddens):
        q = np.array(Q, np.float64, copy=True, order="C")
        self.lib.orc_trc_tmar(self._h, _ptr(q), _ptr(_c64(ddens)))
        return q

    def trc_filter(self, Q, ddens, etac_h=2.0 / 3.0, alpha_h=36.0, ord_h=16, etac_v=2.0 / 3.0, alpha_v=36.0,
                   ord_v=16):
        q = np.array(Q, np.float64, copy=True, order="C")
        self.lib.orc_trc_filter(self._h, _ptr(q), _ptr(_c64(ddens)), float(etac_h), float(alpha_h), int(ord_h),
                                float(etac_v), float(alpha_v), int(ord_v))
        return q

    def trc_step(self, QTRC, mflx, aM, aP, ddens_trc, ddens0_trc, dt, nsteps=1, ddens=None, rhoq_tp=None,
                 scheme="ERK_SSP_3s3o", limiter=True, tmar=True, filter=None):
        """nsteps tracer steps (fixed mass flux and densities); filter = None or a dict of the six
        tracer filter parameters (etac_h, alpha_h, ord_h, etac_v, alpha_v, ord_v)."""
        from timeint_ref import tables

        tb = tables(scheme)
        q = np.array(QTRC, np.float64, copy=True, order="C")
        ms = [_c64(x) for x in mflx]
        pm, _k = _pp(ms)
        sig = np.ascontiguousarray(tb["sig"], np.float64)
        gam = np.ascontiguousarray(tb["gam"], np.float64)
        c = np.ascontiguousarray(tb["c"], np.float64)
        fp = dict(etac_h=2.0 / 3.0, alpha_h=36.0, ord_h=16, etac_v=2.0 / 3.0, alpha_v=36.0, ord_v=16)
        if filter:
            fp.update(filter)
        filt = np.array([fp["etac_h"], fp["alpha_h"], fp["ord_h"], fp["etac_v"], fp["alpha_v"], fp["ord_v"]],
                        np.float64)
        self.lib.orc_trc_step(self._h, _ptr(q), pm, _ptr(_c64(aM)), _ptr(_c64(aP)), _ptr(_c64(ddens_trc)),
                              _ptr(_c64(ddens0_trc)), _optr(_c64(ddens)), _optr(_c64(rhoq_tp)), int(tb["nstage"]),
                              _ptr(sig), _ptr(gam), _ptr(c), float(dt), int(bool(limiter)), int(bool(tmar)),
                              int(bool(filter)), _ptr(filt), int(nsteps))
        return q

    # ---- numerical diffusion (nonhydro3d_numdiff.F90) and sponge layer (dgm_spongelayer.F90) ----
    def numdiff_apply(self, q, nlap, coef_h, coef_v, dt):
        """returns a copy of the 5 fields after the hyperdiffusion filter"""
        qs = [np.array(a, np.float64, copy=True, order="C") for a in q]
        pq, _k = _pp(qs)
        self.lib.orc_numdiff_apply(self._h, pq, int(nlap), float(coef_h), float(coef_v), float(dt))
        return qs

    def sponge_add_tend(self, tend, mom, tau, height, hvel=False):
        """returns copies of (MOMX_dt, MOMY_dt, MOMZ_dt) with the Rayleigh damping added"""
        ts = [np.array(a, np.float64, copy=True, order="C") for a in tend]
        ms = [_c64(a) for a in mom]
        pt, _k1 = _pp(ts)
        pm, _k2 = _pp(ms)
        self.lib.orc_sponge_add_tend(self._h, pt, pm, float(tau), float(height), int(bool(hvel)))
        return ts

    def set_trc_flux(self, outs):
        """outs = [MFLX_x, MFLX_y, MFLX_z, alph_M, alph_P, DDENS_TRC, DDENS0_TRC] (filled by step_heve /
        step_hevi in place) or None"""
        if outs is None:
            self.lib.orc_set_trc_flux(self._h, None)
            self._trc_keep = None
            return
        for a in outs:
            assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
        pq, keep = _pp(outs)
        self._trc_keep = (pq, keep)
        self.lib.orc_set_trc_flux(self._h, pq)

    def set_sponge(self, tau, height=0.0, hvel=False):
        """sponge layer inside step_heve / step_hevi (tau <= 0: off)"""
        self.lib.orc_set_sponge(self._h, float(tau), float(height), int(bool(hvel)))
