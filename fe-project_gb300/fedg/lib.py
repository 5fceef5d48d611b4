"""ctypes binding of ``libfedg.so`` (the C ABI declared in ``include/fedg.h``).

This is the host-side mirror of FElib's operator interface for the dynamics hot path:
``cal_tend_ex`` / ``cal_vi`` (FElib/src/fluid_dyn_solver/scale_atm_dyn_dgm_driver_nonhydro3d.F90:
152-250), the ``timeint_rk`` stage methods (FElib/src/common/scale_timeint_rk.F90:81-104) and
the driver's ``update`` loop (:614-963).  Device memory is held in torch CUDA tensors; the
library only sees raw device pointers.  There is no CPU fallback: constructing a
:class:`Context` without the compiled library or without a GPU raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(_HERE)
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libfedg.so")

HEVE, HEVI = 0, 1
SSP_RK3, IMEX_ARK232 = 0, 1
PREC_FP64, PREC_MIXED, PREC_PAIR = 0, 1, 2

EXPORTED = [
    "fedg_last_error", "fedg_ctx_create", "fedg_ctx_destroy", "fedg_ctx_stream", "fedg_synchronize",
    "fedg_set_base_state", "fedg_drhot2pres", "fedg_cal_tend_ex", "fedg_cal_vi", "fedg_modalfilter",
    "fedg_tint_create", "fedg_tint_destroy", "fedg_tint_nstage", "fedg_tint_implicit_diagfac",
    "fedg_tint_tend_ex", "fedg_tint_tend_im", "fedg_tint_var0", "fedg_tint_store_var0",
    "fedg_tint_store_implicit", "fedg_tint_advance", "fedg_update",
    "fedg_prof_enable", "fedg_prof_reset", "fedg_prof_read",
    "fedg_guess_create", "fedg_guess_destroy", "fedg_guess_num_params", "fedg_guess_set_scales",
    "fedg_guess_set_params", "fedg_guess_get_params", "fedg_guess_train_step", "fedg_guess_loss_grad",
    "fedg_guess_predict", "fedg_guess_load", "fedg_cal_tend_ex_noalloc",
    "fedg_trc_alphdens_advtest", "fedg_trc_save_massflux", "fedg_trc_fct_coef", "fedg_trc_cal_tend",
    "fedg_trc_tmar", "fedg_trc_modalfilter", "fedg_trc_update", "fedg_trc_negative_fixer",
    "fedg_trc_specific_heat_pressure", "fedg_numdiff_apply",
    "fedg_sponge_add_tend",
    "fedg_update_set_tracer_flux", "fedg_update_set_sponge", "fedg_numdiff_apply_prec",
    "fedg_guess_set_wait_limit", "fedg_update_set_vi_neumann", "fedg_update_set_wait_limit",
    "fedg_restart_write", "fedg_restart_read",
    "fedg_halo_bytes", "fedg_update_set_halo", "fedg_halo_pack", "fedg_update_set_ref_wind",
    "fedg_update_get_ref_wind", "fedg_update_host",
]

HALO = 2  # fedg_mesh_desc.periodic_x of a slab (FEDG_HALO)
# fedg_halo_fn: int (*)(void* user, int stage)
HALO_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int)

# kernel classes of fedg_prof_read (include/fedg.h)
K_TEND, K_VI, K_RK, K_FILTER, K_PRES, K_MTEND, K_MVI, K_MLP, K_AUX, K_TRC_FCT, K_TRC_TEND, K_TRC_AUX, K_ND, \
    K_COUNT = range(14)
KERNEL_NAMES = ["tend_fp64", "vi_fp64", "rk", "filter", "drhot2pres", "stage_mixed", "vi_mixed", "mlp", "aux",
                "trc_fct", "trc_stage", "trc_aux", "numdiff"]


class MeshDesc(ctypes.Structure):
    _fields_ = [
        ("porder", ctypes.c_int),
        ("NeX", ctypes.c_int), ("NeY", ctypes.c_int), ("NeZ", ctypes.c_int),
        ("xmin", ctypes.c_double), ("xmax", ctypes.c_double),
        ("ymin", ctypes.c_double), ("ymax", ctypes.c_double),
        ("zmin", ctypes.c_double), ("zmax", ctypes.c_double),
        ("periodic_x", ctypes.c_int), ("periodic_y", ctypes.c_int),
        ("grav", ctypes.c_double), ("rdry", ctypes.c_double), ("cpdry", ctypes.c_double),
        ("cvdry", ctypes.c_double), ("pres00", ctypes.c_double),
        ("mf_on", ctypes.c_int),
        ("mf_etac_h", ctypes.c_double), ("mf_alpha_h", ctypes.c_double), ("mf_order_h", ctypes.c_int),
        ("mf_etac_v", ctypes.c_double), ("mf_alpha_v", ctypes.c_double), ("mf_order_v", ctypes.c_int),
        ("device", ctypes.c_int),
    ]


class TrcOpts(ctypes.Structure):
    _fields_ = [("scheme", ctypes.c_int), ("dt", ctypes.c_double), ("nsteps", ctypes.c_int),
                ("limiter", ctypes.c_int), ("tmar", ctypes.c_int), ("filter", ctypes.c_int),
                ("mf_etac_h", ctypes.c_double), ("mf_alpha_h", ctypes.c_double), ("mf_order_h", ctypes.c_int),
                ("mf_etac_v", ctypes.c_double), ("mf_alpha_v", ctypes.c_double), ("mf_order_v", ctypes.c_int),
                ("prec", ctypes.c_int)]


class UpdateOpts(ctypes.Structure):
    _fields_ = [("eqs", ctypes.c_int), ("prec", ctypes.c_int), ("max_iter", ctypes.c_int),
                ("use_guess", ctypes.c_int), ("dt", ctypes.c_double), ("tol", ctypes.c_double)]


_lib = None
_vp = ctypes.c_void_p
_P5 = ctypes.c_void_p * 5


class RestartInfo(ctypes.Structure):
    _fields_ = [("step", ctypes.c_longlong), ("time", ctypes.c_double), ("dt", ctypes.c_double),
                ("scheme", ctypes.c_char * 32)]


def load():
    """Load libfedg.so; raises if it has not been built (no silent fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libfedg.so not built ({LIB_PATH}); run __graft_entry__.build()")
    lib = ctypes.CDLL(LIB_PATH)
    lib.fedg_last_error.restype = ctypes.c_char_p
    lib.fedg_ctx_create.argtypes = [ctypes.POINTER(MeshDesc), ctypes.POINTER(_vp)]
    lib.fedg_ctx_destroy.argtypes = [_vp]
    lib.fedg_ctx_stream.restype = _vp
    lib.fedg_ctx_stream.argtypes = [_vp]
    lib.fedg_synchronize.argtypes = [_vp]
    lib.fedg_set_base_state.argtypes = [_vp] + [_vp] * 9
    lib.fedg_drhot2pres.argtypes = [_vp, _vp, _vp, _vp]
    lib.fedg_cal_tend_ex.argtypes = [_vp, ctypes.c_void_p * 16, _P5, ctypes.c_int]
    lib.fedg_cal_tend_ex_noalloc.argtypes = [_vp, ctypes.c_void_p * 16, _P5, ctypes.c_int]
    lib.fedg_cal_vi.argtypes = [_vp, ctypes.c_void_p * 12, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                ctypes.c_double, _P5, _vp]
    lib.fedg_modalfilter.argtypes = [_vp, _P5]
    lib.fedg_tint_create.argtypes = [_vp, ctypes.c_int, ctypes.c_double, ctypes.POINTER(_vp)]
    lib.fedg_tint_destroy.argtypes = [_vp]
    lib.fedg_tint_nstage.argtypes = [_vp]
    lib.fedg_tint_implicit_diagfac.restype = ctypes.c_double
    lib.fedg_tint_implicit_diagfac.argtypes = [_vp, ctypes.c_int]
    for nm in ("fedg_tint_tend_ex", "fedg_tint_tend_im"):
        getattr(lib, nm).restype = _vp
        getattr(lib, nm).argtypes = [_vp, ctypes.c_int, ctypes.c_int]
    lib.fedg_tint_var0.restype = _vp
    lib.fedg_tint_var0.argtypes = [_vp, ctypes.c_int]
    lib.fedg_tint_store_var0.argtypes = [_vp, _P5]
    lib.fedg_tint_store_implicit.argtypes = [_vp, ctypes.c_int, _P5]
    lib.fedg_tint_advance.argtypes = [_vp, ctypes.c_int, _P5]
    lib.fedg_update.argtypes = [_vp, _P5, ctypes.c_int, ctypes.POINTER(UpdateOpts), ctypes.POINTER(ctypes.c_double)]
    _fp = ctypes.POINTER(ctypes.c_float)
    lib.fedg_guess_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp)]
    lib.fedg_guess_destroy.argtypes = [_vp]
    lib.fedg_guess_num_params.restype = ctypes.c_longlong
    lib.fedg_guess_num_params.argtypes = [_vp]
    lib.fedg_guess_set_scales.argtypes = [_vp, _fp, _fp]
    lib.fedg_guess_set_params.argtypes = [_vp, _fp, ctypes.c_longlong]
    lib.fedg_guess_get_params.argtypes = [_vp, _fp, ctypes.c_longlong]
    lib.fedg_guess_train_step.argtypes = [_vp, _vp, _vp, ctypes.c_int, ctypes.c_float, _fp]
    lib.fedg_guess_loss_grad.argtypes = [_vp, _vp, _vp, ctypes.c_int, _fp, _fp]
    lib.fedg_guess_predict.argtypes = [_vp, _vp, _vp, ctypes.c_int]
    lib.fedg_guess_load.argtypes = [_vp, _vp]
    lib.fedg_guess_set_wait_limit.argtypes = [_vp, ctypes.c_int]
    lib.fedg_update_set_vi_neumann.argtypes = [_vp, ctypes.c_int]
    lib.fedg_update_set_wait_limit.argtypes = [_vp, ctypes.c_int]
    lib.fedg_restart_write.argtypes = [_vp, ctypes.c_char_p, _P5, ctypes.POINTER(RestartInfo)]
    lib.fedg_restart_read.argtypes = [_vp, ctypes.c_char_p, _P5, ctypes.c_void_p, ctypes.POINTER(RestartInfo)]
    _P3 = ctypes.c_void_p * 3
    lib.fedg_trc_alphdens_advtest.argtypes = [_vp] + [_vp] * 6
    lib.fedg_trc_save_massflux.argtypes = [_vp, ctypes.c_int, _P5, _vp, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_int, _P3, _vp, _vp]
    lib.fedg_trc_fct_coef.argtypes = [_vp, _vp, _P3, _vp, _vp, _vp, _vp, _vp, ctypes.c_double, ctypes.c_double, _vp]
    lib.fedg_trc_cal_tend.argtypes = [_vp, _vp, _P3, _vp, _vp, _vp, _vp, _vp]
    lib.fedg_trc_tmar.argtypes = [_vp, _vp, _vp]
    _dp = ctypes.POINTER(ctypes.c_double)
    lib.fedg_trc_negative_fixer.argtypes = [_vp, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, _dp, _dp, _dp, _dp] + [_vp] * 8 + [ctypes.c_double]
    lib.fedg_trc_specific_heat_pressure.argtypes = [_vp, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                                    _dp, _dp, _dp, _dp] + [_vp] * 8
    lib.fedg_trc_modalfilter.argtypes = [_vp, _vp, _vp, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_int]
    lib.fedg_trc_update.argtypes = [_vp, _vp, _P3, _vp, _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(TrcOpts)]
    lib.fedg_update_set_tracer_flux.argtypes = [_vp, ctypes.POINTER(ctypes.c_void_p), _vp, _vp, _vp, _vp]
    lib.fedg_update_set_sponge.argtypes = [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    lib.fedg_numdiff_apply.argtypes = [_vp, _P5, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double]
    lib.fedg_numdiff_apply_prec.argtypes = [_vp, _P5, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_int]
    lib.fedg_sponge_add_tend.argtypes = [_vp, _P3, _P3, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    lib.fedg_prof_enable.argtypes = [_vp, ctypes.c_int]
    lib.fedg_prof_reset.argtypes = [_vp]
    lib.fedg_prof_read.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                   ctypes.POINTER(ctypes.c_longlong)]
    lib.fedg_update_host.argtypes = [_vp, _P5, ctypes.c_int, ctypes.POINTER(UpdateOpts), ctypes.POINTER(ctypes.c_double)]
    lib.fedg_halo_bytes.restype = ctypes.c_size_t
    lib.fedg_halo_bytes.argtypes = [_vp, ctypes.c_int]
    lib.fedg_update_set_halo.argtypes = [_vp, ctypes.c_void_p * 4, ctypes.c_void_p * 4, HALO_FN, ctypes.c_void_p]
    lib.fedg_halo_pack.argtypes = [_vp, _P5, _vp]
    lib.fedg_update_set_ref_wind.argtypes = [_vp, ctypes.c_double, ctypes.c_double]
    lib.fedg_update_get_ref_wind.argtypes = [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    _lib = lib
    return lib


def last_error() -> str:
    return load().fedg_last_error().decode()


class FedgError(RuntimeError):
    pass


def _check(rc: int, what: str) -> int:
    if rc < 0:
        raise FedgError(f"{what} failed ({rc}): {last_error()}")
    return rc


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _p5(ts):
    return _P5(*[t.data_ptr() for t in ts])


class Context:
    """One fedg context (mesh, operators, base state, CUDA stream) on one GPU."""

    def __init__(self, case, device: int = 0, filter_on=None, periodic_x: int = 1, periodic_y: int = 1):
        import torch

        if not torch.cuda.is_available():
            raise RuntimeError("fedg: no CUDA device (the library has no CPU fallback)")
        self.lib = load()
        self.case = case
        self.torch = torch
        self.dev = torch.device("cuda", device)
        xmin, xmax, ymin, ymax, zmin, zmax = case.dom
        from .cases import CPDRY, CVDRY, GRAV, PRES00, RDRY

        fo = case.filter_on if filter_on is None else filter_on
        d = MeshDesc(case.porder, case.NeX, case.NeY, case.NeZ, xmin, xmax, ymin, ymax, zmin, zmax, int(periodic_x), int(periodic_y),
                     getattr(case, "grav", GRAV), RDRY, CPDRY, CVDRY, PRES00, int(fo), 2.0 / 3.0, 36.0, 16,
                     2.0 / 3.0, 36.0, 16, device)
        h = _vp()
        _check(self.lib.fedg_ctx_create(ctypes.byref(d), ctypes.byref(h)), "fedg_ctx_create")
        self.h = h
        self.shape = (case.Ne, case.Np)
        self.ncol = case.NeX * case.NeY * case.N1 * case.N1
        self._base = None
        self._coriolis = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.fedg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- helpers --
    def tensor(self, a):
        t = self.torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).to(self.dev)
        return t.contiguous()

    def empty(self):
        return self.torch.empty(self.shape, dtype=self.torch.float64, device=self.dev)

    def sync(self):
        _check(self.lib.fedg_synchronize(self.h), "fedg_synchronize")

    @property
    def stream_handle(self):
        return self.lib.fedg_ctx_stream(self.h)

    # -- FElib interface --
    def set_base_state(self, dens_hyd, pres_hyd, therm_hyd, coriolis_f=0.0):
        """Registers the base state; coriolis_f != 0 passes a constant 2D CORIOLIS(Np2D, NeA2D) field
        (an f-plane), as FElib's AUX_VARS2D would hold it."""
        b = [self.tensor(dens_hyd), self.tensor(pres_hyd), self.tensor(therm_hyd)]
        cor = None
        if coriolis_f:
            c = self.case
            cor = self.torch.full((c.NeX * c.NeY, c.N1 * c.N1), float(coriolis_f), dtype=self.torch.float64,
                                  device=self.dev)
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_set_base_state(self.h, _ptr(b[0]), _ptr(b[1]), _ptr(b[2]), None, None, None, None,
                                            None, _ptr(cor) if cor is not None else None), "fedg_set_base_state")
        self._base = b
        self._coriolis = cor
        return b

    def drhot2pres(self, drhot):
        pres, dpres = self.empty(), self.empty()
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_drhot2pres(self.h, _ptr(drhot), _ptr(pres), _ptr(dpres)), "fedg_drhot2pres")
        self.sync()
        return pres, dpres

    def cal_tend_ex(self, q, eqs, dpres=None):
        out = [self.empty() for _ in range(5)]
        b = self._base
        cor = getattr(self, "_coriolis", None)
        ins = (ctypes.c_void_p * 16)(*[t.data_ptr() for t in q], dpres.data_ptr() if dpres is not None else None,
                                     b[0].data_ptr(), b[1].data_ptr(), None, b[2].data_ptr(),
                                     cor.data_ptr() if cor is not None else None, None, None, None, None, None)
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_cal_tend_ex(self.h, ins, _p5(out), int(eqs)), "fedg_cal_tend_ex")
        self.sync()
        return out

    def cal_vi(self, q, q0, impl_fac, dt, max_iter=1, tol=0.0, want_status=False):
        out = [self.empty() for _ in range(5)]
        b = self._base
        ins = (ctypes.c_void_p * 12)(*[t.data_ptr() for t in q], b[0].data_ptr(), b[1].data_ptr(),
                                     *[t.data_ptr() for t in q0])
        st = self.torch.zeros(self.ncol, dtype=self.torch.int32, device=self.dev)
        self.torch.cuda.synchronize()
        nfail = _check(self.lib.fedg_cal_vi(self.h, ins, float(impl_fac), float(dt), int(max_iter), float(tol),
                                            _p5(out), _ptr(st)), "fedg_cal_vi")
        self.sync()
        if want_status:
            return out, nfail, st
        return out

    def modalfilter(self, q):
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_modalfilter(self.h, _p5(q)), "fedg_modalfilter")
        self.sync()
        return q

    def update(self, q, nsteps, *, eqs=None, prec=PREC_FP64, dt=None, max_iter=1, tol=0.0, use_guess=False,
               sync=True):
        eqs = (HEVE if self.case.eqs == "HEVE" else HEVI) if eqs is None else eqs
        o = UpdateOpts(int(eqs), int(prec), int(max_iter), int(bool(use_guess)),
                       float(self.case.dt if dt is None else dt), float(tol))
        mi = ctypes.c_double(0.0)
        if sync:
            self.torch.cuda.synchronize()
        nfail = _check(self.lib.fedg_update(self.h, _p5(q), int(nsteps), ctypes.byref(o), ctypes.byref(mi)),
                       "fedg_update")
        if sync:
            self.sync()
        return nfail, float(mi.value)

    # -- part of a decomposed domain (MeshFieldComm exchange, scale_meshfieldcomm_base.F90:340-470) --
    def halo_bytes(self, side: int) -> int:
        """bytes of the halo buffer of side 0..3 (x-, x+, y-, y+); 0 where the mesh is periodic"""
        return int(self.lib.fedg_halo_bytes(self.h, int(side)))

    def set_halo(self, send, recv, exchange=None):
        """send, recv: four device buffers each (torch tensors of halo_bytes(side) bytes, None on
        periodic sides, kept alive here); exchange(stage) -> None moves send[1] to the x+ neighbour's
        recv[0], send[0] to the x- neighbour's recv[1], send[3] to the y+ neighbour's recv[2] and
        send[2] to the y- neighbour's recv[3], and returns once recv holds the neighbours' data."""
        def fn(_user, stage):
            try:
                exchange(int(stage))
                return 0
            except Exception as e:  # the C caller only sees the status; keep the reason
                self.halo_error = e
                return 1
        self._halo_fn = HALO_FN(fn) if exchange is not None else ctypes.cast(None, HALO_FN)
        self._halo_bufs = (send, recv)
        sp = (ctypes.c_void_p * 4)(*[None if t is None else t.data_ptr() for t in send])
        rp = (ctypes.c_void_p * 4)(*[None if t is None else t.data_ptr() for t in recv])
        _check(self.lib.fedg_update_set_halo(self.h, sp, rp, self._halo_fn, None), "fedg_update_set_halo")

    def halo_pack(self, q, dpres=None):
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_halo_pack(self.h, _p5(q), _ptr(dpres)), "fedg_halo_pack")

    def set_ref_wind(self, u, v):
        _check(self.lib.fedg_update_set_ref_wind(self.h, float(u), float(v)), "fedg_update_set_ref_wind")

    def get_ref_wind(self):
        u, v = ctypes.c_double(), ctypes.c_double()
        r = _check(self.lib.fedg_update_get_ref_wind(self.h, ctypes.byref(u), ctypes.byref(v)), "fedg_update_get_ref_wind")
        return (u.value, v.value) if r else None

    def update_host(self, q_host, nsteps, *, eqs=None, prec=PREC_FP64, dt=None, max_iter=1, tol=0.0,
                    use_guess=False):
        """fedg_update_host: q_host are five page-locked host tensors (torch pin_memory), updated in place"""
        eqs = (HEVE if self.case.eqs == "HEVE" else HEVI) if eqs is None else eqs
        o = UpdateOpts(int(eqs), int(prec), int(max_iter), int(bool(use_guess)),
                       float(self.case.dt if dt is None else dt), float(tol))
        mi = ctypes.c_double(0.0)
        nfail = _check(self.lib.fedg_update_host(self.h, _p5(q_host), int(nsteps), ctypes.byref(o), ctypes.byref(mi)),
                       "fedg_update_host")
        return nfail, float(mi.value)

    # -- restart files (scale_file_restart_meshfield.F90) --
    def restart_write(self, path, q, step=0, time=0.0, dt=0.0, scheme=""):
        info = RestartInfo(int(step), float(time), float(dt), scheme.encode()[:31])
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_restart_write(self.h, str(path).encode(), _p5(q), ctypes.byref(info)),
               "fedg_restart_write")

    def restart_read(self, path, q, base=None):
        """fills the five device fields q (and, when given, the three base-state fields); returns
        (step, time, dt, scheme)"""
        info = RestartInfo()
        bp = (ctypes.c_void_p * 3)(*[t.data_ptr() for t in base]) if base is not None else None
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_restart_read(self.h, str(path).encode(), _p5(q), bp, ctypes.byref(info)),
               "fedg_restart_read")
        return int(info.step), float(info.time), float(info.dt), info.scheme.decode()

    def set_wait_limit(self, polls):
        """polls of the update path's tensor-core barrier waits before they give up (default 1 << 20)"""
        _check(self.lib.fedg_update_set_wait_limit(self.h, int(polls)), "fedg_update_set_wait_limit")

    def set_vi_neumann(self, nterm):
        """Jacobian-vector products of the column solve's Neumann corrections (0: LU only)."""
        _check(self.lib.fedg_update_set_vi_neumann(self.h, int(nterm)), "fedg_update_set_vi_neumann")

    # -- tracer advection (trcadvect3d_heve.F90, driver_trcadv3d.F90) --
    @property
    def face_shape(self):
        return (self.case.Ne, 6, self.case.N1 * self.case.N1)

    def empty_face(self):
        return self.torch.empty(self.face_shape, dtype=self.torch.float64, device=self.dev)

    def trc_alphdens_advtest(self, ddens, momx, momy, momz):
        aM, aP = self.empty_face(), self.empty_face()
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_trc_alphdens_advtest(self.h, _ptr(ddens), _ptr(momx), _ptr(momy), _ptr(momz), _ptr(aM),
                                                  _ptr(aP)), "fedg_trc_alphdens_advtest")
        self.sync()
        return aM, aP

    def trc_save_massflux(self, rkstage, q, w_h, w_v, is_hevi, mflx, aM, aP, dpres=None):
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_trc_save_massflux(self.h, int(rkstage), _p5(q), _ptr(dpres), float(w_h), float(w_v),
                                               int(is_hevi), (ctypes.c_void_p * 3)(*[m.data_ptr() for m in mflx]),
                                               _ptr(aM), _ptr(aP)), "fedg_trc_save_massflux")
        self.sync()

    def trc_fct_coef(self, Q, mflx, aM, aP, ddens, ddens0, c_ssm1, dt, rhoq_tp=None):
        fct = self.empty()
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_trc_fct_coef(self.h, _ptr(Q), (ctypes.c_void_p * 3)(*[m.data_ptr() for m in mflx]),
                                          _ptr(rhoq_tp), _ptr(aM), _ptr(aP), _ptr(ddens), _ptr(ddens0),
                                          float(c_ssm1), float(dt), _ptr(fct)), "fedg_trc_fct_coef")
        self.sync()
        return fct

    def trc_cal_tend(self, Q, mflx, aM, aP, fct=None, rhoq_tp=None):
        out = self.empty()
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_trc_cal_tend(self.h, _ptr(Q), (ctypes.c_void_p * 3)(*[m.data_ptr() for m in mflx]),
                                          _ptr(aM), _ptr(aP), _ptr(fct), _ptr(rhoq_tp), _ptr(out)),
               "fedg_trc_cal_tend")
        self.sync()
        return out

    def trc_tmar(self, Q, ddens):
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_trc_tmar(self.h, _ptr(Q), _ptr(ddens)), "fedg_trc_tmar")
        self.sync()
        return Q

    def trc_negative_fixer(self, qtrc, qla, qia, mass, r, cv, cp, ddens, pres, cvtot, cptot, rtot, dens_hyd,
                           pres_hyd, drhot=None, dt=0.0):
        """fedg_trc_negative_fixer in place on the device tensors qtrc (list of QA), ddens, pres, cvtot,
        cptot, rtot and drhot (or None); mass/r/cv/cp: the QA tracer property values"""
        qa = len(qtrc)
        qp = (ctypes.c_void_p * qa)(*[t.data_ptr() for t in qtrc])
        tab = [(ctypes.c_double * qa)(*[float(x) for x in list(a)[:qa]]) for a in (mass, r, cv, cp)]
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_trc_negative_fixer(self.h, qp, qa, int(qla), int(qia), *tab, _ptr(ddens), _ptr(pres),
                                                _ptr(cvtot), _ptr(cptot), _ptr(rtot), _ptr(dens_hyd),
                                                _ptr(pres_hyd), _ptr(drhot), float(dt)),
               "fedg_trc_negative_fixer")
        self.sync()

    def trc_specific_heat_pressure(self, qtrc, mass, r, cv, cp, drhot, pres_hyd, therm_hyd, rtot, cvtot, cptot, pres,
                                   dpres=None):
        """fedg_trc_specific_heat_pressure: Rtot, CVtot, CPtot, PRES (and DPRES) from the device tensors
        qtrc (list of QA) and DRHOT"""
        qa = len(qtrc)
        qp = (ctypes.c_void_p * max(qa, 1))(*[t.data_ptr() for t in qtrc])
        tab = [(ctypes.c_double * max(qa, 1))(*[float(x) for x in list(a)[:qa]]) for a in (mass, r, cv, cp)]
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_trc_specific_heat_pressure(self.h, qp, qa, *tab, _ptr(drhot), _ptr(pres_hyd),
                                                        _ptr(therm_hyd), _ptr(rtot), _ptr(cvtot), _ptr(cptot),
                                                        _ptr(pres), _ptr(dpres)),
               "fedg_trc_specific_heat_pressure")
        self.sync()

    def trc_modalfilter(self, Q, ddens, etac_h=2.0 / 3.0, alpha_h=36.0, ord_h=16, etac_v=2.0 / 3.0, alpha_v=36.0,
                        ord_v=16):
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_trc_modalfilter(self.h, _ptr(Q), _ptr(ddens), float(etac_h), float(alpha_h), int(ord_h),
                                             float(etac_v), float(alpha_v), int(ord_v)), "fedg_trc_modalfilter")
        self.sync()
        return Q

    def trc_update(self, Q, mflx, aM, aP, ddens_trc, ddens0_trc, dt, nsteps=1, ddens=None, rhoq_tp=None,
                   limiter=True, tmar=True, filter=None, sync=True, prec=PREC_FP64):
        """nsteps tracer steps in place on Q (ERK_SSP_3s3o); filter = None or a dict of the six tracer
        filter parameters (etac_h, alpha_h, ord_h, etac_v, alpha_v, ord_v)."""
        fp = dict(etac_h=2.0 / 3.0, alpha_h=36.0, ord_h=16, etac_v=2.0 / 3.0, alpha_v=36.0, ord_v=16)
        if filter:
            fp.update(filter)
        o = TrcOpts(SSP_RK3, float(dt), int(nsteps), int(bool(limiter)), int(bool(tmar)), int(bool(filter)),
                    fp["etac_h"], fp["alpha_h"], int(fp["ord_h"]), fp["etac_v"], fp["alpha_v"], int(fp["ord_v"]),
                    int(prec))
        if sync:
            self.torch.cuda.synchronize()
        _check(self.lib.fedg_trc_update(self.h, _ptr(Q), (ctypes.c_void_p * 3)(*[m.data_ptr() for m in mflx]),
                                        _ptr(aM), _ptr(aP), _ptr(ddens_trc), _ptr(ddens0_trc), _ptr(ddens),
                                        _ptr(rhoq_tp), ctypes.byref(o)), "fedg_trc_update")
        if sync:
            self.sync()
        return Q

    def set_sponge(self, tau, height=0.0, hveldamp=False):
        """sponge layer inside update() (FP64 path); tau <= 0 turns it off"""
        _check(self.lib.fedg_update_set_sponge(self.h, float(tau), float(height), int(bool(hveldamp))),
               "fedg_update_set_sponge")

    def set_tracer_flux(self, outs):
        """outs = [MFLX_x, MFLX_y, MFLX_z, alph_M, alph_P, DDENS_TRC, DDENS0_TRC] device tensors filled by
        update() (FP64 path), or None to clear"""
        if outs is None:
            _check(self.lib.fedg_update_set_tracer_flux(self.h, None, None, None, None, None),
                   "fedg_update_set_tracer_flux")
            self._trc_keep = None
            return
        self._trc_keep = outs
        _check(self.lib.fedg_update_set_tracer_flux(self.h, (ctypes.c_void_p * 3)(*[m.data_ptr() for m in outs[:3]]),
                                                    _ptr(outs[3]), _ptr(outs[4]), _ptr(outs[5]), _ptr(outs[6])),
               "fedg_update_set_tracer_flux")

    # -- numerical diffusion (nonhydro3d_numdiff.F90) and sponge layer (dgm_spongelayer.F90) --
    def numdiff_apply(self, q, nlap, coef_h, coef_v, dt, prec=PREC_FP64):
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_numdiff_apply_prec(self.h, _p5(q), int(nlap), float(coef_h), float(coef_v), float(dt),
                                                int(prec)), "fedg_numdiff_apply")
        self.sync()
        return q

    def sponge_add_tend(self, tend, mom, tau, height, hveldamp=False):
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_sponge_add_tend(self.h, (ctypes.c_void_p * 3)(*[t.data_ptr() for t in tend]),
                                             (ctypes.c_void_p * 3)(*[m.data_ptr() for m in mom]), float(tau),
                                             float(height), int(bool(hveldamp))), "fedg_sponge_add_tend")
        self.sync()
        return tend


def prof_enable(ctx, on=True):
    _check(ctx.lib.fedg_prof_enable(ctx.h, int(bool(on))), "fedg_prof_enable")


def prof_reset(ctx):
    _check(ctx.lib.fedg_prof_reset(ctx.h), "fedg_prof_reset")


def prof_read(ctx):
    """{kernel_name: (total_ms, launches)} for every kernel class of the context."""
    out = {}
    for k, nm in enumerate(KERNEL_NAMES):
        t = ctypes.c_double(0.0)
        n = ctypes.c_longlong(0)
        _check(ctx.lib.fedg_prof_read(ctx.h, k, ctypes.byref(t), ctypes.byref(n)), "fedg_prof_read")
        out[nm] = (float(t.value), int(n.value))
    return out


class TimeInt:
    """fedg_tint: FElib's timeint_rk object (var0, varTmp, tendency buffers) on the device."""

    def __init__(self, ctx: Context, scheme: int, dt: float):
        self.ctx = ctx
        h = _vp()
        _check(ctx.lib.fedg_tint_create(ctx.h, int(scheme), float(dt), ctypes.byref(h)), "fedg_tint_create")
        self.h = h
        self.nstage = ctx.lib.fedg_tint_nstage(h)

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.fedg_tint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def implicit_diagfac(self, s):
        return self.ctx.lib.fedg_tint_implicit_diagfac(self.h, int(s))

    def _wrap(self, ptr):
        """A torch view of a library-owned device buffer (Ne, Np) float64."""
        torch = self.ctx.torch
        n = self.ctx.shape[0] * self.ctx.shape[1]
        # build a tensor from the raw pointer via __cuda_array_interface__
        class _CAI:
            __cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (int(ptr), False), "version": 3,
                                        "strides": None}
        return torch.as_tensor(_CAI(), device=self.ctx.dev).view(self.ctx.shape)

    def tend_ex(self, s, v):
        return self._wrap(self.ctx.lib.fedg_tint_tend_ex(self.h, int(s), int(v)))

    def tend_im(self, s, v):
        return self._wrap(self.ctx.lib.fedg_tint_tend_im(self.h, int(s), int(v)))

    def var0(self, v):
        return self._wrap(self.ctx.lib.fedg_tint_var0(self.h, int(v)))

    def store_var0(self, q):
        _check(self.ctx.lib.fedg_tint_store_var0(self.h, _p5(q)), "fedg_tint_store_var0")

    def store_implicit(self, s, q):
        _check(self.ctx.lib.fedg_tint_store_implicit(self.h, int(s), _p5(q)), "fedg_tint_store_implicit")

    def advance(self, s, q):
        _check(self.ctx.lib.fedg_tint_advance(self.h, int(s), _p5(q)), "fedg_tint_advance")


class Guess:
    """fedg_guess: the column-guess MLP (levels -> din = 3*levels+1, dout = 3*levels)."""

    def __init__(self, levels: int, hidden: int = 256):
        self.lib = load()
        h = _vp()
        _check(self.lib.fedg_guess_create(int(levels), int(hidden), ctypes.byref(h)), "fedg_guess_create")
        self.h = h
        self.levels, self.hidden = levels, hidden
        self.din, self.dout = 3 * levels + 1, 3 * levels
        self.n = int(self.lib.fedg_guess_num_params(h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.fedg_guess_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shapes(self):
        h, di, do = self.hidden, self.din, self.dout
        return [(h, di), (h,), (h, h), (h,), (do, h), (do,)]

    def set_scales(self, in_scale, out_scale):
        a = (ctypes.c_float * 4)(*[float(x) for x in in_scale])
        b = (ctypes.c_float * 3)(*[float(x) for x in out_scale])
        _check(self.lib.fedg_guess_set_scales(self.h, a, b), "fedg_guess_set_scales")
        self.in_scale, self.out_scale = list(in_scale), list(out_scale)

    def set_params(self, flat):
        flat = np.ascontiguousarray(flat, dtype=np.float32)
        assert flat.size == self.n
        _check(self.lib.fedg_guess_set_params(self.h, flat.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), self.n),
               "fedg_guess_set_params")

    def get_params(self):
        out = np.zeros(self.n, np.float32)
        _check(self.lib.fedg_guess_get_params(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), self.n),
               "fedg_guess_get_params")
        return out

    def init_params(self, seed=0):
        rng = np.random.default_rng(seed)
        parts = []
        for shp in self.shapes():
            if len(shp) == 2:
                parts.append((rng.standard_normal(shp) * np.sqrt(2.0 / (shp[0] + shp[1]))).ravel())
            else:
                parts.append(np.zeros(shp))
        self.set_params(np.concatenate(parts).astype(np.float32))

    def train_step(self, X, T, lr=1e-3):
        loss = ctypes.c_float(0.0)
        import torch

        torch.cuda.synchronize()
        _check(self.lib.fedg_guess_train_step(self.h, _ptr(X), _ptr(T), int(X.shape[0]), float(lr),
                                              ctypes.byref(loss)), "fedg_guess_train_step")
        return float(loss.value)

    def loss_grad(self, X, T):
        import torch

        loss = ctypes.c_float(0.0)
        g = np.zeros(self.n, np.float32)
        torch.cuda.synchronize()
        _check(self.lib.fedg_guess_loss_grad(self.h, _ptr(X), _ptr(T), int(X.shape[0]), ctypes.byref(loss),
                                             g.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
               "fedg_guess_loss_grad")
        return float(loss.value), g

    def predict(self, X):
        import torch

        Y = torch.empty((X.shape[0], self.dout), dtype=torch.float32, device=X.device)
        torch.cuda.synchronize()
        _check(self.lib.fedg_guess_predict(self.h, _ptr(X), _ptr(Y), int(X.shape[0])), "fedg_guess_predict")
        torch.cuda.synchronize()
        return Y

    # -- part of a decomposed domain (MeshFieldComm exchange, scale_meshfieldcomm_base.F90:340-470) --
    def halo_bytes(self, side: int) -> int:
        """bytes of the halo buffer of side 0..3 (x-, x+, y-, y+); 0 where the mesh is periodic"""
        return int(self.lib.fedg_halo_bytes(self.h, int(side)))

    def set_halo(self, send, recv, exchange=None):
        """send, recv: four device buffers each (torch tensors of halo_bytes(side) bytes, None on
        periodic sides, kept alive here); exchange(stage) -> None moves send[1] to the x+ neighbour's
        recv[0], send[0] to the x- neighbour's recv[1], send[3] to the y+ neighbour's recv[2] and
        send[2] to the y- neighbour's recv[3], and returns once recv holds the neighbours' data."""
        def fn(_user, stage):
            try:
                exchange(int(stage))
                return 0
            except Exception as e:  # the C caller only sees the status; keep the reason
                self.halo_error = e
                return 1
        self._halo_fn = HALO_FN(fn) if exchange is not None else ctypes.cast(None, HALO_FN)
        self._halo_bufs = (send, recv)
        sp = (ctypes.c_void_p * 4)(*[None if t is None else t.data_ptr() for t in send])
        rp = (ctypes.c_void_p * 4)(*[None if t is None else t.data_ptr() for t in recv])
        _check(self.lib.fedg_update_set_halo(self.h, sp, rp, self._halo_fn, None), "fedg_update_set_halo")

    def halo_pack(self, q, dpres=None):
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_halo_pack(self.h, _p5(q), _ptr(dpres)), "fedg_halo_pack")

    def set_ref_wind(self, u, v):
        _check(self.lib.fedg_update_set_ref_wind(self.h, float(u), float(v)), "fedg_update_set_ref_wind")

    def get_ref_wind(self):
        u, v = ctypes.c_double(), ctypes.c_double()
        r = _check(self.lib.fedg_update_get_ref_wind(self.h, ctypes.byref(u), ctypes.byref(v)), "fedg_update_get_ref_wind")
        return (u.value, v.value) if r else None

    def update_host(self, q_host, nsteps, *, eqs=None, prec=PREC_FP64, dt=None, max_iter=1, tol=0.0,
                    use_guess=False):
        """fedg_update_host: q_host are five page-locked host tensors (torch pin_memory), updated in place"""
        eqs = (HEVE if self.case.eqs == "HEVE" else HEVI) if eqs is None else eqs
        o = UpdateOpts(int(eqs), int(prec), int(max_iter), int(bool(use_guess)),
                       float(self.case.dt if dt is None else dt), float(tol))
        mi = ctypes.c_double(0.0)
        nfail = _check(self.lib.fedg_update_host(self.h, _p5(q_host), int(nsteps), ctypes.byref(o), ctypes.byref(mi)),
                       "fedg_update_host")
        return nfail, float(mi.value)

    # -- restart files (scale_file_restart_meshfield.F90) --
    def restart_write(self, path, q, step=0, time=0.0, dt=0.0, scheme=""):
        info = RestartInfo(int(step), float(time), float(dt), scheme.encode()[:31])
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_restart_write(self.h, str(path).encode(), _p5(q), ctypes.byref(info)),
               "fedg_restart_write")

    def restart_read(self, path, q, base=None):
        """fills the five device fields q (and, when given, the three base-state fields); returns
        (step, time, dt, scheme)"""
        info = RestartInfo()
        bp = (ctypes.c_void_p * 3)(*[t.data_ptr() for t in base]) if base is not None else None
        self.torch.cuda.synchronize()
        _check(self.lib.fedg_restart_read(self.h, str(path).encode(), _p5(q), bp, ctypes.byref(info)),
               "fedg_restart_read")
        return int(info.step), float(info.time), float(info.dt), info.scheme.decode()

    def set_wait_limit(self, polls):
        """polls of the tensor-core GEMMs' barrier waits before they give up (default 1 << 20)"""
        _check(self.lib.fedg_guess_set_wait_limit(self.h, int(polls)), "fedg_guess_set_wait_limit")

    def attach(self, ctx):
        _check(self.lib.fedg_guess_load(ctx.h, self.h), "fedg_guess_load")
        ctx._guess = self


def detach_guess(ctx):
    _check(ctx.lib.fedg_guess_load(ctx.h, None), "fedg_guess_load")
    ctx._guess = None
