"""ctypes binding of the phantom_gb300 C ABI (include/phantom_gb300.h).

This is the Python-side mirror of the reference's call surface for the hot
path: ``build_tree`` (maketree, kdtree.F90:117), ``densityiterate``
(dens.F90:117), ``force`` (force.F90:193), ``derivs`` (deriv.f90:37) and
``step`` (step_leapfrog.f90:91). Arrays use the reference layout: one row of
4 values per particle for xyzh/vxyzu/Bevol/fxyzu/dBevol (float64), float32 for
gradh/divcurlv/divcurlB/divBsymm/poten.

The CUDA library is required: importing succeeds without it, but every call
raises ``RuntimeError`` if ``libphantom_gb300.so`` is missing or no GPU is
visible. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libphantom_gb300.so")

PH_PREC_FP64 = 0
PH_PREC_MIXED = 1
PH_ERR_NOT_BUILT = 14
PH_ERR_SCRATCH_LIMIT = 15
PH_ERR_IND = 16
PH_ERR_IND_DT = 17
PH_NOALLOC_MAX_PARTICLES = 4194304  # static scratch limit of ph_conservation_noalloc


class PhParams(C.Structure):
    _fields_ = [
        ("periodic", C.c_int32), ("mhd", C.c_int32), ("gravity", C.c_int32),
        ("isothermal", C.c_int32), ("ieos", C.c_int32), ("ipdv_heating", C.c_int32),
        ("ishock_heating", C.c_int32), ("iresistive_heating", C.c_int32),
        ("precision", C.c_int32), ("minpart", C.c_int32),
        ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double),
        ("ymax", C.c_double), ("zmin", C.c_double), ("zmax", C.c_double),
        ("hfact", C.c_double), ("tolh", C.c_double), ("massoftype", C.c_double),
        ("alpha", C.c_double), ("alphau", C.c_double), ("alphaB", C.c_double),
        ("beta", C.c_double), ("gamma", C.c_double), ("polyk", C.c_double),
        ("C_cour", C.c_double), ("C_force", C.c_double), ("tolv", C.c_double),
        ("dtmax", C.c_double), ("psidecayfac", C.c_double), ("overcleanfac", C.c_double),
        ("tree_accuracy", C.c_double), ("maxp", C.c_int64),
        ("alphamax", C.c_double), ("nalpha", C.c_int32), ("ind_timesteps", C.c_int32), ("maxvxyzu", C.c_int32),
        ("curlv", C.c_int32),
    ]


class PhTune(C.Structure):
    _fields_ = [("minpart", C.c_int32), ("dens_warps", C.c_int32), ("force_warps", C.c_int32),
                ("walk_warps", C.c_int32), ("ms_before", C.c_double), ("ms_after", C.c_double),
                ("force_sym", C.c_int32)]


PH_TUNE_LEAF = 1


class PhNeighStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in (
        "nneightry", "nneighact", "maxneightry", "maxneighact", "ncalc", "np",
        "ncalls_neigh", "ncells", "maxlevel", "minlevel")] + [("rhomax", C.c_double)]


# every symbol the header declares, with its ctypes signature
_vp = C.c_void_p
_SIGS = {
    "ph_init": (C.c_int, [C.POINTER(PhParams), C.c_int64, C.POINTER(_vp)]),
    "ph_set_params": (C.c_int, [_vp, C.POINTER(PhParams)]),
    "ph_finalize": (None, [_vp]),
    "ph_strerror": (C.c_char_p, [C.c_int]),
    "ph_upload": (C.c_int, [_vp, C.c_int64, _vp, _vp, _vp]),
    "ph_download": (C.c_int, [_vp, _vp, _vp, _vp]),
    "ph_build_tree": (C.c_int, [_vp, _vp, _vp, C.POINTER(C.c_int64)]),
    "ph_density": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, C.POINTER(PhNeighStats)]),
    "ph_force": (C.c_int, [_vp, C.c_int, C.c_double, _vp, _vp, _vp, _vp, _vp,
                           C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "ph_derivs": (C.c_int, [_vp, C.c_int, C.c_double, C.POINTER(C.c_double)]),
    "ph_step": (C.c_int, [_vp, C.c_double, C.c_double, C.POINTER(C.c_double),
                          C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "ph_conservation": (C.c_int, [_vp, _vp]),
    "ph_upload_state": (C.c_int, [_vp, C.c_int64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ph_download_state": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ph_work_counters": (C.c_int, [_vp, _vp]),
    "ph_last_timings": (C.c_int, [_vp, _vp]),
    "ph_kernel_launches": (C.c_int64, [_vp]),
    "ph_adjoint": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "ph_adjoint_full": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "ph_conservation_noalloc": (C.c_int, [C.POINTER(PhParams), C.c_int64, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ph_revtree": (C.c_int, [_vp, _vp]),
    "ph_set_alpha": (C.c_int, [_vp, _vp]),
    "ph_ind_init": (C.c_int, [_vp, C.c_double]),
    "ph_ind_substep": (C.c_int, [_vp, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "ph_ind_state": (C.c_int, [_vp, _vp, _vp, _vp]),
    "ph_get_alpha": (C.c_int, [_vp, _vp, _vp]),
    "ph_alpha_initial": (C.c_int, [_vp]),
    "ph_get_nodes": (C.c_int, [_vp, C.POINTER(C.c_int64), _vp, _vp, _vp, _vp, _vp, _vp]),
    "ph_autotune": (C.c_int, [_vp, C.c_int, C.POINTER(PhTune)]),
    "ph_get_tune": (C.c_int, [_vp, C.POINTER(PhTune)]),
    "ph_set_tune": (C.c_int, [_vp, C.POINTER(PhTune)]),
    "ph_rollout_adjoint": (C.c_int, [_vp, C.c_int32, _vp, C.c_int32, _vp, C.POINTER(C.c_double), _vp, _vp]),
    "ph_rollout_adjoint_full": (C.c_int, [_vp, C.c_int32, _vp, C.c_int32, _vp, _vp, C.POINTER(C.c_double), _vp, _vp,
                                          _vp]),
}

_lib = None


def lib(path: str | None = None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(f"phantom_gb300 CUDA library not built: {p} missing "
                               "(run python -m phantom_gb300.build)")
        L = C.CDLL(p)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def make_params(cfg: dict, precision: int = PH_PREC_FP64) -> PhParams:
    p = PhParams()
    for k, _ in PhParams._fields_:
        if k == "precision":
            p.precision = precision
        elif k in cfg:
            setattr(p, k, cfg[k])
    return p


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class PhantomError(RuntimeError):
    def __init__(self, code, what):
        super().__init__(f"{what}: {lib().ph_strerror(code).decode()} (code {code})")
        self.code = code


class Context:
    """A device context holding one particle set (reference array layout)."""

    def __init__(self, cfg: dict, maxp: int | None = None, precision: int = PH_PREC_FP64):
        self.L = lib()
        self.cfg = dict(cfg)
        self.params = make_params(cfg, precision)
        self.maxp = int(maxp or cfg.get("maxp") or 0)
        if self.maxp <= 0:
            raise ValueError("maxp must be positive")
        h = _vp()
        self._chk(self.L.ph_init(C.byref(self.params), self.maxp, C.byref(h)), "ph_init")
        self.h = h
        self.n = 0

    def divcurlv_array(self) -> np.ndarray:
        """An empty divcurlv(ndivcurlv, N) in this binding's (N, ndivcurlv)
        layout: (N,) with one row, (N, 4) with curl v (params.curlv)."""
        return np.empty((self.n, 4) if self.params.curlv else self.n, np.float32)

    @property
    def vrows(self) -> int:
        """Rows of the caller's vxyzu / fxyzu arrays (maxvxyzu)."""
        return 3 if self.params.maxvxyzu == 3 else 4

    def _chk(self, rc, what):
        if rc != 0:
            raise PhantomError(rc, what)

    def close(self):
        if getattr(self, "h", None):
            self.L.ph_finalize(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, cfg: dict, precision: int | None = None):
        self.cfg.update(cfg)
        prec = self.params.precision if precision is None else precision
        self.params = make_params(self.cfg, prec)
        self._chk(self.L.ph_set_params(self.h, C.byref(self.params)), "ph_set_params")

    def upload(self, xyzh, vxyzu, Bevol=None):
        xyzh = np.ascontiguousarray(xyzh, np.float64)
        vxyzu = np.ascontiguousarray(vxyzu, np.float64)
        Bevol = None if Bevol is None else np.ascontiguousarray(Bevol, np.float64)
        self.n = int(xyzh.shape[0])
        self._chk(self.L.ph_upload(self.h, self.n, _ptr(xyzh), _ptr(vxyzu), _ptr(Bevol)), "ph_upload")

    def download(self):
        x = np.empty((self.n, 4)); v = np.empty((self.n, self.vrows)); b = np.empty((self.n, 4))
        self._chk(self.L.ph_download(self.h, _ptr(x), _ptr(v), _ptr(b)), "ph_download")
        return x, v, b

    # ---- reference call surface
    def build_tree(self):
        """maketree: returns (wrapped xyzh, inodeparts (1-based), ncells)."""
        x = np.empty((self.n, 4)); perm = np.empty(self.n, np.int32); nc = C.c_int64()
        self._chk(self.L.ph_build_tree(self.h, _ptr(x), _ptr(perm), C.byref(nc)), "ph_build_tree")
        return x, perm, nc.value

    def ind_init(self, time: float = 0.0):
        """ph_ind_init: start individual timesteps after the initial derivs."""
        self._chk(self.L.ph_ind_init(self.h, time), "ph_ind_init")

    def ind_substep(self, time: float):
        """ph_ind_substep: one pass of the evolve loop; returns (time, nactive)."""
        t = C.c_double(time)
        na = C.c_int64(0)
        self._chk(self.L.ph_ind_substep(self.h, C.byref(t), C.byref(na)), "ph_ind_substep")
        return t.value, na.value

    def ind_counters(self):
        """(nbinmax, istepfrac, ibinnow) without copying the per-particle arrays."""
        cnt = np.zeros(4, np.int32)
        self._chk(self.L.ph_ind_state(self.h, None, None, _ptr(cnt)), "ph_ind_state")
        return tuple(int(v) for v in cnt[:3])

    def ind_state(self):
        """ph_ind_state: (ibin int8, twas, (nbinmax, istepfrac, ibinnow))."""
        b = np.empty(self.n, np.int8)
        tw = np.empty(self.n)
        cnt = np.zeros(4, np.int32)
        self._chk(self.L.ph_ind_state(self.h, _ptr(b), _ptr(tw), _ptr(cnt)), "ph_ind_state")
        return b, tw, tuple(int(v) for v in cnt[:3])

    def set_alpha(self, alpha):
        """ph_set_alpha: alphaind(1,:) (float32, caller order)."""
        a = np.ascontiguousarray(alpha, np.float32)
        assert a.shape == (self.n,)
        self._chk(self.L.ph_set_alpha(self.h, _ptr(a)), "ph_set_alpha")

    def get_alpha(self):
        """ph_get_alpha: (alphaind(3,N): alpha, alphaloc, d(div v)/dt; dvdx(9,N)), float32."""
        a = np.empty((self.n, 3), np.float32)
        d = np.empty((self.n, 9), np.float32)
        self._chk(self.L.ph_get_alpha(self.h, _ptr(a), _ptr(d)), "ph_get_alpha")
        return a, d

    def alpha_initial(self):
        """ph_alpha_initial: alpha = max(alpha, alphaloc) (initial.F90:736-742)."""
        self._chk(self.L.ph_alpha_initial(self.h), "ph_alpha_initial")

    def revtree(self, xyzh):
        """ph_revtree: refit the current tree to new positions of the same particles."""
        xyzh = np.ascontiguousarray(xyzh, np.float64)
        assert xyzh.shape == (self.n, 4)
        self._chk(self.L.ph_revtree(self.h, _ptr(xyzh)), "ph_revtree")

    def nodes(self) -> dict:
        """ph_get_nodes: the current tree's nodes (library order)."""
        m = C.c_int64(0)
        self._chk(self.L.ph_get_nodes(self.h, C.byref(m), None, None, None, None, None, None), "ph_get_nodes")
        k = int(m.value)
        t = dict(inoderange=np.empty((k, 2), np.int32), xcen=np.empty((k, 3)), size=np.empty(k),
                 hmax=np.empty(k), mass=np.empty(k), isleaf=np.empty(k, np.int32))
        self._chk(self.L.ph_get_nodes(self.h, C.byref(m), *[_ptr(t[q]) for q in (
            "inoderange", "xcen", "size", "hmax", "mass", "isleaf")]), "ph_get_nodes")
        return t

    def densityiterate(self, icall: int = 1, outputs: bool = True):
        if not outputs:
            self._chk(self.L.ph_density(self.h, icall, None, None, None, None, None, None, None),
                      "ph_density")
            return None
        x = np.empty((self.n, 4)); gradh = np.empty((self.n, 2), np.float32)
        divv = self.divcurlv_array(); divB = np.empty((self.n, 4), np.float32)
        nn = np.empty(self.n, np.int32); nh = np.empty(self.n, np.uint64); st = PhNeighStats()
        self._chk(self.L.ph_density(self.h, icall, _ptr(x), _ptr(gradh), _ptr(divv), _ptr(divB),
                                    _ptr(nn), _ptr(nh), C.byref(st)), "ph_density")
        stats = {k: getattr(st, k) for k, _ in PhNeighStats._fields_}
        return dict(xyzh=x, gradh=gradh, divcurlv=divv, divcurlB=divB, nneigh=nn, neighhash=nh,
                    stats=stats)

    def force(self, icall: int = 1, dt: float = 0.0, outputs: bool = True):
        dtc = C.c_double(); dtf = C.c_double()
        if not outputs:
            self._chk(self.L.ph_force(self.h, icall, dt, None, None, None, None, None,
                                      C.byref(dtc), C.byref(dtf)), "ph_force")
            return dict(dtcourant=dtc.value, dtforce=dtf.value)
        f = np.empty((self.n, self.vrows)); db = np.empty((self.n, 4))
        divv = self.divcurlv_array(); dbs = np.empty(self.n, np.float32)
        pot = np.empty(self.n, np.float32)
        self._chk(self.L.ph_force(self.h, icall, dt, _ptr(f), _ptr(db), _ptr(divv), _ptr(dbs), _ptr(pot),
                                  C.byref(dtc), C.byref(dtf)), "ph_force")
        return dict(fxyzu=f, dBevol=db, divcurlv=divv, divBsymm=dbs, poten=pot,
                    dtcourant=dtc.value, dtforce=dtf.value)

    def derivs(self, icall: int = 1, dt: float = 0.0) -> float:
        dtnew = C.c_double()
        self._chk(self.L.ph_derivs(self.h, icall, dt, C.byref(dtnew)), "ph_derivs")
        return dtnew.value

    def step(self, t: float, dt: float):
        dtnew = C.c_double(); its = C.c_int32(); dterr = C.c_double()
        self._chk(self.L.ph_step(self.h, t, dt, C.byref(dtnew), C.byref(its), C.byref(dterr)), "ph_step")
        return dtnew.value, its.value, dterr.value

    def conservation(self):
        out = np.zeros(8)
        self._chk(self.L.ph_conservation(self.h, _ptr(out)), "ph_conservation")
        return out

    def upload_state(self, xyzh, vxyzu, Bevol, fxyzu, dBevol, divcurlv):
        """Host state -> device, ready for ``step`` (arrays must be C-contiguous)."""
        self.n = int(xyzh.shape[0])
        self._chk(self.L.ph_upload_state(self.h, self.n, _ptr(xyzh), _ptr(vxyzu), _ptr(Bevol), _ptr(fxyzu),
                                         _ptr(dBevol), _ptr(divcurlv)), "ph_upload_state")

    def download_state(self, xyzh, vxyzu, Bevol, fxyzu, dBevol, divcurlv):
        self._chk(self.L.ph_download_state(self.h, _ptr(xyzh), _ptr(vxyzu), _ptr(Bevol), _ptr(fxyzu),
                                           _ptr(dBevol), _ptr(divcurlv)), "ph_download_state")

    def adjoint(self, w_fxyzu, with_B: bool = False):
        """Gradients of sum(w_fxyzu * fxyzu) of one derivs evaluation at the
        current state: (g_xyzh, g_vxyzu[, g_Bevol]), each (N, 4); g_Bevol is
        computed for MHD contexts (always requested from the library there)."""
        w = np.ascontiguousarray(w_fxyzu, np.float64)
        gx = np.empty((self.n, 4)); gv = np.empty((self.n, self.vrows))
        gb = np.zeros((self.n, 4)) if (with_B or self.cfg.get("mhd")) else None
        self._chk(self.L.ph_adjoint(self.h, _ptr(w), _ptr(gx), _ptr(gv), _ptr(gb)), "ph_adjoint")
        return (gx, gv, gb) if with_B else (gx, gv)

    def adjoint_full(self, w_fxyzu, w_dBevol=None):
        """ph_adjoint_full: gradients of sum(w_fxyzu * fxyzu) + sum(w_dBevol *
        dBevol) of one derivs evaluation at the current state: (g_xyzh,
        g_vxyzu, g_Bevol), g_Bevol (N, 4) with MHD (B/rho and psi), else None."""
        w = np.ascontiguousarray(w_fxyzu, np.float64)
        wb = None if w_dBevol is None else np.ascontiguousarray(w_dBevol, np.float64)
        gx = np.empty((self.n, 4)); gv = np.empty((self.n, self.vrows))
        gb = np.zeros((self.n, 4)) if self.cfg.get("mhd") else None
        self._chk(self.L.ph_adjoint_full(self.h, _ptr(w), _ptr(wb), _ptr(gx), _ptr(gv), _ptr(gb)), "ph_adjoint_full")
        return gx, gv, gb

    def rollout_adjoint_full(self, dts, w_fxyzu, w_dBevol=None, ckpt: int = 4):
        """ph_rollout_adjoint_full: as rollout_adjoint, with the cotangent of the
        last evaluation's dBevol and the gradient with respect to the initial
        Bevol (MHD). Returns (L, g_xyzh, g_vxyzu, g_Bevol or None)."""
        d = np.ascontiguousarray(dts, np.float64)
        w = np.ascontiguousarray(w_fxyzu, np.float64)
        assert w.shape == (self.n, self.vrows)
        wb = None if w_dBevol is None else np.ascontiguousarray(w_dBevol, np.float64)
        gx = np.empty((self.n, 4)); gv = np.empty((self.n, self.vrows))
        gb = np.zeros((self.n, 4)) if self.cfg.get("mhd") else None
        L = C.c_double()
        self._chk(self.L.ph_rollout_adjoint_full(self.h, len(d), _ptr(d), ckpt, _ptr(w), _ptr(wb), C.byref(L),
                                                 _ptr(gx), _ptr(gv), _ptr(gb)), "ph_rollout_adjoint_full")
        return L.value, gx, gv, gb

    def rollout_adjoint(self, dts, w_fxyzu, ckpt: int = 4):
        """ph_rollout_adjoint from the state last uploaded: len(dts) leapfrog
        steps on the device, L = sum(w_fxyzu * fxyzu) of the last evaluation
        and its gradient with respect to the initial positions and velocities
        (and u). Returns (L, g_xyzh (N,4), g_vxyzu (N, vrows))."""
        d = np.ascontiguousarray(dts, np.float64)
        w = np.ascontiguousarray(w_fxyzu, np.float64)
        assert w.shape == (self.n, self.vrows)
        gx = np.empty((self.n, 4)); gv = np.empty((self.n, self.vrows))
        L = C.c_double()
        self._chk(self.L.ph_rollout_adjoint(self.h, len(d), _ptr(d), ckpt, _ptr(w), C.byref(L), _ptr(gx), _ptr(gv)),
                  "ph_rollout_adjoint")
        return L.value, gx, gv

    def autotune(self, leaf: bool = False) -> dict:
        """ph_autotune on the state last uploaded: warps per block of the density
        pair, force pair and walk kernels (results unchanged bit for bit) and,
        with leaf=True, the leaf size (results then agree to rounding). The
        context is left as after the last upload."""
        t = PhTune()
        self._chk(self.L.ph_autotune(self.h, PH_TUNE_LEAF if leaf else 0, C.byref(t)), "ph_autotune")
        return {k: getattr(t, k) for k, _ in PhTune._fields_}

    def tune(self) -> dict:
        t = PhTune()
        self._chk(self.L.ph_get_tune(self.h, C.byref(t)), "ph_get_tune")
        return {k: getattr(t, k) for k, _ in PhTune._fields_}

    def set_tune(self, **kw):
        t = PhTune()
        self._chk(self.L.ph_get_tune(self.h, C.byref(t)), "ph_get_tune")
        for k, v in kw.items():
            setattr(t, k, v)
        self._chk(self.L.ph_set_tune(self.h, C.byref(t)), "ph_set_tune")

    def timings(self):
        """ms of the last call: tree, density, force, integrate phases; force
        pair-loop kernel; density pass kernels; neighbour walks; reserved."""
        out = np.zeros(8)
        self._chk(self.L.ph_last_timings(self.h, _ptr(out)), "ph_last_timings")
        return out

    def work_counters(self):
        out = np.zeros(4, np.int64)
        self._chk(self.L.ph_work_counters(self.h, _ptr(out)), "ph_work_counters")
        return out

    def launches(self) -> int:
        return int(self.L.ph_kernel_launches(self.h))
