"""ctypes wrapper of the CPU oracle (test infrastructure only).

The oracle is a C++ restatement of the reference Fortran hot path
(``phantom_oracle.cpp``); tests, the smoke check and the CPU-baseline leg of
``bench.py`` use it as the checker. The product library never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_lock = threading.Lock()


class OraParams(C.Structure):
    _fields_ = [
        ("periodic", C.c_int32), ("mhd", C.c_int32), ("gravity", C.c_int32),
        ("isothermal", C.c_int32), ("ieos", C.c_int32), ("ipdv_heating", C.c_int32),
        ("ishock_heating", C.c_int32), ("iresistive_heating", C.c_int32),
        ("divB_hj_prepass", C.c_int32), ("nthreads", C.c_int32),
        ("f64_store", C.c_int32), ("minpart", C.c_int32),
        ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double),
        ("ymax", C.c_double), ("zmin", C.c_double), ("zmax", C.c_double),
        ("hfact", C.c_double), ("tolh", C.c_double), ("massoftype", C.c_double),
        ("alpha", C.c_double), ("alphau", C.c_double), ("alphaB", C.c_double),
        ("beta", C.c_double), ("gamma", C.c_double), ("polyk", C.c_double),
        ("C_cour", C.c_double), ("C_force", C.c_double), ("tolv", C.c_double),
        ("dtmax", C.c_double), ("psidecayfac", C.c_double), ("overcleanfac", C.c_double),
        ("tree_accuracy", C.c_double), ("maxp", C.c_int64),
        ("alphamax", C.c_double), ("nalpha", C.c_int32), ("ind_timesteps", C.c_int32),
        ("curlv", C.c_int32),
    ]


class OraStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in (
        "nneightry", "nneighact", "maxneightry", "maxneighact", "ncalc", "np",
        "ncalls_neigh", "ncells", "maxlevel", "minlevel")] + [("rhomax", C.c_double)]


def build(force: bool = False) -> str:
    """Compile the oracle with the flags that mirror gfortran -O3 on x86-64
    (no FMA contraction)."""
    src = os.path.join(HERE, "phantom_oracle.cpp")
    with _lock:
        if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
            cmd = ["g++", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
                   "-shared", "-o", LIB_PATH, src]
            subprocess.check_call(cmd)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        L.ora_create.restype = vp
        L.ora_create.argtypes = [C.POINTER(OraParams)]
        L.ora_destroy.argtypes = [vp]
        L.ora_set_params.argtypes = [vp, C.POINTER(OraParams)]
        L.ora_set_particles.argtypes = [vp, C.c_int64, vp, vp, vp]
        L.ora_get_particles.argtypes = [vp, vp, vp, vp]
        L.ora_maketree.argtypes = [vp]
        L.ora_revtree.argtypes = [vp, dp]
        L.ora_set_alpha.argtypes = [vp, np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")]
        L.ora_get_alpha.argtypes = [vp, vp, vp]
        L.ora_alpha_initial.argtypes = [vp]
        L.ora_ind_init.argtypes = [vp, C.c_double]
        L.ora_ind_substep.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
        L.ora_ind_state.argtypes = [vp, vp, vp, vp]
        L.ora_get_ncells.argtypes = [vp]
        L.ora_get_ncells.restype = C.c_int64
        L.ora_get_tree.argtypes = [vp] + [vp] * 11
        L.ora_densityiterate.argtypes = [vp, C.c_int]
        L.ora_get_density.argtypes = [vp, vp, vp, vp, vp, vp, C.POINTER(OraStats)]
        L.ora_cons2prim.argtypes = [vp]
        L.ora_force.argtypes = [vp, C.c_int, C.c_double]
        L.ora_get_force.argtypes = [vp] + [vp] * 6 + [C.POINTER(C.c_double)] * 2
        L.ora_derivs.argtypes = [vp, C.c_int, C.c_double, C.POINTER(C.c_double)]
        L.ora_step.argtypes = [vp, C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_int32)]
        L.ora_get_dterr.argtypes = [vp]
        L.ora_get_dterr.restype = C.c_double
        L.ora_bruteforce_count.argtypes = [vp, C.c_int64, C.POINTER(C.c_int32)]
        L.ora_kernel.argtypes = [C.c_double, C.c_double] + [C.POINTER(C.c_double)] * 5
        L.ora_m2l.argtypes = [C.c_double] * 5 + [C.c_void_p, C.c_void_p]
        L.ora_m2l.restype = None
        L.ora_taylor.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_void_p]
        L.ora_taylor.restype = None
        del dp
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def make_params(cfg: dict, nthreads: int = 1) -> OraParams:
    p = OraParams()
    for k, _ in OraParams._fields_:
        if k == "nthreads":
            p.nthreads = nthreads
        elif k in cfg:
            setattr(p, k, cfg[k])
    return p


class Oracle:
    """One simulation state held by the C++ oracle."""

    def __init__(self, cfg: dict, nthreads: int = 1):
        self.L = lib()
        self.cfg = dict(cfg)
        self.params = make_params(cfg, nthreads)
        self.h = self.L.ora_create(C.byref(self.params))
        if not self.h:
            raise ValueError("oracle: invalid parameters (minpart must be 0 or 2..16)")
        self.n = 0

    def close(self):
        if self.h:
            self.L.ora_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"oracle {what} failed with status {rc}")

    def set_particles(self, xyzh, vxyzu, Bevol=None):
        xyzh = np.ascontiguousarray(xyzh, np.float64)
        vxyzu = np.ascontiguousarray(vxyzu, np.float64)
        Bevol = None if Bevol is None else np.ascontiguousarray(Bevol, np.float64)
        self.n = xyzh.shape[0]
        self._chk(self.L.ora_set_particles(self.h, self.n, _ptr(xyzh), _ptr(vxyzu), _ptr(Bevol)), "set_particles")

    def get_particles(self):
        x = np.empty((self.n, 4)); v = np.empty((self.n, 4)); b = np.empty((self.n, 4))
        self.L.ora_get_particles(self.h, _ptr(x), _ptr(v), _ptr(b))
        return x, v, b

    def maketree(self):
        self._chk(self.L.ora_maketree(self.h), "maketree")

    def set_alpha(self, alpha):
        """alphaind(1,:) (float32, caller order)."""
        self._chk(self.L.ora_set_alpha(self.h, np.ascontiguousarray(alpha, np.float32)), "set_alpha")

    def get_alpha(self):
        """(alphaind(3,N): alpha, alphaloc, d(div v)/dt; dvdx(9,N)), float32."""
        a = np.empty((self.n, 3), np.float32)
        d = np.empty((self.n, 9), np.float32)
        self._chk(self.L.ora_get_alpha(self.h, _ptr(a), _ptr(d)), "get_alpha")
        return a, d

    def alpha_initial(self):
        """initial.F90:736-742: alpha = max(alpha, alphaloc) after the initial derivs."""
        self._chk(self.L.ora_alpha_initial(self.h), "alpha_initial")

    def ind_init(self, time=0.0):
        """Individual timesteps: bins and twas after the initial derivs (init_step)."""
        self._chk(self.L.ora_ind_init(self.h, time), "ind_init")

    def ind_substep(self, time):
        """One pass of the evolve loop with individual timesteps; returns (time, nactive)."""
        t = C.c_double(time)
        na = C.c_int64(0)
        self._chk(self.L.ora_ind_substep(self.h, C.byref(t), C.byref(na)), "ind_substep")
        return t.value, na.value

    def ind_state(self):
        """(ibin int8, twas, (nbinmax, istepfrac, ibinnow))."""
        b = np.empty(self.n, np.int8)
        tw = np.empty(self.n)
        cnt = np.zeros(4, np.int32)
        self._chk(self.L.ora_ind_state(self.h, _ptr(b), _ptr(tw), _ptr(cnt)), "ind_state")
        return b, tw, tuple(int(v) for v in cnt[:3])

    def revtree(self, xyzh):
        """revtree (kdtree.F90:1851-2037): the tree built last, refitted to new
        positions of the same particles (caller order)."""
        xyzh = np.ascontiguousarray(xyzh, np.float64)
        assert xyzh.shape == (self.n, 4)
        self._chk(self.L.ora_revtree(self.h, xyzh), "revtree")

    def get_tree(self):
        nc = int(self.L.ora_get_ncells(self.h))
        t = dict(
            inodeparts=np.empty(self.n, np.int32), inoderange=np.empty((nc, 2), np.int32),
            xcen=np.empty((nc, 3)), size=np.empty(nc), hmax=np.empty(nc), mass=np.empty(nc),
            left=np.empty(nc, np.int32), right=np.empty(nc, np.int32), parent=np.empty(nc, np.int32),
            leaf_is_active=np.empty(nc, np.int32), quads=np.empty((nc, 6)))
        self.L.ora_get_tree(self.h, *[_ptr(t[k]) for k in (
            "inodeparts", "inoderange", "xcen", "size", "hmax", "mass", "left", "right", "parent",
            "leaf_is_active", "quads")])
        t["ncells"] = nc
        return t

    def densityiterate(self, icall=1):
        self._chk(self.L.ora_densityiterate(self.h, icall), "densityiterate")

    def get_density(self):
        gradh = np.empty((self.n, 2), np.float32)
        divv = self._divcurlv()
        divB = np.empty((self.n, 4), np.float32)
        nn = np.empty(self.n, np.int32)
        nh = np.empty(self.n, np.uint64)
        st = OraStats()
        self.L.ora_get_density(self.h, _ptr(gradh), _ptr(divv), _ptr(divB), _ptr(nn), _ptr(nh), C.byref(st))
        stats = {k: getattr(st, k) for k, _ in OraStats._fields_}
        return dict(gradh=gradh, divcurlv=divv, divcurlB=divB, nneigh=nn, neighhash=nh, stats=stats)

    def _divcurlv(self):
        # divcurlv(ndivcurlv, n): (n,) with one row, (n, 4) with curl v
        return np.empty((self.n, 4) if self.params.curlv else self.n, np.float32)

    def cons2prim(self):
        self._chk(self.L.ora_cons2prim(self.h), "cons2prim")

    def force(self, icall=1, dt=0.0):
        self._chk(self.L.ora_force(self.h, icall, dt), "force")

    def get_force(self):
        f = np.empty((self.n, 4)); db = np.empty((self.n, 4))
        divv = self._divcurlv(); dbs = np.empty(self.n, np.float32)
        pot = np.empty(self.n, np.float32); eos = np.empty((self.n, 2))
        dtc = C.c_double(); dtf = C.c_double()
        self.L.ora_get_force(self.h, _ptr(f), _ptr(db), _ptr(divv), _ptr(dbs), _ptr(pot), _ptr(eos),
                             C.byref(dtc), C.byref(dtf))
        return dict(fxyzu=f, dBevol=db, divcurlv=divv, divBsymm=dbs, poten=pot, eos=eos,
                    dtcourant=dtc.value, dtforce=dtf.value)

    def derivs(self, icall=1, dt=0.0):
        dtnew = C.c_double()
        self._chk(self.L.ora_derivs(self.h, icall, dt, C.byref(dtnew)), "derivs")
        return dtnew.value

    def step(self, t, dt):
        dtnew = C.c_double(); its = C.c_int32()
        self._chk(self.L.ora_step(self.h, t, dt, C.byref(dtnew), C.byref(its)), "step")
        return dtnew.value, its.value, float(self.L.ora_get_dterr(self.h))

    def bruteforce_count(self, i):
        c = C.c_int32()
        self._chk(self.L.ora_bruteforce_count(self.h, i, C.byref(c)), "bruteforce")
        return c.value


def m2l(dx, dr1, mass, quads, fnode=None):
    """compute_M2L: returns fnode(20) with the node's expansion added."""
    f = np.zeros(20) if fnode is None else np.ascontiguousarray(fnode, np.float64).copy()
    q = np.ascontiguousarray(quads, np.float64)
    lib().ora_m2l(float(dx[0]), float(dx[1]), float(dx[2]), float(dr1), float(mass),
                  q.ctypes.data_as(C.c_void_p), f.ctypes.data_as(C.c_void_p))
    return f


def taylor(fnode, dx):
    """expand_fgrav_in_taylor_series: (force(3), potential) at offset dx."""
    fn = np.ascontiguousarray(fnode, np.float64)
    f3 = np.zeros(3)
    phi = C.c_double()
    lib().ora_taylor(fn.ctypes.data_as(C.c_void_p), float(dx[0]), float(dx[1]), float(dx[2]),
                     f3.ctypes.data_as(C.c_void_p), C.byref(phi))
    return f3, phi.value


def kernel(q):
    out = [C.c_double() for _ in range(5)]
    lib().ora_kernel(q * q, q, *[C.byref(o) for o in out])
    return [o.value for o in out]
