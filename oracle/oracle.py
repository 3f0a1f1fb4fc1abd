"""Python binding of the CPU oracle (oracle/saras_oracle.cc).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py, never by the saras_gb300 package.  The oracle
exposes the same operations as the C ABI of the product (include/saras_gb300.h)
so a parity test runs one call sequence on both and compares the arrays.
"""
import ctypes
import os
import subprocess

import numpy as np

from saras_gb300._abi import saras_params, saras_step_stats

_HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(_HERE, "saras_oracle.cc")
LIB = os.path.join(_HERE, "_build", "libsaras_oracle.so")
# Strict IEEE: no FMA contraction, no fast-math, so every expression is
# evaluated in the order the reference writes it.
# OpenMP parallelises only loops whose iterations write disjoint points (and
# exact max reductions), so results do not depend on the thread count.
CXXFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-fPIC", "-shared", "-fopenmp"]


def build(force=False):
    """Compile the oracle with g++ (seconds)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["g++"] + CXXFLAGS + ["-o", LIB + ".tmp", SRC]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        vp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
        I, D = ctypes.c_int, ctypes.c_double
        sigs = {
            "orc_create": (vp, [ctypes.POINTER(saras_params)]),
            "orc_destroy": (None, [vp]),
            "orc_field_dims": (I, [vp, I, ip]),
            "orc_get": (I, [vp, I, dp]),
            "orc_set": (I, [vp, I, dp]),
            "orc_apply_bc": (I, [vp, I]),
            "orc_sync_field": (I, [vp, I]),
            "orc_vfield_compute_diff": (I, [vp]),
            "orc_vfield_compute_nlin": (I, [vp]),
            "orc_sfield_gradient": (I, [vp, I]),
            "orc_vfield_divergence": (I, [vp]),
            "orc_tfield_compute_diff": (I, [vp]),
            "orc_tfield_compute_nlin": (I, [vp]),
            "orc_axpby": (I, [vp, I, D, I, D]),
            "orc_cn_solve": (I, [vp, I, ip, dp]),
            "orc_cn_residual": (I, [vp, I, dp]),
            "orc_mg_solve": (I, [vp, ip, dp]),
            "orc_coarse_iters": (ctypes.c_longlong, [vp]),
            "orc_time_advance": (I, [vp, ctypes.POINTER(saras_step_stats)]),
            "orc_diagnostics": (I, [vp, dp, dp, dp]),
            "orc_compute_tstp": (I, [vp, dp]),
            "orc_set_dt": (I, [vp, D]),
            "orc_mg_test_prolong": (I, [vp, dp]),
            "orc_mg_test_transfer": (I, [vp, dp]),
            "orc_mg_test_periodic": (I, [vp, dp]),
            "orc_hydro_test_periodic": (I, [vp, dp]),
            "orc_mg_level_dims": (I, [vp, I, ip]),
            "orc_mg_set_level": (I, [vp, I, I, dp]),
            "orc_mg_get_level": (I, [vp, I, I, dp]),
            "orc_mg_smooth": (I, [vp, I, I]),
            "orc_mg_restrict": (I, [vp, I]),
            "orc_mg_prolong_add": (I, [vp, I]),
            "orc_mg_compute_error": (I, [vp, I, dp]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """One CPU solver instance with the reference's np = 1 semantics."""

    def __init__(self, params):
        self.lib = _load()
        self.params = params
        self.h = self.lib.orc_create(ctypes.byref(params))

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, s, what):
        if s != 0:
            raise RuntimeError("oracle %s failed with status %d" % (what, s))
        return s

    def dims(self, field):
        d = (ctypes.c_int * 3)()
        self._chk(self.lib.orc_field_dims(self.h, field, d), "dims")
        return tuple(d)

    def get(self, field):
        a = np.empty(self.dims(field), dtype=np.float64)
        self._chk(self.lib.orc_get(self.h, field, _dp(a)), "get")
        return a

    def set(self, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == self.dims(field)
        self._chk(self.lib.orc_set(self.h, field, _dp(a)), "set")

    def apply_bc(self, field):
        self._chk(self.lib.orc_apply_bc(self.h, field), "apply_bc")

    def sync_field(self, field):
        self._chk(self.lib.orc_sync_field(self.h, field), "sync_field")

    def vfield_compute_diff(self):
        self._chk(self.lib.orc_vfield_compute_diff(self.h), "computeDiff")

    def vfield_compute_nlin(self):
        self._chk(self.lib.orc_vfield_compute_nlin(self.h), "computeNLin")

    def sfield_gradient(self, field):
        self._chk(self.lib.orc_sfield_gradient(self.h, field), "gradient")

    def vfield_divergence(self):
        self._chk(self.lib.orc_vfield_divergence(self.h), "divergence")

    def tfield_compute_diff(self):
        self._chk(self.lib.orc_tfield_compute_diff(self.h), "T.computeDiff")

    def tfield_compute_nlin(self):
        self._chk(self.lib.orc_tfield_compute_nlin(self.h), "T.computeNLin")

    def axpby(self, dst, a, src, b):
        self._chk(self.lib.orc_axpby(self.h, dst, a, src, b), "axpby")

    def cn_solve(self, comp):
        it, err = ctypes.c_int(), ctypes.c_double()
        s = self.lib.orc_cn_solve(self.h, comp, ctypes.byref(it), ctypes.byref(err))
        return s, it.value, err.value

    def cn_residual(self, comp):
        """The Crank-Nicolson residual test of the current field (no sweep)."""
        r = ctypes.c_double()
        self._chk(self.lib.orc_cn_residual(self.h, comp, ctypes.byref(r)), "cn_residual")
        return r.value

    def mg_solve(self):
        cyc, res = ctypes.c_int(), ctypes.c_double()
        self._chk(self.lib.orc_mg_solve(self.h, ctypes.byref(cyc), ctypes.byref(res)), "mgSolve")
        return cyc.value, res.value

    def coarse_iters(self):
        return self.lib.orc_coarse_iters(self.h)

    def time_advance(self):
        st = saras_step_stats()
        s = self.lib.orc_time_advance(self.h, ctypes.byref(st))
        return s, st

    def diagnostics(self):
        e, d, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        s = self.lib.orc_diagnostics(self.h, ctypes.byref(e), ctypes.byref(d), ctypes.byref(n))
        return s, e.value, d.value, n.value

    def compute_tstp(self):
        dt = ctypes.c_double()
        self._chk(self.lib.orc_compute_tstp(self.h, ctypes.byref(dt)), "computeTStp")
        return dt.value

    def set_dt(self, dt):
        self._chk(self.lib.orc_set_dt(self.h, float(dt)), "set_dt")

    def _kat(self, fn):
        e = ctypes.c_double()
        self._chk(fn(self.h, ctypes.byref(e)), "kat")
        return e.value

    def mg_test_prolong(self):
        return self._kat(self.lib.orc_mg_test_prolong)

    def mg_test_transfer(self):
        return self._kat(self.lib.orc_mg_test_transfer)

    def mg_test_periodic(self):
        return self._kat(self.lib.orc_mg_test_periodic)

    def hydro_test_periodic(self):
        return self._kat(self.lib.orc_hydro_test_periodic)

    def level_dims(self, level):
        d = (ctypes.c_int * 3)()
        self._chk(self.lib.orc_mg_level_dims(self.h, level, d), "level_dims")
        return tuple(d)

    def get_level(self, level, which):
        a = np.empty(self.level_dims(level))
        self._chk(self.lib.orc_mg_get_level(self.h, level, which, _dp(a)), "get_level")
        return a

    def set_level(self, level, which, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._chk(self.lib.orc_mg_set_level(self.h, level, which, _dp(a)), "set_level")

    def mg_smooth(self, level, count):
        self._chk(self.lib.orc_mg_smooth(self.h, level, count), "smooth")

    def mg_restrict(self, level):
        self._chk(self.lib.orc_mg_restrict(self.h, level), "restrict")

    def mg_prolong_add(self, level):
        self._chk(self.lib.orc_mg_prolong_add(self.h, level), "prolong")

    def mg_compute_error(self, norm):
        e = ctypes.c_double()
        self._chk(self.lib.orc_mg_compute_error(self.h, norm, ctypes.byref(e)), "computeError")
        return e.value
