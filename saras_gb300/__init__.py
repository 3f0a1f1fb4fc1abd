"""saras_gb300 -- GB300-native SARAS time-step hot path.

Host-side mirror of the reference's solver interfaces over the C ABI of
``include/saras_gb300.h``:

* :func:`parser` reads ``input/parameters.yaml`` (lib/io/parser.cc).
* :class:`Solver` owns one device context: the fields of ``hydro`` /
  ``scalar`` (V, P, T, Pp, mgRHS, nseRHS, ...), the multigrid hierarchy of
  ``multigrid_d3`` and every operator of lib/field and lib/boundary.
* :class:`hydro_d3` / :class:`scalar_d3` reproduce the constructors and
  ``solvePDE`` loops of src/solvers/hydro/hydro_d3.cc and
  src/solvers/scalar/scalar_d3.cc on top of :class:`Solver`.

All compute runs in the CUDA library; when it is missing or no GPU is visible
every call raises -- there is no CPU fallback.
"""
import ctypes
import math

import numpy as np

from . import _abi
from ._abi import (saras_params, saras_step_stats, default_params, FIELD_VX, FIELD_VY, FIELD_VZ, FIELD_P,
                   FIELD_T, FIELD_PP, FIELD_MGRHS, FIELD_NSE_X, FIELD_NSE_Y, FIELD_NSE_Z, FIELD_TRHS,
                   FIELD_GRAD_X, FIELD_GRAD_Y, FIELD_GRAD_Z, MG_REFERENCE, MG_PLAIN_TARGET, MG_MIXED,
                   GUESS_PREVIOUS, GUESS_LEARNED)

__all__ = ["SarasError", "Solver", "parser", "hydro_d3", "scalar_d3", "default_params", "build"]


class SarasError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (_abi.STATUS_NAMES.get(status, status), msg))
        self.status = status


def build(verbose=False):
    from .build import build as _b
    return _b(verbose=verbose)


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def parse_probes(path):
    """parser::parseProbes / testProbes (parser.cc:424-575): the probe points of a
    parameters file as an (n, 3) array of (i, j, k)."""
    lib = _abi.load()
    err = ctypes.create_string_buffer(512)
    n = ctypes.c_int()
    IP = ctypes.POINTER(ctypes.c_int)
    s = lib.saras_parse_probes(str(path).encode(), None, 0, ctypes.byref(n), err, 512)
    if s != 0:
        raise SarasError(s, err.value.decode())
    out = np.zeros((n.value, 3), dtype=np.int32)
    if n.value:
        s = lib.saras_parse_probes(str(path).encode(), out.ctypes.data_as(IP), n.value, ctypes.byref(n), err, 512)
        if s != 0:
            raise SarasError(s, err.value.decode())
    return out


def parser(path):
    """parser::parser (lib/io/parser.cc:47-59): read and check parameters.yaml."""
    lib = _abi.load()
    p = saras_params()
    err = ctypes.create_string_buffer(512)
    s = lib.saras_parse_yaml(path.encode(), ctypes.byref(p), err, 512)
    if s != 0:
        raise SarasError(s, err.value.decode())
    return p


class Solver:
    """One GB300 solver context (grid + fields + multigrid hierarchy)."""

    def __init__(self, params):
        self.lib = _abi.load()
        self.params = params
        h = ctypes.c_void_p()
        s = self.lib.saras_create(ctypes.byref(params), ctypes.byref(h))
        if s != 0:
            raise SarasError(s, self.lib.saras_last_error(None).decode())
        self.h = h

    # -- lifetime
    def close(self):
        if getattr(self, "h", None):
            self.lib.saras_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, s):
        if s != 0:
            raise SarasError(s, self.lib.saras_last_error(self.h).decode())
        return s

    # -- data movement
    def dims(self, field):
        d = (ctypes.c_int * 3)()
        self._chk(self.lib.saras_field_dims(self.h, field, d))
        return tuple(d)

    def grid_coords(self, axis, staggered):
        """The library's coordinates along `axis` (ghosts included, index -1 first)."""
        n = ctypes.c_int()
        self._chk(self.lib.saras_grid_coords(self.h, axis, 1 if staggered else 0, None, 0, ctypes.byref(n)))
        a = np.empty(n.value)
        self._chk(self.lib.saras_grid_coords(self.h, axis, 1 if staggered else 0, _dp(a), n.value, ctypes.byref(n)))
        return a

    def get(self, field):
        a = np.empty(self.dims(field), dtype=np.float64)
        self._chk(self.lib.saras_download(self.h, field, _dp(a)))
        return a

    def set(self, field, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        if a.shape != self.dims(field):
            raise ValueError("shape %s != %s" % (a.shape, self.dims(field)))
        self._chk(self.lib.saras_upload(self.h, field, _dp(a)))

    def synchronize(self):
        self._chk(self.lib.saras_synchronize(self.h))

    def launch_count(self):
        return self.lib.saras_launch_count(self.h)

    def plane_tma_active(self):
        """Whether the finest-level FP32 stencils run through the TMA kernels."""
        return bool(self.lib.saras_plane_tma_active(self.h))

    # -- boundary and field operators
    def apply_bc(self, field):
        self._chk(self.lib.saras_apply_bc(self.h, field))

    def sync_field(self, field):
        self._chk(self.lib.saras_sync_field(self.h, field))

    def vfield_compute_diff(self):
        self._chk(self.lib.saras_vfield_compute_diff(self.h))

    def vfield_compute_nlin(self):
        self._chk(self.lib.saras_vfield_compute_nlin(self.h))

    def sfield_gradient(self, field):
        self._chk(self.lib.saras_sfield_gradient(self.h, field))

    def vfield_divergence(self):
        self._chk(self.lib.saras_vfield_divergence(self.h))

    def tfield_compute_diff(self):
        self._chk(self.lib.saras_tfield_compute_diff(self.h))

    def tfield_compute_nlin(self):
        self._chk(self.lib.saras_tfield_compute_nlin(self.h))

    def axpby(self, dst, a, src, b):
        self._chk(self.lib.saras_axpby(self.h, dst, a, src, b))

    # -- solves
    def cn_solve(self, comp):
        it, err = ctypes.c_int(), ctypes.c_double()
        s = self.lib.saras_cn_solve(self.h, comp, ctypes.byref(it), ctypes.byref(err))
        if s not in (0, _abi.NOT_CONVERGED):
            self._chk(s)
        return s, it.value, err.value

    def mg_solve(self):
        cyc, res = ctypes.c_int(), ctypes.c_double()
        self._chk(self.lib.saras_mg_solve(self.h, ctypes.byref(cyc), ctypes.byref(res)))
        return cyc.value, res.value

    def mg_set_mode(self, mode, target=1e-8, max_cycles=200):
        self._chk(self.lib.saras_mg_set_mode(self.h, mode, target, max_cycles))

    def time_advance(self):
        st = saras_step_stats()
        s = self.lib.saras_time_advance(self.h, ctypes.byref(st))
        if s not in (0, _abi.NOT_CONVERGED):
            self._chk(s)
        return s, st

    def diagnostics(self):
        e, d, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        s = self.lib.saras_diagnostics(self.h, ctypes.byref(e), ctypes.byref(d), ctypes.byref(n))
        if s not in (0, _abi.DIVERGENCE_LIMIT):
            self._chk(s)
        return s, e.value, d.value, n.value

    # -- time step, probes, restart
    def compute_tstp(self):
        """vfield::computeTStp (vfield.cc:267-284)."""
        dt = ctypes.c_double()
        self._chk(self.lib.saras_compute_tstp(self.h, ctypes.byref(dt)))
        return dt.value

    def set_dt(self, dt):
        self._chk(self.lib.saras_set_dt(self.h, float(dt)))

    def probe(self, ijk, fields=(FIELD_VX, FIELD_VY, FIELD_VZ, FIELD_P)):
        """probes::getData (probes.cc:174-189): values of `fields` at the (i, j, k) triplets."""
        a = np.ascontiguousarray(np.asarray(ijk, dtype=np.int32).reshape(-1, 3))
        f = np.ascontiguousarray(np.asarray(fields, dtype=np.int32))
        out = np.empty((a.shape[0], f.size), dtype=np.float64)
        IP = ctypes.POINTER(ctypes.c_int)
        self._chk(self.lib.saras_probe(self.h, a.shape[0], a.ctypes.data_as(IP), f.size, f.ctypes.data_as(IP), _dp(out)))
        return out

    def write_restart(self, path, time):
        self._chk(self.lib.saras_write_restart(self.h, str(path).encode(), float(time)))

    def read_restart(self, path):
        t = ctypes.c_double()
        self._chk(self.lib.saras_read_restart(self.h, str(path).encode(), ctypes.byref(t)))
        return t.value

    # -- multigrid test hooks
    def _kat(self, fn):
        e = ctypes.c_double()
        self._chk(fn(self.h, ctypes.byref(e)))
        return e.value

    def mg_test_prolong(self):
        return self._kat(self.lib.saras_mg_test_prolong)

    def mg_test_transfer(self):
        return self._kat(self.lib.saras_mg_test_transfer)

    def mg_test_periodic(self):
        return self._kat(self.lib.saras_mg_test_periodic)

    def hydro_test_periodic(self):
        return self._kat(self.lib.saras_hydro_test_periodic)

    def level_dims(self, level):
        d = (ctypes.c_int * 3)()
        self._chk(self.lib.saras_mg_level_dims(self.h, level, d))
        return tuple(d)

    def get_level(self, level, which):
        a = np.empty(self.level_dims(level))
        self._chk(self.lib.saras_mg_get_level(self.h, level, which, _dp(a)))
        return a

    def set_level(self, level, which, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._chk(self.lib.saras_mg_set_level(self.h, level, which, _dp(a)))

    def mg_smooth(self, level, count):
        self._chk(self.lib.saras_mg_smooth(self.h, level, count))

    def mg_restrict(self, level):
        self._chk(self.lib.saras_mg_restrict(self.h, level))

    def mg_prolong_add(self, level):
        self._chk(self.lib.saras_mg_prolong_add(self.h, level))

    def mg_compute_error(self, norm):
        e = ctypes.c_double()
        self._chk(self.lib.saras_mg_compute_error(self.h, norm, ctypes.byref(e)))
        return e.value

    # -- learned warm start
    def unet_collect(self):
        self._chk(self.lib.saras_unet_collect(self.h))

    def unet_train(self, iters, lr):
        loss = ctypes.c_double()
        self._chk(self.lib.saras_unet_train(self.h, iters, lr, ctypes.byref(loss)))
        return loss.value

    def unet_infer(self):
        self._chk(self.lib.saras_unet_infer(self.h, FIELD_PP))

    def unet_shape(self):
        """(parameter count, (D, H, W) of the network's finest grid)."""
        n = ctypes.c_longlong()
        d = (ctypes.c_int * 3)()
        self._chk(self.lib.saras_unet_shape(self.h, ctypes.byref(n), d))
        return n.value, tuple(d)

    def unet_grad_check(self, feat, target, params=None):
        """One forward/backward pass of the U-Net (saras_unet_grad_check): returns
        (output d, loss, gradient with respect to the parameters)."""
        nparam, dims = self.unet_shape()
        nv = dims[0] * dims[1] * dims[2]
        f = np.ascontiguousarray(feat, dtype=np.float32).reshape(nv, 3)
        t = np.ascontiguousarray(target, dtype=np.float32).reshape(nv)
        pp = None if params is None else np.ascontiguousarray(params, dtype=np.float32).reshape(nparam)
        out = np.empty(nv, dtype=np.float32)
        grad = np.empty(nparam, dtype=np.float32)
        loss = ctypes.c_double()
        self._chk(self.lib.saras_unet_grad_check(self.h, f.ctypes.data, t.ctypes.data, None if pp is None else pp.ctypes.data,
                                                 out.ctypes.data, ctypes.byref(loss), grad.ctypes.data))
        return out.reshape(dims), loss.value, grad

    def set_guess_mode(self, mode):
        self._chk(self.lib.saras_set_guess_mode(self.h, mode))

    # -- measurement
    def profile_enable(self, kernel_id, enable=True):
        self._chk(self.lib.saras_profile_enable(self.h, kernel_id, 1 if enable else 0))

    def profile_sample(self, every):
        """Time the kernels of one replayed V-cycle in `every` (saras_profile_sample)."""
        self._chk(self.lib.saras_profile_sample(self.h, int(every)))

    def profile_read(self, kernel_id):
        n, ms, b = ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double()
        self._chk(self.lib.saras_profile_read(self.h, kernel_id, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(b)))
        return n.value, ms.value, b.value

    def event_record(self, slot):
        self._chk(self.lib.saras_event_record(self.h, slot))

    def event_elapsed(self, a, b):
        ms = ctypes.c_double()
        self._chk(self.lib.saras_event_elapsed(self.h, a, b, ctypes.byref(ms)))
        return ms.value

    def upload_ptr(self, field, ptr):
        """Upload from a raw host pointer (e.g. pinned memory)."""
        self._chk(self.lib.saras_upload(self.h, field, ctypes.cast(ptr, ctypes.POINTER(ctypes.c_double))))

    def download_ptr(self, field, ptr):
        self._chk(self.lib.saras_download(self.h, field, ctypes.cast(ptr, ctypes.POINTER(ctypes.c_double))))

    def _fields_ptrs(self, fields, ptrs):
        n = len(fields)
        f = (ctypes.c_int * n)(*fields)
        P = ctypes.POINTER(ctypes.c_double)
        p = (P * n)(*[ctypes.cast(x, P) for x in ptrs])
        return n, f, p

    def upload_fields_ptr(self, fields, ptrs):
        """Upload several fields at once from raw host pointers (concurrent copies)."""
        self._chk(self.lib.saras_upload_fields(self.h, *self._fields_ptrs(fields, ptrs)))

    def download_fields_ptr(self, fields, ptrs):
        """Download several fields at once into raw host pointers (concurrent copies)."""
        self._chk(self.lib.saras_download_fields(self.h, *self._fields_ptrs(fields, ptrs)))

    @staticmethod
    def profile_names():
        lib = _abi.load()
        return [lib.saras_profile_name(i).decode() for i in range(lib.saras_profile_count())]


def to_bf16_bits(a):
    """Round an FP32 array to BF16 (round to nearest even) and return the raw bits."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def from_bf16_bits(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


def conv3d_check(mode, x_bits, dy_bits, w, bias, relu, dims, cin, cout):
    """Run the tensor-core 3x3x3 convolution stand-alone (saras_conv3d_check).
    x_bits / dy_bits: channels-last BF16 bit arrays; w: FP32 [cout][27][cin]."""
    lib = _abi.load()
    D, H, W = dims
    nv = D * H * W
    if mode == 0:
        out = np.empty(nv * cout, dtype=np.float32)
    elif mode == 1:
        out = np.empty(nv * cin, dtype=np.float32)
    else:
        out = np.empty(27 * cin * cout + cout, dtype=np.float32)
    wd = np.ascontiguousarray(w, dtype=np.float64).astype(np.float32)
    bd = None if bias is None else np.ascontiguousarray(bias, dtype=np.float32)
    xp = None if x_bits is None else np.ascontiguousarray(x_bits, dtype=np.uint16)
    dp = None if dy_bits is None else np.ascontiguousarray(dy_bits, dtype=np.uint16)
    fp = ctypes.POINTER(ctypes.c_float)
    s = lib.saras_conv3d_check(mode, D, H, W, cin, cout,
                               None if xp is None else xp.ctypes.data, None if dp is None else dp.ctypes.data,
                               wd.ctypes.data, None if bd is None else bd.ctypes.data,
                               relu, out.ctypes.data_as(fp))
    if s != 0:
        raise SarasError(s, lib.saras_last_error(None).decode())
    return out


# ---------------------------------------------------------------- initial conditions
def grid_coords(params):
    """Vertex ("staggered") and cell ("collocated") coordinates including the
    pads, grid.cc:370-403: xStaggr(i) = L*i*dXi, xColloc(i) = L*(xi(i)+xi(i+1))/2;
    on an axis with mesh type 'D' the core points follow the double-sided
    tangent-hyperbolic map of grid.cc:442-519 (numpy's tanh: these arrays build
    initial conditions; the solver's own coordinates are Solver.grid_coords)."""
    out = []
    for axis, (ind, L, gt, beta) in enumerate(((params.xInd, params.Lx, params.xGrid, params.betaX),
                                                (params.yInd, params.Ly, params.yGrid, params.betaY),
                                                (params.zInd, params.Lz, params.zGrid, params.betaZ))):
        n = 2 ** ind
        d = 1.0 / n
        xi = np.arange(-1, n + 2, dtype=np.float64) * d
        xs = L * xi
        xc = L * (xi[:-1] + xi[1:]) / 2.0
        if ind == 0 and axis == 1:
            # the 2D solver's single y point: coordinates keep their default 1
            # (grid.cc:300-320, createUniformGrid skips y under PLANAR)
            out.append((np.ones(3), np.ones(3)))
            continue
        if gt == 2:
            t = np.tanh(beta)
            xs[1:n + 2] = L * (1.0 - np.tanh(beta * (1.0 - 2.0 * xi[1:n + 2])) / t) / 2.0
            xc[1:n + 1] = L * (1.0 - np.tanh(beta * (1.0 - (xi[1:n + 1] + xi[2:n + 2]))) / t) / 2.0
        out.append((xs, xc))
    return out


_TRIG_CACHE = {}


def _sin_pi(q, m):
    """sin(pi q / m) for integer arrays q, correctly rounded to FP64.

    Evaluated in 50-digit decimal arithmetic (Machin's formula for pi, the
    Taylor series of sin on the reduced argument), so the initial fields are
    the same bits on every host: a library sin/cos may differ by an ulp
    between machines, and a one-ulp difference in an initial field can move a
    tolerance-stopped iteration count by one step in a long parity run."""
    import decimal
    key = int(m)
    if key not in _TRIG_CACHE:
        ctx = decimal.Context(prec=50)
        D = ctx.create_decimal

        def arctan_inv(x):     # arctan(1/x) for an integer x
            x = D(x)
            x2 = ctx.multiply(x, x)
            term = ctx.divide(D(1), x)
            total, n, sign = term, 1, 1
            while True:
                term = ctx.divide(term, x2)
                n += 2
                sign = -sign
                t = ctx.divide(term, D(n))
                if t.adjusted() < -60:
                    break
                total = ctx.add(total, t) if sign > 0 else ctx.subtract(total, t)
            return total
        pi = ctx.multiply(D(4), ctx.subtract(ctx.multiply(D(4), arctan_inv(5)), arctan_inv(239)))
        table = np.empty(2 * key, dtype=np.float64)
        for r in range(2 * key):
            rr = r if r <= key else r - 2 * key          # argument in [-pi, pi]
            if rr % key == 0:                            # sin(0) = sin(pi) = 0 exactly
                table[r] = 0.0
                continue
            x = ctx.divide(ctx.multiply(pi, D(rr)), D(key))
            x2 = ctx.multiply(x, x)
            term, total, n = x, x, 1
            while True:
                term = ctx.divide(ctx.multiply(term, x2), D((n + 1) * (n + 2)))
                n += 2
                if term.is_zero() or term.adjusted() < -60:
                    break
                total = ctx.subtract(total, term) if (n // 2) % 2 == 1 else ctx.add(total, term)
            table[r] = float(total)
        _TRIG_CACHE[key] = table
    t = _TRIG_CACHE[key]
    return t[np.mod(np.asarray(q, dtype=np.int64), 2 * key)]


def _cos_pi(q, m):
    """cos(pi q / m) = sin(pi (q + m/2) / m), correctly rounded (q, m integers)."""
    return _sin_pi(2 * np.asarray(q, dtype=np.int64) + m, 2 * m)


def taylor_green_velocity(params):
    """taylorGreen::initializeField (lib/initial/taylorGreen.cc:54-100) over the padded arrays:
    u = sin(2 pi x / L) cos(2 pi y / L) cos(2 pi z / L), v = -cos sin cos.  Vertex
    coordinates are x_i = L i / n and face coordinates L (i + 1/2) / n (i from -1),
    so every factor is sin or cos of pi q / n for an integer q (correctly rounded).
    On a stretched mesh the factors are numpy's sin and cos of the coordinates
    of grid_coords."""
    if params.xGrid == 2 or params.yGrid == 2 or params.zGrid == 2:
        (xs, xc), (ys, yc), (zs, zc) = grid_coords(params)
        w = [2.0 * np.pi / params.Lx, 2.0 * np.pi / params.Ly, 2.0 * np.pi / params.Lz]
        Vx = np.sin(w[0] * xc)[:, None, None] * np.cos(w[1] * ys)[None, :, None] * np.cos(w[2] * zs)[None, None, :]
        Vy = -np.cos(w[0] * xs)[:, None, None] * np.sin(w[1] * yc)[None, :, None] * np.cos(w[2] * zs)[None, None, :]
        return Vx, Vy
    n = [2 ** params.xInd, 2 ** params.yInd, 2 ** params.zInd]
    vs = [2 * np.arange(-1, m + 2, dtype=np.int64) for m in n]        # 2 pi x_i / L = pi (2 i) / n
    fc = [2 * np.arange(-1, m + 1, dtype=np.int64) + 1 for m in n]    # 2 pi x_(i+1/2) / L = pi (2 i + 1) / n
    Vx = (_sin_pi(fc[0], n[0])[:, None, None] * _cos_pi(vs[1], n[1])[None, :, None] *
          _cos_pi(vs[2], n[2])[None, None, :])
    Vy = (-_cos_pi(vs[0], n[0])[:, None, None] * _sin_pi(fc[1], n[1])[None, :, None] *
          _cos_pi(vs[2], n[2])[None, None, :])
    return Vx, Vy


def taylor_green_velocity_2d(params):
    """taylorGreen::initializeField in 2D (taylorGreen.cc:57-79): on the y = 0
    plane u = sin(2 pi x / Lx) cos(2 pi z / Lz), w = -cos(2 pi x / Lx) sin(2 pi z / Lz),
    correctly rounded as in 3D; the y ghost planes stay 0.  Returns (Vx, Vz)."""
    n = [2 ** params.xInd, 2 ** params.zInd]
    vs = [2 * np.arange(-1, m + 2, dtype=np.int64) for m in n]
    fc = [2 * np.arange(-1, m + 1, dtype=np.int64) + 1 for m in n]
    Vx = np.zeros((n[0] + 2, 3, n[1] + 3))
    Vz = np.zeros((n[0] + 3, 3, n[1] + 2))
    Vx[:, 1, :] = _sin_pi(fc[0], n[0])[:, None] * _cos_pi(vs[1], n[1])[None, :]
    Vz[:, 1, :] = -_cos_pi(vs[0], n[0])[:, None] * _sin_pi(fc[1], n[1])[None, :]
    return Vx, Vz


def taylor_green_pressure(params):
    """p = (cos 2x + cos 2y)(cos 2z + 2)/16 on the vertex grid (x scaled by 2 pi / L),
    with correctly rounded cosines of pi (4 i) / n."""
    n = [2 ** params.xInd, 2 ** params.yInd, 2 ** params.zInd]
    c = [_cos_pi(4 * np.arange(-1, m + 2, dtype=np.int64), m) for m in n]
    return ((c[0][:, None, None] + c[1][None, :, None]) * (c[2][None, None, :] + 2.0) / 16.0)


def splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


def rbc_temperature(params, seed=42, amplitude=1.0e-3):
    """Linear conduction profile T = 1 - z/Lz plus a counter-based uniform
    perturbation in [-amplitude, amplitude] (SplitMix64 of seed ^ global index)."""
    (xs, _), (ys, _), (zs, _) = grid_coords(params)
    nx, ny, nz = len(xs), len(ys), len(zs)
    idx = np.arange(nx * ny * nz, dtype=np.uint64).reshape(nx, ny, nz)
    with np.errstate(over="ignore"):
        x = (idx ^ np.uint64(seed)) + np.uint64(0x9E3779B97F4A7C15)
        z = x
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    T = (1.0 - zs / params.Lz)[None, None, :] + amplitude * (2.0 * u - 1.0)
    return np.ascontiguousarray(np.broadcast_to(T, (nx, ny, nz)))


class hydro_d3:
    """hydro_d3 (src/solvers/hydro/hydro_d3.cc:63-119): with "Restart Run"
    (params.restartFlag) the fields and the time from the restart file;
    otherwise P = 1 (or a given pressure) and the initial condition of icType;
    then the velocity BCs."""

    restart_path = "output/restartFile.saras"

    def __init__(self, params, pressure=None, velocity=None, restart=None):
        self.params = params
        self.solver = Solver(params)
        s = self.solver
        self.time = 0.0
        if params.restartFlag:
            self.time = s.read_restart(restart or self.restart_path)
        else:
            P = np.ones(s.dims(FIELD_P)) if pressure is None else pressure
            s.set(FIELD_P, P)
            if velocity is not None:
                for f, a in zip((FIELD_VX, FIELD_VY, FIELD_VZ), velocity):
                    if a is not None:
                        s.set(f, a)
            elif params.icType == 1:
                Vx, Vy = taylor_green_velocity(params)
                s.set(FIELD_VX, Vx)
                s.set(FIELD_VY, Vy)
        for f in self._bc_fields():
            s.apply_bc(f)
        self.timeStepCount = 0

    def _bc_fields(self):
        return (FIELD_VX, FIELD_VY, FIELD_VZ)

    def _probe_fields(self):
        return (FIELD_VX, FIELD_VY, FIELD_VZ, FIELD_P)

    def timeAdvance(self):
        st, stats = self.solver.time_advance()
        if st != 0:
            raise SarasError(st, "Jacobi iterations not converging")
        return stats

    def _write_probes(self, f, probes, time):
        """probes::probeData (probes.cc:120-166): one line a probe."""
        vals = self.solver.probe(probes, self._probe_fields())
        for (i, j, k), row in zip(probes, vals):
            f.write("%6.4f\t%4d\t%4d\t%4d\t" % (time, i, j, k) + "\t".join("%16.8f" % v for v in row) + "\n")

    def solvePDE(self, on_step=None, probes=None, output=None):
        """hydro_d3::solvePDE (hydro_d3.cc:122-251): the time loop with the CFL
        time step ("Use CFL Condition": computeTStp after each step, capped at
        "Time-Step"), the time series every "I/O Count" steps, probes every
        "Probe Time Interval" (ProbesData.dat) and restart files every
        "Restart Write Interval" (restartFile.saras) in the directory `output`
        when it is given.  Solution files are not written.  Returns the time
        series [(time, energy, max divergence, Nusselt)]."""
        import os
        p = self.params
        dt = p.tStp
        self.solver.set_dt(dt)
        series = []
        pfile = None
        if output is not None:
            os.makedirs(output, exist_ok=True)
        if probes is not None and len(probes) and p.readProbes and output is not None:
            pfile = open(os.path.join(output, "ProbesData.dat"), "a")
            if not p.restartFlag:
                names = ["Vx", "Vy", "Vz", "P", "T"][:len(self._probe_fields())]
                pfile.write("#VARIABLES = Time, X, Y, Z, " + ", ".join(names) + "\n")
                self._write_probes(pfile, probes, self.time)
        s0, e0, d0, n0 = self.solver.diagnostics()
        series.append((self.time, e0, d0, n0))
        prTime = self.time + p.prInt - math.fmod(self.time, p.prInt)
        rsTime = self.time + p.rsInt - math.fmod(self.time, p.rsInt)
        try:
            while True:
                stats = self.timeAdvance()
                if p.useCFL:
                    dt = self.solver.compute_tstp()
                    if dt > p.tStp:
                        dt = p.tStp
                    self.solver.set_dt(dt)
                self.timeStepCount += 1
                self.time += dt
                if self.timeStepCount % max(1, p.ioCnt) == 0:
                    s, e, d, n = self.solver.diagnostics()
                    series.append((self.time, e, d, n))
                    if s != 0:
                        raise SarasError(s, "Maximum divergence exceeds limit")
                if pfile is not None and abs(prTime - self.time) < 0.5 * dt:
                    self._write_probes(pfile, probes, self.time)
                    prTime += p.prInt
                if output is not None and abs(rsTime - self.time) < 0.5 * dt:
                    self.solver.write_restart(os.path.join(output, "restartFile.saras"), self.time)
                    rsTime += p.rsInt
                if on_step:
                    on_step(self, stats)
                if abs(p.tMax - self.time) < 0.5 * dt:
                    break
        finally:
            if pfile is not None:
                pfile.close()
        return series


class scalar_d3(hydro_d3):
    """scalar_d3 (src/solvers/scalar/scalar_d3.cc:62-107): with "Restart Run"
    the fields (T included) and the time from the restart file, otherwise
    P = 1, T = 0 (or a given temperature), V = 0; then the velocity and
    temperature BCs."""

    def __init__(self, params, temperature=None, pressure=None, restart=None):
        self.params = params
        self.solver = Solver(params)
        s = self.solver
        self.time = 0.0
        if params.restartFlag:
            self.time = s.read_restart(restart or self.restart_path)
        else:
            s.set(FIELD_P, np.ones(s.dims(FIELD_P)) if pressure is None else pressure)
            s.set(FIELD_T, np.zeros(s.dims(FIELD_T)) if temperature is None else temperature)
        for f in self._bc_fields():
            s.apply_bc(f)
        self.timeStepCount = 0

    def _bc_fields(self):
        return (FIELD_VX, FIELD_VY, FIELD_VZ, FIELD_T)

    def _probe_fields(self):
        return (FIELD_VX, FIELD_VY, FIELD_VZ, FIELD_P, FIELD_T)
