"""GPU parity: every hot-path operator of the C ABI against the CPU oracle.

Every case runs on a uniform mesh and, for the "_d" kinds, on a mesh with
double-sided tangent-hyperbolic stretching (grid.cc:442-519), where every
stencil reads the metric arrays at its point (xixx terms included).

The CUDA path runs the reference arithmetic in the reference order (no FMA
contraction), so agreement is expected to the last bit for all local
operators; reductions whose summation order differs (the padded-array mean of
the multigrid RHS, the energy sum) agree to rounding.  The bar written in every
assertion is the drop-in's parity tolerance: 1e-10 relative to the field's maximum.
"""
import numpy as np
import pytest

from saras_gb300 import Solver, _abi as F
from oracle.oracle import Oracle
from tests import _cases as C

pytestmark = pytest.mark.gpu
TOL = 1e-10


def pair(kind, **kw):
    p = C.CASES[kind](**kw)
    g, o = Solver(p), Oracle(p)
    C.initialise(g, p, kind)
    C.initialise(o, p, kind)
    return p, g, o


def assert_close(a, b, what, tol=TOL):
    e = C.rel_err(a, b)
    assert e <= tol, "%s: relative error %.3e > %.1e" % (what, e, tol)


FIELDS = {"ldc": [F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ], "tgv": [F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ],
          "rbc": [F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_T]}
KINDS = ["ldc", "tgv", "rbc"] + C.STRETCHED


def fields_of(kind):
    return FIELDS[C.base_kind(kind)]


@pytest.mark.parametrize("kind", KINDS)
def test_initial_bc_state(kind):
    p, g, o = pair(kind)
    for f in fields_of(kind) + [F.FIELD_P]:
        assert np.array_equal(g.get(f), o.get(f)), F.FIELD_NAMES[f]


@pytest.mark.parametrize("kind", KINDS)
def test_boundary_fill_random(kind):
    """imposeU/V/W/TBCs on random data: syncData + wall objects, bit-exact."""
    p, g, o = pair(kind)
    rng = np.random.default_rng(7)
    for f in fields_of(kind):
        a = rng.standard_normal(g.dims(f))
        g.set(f, a); o.set(f, a)
        g.apply_bc(f); o.apply_bc(f)
        assert np.array_equal(g.get(f), o.get(f)), F.FIELD_NAMES[f]
    a = rng.standard_normal(g.dims(F.FIELD_PP))
    g.set(F.FIELD_PP, a); o.set(F.FIELD_PP, a)
    g.sync_field(F.FIELD_PP); o.sync_field(F.FIELD_PP)
    assert np.array_equal(g.get(F.FIELD_PP), o.get(F.FIELD_PP))


@pytest.mark.parametrize("kind", KINDS)
def test_field_operators(kind):
    """computeDiff, computeNLin, gradient, divergence (and T's) on random fields."""
    p, g, o = pair(kind)
    rng = np.random.default_rng(11)
    for f in fields_of(kind):
        a = rng.standard_normal(g.dims(f))
        g.set(f, a); o.set(f, a)
        g.apply_bc(f); o.apply_bc(f)
    for f in (F.FIELD_P, F.FIELD_PP):
        a = rng.standard_normal(g.dims(f))
        g.set(f, a); o.set(f, a)
    for f in (F.FIELD_NSE_X, F.FIELD_NSE_Y, F.FIELD_NSE_Z):
        z = np.zeros(g.dims(f)); g.set(f, z); o.set(f, z)
    g.vfield_compute_diff(); o.vfield_compute_diff()
    for f in (F.FIELD_NSE_X, F.FIELD_NSE_Y, F.FIELD_NSE_Z):
        assert_close(g.get(f), o.get(f), "computeDiff " + F.FIELD_NAMES[f], 0.0)
    g.vfield_compute_nlin(); o.vfield_compute_nlin()
    for f in (F.FIELD_NSE_X, F.FIELD_NSE_Y, F.FIELD_NSE_Z):
        assert_close(g.get(f), o.get(f), "computeNLin " + F.FIELD_NAMES[f], 0.0)
    for sf in (F.FIELD_P, F.FIELD_PP):
        g.sfield_gradient(sf); o.sfield_gradient(sf)
        for f in (F.FIELD_GRAD_X, F.FIELD_GRAD_Y, F.FIELD_GRAD_Z):
            assert np.array_equal(g.get(f), o.get(f)), "gradient " + F.FIELD_NAMES[f]
    g.vfield_divergence(); o.vfield_divergence()
    assert np.array_equal(g.get(F.FIELD_MGRHS), o.get(F.FIELD_MGRHS))
    if C.base_kind(kind) == "rbc":
        z = np.zeros(g.dims(F.FIELD_TRHS)); g.set(F.FIELD_TRHS, z); o.set(F.FIELD_TRHS, z)
        g.tfield_compute_diff(); o.tfield_compute_diff()
        g.tfield_compute_nlin(); o.tfield_compute_nlin()
        assert np.array_equal(g.get(F.FIELD_TRHS), o.get(F.FIELD_TRHS))


@pytest.mark.parametrize("kind", KINDS)
def test_cn_solve(kind):
    """solveVx/Vy/Vz (and solveT): iterations equal, fields to 1e-10."""
    p, g, o = pair(kind)
    rng = np.random.default_rng(5)
    comps = [0, 1, 2] + ([3] if C.base_kind(kind) == "rbc" else [])
    for c in comps:
        f = F.FIELD_T if c == 3 else F.FIELD_VX + c
        r = F.FIELD_TRHS if c == 3 else F.FIELD_NSE_X + c
        V = g.get(f)
        rhs = V + 1e-3 * rng.standard_normal(V.shape)
        g.set(r, rhs); o.set(r, rhs)
        sg, ig, eg = g.cn_solve(c)
        so, io, eo = o.cn_solve(c)
        assert sg == so == 0
        assert ig == io, (c, ig, io)
        assert_close(g.get(f), o.get(f), "CN " + F.FIELD_NAMES[f])


LEVEL_CASES = ([(k, 4, 0) for k in ("ldc", "tgv", "rbc")] + [(k, ind, 1) for k in ("ldc", "tgv", "rbc") for ind in (4, 5)] +
               [(k, 4, gs) for k in C.STRETCHED for gs in (0, 1)] + [(k, 5, 1) for k in C.STRETCHED])


@pytest.mark.parametrize("kind,ind,gs", LEVEL_CASES)
def test_multigrid_level_operators(kind, ind, gs):
    """smooth / residual+restriction / coarsest GS / prolongation+add / computeError,
    fed level by level the way vCycle feeds them (poisson.cc:219-280).  Level
    data is set right before use: the reference's Jacobi swap exchanges the
    arrays of every level at once (poisson_d3.cc:168), so data parked on other
    levels does not survive a smoothing call.  gs = 1: lexicographic
    Gauss-Seidel smoothing (poisson_d3.cc:137-150), bit for bit; at ind 5 the
    finest level (35^3 padded) runs the multi-CTA wavefront kernel, the others
    the shared-memory one."""
    kw = dict(ind=(ind, ind, ind - 1) if C.base_kind(kind) == "rbc" else ind, depth=2)
    p = C.CASES[kind](**kw)
    p.gsSmooth = gs
    g, o = Solver(p), Oracle(p)
    C.initialise(g, p, kind)
    C.initialise(o, p, kind)
    rng = np.random.default_rng(3)

    def put(lvl, which, a):
        g.set_level(lvl, which, a); o.set_level(lvl, which, a)

    def core(a):
        return a[1:-1, 1:-1, 1:-1]
    put(0, 0, rng.standard_normal(g.level_dims(0)))
    put(0, 1, rng.standard_normal(g.level_dims(0)))
    g.mg_smooth(0, 3); o.mg_smooth(0, 3)
    assert np.array_equal(core(g.get_level(0, 0)), core(o.get_level(0, 0)))
    g.mg_restrict(0); o.mg_restrict(0)
    assert np.array_equal(core(g.get_level(1, 1)), core(o.get_level(1, 1)))
    put(1, 0, 0.1 * rng.standard_normal(g.level_dims(1)))
    g.mg_smooth(1, 2); o.mg_smooth(1, 2)
    assert np.array_equal(core(g.get_level(1, 0)), core(o.get_level(1, 0)))
    g.mg_restrict(1); o.mg_restrict(1)
    assert np.array_equal(core(g.get_level(2, 1)), core(o.get_level(2, 1)))
    put(2, 0, np.zeros(g.level_dims(2)))
    g.mg_smooth(2, -1); o.mg_smooth(2, -1)       # coarsest Gauss-Seidel solve
    assert_close(core(g.get_level(2, 0)), core(o.get_level(2, 0)), "coarsest solve", 0.0)
    g.mg_prolong_add(1); o.mg_prolong_add(1)
    assert np.array_equal(core(g.get_level(1, 0)), core(o.get_level(1, 0)))
    g.mg_prolong_add(0); o.mg_prolong_add(0)
    assert np.array_equal(core(g.get_level(0, 0)), core(o.get_level(0, 0)))
    g.mg_smooth(0, 3); o.mg_smooth(0, 3)          # post-smoothing ends with imposeBC
    assert np.array_equal(core(g.get_level(0, 0)), core(o.get_level(0, 0)))
    for norm in (1, 2):
        eg, eo = g.mg_compute_error(norm), o.mg_compute_error(norm)
        assert eg == eo, (norm, eg, eo)


@pytest.mark.parametrize("kind,ind,gs", [(k, 4, 0) for k in KINDS] + [(k, 5, 1) for k in KINDS])
def test_mg_solve(kind, ind, gs):
    """poisson::mgSolve on the divergence of a random velocity field (gs = 1:
    Gauss-Seidel smoothing on every level, as the reference's shipped input)."""
    p = C.CASES[kind](ind=(ind, ind, ind - 1) if C.base_kind(kind) == "rbc" else ind, depth=2 if ind == 4 else 3)
    p.gsSmooth = gs
    g, o = Solver(p), Oracle(p)
    C.initialise(g, p, kind)
    C.initialise(o, p, kind)
    rng = np.random.default_rng(17)
    for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ):
        a = g.get(f) + 0.1 * rng.standard_normal(g.dims(f))
        g.set(f, a); o.set(f, a)
        g.apply_bc(f); o.apply_bc(f)
    g.vfield_divergence(); o.vfield_divergence()
    cg, rg = g.mg_solve()
    co, ro = o.mg_solve()
    assert cg == co
    assert abs(rg - ro) <= 1e-9 * abs(ro)
    assert_close(g.get(F.FIELD_PP), o.get(F.FIELD_PP), "Pp")


@pytest.mark.parametrize("kind,steps,gs", [("ldc", 10, 0), ("tgv", 10, 0), ("rbc", 10, 0), ("ldc", 5, 1), ("tgv", 5, 1),
                                           ("rbc", 5, 1), ("ldc_d", 10, 0), ("tgv_d", 10, 0), ("rbc_d", 10, 0), ("ldc_d", 5, 1),
                                           ("rbc_d", 5, 1)])
def test_time_advance(kind, steps, gs):
    """hydro_d3 / scalar_d3 timeAdvance: equal iteration counts every step and
    V, P (and T) within 1e-10 after the run (gs = 1: Gauss-Seidel smoothing)."""
    p = C.CASES[kind]()
    p.gsSmooth = gs
    g, o = Solver(p), Oracle(p)
    C.initialise(g, p, kind)
    C.initialise(o, p, kind)
    fields = [F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_P, F.FIELD_PP] + ([F.FIELD_T] if C.base_kind(kind) == "rbc" else [])
    for step in range(steps):
        sg, stg = g.time_advance()
        so, sto = o.time_advance()
        assert sg == so == 0
        errs = {F.FIELD_NAMES[f]: C.rel_err(g.get(f), o.get(f)) for f in fields}
        assert list(stg.cn_iters) == list(sto.cn_iters), (step, errs)
        assert stg.vcycles == sto.vcycles, (step, stg.vcycles, sto.vcycles, errs)
    for f in fields:
        assert_close(g.get(f), o.get(f), F.FIELD_NAMES[f])
    _, eg, dg, ng = g.diagnostics()
    _, eo, do, no = o.diagnostics()
    assert abs(eg - eo) <= 1e-12 * abs(eo)
    assert abs(dg - do) <= 1e-10 * max(abs(do), 1e-300) + 1e-14


@pytest.mark.parametrize("kind", ["tgv"])
def test_reference_kats(kind):
    """multigrid_d3::testProlong/testTransfer/testPeriodic and hydro_d3::testPeriodic
    (poisson_test.cc:74-98, hydro_test.cc:66-72: tolerance 1e-10)."""
    p, g, o = pair(kind, ind=4, depth=2)
    assert g.mg_test_prolong() <= 1e-10
    assert g.mg_test_transfer() <= 1e-10
    assert g.mg_test_periodic() <= 1e-10
    assert g.hydro_test_periodic() <= 1e-10


@pytest.mark.parametrize("ind,gs", [(4, 0), (4, 1), (5, 1)])
def test_dirichlet_poisson_check(ind, gs):
    """TEST_POISSON: rhs = 1, Dirichlet walls r^2/6 (poisson_d3.cc:513-572); the
    discrete Laplacian is exact for quadratics, so the solve recovers r^2/6
    (gs = 1: Gauss-Seidel smoothing with the fixed wall values in the ghosts)."""
    p = C.ldc(ind=ind, depth=2)
    p.gsSmooth = gs
    p.probType = 2
    p.testPoisson = 1
    p.vcCount = 25
    p.resType = 2
    g, o = Solver(p), Oracle(p)
    g.set(F.FIELD_MGRHS, np.ones(g.dims(F.FIELD_MGRHS)))
    o.set(F.FIELD_MGRHS, np.ones(o.dims(F.FIELD_MGRHS)))
    cg, rg = g.mg_solve()
    co, ro = o.mg_solve()
    assert cg == co == 25
    Pg, Po = g.get(F.FIELD_PP), o.get(F.FIELD_PP)
    assert_close(Pg, Po, "Dirichlet Pp")
    n = 2 ** p.xInd
    h = 1.0 / n
    x = (np.arange(n + 1) - n // 2) * h
    ana = (x[:, None, None] ** 2 + x[None, :, None] ** 2 + x[None, None, :] ** 2) / 6.0
    assert np.max(np.abs(Pg[1:-1, 1:-1, 1:-1] - ana)) < 1e-3
