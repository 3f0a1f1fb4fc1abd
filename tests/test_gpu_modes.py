"""GPU checks of the GB300 extensions: the residual-target multigrid modes
(plain FP64 and FP32-in-FP64 refinement), the fused-multiply-add kernel forms,
and failure reporting (status codes, never a GPU fault)."""
import math

import numpy as np
import pytest

import saras_gb300 as S
from saras_gb300 import _abi as F
from oracle.oracle import Oracle
from tests import _cases as C

pytestmark = pytest.mark.gpu


def target_case(mode, fast=1, ind=5, depth=3):
    p = C.tgv(ind=ind, depth=depth, dt=5e-4)
    p.mgMode = mode
    p.mgTarget = 1e-8
    p.mgMaxCycles = 100
    p.jacobiWeight = 6.0 / 7.0
    p.fastKernels = fast
    g = S.Solver(p)
    C.initialise(g, p, "tgv")
    return p, g


@pytest.mark.parametrize("mode", [F.MG_PLAIN_TARGET, F.MG_MIXED])
def test_target_modes_reach_residual(mode):
    p, g = target_case(mode)
    for _ in range(3):
        s, st = g.time_advance()
        assert s == 0
        assert st.fine_residual <= 1e-8
        assert 0 < st.vcycles < 100


def test_mixed_solve_v44_three_cycles():
    """A 65^3 mixed solve with the benchmark's cycle shape (V(4,4), three FP32
    cycles in the first refinement step) reaches the target and agrees with
    the plain FP64 solve."""
    def case(mode):
        p = C.tgv(ind=6, depth=4, dt=5e-4)
        p.mgMode = mode
        p.mgTarget = 1e-8
        p.mgMaxCycles = 100
        p.jacobiWeight = 6.0 / 7.0
        p.fastKernels = 2
        p.preSmooth = p.postSmooth = 4
        p.mixedCycles = 3
        g = S.Solver(p)
        C.initialise(g, p, "tgv")
        return g
    m, f = case(F.MG_MIXED), case(F.MG_PLAIN_TARGET)
    for _ in range(3):
        s1, st1 = m.time_advance()
        s2, _ = f.time_advance()
        assert s1 == 0 and s2 == 0 and st1.fine_residual <= 1e-8
    assert C.rel_err(m.get(F.FIELD_P), f.get(F.FIELD_P)) < 1e-7


@pytest.mark.parametrize("smoother,coarse_smooth,coarse_cycles", [(0, 0, 1), (1, 0, 1), (1, 6, 1), (1, 0, 2), (1, 4, 2)])
def test_cycle_shapes_reach_target(smoother, coarse_smooth, coarse_cycles):
    """Every smoother / coarse-smoothing / coarse-cycle combination reaches the
    residual target in both target modes, and the two modes' pressures agree;
    the Chebyshev smoother needs no more cycles than damped Jacobi."""
    out = {}
    for mode in (F.MG_PLAIN_TARGET, F.MG_MIXED):
        p = C.tgv(ind=5, depth=3, dt=5e-4)
        p.mgMode = mode
        p.mgTarget = 1e-8
        p.mgMaxCycles = 100
        p.jacobiWeight = 6.0 / 7.0
        p.fastKernels = 2
        p.smoother = smoother
        p.coarseSmooth = coarse_smooth
        p.coarseCycles = coarse_cycles
        p.mixedCycles = 0
        g = S.Solver(p)
        C.initialise(g, p, "tgv")
        cyc = 0
        for _ in range(3):
            s, st = g.time_advance()
            assert s == 0 and st.fine_residual <= 1e-8
            cyc += st.vcycles
        out[mode] = (g.get(F.FIELD_P), cyc)
        g.close()
    assert C.rel_err(out[F.MG_MIXED][0], out[F.MG_PLAIN_TARGET][0]) < 1e-7
    if smoother == 1 and coarse_smooth == 0 and coarse_cycles == 1:
        _, jac = target_case(F.MG_PLAIN_TARGET, fast=2)
        cj = sum(jac.time_advance()[1].vcycles for _ in range(3))
        assert out[F.MG_PLAIN_TARGET][1] <= cj


def test_profiling_inside_replayed_vcycles():
    """A profile slot enabled after the V-cycle graphs exist is recorded by
    event nodes inside the replayed graphs: one launch per level-0 sweep."""
    p, g = target_case(F.MG_MIXED)
    names = S.Solver.profile_names()
    k = names.index("mg_smooth_fp32")
    for _ in range(2):
        assert g.time_advance()[0] == 0
    g.profile_enable(k, True)
    cycles = steps = 0
    for _ in range(3):
        s, st = g.time_advance()
        assert s == 0 and st.fine_residual <= 1e-8
        cycles += st.vcycles
        steps += st.refine_steps
    n, ms, b = g.profile_read(k)
    # the first cycle of each refinement step starts from zero, and its first two
    # level-0 sweeps are one launch (k_tgt_sweep2z)
    assert n == cycles * (p.preSmooth + p.postSmooth) - steps
    assert ms > 0.0 and b > 0.0


def test_profiling_sampled_vcycles():
    """saras_profile_sample(every): one replayed V-cycle in `every` carries the
    timing events (the first of the run, then every `every`-th); the others
    run the untimed graph, and the solves are unchanged."""
    p, g = target_case(F.MG_MIXED)
    _, ref = target_case(F.MG_MIXED)
    names = S.Solver.profile_names()
    k = names.index("mg_smooth_fp32")
    for _ in range(2):
        assert g.time_advance()[0] == 0
        assert ref.time_advance()[0] == 0
    g.profile_enable(k, True)
    g.profile_sample(3)
    cycles = steps = 0
    for _ in range(4):
        s, st = g.time_advance()
        s2, st2 = ref.time_advance()
        assert s == 0 and s2 == 0 and st.vcycles == st2.vcycles
        cycles += st.vcycles
        steps += st.refine_steps
    n, ms, b = g.profile_read(k)
    sampled, per = (cycles + 2) // 3, p.preSmooth + p.postSmooth
    # a sampled cycle that starts a refinement step has one launch fewer
    assert sampled * (per - 1) <= n <= sampled * per
    if steps == cycles:
        assert n == sampled * (per - 1)
    assert ms > 0.0 and b > 0.0
    assert np.array_equal(g.get(F.FIELD_P), ref.get(F.FIELD_P))


def test_adaptive_refinement_cycles():
    """mixedCycles = 0: each refinement step runs the V-cycles that the measured
    contraction predicts; the target is met with fewer refinement steps than
    one cycle per step, the V-cycle count stays that of the fixed form within
    one, and the pressure agrees with the plain FP64 solve."""
    _, fixed = target_case(F.MG_MIXED)            # mixedCycles = 1
    p, adapt = target_case(F.MG_MIXED)
    adapt.close()
    p.mixedCycles = 0
    adapt = S.Solver(p)
    C.initialise(adapt, p, "tgv")
    _, plain = target_case(F.MG_PLAIN_TARGET)
    steps = {"fixed": 0, "adapt": 0}
    for step in range(6):
        s1, st1 = fixed.time_advance()
        s2, st2 = adapt.time_advance()
        s3, _ = plain.time_advance()
        assert s1 == 0 and s2 == 0 and s3 == 0
        assert st2.fine_residual <= 1e-8
        if step >= 2:
            steps["fixed"] += st1.refine_steps
            steps["adapt"] += st2.refine_steps
            assert st2.vcycles <= st1.vcycles + 1
    assert steps["adapt"] < steps["fixed"]
    assert C.rel_err(adapt.get(F.FIELD_P), plain.get(F.FIELD_P)) < 1e-7


@pytest.mark.parametrize("guess", [F.GUESS_EXTRAPOLATE, F.GUESS_QUADRATIC, F.GUESS_PARITY])
def test_history_guesses_reach_target_with_fewer_cycles(guess):
    """The history-based initial guesses (extrapolations of the previous
    pressure corrections) reach the same residual target as the previous
    pressure, in no more V-cycles, and are reported as the guess source."""
    _, prev = target_case(F.MG_MIXED)
    _, g = target_case(F.MG_MIXED)
    g.set_guess_mode(guess)
    cyc = {"prev": [], "guess": []}
    sources = []
    for step in range(8):
        s1, st1 = prev.time_advance()
        s2, st2 = g.time_advance()
        assert s1 == 0 and s2 == 0
        assert st2.fine_residual <= 1e-8
        if step >= 4:
            cyc["prev"].append(st1.vcycles)
            cyc["guess"].append(st2.vcycles)
            sources.append(st2.guess_source)
    assert sum(cyc["guess"]) <= sum(cyc["prev"])
    assert all(src in (0, guess) for src in sources) and guess in sources
    assert C.rel_err(g.get(F.FIELD_P), prev.get(F.FIELD_P)) < 1e-7


def test_mixed_matches_plain_fp64():
    """Every result of the precision form states its error against the plain FP64 solve."""
    _, a = target_case(F.MG_PLAIN_TARGET)
    _, b = target_case(F.MG_MIXED)
    for _ in range(4):
        a.time_advance()
        b.time_advance()
    for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_P):
        assert C.rel_err(b.get(f), a.get(f)) < 1e-8, F.FIELD_NAMES[f]


@pytest.mark.parametrize("fast", [1, 2])
def test_fast_kernels_match_reference_arithmetic(fast):
    """fastKernels=1 (fused forms) and 2 (split-FP64 CN update) change rounding
    only: all solve the same CN and Poisson systems."""
    _, a = target_case(F.MG_PLAIN_TARGET, fast=0)
    _, b = target_case(F.MG_PLAIN_TARGET, fast=fast)
    for _ in range(3):
        a.time_advance()
        b.time_advance()
    for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ):
        assert C.rel_err(b.get(f), a.get(f)) < 1e-8, F.FIELD_NAMES[f]


def test_split_fp64_step_with_walls():
    """Lid-driven cavity (Dirichlet walls, a velocity jump at the lid): three
    steps with fastKernels=2 (split-FP64 RHS with the Jacobi N0 fused into it,
    delta-form Jacobi) against the reference arithmetic, both solving the
    pressure to the same residual target."""
    out = {}
    for fast in (0, 2):
        p = C.ldc(ind=5, depth=3)
        p.mgMode = F.MG_PLAIN_TARGET
        p.mgTarget = 1e-8
        p.mgMaxCycles = 100
        p.jacobiWeight = 6.0 / 7.0
        p.fastKernels = fast
        g = S.Solver(p)
        C.initialise(g, p, "ldc")
        its = []
        for _ in range(3):
            s, st = g.time_advance()
            assert s == 0
            its.append(list(st.cn_iters))
        out[fast] = (its, [g.get(f) for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ)])
        g.close()
    assert out[0][0] == out[2][0]
    for a, b in zip(out[0][1], out[2][1]):
        assert C.rel_err(b, a) < 1e-8


@pytest.mark.parametrize("kind", ["ldc", "rbc"])
def test_split_fp64_cn_matches_fp64(kind):
    """One CN Jacobi solve per component with the split-FP64 update
    (fastKernels=2) against the FP64 fused form (fastKernels=1): same
    iteration counts, fields within 1e-11 (the Jacobi tolerance is 1e-8)."""
    mk = C.ldc if kind == "ldc" else C.rbc
    rng = np.random.default_rng(11)
    out = {}
    for fast in (1, 2):
        p = mk(ind=5, depth=3) if kind == "ldc" else mk(ind=(5, 5, 4), depth=3)
        p.fastKernels = fast
        g = S.Solver(p)
        C.initialise(g, p, kind)
        r = np.random.default_rng(11)
        comps = [0, 1, 2] + ([3] if kind == "rbc" else [])
        res = []
        for c in comps:
            f = F.FIELD_T if c == 3 else F.FIELD_VX + c
            rf = F.FIELD_TRHS if c == 3 else F.FIELD_NSE_X + c
            V = g.get(f)
            g.set(rf, V + 1e-3 * r.standard_normal(V.shape))
            s, it, err = g.cn_solve(c)
            assert s == 0
            res.append((it, g.get(f)))
        out[fast] = res
        g.close()
    for (ia, a), (ib, b) in zip(out[1], out[2]):
        assert ia == ib
        assert np.max(np.abs(a - b)) < 1e-11


def test_nan_input_reports_not_finite():
    """A NaN in the velocity is reported by the Jacobi solve, not hung on."""
    p = C.ldc(ind=3, depth=1)
    g = S.Solver(p)
    C.initialise(g, p, "ldc")
    V = g.get(F.FIELD_VX)
    V[4, 4, 4] = float("nan")
    g.set(F.FIELD_VX, V)
    with pytest.raises(S.SarasError) as e:
        g.time_advance()
    assert e.value.status == F.NOT_FINITE
    # the context stays usable after the error
    C.initialise(g, p, "ldc")
    g.set(F.FIELD_VX, np.zeros(g.dims(F.FIELD_VX)))
    g.apply_bc(F.FIELD_VX)
    s, st = g.time_advance()
    assert s == 0


def test_unreachable_cn_tolerance_reports_not_converged():
    """hydro_d3.cc:415-421 aborts after maxIterations; the C ABI returns a status instead."""
    p = C.ldc(ind=3, depth=1)
    p.cnTolerance = 0.0
    g = S.Solver(p)
    C.initialise(g, p, "ldc")
    s, st = g.time_advance()
    assert s == F.NOT_CONVERGED


def test_cycle_cap_reports_not_converged():
    p, g = target_case(F.MG_PLAIN_TARGET)
    g.mg_set_mode(F.MG_PLAIN_TARGET, 1e-14, 1)
    s, st = g.time_advance()
    assert s == F.NOT_CONVERGED
    assert st.vcycles == 1


def test_solvepde_ldc_runs_and_stays_bounded():
    """hydro_d3::solvePDE on the LDC case: energy grows from the lid, divergence
    stays small; the series holds the initial state (tseries::writeTSData before
    the loop, hydro_d3.cc:167) and every fifth step."""
    p = C.ldc(ind=4, depth=2)
    p.tMax = 0.02
    p.ioCnt = 5
    solver = S.hydro_d3(p)
    series = solver.solvePDE()
    assert solver.timeStepCount == 20
    assert len(series) == 5 and series[0][0] == 0.0
    assert all(0.0 < e < 1.0 for _, e, _, _ in series)
    assert all(abs(d) < 1.0 for _, _, d, _ in series)


def test_batched_field_transfers_match_single():
    """saras_upload_fields / saras_download_fields move the same bytes as
    per-field saras_upload / saras_download, from and into page-locked memory."""
    torch = pytest.importorskip("torch")
    p, g = target_case(F.MG_MIXED)
    fields = [F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_P]
    assert g.time_advance()[0] == 0
    host = [torch.empty(g.dims(f), dtype=torch.float64, pin_memory=True) for f in fields]
    g.download_fields_ptr(fields, [t.data_ptr() for t in host])
    for f, t in zip(fields, host):
        assert np.array_equal(t.numpy(), g.get(f))
    rng = np.random.default_rng(7)
    new = [rng.standard_normal(g.dims(f)) for f in fields]
    for t, a in zip(host, new):
        t.numpy()[...] = a
    g.upload_fields_ptr(fields, [t.data_ptr() for t in host])
    for f, a in zip(fields, new):
        assert np.array_equal(g.get(f), a)


@pytest.mark.parametrize("kind", ["tgv", "ldc", "rbc"])
def test_plane_streaming_stencils_match_column_kernels(kind):
    """The finest-level FP32 sweep and residual staged through shared memory by
    the TMA (k_tgt_plane_tma) compute the same bits as the column kernels
    (k_tgt_sweep, k_tgt_residual): three mixed-mode steps with each, fields
    bitwise equal, equal V-cycle counts.  Periodic (TGV), mirror (LDC) and
    mixed (RBC: PPN) faces; SARAS_PLANE_TMA=1 selects the TMA kernels (the
    column kernels are the default)."""
    import os
    mk = {"tgv": C.tgv, "ldc": C.ldc, "rbc": C.rbc}[kind]
    out = {}
    for tma in (True, False):
        p = mk(ind=(6, 6, 5) if kind == "rbc" else 6, depth=4)
        p.mgMode = F.MG_MIXED
        p.mgTarget = 1e-8
        p.mgMaxCycles = 100
        p.jacobiWeight = 6.0 / 7.0
        p.fastKernels = 2
        p.smoother = F.SMOOTHER_CHEBYSHEV
        old = os.environ.get("SARAS_PLANE_TMA")
        os.environ["SARAS_PLANE_TMA"] = "1" if tma else "0"
        try:
            g = S.Solver(p)
            assert g.plane_tma_active() == tma
        finally:
            if old is None:
                os.environ.pop("SARAS_PLANE_TMA", None)
            else:
                os.environ["SARAS_PLANE_TMA"] = old
        C.initialise(g, p, kind)
        cyc = []
        for _ in range(3):
            s, st = g.time_advance()
            assert s == 0
            cyc.append(st.vcycles)
        out[tma] = (cyc, [g.get(f) for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_P)])
        g.close()
    assert out[True][0] == out[False][0]
    for a, b in zip(out[True][1], out[False][1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("kind", ["ldc", "rbc"])
def test_split_cn_accepted_iterate_meets_tolerance(kind):
    """fastKernels = 2 accepts a Crank-Nicolson iterate on a bound (the last
    correction's size times the measured contraction) instead of evaluating its
    residual: the accepted field's residual, evaluated by the oracle with the
    reference's expression (hydro_d3.cc:392-400), is below cnTolerance for every
    component, on walls (LDC) and with the scalar (RBC)."""
    p = C.CASES[kind]()
    p.fastKernels = 2
    g, o = S.Solver(p), Oracle(p)
    C.initialise(g, p, kind)
    C.initialise(o, p, kind)
    rng = np.random.default_rng(31)
    comps = [0, 1, 2] + ([3] if kind == "rbc" else [])
    for c in comps:
        f = F.FIELD_T if c == 3 else F.FIELD_VX + c
        r = F.FIELD_TRHS if c == 3 else F.FIELD_NSE_X + c
        V = g.get(f)
        rhs = V + 1e-2 * rng.standard_normal(V.shape)
        g.set(r, rhs)
        o.set(r, rhs)
        s, iters, _ = g.cn_solve(c)
        assert s == 0 and iters >= 2, (c, iters)
        o.set(f, g.get(f))
        res = o.cn_residual(c)
        assert res < p.cnTolerance, (c, iters, res, p.cnTolerance)
