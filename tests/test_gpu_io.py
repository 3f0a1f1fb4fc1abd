"""The time-loop services around the hot path, on the GPU against the oracle:
the CFL time step (vfield::computeTStp, vfield.cc:267-284, and its use in
hydro_d3::solvePDE, hydro_d3.cc:196-206), probes (probes.cc:174-189) and
restart files (writer.cc:455-540, reader.cc:213-296)."""
import os

import numpy as np
import pytest

import saras_gb300 as S
from saras_gb300 import _abi as F
from oracle.oracle import Oracle
from tests import _cases as C

pytestmark = pytest.mark.gpu
TOL = 1e-10


def pair(kind, **kw):
    p = C.CASES[kind](**kw)
    g, o = S.Solver(p), Oracle(p)
    C.initialise(g, p, kind)
    C.initialise(o, p, kind)
    return p, g, o


@pytest.mark.parametrize("courant", [1e-3, 0.1])
def test_cfl_time_step_matches_oracle(courant):
    """Each step: computeTStp on both sides (bit-equal: exact maxima, the
    reference's expression), capped at "Time-Step", then the next step runs
    with it; iteration counts equal every step, fields to 1e-10 at the end.
    A random start (every velocity component of order one) makes Courant
    1e-3 give steps below the cap and 0.1 steps at it."""
    p = C.ldc()
    p.useCFL = 1
    p.courantNumber = courant
    g, o = S.Solver(p), Oracle(p)
    C.initialise(g, p, "ldc")
    C.initialise(o, p, "ldc")
    rng = np.random.default_rng(13)
    for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ):
        a = rng.uniform(-1.0, 1.0, g.dims(f))
        g.set(f, a)
        o.set(f, a)
        g.apply_bc(f)
        o.apply_bc(f)
    capped = []
    for step in range(6):
        sg, stg = g.time_advance()
        so, sto = o.time_advance()
        assert sg == so == 0
        assert list(stg.cn_iters) == list(sto.cn_iters) and stg.vcycles == sto.vcycles, step
        dg, do = g.compute_tstp(), o.compute_tstp()
        assert dg == do, (step, dg, do)
        dt = min(dg, p.tStp)
        capped.append(dt == p.tStp)
        g.set_dt(dt)
        o.set_dt(dt)
    assert capped == [courant == 0.1] * 6, capped
    for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_P):
        assert C.rel_err(g.get(f), o.get(f)) <= TOL, F.FIELD_NAMES[f]


def test_probes_read_the_fields(tmp_path):
    """saras_probe returns the field values at the probe points (logical
    indices, ghosts allowed), equal to the oracle's arrays there."""
    p, g, o = pair("ldc")
    for _ in range(3):
        g.time_advance()
        o.time_advance()
    n = 2 ** p.xInd
    # indices inside every field's padded range (-1 .. n along a face-centred axis)
    probes = np.array([[i, j, k] for i in (0, 5, n) for j in (-1, 7) for k in (1, n // 2, n)], dtype=np.int32)
    fields = (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_P)
    vals = g.probe(probes, fields)
    for q, f in enumerate(fields):
        a = o.get(f)
        for r, (i, j, k) in enumerate(probes):
            assert vals[r, q] == a[i + 1, j + 1, k + 1], (F.FIELD_NAMES[f], i, j, k)
    with pytest.raises(S.SarasError):
        g.probe([[n + 3, 0, 0]], fields)


def test_restart_round_trip_and_continuation(tmp_path):
    """A restart file written after four steps restores the cores of V and P
    and the time into a fresh context (hydro_d3 constructor with Restart Run:
    then the velocity BCs); the continued run matches the oracle restored from
    the same cores, step by step (Pp starts at 0 after a restart on both sides,
    as the reference's restart file does not hold it)."""
    p, g, o = pair("tgv")
    for _ in range(4):
        g.time_advance()
    path = str(tmp_path / "restartFile.saras")
    g.write_restart(path, 0.004)
    q = C.tgv()
    q.restartFlag = 1
    h = S.hydro_d3(q, restart=path)
    assert h.time == 0.004
    fields = (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_P)
    for f in fields:
        a, b = g.get(f), h.solver.get(f)
        assert np.array_equal(a[1:-1, 1:-1, 1:-1], b[1:-1, 1:-1, 1:-1]), F.FIELD_NAMES[f]
    r = Oracle(q)
    for f in fields:
        a = np.zeros(r.dims(f))
        a[1:-1, 1:-1, 1:-1] = g.get(f)[1:-1, 1:-1, 1:-1]
        r.set(f, a)
    for f in fields[:3]:
        r.apply_bc(f)
    for f in fields[:3]:
        assert np.array_equal(h.solver.get(f), r.get(f)), F.FIELD_NAMES[f]
    for step in range(4):
        sh, sth = h.solver.time_advance()
        sr, str_ = r.time_advance()
        assert sh == sr == 0
        assert list(sth.cn_iters) == list(str_.cn_iters) and sth.vcycles == str_.vcycles, step
    for f in fields:
        assert C.rel_err(h.solver.get(f), r.get(f)) <= TOL, F.FIELD_NAMES[f]
    bad = C.tgv(ind=5, depth=3)
    bad.restartFlag = 1
    with pytest.raises(S.SarasError) as e:
        S.hydro_d3(bad, restart=path)
    assert e.value.status == F.BAD_CONFIG


def test_solvepde_writes_probes_and_restart(tmp_path):
    """hydro_d3.solvePDE with probes every "Probe Time Interval" and a restart
    file every "Restart Write Interval" (hydro_d3.cc:208-233)."""
    p = C.ldc()
    p.tMax = 0.01
    p.readProbes = 1
    p.prInt = 0.004
    p.rsInt = 0.005
    h = S.hydro_d3(p)
    probes = np.array([[4, 4, 4], [8, 8, 8]], dtype=np.int32)
    series = h.solvePDE(probes=probes, output=str(tmp_path))
    assert len(series) == 11 and abs(h.time - 0.01) < 1e-12
    lines = open(tmp_path / "ProbesData.dat").read().splitlines()
    assert lines[0].startswith("#VARIABLES = Time, X, Y, Z, Vx, Vy, Vz, P")
    rows = [ln.split("\t") for ln in lines[1:]]
    assert len(rows) == 2 * 3                      # t = 0, 0.004, 0.008
    assert [float(r[0]) for r in rows[::2]] == [0.0, 0.004, 0.008]
    assert all(len(r) == 8 for r in rows)
    q = C.ldc()
    q.restartFlag = 1
    r = S.hydro_d3(q, restart=str(tmp_path / "restartFile.saras"))
    assert abs(r.time - 0.01) < 1e-12


@pytest.mark.parametrize("kind,scale", [("rbc", 1.0), ("rbc", 1e7), ("ldc", 1e7)])
def test_tseries_values_and_divergence_abort(kind, scale):
    """tseries::writeTSData (tseries.cc:137-178, 195-246) on a random state:
    energy to 1e-12 relative, the Nusselt number to 1e-10 (1 + a signed sum over
    kappa: summation order), the signed maximum divergence to 1e-12, and the
    abort status of tseries.cc:141-145 (divergence above 1e5) returned on both
    sides when the velocities are scaled up."""
    p, g, o = pair(kind)
    rng = np.random.default_rng(29)
    fields = [F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ] + ([F.FIELD_T] if kind == "rbc" else [])
    for f in fields:
        a = scale * rng.uniform(-1.0, 1.0, g.dims(f)) if f != F.FIELD_T else rng.uniform(0.0, 1.0, g.dims(f))
        g.set(f, a)
        o.set(f, a)
        g.apply_bc(f)
        o.apply_bc(f)
    sg, eg, dg, ng = g.diagnostics()
    so, eo, do, no = o.diagnostics()
    limit = F.DIVERGENCE_LIMIT if scale > 1.0 else 0
    assert sg == so == limit
    assert abs(eg - eo) <= 1e-12 * abs(eo)
    assert abs(dg - do) <= 1e-12 * abs(do)
    if kind == "rbc":
        assert abs(ng - no) <= 1e-10 * abs(no), (ng, no)
