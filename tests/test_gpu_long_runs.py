"""GPU parity at the configured sizes and step counts.

Each case replays one configured workload for its full step count on the GPU
and compares it with the CPU oracle's run of the same workload, stored in
tests/golden/<case>.npz by tests/golden/make_fixtures.py:

  ldc33    lid-driven cavity 33^3, 200 steps (the drop-in's Jacobi V(3,3))
  tgv129   Taylor-Green 129^3, 500 steps; energy and dissipation series
  rbc65    Rayleigh-Benard 65 x 65 x 33, 100 steps; Nusselt number series
  tgv65gs  the reference's shipped input file (Gauss-Seidel V(4,4)), 100 steps

Every step must take the oracle's Jacobi iteration counts and V-cycle count
exactly; at the end V, P, Pp (and T) must agree to 1e-10 relative to each
field's maximum at the stored sample points, and in the field's max, sum of
|F| and sum of F^2.  The tseries quantities (tseries.cc:137-246) are compared
every step: energy to 1e-12 relative, the signed maximum divergence to 1e-10
of its scale, Nu to 1e-10.  The dissipation -dE/dt (central differences of
the energy series, the same formula on both sides) to 1e-6 of its maximum:
a difference of two energies 1e-4 apart carries their 1e-12 agreement as
about 1e-8.
"""
import os

import numpy as np
import pytest

from saras_gb300 import Solver, _abi as F
from tests import _cases as C
from tests.golden import make_fixtures as M

pytestmark = pytest.mark.gpu
TOL = 1e-10
HERE = os.path.dirname(os.path.abspath(__file__))


def load(name):
    path = os.path.join(HERE, "golden", name + ".npz")
    if not os.path.exists(path):
        pytest.skip("fixture %s not generated (python tests/golden/make_fixtures.py %s)" % (path, name))
    return np.load(path)


def dissipation(energy, dt):
    e = np.asarray(energy)
    return -(e[2:] - e[:-2]) / (2.0 * dt)


@pytest.mark.parametrize("name", ["ldc33", "tgv129", "rbc65", "tgv65gs"])
def test_long_run_matches_oracle(name):
    ref = load(name)
    p, kind, steps = M.case_params(name)
    assert steps == int(ref["steps"])
    base = C.base_kind(kind)
    g = Solver(p)
    C.initialise(g, p, kind)
    assert M.initial_hash(g, base) == str(ref["initial_sha256"]), "initial state differs from the fixture's"

    def check_step(step, st):
        assert list(st.cn_iters) == list(ref["cn_iters"][step]), (step, list(st.cn_iters), list(ref["cn_iters"][step]))
        assert st.vcycles == int(ref["vcycles"][step]), (step, st.vcycles, int(ref["vcycles"][step]))

    rec = M.run(g, base, steps, check_step)
    assert np.all(rec["status"] == 0), rec["status"]
    mg = np.abs(rec["mg_residual"] - ref["mg_residual"]) <= 1e-9 * np.abs(ref["mg_residual"]) + 1e-300
    assert mg.all(), np.nonzero(~mg)[0][:5]
    e_err = np.max(np.abs(rec["energy"] - ref["energy"]) / np.abs(ref["energy"]))
    assert e_err <= 1e-12, e_err
    d_scale = np.max(np.abs(ref["max_div"]))
    assert np.max(np.abs(rec["max_div"] - ref["max_div"])) <= TOL * d_scale + 1e-14
    if base == "rbc":
        nu_err = np.max(np.abs(rec["nusselt"] - ref["nusselt"]) / np.maximum(np.abs(ref["nusselt"]), 1e-300))
        assert nu_err <= TOL, nu_err
    if base == "tgv":
        dg, do = dissipation(rec["energy"], p.tStp), dissipation(ref["energy"], p.tStp)
        assert np.max(np.abs(dg - do)) <= 1e-6 * np.max(np.abs(do))
    for f in M.state_fields(base):
        a = g.get(f)
        nm = F.FIELD_NAMES[f]
        scale = float(ref["max_" + nm])
        assert abs(np.max(np.abs(a)) - scale) <= TOL * scale, nm
        err = np.max(np.abs(M.sample(a) - ref["sample_" + nm])) / max(scale, 1e-300)
        assert err <= TOL, (nm, err)
        for q, v in (("sumabs_", np.sum(np.abs(a))), ("sumsq_", np.sum(a * a))):
            r = float(ref[q + nm])
            assert abs(v - r) <= TOL * abs(r) + 1e-300, (q + nm, v, r)
