"""Write the long-run parity fixtures of tests/test_gpu_long_runs.py.

Each fixture is the CPU oracle (oracle/saras_oracle.cc, the reference's
algorithm at np = 1) run for a configured workload's full step count:

  ldc33    3D lid-driven cavity 33^3, Re 1000, dt 1e-3, 200 steps, Jacobi V(3,3)
  tgv129   Taylor-Green vortex 129^3, Re 1600, dt 1e-3, 500 steps, depth 5
  rbc65    Rayleigh-Benard 65 x 65 x 33 (2:2:1, PPN, Ra 1e7, Pr 1), dt 5e-4, 100 steps
  tgv65gs  the reference's shipped input file: Taylor-Green 65^3, Re 1000, dt 1e-3,
           100 steps, Gauss-Seidel V(4,4), 5 V-cycles at most, tolerances 1e-6

Stored per step: the Jacobi iteration counts of every component, the V-cycle
count, the last computeError value, and the tseries quantities (energy,
signed maximum divergence, Nusselt number).  Stored at the end: a strided
sample of every state field, with each field's maximum, sum of |F| and sum
of F^2 over the whole padded array.  A SHA-256 of the initial fields ties the
fixture to the initial state the GPU run must start from (the Taylor-Green
fields use correctly rounded sines, so they are the same bits on any host).

Usage: python tests/golden/make_fixtures.py [case ...]   (all cases by default)
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from saras_gb300 import _abi as F  # noqa: E402
from tests import _cases as C  # noqa: E402


def sample(a):
    """Strided sample of a padded field (about 13 points per axis, offset from the walls)."""
    s = [max(1, (n - 3) // 12) for n in a.shape]
    return np.ascontiguousarray(a[1::s[0], 2::s[1], 3::s[2]])


def state_fields(kind):
    f = [F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_P, F.FIELD_PP]
    return f + [F.FIELD_T] if kind == "rbc" else f


def initial_hash(solver, kind):
    h = hashlib.sha256()
    for f in state_fields(kind):
        h.update(np.ascontiguousarray(solver.get(f)).tobytes())
    return h.hexdigest()


def run(solver, kind, steps, on_step=None):
    """Advance `steps` steps; per-step counts and tseries values as arrays."""
    rec = {k: [] for k in ("cn_iters", "vcycles", "mg_residual", "energy", "max_div", "nusselt", "status")}
    for step in range(steps):
        s, st = solver.time_advance()
        _, e, d, nu = solver.diagnostics()
        rec["status"].append(s)
        rec["cn_iters"].append(list(st.cn_iters))
        rec["vcycles"].append(st.vcycles)
        rec["mg_residual"].append(st.mg_residual)
        rec["energy"].append(e)
        rec["max_div"].append(d)
        rec["nusselt"].append(nu)
        if on_step:
            on_step(step, st)
    return {k: np.asarray(v) for k, v in rec.items()}


def summary(solver, kind):
    out = {}
    for f in state_fields(kind):
        a = solver.get(f)
        name = F.FIELD_NAMES[f]
        out["sample_" + name] = sample(a)
        out["max_" + name] = np.max(np.abs(a))
        out["sumabs_" + name] = np.sum(np.abs(a))
        out["sumsq_" + name] = np.sum(a * a)
    return out


def case_params(name):
    """Parameters and initial-state kind of a fixture case."""
    if name == "ldc33":
        return C.ldc(ind=5, depth=3), "ldc", 200
    if name == "tgv129":
        return C.tgv(ind=7, depth=5), "tgv", 500
    if name == "rbc65":
        return C.rbc(ind=(6, 6, 5), depth=3), "rbc", 100
    if name == "tgv65gs":
        import saras_gb300
        p = saras_gb300.parser(os.path.join(HERE, "configs", "tgv_65_gs.yaml"))
        return p, "tgv_p1", int(round(p.tMax / p.tStp))
    raise KeyError(name)


CASES = ("ldc33", "rbc65", "tgv65gs", "tgv129")


def make(name):
    from oracle.oracle import Oracle
    p, kind, steps = case_params(name)
    o = Oracle(p)
    C.initialise(o, p, kind)
    ih = initial_hash(o, C.base_kind(kind))
    t0 = time.time()

    def log(step, st):
        if step % 10 == 0:
            print("%s step %d: cn %s, V-cycles %d (%.0f s)" % (name, step, list(st.cn_iters), st.vcycles, time.time() - t0),
                  flush=True)
    rec = run(o, C.base_kind(kind), steps, log)
    out = dict(rec)
    out.update(summary(o, C.base_kind(kind)))
    out["initial_sha256"] = np.array(ih)
    out["steps"] = np.array(steps)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("wrote %s (%.0f s)" % (path, time.time() - t0))


if __name__ == "__main__":
    for n in (sys.argv[1:] or CASES):
        make(n)
