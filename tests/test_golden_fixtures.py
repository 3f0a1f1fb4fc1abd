"""The long-run fixtures (tests/golden/*.npz) belong to this oracle and this
initial state: the initial fields hash to the recorded SHA-256, and the
oracle's first steps reproduce the recorded per-step counts and tseries
values exactly.  CPU only; the GPU side is tests/test_gpu_long_runs.py."""
import os

import numpy as np
import pytest

from oracle.oracle import Oracle
from tests import _cases as C
from tests.golden import make_fixtures as M

HERE = os.path.dirname(os.path.abspath(__file__))


def load(name):
    path = os.path.join(HERE, "golden", name + ".npz")
    if not os.path.exists(path):
        pytest.skip("fixture %s not generated (python tests/golden/make_fixtures.py %s)" % (path, name))
    return np.load(path)


@pytest.mark.parametrize("name,steps", [("ldc33", 3), ("rbc65", 1), ("tgv65gs", 2), ("tgv129", 1)])
def test_fixture_replays_on_the_oracle(name, steps):
    ref = load(name)
    p, kind, total = M.case_params(name)
    assert int(ref["steps"]) == total
    assert len(ref["vcycles"]) == total and ref["cn_iters"].shape == (total, 4)
    base = C.base_kind(kind)
    o = Oracle(p)
    C.initialise(o, p, kind)
    assert M.initial_hash(o, base) == str(ref["initial_sha256"])
    rec = M.run(o, base, steps)
    for k in ("cn_iters", "vcycles", "mg_residual", "energy", "max_div", "nusselt"):
        assert np.array_equal(rec[k], ref[k][:steps]), k
