"""The configurations bench.py runs are ones the library accepts: each passes the
parameter checks of saras_create and, with no GPU here, fails only for want of a
device.  The 2D solver ("Y Index" 0) is the reference's PLANAR path in the
drop-in mode; the GB300 extensions reject it before any device work."""
import importlib
import os
import sys

import pytest

import saras_gb300
from saras_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
bench = importlib.import_module("bench")


def status_of(p):
    try:
        saras_gb300.Solver(p)
    except saras_gb300.SarasError as e:
        return e.status
    return _abi.OK


def _has_device():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


pytestmark = pytest.mark.skipif(_has_device(), reason="checks the refusal for want of a device")


@pytest.mark.parametrize("name", ["plain", "plain_strict", "mixed", "reference", "rbc", "ldc33", "ldc2d65", "ldc2d33"])
def test_bench_configuration_is_accepted(name):
    if name == "plain":
        p = bench.tgv_params(_abi.MG_PLAIN_TARGET, _abi.GUESS_PREVIOUS)
    elif name == "plain_strict":
        p = bench.tgv_params(_abi.MG_PLAIN_TARGET, _abi.GUESS_PREVIOUS)
        p.fastKernels = 0
    elif name == "mixed":
        p = bench.tgv_params(_abi.MG_MIXED, _abi.GUESS_LEARNED)
    elif name == "reference":
        p = bench.tgv_params(_abi.MG_REFERENCE, _abi.GUESS_PREVIOUS)
    elif name == "rbc":
        p = bench.rbc_params(_abi.GUESS_LEARNED)
    elif name == "ldc33":
        p = bench.ldc33_params()
    else:
        p = bench.ldc2d_params(6 if name == "ldc2d65" else 5)
    assert status_of(p) == _abi.NO_DEVICE


def test_planar_solver_is_the_drop_in_only():
    """Y Index 0 with the reference's settings is accepted; with a target
    multigrid mode, the fast kernels or a history guess it is refused."""
    p = bench.ldc2d_params(5)
    assert status_of(p) == _abi.NO_DEVICE
    for field, value in (("mgMode", _abi.MG_MIXED), ("fastKernels", 2), ("guessMode", _abi.GUESS_EXTRAPOLATE)):
        q = bench.ldc2d_params(5)
        setattr(q, field, value)
        if field == "mgMode":
            q.gsSmooth = 0
            q.preSmooth = q.postSmooth = 3
        assert status_of(q) == _abi.BAD_CONFIG, field


def test_2d_cavity_parameters_file_is_the_study():
    """tests/golden/configs/ldc2d_65.yaml, the reference's 2D cavity check on 65 x 65
    points as a parameters file, parses to the configuration of the ldc2d_ghia study."""
    p = saras_gb300.parser(os.path.join(ROOT, "tests", "golden", "configs", "ldc2d_65.yaml"))
    q = bench.ldc2d_params(6)
    for k in ("probType", "xInd", "yInd", "zInd", "vcDepth", "vcCount", "gsSmooth", "preSmooth", "postSmooth", "resType",
              "mgTolerance", "cnTolerance", "useCFL", "courantNumber", "tStp", "tMax", "Re", "xPer", "yPer", "zPer"):
        assert getattr(p, k) == getattr(q, k), k
    assert status_of(p) == _abi.NO_DEVICE
