"""CPU checks of the C ABI boundary: the library loads, exports every entry
point that include/saras_gb300.h declares, parses parameters.yaml files, and
fails loudly (no CPU fallback) when no GPU is visible."""
import ctypes
import os

import pytest

from saras_gb300 import _abi
import saras_gb300
from tests.conftest import gpu_available

HERE = os.path.dirname(os.path.abspath(__file__))


def test_exports_every_header_symbol():
    lib = _abi.load()
    names = _abi.header_symbols()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_params_struct_matches_library_defaults():
    lib = _abi.load()
    p = _abi.saras_params()
    assert lib.saras_default_params(ctypes.byref(p)) == 0
    q = _abi.default_params()
    for name, _ in _abi.saras_params._fields_:
        assert getattr(p, name) == getattr(q, name), name


@pytest.mark.parametrize("cfg", ["ldc_33.yaml", "tgv_129.yaml", "tgv_257.yaml", "rbc_257.yaml", "tgv_513.yaml", "tgv_65_gs.yaml"])
def test_parse_shipped_configs(cfg):
    p = saras_gb300.parser(os.path.join(HERE, "golden", "configs", cfg))
    assert p.xInd >= 5 and p.vcDepth >= 3


REFERENCE_INPUT = "/root/reference/input/parameters.yaml"


@pytest.mark.skipif(not os.path.exists(REFERENCE_INPUT), reason="the reference checkout is not on this machine")
def test_shipped_input_file_values():
    """tests/golden/configs/tgv_65_gs.yaml holds the values of the reference's own
    input/parameters.yaml (Gauss-Seidel V(4,4), 65^3 Taylor-Green): every reference
    key parses to the same value from both files."""
    a = saras_gb300.parser(REFERENCE_INPUT).to_dict()
    b = saras_gb300.parser(os.path.join(HERE, "golden", "configs", "tgv_65_gs.yaml")).to_dict()
    ext = {"testPoisson", "mgMode", "mgTarget", "mgMaxCycles", "mixedCycles", "guessMode", "jacobiWeight", "seed",
           "fastKernels", "smoother", "coarseSmooth", "coarseCycles"}
    diff = {k: (a[k], b[k]) for k in a if k not in ext and a[k] != b[k]}
    assert not diff, diff
    assert a["gsSmooth"] == 1


def test_parse_rejects_bad_config(tmp_path):
    f = tmp_path / "bad.yaml"
    f.write_text('"Program":\n    "Problem Type": 1\n    "Domain Type": "NN"\n"Mesh":\n    "Mesh Type": "UUU"\n'
                 '    "X Index": 5\n    "Y Index": 5\n    "Z Index": 5\n"Solver":\n    "Time-Step": 0.001\n'
                 '    "Final Time": 0.1\n"Multigrid":\n    "V-Cycle Depth": 3\n')
    with pytest.raises(saras_gb300.SarasError) as e:
        saras_gb300.parser(str(f))
    assert e.value.status == _abi.BAD_CONFIG
    f.write_text("not yaml at all")
    with pytest.raises(saras_gb300.SarasError):
        saras_gb300.parser(str(f))


def test_dt_larger_than_final_time_rejected(tmp_path):
    src = open(os.path.join(HERE, "golden", "configs", "ldc_33.yaml")).read()
    f = tmp_path / "dt.yaml"
    f.write_text(src.replace('"Final Time": 0.2', '"Final Time": 0.0001'))
    with pytest.raises(saras_gb300.SarasError):
        saras_gb300.parser(str(f))


@pytest.mark.skipif(gpu_available(), reason="checks the no-device path")
def test_no_device_fails_loudly():
    with pytest.raises(saras_gb300.SarasError) as e:
        saras_gb300.Solver(_abi.default_params())
    assert e.value.status == _abi.NO_DEVICE


def test_bad_config_rejected_before_device():
    for field, value in (("gsSmooth", 2), ("dScheme", 2), ("resType", 3)):
        p = _abi.default_params()
        setattr(p, field, value)
        with pytest.raises(saras_gb300.SarasError) as e:
            saras_gb300.Solver(p)
        assert e.value.status == _abi.BAD_CONFIG, field


def test_periodic_target_mode_needs_three_sweeps():
    """V(1,1) target-mode cycles diverge on periodic axes: rejected before any device work."""
    for pre, post, cs in ((1, 1, 0), (2, 2, 1)):
        p = _abi.default_params()
        p.mgMode = _abi.MG_MIXED
        p.preSmooth, p.postSmooth, p.coarseSmooth = pre, post, cs
        with pytest.raises(saras_gb300.SarasError) as e:
            saras_gb300.Solver(p)
        assert e.value.status == _abi.BAD_CONFIG


def test_stretched_mesh_runs_the_drop_in_only(tmp_path):
    """Mesh Type 'D' (tangent-hyperbolic stretching) parses and is accepted in
    the drop-in mode (it then fails only for want of a device); with a GB300
    extension (target multigrid, fast kernels, a history guess) or a
    non-positive Beta it is rejected before any device work."""
    p = _abi.default_params()
    p.xGrid, p.betaX = 2, 1.3
    with pytest.raises(saras_gb300.SarasError) as e:
        saras_gb300.Solver(p)
    assert e.value.status == _abi.NO_DEVICE
    for field, value in (("mgMode", _abi.MG_MIXED), ("fastKernels", 2), ("guessMode", _abi.GUESS_EXTRAPOLATE), ("betaX", 0.0)):
        q = _abi.default_params()
        q.xGrid, q.betaX = 2, 1.3
        if field == "mgMode":
            q.preSmooth = q.postSmooth = 2
        setattr(q, field, value)
        with pytest.raises(saras_gb300.SarasError) as e:
            saras_gb300.Solver(q)
        assert e.value.status == _abi.BAD_CONFIG, field
    text = open(os.path.join(HERE, "golden", "configs", "tgv_65_gs.yaml")).read().replace('"Mesh Type": "UUU"', '"Mesh Type": "UDS"')
    path = tmp_path / "stretched.yaml"
    path.write_text(text)
    q = saras_gb300.parser(str(path))
    assert (q.xGrid, q.yGrid, q.zGrid) == (0, 2, 1)
