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


@pytest.mark.parametrize("cfg", ["ldc_33.yaml", "tgv_129.yaml", "tgv_257.yaml", "rbc_257.yaml", "tgv_513.yaml"])
def test_parse_shipped_configs(cfg):
    p = saras_gb300.parser(os.path.join(HERE, "golden", "configs", cfg))
    assert p.xInd >= 5 and p.vcDepth >= 3


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
    p = _abi.default_params()
    p.gsSmooth = 1
    with pytest.raises(saras_gb300.SarasError) as e:
        saras_gb300.Solver(p)
    assert e.value.status == _abi.BAD_CONFIG


def test_periodic_target_mode_needs_three_sweeps():
    """V(1,1) target-mode cycles diverge on periodic axes: rejected before any device work."""
    for pre, post, cs in ((1, 1, 0), (2, 2, 1)):
        p = _abi.default_params()
        p.mgMode = _abi.MG_MIXED
        p.preSmooth, p.postSmooth, p.coarseSmooth = pre, post, cs
        with pytest.raises(saras_gb300.SarasError) as e:
            saras_gb300.Solver(p)
        assert e.value.status == _abi.BAD_CONFIG
