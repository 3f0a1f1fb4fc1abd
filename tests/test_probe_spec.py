"""parser::parseProbes / testProbes (parser.cc:424-575) through the C ABI on
the CPU: the "Probes" sets of a parameters file expand to the same (i, j, k)
list as a restatement of the reference's loop, and out-of-range indices are
rejected."""
import math
import os

import numpy as np
import pytest

import saras_gb300 as S
from saras_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_INPUT = "/root/reference/input/parameters.yaml"


def restated(spec):
    """parser.cc:424-531 for 3D runs: each [..] set, each entry an index or
    start:end:count, Cartesian product with x outermost."""
    out = []
    for body in spec.split("[")[1:]:
        body = body.split("]")[0]
        lists = []
        for item in body.split(","):
            item = item.strip()
            if ":" not in item:
                lists.append([int(item)])
                continue
            a, b, n = (int(x) for x in item.split(":"))
            if a == b or n == 1:
                lists.append([a])
            else:
                inc = (float(b) - float(a)) / (float(n) - 1.0)
                # C round: half away from zero
                lists.append([a + int(math.floor(i * inc + 0.5)) for i in range(n)])
        assert len(lists) == 3
        out += [[x, y, z] for x in lists[0] for y in lists[1] for z in lists[2]]
    return np.array(out, dtype=np.int32).reshape(-1, 3)


def write_cfg(tmp_path, probes):
    src = open(os.path.join(HERE, "golden", "configs", "tgv_65_gs.yaml")).read()
    src = src.replace('"Probes": >\n        [5, 5, 5]', '"Probes": >\n' + "\n".join("        " + q for q in probes))
    f = tmp_path / "p.yaml"
    f.write_text(src)
    return str(f)


def test_probe_ranges_expand_like_the_reference(tmp_path):
    sets = ["[5, 5, 5]", "[1:62:3, 1:62:3, 1:62:3]", "[1:62:3, 7, 1:62:3]", "[0:65:4, 2, 3:3:5]", "[10:20:1, 4, 64]"]
    path = write_cfg(tmp_path, sets)
    got = S.parse_probes(path)
    want = restated(" ".join(sets))
    assert got.shape == want.shape == (1 + 27 + 9 + 4 + 1, 3)
    assert np.array_equal(got, want)
    assert got[1].tolist() == [1, 1, 1] and got[2].tolist() == [1, 1, 32] and got[3].tolist() == [1, 1, 62]


def test_probe_outside_the_domain_is_rejected(tmp_path):
    path = write_cfg(tmp_path, ["[5, 5, 67]"])          # 2^6 + 1 = 65 is the last index allowed
    with pytest.raises(S.SarasError) as e:
        S.parse_probes(path)
    assert e.value.status == _abi.BAD_CONFIG
    path = write_cfg(tmp_path, ["[5, 5]"])
    with pytest.raises(S.SarasError):
        S.parse_probes(path)


@pytest.mark.skipif(not os.path.exists(REFERENCE_INPUT), reason="the reference checkout is not on this machine")
def test_shipped_input_file_probes():
    got = S.parse_probes(REFERENCE_INPUT)
    spec = open(REFERENCE_INPUT).read().split('"Probes": >')[1].split('"Multigrid"')[0]
    spec = "\n".join(line.split("#")[0] for line in spec.splitlines())
    assert np.array_equal(got, restated(spec))
    assert len(got) == 38
