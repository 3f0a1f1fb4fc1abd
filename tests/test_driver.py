"""The reference-side integration: the C++ binding of INTEGRATION.md compiles
against the header (with stand-ins for the reference's classes) and links
against the library, and the C++ program saras_gb300_run (the reference's
main.cc and solvePDE over the C ABI, saras_gb300/csrc/saras_main.cc) runs a
parameters file: here it reports the missing device and exits 0 as the
reference's error paths do; on a GPU its TimeSeries.dat matches the oracle."""
import importlib
import os
import re
import subprocess

import numpy as np
import pytest

import saras_gb300 as S
B = importlib.import_module("saras_gb300.build")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CONFIG = os.path.join(ROOT, "tests", "golden", "configs", "tgv_65_gs.yaml")

# the reference's classes, as far as the binding touches them
STANDINS = """
#include <cstdlib>
#include <iostream>
struct BlitzArray { double *dataFirst() { return nullptr; } };
struct field { BlitzArray F; };
struct vfield { field Vx, Vy, Vz; };
struct sfield { field F; };
struct grid {};
struct parser {};
struct hydro_d3 { vfield V; sfield P; };
"""


def binding_snippet():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    m = re.search(r"```cpp\n(.*?)```", text, re.S)
    assert m, "no C++ binding in INTEGRATION.md"
    return m.group(1)


def test_binding_snippet_compiles_and_links(tmp_path):
    lib = B.build()
    src = tmp_path / "binding.cc"
    src.write_text(STANDINS + binding_snippet() + """
int main(int argc, char **) {
    if (argc > 5) {   // never taken: the link resolves every symbol the binding uses
        grid g; parser p; hydro_d3 h;
        hydro_gb300 s(g, p, h);
        s.timeAdvance();
        s.download();
    }
    return 0;
}
""")
    out = tmp_path / "binding"
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-o", str(out), str(src), "-I" + os.path.join(ROOT, "include"),
                        "-L" + os.path.dirname(lib), "-lsaras_gb300", "-Wl,-rpath," + os.path.dirname(lib)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_driver_is_built():
    B.build()
    assert os.access(B.DRIVER, os.X_OK)


def small_config(tmp_path):
    """The shipped parameters file shrunk to 17^3, depth 2, 10 steps, with probes
    every 5 steps and a restart file every 5."""
    text = open(CONFIG).read()
    for key, old, new in [("X Index", "6", "4"), ("Y Index", "6", "4"), ("Z Index", "6", "4"),
                          ("V-Cycle Depth", "3", "2"), ("Final Time", "0.1", "0.01"),
                          ("Record Probes", "false", "true"), ("Probe Time Interval", "0.1", "0.005"),
                          ("Restart Write Interval", "0.02", "0.005")]:
        pat = '"%s": %s\n' % (key, old)
        assert pat in text, key
        text = text.replace(pat, '"%s": %s\n' % (key, new))
    path = tmp_path / "parameters.yaml"
    path.write_text(text)
    return str(path)


def run_driver(cfg, outdir):
    return subprocess.run([B.DRIVER, cfg, outdir], capture_output=True, text=True, timeout=600)


def test_driver_without_device_exits_like_the_reference(tmp_path):
    """No GPU: the reference's error convention (message, exit status 0)."""
    if _has_device():
        pytest.skip("a GPU is visible")
    B.build()
    r = run_driver(small_config(tmp_path), str(tmp_path / "out"))
    assert r.returncode == 0
    assert "ERROR" in r.stdout and "device" in r.stdout, r.stdout


def _has_device():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.gpu
def test_driver_time_series_matches_oracle(tmp_path):
    """Ten steps of the shipped Taylor-Green case (Gauss-Seidel V(4,4), 17^3):
    TimeSeries.dat (time, energy, divergence, dt as tseries.cc writes them, 8
    decimals) equals the oracle's energies to the file's resolution; probes and
    the restart file are written."""
    from oracle.oracle import Oracle
    from tests import _cases as C
    B.build()
    cfg = small_config(tmp_path)
    out = tmp_path / "out"
    r = run_driver(cfg, str(out))
    assert r.returncode == 0 and "Simulation completed" in r.stdout, r.stdout[-2000:]
    rows = [list(map(float, ln.split())) for ln in open(out / "TimeSeries.dat") if not ln.startswith("#")]
    assert len(rows) == 11
    p = S.parser(cfg)
    o = Oracle(p)
    C.initialise(o, p, "tgv_p1")
    energies = [o.diagnostics()[1]]
    for _ in range(10):
        s, _st = o.time_advance()
        assert s == 0
        energies.append(o.diagnostics()[1])
    t = np.array([row[0] for row in rows])
    e = np.array([row[1] for row in rows])
    assert np.allclose(t, np.arange(11) * 1e-3, atol=1e-9)
    assert np.max(np.abs(e - np.array(energies))) <= 1.1e-8, (e, energies)
    probe_rows = [ln for ln in open(out / "ProbesData.dat") if not ln.startswith("#")]
    assert len(probe_rows) == 3   # t = 0, 0.005, 0.01
    assert os.path.getsize(out / "restartFile.saras") > 0
