"""saras_cn_solve_noalloc: the Jacobi solve for callers that cannot allocate
device memory when they need it (a fixed memory budget handed over at
start-up, or a pool allocator that refuses new requests inside the simulation
loop).  It runs the same kernels as saras_cn_solve on the caller's device
arrays, with its second iterate in a fixed device array owned by the library.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.  It must pass both on its own
in a fresh process (where its first call performs the one-time scratch
lookup) and after the rest of the suite."""
import ctypes

import numpy as np
import pytest

import saras_gb300 as S
from saras_gb300 import _abi as F
from tests import _cases as C

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _reference_solve(p, kind, V0, rhs, comp):
    g = S.Solver(p)
    C.initialise(g, p, kind)
    f = F.FIELD_VX + comp
    g.set(f, V0)
    g.set(F.FIELD_NSE_X + comp, rhs)
    s, it, err = g.cn_solve(comp)
    assert s == 0
    return g.get(f), it, err


@pytest.mark.parametrize("kind,comp", [("ldc", 0), ("tgv", 1), ("ldc", 2)])
def test_noalloc_matches_cn_solve_twice(kind, comp):
    p = C.CASES[kind](ind=5, depth=3)
    lib = F.load()
    g = S.Solver(p)
    C.initialise(g, p, kind)
    f = F.FIELD_VX + comp
    rng = np.random.default_rng(21 + comp)
    V0 = g.get(f)
    dev = torch.device("cuda:0")
    for call in range(2):   # two calls in a row share (and reuse) the scratch array
        rhs = V0 + (1e-3 * (call + 1)) * rng.standard_normal(V0.shape)
        ref, it_ref, err_ref = _reference_solve(p, kind, V0, rhs, comp)
        v_dev = torch.tensor(V0, dtype=torch.float64, device=dev).contiguous()
        r_dev = torch.tensor(rhs, dtype=torch.float64, device=dev).contiguous()
        torch.cuda.synchronize()
        it, err = ctypes.c_int(), ctypes.c_double()
        s = lib.saras_cn_solve_noalloc(ctypes.byref(p), comp, ctypes.c_void_p(v_dev.data_ptr()),
                                       ctypes.c_void_p(r_dev.data_ptr()), None, ctypes.byref(it), ctypes.byref(err))
        assert s == 0, lib.saras_last_error(None)
        out = v_dev.cpu().numpy()
        assert it.value == it_ref
        assert C.rel_err(out, ref) <= 1e-10
        V0 = ref


def test_noalloc_rejects_oversized_field():
    p = C.tgv(ind=8, depth=4)       # 257^3: padded Vx exceeds the fixed scratch
    lib = F.load()
    dev = torch.device("cuda:0")
    tiny = torch.zeros(8, dtype=torch.float64, device=dev)
    it, err = ctypes.c_int(), ctypes.c_double()
    s = lib.saras_cn_solve_noalloc(ctypes.byref(p), 0, ctypes.c_void_p(tiny.data_ptr()), ctypes.c_void_p(tiny.data_ptr()),
                                   None, ctypes.byref(it), ctypes.byref(err))
    assert s == F.TOO_LARGE
    assert b"scratch" in lib.saras_last_error(None)
