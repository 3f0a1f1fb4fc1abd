"""saras_cn_solve_noalloc: the Jacobi solve for callers that cannot allocate
device memory when they need it (a fixed memory budget handed over at
start-up, or a pool allocator that refuses new requests inside the simulation
loop).  It runs the same iteration as saras_cn_solve on the caller's device
arrays, with its second iterate in a fixed device array owned by the library;
with fastKernels = 2 it runs the fastKernels = 1 iteration, which solves the
same system to the same tolerance with different rounding.

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


def _fields(comp):
    return (F.FIELD_T, F.FIELD_TRHS) if comp == 3 else (F.FIELD_VX + comp, F.FIELD_NSE_X + comp)


def _reference_solve(p, kind, V0, rhs, comp):
    g = S.Solver(p)
    C.initialise(g, p, kind)
    f, r = _fields(comp)
    g.set(f, V0)
    g.set(r, rhs)
    s, it, err = g.cn_solve(comp)
    assert s == 0
    return g.get(f), it, err


def _noalloc(lib, p, comp, v_dev, r_dev, stream):
    it, err = ctypes.c_int(), ctypes.c_double()
    s = lib.saras_cn_solve_noalloc(ctypes.byref(p), comp, ctypes.c_void_p(v_dev.data_ptr()),
                                   ctypes.c_void_p(r_dev.data_ptr()), stream, ctypes.byref(it), ctypes.byref(err))
    assert s == 0, lib.saras_last_error(None)
    return it.value, err.value


CASES = [("ldc", 0, 0, False), ("tgv", 1, 0, False), ("ldc", 2, 0, True), ("rbc", 3, 0, True), ("tgv", 0, 1, True),
         ("rbc", 2, 1, False), ("ldc", 0, 2, False), ("rbc", 3, 2, True)]


@pytest.mark.parametrize("kind,comp,fast,own_stream", CASES)
def test_noalloc_matches_cn_solve_twice(kind, comp, fast, own_stream):
    """Two calls in a row (sharing, and reusing, the fixed array) against
    saras_cn_solve on the same data: equal iteration counts and 1e-10 for
    fastKernels 0 and 1; for fastKernels = 2, where saras_cn_solve runs the
    split-FP64 form, at most one iteration apart and within 10 x cnTolerance
    of the field's maximum (both stop below cnTolerance).  Device free memory
    is unchanged across the second call: nothing is allocated."""
    p = C.CASES[kind](ind=(5, 5, 4) if kind == "rbc" else 5, depth=3)
    p.fastKernels = fast
    lib = F.load()
    g = S.Solver(p)
    C.initialise(g, p, kind)
    f, _ = _fields(comp)
    rng = np.random.default_rng(21 + comp + 10 * fast)
    V0 = g.get(f)
    dev = torch.device("cuda:0")
    stream = torch.cuda.Stream() if own_stream else None
    handle = ctypes.c_void_p(stream.cuda_stream) if own_stream else None
    for call in range(2):
        rhs = V0 + (1e-3 * (call + 1)) * rng.standard_normal(V0.shape)
        ref, it_ref, _ = _reference_solve(p, kind, V0, rhs, comp)
        v_dev = torch.tensor(V0, dtype=torch.float64, device=dev).contiguous()
        r_dev = torch.tensor(rhs, dtype=torch.float64, device=dev).contiguous()
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        it, _ = _noalloc(lib, p, comp, v_dev, r_dev, handle)
        free1 = torch.cuda.mem_get_info()[0]
        if call == 1:
            assert free1 == free0, (free0, free1)
        out = v_dev.cpu().numpy()
        if fast == 2:
            assert abs(it - it_ref) <= 1, (it, it_ref)
            assert C.rel_err(out, ref) <= 10 * p.cnTolerance
        else:
            assert it == it_ref
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
