"""Solver configurations and initial states shared by the parity tests.

Each case mirrors one of the reference's benchmark workloads (Taylor-Green
vortex, lid-driven cavity, Rayleigh-Benard convection) at a size the CPU
oracle finishes in seconds (the same code paths as the full-size runs: same
boundary types, multigrid depth pattern and tolerances).
"""
import math

import numpy as np

from saras_gb300 import _abi
from saras_gb300 import taylor_green_velocity, taylor_green_velocity_2d, taylor_green_pressure, rbc_temperature


def base():
    p = _abi.default_params()
    p.cnTolerance = 1.0e-8
    p.mgTolerance = 1.0e-8
    p.preSmooth = p.postSmooth = 3
    p.gsSmooth = 0
    p.vcCount = 200
    p.resType = 1
    return p


def ldc(ind=4, depth=2, dt=1.0e-3):
    """3D lid-driven cavity: unit cube, NNN, Re 1000, lid Vx = 1 on z = 1."""
    p = base()
    p.probType, p.icType = 1, 0
    p.xPer = p.yPer = p.zPer = 0
    p.Lx = p.Ly = p.Lz = 1.0
    p.xInd = p.yInd = p.zInd = ind
    p.vcDepth = depth
    p.Re = 1000.0
    p.tStp = dt
    return p


def tgv(ind=4, depth=2, dt=1.0e-3):
    """Taylor-Green vortex: [0, 2 pi]^3 triply periodic, Re 1600."""
    p = base()
    p.probType, p.icType = 2, 1
    p.xPer = p.yPer = p.zPer = 1
    p.Lx = p.Ly = p.Lz = 2.0 * math.pi
    p.xInd = p.yInd = p.zInd = ind
    p.vcDepth = depth
    p.Re = 1600.0
    p.tStp = dt
    return p


def rbc(ind=(4, 4, 3), depth=2, dt=5.0e-4):
    """Rayleigh-Benard: 2:2:1 box, PPN, Ra 1e7, Pr 1, rbcType 2, buoyancy."""
    p = base()
    p.probType, p.icType = 5, 0
    p.xPer = p.yPer = 1
    p.zPer = 0
    p.Lx, p.Ly, p.Lz = 2.0, 2.0, 1.0
    p.xInd, p.yInd, p.zInd = ind
    p.vcDepth = depth
    p.Ra, p.Pr, p.rbcType, p.forceType = 1.0e7, 1.0, 2, 3
    p.Re = 1.0
    p.tStp = dt
    return p


def stretched(make, axes, beta):
    """A case on a mesh with double-sided tangent-hyperbolic stretching (Mesh
    Type 'D', grid.cc:442-519) along `axes`, stretching factor `beta`."""
    def build(**kw):
        p = make(**kw)
        for a in axes:
            setattr(p, "xyz"[a] + "Grid", 2)
            setattr(p, "beta" + "XYZ"[a], beta)
        return p
    return build


def base_kind(kind):
    """The case family of an initial-state kind ("tgv_p1" is a Taylor-Green
    case, "ldc_d" the lid-driven cavity on a stretched mesh)."""
    return "tgv" if kind.startswith("tgv") else kind.split("_")[0]


def initialise(solver, p, kind):
    """Apply the constructor sequence of hydro_d3 / scalar_d3 to a Solver or Oracle.

    kind "tgv" adds the harness-set Taylor-Green pressure; "tgv_p1" keeps the
    reference's own P = 1 (hydro_d3.cc:90) under the Taylor-Green velocity."""
    F = _abi
    if base_kind(kind) == "rbc":
        solver.set(F.FIELD_P, np.ones(solver.dims(F.FIELD_P)))
        solver.set(F.FIELD_T, rbc_temperature(p, seed=42))
        for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_T):
            solver.apply_bc(f)
        return
    if base_kind(kind) == "tgv" and p.yInd == 0:
        Vx, Vz = taylor_green_velocity_2d(p)
        solver.set(F.FIELD_VX, Vx)
        solver.set(F.FIELD_VZ, Vz)
        solver.set(F.FIELD_P, np.ones(solver.dims(F.FIELD_P)))
    elif base_kind(kind) == "tgv":
        Vx, Vy = taylor_green_velocity(p)
        solver.set(F.FIELD_VX, Vx)
        solver.set(F.FIELD_VY, Vy)
        solver.set(F.FIELD_P, taylor_green_pressure(p) if kind == "tgv" else np.ones(solver.dims(F.FIELD_P)))
    else:
        solver.set(F.FIELD_P, np.ones(solver.dims(F.FIELD_P)))
    for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ):
        solver.apply_bc(f)


CASES = {"ldc": ldc, "tgv": tgv, "rbc": rbc,
         # stretched meshes: the cavity along every axis, the convection cell
         # along z (its walls), the periodic vortex along x
         "ldc_d": stretched(ldc, (0, 1, 2), 1.3), "rbc_d": stretched(rbc, (2,), 1.2), "tgv_d": stretched(tgv, (0,), 1.1)}
STRETCHED = ["ldc_d", "tgv_d", "rbc_d"]


def rel_err(a, b):
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)
