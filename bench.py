#!/usr/bin/env python
"""Throughput of the SARAS time step on GB300.

Workload: 3D Taylor-Green vortex, 257^3 vertex grid on [0, 2 pi]^3, Re 1600,
dt 5e-4 (the precision-form / learned-warm-start configuration).  A "step" is
one hydro_d3::timeAdvance: NSE right-hand side, three Crank-Nicolson Jacobi
solves, divergence, the pressure-correction solve to the FP64 residual target
max|b - Ap| / max|b| <= 1e-8, projection and boundary fills.

Our arm runs the pressure solve as FP32 V-cycles inside FP64 iterative
refinement (optionally warm-started by the U-Net); the same run also times the
plain FP64 V-cycle solve to the same residual target and reports both.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU: the path does not shard (one GPU owns the whole domain), so N > 1
runs N independent replicas and `value` sums their steps.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GRID_INDEX = 8          # 2^8 + 1 = 257 points per axis
DEPTH = 6
DT = 5.0e-4
TARGET = 1.0e-8
METRIC = "steps/s at 257^3: learned+mixed MG vs plain FP64 MG at equal 1e-8 residual"
PROF_EVERY = 8          # timed V-cycles: one replay in PROF_EVERY


def tgv_params(mode, guess=0, ind=GRID_INDEX, depth=DEPTH):
    from saras_gb300 import _abi
    p = _abi.default_params()
    p.probType, p.icType = 2, 1
    p.xPer = p.yPer = p.zPer = 1
    p.Lx = p.Ly = p.Lz = 2.0 * math.pi
    p.xInd = p.yInd = p.zInd = ind
    p.vcDepth = depth
    p.Re = 1600.0
    p.tStp = DT
    p.cnTolerance = 1.0e-8
    p.mgTolerance = 1.0e-8
    # both target-mode arms with the cycle each is fastest with at 257^3
    # (ms a step): plain FP64 -- Chebyshev (2,2) cycles with three cycles at
    # the second level a visit, 15.5 (4 cycles; with two 16.6, four 17.1,
    # Chebyshev (3,3) with three 19.0, damped-Jacobi (2,2) with three 21.7,
    # Chebyshev V(3,3) 23.9); mixed -- Chebyshev V(3,3) 4.61 (3 cycles in one
    # refinement step; V(2,2) 4.68 with 4, (2,2) with two cycles at the second
    # level 4.70, (3,3) with three 4.86), refinement steps sized by the
    # measured contraction per cycle
    plain = mode == _abi.MG_PLAIN_TARGET
    p.preSmooth = p.postSmooth = 2 if plain else 3
    p.smoother = _abi.SMOOTHER_CHEBYSHEV if mode != _abi.MG_REFERENCE else _abi.SMOOTHER_JACOBI
    p.coarseCycles = 3 if plain else 1
    p.mgMode = mode
    p.mgTarget = TARGET
    p.mgMaxCycles = 100
    p.mixedCycles = 0
    p.jacobiWeight = 6.0 / 7.0 if mode != _abi.MG_REFERENCE else 1.0
    p.fastKernels = 2 if mode != _abi.MG_REFERENCE else 0
    p.guessMode = guess
    return p


def init_tgv(solver, p):
    import saras_gb300 as S
    from saras_gb300 import _abi as F
    Vx, Vy = S.taylor_green_velocity(p)
    solver.set(F.FIELD_VX, Vx)
    solver.set(F.FIELD_VY, Vy)
    solver.set(F.FIELD_P, S.taylor_green_pressure(p))
    for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ):
        solver.apply_bc(f)


# ------------------------------------------------------------------ distributed
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo", init_method="env://")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ------------------------------------------------------------------ clocks
class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
            sm = [float(r[1]) for r in rows if len(r) >= 9]
            mx = [float(r[2]) for r in rows if len(r) >= 9]
            reasons = set()
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for r in rows:
                if len(r) < 9:
                    continue
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                   "reasons": sorted(reasons), "samples": len(sm)}
        except Exception:
            pass
        try:
            os.unlink(self.path)
        except Exception:
            pass
        return out


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel):
    """Per-launch DRAM traffic (bytes) of profile slot `kernel` at this workload, from
    the table in the committed ncu summary profiles/ncu_traffic.md (None if absent)."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.md")) as f:
            for line in f:
                cells = [x.strip() for x in line.strip().strip("|").split("|")]
                if len(cells) >= 3 and cells[0] == kernel:
                    return float(cells[2])
    except Exception:
        pass
    return None


# ------------------------------------------------------------------ arms
def prepare_headline(g, args):
    """Bring the headline solver to its timed state: warm-up steps (with the
    learned warm start they also yield the U-Net's training pairs), training,
    then the guess mode of the timed steps.  Returns (learned info, steps done)."""
    from saras_gb300 import _abi as F
    warm_steps = max(args.warmup, args.collect) if args.learned else args.warmup
    learn = None
    done = 0
    if args.learned:
        g.unet_collect()
    warm_vc = []
    for k in range(warm_steps):
        s, st = g.time_advance()
        if s != 0:
            raise RuntimeError("warm-up step failed: %d" % s)
        warm_vc.append(st.vcycles)
    done += warm_steps
    if args.learned:
        t0 = time.perf_counter()
        loss = g.unet_train(args.train_iters, args.lr)
        g.synchronize()
        learn = {"pairs": max(0, warm_steps - 2), "train_iters": args.train_iters, "lr": args.lr,
                 "final_loss": loss, "train_seconds": round(time.perf_counter() - t0, 3),
                 "vcycles_per_step_warmup_previous_guess": sum(warm_vc[-5:]) / len(warm_vc[-5:])}
        g.set_guess_mode(F.GUESS_LEARNED)
        g.time_advance()
        done += 1
    elif args.guess != "previous":
        g.set_guess_mode({"extrapolate": F.GUESS_EXTRAPOLATE, "quadratic": F.GUESS_QUADRATIC}[args.guess])
        for k in range(3):
            g.time_advance()
        done += 3
    return learn, done


def time_steps(g, n):
    """n steps between two events on the solver's stream: (ms, per-step stats)."""
    g.synchronize()
    g.event_record(0)
    sts = []
    for k in range(n):
        s, st = g.time_advance()
        if s != 0:
            raise RuntimeError("timed step failed: %d" % s)
        sts.append((st.vcycles, st.refine_steps, st.fine_residual, st.guess_source))
    g.event_record(1)
    g.synchronize()
    return g.event_elapsed(0, 1), sts


def plain_arm(args, fast, before):
    """Plain FP64 multigrid (FP64 V-cycles to the same residual target) over the
    headline arm's step window: `before` untimed steps, then args.steps timed."""
    import saras_gb300 as S
    from saras_gb300 import _abi as F
    q = tgv_params(F.MG_PLAIN_TARGET, F.GUESS_PREVIOUS)
    q.fastKernels = fast
    h = S.Solver(q)
    init_tgv(h, q)
    for k in range(before):
        h.time_advance()
    ms, sts = time_steps(h, args.steps)
    h.close()
    return {"steps_per_s": round(args.steps / (ms / 1e3), 3), "ms_per_step": round(ms / args.steps, 3),
            "vcycles_per_step": sum(x[0] for x in sts) / len(sts), "steps": args.steps, "steps_before": before,
            "fastKernels": fast}


def tma_arm(args, before):
    """The headline arm with the finest level's FP32 sweeps and residuals run
    through the TMA plane-streaming kernels (SARAS_PLANE_TMA=1; the same bits as
    the default column kernels): steps/s over the headline's step window and the
    level-0 sweep's HBM rate, beside the default's."""
    import saras_gb300 as S
    from saras_gb300 import _abi as F
    old = os.environ.get("SARAS_PLANE_TMA")
    os.environ["SARAS_PLANE_TMA"] = "1"
    try:
        p = tgv_params(F.MG_MIXED, F.GUESS_PREVIOUS)
        g = S.Solver(p)
    finally:
        if old is None:
            os.environ.pop("SARAS_PLANE_TMA", None)
        else:
            os.environ["SARAS_PLANE_TMA"] = old
    active = g.plane_tma_active()
    init_tgv(g, p)
    g.set_guess_mode(F.GUESS_EXTRAPOLATE)
    for k in range(before):
        g.time_advance()
    names = S.Solver.profile_names()
    k_s = names.index("mg_smooth_fp32")
    g.profile_enable(k_s, True)
    g.profile_sample(PROF_EVERY)
    ms, sts = time_steps(g, args.steps)
    n_k, ms_k, b_k = g.profile_read(k_s)
    g.close()
    peak, _ = measured_peak_hbm()
    avg = ms_k / n_k if n_k else None
    gbs = (b_k / n_k) / (avg * 1e-3) / 1e9 if avg else None
    return {"active": active, "steps_per_s": round(args.steps / (ms / 1e3), 3), "guess": "extrapolate",
            "mg_smooth_fp32_avg_ms": round(avg, 4) if avg else None, "mg_smooth_fp32_GBs": round(gbs, 1) if gbs else None,
            "mg_smooth_fp32_frac": round(gbs / peak, 4) if gbs else None, "kernel": "k_tgt_plane_tma"}


def accuracy_run(args):
    """Config 3's accuracy figures: the headline arm (its guess mode, mixed
    refinement, fastKernels = 2) and the plain FP64 arm with the reference's
    arithmetic (fastKernels = 0) both run args.accuracy_steps steps from the
    initial condition; the energy series (tseries.cc:137-178) every step and
    the fields at the end are compared."""
    import numpy as np
    import saras_gb300 as S
    from saras_gb300 import _abi as F
    n = args.accuracy_steps
    series = {}
    fields = {}
    sec = {}
    for arm in ("headline", "plain_fp64"):
        t0 = time.perf_counter()
        if arm == "headline":
            p = tgv_params(F.MG_MIXED, F.GUESS_PREVIOUS)
            g = S.Solver(p)
            init_tgv(g, p)
            _, done = prepare_headline(g, args)
        else:
            p = tgv_params(F.MG_PLAIN_TARGET, F.GUESS_PREVIOUS)
            p.fastKernels = 0
            g = S.Solver(p)
            init_tgv(g, p)
            done = 0
        e = [None] * done   # energies of the headline arm's preparation steps are not read
        for k in range(done, n):
            s, st = g.time_advance()
            if s != 0:
                raise RuntimeError("accuracy step failed: %d" % s)
            _, en, _, _ = g.diagnostics()
            e.append(en)
        series[arm] = e
        fields[arm] = {nm: g.get(f) for f, nm in ((F.FIELD_VX, "Vx"), (F.FIELD_VY, "Vy"), (F.FIELD_VZ, "Vz"), (F.FIELD_P, "P"))}
        sec[arm] = round(time.perf_counter() - t0, 2)
        g.close()
    a, b = fields["headline"], fields["plain_fp64"]
    err = {nm: float(np.max(np.abs(a[nm] - b[nm])) / max(np.max(np.abs(b[nm])), 1e-300)) for nm in a}
    first = len(series["headline"]) - sum(x is not None for x in series["headline"])
    eh, ep = np.array(series["headline"][first:], dtype=float), np.array(series["plain_fp64"][first:], dtype=float)
    ke = float(np.max(np.abs(eh - ep) / np.abs(ep)))
    return {"steps": n, "dt": DT, "reference": "plain FP64 V-cycles to 1e-8, fastKernels 0 (FP64 throughout)",
            "max_pointwise_rel_err": err, "kinetic_energy_max_rel_err": ke,
            "kinetic_energy_compared_steps": [first + 1, n],
            "kinetic_energy_final": [float(eh[-1]), float(ep[-1])], "seconds": sec}


def run_ours(args, dist):
    import saras_gb300 as S
    from saras_gb300 import _abi as F
    S._abi.load()
    gpu = dist.local
    try:
        import torch
        torch.cuda.set_device(gpu)
    except Exception:
        torch = None
    p = tgv_params(F.MG_MIXED, F.GUESS_PREVIOUS)
    g = S.Solver(p)
    init_tgv(g, p)
    names = S.Solver.profile_names()
    learn, done = prepare_headline(g, args)
    # the kernels with the largest shares of one profiled step
    for k in range(len(names)):
        g.profile_enable(k, True)
    g.time_advance()
    done += 1
    totals = []
    for k in range(len(names)):
        n, ms, b = g.profile_read(k)
        if b > 0:   # kernel slots with algorithmic bytes (not the initial-guess phase)
            totals.append((ms, k))
        g.profile_enable(k, False)
    timed_slots = [k for _, k in sorted(totals, reverse=True)[:4]]
    for k in timed_slots:
        g.profile_enable(k, True)
    # the timing events inside a replayed V-cycle separate its kernels on the
    # GPU: time the kernels of one replayed cycle in PROF_EVERY, spread over
    # the whole timed region (launches outside V-cycles are all timed)
    g.profile_sample(PROF_EVERY)
    # --- timed region
    clocks = Clocks(gpu)
    clocks.start()
    dist.barrier()
    g.synchronize()
    launches0 = g.launch_count()
    ms, sts = time_steps(g, args.steps)
    dist.barrier()
    clk = clocks.stop()
    launches = g.launch_count() - launches0
    vc = [x[0] for x in sts]
    rs = [x[1] for x in sts]
    fine = [x[2] for x in sts]
    src = [x[3] for x in sts]
    prof = {k: g.profile_read(k) for k in timed_slots}
    for k in timed_slots:
        g.profile_enable(k, False)
    g.profile_sample(1)
    ms_max = dist.max(ms)
    value = dist.world * args.steps / (ms_max / 1e3)
    # --- plain FP64 multigrid over the same step window
    plain = plain_strict = None
    if not args.no_plain and dist.rank == 0:
        plain = plain_arm(args, 2, done)
        plain_strict = plain_arm(args, 0, done)
    tma = tma_arm(args, done) if (not args.no_plain and dist.rank == 0) else None
    acc = accuracy_run(args) if (not args.no_accuracy and dist.rank == 0) else None
    # --- end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        import numpy as np
        fields = (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_P)
        host = {}
        if torch is not None:
            for f in fields:
                t = torch.empty(g.dims(f), dtype=torch.float64, pin_memory=True)
                host[f] = (t, t.data_ptr())
        else:
            for f in fields:
                a = np.empty(g.dims(f))
                host[f] = (a, a.ctypes.data)
        ptrs = [host[f][1] for f in fields]
        g.download_fields_ptr(fields, ptrs)
        h2d = sum(8 * int(np.prod(g.dims(f))) for f in fields)
        d2h = h2d
        steps_e = max(2, min(args.steps, 5))
        g.synchronize()
        t0 = time.perf_counter()
        for k in range(steps_e):
            g.upload_fields_ptr(fields, ptrs)
            s, st = g.time_advance()
            g.download_fields_ptr(fields, ptrs)
        g.synchronize()
        el = dist.max(time.perf_counter() - t0)
        e2e = {"value": dist.world * steps_e / el, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "steps": steps_e, "copies": "Vx, Vy, Vz, P from and into page-locked host memory every step, concurrent copies"}
    # --- rooflines of the timed kernels; the one with the largest share leads
    peak, peak_kind = measured_peak_hbm()
    per_cycle = {"mg_smooth_fp32": p.preSmooth + p.postSmooth, "mg_residual_fp32": 1, "mg_restrict_fp32": 1,
                 "mg_prolong_fp32": 1}
    roofs = []
    for k in timed_slots:
        n_k, ms_k, b_k = prof[k]
        if not n_k:
            continue
        avg_ms = ms_k / n_k
        achieved = (b_k / n_k) / (avg_ms * 1e-3) / 1e9 if avg_ms > 0 else 0.0
        pc = per_cycle.get(names[k])
        n_all = pc * sum(vc) if pc else n_k
        if pc and names[k] == "mg_smooth_fp32":
            n_all -= sum(rs)   # each refinement step's first cycle starts from zero: its first two sweeps are one launch
        roofs.append({"kernel": names[k], "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                      "frac": round(achieved / peak, 4), "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                      "traffic": ncu_traffic(names[k]), "traffic_source": "ncu capture, profiles/ncu_traffic.md",
                      "launches": n_all, "launches_timed": n_k,
                      "timed": "one V-cycle in %d, over the timed region" % PROF_EVERY if pc else "every launch",
                      "avg_ms": round(avg_ms, 4), "share_of_step": round(avg_ms * n_all / ms, 4) if ms > 0 else None})
    roofs.sort(key=lambda r: -(r["share_of_step"] or 0))
    roof = roofs[0] if roofs else None
    out = {
        "metric": METRIC, "value": round(value, 4), "unit": "steps/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic (Taylor-Green initial condition)",
        "config": {
            "workload": "Taylor-Green vortex 257^3 (2^8+1 vertex points per axis), [0,2pi]^3 PPP, Re 1600, dt 5e-4; "
                        "pressure solve: FP32 V(3,3) cycles (Chebyshev-weighted Jacobi smoothing) inside iterative refinement with an "
                        "exact fixed-point residual, refinement steps sized by the measured contraction per cycle, to "
                        "max|b-Ap|/max|b| <= 1e-8; Crank-Nicolson and right-hand side in split-FP64 (fastKernels 2); "
                        "plain arms: FP64 Chebyshev (2,2) cycles with three cycles at the second level a visit, same residual, "
                        "over the same step window",
            "grid": [257, 257, 257], "vcycle_depth": DEPTH, "mg_mode": "mixed_fp32_in_fp64", "fastKernels": p.fastKernels,
            "warm_start": "unet (3-level 16/32/64, tcgen05 BF16 convs) correcting 2 Pp(n-1) - Pp(n-2), "
                          "least-squares step length, fallback to the previous pressure"
                          if args.learned else args.guess,
            "learned": learn,
            "guess_sources_timed": {"previous": src.count(0), "network": src.count(1), "extrapolation": src.count(2),
                                    "quadratic": src.count(3)},
            "steps_before_timed": done,
            "residual_target": TARGET, "vcycles_per_step": sum(vc) / len(vc),
            "refine_steps_per_step": sum(rs) / len(rs), "max_fine_residual": max(fine),
            "plain_fp64": plain,
            "plain_fp64_strict": plain_strict,
            "speedup_vs_plain_fp64": round(value / dist.world / plain["steps_per_s"], 3) if plain else None,
            "speedup_vs_plain_fp64_strict": round(value / dist.world / plain_strict["steps_per_s"], 3) if plain_strict else None,
            "accuracy_vs_plain_fp64": acc,
            "plane_tma_variant": tma,
            "l2": "inputs larger than L2: every FP64 field is 259^3*8 B = 139 MB > 129 MB L2",
            "parallelism": "replicas" if dist.world > 1 else "single GPU",
        },
        "roofline": roof, "roofline_kernels": roofs, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk,
    }
    if dist.rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    g.close()
    return out


def cpu_baseline(budget_s=30.0, ind=GRID_INDEX, depth=DEPTH, vc_cap=2):
    """The oracle (CPU restatement of the reference algorithm) on the host
    cores: one reference time step of the same workload with the V-cycle loop
    capped at `vc_cap` cycles, a bounded sample and a lower bound on the
    reference's CPU step time; and one uncapped step (the reference's own
    stopping rule) of the same workload at 129^3 beside it."""
    from oracle.oracle import Oracle
    from saras_gb300 import _abi as F
    threads = int(os.environ.get("OMP_NUM_THREADS", str(os.cpu_count() or 1)))
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    p = tgv_params(F.MG_REFERENCE, F.GUESS_PREVIOUS, ind, depth)
    p.vcCount = vc_cap
    o = Oracle(p)
    init_tgv(o, p)
    t0 = time.perf_counter()
    s, st = o.time_advance()
    el = time.perf_counter() - t0
    o.close()
    out = {"value": round(1.0 / el, 6), "unit": "steps/s", "cores": threads, "kind": "port", "capped": True,
           "sample": "one reference time step of TGV %d^3 with the V-cycle loop capped at %d cycles (%.1f s on %d threads); "
                     "the cap makes this a lower bound on the reference's step time" % (2 ** ind + 1, vc_cap, el, threads)}
    if budget_s > 0:
        q = tgv_params(F.MG_REFERENCE, F.GUESS_PREVIOUS, ind - 1, depth - 1)
        o = Oracle(q)
        init_tgv(o, q)
        t0 = time.perf_counter()
        s, st = o.time_advance()
        el2 = time.perf_counter() - t0
        o.close()
        out["uncapped_sample"] = {"grid": 2 ** (ind - 1) + 1, "steps_per_s": round(1.0 / el2, 6), "vcycles": st.vcycles,
                                  "seconds": round(el2, 2),
                                  "sample": "the first reference time step of TGV %d^3 with the reference's own V-cycle "
                                            "stopping rule" % (2 ** (ind - 1) + 1)}
    return out


def run_reference(args, dist):
    """The reference algorithm on the host cores: the CPU oracle (the reference
    is C++ with MPI/Blitz++/yaml-cpp/HDF5, none of which is installed, so the
    oracle's strict restatement stands in for it), each step a bounded sample."""
    if dist.rank != 0:
        return None
    from oracle.oracle import Oracle
    from saras_gb300 import _abi as F
    threads = int(os.environ.get("OMP_NUM_THREADS", str(os.cpu_count() or 1)))
    p = tgv_params(F.MG_REFERENCE, F.GUESS_PREVIOUS)
    p.vcCount = 2
    o = Oracle(p)
    init_tgv(o, p)
    for k in range(args.warmup):
        o.time_advance()
    steps = min(args.steps, 20)   # about a second a step on 16 cores: the run stays within a few minutes
    t0 = time.perf_counter()
    for k in range(steps):
        o.time_advance()
    el = time.perf_counter() - t0
    v = steps / el
    return {
        "impl": "reference", "metric": METRIC, "value": round(v, 6), "unit": "steps/s", "n_gpus": dist.world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": round(1e3 * el / steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (Taylor-Green initial condition)",
        "config": {"workload": "Taylor-Green vortex 257^3, Re 1600, dt 5e-4; reference multigrid (Jacobi V(3,3), "
                               "V-cycle loop capped at 2 cycles per step as the bounded sample)",
                   "grid": [257, 257, 257], "implementation": "CPU oracle (strict restatement of the reference), OpenMP"},
        "cpu_baseline": {"value": round(v, 6), "unit": "steps/s", "cores": threads, "kind": "port",
                         "sample": "%d reference steps of TGV 257^3, V-cycle loop capped at 2 cycles" % steps},
        "e2e": {"value": round(v, 6), "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ------------------------------------------------------------------ studies
# Further workloads, run on request (--workload); each prints one JSON line of
# its own: the learned-warm-start and at-scale studies of the same time step,
# the plain method's drop-in configuration, and the 2D validation.  None is the
# headline metric.
def rbc_params(guess, ind=(8, 8, 7), depth=6, dt=5.0e-4):
    """Rayleigh-Benard convection: 257 x 257 x 129 on a 2:2:1 box, periodic
    sides, no-slip top and bottom (T = 1 bottom, 0 top), Ra 1e7, Pr 1; the
    mixed-precision solve with the headline's cycle to the same 1e-8 residual."""
    from saras_gb300 import _abi
    p = _abi.default_params()
    p.probType, p.icType = 5, 0
    p.xPer = p.yPer = 1
    p.zPer = 0
    p.Lx, p.Ly, p.Lz = 2.0, 2.0, 1.0
    p.xInd, p.yInd, p.zInd = ind
    p.vcDepth = depth
    p.Ra, p.Pr, p.rbcType, p.forceType = 1.0e7, 1.0, 2, 3
    p.Re = 1.0
    p.tStp = dt
    p.cnTolerance = 1.0e-8
    p.mgTolerance = 1.0e-8
    p.preSmooth = p.postSmooth = 3
    p.smoother = _abi.SMOOTHER_CHEBYSHEV
    p.coarseCycles = 1
    p.mgMode = _abi.MG_MIXED
    p.mgTarget = TARGET
    p.mgMaxCycles = 100
    p.mixedCycles = 0
    p.jacobiWeight = 6.0 / 7.0
    p.fastKernels = 2
    p.guessMode = guess
    return p


def study_rbc_learned(args):
    """Rayleigh-Benard 257 x 257 x 129, 2000 steps: the first 300 with the
    previous pressure as the guess (the U-Net arms collect training pairs there,
    the last 32 of which are kept), then the U-Net is trained on the GPU and the
    remaining steps run with it (the per-solve selector, and the network in
    every solve), against the same steps with extrapolation and with the
    previous pressure (the solver without the network)."""
    import numpy as np
    import saras_gb300 as S
    from saras_gb300 import _abi as F
    total, warm = args.study_steps or 2000, 300
    arms = {"learned": F.GUESS_LEARNED, "network_every_solve": F.GUESS_NETWORK,
            "extrapolation": F.GUESS_EXTRAPOLATE, "previous_pressure": F.GUESS_PREVIOUS}
    res = {}
    for name, mode in arms.items():
        p = rbc_params(F.GUESS_PREVIOUS)
        g = S.Solver(p)
        g.set(F.FIELD_P, np.ones(g.dims(F.FIELD_P)))
        g.set(F.FIELD_T, S.rbc_temperature(p, seed=42))
        for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ, F.FIELD_T):
            g.apply_bc(f)
        learned = mode in (F.GUESS_LEARNED, F.GUESS_NETWORK)
        if learned:
            g.unet_collect()
        for k in range(warm):
            s, st = g.time_advance()
            if s != 0:
                raise RuntimeError("%s: warm-up step %d failed: %d" % (name, k, s))
        info = {}
        if learned:
            t0 = time.perf_counter()
            info["final_loss"] = g.unet_train(args.train_iters, args.lr)
            g.synchronize()
            info["train_seconds"] = round(time.perf_counter() - t0, 2)
            info["train_iters"] = args.train_iters
        g.set_guess_mode(mode)
        ms, sts = time_steps(g, total - warm)
        vc = np.array([x[0] for x in sts], dtype=float)
        src = [x[3] for x in sts]
        res[name] = dict(info, vcycles_per_step=round(float(vc.mean()), 4),
                         vcycles_per_step_last_1000=round(float(vc[-1000:].mean()), 4),
                         steps_per_s=round(len(sts) / (ms / 1e3), 2), max_fine_residual=max(x[2] for x in sts),
                         guess_sources={"previous": src.count(0), "network": src.count(1), "extrapolation": src.count(2)})
        _, e, d, nu = g.diagnostics()
        res[name]["end_state"] = {"energy": e, "max_div": d, "nusselt": nu}
        g.close()
    base = res["previous_pressure"]["vcycles_per_step"]
    return {"study": "learned warm start, Rayleigh-Benard", "metric": "V-cycles per step (mixed solve to 1e-8)",
            "workload": "Rayleigh-Benard 257x257x129, 2:2:1 box, PPN, Ra 1e7, Pr 1, dt 5e-4, %d steps; guess from step %d on "
                        "(before: previous pressure; U-Net trained on pairs of those steps)" % (total, warm),
            "arms": res,
            "vcycle_reduction_vs_previous_pressure": {k: round(1.0 - v["vcycles_per_step"] / base, 4) for k, v in res.items()},
            "data": "synthetic (linear conduction profile plus seeded uniform perturbation of amplitude 1e-3)"}


def study_tgv513(args):
    """Taylor-Green 513^3, dt 2.5e-4, 200 steps: the learned + mixed solve
    against the plain FP64 solve to the same 1e-8 residual, with the HBM rate of
    the kernels with the largest shares of the mixed arm."""
    import saras_gb300 as S
    from saras_gb300 import _abi as F
    steps = args.study_steps or 200
    out = {}
    for arm in ("learned_mixed", "plain_fp64"):
        mode = F.MG_MIXED if arm == "learned_mixed" else F.MG_PLAIN_TARGET
        p = tgv_params(mode, F.GUESS_PREVIOUS, ind=9, depth=7)
        p.tStp = 2.5e-4
        g = S.Solver(p)
        init_tgv(g, p)
        done = 0
        info = None
        if arm == "learned_mixed":
            g.unet_collect()
            for k in range(args.collect):
                g.time_advance()
            t0 = time.perf_counter()
            loss = g.unet_train(args.train_iters, args.lr)
            g.synchronize()
            info = {"final_loss": loss, "train_seconds": round(time.perf_counter() - t0, 2)}
            g.set_guess_mode(F.GUESS_LEARNED)
            done = args.collect
        else:
            for k in range(args.collect):
                g.time_advance()
            done = args.collect
        names = S.Solver.profile_names()
        for k in range(len(names)):
            g.profile_enable(k, True)
        g.profile_sample(PROF_EVERY)
        ms, sts = time_steps(g, steps - done)
        peak, _ = measured_peak_hbm()
        kern = []
        for k in range(len(names)):
            n_k, ms_k, b_k = g.profile_read(k)
            if n_k and b_k > 0 and ms_k > 0:
                gbs = (b_k / n_k) / ((ms_k / n_k) * 1e-3) / 1e9
                kern.append({"kernel": names[k], "avg_ms": round(ms_k / n_k, 4), "GB/s": round(gbs, 1),
                             "frac_of_measured_hbm": round(gbs / peak, 3), "launches_timed": n_k})
        kern.sort(key=lambda r: -r["avg_ms"] * r["launches_timed"])
        vc = [x[0] for x in sts]
        out[arm] = {"steps_timed": len(sts), "steps_before": done, "ms_per_step": round(ms / len(sts), 3),
                    "steps_per_s": round(len(sts) / (ms / 1e3), 3), "vcycles_per_step": round(sum(vc) / len(vc), 3),
                    "max_fine_residual": max(x[2] for x in sts), "learned": info, "kernels": kern[:8],
                    "timing": "profiling events on (one V-cycle in %d timed)" % PROF_EVERY}
        g.close()
    return {"study": "combined at scale", "metric": "steps/s at 513^3, learned+mixed vs plain FP64 at equal 1e-8 residual",
            "workload": "Taylor-Green 513^3, [0,2pi]^3 PPP, Re 1600, dt 2.5e-4, %d steps" % steps,
            "arms": out, "speedup": round(out["learned_mixed"]["steps_per_s"] / out["plain_fp64"]["steps_per_s"], 3),
            "data": "synthetic (Taylor-Green initial condition)"}


def ldc33_params():
    """The plain method's own configuration: lid-driven cavity in the unit cube,
    33^3 points, 4 multigrid levels, Re 1000, lid Vx = 1 on z = 1, no-slip
    elsewhere, zero initial state (P = 1), dt 1e-3, Crank-Nicolson and damped
    Jacobi V(3,3) cycles to 1e-8: the reference's algorithm (the drop-in mode)."""
    from saras_gb300 import _abi
    p = _abi.default_params()
    p.probType, p.icType = 1, 0
    p.xPer = p.yPer = p.zPer = 0
    p.Lx = p.Ly = p.Lz = 1.0
    p.xInd = p.yInd = p.zInd = 5
    p.vcDepth = 3
    p.Re = 1000.0
    p.tStp = 1.0e-3
    p.cnTolerance = 1.0e-8
    p.mgTolerance = 1.0e-8
    p.preSmooth = p.postSmooth = 3
    p.gsSmooth = 0
    p.vcCount = 200
    p.resType = 1
    return p


def study_ldc33(args):
    """The drop-in (reference algorithm, FP64 throughout) on the cavity at 33^3
    for 200 steps on the GPU, and the same steps of the reference's algorithm on
    the host cores (the oracle, OpenMP) for a bounded sample: steps/s, V-cycles
    and Jacobi iterations per step on both."""
    import numpy as np
    import saras_gb300 as S
    from saras_gb300 import _abi as F
    steps = args.study_steps or 200

    def init(x, p):
        x.set(F.FIELD_P, np.ones(x.dims(F.FIELD_P)))
        for f in (F.FIELD_VX, F.FIELD_VY, F.FIELD_VZ):
            x.apply_bc(f)

    p = ldc33_params()
    g = S.Solver(p)
    init(g, p)
    g.synchronize()
    vc, cn = [], []
    t0 = time.perf_counter()
    for k in range(steps):
        s, st = g.time_advance()
        if s != 0:
            raise RuntimeError("drop-in step failed: %d" % s)
        vc.append(st.vcycles)
        cn.append(sum(st.cn_iters))
    g.synchronize()
    gpu_s = time.perf_counter() - t0
    launches = g.launch_count()
    g.close()
    out = {"study": "plain method, lid-driven cavity 33^3 (the drop-in)", "workload":
           "LDC 33^3, unit cube, Re 1000, dt 1e-3, %d steps, CN Jacobi to 1e-8, Jacobi V(3,3) to 1e-8, FP64 throughout" % steps,
           "gpu": {"steps": steps, "seconds": round(gpu_s, 3), "steps_per_s": round(steps / gpu_s, 3),
                   "vcycles_per_step": round(sum(vc) / steps, 2), "ms_per_vcycle": round(1e3 * gpu_s / max(1, sum(vc)), 4),
                   "cn_iterations_per_step": round(sum(cn) / steps, 2), "launches": launches}}
    if not args.no_cpu:
        from oracle.oracle import Oracle
        o = Oracle(ldc33_params())
        init(o, p)
        n, vco, t0 = 0, [], time.perf_counter()
        while n < steps and time.perf_counter() - t0 < args.cpu_seconds:
            s, st = o.time_advance()
            vco.append(st.vcycles)
            n += 1
        cpu_s = time.perf_counter() - t0
        out["cpu_oracle"] = {"steps": n, "seconds": round(cpu_s, 3), "steps_per_s": round(n / cpu_s, 3),
                             "vcycles_per_step": round(sum(vco) / max(1, n), 2), "cores": os.cpu_count(),
                             "kind": "port", "same_counts_as_gpu": vco == vc[:n]}
    return out


def ldc2d_params(ind=6):
    """The reference's 2D cavity check (its tests/ldcTest input): Re 1000, unit
    square in x-z ("Y Index" 0), lid Vx = 1 on z = 1, Gauss-Seidel V(2,2) cycles
    on five levels, at most 7 a step, multigrid and Jacobi tolerances 1e-6, the
    CFL time step (Courant number 0.1) capped at 1e-3, to t = 50; here on 65 x 65
    points (X and Z Index 6) where the check uses 129 x 129."""
    from saras_gb300 import _abi
    p = _abi.default_params()
    p.probType, p.icType = 1, 0
    p.xPer = p.yPer = p.zPer = 0
    p.Lx = p.Ly = p.Lz = 1.0
    p.xInd, p.yInd, p.zInd = ind, 0, ind
    p.vcDepth = 4
    p.Re = 1000.0
    p.tStp, p.tMax = 1.0e-3, 50.0
    p.useCFL, p.courantNumber = 1, 0.1
    p.cnTolerance = p.mgTolerance = 1.0e-6
    p.gsSmooth, p.preSmooth, p.postSmooth = 1, 2, 2
    p.vcCount = 7
    p.resType = 1
    p.ioCnt = 1000
    return p


def study_ldc2d_ghia(args):
    """The 2D cavity at Re 1000 to t = 50 (the drop-in's 2D solver), then its
    centre-line profiles -- u along x = 0.5 against the height, w along z = 0.5
    against x -- against Ghia, Ghia and Shin (1982) as the reference ships them
    (tests/golden/ghia_re1000.npz, made by tests/golden/make_ghia.py)."""
    import numpy as np
    import saras_gb300 as S
    from saras_gb300 import _abi as F
    p = ldc2d_params(args.grid_index)
    if args.study_steps:
        p.tMax = args.study_steps * p.tStp
    h = S.hydro_d3(p)
    g = h.solver
    vc = []
    t0 = time.perf_counter()
    series = h.solvePDE(on_step=lambda hh, st: vc.append(st.vcycles))
    secs = time.perf_counter() - t0
    ghia = np.load(os.path.join(ROOT, "tests", "golden", "ghia_re1000.npz"))
    xc, xs = g.grid_coords(0, False), g.grid_coords(0, True)
    zc, zs = g.grid_coords(2, False), g.grid_coords(2, True)
    Vx, Vz = g.get(F.FIELD_VX)[:, 1, :], g.get(F.FIELD_VZ)[:, 1, :]
    # Vx: cell centres along x, vertices along z; Vz: vertices along x, cell centres along z
    u_line = np.array([np.interp(0.5, xc, Vx[:, k]) for k in range(Vx.shape[1])])
    w_line = np.array([np.interp(0.5, zc, Vz[i, :]) for i in range(Vz.shape[0])])
    u = np.interp(ghia["z"], zs, u_line)
    w = np.interp(ghia["x"], xs, w_line)
    du, dw = u - ghia["u"], w - ghia["w"]
    return {"study": "2D lid-driven cavity against Ghia et al. (the reference's ldcTest check)",
            "workload": "2D LDC Re 1000, %d x %d, Gauss-Seidel V(2,2) <= 7 cycles a step, tolerances 1e-6, CFL 0.1 capped "
                        "at dt 1e-3, to t = %g" % (2 ** p.xInd + 1, 2 ** p.zInd + 1, p.tMax),
            "steps": h.timeStepCount, "time": round(h.time, 6), "seconds": round(secs, 2),
            "steps_per_s": round(h.timeStepCount / secs, 1), "vcycles_per_step": round(sum(vc) / max(1, len(vc)), 2),
            "energy_last": series[-1][1], "max_divergence_last": series[-1][2],
            "u_centre_line": {"max_abs_dev": round(float(np.max(np.abs(du))), 4), "rms_dev": round(float(np.sqrt(np.mean(du ** 2))), 4),
                              "min_u": round(float(u_line.min()), 4), "ghia_min_u": float(ghia["u"].min())},
            "w_centre_line": {"max_abs_dev": round(float(np.max(np.abs(dw))), 4), "rms_dev": round(float(np.sqrt(np.mean(dw ** 2))), 4),
                              "max_w": round(float(w_line.max()), 4), "min_w": round(float(w_line.min()), 4),
                              "ghia_max_w": float(ghia["w"].max()), "ghia_min_w": float(ghia["w"].min())},
            "profiles": {"z": ghia["z"].tolist(), "u": [round(float(a), 5) for a in u],
                         "x": ghia["x"].tolist(), "w": [round(float(a), 5) for a in w]}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=250)   # about 1 s timed: ten nvidia-smi clock samples (100 ms apart)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--guess", default="learned", choices=["learned", "extrapolate", "quadratic", "previous"],
                    help="initial guess of the pressure-correction solve in the timed steps")
    ap.add_argument("--collect", type=int, default=14)
    ap.add_argument("--train-iters", type=int, default=200)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--accuracy-steps", type=int, default=500)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=30.0)
    ap.add_argument("--workload", default="tgv257", choices=["tgv257", "rbc_learned", "tgv513", "ldc33", "ldc2d_ghia"],
                    help="tgv257: the headline line; rbc_learned, tgv513, ldc33, ldc2d_ghia: the learned, at-scale, "
                         "drop-in and 2D validation studies")
    ap.add_argument("--study-steps", type=int, default=0, help="total steps of a study (0: its configured count)")
    ap.add_argument("--grid-index", type=int, default=6, help="ldc2d_ghia: X and Z Index (6: 65 x 65, 5: 33 x 33)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    args.learned = args.guess == "learned"
    if args.workload != "tgv257":
        study = {"rbc_learned": study_rbc_learned, "tgv513": study_tgv513, "ldc33": study_ldc33,
                 "ldc2d_ghia": study_ldc2d_ghia}[args.workload]
        print(json.dumps(study(args)), flush=True)
        return
    dist = Dist()
    try:
        out = run_reference(args, dist) if args.impl == "reference" else run_ours(args, dist)
        if dist.rank == 0 and out is not None:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
