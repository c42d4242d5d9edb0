"""Benchmark of the implicit edge-based residual path on GB300.

A step is one residual evaluation of the NewtonIterate sequence
(UpdateBCs, LSQ gradient, modified-Venkatakrishnan limiter, Roe + viscous
edge fluxes, boundary fluxes, residual gather and norms) on the second-order
laminar Navier-Stokes workload: a 128x96x96-node jittered Kuhn-tet box,
1,179,648 nodes, 8,123,007 interior edges.  The metric is edge-flux
throughput, Medges/s = interior edges / step time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line on rank 0.  Under torchrun each rank runs an independent
replica of the workload on its own GPU (the path does not shard; replicas
only) and the slowest rank's time is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Edge-flux Medges/s; wall-time to 1e-10 residual drop, mixed/learned vs FP64"
UNIT = "Medges/s"
WORKLOADS = {
    "ns128": dict(nx=128, ny=96, nz=96),
    "ns64": dict(nx=64, ny=48, nz=48),
    "ns256": dict(nx=256, ny=176, nz=176),
}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as td
        td.init_process_group("gloo")
        pg = td
    return ws, rank, local, pg


def barrier(pg):
    if pg:
        pg.barrier()


def max_over_ranks(pg, x):
    if not pg:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def replica_value(ws, units_per_rank, slowest_ms_per_step):
    """Whole-job throughput in M units/s: every replica's units over the
    slowest rank's step time."""
    return ws * units_per_rank / (slowest_ms_per_step * 1e-3) / 1e6


# The CPU baseline's bounded sample of the workload family: a box of the
# same generator, clustering and boundary conditions, small enough that
# every host thread evaluates its own residual within a second or so.
CPU_SAMPLE_DIMS = (64, 44, 44)


def product_loaded():
    """Whether this process has mapped the product library (it must not, in
    the reference arm)."""
    try:
        return "libpcfd.so" in Path("/proc/self/maps").read_text()
    except OSError:
        return None


def cpu_sample(budget_s=15.0, threads=1, dims=CPU_SAMPLE_DIMS):
    """The oracle - a C restatement of the reference path, bit-identical to
    it on the reference's own outputs - timed on the host cores: each thread
    runs whole residual evaluations (boundary update, LSQ gradient, limiter,
    fluxes, norms) of the sample box, built by the oracle's own mesh
    generator (nothing of the product is loaded).  Returns (baseline dict,
    seconds, evaluations)."""
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_lib import OracleMesh, OracleSpace
    from proteuscfd_gb300 import cases
    case = cases.ns_flatplate(*dims)
    m = OracleMesh.box(dims[0], dims[1], dims[2], **case.mesh_kw)
    O = OracleSpace(m, case.param)
    nrows = m.nnode + m.nbedge
    q0 = cases.perturbed_state(O.qinf(), nrows, seed=1)
    from concurrent.futures import ThreadPoolExecutor
    done = 0
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        while time.perf_counter() - t0 < budget_s or done == 0:
            list(ex.map(lambda _: O.full(q0), range(threads)))
            done += threads
    dt = time.perf_counter() - t0
    return {"value": done * m.nedge / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d second-order NS residual evaluations (UpdateBCs, LSQ gradient, limiter, Roe + viscous "
                      "fluxes, norms) of the %dx%dx%d box of the same family (%d edges) by the oracle, %d "
                      "thread(s) each evaluating its own, %.1f s" % (done, dims[0], dims[1], dims[2], m.nedge,
                                                                      threads, dt)}, dt, done


def run_reference(args, rank, pg):
    """--impl reference: the reference's CPU path - the oracle port, which is
    bit-identical to the reference's own residual on its outputs (the
    reference itself needs HDF5/MPI/METIS and its source tree, absent on the
    machines the benchmark runs on) - on all host threads, rank 0 only, over a bounded sample of the
    workload; the process loads nothing of the product."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    w = WORKLOADS[args.workload]
    cpu_sample(0.0, threads)  # warm-up: page in, one round per thread
    base, dt, done = cpu_sample(max(5.0, 1.0 * args.steps), threads)
    rounds = max(done // threads, 1)
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / rounds,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "ns_flatplate %dx%dx%d (second-order laminar NS residual, Mach 0.8, Re 1e5); "
                                   "CPU sample: the %dx%dx%d box of the same family" % (
                                       w["nx"], w["ny"], w["nz"], *CPU_SAMPLE_DIMS)},
            "cpu_baseline": base,
            "product_library_loaded": product_loaded(),
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# The convergence study.  Every arm starts from the same state: a shared
# start-up of CONV_PREFIX["steps"] plain FP64 steps (first order, then second
# order with the limiter live, CFL ramped from 1 to 20) that ends with the
# limiter frozen (limiterFreeze, ucs/solutionSpace.tcc:681).  From there all
# arms solve the same discrete equations with the same frozen limiter, and
# differ only in the linear solve and its arithmetic; the Newton residual,
# gradients, limiter and norms stay FP64 in every arm.  Each arm ramps its
# CFL linearly from the start-up's 20 to its own over CONV_RAMP steps.  (On
# the 256x176x176 box a start-up ramping to 50 diverged within a few steps of
# the switch to second order; ramping to 20 does not.)
#   fp64:  the reference's method, block-SGS sweeps on the FP64 Jacobian; 30
#          sweeps at CFL 1000 were the fastest of the settings tried on the
#          128x96x96 box (10 sweeps at CFL 200, 20 at CFL 1000, 30 at CFL 3000
#          were slower or stalled)
#   mixed: FP32 Jacobian (differences in double-float), FGMRES(30)
#          right-preconditioned by two FP32 SGS sweeps, stopped at a 0.1
#          reduction of the linear residual (an inexact-Newton forcing term),
#          CFL 1000
#   mixed_bf16: the same with BF16 off-diagonal storage (FP32 accumulation)
#   mixed_learned: mixed with the learned correction on the first Krylov
#          direction of each cycle (the residual itself, the right-hand side
#          the network is trained on)
#   mixed_learned_aug: mixed with the learned vector of each cycle's residual
#          direction as the cycle's second direction, after plain SGS of it
CONV_PREFIX = dict(steps=100, cfl=20.0, cfl_start=1.0, cfl_ramp_steps=60, nsgs=10, first_order_steps=20,
                   linear_solver=0, jac_precision=0)
CONV_RAMP = 50
_MIXED = dict(nsgs=2, linear_solver=1, fgmres_m=30, fgmres_restarts=1, fgmres_rtol=0.1, jac_precision=1,
              first_order_steps=20)
CONV_ARMS = {
    "fp64": dict(cfl=1000.0, nsgs=30, linear_solver=0, jac_precision=0, first_order_steps=20),
    "fp64_s20": dict(cfl=1000.0, nsgs=20, linear_solver=0, jac_precision=0, first_order_steps=20),
    "mixed": dict(_MIXED, cfl=1000.0),
    "mixed_s1": dict(_MIXED, cfl=300.0, nsgs=1),
    "mixed_bf16": dict(_MIXED, cfl=1000.0, jac_precision=2),
    "mixed_learned": dict(_MIXED, cfl=1000.0, linear_solver=2, lp_directions=1),
    "mixed_learned_aug": dict(_MIXED, cfl=1000.0, linear_solver=3),
}


def flatplate(dims, seed=2, mach=None, aoa_deg=0.0, Re=None):
    """The convergence family's case (cases.ns_flatplate) at other flow
    conditions: Mach, angle of attack in the x-y plane, Reynolds number."""
    from proteuscfd_gb300 import cases
    case = cases.ns_flatplate(*dims, seed=seed)
    if mach is not None:
        case.param.mach = mach
    if Re is not None:
        case.param.Re = Re
    a = np.radians(aoa_deg)
    case.param.flowdir = (float(np.cos(a)), float(np.sin(a)), 0.0)
    return case


def train_learned(dims, nruns, steps, every, epochs, lr, seed=1000):
    """Training of the learned preconditioner on pairs the plain mixed solver
    generates.  Each run draws a flow (Mach ~ U[0.5, 2], angle of attack ~
    U[-5, 5] degrees, Re ~ log-U[1e4, 1e6]) on a box of the family with its
    own mesh and state seeds (none is the study's), runs the mixed method
    from the perturbed freestream through the study's schedule (CFL ramped
    to 20 over the start-up, limiter frozen at its end, then ramped to the
    arms' CFL), and every `every` steps after the start-up stores the pair
    (residual, Newton update solved to 1e-6) with its first Krylov pairs.
    The network trains on each run's pairs in turn (Adam), carrying its
    parameters from run to run.  A run whose state stops being finite
    contributes the pairs it stored before."""
    from proteuscfd_gb300 import SolutionSpace, cases
    rng = np.random.default_rng(seed)
    w, runs, t0 = None, [], time.perf_counter()
    for r in range(nruns):
        mach = float(rng.uniform(0.5, 2.0))
        aoa = float(rng.uniform(-5.0, 5.0))
        Re = float(10.0 ** rng.uniform(4.0, 6.0))
        case = flatplate(dims, seed=seed + 2 * r + 1, mach=mach, aoa_deg=aoa, Re=Re)
        m = cases.build_mesh(case)
        S = SolutionSpace(m, case.param)
        S.set_state(cases.perturbed_state(S.qinf(), m.nnode + m.nbedge, seed + 2 * r + 2))
        S.lp_init(1)
        if w is not None:
            S.lp_set_params(w)
        npairs, ok = 0, True
        P = CONV_PREFIX["steps"]
        for it in range(steps):
            if it < P:
                opts = dict(_MIXED, cfl=CONV_PREFIX["cfl"], cfl_start=CONV_PREFIX["cfl_start"],
                            cfl_ramp_steps=CONV_PREFIX["cfl_ramp_steps"])
            else:
                c0, c1 = CONV_PREFIX["cfl"], CONV_ARMS["mixed"]["cfl"]
                opts = dict(_MIXED, cfl=c0 + (c1 - c0) * min(1.0, (it - P + 1) / CONV_RAMP))
            rep = S.newton_iterate(it, limiter_freeze=P, **opts)
            if not np.isfinite(rep["res"][0]):
                ok = False
                break
            if it >= P and (it - P) % every == 0:
                try:
                    npairs = S.lp_collect(nsgs=_MIXED["nsgs"], rtol=1e-6, krylov_pairs=2)
                except Exception as exc:  # a linear system the solve cannot reach 1e-6 on
                    ok = "collect: %s" % exc
                    break
        rec = {"mach": round(mach, 3), "aoa_deg": round(aoa, 2), "Re": round(Re), "pairs": npairs, "finite": ok}
        if npairs:
            l0, l1 = S.lp_train(epochs=epochs, lr=lr)
            w = S.lp_get_params()
            rec.update(loss_first_epoch=l0, loss_last_epoch=l1)
        runs.append(rec)
        S.close()
    return w, {"mesh": "%dx%dx%d" % dims, "runs": runs, "pairs": sum(x["pairs"] for x in runs),
               "epochs_per_run": epochs, "lr": lr, "train_s": round(time.perf_counter() - t0, 2)}


def converge_study(args):
    """Wall time to a 1e-10 drop of resGlobal on one GPU, per arm, from the
    shared start-up; each arm's final field and body force (pressure plus
    viscous, FORCE_Kernel) against the FP64 arm's."""
    from proteuscfd_gb300 import SolutionSpace, cases
    from proteuscfd_gb300 import _native as N
    w = WORKLOADS[args.converge_workload]
    dims = (w["nx"], w["ny"], w["nz"])
    case = flatplate(dims)
    walls = [t for t, b in case.param.bc_type.items() if b == N.BC_NOSLIP]
    t0 = time.perf_counter()
    m = cases.build_mesh(case)
    out = {"workload": "ns_flatplate %dx%dx%d (mesh seed 2, state seed 1), second order, Mach 0.8, Re 1e5, "
                       "modified Venkatakrishnan K=%g" % (dims + (case.param.venkat_K,)),
           "nodes": m.nnode, "edges": m.nedge, "mesh_build_s": round(time.perf_counter() - t0, 2),
           "target_drop": 1e-10, "time_cap_s": args.converge_cap, "arms": {}}
    lp_w = None
    if "mixed_learned" in args.converge_arms:
        tdims = WORKLOADS[args.learned_train_workload]
        lp_w, out["learned_training"] = train_learned((tdims["nx"], tdims["ny"], tdims["nz"]), args.learned_runs,
                                                      CONV_PREFIX["steps"] + 60, 10, 30, 2e-3)
    # the shared start-up
    P = CONV_PREFIX["steps"]
    S = SolutionSpace(m, case.param)
    S.set_state(cases.perturbed_state(S.qinf(), m.nnode + m.nbedge, 1))
    N.check(N.load().pcfd_device_sync(), "sync")
    t0 = time.perf_counter()
    hist = []
    for it in range(P):
        opts = {k: v for k, v in CONV_PREFIX.items() if k != "steps"}
        hist.append(S.newton_iterate(it, limiter_freeze=P, **opts)["res"][0])
    t_pre = time.perf_counter() - t0
    r0 = hist[0]
    q_pre, lim_pre = S.get_state(), S.get_limiter()
    S.close()
    out["startup"] = {"steps": P, "wall_s": round(t_pre, 3), "drop": hist[-1] / r0, "opts": CONV_PREFIX}
    print(json.dumps({"startup": out["startup"], "nodes": m.nnode}), file=sys.stderr, flush=True)
    finals = {}
    for name in args.converge_arms:
        arm = CONV_ARMS[name]
        S = SolutionSpace(m, case.param)
        S.set_state(q_pre)
        S.set_limiter(lim_pre)
        if arm["linear_solver"] >= 2:
            S.lp_init(1)
            if lp_w is not None:
                S.lp_set_params(lp_w)
        N.check(N.load().pcfd_device_sync(), "sync")
        h, t_at, lin, fb = [], {}, 0, 0
        t0 = time.perf_counter()
        it = P
        while True:
            c0, c1 = CONV_PREFIX["cfl"], arm["cfl"]
            cfl = c0 + (c1 - c0) * min(1.0, (it - P + 1) / CONV_RAMP)
            rep = S.newton_iterate(it, limiter_freeze=P, **dict(arm, cfl=cfl))
            it += 1
            r = rep["res"][0] / r0
            h.append(r)
            lin += rep["lin_iters"]
            fb += rep["lp_fallbacks"]
            el = time.perf_counter() - t0
            for d in (1e-4, 1e-6, 1e-8, 1e-10):
                if d not in t_at and r <= d:
                    t_at[d] = [P + len(h), round(t_pre + el, 3)]
            if len(h) % 25 == 0:
                # progress on stderr, so a run cut short still leaves its history
                print(json.dumps({"arm": name, "step": P + len(h), "drop": r, "wall_s": round(el, 2),
                                  "lin": rep["lin_iters"]}), file=sys.stderr, flush=True)
            if not np.isfinite(r) or r <= 1e-10 or el > args.converge_cap or len(h) >= args.converge_iters:
                break
        wall = time.perf_counter() - t0
        fp, fv = S.forces(walls)
        finals[name] = (S.get_state()[:m.nnode, :5].copy(), np.r_[fp, fv])
        # where a late step's time goes: three more steps with a CUDA event
        # pair around every launch (after the timed run and its final field)
        S.profile(True)
        S.profile_reset()
        for k in range(3):
            S.newton_iterate(it + k, limiter_freeze=P, **dict(arm, cfl=cfl))
        tm = S.timers()
        S.profile(False)
        rec = {"steps_after_startup": len(h), "wall_s_after_startup": round(wall, 3),
               "wall_s_total": round(t_pre + wall, 3), "drop": h[-1], "reached_1e-10": 1e-10 in t_at,
               "steps_s_to_drop": {str(k): v for k, v in t_at.items()},
               "linear_iters_per_step": lin / len(h), "ms_per_step": 1e3 * wall / len(h),
               "opts": arm, "health": S.health(),
               "late_step_ms_by_kernel_group": {k: round(v[0] / 3, 3) for k, v in tm.items() if v[1]}}
        if fb:
            rec["sgs_fallbacks"] = fb
        if not np.isfinite(h[-1]):
            rec["stopped"] = "non-finite residual"
        out["arms"][name] = rec
        print(json.dumps({"arm_done": name, "rec": rec}), file=sys.stderr, flush=True)
        S.close()
    ref = "fp64" if "fp64" in finals else None
    if ref:
        qref, fref = finals[ref]
        drag_ref = fref[0] + fref[3]
        for name, (qa, fa) in finals.items():
            rec = out["arms"][name]
            rec["force_pressure"] = [float(v) for v in fa[:3]]
            rec["force_viscous"] = [float(v) for v in fa[3:]]
            if name == ref:
                continue
            rec["field_rel_l2_vs_fp64"] = float(np.linalg.norm(qa - qref) / np.linalg.norm(qref))
            rec["force_rel_err_vs_fp64"] = float(np.linalg.norm(fa - fref) / np.linalg.norm(fref))
            rec["drag_rel_err_vs_fp64"] = float(abs(fa[0] + fa[3] - drag_ref) / abs(drag_ref))
            if rec["reached_1e-10"] and out["arms"][ref]["reached_1e-10"]:
                rec["speedup_vs_fp64"] = out["arms"][ref]["wall_s_total"] / rec["wall_s_total"]
                rec["speedup_vs_fp64_after_startup"] = (out["arms"][ref]["wall_s_after_startup"] /
                                                        rec["wall_s_after_startup"])
    return out


def chemistry_study(args):
    """Finite-rate chemistry of the reacting workload: the 5-species air
    mechanism's production rates on 2,007,040 nodes (the reacting box's node
    count), inputs resident in HBM, device time by CUDA events; the host-API
    form with its copies; the oracle on a host sample."""
    import torch
    sys.path.insert(0, str(ROOT / "tests"))
    from chem_cases import mechanism, states
    from oracle_lib import chem_rates
    from proteuscfd_gb300.chem import ChemModel, model_struct
    spec = mechanism()
    n = 2007040
    rho, T = states(n, seed=5, tmin=300.0, tmax=8000.0)
    c = ChemModel(spec)
    d_rho = torch.from_numpy(rho).cuda()
    d_T = torch.from_numpy(T).cuda()
    d_w = torch.empty_like(d_rho)
    for _ in range(3):
        c.production_rates_dev(n, d_rho.data_ptr(), d_T.data_ptr(), d_w.data_ptr())
    ms = [c.production_rates_dev(n, d_rho.data_ptr(), d_T.data_ptr(), d_w.data_ptr()) for _ in range(args.steps)]
    ms_avg = float(np.mean(ms))
    # host API with pinned host buffers (copies in, rates out)
    rho_h = torch.empty(rho.shape, dtype=torch.float64, pin_memory=True).numpy()
    T_h = torch.empty(T.shape, dtype=torch.float64, pin_memory=True).numpy()
    w_h = torch.empty(rho.shape, dtype=torch.float64, pin_memory=True).numpy()
    rho_h[:] = rho
    T_h[:] = T
    c.production_rates(rho_h, T_h, out=w_h)
    t0 = time.perf_counter()
    k = 3
    for _ in range(k):
        c.production_rates(rho_h, T_h, out=w_h)
    e2e = (time.perf_counter() - t0) / k
    ns = 20000
    t0 = time.perf_counter()
    chem_rates(model_struct(spec), rho[:ns], T[:ns])
    tcpu = time.perf_counter() - t0
    # the FP64 temperature Newton of ConservativeToNative on the same node
    # count: device arrays, a stale stored pressure (x1.3) as the start
    from chem_cases import fr_states
    from oracle_lib import OracleChemState
    ref, frho, vel, fT = fr_states(n, seed=6)
    P, _, _ = c.aux(ref, frho, fT)
    qm = c.native_to_conservative(ref, frho, np.c_[vel, fT], P)
    q = np.ascontiguousarray(np.c_[frho, qm])
    d_q = torch.from_numpy(q).cuda()
    d_P = torch.from_numpy(P * 1.3).cuda()
    d_out = torch.empty((n, 4), dtype=torch.float64, device="cuda")
    for _ in range(3):
        c.conservative_to_native_dev(ref, n, d_q.data_ptr(), d_P.data_ptr(), d_out.data_ptr())
    t0 = time.perf_counter()
    for _ in range(args.steps):
        c.conservative_to_native_dev(ref, n, d_q.data_ptr(), d_P.data_ptr(), d_out.data_ptr())
    tn_ms = (time.perf_counter() - t0) / args.steps * 1e3
    tn_err = float(np.abs(d_out[:, 3].cpu().numpy() - fT).max() / fT.max())
    nsn = 20000
    O = OracleChemState(model_struct(spec), ref)
    t0 = time.perf_counter()
    O.c2n_batch(q[:nsn], P[:nsn] * 1.3)
    tn_cpu = time.perf_counter() - t0
    # the reacting inviscid edge flux (HLLC) over the edges of the
    # 160x112x112 box (2,007,040 nodes), device arrays
    from proteuscfd_gb300 import Mesh
    from chem_cases import fr_records
    mesh = Mesh.box(160, 112, 112, jitter=0.2, seed=2)
    ne = mesh.nedge
    ea = np.asarray(mesh.edge_area)
    avec = np.ascontiguousarray(ea)
    recs = c.node_records(ref, frho, vel, fT)
    d_rec = torch.from_numpy(recs).cuda()
    d_e = torch.from_numpy(np.ascontiguousarray(np.asarray(mesh.edges, dtype=np.int32))).cuda()
    d_a = torch.from_numpy(avec).cuda()
    d_f = torch.empty((ne, len(spec["species"]) + 4), dtype=torch.float64, device="cuda")
    fopts = c.flux_opts(1.0, 0.0, 0)
    for _ in range(3):
        c.hllc_flux_dev(ref, fopts, n, d_rec.data_ptr(), ne, d_e.data_ptr(), d_a.data_ptr(), d_f.data_ptr())
    t0 = time.perf_counter()
    for _ in range(args.steps):
        c.hllc_flux_dev(ref, fopts, n, d_rec.data_ptr(), ne, d_e.data_ptr(), d_a.data_ptr(), d_f.data_ptr())
    hl_ms = (time.perf_counter() - t0) / args.steps * 1e3
    nse = 20000
    t0 = time.perf_counter()
    O.hllc_batch(fopts, recs, np.asarray(mesh.edges[:nse], dtype=np.int32), avec[:nse])
    hl_cpu = time.perf_counter() - t0
    # the first-order reacting residual on that box (fluxes, boundary
    # half-edges against phantom records, gather, chemistry source, norms)
    c.attach_mesh(mesh)
    nb = mesh.nbedge
    prow = np.random.default_rng(7).integers(0, n, size=nb)
    d_qall = torch.from_numpy(np.ascontiguousarray(np.r_[recs, recs[prow]])).cuda()
    d_b = torch.empty((n, len(spec["species"]) + 4), dtype=torch.float64, device="cuda")
    ref_time = 1.0e-4
    for _ in range(3):
        c.residual_dev(ref, fopts, ref_time, 1, d_qall.data_ptr(), d_b.data_ptr())
    t0 = time.perf_counter()
    for _ in range(args.steps):
        c.residual_dev(ref, fopts, ref_time, 1, d_qall.data_ptr(), d_b.data_ptr())
    rs_ms = (time.perf_counter() - t0) / args.steps * 1e3
    # the source-term Jacobian (one-sided differences of the chemistry source,
    # one 9x9 block per node) on the same node records, device arrays
    nq = len(spec["species"]) + 4
    d_vol = torch.ones(n, dtype=torch.float64, device="cuda")
    d_A = torch.empty((n, nq, nq), dtype=torch.float64, device="cuda")
    for _ in range(3):
        c.source_jacobian_dev(ref, ref_time, n, d_rec.data_ptr(), d_vol.data_ptr(), d_A.data_ptr())
    t0 = time.perf_counter()
    for _ in range(args.steps):
        c.source_jacobian_dev(ref, ref_time, n, d_rec.data_ptr(), d_vol.data_ptr(), d_A.data_ptr())
    sj_ms = (time.perf_counter() - t0) / args.steps * 1e3
    nsj = 5000
    t0 = time.perf_counter()
    O.source_jacobian(recs[:nsj], np.ones(nsj), ref_time)
    sj_cpu = time.perf_counter() - t0
    # the native-variable temporal terms added in place into those blocks
    rng = np.random.default_rng(9)
    d_dtau = torch.from_numpy(rng.uniform(1e-3, 1e-1, size=n)).cuda()
    d_beta = torch.from_numpy(rng.uniform(0.2, 1.0, size=n)).cuda()
    for _ in range(3):
        c.temporal_terms_dev(ref, n, d_rec.data_ptr(), d_vol.data_ptr(), d_dtau.data_ptr(), d_beta.data_ptr(), 1.0,
                             0.0, 0, d_A.data_ptr())
    t0 = time.perf_counter()
    for _ in range(args.steps):
        c.temporal_terms_dev(ref, n, d_rec.data_ptr(), d_vol.data_ptr(), d_dtau.data_ptr(), d_beta.data_ptr(), 1.0,
                             0.0, 0, d_A.data_ptr())
    tt_ms = (time.perf_counter() - t0) / args.steps * 1e3
    c.close()
    return {"workload": "5-species air, 6 reactions (chemModels/5speciesAir.rxn), %d nodes, T 300-8000 K" % n,
            "mnodes_per_s": n / (ms_avg * 1e-3) / 1e6, "ms": ms_avg,
            "e2e_mnodes_per_s": n / e2e / 1e6,
            "cpu_baseline": {"mnodes_per_s": ns / tcpu / 1e6, "cores": 1, "kind": "port",
                             "sample": "%d nodes by the oracle, 1 thread" % ns},
            "hllc_flux": {
                "what": "CompressibleFREqnSet::HLLCFlux over the %d edges of the 160x112x112 box (%d node records, "
                        "random states as above), FP64; wall time of the device-array call" % (ne, n),
                "ms": hl_ms, "medges_per_s": ne / (hl_ms * 1e-3) / 1e6,
                "cpu_baseline": {"medges_per_s": nse / hl_cpu / 1e6, "cores": 1, "kind": "port",
                                 "sample": "%d edges by the oracle, 1 thread" % nse}},
            "reacting_residual": {
                "what": "first-order inviscid residual of the reacting set with chemistry source on the 160x112x112 "
                        "box: %d edges, %d boundary half-edges, %d nodes; wall time of the device-array call" % (
                            ne, nb, n),
                "ms": rs_ms, "medges_per_s": ne / (rs_ms * 1e-3) / 1e6},
            "temporal_terms": {
                "what": "ContributeTemporalTerms: native-variable temporal terms with beta preconditioning added in "
                        "place into %d %dx%d blocks; wall time of the device-array call" % (n, nq, nq),
                "ms": tt_ms, "mnodes_per_s": n / (tt_ms * 1e-3) / 1e6},
            "source_jacobian": {
                "what": "SourceTermJacobian: one-sided differences of the chemistry source, a %dx%d block per node, "
                        "%d nodes (records as above); wall time of the device-array call" % (nq, nq, n),
                "ms": sj_ms, "mnodes_per_s": n / (sj_ms * 1e-3) / 1e6,
                "cpu_baseline": {"mnodes_per_s": nsj / sj_cpu / 1e6, "cores": 1, "kind": "port",
                                 "sample": "%d nodes by the oracle, 1 thread" % nsj}},
            "temperature_newton": {
                "what": "ConservativeToNative: FP64 temperature Newton from total energy, %d nodes, 250-6000 K, "
                        "stored pressure x1.3 as the start; wall time of the device-array call" % n,
                "ms": tn_ms, "mnodes_per_s": n / (tn_ms * 1e-3) / 1e6, "max_rel_T_error": tn_err,
                "cpu_baseline": {"mnodes_per_s": nsn / tn_cpu / 1e6, "cores": 1, "kind": "port",
                                 "sample": "%d nodes by the oracle, 1 thread" % nsn}}}


def run_gb300(args, ws, rank, local, pg):
    from proteuscfd_gb300 import Mesh, SolutionSpace, cases
    from proteuscfd_gb300 import _native as N
    lib = N.load()
    N.check(lib.pcfd_set_device(local), "pcfd_set_device")
    w = WORKLOADS[args.workload]
    case = cases.ns_flatplate(w["nx"], w["ny"], w["nz"])
    t_mesh = time.perf_counter()
    m = cases.build_mesh(case)
    t_mesh = time.perf_counter() - t_mesh
    S = SolutionSpace(m, case.param)
    nrows = m.nnode + m.nbedge
    q0 = cases.perturbed_state(S.qinf(), nrows, seed=1)

    def timed(arith):
        """K device-timed steps of the residual in the given arithmetic."""
        S.set_residual_arithmetic(arith)
        S.set_state(q0)
        S.bench_residual_full(max(args.warmup, 3))
        barrier(pg)
        N.check(lib.pcfd_device_sync(), "sync")
        l0 = S.launch_count()
        with ClockSampler(local) as clk:
            ms, norms = S.bench_residual_full(args.steps)
        launches = S.launch_count() - l0
        barrier(pg)
        return max_over_ranks(pg, ms), norms, launches, clk

    # the headline is the reference's arithmetic, FP64; the double-float
    # kernels (FP32 pairs on the FP32 pipes, ~48-bit significand) are
    # reported beside it
    results = {0: timed(0)}
    if args.arith != "f64":
        results[1] = timed(1)
    ms, norms, launches, clk = results[0]
    S.set_residual_arithmetic(0)
    ms_per_step = ms / args.steps
    value = replica_value(ws, m.nedge, ms_per_step)

    def kernel_times(arith, nprof=3):
        """per-kernel device times (events around each launch on the
        library's stream) over nprof evaluations in the given arithmetic"""
        S.set_residual_arithmetic(arith)
        S.set_state(q0)
        S.profile(True)
        S.profile_reset()
        for _ in range(nprof):
            S.residual_full()
        t = S.timers()
        S.profile(False)
        tot = sum(v[0] for v in t.values() if v[1]) or 1.0
        return {k: {"ms_per_step": v[0] / nprof, "launches_per_step": v[1] / nprof, "share": v[0] / tot}
                for k, v in t.items() if v[1]}

    kernels = kernel_times(0)
    kernels_df = kernel_times(1) if 1 in results else None
    S.set_residual_arithmetic(0)

    # end to end through the C ABI with host buffers in pinned memory: H2D of
    # q, the step, D2H of b and the norms, every step
    import torch
    qh = torch.empty(q0.shape, dtype=torch.float64, pin_memory=True).numpy()
    qh[:] = q0
    bh = torch.empty((m.nnode, 5), dtype=torch.float64, pin_memory=True).numpy()
    S.set_state(qh)
    S.residual_full()
    S.get_residual(out=bh)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        S.set_state(qh)
        S.residual_full()
        b = S.get_residual(out=bh)
    N.check(lib.pcfd_device_sync(), "sync")
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(pg, e2e_s)
    h2d = qh.nbytes
    d2h = b.nbytes + 6 * 8

    # roofline of the dominant FP64 kernel.  Algorithmic bytes per launch,
    # each array once (B/edge, B/node):
    #   edge_flux   (MUSCL + Roe + clip test, both ends' corrections stored
    #               by the limiter pass): 160 = ids 8, area 32, corrections
    #               80, flux written 40; 80 = q 40, limiter 40
    #   edge_viscous: 144 = ids 8, area 32, half-vector 24, flux read and
    #               written 80; 256 = q 40, gradient 216
    #   lsq_gradient: 56 = ids 8, LSQ weights of both ends 48; 288 = the 9
    #               gradient variables 72, gradient written 216
    #   venkat_limiter: 112 = ids 8, half-vector 24, both ends' corrections
    #               written 80; 208 = q 40, gradient 120, volume 8, limiter
    #               written 40
    #   residual_gather: 88 = the edge's flux read at both ends 80, its id in
    #               the node list 8; 80 = q_old 40, b written 40
    alg_per = {"edge_flux": (160.0, 80.0), "edge_viscous": (144.0, 256.0), "lsq_gradient": (56.0, 288.0),
               "venkat_limiter": (112.0, 208.0), "residual_gather": (88.0, 80.0)}
    top = max((k for k in kernels if k in alg_per), key=lambda k: kernels[k]["ms_per_step"])
    top_ms = kernels[top]["ms_per_step"] / max(kernels[top]["launches_per_step"], 1.0)
    alg_bytes = alg_per[top][0] * m.nedge + alg_per[top][1] * m.nnode
    achieved = alg_bytes / (top_ms * 1e-3) / 1e9 if top_ms > 0 else None
    # DRAM traffic per launch from one ncu capture of the kernels on the
    # 128x96x96 box (profiles/residual_fp64_ns128.md), as a ratio to their
    # algorithmic bytes there, scaled to this box: the traffic grows with the
    # edges and nodes streamed
    traffic_ratio = {"edge_flux": 1462.9 / 1393.9, "venkat_limiter": 1700.8 / 1155.1, "edge_viscous": 1498.7 / 1471.6,
                     "lsq_gradient": 790.8 / 794.6, "residual_gather": 640.3 / 809.2}
    traffic = alg_bytes * traffic_ratio[top] if top in traffic_ratio else None
    peak, peak_kind = peaks()
    # The FP64 kernels are bound by the FP64 pipe (2 FP64 instructions per
    # clock per SM on GB300).  FP64 thread instructions per edge and per node
    # of each kernel, from one ncu capture on the 128x96x96 box
    # (sm__inst_executed_pipe_fp64 x 32, profiles/residual_fp64_ns128.md);
    # achieved = those instructions over the kernel's event-timed launch,
    # peak = 2 x SMs x the median SM clock sampled during the timed region.
    fp64_inst = {"edge_flux": (257.0, 0.0), "venkat_limiter": (0.0, 1145.0), "edge_viscous": (152.0, 0.0),
                 "lsq_gradient": (0.0, 506.0), "residual_gather": (0.0, 184.0)}
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = clk.summary().get("sm_mhz") or 0.0
    fp64_peak = 2.0 * nsm * sm_mhz * 1e6 / 1e9  # G instructions / s
    fp64_ach = (fp64_inst[top][0] * m.nedge + fp64_inst[top][1] * m.nnode) / (top_ms * 1e-3) / 1e9
    # the whole residual against its algorithmic bytes: 40 B/edge + 360 B/node
    # + 84 B/half-edge (gradients and limiter given)
    res_bytes = 40.0 * m.nedge + 360.0 * m.nnode + 84.0 * m.nbedge

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "residual_evals_per_s": ws * 1e3 / ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "ns_flatplate %dx%dx%d: 2nd-order laminar NS residual (BCs+LSQ grad+modified "
                               "Venkatakrishnan limiter K=%g+Roe+viscous), Mach 0.8, Re 1e5"
                               % (w["nx"], w["ny"], w["nz"], case.param.venkat_K),
                   "nodes": m.nnode, "edges": m.nedge, "half_edges": m.nbedge,
                   "l2": "inputs larger than L2 (edge arrays alone %.0f MB)" % (m.nedge * 104 / 1e6),
                   "parallelism": "replicas" if ws > 1 else "single GPU", "mesh_build_s": round(t_mesh, 2),
                   "limiter_K": case.param.venkat_K},
        "resGlobal": float(norms[0]),
        "residual_hbm_frac": res_bytes / (ms_per_step * 1e-3) / 1e9 / peak,
        "df64": ({"what": "the same residual in double-float arithmetic (FP32 pairs, ~48-bit significand)",
                  "value": ws * m.nedge / (results[1][0] / args.steps * 1e-3) / 1e6,
                  "ms_per_step": results[1][0] / args.steps, "resGlobal": float(results[1][1][0]),
                  "resGlobal_rel_diff_vs_f64": abs(results[1][1][0] - norms[0]) / abs(norms[0]),
                  "kernels": kernels_df} if 1 in results else None),
        "gpu_launches": int(launches),
        "kernels": kernels,
        "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "peak_source": peak_kind,
                     "note": "HBM fraction of the measured copy peak; the FP64 kernels are bound by the FP64 pipe "
                             "(2 FP64 fused multiply-adds per clock per SM on GB300), not by HBM"},
        "roofline_fp64": {"bound": "fp64 pipe", "kernel": top, "achieved": fp64_ach, "peak": fp64_peak,
                          "unit": "G FP64 instructions/s", "frac": fp64_ach / fp64_peak if fp64_peak else None,
                          "instructions_per_edge_node": fp64_inst[top],
                          "source": "instruction counts from ncu (profiles/residual_fp64_ns128.md); peak 2/clock/SM "
                                    "x %d SMs x median SM clock" % nsm},
        "clocks": clk.summary(),
        "e2e": {"value": ws * m.nedge / e2e_s / 1e6, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
    }
    if rank == 0 and not args.no_cpu_baseline:
        base, _, _ = cpu_sample(12.0, os.cpu_count() or 1)
        line["cpu_baseline"] = base

    # node numbering: the FP64 residual on the same box numbered by the
    # reference's set-up reorder (its reverse Cuthill-McKee list used as an
    # old-to-new map, ucs/mesh.tcc:224) and by that sequence itself
    def order_entry(S_, ms_):
        S_.profile(True)
        S_.profile_reset()
        S_.residual_full()
        t = S_.timers()
        S_.profile(False)
        return {"ms_per_step": ms_, "edge_flux_ms": t["edge_flux"][0], "lsq_gradient_ms": t["lsq_gradient"][0],
                "venkat_limiter_ms": t["venkat_limiter"][0], "edge_viscous_ms": t["edge_viscous"][0]}

    S.set_state(q0)
    S.set_residual_arithmetic(0)
    line["node_order"] = {"what": "FP64 residual, ms per evaluation and its largest kernels, by node numbering",
                          "natural": order_entry(S, ms_per_step)}
    if not args.no_node_order:
        for name, ro in (("reference_reorder", True), ("rcm", "rcm")):
            t0 = time.perf_counter()
            m2 = Mesh.box(w["nx"], w["ny"], w["nz"], reorder=ro, **case.mesh_kw)
            tb = time.perf_counter() - t0
            S2 = SolutionSpace(m2, case.param)
            S2.set_state(cases.perturbed_state(S2.qinf(), m2.nnode + m2.nbedge, seed=1))
            S2.bench_residual_full(3)
            ms2, _ = S2.bench_residual_full(args.steps)
            line["node_order"][name] = dict(order_entry(S2, ms2 / args.steps), mesh_build_s=round(tb, 2))
            S2.close()
            del m2
    # the FP32 block SpMV of the mixed solver on this machine's matrix: one mixed
    # Newton step assembles it (FP32 storage), then K device-timed products
    # on resident vectors (the matrix is larger than L2)
    S.set_state(q0)
    S.set_residual_arithmetic(1)
    S.newton_iterate(1, **dict(CONV_ARMS["mixed"], fgmres_m=2))
    S.bench_spmv(3)
    spmv_ms = S.bench_spmv(args.steps) / args.steps
    nb = S.nblocks()
    spmv_bytes = (nb - m.nnode) * (25 * 4 + 4) + m.nnode * (4 + 5 * 4 + 5 * 4 + 25 * 4)
    line["spmv"] = {"what": "FP32 block SpMV y = A x (k_spmv_staged) of the mixed solver's %d-block matrix, "
                            "vectors resident" % nb,
                    "ms": spmv_ms, "bytes": spmv_bytes, "achieved_gbs": spmv_bytes / (spmv_ms * 1e-3) / 1e9,
                    "peak_gbs": peak, "frac": spmv_bytes / (spmv_ms * 1e-3) / 1e9 / peak if peak else None}

    # the block-SGS sweep (k_sgs_sweep_staged, one cooperative launch per
    # call): the mixed solver's FP32 preconditioner sweep on the FP32 matrix,
    # then the FP64 arm's 10 FP64 sweeps on the FP64 matrix.  Algorithmic
    # bytes per sweep: the matrix twice (forward and backward pass) as in the
    # SpMV, plus the LU'd diagonal and pivots and the vectors,
    # 2 x SpMV + N (25 s + 20) with s the matrix scalar size.
    def sgs_bytes(sz):
        spmv = (nb - m.nnode) * (25 * sz + 4) + m.nnode * (4 + 5 * sz + 5 * sz + 25 * sz)
        return 2 * spmv + m.nnode * (25 * sz + 20)

    S.bench_sgs(3, 1, fp32=True)
    sgs32_ms = S.bench_sgs(args.steps, 1, fp32=True) / args.steps
    S.set_residual_arithmetic(0)
    S.newton_iterate(1, **dict(CONV_ARMS["fp64"], nsgs=1))
    S.bench_sgs(1, 10, fp32=False)
    nrep64 = max(2, args.steps // 5)
    sgs64_ms = S.bench_sgs(nrep64, 10, fp32=False) / (10 * nrep64)
    line["sgs"] = {"what": "block-SGS sweep (forward + backward, k_sgs_sweep_staged) on this box's %d-block "
                           "matrix, vectors resident; ms per sweep" % nb,
                   "fp32": {"ms": sgs32_ms, "bytes": sgs_bytes(4),
                            "achieved_gbs": sgs_bytes(4) / (sgs32_ms * 1e-3) / 1e9,
                            "frac": sgs_bytes(4) / (sgs32_ms * 1e-3) / 1e9 / peak if peak else None},
                   "fp64": {"ms": sgs64_ms, "bytes": sgs_bytes(8),
                            "achieved_gbs": sgs_bytes(8) / (sgs64_ms * 1e-3) / 1e9,
                            "frac": sgs_bytes(8) / (sgs64_ms * 1e-3) / 1e9 / peak if peak else None},
                   "colors": S.crs_structure()[2]}
    S.close()
    if rank == 0 and ws == 1 and not args.no_chemistry:
        line["chemistry"] = chemistry_study(args)
    if rank == 0 and ws == 1 and args.converge_arms:
        line["convergence"] = converge_study(args)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ns256", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--arith", default="both", choices=["f64", "both"],
                    help="time the FP64 residual only, or the double-float one beside it")
    ap.add_argument("--converge", default="fp64,mixed,mixed_learned",
                    help="comma-separated arms of the time-to-1e-10 study on one GPU ('' to skip)")
    ap.add_argument("--converge-workload", default="ns64", choices=sorted(WORKLOADS))
    ap.add_argument("--converge-cap", type=float, default=60.0, help="wall-time cap per arm, seconds")
    ap.add_argument("--converge-iters", type=int, default=5000, help="Newton iteration cap per arm")
    ap.add_argument("--learned-train-workload", default="ns64", choices=sorted(WORKLOADS),
                    help="box of the learned preconditioner's training runs")
    ap.add_argument("--learned-runs", type=int, default=4, help="training runs (sampled flows)")
    ap.add_argument("--converge-only", action="store_true", help="run only the convergence study")
    ap.add_argument("--no-chemistry", action="store_true", help="skip the finite-rate chemistry measurement")
    ap.add_argument("--no-node-order", action="store_true", help="skip the residual on the renumbered meshes")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    args.converge_arms = [a for a in args.converge.split(",") if a]
    for a in args.converge_arms:
        if a not in CONV_ARMS:
            ap.error("unknown convergence arm %r" % a)
    ws, rank, local, pg = dist()
    if args.impl == "reference":
        run_reference(args, rank, pg)
    elif args.converge_only:
        if rank == 0:
            print(json.dumps({"convergence": converge_study(args)}), flush=True)
    else:
        run_gb300(args, ws, rank, local, pg)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
