#!/usr/bin/env python
"""Benchmark of one PFEM-2 time step (ms per step) on the GB300 engine.

Default workload: the channel-with-cylinder case (2.2 x 0.41 channel, cylinder r=0.05
at (0.2, 0.2), 994,240 P1 triangles from the committed generator, 16 particles per
cell, Scheme B, rho=1, mu=1e-3, dt=5e-4, drag/lift each step).  Synthetic input of the
named shape: the mesh and particles are generated, the flow starts from rest and
`--warmup` steps run before the timed ones.

Arms:
  default           the engine (C ABI via ctypes, CUDA kernels for sm_103a); beside it the
                    reference's own CUDA build on the same workload and GPU
                    (`reference_cuda`, oracle/build_ref_cuda.sh) and the CPU oracle from
                    the engine's state (`cpu_baseline`)
  --impl reference  the CPU oracle of the same step (oracle/, an FP64 C port of the
                    reference's algorithm with the engine arm's solver choices, OpenMP on
                    the host cores), the same warm-up from rest, then timed steps

Prints ONE JSON line (rank 0).  `value` is device time per step with all state
resident in HBM; `e2e` is the same step driven through the C ABI with the inflow
boundary values uploaded from pinned host memory and the fields (u, v, p) plus the
step record copied back to pinned host memory every step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from gpupfem2_gb300 import meshgen as mg  # noqa: E402

WORKLOADS = {
    # name: (mesh factory, channel length, height, cylinder, params)
    "cylinder": dict(mesh=lambda: mg.cylinder_channel(), lx=2.2, ly=0.41, cyl=(0.2, 0.2, 0.05),
                     params=dict(rho=1.0, mu=1e-3, dt=5e-4, scheme=1, level=4, n_outer=2, substeps=3,
                                 pressure_precond=2, calculate_loads=1, body_boundary_id=3, thickness=0.1,
                                 mean_velocity=1.0, pressure_ordering=1, gmres_orthogonalization=1,
                                 prediction_solver=2)),
    # the same case at a quarter of the cells (248,560 triangles): small captures under ncu
    "cylinder_quarter": dict(mesh=lambda: mg.cylinder_channel(nxh=350, nyh=400, nr=12), lx=2.2, ly=0.41,
                             cyl=(0.2, 0.2, 0.05),
                             params=dict(rho=1.0, mu=1e-3, dt=5e-4, scheme=1, level=4, n_outer=2, substeps=3,
                                         pressure_precond=2, calculate_loads=1, body_boundary_id=3, thickness=0.1,
                                         mean_velocity=1.0, pressure_ordering=1, gmres_orthogonalization=1,
                                         prediction_solver=2)),
    "channel": dict(mesh=lambda: mg.channel(), lx=4.0, ly=1.0, cyl=None,
                    params=dict(rho=1.0, mu=0.01, dt=0.005, scheme=0, level=3, n_outer=2, substeps=3,
                                pressure_precond=1)),
    "square": dict(mesh=lambda: mg.unit_square(64), lx=1.0, ly=1.0, cyl=None,
                   params=dict(rho=1.0, mu=0.01, dt=0.005, scheme=0, level=2, n_outer=2, substeps=3,
                               pressure_precond=0)),
}
PRECOND_NAMES = {-1: "none", 0: "jacobi", 1: "ilu", 2: "ic"}
PHASES = ["particles", "projection", "prediction_assembly", "prediction_solve", "pressure_assembly",
          "pressure_solve", "correction_assembly", "correction_solve", "particle_correction"]


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def replica_max(value, device):
    """The slowest replica's value: with one independent replica per GPU (the step does
    not shard), the job's ms per step is the maximum over the ranks."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def build_case(name, precond=None, ordering=None, gs=None, cg=None, pred=None):
    w = WORKLOADS[name]
    xy, tri = w["mesh"]()
    bu, bv, bp = mg.channel_boundary_nodes(xy, w["lx"], w["ly"], 1.5, cylinder=w["cyl"])
    prm = dict(w["params"])
    if precond is not None:
        prm["pressure_precond"] = precond
    if ordering is not None:
        prm["pressure_ordering"] = ordering
    if gs is not None:
        prm["gmres_orthogonalization"] = gs
    if cg is not None:
        prm["cg_variant"] = cg
    if pred is not None:
        prm["prediction_solver"] = pred
    return w, xy, tri, bu, bv, bp, prm


class ClockSampler:
    """nvidia-smi clocks during the timed region (200 ms period)."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-i", "0", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def oracle_params(name, prm):
    """The oracle's parameters for a workload, with the engine arm's solver choices: the
    pressure preconditioner and its ordering (the multicolour order is the engine's
    colouring, restated in the oracle), the prediction solver, GMRES's Gram-Schmidt and
    the stopping tests."""
    from oracle import oracle as O
    w = WORKLOADS[name]
    cyl = w["cyl"]
    return O.make_params(
        rho=prm["rho"], mu=prm["mu"], dt=prm["dt"], scheme=prm["scheme"], level=prm["level"], n_outer=prm["n_outer"],
        substeps=prm["substeps"], pressure_precond=prm["pressure_precond"], tol=prm.get("tolerance", 1e-8),
        maxit=prm.get("max_iterations", 1000), lx=w["lx"], ly=w["ly"], has_cylinder=int(cyl is not None),
        cx=cyl[0] if cyl else 0.2, cy=cyl[1] if cyl else 0.2, radius=cyl[2] if cyl else 0.05,
        calc_loads=prm.get("calculate_loads", 0), body_id=prm.get("body_boundary_id", -1),
        thickness=prm.get("thickness", 1.0), pressure_ordering=prm.get("pressure_ordering", 0),
        prediction_solver=prm.get("prediction_solver", 1), gmres_orth=prm.get("gmres_orthogonalization", 0),
        pressure_criterion=prm.get("pressure_criterion", 0))


def same_solver_config(prm):
    """True when the oracle runs exactly the engine arm's solver algorithms (the oracle
    has the standard CG iteration only)."""
    return prm.get("cg_variant", 0) == 0 and prm.get("pressure_precision", 0) == 0 and prm.get("pressure_x0", 0) == 0


def _omp_threads():
    return int(os.environ.get("OMP_NUM_THREADS", "0") or 0) or os.cpu_count() or 1


def cpu_baseline(name, prm, eng, xy, tri, bu, bv, bp, max_seconds=25.0):
    """The oracle's step, with the engine arm's solver choices, from the state the engine
    reached (its particles and the eight node fields copied into the oracle): a bounded
    sample of the same workload at the same step."""
    from oracle import oracle as O
    P = eng.particles.download()
    np0 = int(P["cell"].size)
    flow = O.Flow(xy, tri, oracle_params(name, prm), bu, bv, bp, particle_cap=int(1.5 * np0) + 1024)
    flow.set_particles(P)
    del P
    for f in O.Flow.FIELDS:
        flow.set_field(f, eng.field(f))
    times = []
    t_all = time.perf_counter()
    while not times or (time.perf_counter() - t_all < max_seconds and len(times) < 3):
        t0 = time.perf_counter()
        flow.step()
        times.append(time.perf_counter() - t0)
    threads = _omp_threads()
    return {"value": 1000.0 * statistics.median(times), "unit": "ms/step", "cores": threads, "kind": "port",
            "same_config": same_solver_config(prm),
            "sample": "%d oracle step(s) of the full %s workload from the engine's state after its timed steps "
                      "(%d triangles, %d particles), median; FP64 C port with the engine arm's solver choices, "
                      "OpenMP (%d threads) over particles, SpMV rows, colour classes and vector updates"
                      % (len(times), name, tri.shape[0], np0, threads)}


def run_reference(args):
    """The reference arm: the oracle (a C port of the reference's step, with the same
    solver choices as the engine arm) on the same workload, warmed up by the same number of
    steps from rest, then timed step by step until --steps steps or --ref-budget seconds
    (at least one step).  The steps actually timed are reported.  One more step from the
    same state with the reference's own solver algorithms (natural-order ILU/IC, GMRES with
    modified Gram-Schmidt) is reported beside it."""
    from oracle import oracle as O
    name = args.workload
    w, xy, tri, bu, bv, bp, prm = build_case(name, args.precond, args.ordering, args.gs, args.cg, args.pred)
    level = prm["level"]
    flow = O.Flow(xy, tri, oracle_params(name, prm), bu, bv, bp, particle_cap=4 * tri.shape[0] * level * level)
    t_start = time.perf_counter()
    for _ in range(args.warmup):
        flow.step()
    warm_s = time.perf_counter() - t_start
    times, info = [], None
    t0 = time.perf_counter()
    while len(times) < args.steps and (not times or time.perf_counter() - t0 < args.ref_budget):
        t1 = time.perf_counter()
        info = flow.step()
        times.append(time.perf_counter() - t1)
    ms = 1000.0 * statistics.mean(times)
    particles = int(info.particles)
    ref_alg_ms = None
    if args.ref_algorithms:
        # the reference's own algorithms from the same state
        flow.set_solvers(prm["pressure_precond"], 0, 1, 0, 0)
        t1 = time.perf_counter()
        flow.step()
        ref_alg_ms = 1000.0 * (time.perf_counter() - t1)
    threads = _omp_threads()
    cfg = {"workload": name, "triangles": int(tri.shape[0]), "particles": particles,
           "pressure_precond": PRECOND_NAMES[prm["pressure_precond"]],
           "pressure_ordering": ["natural", "multicolour"][prm.get("pressure_ordering", 0)],
           "prediction_solver": {1: "gmres", 2: "bicgstab"}[prm.get("prediction_solver", 1)],
           "scheme": "AB"[prm["scheme"]], "level": level, "n_outer": prm["n_outer"],
           "tolerance": prm.get("tolerance", 1e-8), "max_iterations": prm.get("max_iterations", 1000),
           "same_config_as_engine_arm": same_solver_config(prm),
           "steps_requested": args.steps, "timed_from_step": args.warmup + 1}
    if prm.get("prediction_solver", 1) == 1:
        cfg["gmres_gram_schmidt"] = ["modified", "classical_twice"][prm.get("gmres_orthogonalization", 0)]
    base = {"value": ms, "unit": "ms/step", "cores": threads, "kind": "port",
            "sample": "%d oracle step(s) of the full %s workload, steps %d-%d after %d warm-up steps from rest "
                      "(%.0f s), mean; FP64 C port of the reference's step with the engine arm's solver choices, "
                      "OpenMP (%d threads) over particles, SpMV rows, colour classes and vector updates"
                      % (len(times), name, args.warmup + 1, args.warmup + len(times), args.warmup, warm_s, threads)}
    line = {"metric": "ms per PFEM-2 step", "value": ms, "unit": "ms/step", "n_gpus": args.gpus,
            "steps": len(times), "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "impl": "reference", "cpu_baseline": base,
            "e2e": {"value": ms, "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if ref_alg_ms is not None:
        line["reference_algorithms"] = {
            "ms_per_step": ref_alg_ms, "step": args.warmup + len(times) + 1, "pressure_ordering": "natural",
            "prediction_solver": "gmres", "gmres_gram_schmidt": "modified",
            "note": "one step of the reference's own solver algorithms from the same state"}
    print(json.dumps(line))


REF_CUDA = os.path.join(ROOT, "baseline", "_ref", "bin", "ref_cylinder")
REF_STAGE = os.path.join(ROOT, "baseline", "_ref", "gpuPfem2", "src")


def reference_cuda(name, xy, tri, prm, precond="jacobi", warmup=5, steps=20, timeout=900):
    """The reference's own CUDA build (its library and Cylinder2D case code, compiled for
    sm_103a by oracle/build_ref_cuda.sh) running the same cylinder workload on this GPU:
    per-step time from its own GpuTimer, warm mean and median over `steps` steps after
    `warmup` steps from rest.  Returns None for workloads other than the cylinder."""
    if name not in ("cylinder", "cylinder_quarter"):
        return None
    if not os.path.exists(REF_CUDA):
        if not os.path.isdir(REF_STAGE):
            return {"unavailable": "reference sources not staged (oracle/build_ref_cuda.sh stage)"}
        r = subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref_cuda.sh")], capture_output=True, text=True)
        if r.returncode != 0 or not os.path.exists(REF_CUDA):
            return {"unavailable": "reference build failed: " + (r.stderr.strip().splitlines() or [""])[-1][:200]}
    with tempfile.TemporaryDirectory() as td:
        mesh = os.path.join(td, "mesh.dat")
        mg.write_dat(mesh, xy, tri)
        out = os.path.join(td, "ref.json")
        t0 = time.perf_counter()
        try:
            with open(os.path.join(td, "stdout.txt"), "w") as so:
                r = subprocess.run([REF_CUDA, mesh, str(prm["level"]), repr(prm["dt"]), str(prm["scheme"]), precond,
                                    str(warmup), str(steps), out], cwd=td, stdout=so, stderr=subprocess.STDOUT,
                                   timeout=timeout)
        except subprocess.TimeoutExpired:
            return {"unavailable": "reference run exceeded %d s" % timeout}
        wall = time.perf_counter() - t0
        text = open(os.path.join(td, "stdout.txt")).read()
        if r.returncode != 0 or not os.path.exists(out):
            return {"unavailable": "reference run failed (rc %d): %s" % (r.returncode, text[-300:])}
        res = json.load(open(out))
        # the solvers' own prints: iterations of the last step's solves in their order
        # (prediction x, y, pressure, correction x, y per outer iteration)
        last = text[text.rfind("Time step no."):]
        its = []
        for ln in last.splitlines():
            if ln.startswith("Solver converged"):
                its.append(int(ln.rsplit("=", 1)[1]))
            elif ln.startswith("Solver failed"):
                its.append(-1)
        forces = [ln.split(";") for ln in open(os.path.join(td, "Forces.csv")).read().split("\n")[1:] if ln]
    sm = res["step_ms"]
    return {"ms_per_step": statistics.mean(sm), "ms_per_step_median": statistics.median(sm), "steps": len(sm),
            "warmup": warmup, "pressure_precond": precond,
            "phase_ms": {k: round(v, 3) for k, v in res["phase_ms"].items()}, "particles": res["particles"],
            "iterations_last_step": its, "cx": float(forces[-1][1]) if forces else None,
            "cy": float(forces[-1][2]) if forces else None, "wall_s": round(wall, 1),
            "timer": "the reference's GpuTimer (common/gpu_timer.cuh) per step",
            "build": "reference src/ and cases/Cylinder2D kernels for sm_103a (-O2, rdc), neighbour lists "
                     "filled in O(N) outside the timed steps; -1 in iterations_last_step: not converged"}


def _timed(fn):
    import torch
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record()
    out = fn()
    b.record()
    torch.cuda.synchronize()
    return out, a.elapsed_time(b)


def study_solver(args):
    """Pressure solve to a 1e-8 relative residual on the flow's own pressure matrix after
    --record steps of the cylinder case, on the 994,240-triangle mesh and its 1:4
    refinement (3,976,960 triangles): FP64 PCG (standard, one-reduction and pipelined)
    and the mixed-precision refinement, with Jacobi and IC(0) on the multicolour order.  b = A x* with x* uniform in
    [-1, 1] (splitmix64 seed 0), x0 = 0; median of 3 solves after one warm-up."""
    import torch
    import gpupfem2_gb300 as g
    w = WORKLOADS["cylinder"]
    xy, tri = w["mesh"]()
    meshes = [("cylinder_1M", xy, tri)]
    if not args.quick:
        x4, t4 = mg.refine_uniform(xy, tri, snap_circle=(0.2, 0.2, 0.05, 1e-3))
        meshes.append(("cylinder_4M", x4, t4))
    out = []
    for name, mxy, mtri in meshes:
        m = g.Mesh2D.from_arrays(mxy, mtri)
        m.set_channel_boundary_ids(w["lx"], w["ly"], w["cyl"])
        bu, bv, bp = mg.channel_boundary_nodes(mxy, w["lx"], w["ly"], 1.5, cylinder=w["cyl"])
        prm = dict(w["params"], calculate_loads=0)
        eng = g.FlowEngine(m, g.default_params(**prm), bu, bv, bp, capacity_factor=2.0)
        eng.seed()
        for _ in range(args.record):
            eng.step()
        A, _ = eng.system(2)
        xs = torch.tensor(mg.uniform_pm1(0, m.nv), device="cuda")
        b = torch.empty_like(xs)
        g.spmv(A, xs, b)
        bn = float(torch.linalg.norm(b))
        rows = []
        # (IC(0) in the natural order is left out: its triangular sweeps follow ~1,900
        # sequential levels here and one apply costs milliseconds)
        cases = [("fp64_jacobi", dict(precond="jacobi")),
                 ("fp64_ic0_multicolour", dict(precond="ic", ordering=1)),
                 ("fp64_jacobi_one_reduction", dict(precond="jacobi", cg_variant=g.CG_ONE_REDUCTION)),
                 ("fp64_ic0_multicolour_one_reduction", dict(precond="ic", ordering=1, cg_variant=g.CG_ONE_REDUCTION)),
                 ("mixed_jacobi", dict(precond="jacobi", precision=g.PRECISION_MIXED)),
                 ("mixed_ic0_multicolour", dict(precond="ic", ordering=1, precision=g.PRECISION_MIXED)),
                 ("fp64_ic0_multicolour_pipelined", dict(precond="ic", ordering=1, cg_variant=g.CG_PIPELINED))]
        if args.quick:  # FP64 and mixed, standard and pipelined CG
            cases = [cases[i] for i in (0, 1, 4, 5, 6)]
        for label, kw in cases:
            s = g.LinearSolver(A, "cg", tol=1e-8, maxit=20000, criterion=g.CRITERION_REL, **kw)
            times, info, x0 = [], None, None
            for rep in range(4):
                x0 = torch.zeros_like(b)
                info, ms = _timed(lambda: s.solve(A, x0, b, check=False))
                if rep:
                    times.append(ms)
            r = torch.empty_like(b)
            g.spmv(A, x0, r)
            rows.append({"solver": label, "ms": round(statistics.median(times), 3), "iterations": info.iterations,
                         "outer": info.outer_iterations, "converged": info.converged, "status": info.status,
                         "rel_residual_fp64": float(torch.linalg.norm(b - r)) / bn,
                         "x_err": float(torch.linalg.norm(x0 - xs) / torch.linalg.norm(xs))})
            del s
        base = rows[0]["ms"]
        for r_ in rows:
            r_["time_vs_fp64_jacobi"] = round(r_["ms"] / base, 4)
        out.append({"mesh": name, "triangles": int(mtri.shape[0]), "nodes": m.nv, "nnz": A.nnz,
                    "matrix": "pressure system of the flow after %d steps" % args.record, "solvers": rows})
        del eng, A
        torch.cuda.synchronize()
    print(json.dumps({"study": "pressure_solver", "criterion": "||b - A x|| <= 1e-8 ||b||", "results": out}))


def learned_metric(args, mesh, bu, bv, bp, prm):
    """The second headline metric: pressure-solve time to ||b - A x|| <= 1e-8 ||b|| inside
    the flow, mixed precision with the learned initial guess against the plain FP64 PCG
    (the same IC(0) preconditioner on the multicolour order, previous pressure as the
    start) and against mixed precision alone.  Each variant runs the same case from rest:
    --learned-train steps (the network trains online on the plain solver's increments of
    those steps), then --learned-eval timed steps.  Every eval step's final pressure is
    compared with an FP64 re-solve of the same system (||r|| <= 1e-12 ||b||, started from
    it): the error per result of each variant's 1e-8 solve, FP64 plain included."""
    import ctypes
    import torch
    import gpupfem2_gb300 as g
    L = g.lib()
    base = dict(prm, pressure_criterion=1, pressure_tolerance=1e-8, pressure_max_iterations=20000,
                learn_steps=args.learned_train, learn_rate=1e-3)
    # "mixed_learned_tol1e-9": the same with a ten times stricter stop, to see what the mixed
    # form's error against the FP64 re-solve costs (the metric's value stays the 1e-8 one)
    variants = [("fp64_plain", dict(pressure_precision=0, pressure_x0=0)),
                ("mixed", dict(pressure_precision=1, pressure_x0=0)),
                ("mixed_learned", dict(pressure_precision=1, pressure_x0=1)),
                ("mixed_learned_tol1e-9", dict(pressure_precision=1, pressure_x0=1, pressure_tolerance=1e-9))]
    res = {}
    for label, kw in variants:
        eng = g.FlowEngine(mesh, g.default_params(**dict(base, **kw)), bu, bv, bp, capacity_factor=4.0)
        eng.seed()
        for _ in range(args.learned_train):
            eng.step()
        eng.info()
        g._check(L.pf2_flow_enable_timing(eng.h, args.learned_eval), "timing")
        its, errs, ratios, used = [], [], [], 0
        ref_solver = None
        for _ in range(args.learned_eval):
            eng.step()
            inf = eng.info()
            its.append(sum(inf.it_pressure[k] for k in range(prm["n_outer"])))
            used += inf.guess_used
            if inf.guess_residual[0] > 0:
                ratios.append(inf.guess_residual[1] / inf.guess_residual[0])
            # the error of this step's 1e-8 solve against a tight FP64 re-solve
            A, rhs = eng.system(2)
            if ref_solver is None:
                ref_solver = g.LinearSolver(A, "cg", "ic", tol=1e-12, maxit=20000, criterion=g.CRITERION_REL,
                                            ordering=1)
            p = _wrap(eng.field_ptr("p"), mesh.nv)
            x = p.clone()
            ref_solver.solve(A, x, _wrap(rhs, mesh.nv), check=False)
            errs.append(float(torch.linalg.norm(p - x) / torch.linalg.norm(x)))
        ph = (ctypes.c_double * 9)()
        nst = ctypes.c_int()
        g._check(L.pf2_flow_phase_times(eng.h, ph, ctypes.byref(nst)), "phase times")
        res[label] = {"pressure_ms_per_step": ph[5] / max(nst.value, 1),
                      "pressure_iterations_per_step": statistics.mean(its),
                      "start_residual_ratio": statistics.mean(ratios) if ratios else None,
                      "guess_used_steps": used}
        if errs:
            res[label]["p_rel_err_vs_fp64_resolve_max"] = max(errs)
        del ref_solver, eng
        torch.cuda.synchronize()
    b0 = res["fp64_plain"]["pressure_ms_per_step"]
    for v in res.values():
        v["time_vs_fp64_plain"] = v["pressure_ms_per_step"] / b0
    return {"value": res["mixed_learned"]["time_vs_fp64_plain"], "target": 0.5,
            "criterion": "||b - A x|| <= 1e-8 ||b|| per pressure solve (mixed_learned_tol1e-9: 1e-9), "
                         "IC(0) multicolour",
            "protocol": "from rest: %d training steps, then %d timed steps per variant (the full protocol trains "
                        "500 and evaluates 2,000)" % (args.learned_train, args.learned_eval),
            "variants": res}


def study_learned(args):
    """The pressure solve of each step (1e-8 relative residual) with the plain FP64 PCG
    against mixed precision alone and mixed precision with the learned initial guess
    (trained online on the first --train steps, used afterwards).  On the cylinder flow
    (default) six variants; with `--workload channel`, the 4 x 1 channel at its stated
    size (256 x 64, level 3, Scheme A) with ILU(0) on the multicolour order for every
    variant (the mixed solver's ILU(0) runs on that order), four variants: the
    learned-start protocol of 500 training steps and 2,000 evaluated steps is
    `--train 500 --eval 2000`."""
    import ctypes
    import torch
    import gpupfem2_gb300 as g
    name = "channel" if args.workload == "channel" else "cylinder"
    w, xy, tri, bu, bv, bp, prm = build_case(name)
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(w["lx"], w["ly"], w["cyl"])
    res = {}
    # IC(0) or ILU(0) (multicolour order) pressure solves to ||b - A x|| <= 1e-8 ||b||
    # with an iteration limit high enough for every variant to converge
    prm = dict(prm, max_iterations=20000, pressure_ordering=1)
    # "untrained": the same start with a network that never trains, which isolates what
    # the trained network adds to the projection onto the last increments
    # "fp64_jacobi": the reference cylinder driver's own pressure solver (Jacobi PCG,
    # Cylinder2D/main.cu:769-771) on the same steps
    if name == "channel":
        variants = [("fp64_plain", dict(pressure_precision=0, pressure_x0=0)),
                    ("mixed", dict(pressure_precision=1, pressure_x0=0)),
                    ("mixed_untrained", dict(pressure_precision=1, pressure_x0=1, learn_steps=0)),
                    ("mixed_learned", dict(pressure_precision=1, pressure_x0=1))]
    else:
        variants = [("fp64_plain", dict(pressure_precision=0, pressure_x0=0)),
                    ("fp64_jacobi", dict(pressure_precision=0, pressure_x0=0, pressure_precond=0)),
                    ("fp64_learned", dict(pressure_precision=0, pressure_x0=1)),
                    ("fp64_untrained", dict(pressure_precision=0, pressure_x0=1, learn_steps=0)),
                    ("mixed", dict(pressure_precision=1, pressure_x0=0)),
                    ("mixed_learned", dict(pressure_precision=1, pressure_x0=1))]
    L = g.lib()
    finals = {}
    for label, kw in variants:
        prm2 = dict(prm, pressure_criterion=1, learn_steps=args.train, learn_rate=1e-3)
        prm2.update(kw)
        # particles accumulate where the flow converges: room for 4x the seeded count
        eng = g.FlowEngine(m, g.default_params(**prm2), bu, bv, bp, capacity_factor=4.0)
        eng.seed()
        for _ in range(args.train):
            eng.step()
        eng.info()
        g._check(L.pf2_flow_enable_timing(eng.h, args.eval), "timing")
        its, its_first, ratios, used = [], [], [], 0
        for _ in range(args.eval):
            eng.step()
            inf = eng.info()
            its.append(sum(inf.it_pressure[k] for k in range(prm["n_outer"])))
            its_first.append(inf.it_pressure[0])
            if inf.guess_residual[0] > 0:
                ratios.append(inf.guess_residual[1] / inf.guess_residual[0])
            used += inf.guess_used
        ph = (ctypes.c_double * 9)()
        nst = ctypes.c_int()
        g._check(L.pf2_flow_phase_times(eng.h, ph, ctypes.byref(nst)), "phase times")
        res[label] = {"pressure_ms_per_step": ph[5] / max(nst.value, 1), "iterations_per_step": statistics.mean(its),
                      "iterations_first_solve": statistics.mean(its_first),
                      "start_residual_ratio": statistics.mean(ratios) if ratios else None,
                      "guess_used_steps": used, "cx": inf.cx, "cy": inf.cy, "particles": inf.particles}
        print(label, json.dumps(res[label]), file=sys.stderr, flush=True)
        finals[label] = (eng.field("p"), eng.field("ux"))
        del eng
        torch.cuda.synchronize()
    base = res["fp64_plain"]["pressure_ms_per_step"]
    p0, u0 = finals["fp64_plain"]
    for label, v in res.items():
        v["time_vs_fp64_plain"] = v["pressure_ms_per_step"] / base
        if "fp64_jacobi" in res:
            v["time_vs_fp64_jacobi"] = v["pressure_ms_per_step"] / res["fp64_jacobi"]["pressure_ms_per_step"]
        # fields after the same steps against the plain FP64 run
        v["p_rel_diff_vs_fp64_plain"] = float(np.linalg.norm(finals[label][0] - p0) / np.linalg.norm(p0))
        v["ux_rel_diff_vs_fp64_plain"] = float(np.linalg.norm(finals[label][1] - u0) / np.linalg.norm(u0))
        if w["cyl"] is not None:
            v["cx_rel_diff_vs_fp64_plain"] = abs(v["cx"] - res["fp64_plain"]["cx"]) / abs(res["fp64_plain"]["cx"])
    print(json.dumps({"study": "learned_guess", "workload": name, "train_steps": args.train,
                      "eval_steps": args.eval, "pressure_precond": PRECOND_NAMES[prm["pressure_precond"]],
                      "pressure_ordering": "multicolour", "criterion": "||b - A x|| <= 1e-8 ||b||",
                      "results": res}))


def parabola_error(xy, ux, uy, stations=(1.0, 2.0, 3.0, 3.5), umax=1.5, ly=1.0):
    """Max |u - 4 umax y (ly - y) / ly^2| / umax and max |v| / umax over the nodes within
    half a cell width of each station x (the analytic Poiseuille profile of the channel)."""
    hx = 4.0 / 256
    out = {}
    for xs in stations:
        sel = np.abs(xy[:, 0] - xs) < 0.5 * hx
        y = xy[sel, 1]
        exact = 4.0 * umax * y * (ly - y) / (ly * ly)
        out["x=%g" % xs] = {"u": float(np.abs(ux[sel] - exact).max() / umax),
                            "v": float(np.abs(uy[sel]).max() / umax), "nodes": int(sel.sum())}
    return out


def study_channel(args):
    """The 4 x 1 channel at its stated size (256 x 64 quads, level 3, Scheme A, ILU(0),
    dt 0.005, 200 steps): ms per step and the velocity profile against the analytic
    parabola at four stations along the channel, every 50 steps.  Three runs: from rest
    with ILU(0) in the natural order (the stated configuration; the profile approaches
    the parabola on the viscous time H^2 / nu = 100), from rest with ILU(0) on the
    multicolour order (the same flow, faster sweeps), and started on the parabola itself
    (the steady solution, which the step must keep)."""
    import gpupfem2_gb300 as g
    w, xy, tri, bu, bv, bp, prm = build_case("channel")
    m = g.Mesh2D.from_arrays(xy, tri)
    m.set_channel_boundary_ids(w["lx"], w["ly"], w["cyl"])
    runs = {}
    for label, kw, start in (("from_rest_ilu_natural", {}, False),
                             ("from_rest_ilu_multicolour", dict(pressure_ordering=1), False),
                             ("from_parabola_ilu_natural", {}, True)):
        eng = g.FlowEngine(m, g.default_params(**dict(prm, **kw)), bu, bv, bp, capacity_factor=4.0)
        if start:
            y = xy[:, 1]
            eng.set_field("ux", 6.0 * y * (1.0 - y))
        eng.seed()
        hist, times = [], []
        for s in range(args.channel_steps):
            _, ms = _timed(eng.step)
            times.append(ms)
            if (s + 1) % 50 == 0 or s + 1 == args.channel_steps:
                info = eng.info()
                hist.append({"step": s + 1, "t": round((s + 1) * prm["dt"], 4), "converged": int(info.converged),
                             "particles": int(info.particles),
                             "profile": parabola_error(xy, eng.field("ux"), eng.field("uy"))})
        runs[label] = {"ms_per_step_median": statistics.median(times), "profile_vs_parabola": hist}
        del eng
    print(json.dumps({"study": "channel", "steps": args.channel_steps, "triangles": int(tri.shape[0]),
                      "config": {"scheme": "A", "level": prm["level"], "pressure_precond": "ilu", "dt": prm["dt"],
                                 "mu": prm["mu"], "inflow_umax": 1.5},
                      "runs": runs}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cylinder", choices=list(WORKLOADS))
    ap.add_argument("--precond", type=int, default=None, help="pressure preconditioner override (0 J, 1 ILU, 2 IC)")
    ap.add_argument("--ordering", type=int, default=None, help="ILU/IC ordering override (0 natural, 1 multicolour)")
    ap.add_argument("--gs", type=int, default=None, help="GMRES Gram-Schmidt override (0 modified, 1 classical twice)")
    ap.add_argument("--cg", type=int, default=None,
                    help="CG variant override (0 standard, 1 one reduction, 2 pipelined)")
    ap.add_argument("--pred", type=int, default=None, help="prediction solver override (1 GMRES, 2 BiCGStab)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--clock-log", default=None, help="where the nvidia-smi clock samples go (default: a temp file)")
    ap.add_argument("--learned-train", type=int, default=60,
                    help="steps the learned initial guess trains before the metric's timed steps")
    ap.add_argument("--learned-eval", type=int, default=20,
                    help="timed steps of the mixed + learned metric (0: skip it)")
    ap.add_argument("--ref-budget", type=float, default=90.0,
                    help="reference arm: seconds of timed oracle steps at most (at least one step)")
    ap.add_argument("--ref-algorithms", type=int, default=1,
                    help="reference arm: also time one step of the reference's own solver algorithms")
    ap.add_argument("--ref-cuda-steps", type=int, default=20, help="timed steps of the reference CUDA build (0: skip)")
    ap.add_argument("--ref-cuda-warmup", type=int, default=5)
    ap.add_argument("--ref-cuda-ic-steps", type=int, default=0,
                    help="timed steps of the reference CUDA build with its IC(0) pressure solver (0: skip)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--study", default=None, choices=["solver", "learned", "channel"])
    ap.add_argument("--channel-steps", type=int, default=200)
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--train", type=int, default=40)
    ap.add_argument("--eval", type=int, default=40)
    ap.add_argument("--record", type=int, default=3)
    args = ap.parse_args()
    if args.study:
        import torch
        torch.cuda.set_device(0)
        {"solver": study_solver, "learned": study_learned, "channel": study_channel}[args.study](args)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    import torch
    import gpupfem2_gb300 as g

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    w, xy, tri, bu, bv, bp, prm = build_case(args.workload, args.precond, args.ordering, args.gs, args.cg, args.pred)
    mesh = g.Mesh2D.from_arrays(xy, tri)
    mesh.set_channel_boundary_ids(w["lx"], w["ly"], w["cyl"])
    params = g.default_params(**prm)
    # reseeding only adds particles (the reference's population check), and they gather
    # where the flow converges: room for 4x the seeded count covers about 150 steps of
    # the cylinder case (2.8x after 80 steps)
    eng = g.FlowEngine(mesh, params, bu, bv, bp, capacity_factor=4.0)
    eng.seed()
    for _ in range(args.warmup):
        eng.step()
    info = eng.info()
    torch.cuda.synchronize()
    L = g.lib()
    L.pf2_kernel_launches.restype = __import__("ctypes").c_ulonglong
    # ---- timed region: K steps, device time with CUDA events on the launching stream
    g._check(L.pf2_flow_enable_timing(eng.h, args.steps), "enable timing")
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(args.clock_log or os.path.join(tempfile.gettempdir(), "pf2_clocks_%d.csv" % os.getpid()))
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    n0 = L.pf2_kernel_launches()
    with clocks:
        start.record()
        for _ in range(args.steps):
            eng.step()
        end.record()
        torch.cuda.synchronize()
    launches = L.pf2_kernel_launches() - n0
    ms = start.elapsed_time(end) / args.steps
    if world > 1:
        ms = replica_max(ms, "cuda")
    info = eng.info()
    phase = (__import__("ctypes").c_double * 9)()
    nst = __import__("ctypes").c_int()
    g._check(L.pf2_flow_phase_times(eng.h, phase, __import__("ctypes").byref(nst)), "phase times")
    phase_ms = {PHASES[k]: phase[k] / max(nst.value, 1) for k in range(9)}
    g._check(L.pf2_flow_enable_timing(eng.h, 0), "disable timing")
    # ---- end to end through the C ABI with host buffers
    import ctypes as C
    nv = mesh.nv
    host_u = torch.empty(3 * nv, dtype=torch.float64, pin_memory=True)
    inflow = torch.tensor([val for _, val in bu], dtype=torch.float64).pin_memory()
    dev_inflow = torch.empty_like(inflow, device="cuda")
    views = [_wrap(eng.field_ptr(n), nv) for n in ("ux", "uy", "p")]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        dev_inflow.copy_(inflow, non_blocking=True)
        g._check(L.pf2_flow_set_boundary_values(eng.h, 0, g._dev(dev_inflow), g._stream()), "inflow")
        eng.step()
        for k, dv in enumerate(views):
            host_u[k * nv:(k + 1) * nv].copy_(dv, non_blocking=True)
        eng.info()
    torch.cuda.synchronize()
    e2e_ms = 1000.0 * (time.perf_counter() - t0) / args.e2e_steps
    # ---- SpMV on the flow's pressure matrix (device events, 20 launches)
    Ap, _ = eng.system(2)
    nnz = Ap.nnz
    xs = torch.ones(mesh.nv, dtype=torch.float64, device="cuda")
    ys = torch.empty_like(xs)
    g.spmv(Ap, xs, ys)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(20):
        g.spmv(Ap, xs, ys)
    e1.record()
    torch.cuda.synchronize()
    spmv_ms = e0.elapsed_time(e1) / 20
    spmv_bytes = 12.0 * nnz + 4.0 * (mesh.nv + 1) + 16.0 * mesh.nv
    # ---- full assembly (five matrices and right-hand sides from the flow's fields), timed
    # apart: the step assembles the matrices on its first step only, the right-hand sides
    # every step
    fld = {k: _wrap(eng.field_ptr(k), nv) for k in g.FIELDS}
    Ax, Ay = g.SparseMatrixCSR(mesh), g.SparseMatrixCSR(mesh)
    rx = torch.empty(nv, dtype=torch.float64, device="cuda")
    ry = torch.empty_like(rx)
    pold = fld["p_old"] if prm["scheme"] else None

    def full_assembly():
        g.assemble_velocity_prediction(mesh, params, fld["ux"], fld["uy"], fld["ux_old"], fld["uy_old"], pold,
                                       Ax, Ay, rx, ry)
        g.assemble_pressure(mesh, params, fld["pred_x"], fld["pred_y"], pold, Ax, rx)
        g.assemble_velocity_correction(mesh, params, fld["pred_x"], fld["pred_y"], fld["p"], pold, Ax, Ay, rx, ry)

    for _ in range(3):
        full_assembly()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(5):
        full_assembly()
    e1.record()
    torch.cuda.synchronize()
    full_asm_ms = e0.elapsed_time(e1) / 5
    del Ax, Ay
    # ---- roofline of the dominant phase
    peak, peak_kind = measured_peaks()
    np_ = info.particles
    pres_iters = sum(info.it_pressure[k] for k in range(prm["n_outer"]))
    dominant = max(phase_ms, key=phase_ms.get)
    n = nv
    if dominant == "pressure_solve":
        # per CG iteration: SpMV 12 nnz (values + columns) + 4 (n+1) row offsets, vectors
        # x, r, p, q, z read/written + D^-1: 8 doubles per row; ILU(0)/IC(0) adds two
        # triangular sweeps over nnz_L = (nnz + n) / 2 entries (12 B each) plus 4 B of row
        # data per row and sweep, and 32 B per row of vector traffic
        per_it = 12.0 * nnz + 4.0 * (n + 1) + 64.0 * n
        has_tri = prm["pressure_precond"] in (1, 2)
        if has_tri:
            per_it += 2.0 * (12.0 * (nnz + n) / 2.0 + 4.0 * n) + 32.0 * n
        algo = pres_iters * per_it
        unit_desc = ("bytes per CG iteration 12 nnz + 4 (n+1) + 64 n%s = %.0f, x %d iterations in %d solves"
                     % (" + 12 (nnz + n) + 40 n (triangular sweeps)" if has_tri else "", per_it, pres_iters,
                        prm["n_outer"]))
    elif dominant == "particles":
        # advect+locate 76 B/particle, scatter 12 B, gather 104 B (SoA 52 B moved in and out)
        algo = np_ * (76.0 + 12.0 + 104.0)
        unit_desc = "192 bytes per particle x %d particles" % np_
    else:
        algo = None
        unit_desc = dominant
    dom_ms = phase_ms[dominant]
    achieved = (algo / (dom_ms * 1e-3) / 1e9) if algo else None
    # DRAM traffic of one launch of the dominant kernel, from the committed ncu capture
    # (a smaller case of the same kernel, scaled by rows)
    traffic, traffic_note = None, None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if dominant == "pressure_solve" and os.path.exists(tpath):
        t = json.load(open(tpath)).get("pressure_solve")
        if t:
            traffic = t["dram_bytes_per_launch"] / t["rows"] * n
            traffic_note = t["source"]
    line = {
        "metric": "ms per PFEM-2 step", "value": ms, "unit": "ms/step", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "triangles": int(tri.shape[0]), "nodes": int(nv), "nnz": int(nnz),
                   "particles": int(np_), "pressure_precond": PRECOND_NAMES[prm["pressure_precond"]],
                   "pressure_ordering": ["natural", "multicolour"][prm.get("pressure_ordering", 0)],
                   "cg_variant": ["standard", "one_reduction", "pipelined"][prm.get("cg_variant", 0)],
                   "prediction_solver": {1: "gmres", 2: "bicgstab"}[prm.get("prediction_solver", 1)],
                   "scheme": "B" if prm["scheme"] else "A", "level": prm["level"], "n_outer": prm["n_outer"],
                   "tolerance": prm.get("tolerance", 1e-8), "max_iterations": prm.get("max_iterations", 1000),
                   "l2": "working set (particles %.1f GB) larger than L2; no flush" % (np_ * 104 / 1e9),
                   "iterations_last_step": {"prediction": [list(info.it_prediction[c])[:prm["n_outer"]]
                                                           for c in range(2)],
                                            "pressure": list(info.it_pressure)[:prm["n_outer"]],
                                            "pressure_relative_residual": list(info.pressure_residual)[
                                                :prm["n_outer"]],
                                            "correction": [list(info.it_correction[c])[:prm["n_outer"]]
                                                           for c in range(2)]},
                   "phase_ms": {k: round(v, 4) for k, v in phase_ms.items()}, "cx": info.cx, "cy": info.cy},
        "e2e": {"value": e2e_ms, "unit": "ms/step", "h2d_bytes_per_step": int(inflow.numel() * 8),
                "d2h_bytes_per_step": int(3 * nv * 8 + 8 * 5 * 8)},
        "metrics": {
            "particles_per_s": np_ / (phase_ms["particles"] * 1e-3) if phase_ms["particles"] > 0 else None,
            # the timed steps assemble right-hand sides only (five per outer iteration)
            "rhs_elements_assembled_per_s": int(tri.shape[0]) * 5 * prm["n_outer"] / (1e-3 * (
                phase_ms["prediction_assembly"] + phase_ms["pressure_assembly"] + phase_ms["correction_assembly"])),
            # five matrices with their right-hand sides, timed apart
            "matrix_elements_assembled_per_s": int(tri.shape[0]) * 5 / (1e-3 * full_asm_ms),
            "full_assembly_ms": full_asm_ms,
            "spmv_gbs": spmv_bytes / (spmv_ms * 1e-3) / 1e9, "spmv_ms": spmv_ms,
            "spmv_frac_of_hbm": spmv_bytes / (spmv_ms * 1e-3) / 1e9 / peak,
            "pressure_iterations_per_solve": pres_iters / prm["n_outer"],
            "pressure_ms_per_solve": phase_ms["pressure_solve"] / prm["n_outer"]},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel_phase": dominant, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "traffic_per": "bytes per launch (one pressure solve)", "traffic_source": traffic_note,
                     "peak_source": peak_kind, "algorithmic": unit_desc},
        "clocks": clocks.summary(),
    }
    if prm.get("prediction_solver", 1) == 1:
        line["config"]["gmres_gram_schmidt"] = ["modified", "classical_twice"][prm.get("gmres_orthogonalization", 0)]
    if rank == 0 and args.ref_cuda_steps > 0:
        rc = reference_cuda(args.workload, xy, tri, prm, "jacobi", args.ref_cuda_warmup, args.ref_cuda_steps)
        if rc is not None:
            if "ms_per_step" in rc:
                rc["speedup_of_engine"] = rc["ms_per_step"] / ms
                rc["target_speedup"] = 3.0
                # the engine with the reference case's own solver choices (Jacobi CG for the
                # pressure, GMRES(Jacobi) with modified Gram-Schmidt for the prediction), the
                # same warm-up: the like-for-like ratio
                same = dict(prm, pressure_precond=0, pressure_ordering=0, prediction_solver=1,
                            gmres_orthogonalization=0, cg_variant=0)
                e2 = g.FlowEngine(mesh, g.default_params(**same), bu, bv, bp, capacity_factor=4.0)
                e2.seed()
                for _ in range(args.warmup):
                    e2.step()
                torch.cuda.synchronize()
                (_, ms2) = _timed(lambda: [e2.step() for _ in range(args.ref_cuda_steps)])
                ms2 /= args.ref_cuda_steps
                rc["engine_with_reference_solvers_ms_per_step"] = ms2
                rc["speedup_of_engine_same_solvers"] = rc["ms_per_step"] / ms2
                del e2
            line["reference_cuda"] = rc
        if rc is not None and args.ref_cuda_ic_steps > 0:
            ric = reference_cuda(args.workload, xy, tri, prm, "ic", 2, args.ref_cuda_ic_steps)
            if ric and "ms_per_step" in ric:
                ric["speedup_of_engine"] = ric["ms_per_step"] / ms
            line["reference_cuda_ic"] = ric
    if rank == 0 and args.learned_eval > 0 and args.workload in ("cylinder", "cylinder_quarter"):
        line["metrics"]["pcg_mixed_learned_vs_fp64"] = learned_metric(args, mesh, bu, bv, bp, prm)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.workload, prm, eng, xy, tri, bu, bv, bp)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def _wrap(ptr, n):
    """A device tensor view of n doubles at ptr (through the CUDA array interface)."""
    import torch

    class _A:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 3}

    return torch.as_tensor(_A(), device="cuda")


if __name__ == "__main__":
    main()
