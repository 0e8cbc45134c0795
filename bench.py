"""Benchmark: SSA velocity solves per second on one GB300 (UFEMISM ice-velocity solve).

Workload: the 200k-vertex dome (2 km at the margin grading to 20 km, seeded jitter; about
800k AaAc rows), Vialov dome H0 = 3600 m, R = 750 km, flat bed, A = 1e-16 Pa^-3 yr^-1, linear
sliding beta^2 = 1e3 Pa yr/m, Picard tolerance 1e-3, SOR omega 1.3, SOR tolerance 1e-4 m/yr.
One step = one full cold-start solve_SSA (every Picard iteration and SOR sweep until the
reference's stopping rules fire).

  value   mixed-precision solves/s, inputs resident in HBM (ufe_ssa_run)
  e2e     the same through ufe_ssa_solve with host buffers (H2D + solve + D2H each step; the
          host arrays are allocated once and reused, as a model reuses its state arrays)
  fp64    the plain FP64 path, same workload
  roofline  the persistent SSA kernel: algorithmic bytes per launch / launch time vs HBM peak

``--impl reference`` times the reference algorithm on the host cores: the CPU oracle (a C
restatement of the Fortran routines; the Fortran reference cannot be built on this image) runs
full cold-start solves of the same workload, which it builds itself (mesh, neighbour functions,
colouring, geometry) without loading this library. The K timed steps are K consecutive pieces
(by SOR sweep count) of one full solve, so together they are exactly one solve and the value
is measured, not extrapolated; the warm-up is one full solve before it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SSA solves/s mixed vs FP64 on GB300 @ rel-L2<=1e-6; sweep HBM GB/s; adjoint ms"
UNIT = "solves/s"
WORKLOAD = "%s-vertex dome SSA cold-start solve"   # formatted with the mesh size (default 200k)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(size: str):
    from ufemism_gb300 import api, workloads
    from ufemism_gb300.meshgen import dome_mesh
    base = dome_mesh(size)
    mesh = api.build_aaac(base)
    Hi, Hb, SL = workloads.dome_geometry(base)
    ssa, sia = workloads.prepare_inputs(mesh, Hi, Hb, SL)
    return base, mesh, ssa, sia


def mesh_counts(mesh):
    nV = mesh.base.nV
    nA = mesh.nVAaAc
    is_edge = np.concatenate([mesh.base.edge_index > 0, mesh.edge_index_Ac > 0])
    nnz_all = int(mesh.nCAaAc.sum())
    nnz_act = int(mesh.nCAaAc[~is_edge].sum())
    n_act = int((~is_edge).sum())
    n_edge = int(is_edge.sum())
    # Neumann lists: edge rows' non-edge neighbours (+ corners' neighbours)
    nb_bnd = 0
    for ai in np.flatnonzero(is_edge):
        nb = mesh.CAaAc[ai, : mesh.nCAaAc[ai]] - 1
        nb_bnd += int((~is_edge[nb]).sum()) if ai >= 4 else len(nb)
    return dict(nV=nV, nA=nA, nnz_all=nnz_all, nnz_act=nnz_act, n_act=n_act, n_edge=n_edge, nb_bnd=nb_bnd)


def algorithmic_bytes(c, st, mixed: bool, refold: int = 256):
    """Compulsory DRAM bytes of one persistent-kernel launch (each array touched once per
    phase; neighbour gathers of U,V counted once through the row's own U,V)."""
    if not mixed:
        sweep = c["n_act"] * (16 + 16 + 16 + 16 + 8 + 1) + c["nnz_act"] * (4 + 16)
    else:
        sweep = c["n_act"] * (8 + 8 + 8 + 8 + 4 + 1) + c["nnz_act"] * (4 + 8)
    bnd = c["n_edge"] * (16 + 4) + c["nb_bnd"] * 4 + (c["n_edge"] * (8 if mixed else 0))
    sweep += bnd
    # viscosity: U,V + home coefs + A + H + eta + N (w) + Nprev (r) + deg; entries col + (Nx,Ny)
    visc = c["nA"] * (16 + 16 + 8 + 8 + 8 + 8 + 8 + 1) + c["nnz_all"] * (4 + (8 if mixed else 16))
    # coefficients: U,V + tau/beta + eta + H + Hb + SL + hx + hy + home cuv -> S, rhs, euv (+euv32)
    coef = c["nA"] * (16 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 16 + 8) + c["n_act"] * (16 + 16 + (8 if mixed else 0))
    total = st["total_sweeps"] * sweep + st["picard_iterations"] * visc + st["linear_solves"] * coef
    if mixed:
        defect = c["n_act"] * (16 + 8 + 16 + 16 + 8 + 1) + c["nnz_act"] * (4 + 16)
        fold = c["nA"] * (8 + 16 + 16 + 8)
        n_refold = sum(max(0, (s - 1) // refold) for s in st["sweeps"]) if st.get("sweeps") else 0
        total += (st["linear_solves"] + n_refold) * defect + (st["linear_solves"] + n_refold) * fold
    return int(total), int(sweep)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        try:
            rows = [l.strip().split(", ") for l in open(self.path) if l.strip()]
        except Exception:
            return out
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        out.update(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(mx) if mx else None,
                   reasons=sorted(reasons), samples=len(rows))
        try:
            os.unlink(self.path)
        except Exception:
            pass
        return out


L2_FLUSH_BYTES = 256 << 20   # twice the GB300's L2


def timed_runs(dm, params, steps, warmup, stream_ptr):
    """Device-resident solves: ufe_ssa_run on the uploaded inputs, timed with CUDA events
    recorded on the handle's stream, with L2 flushed (a 256 MB write on the same stream)
    before every timed step. Returns per-step ms and the stats of the last run."""
    import torch
    stream = torch.cuda.ExternalStream(stream_ptr)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    st = None
    for _ in range(warmup):
        rc, st = dm.ssa_run(params)
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.fill_(1)
        e0.record(stream)
        rc, st = dm.ssa_run(params)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    return times, st


def oracle_workload(size: str):
    """The benchmark workload built by the oracle alone: the seeded base mesh, the oracle's Ac
    mesh, neighbour functions and five-colouring, and the geometry of
    update_general_ice_model_data from its restatement. This library is not loaded."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from ufemism_gb300 import workloads
    from ufemism_gb300.meshgen import dome_mesh
    base = dome_mesh(size)
    om = orc.build_aaac(base)
    Hi, Hb, SL = workloads.dome_geometry(base)
    g = orc.update_geometry(om, Hi, Hb, SL)
    A = workloads.A_FLOW
    ssa = dict(Hi=Hi, Hb=Hb, SL=SL, dHs_dx_shelf=g["dHs_dx_shelf"], dHs_dy_shelf=g["dHs_dy_shelf"],
               A_flow_mean=np.full(base.nV, A), mask_sheet=g["mask_sheet"], Hi_Ac=g["Hi_Ac"], Hb_Ac=g["Hb_Ac"],
               SL_Ac=g["SL_Ac"], dHs_dx_shelf_Ac=g["dHs_dx_shelf_Ac"], dHs_dy_shelf_Ac=g["dHs_dy_shelf_Ac"],
               A_flow_mean_Ac=np.full(om.nAc, A))
    return orc, base, om, ssa


def oracle_solve_timed(orc, om, ssa, threads, pieces=1, total_sweeps=None):
    """One full cold-start FP64 solve by the oracle on ``threads`` host threads (OpenMP over
    the rows of one colour, the reference's own per-colour decomposition), timed on the host.
    With ``pieces`` > 1 and the solve's sweep count known, the solve is also timed in that
    many consecutive pieces of equal sweep count: the oracle publishes its running sweep
    total after every sweep, and a watcher thread stamps each boundary as it is crossed.
    Returns (rc, outputs, stats, seconds, per-piece seconds)."""
    prog = np.zeros(1, dtype=np.int64)
    p = orc.default_params(n_threads=threads, progress=prog)
    res = {}
    th = threading.Thread(target=lambda: res.setdefault("r", orc.solve_ssa(om, ssa, p)))
    marks = []
    t0 = time.perf_counter()
    th.start()
    if pieces > 1 and total_sweeps:
        for i in range(1, pieces):
            target = (i * total_sweeps) // pieces
            while th.is_alive() and int(prog[0]) < target:
                time.sleep(2e-4)
            marks.append(time.perf_counter())
    th.join()
    t1 = time.perf_counter()
    marks.append(t1)
    rc, out, st = res["r"]
    return rc, out, st, t1 - t0, np.diff(np.array([t0] + marks))


def workload_config(size, base, nVAaAc, nnz):
    """The config keys both arms report: what the workload is, not how an arm runs it."""
    return {"workload": WORKLOAD % size, "nV": int(base.nV), "nVAaAc": int(nVAaAc), "nnz": int(nnz),
            "geometry": "Vialov dome H0 3600 m, R 750 km, flat bed, grounded",
            "sliding": "linear beta^2=1e3", "A_flow": 1e-16,
            "solver": "cold start; Picard tol 1e-3 (<= 50); SOR omega 1.3, tol 1e-4 m/yr (<= 10000 sweeps)",
            "l2": "GPU arm: L2 flushed (256 MB write) before every timed step"}


def cpu_baseline(size, threads=None):
    """The oracle (C restatement of the reference's FP64 solve) on the host cores: one full
    cold-start solve of the same workload, on a mesh and inputs it builds itself, timed
    directly (no extrapolation). Also returns its solution, the checker of the GPU results."""
    threads = threads or os.cpu_count() or 1
    orc, base, om, ssa = oracle_workload(size)
    rc, out, st, secs, _ = oracle_solve_timed(orc, om, ssa, threads)
    info = dict(value=1.0 / secs, unit=UNIT, cores=threads, kind="port",
                sample="one full cold-start FP64 solve of the %s-vertex dome by the oracle (C restatement of the "
                       "reference's Fortran routines, OpenMP over the rows of each colour) on %d host threads: "
                       "%.1f s, %d Picard iterations, %d SOR sweeps; measured, not extrapolated"
                       % (size, threads, secs, st["picard_iterations"], st["total_sweeps"]))
    return info, rc, out, st


def run_reference(args):
    """The reference arm: the oracle's full cold-start solves on all host cores. Warm-up: one
    full solve (which also gives the sweep count that splits the next one). Timed: one full
    solve in ``--steps`` consecutive pieces of equal sweep count; value = 1 / the solve's time."""
    rank, world, local = dist_info()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    orc, base, om, ssa = oracle_workload(args.size)
    nnz = int(np.asarray(om.nCAaAc).sum())
    rc_w, _, st_w, secs_w, _ = oracle_solve_timed(orc, om, ssa, threads)
    rc, out, st, secs, pieces = oracle_solve_timed(orc, om, ssa, threads, pieces=args.steps,
                                                   total_sweeps=st_w["total_sweeps"])
    value = 1.0 / secs
    sample = ("per step: one of %d consecutive pieces (equal SOR sweep counts) of one full cold-start FP64 solve "
              "of the %s-vertex dome by the oracle (C restatement of the reference's Fortran routines, OpenMP "
              "over the rows of each colour) on %d host threads; the %d steps together are exactly one solve "
              "(%.1f s, %d Picard iterations, %d sweeps); warm-up: one full solve (%.1f s)"
              % (args.steps, args.size, threads, args.steps, secs, st["picard_iterations"], st["total_sweeps"],
                 secs_w))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": float(np.mean(pieces)) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded dome geometry and mesh)",
        "config": workload_config(args.size, base, om.nVAaAc, nnz),
        "impl": "reference",
        "precision": "fp64", "status": rc, "picard_iterations": st["picard_iterations"],
        "sor_sweeps": st["total_sweeps"], "sweeps_per_linear_solve": st["sweeps"],
        "full_solve_s": secs, "warmup_solve_s": secs_w, "step_ms": [1e3 * float(x) for x in pieces],
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def adjoint_summary(dm, mesh, ssa, p, forward_ms):
    """The metric's third quantity on the line's own workload: the VJP (ufe_ssa_vjp, GMRES on
    transposed coloured sweeps) of the default-tolerance mixed forward solve, for
    J = 1/2 sum over AaAc of |u - u_obs|^2 with u_obs from a forward solve whose log(beta^2) is
    perturbed by a Gaussian random field (std 0.3, 100 km), timed with CUDA events on the
    device and set against that forward solve's time; and its agreement with central finite
    differences (h = 1e-4, 4 random directions) on a small marine case solved to tight
    tolerances, where the forward's truncation error does not mask the gradient."""
    from ufemism_gb300 import _native as nat
    from ufemism_gb300 import api, workloads
    from ufemism_gb300.meshgen import dome_mesh
    lbo = np.log(1e3) + workloads.log_beta_field(mesh, std=0.3, ell=100e3, seed=20261210, mean=0.0)
    rc, oo, so = dm.solve_ssa(dict(ssa, beta_sq_AaAc=np.exp(lbo)), p, check=False)
    rc, out, st = dm.solve_ssa(ssa, p, check=False)     # the solve the VJP differentiates
    dJ = {k: out[k] - oo[k] for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac")}
    vms = []
    for _ in range(3):
        rcv, g, vs = dm.ssa_vjp(dJ, p, check=False)
        vms.append(vs["device_ms"])
    res = {"workload": "the line's workload; VJP of the mixed default-tolerance forward solve",
           "vjp_ms": float(np.median(vms)), "vjp_status": rcv, "vjp_gmres_sweeps": vs["sweeps"],
           "vjp_rel_residual": vs["last_rel_update"], "forward_ms": forward_ms,
           "vjp_over_forward": float(np.median(vms)) / forward_ms}
    # finite differences on the 1k marine case, forward solved tightly in FP64
    base = dome_mesh("1k")
    m1 = api.build_aaac(base)
    Hi, Hb, SL = workloads.marine_geometry(base, seed=20261206)
    f1, _ = workloads.prepare_inputs(m1, Hi, Hb, SL)
    d1 = api.DeviceMesh(m1)
    tight = api.default_params(precision=nat.UFE_FP64, SSA_RN_tol=1e-13, SSA_max_residual_UV=1e-11,
                               SSA_max_outer_loops=300, SSA_max_inner_loops=1000000)
    lb = workloads.log_beta_field(m1, std=1.0, ell=100e3, seed=5)

    def fwd(l):
        rc1, o1, _ = d1.solve_ssa(dict(f1, beta_sq_AaAc=np.exp(l)), tight, check=False)
        return np.concatenate([o1["U_SSA"], o1["Ux_SSA_Ac"]]), np.concatenate([o1["V_SSA"], o1["Uy_SSA_Ac"]])

    Uo, Vo = fwd(lb + workloads.log_beta_field(m1, std=0.3, ell=100e3, seed=11, mean=0.0))
    U, V = fwd(lb)
    nV = base.nV
    rcv, g1, _ = d1.ssa_vjp({"U_SSA": (U - Uo)[:nV], "Ux_SSA_Ac": (U - Uo)[nV:], "V_SSA": (V - Vo)[:nV],
                             "Uy_SSA_Ac": (V - Vo)[nV:]}, tight, check=False)
    J = lambda a, b: 0.5 * float(np.sum((a - Uo) ** 2 + (b - Vo) ** 2))
    rng = np.random.default_rng(20261212)
    errs = []
    for _ in range(4):
        dvec = rng.normal(size=m1.nVAaAc)
        fd = (J(*fwd(lb + 1e-4 * dvec)) - J(*fwd(lb - 1e-4 * dvec))) / 2e-4
        an = float(g1["dJ_dlogbeta_sq_AaAc"] @ dvec)
        errs.append(abs(fd - an) / abs(an))
    d1.close()
    res["fd_check"] = {"workload": "1k-vertex marine, FP64 forward to Picard 1e-13 / SOR 1e-11, dJ/dlog(beta^2)",
                       "directions": len(errs), "h": 1e-4, "rel_err_max": max(errs)}
    return res


def profile_case(args):
    """One capped solve for profiler captures: a single linear solve of exactly
    ``--profile-sweeps`` SOR sweeps (SSA_max_outer_loops = 1) on the chosen workload size,
    repeated ``--steps`` times after ``--warmup`` untimed runs."""
    import torch
    from ufemism_gb300 import _native as nat
    from ufemism_gb300 import api
    api.init(0)
    base, mesh, ssa, sia = make_workload(args.size)
    dm = api.DeviceMesh(mesh)
    prec = {"mixed": nat.UFE_MIXED, "fp64": nat.UFE_FP64, "exact": nat.UFE_FP64}[args.profile_case]
    p = api.default_params(precision=prec, SSA_max_outer_loops=1, SSA_max_inner_loops=args.profile_sweeps,
                           fp64_exact=1 if args.profile_case == "exact" else 0,
                           mixed_refold_sweeps=args.refold_sweeps)
    dm.ssa_upload(ssa, p)
    L = nat.load()
    timers = hasattr(L, "ufe_debug_phase_cycles")
    if timers:
        import ctypes as ct
        NT = 14   # 8 categories, the sweep count, the 5 colour phases of the halo sweeps
        buf = (ct.c_ulonglong * (NT + 1024 * NT))()
        L.ufe_debug_phase_cycles.restype = ct.c_int
        L.ufe_debug_phase_cycles(buf, NT + 1024 * NT, 1)
    times, st = timed_runs(dm, p, args.steps, args.warmup, dm.stream)
    ms = float(np.mean(times))
    line = {"profile_case": args.profile_case, "size": args.size, "sweeps": st["total_sweeps"],
            "ms_per_solve": ms, "us_per_sweep": 1e3 * ms / max(1, st["total_sweeps"])}
    if timers:
        # totals over CTAs and over the warm-up and timed runs; shares of the per-CTA time, and
        # the same shares of the measured time per sweep
        n = L.ufe_debug_phase_cycles(buf, NT + 1024 * NT, 1)
        names = ["wait_colour", "colour", "arrive", "wait_boundary", "boundary", "decide", "grid_barrier", "other"]
        cyc = np.array([buf[i] for i in range(len(names))], dtype=np.float64)
        sweeps_cta = float(buf[len(names)])
        share = cyc / cyc.sum()
        line["phase_timers"] = {
            "runs": args.steps + args.warmup, "cta_sweeps": sweeps_cta,
            "share": {k: float(v) for k, v in zip(names, share)},
            "us_per_sweep": {k: float(v) * line["us_per_sweep"] for k, v in zip(names, share)},
            "cycles_per_cta_sweep": {k: float(v) / max(sweeps_cta, 1.0) for k, v in zip(names, cyc)}}
        # per CTA: the time it spends working (not waiting for other CTAs) per sweep
        per = np.array([buf[NT + i] for i in range(1024 * NT)], dtype=np.float64).reshape(1024, NT)
        per = per[per[:, 8] > 0]
        waits = per[:, 0] + per[:, 3] + per[:, 5] + per[:, 6]
        tot = per[:, :8].sum(axis=1)
        busy = (tot - waits) / per[:, 8]
        us = line["us_per_sweep"] / (tot / per[:, 8]).mean()
        line["phase_timers"]["colour_phase_us"] = [float((per[:, 9 + f] / per[:, 8]).mean() * us) for f in range(5)]
        line["phase_timers"]["colour_phase_us_max"] = [float((per[:, 9 + f] / per[:, 8]).max() * us) for f in range(5)]
        line["phase_timers"]["busy_us_per_sweep_per_cta"] = {
            "min": float(busy.min() * us), "mean": float(busy.mean() * us), "max": float(busy.max() * us),
            "slowest_ctas": [int(i) for i in np.argsort(-busy)[:8]],
            "colour_us_by_cta_max": float((per[:, 1] / per[:, 8]).max() * us),
            "boundary_us_by_cta_max": float((per[:, 4] / per[:, 8]).max() * us),
            "all_busy_us": [round(float(b * us), 2) for b in busy],
            "per_cta_us": {k: [round(float(v * us), 2) for v in per[:, i] / per[:, 8]]
                           for i, k in enumerate(names)}}
    print(json.dumps(line))
    dm.close()
    return 0


def ensemble_bench(args):
    """Batched ensemble: ``--members`` independent mixed-precision SSA solves on meshes of
    2k-50k vertices (log-uniform), dome thickness with H0 in [2000, 4000] m and a log-normal
    friction field per member, solved in one persistent launch (CUDA graph replay) and
    compared with a loop of single solves of the same members. Under torchrun every rank
    solves its share of the members (greedy cost partition); value = all members / the
    slowest rank's time."""
    from ufemism_gb300 import ensemble as ens
    from ufemism_gb300 import workloads as wl
    rank, world, local = dist_info()
    sizes = wl.ensemble_sizes(args.members)
    parts = ens.partition(ens.member_cost(4 * sizes), world)
    mine = parts[rank]
    t_build = time.time()
    members = ens.build_members(sizes[mine], [ens.member_seed(i) for i in mine])
    t_build = time.time() - t_build
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from ufemism_gb300 import _native as nat
    from ufemism_gb300 import api
    api.init(local)
    p = api.default_params(precision=nat.UFE_MIXED)
    tuned = None
    if args.autotune:
        cfg, tried = api.batch_autotune(members, p)
        tuned = {"best": cfg, "tried": tried}
    else:
        cfg = dict(team_ctas=0, rows_per_cta=args.rows_per_cta, block=args.block, use_graph=1)
    b = api.Batch([m for _, m, _ in members], team_ctas=cfg["team_ctas"], rows_per_cta=cfg["rows_per_cta"],
                  block=cfg["block"], use_graph=True)
    for i, (_, _, f) in enumerate(members):
        b.upload(i, f, p)
    for _ in range(args.warmup):
        b.run(p)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = []
        for _ in range(args.steps):
            rc, stats, tm = b.run(p)
            ms.append(tm["device_ms"])
    clocks = clk.summary()
    batch_ms = float(np.mean(ms))
    # e2e: every step uploads each member's inputs from host arrays, solves the batch and
    # downloads each member's results
    h2d = d2h = 0
    for base, mesh, f in members:
        h2d += sum(np.asarray(v).nbytes for k, v in f.items() if v is not None and k in nat.SSA_IN_FIELDS)
        h2d += 8 * (2 * base.nV + 2 * mesh.nAc + mesh.nVAaAc)
        d2h += 8 * (2 * base.nV + 4 * mesh.nAc + 5 * mesh.nVAaAc)
    # Each member's host arrays are allocated once and reused every step, as a model's state
    # arrays are; resetting them to a cold start is inside the timed region.
    bufs = [api.ssa_buffers(base.nV, mesh.nAc, mesh.nVAaAc) for base, mesh, _ in members]
    e2e = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k, (_, _, f) in enumerate(members):
            for name in api.SSA_INOUT_FIELDS:
                bufs[k][name].fill(0.0)
            b.upload(k, f, p, buffers=bufs[k])
        b.run(p)
        for k in range(len(members)):
            b.download(k, buffers=bufs[k])
        if i >= args.warmup:
            e2e.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = float(np.mean(e2e))
    # the same members as a loop of single solves (each on its own default layout)
    single_ms = []
    single_sweeps = []
    for base, mesh, f in members:
        dm = api.DeviceMesh(mesh)
        dm.ssa_upload(f, p)
        dm.ssa_run(p)
        rc1, st1 = dm.ssa_run(p)
        single_ms.append(st1["device_ms"])
        single_sweeps.append(st1["total_sweeps"])
        dm.close()
    loop_ms = float(np.sum(single_ms))
    same = all(s["total_sweeps"] == q for s, q in zip(stats, single_sweeps))
    b.close()
    vals = torch.tensor([batch_ms, loop_ms, e2e_ms], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(vals, op=torch.distributed.ReduceOp.MAX)
    batch_ms, loop_ms, e2e_ms = (float(x) for x in vals.tolist())
    n_total = int(args.members)
    sm = np.sort(single_ms)
    line = {
        "metric": "SSA ensemble solves/s (batched, mixed)", "value": 1e3 * n_total / batch_ms, "unit": "solves/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": batch_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 sweeps / f64 defect",
        "data": "synthetic (seeded meshes, dome thickness, log-normal friction)",
        "config": {"workload": "ensemble of %d dome solves, 2k-50k vertices log-uniform, H0 U[2000,4000] m, "
                               "log beta^2 GRF(ln 1e3, 1.0, 100 km)" % n_total,
                   "batch_config": cfg, "autotuned_this_run": bool(args.autotune),
                   "members_on_rank0": len(mine), "total_vertices": int(np.sum(sizes)),
                   "l2": "members' arrays together exceed L2; no flush",
                   "parallelism": "members sharded over ranks" if world > 1 else "1 GPU"},
        "member_p50_ms": tm["member_p50_ms"], "member_p99_ms": tm["member_p99_ms"],
        "member_max_ms": tm["member_max_ms"], "grid_ctas": tm["grid_ctas"], "n_classes": tm["n_classes"],
        "loop_of_single_solves": {"value": 1e3 * n_total / loop_ms, "unit": "solves/s", "total_ms": loop_ms,
                                  "p50_ms": float(sm[len(sm) // 2]),
                                  "p99_ms": float(sm[min(len(sm) - 1, int(np.ceil(0.99 * len(sm))) - 1)])},
        "batched_vs_loop_speedup": loop_ms / batch_ms,
        "iteration_counts_match_single_solves": bool(same),
        "e2e": {"value": 1e3 * n_total / e2e_ms, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        # per member k_gather + k_scatter, and the one persistent batched launch
        "gpu_launches": (2 * len(members) + 1) * args.steps,
        "clocks": clocks,
        "host_build_s": t_build,
    }
    if tuned:
        line["autotune"] = tuned["tried"]
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def marine_bench(args):
    """Marine ice sheet with a floating shelf (bed sloping from +500 m to -1000 m plus a
    seeded Gaussian random field, sigma 50 m, correlation 40 km; thickness from the dome
    profile, floating where is_floating), mixed precision timed against FP64 on the same
    mesh; linear sliding beta^2 = 1e3 under grounded ice, none under the shelf."""
    import torch
    from ufemism_gb300 import _native as nat
    from ufemism_gb300 import api, workloads
    from ufemism_gb300.meshgen import dome_mesh
    size = args.size if args.size != "200k" else "300k"
    base = dome_mesh(size)
    mesh = api.build_aaac(base)
    Hi, Hb, SL = workloads.marine_geometry(base, seed=20261208)
    ssa, _ = workloads.prepare_inputs(mesh, Hi, Hb, SL)
    torch.cuda.set_device(0)
    api.init(0)
    dm = api.DeviceMesh(mesh)
    p64 = api.default_params(precision=nat.UFE_FP64)
    p32 = api.default_params(precision=nat.UFE_MIXED)
    rc64, o64, s64 = dm.solve_ssa(ssa, p64, check=False)
    rc32, o32, s32 = dm.solve_ssa(ssa, p32, check=False)
    l2 = max(float(np.linalg.norm(o32[k] - o64[k]) / np.linalg.norm(o64[k]))
             for k in ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac"))
    dm.ssa_upload(ssa, p64)
    with ClockSampler(0) as clk:
        t64, st64 = timed_runs(dm, p64, args.steps, args.warmup, dm.stream)
        t32, st32 = timed_runs(dm, p32, args.steps, args.warmup, dm.stream)
    ms32, ms64 = float(np.mean(t32)), float(np.mean(t64))
    floating = workloads._is_floating(Hi, Hb, SL) & (Hi > 0)
    line = {
        "metric": "SSA solves/s (marine, mixed)", "value": 1e3 / ms32, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 sweeps / f64 defect",
        "data": "synthetic (seeded mesh, sloping bed with Gaussian random field)",
        "config": {"workload": "%s-vertex marine ice sheet with floating shelf" % size, "nV": int(base.nV),
                   "nVAaAc": int(mesh.nVAaAc), "floating_vertices": int(floating.sum()),
                   "picard_iterations": st32["picard_iterations"], "sor_sweeps": st32["total_sweeps"],
                   "status": st32["status"], "parallelism": "1 GPU"},
        "fp64": {"value": 1e3 / ms64, "ms_per_step": ms64, "sor_sweeps": st64["total_sweeps"],
                 "picard_iterations": st64["picard_iterations"], "status": st64["status"]},
        "mixed_vs_fp64_speedup": ms64 / ms32, "rel_l2_mixed_vs_fp64": l2,
        "vertex_sweeps_per_s": mesh.nVAaAc * st32["total_sweeps"] / (ms32 * 1e-3),
        "gpu_launches": 3 * args.steps, "clocks": clk.summary(),
    }
    print(json.dumps(line))
    dm.close()
    return 0


def adjoint_bench(args):
    """Adjoint on the marine setup: u_obs from a forward solve with log(beta^2) perturbed by
    a Gaussian random field (std 0.3), J = 1/2 sum over AaAc of the squared velocity misfit,
    gradient with respect to log(beta^2) (AaAc) and Hi (Aa) by ufe_ssa_vjp at the converged
    state of a forward solve run to tight tolerances; cost against that forward solve, and
    central finite differences (h = 1e-4) of the forward solve on random directions."""
    import torch
    from ufemism_gb300 import _native as nat
    from ufemism_gb300 import api, workloads
    from ufemism_gb300.meshgen import dome_mesh
    size = args.size if args.size != "200k" else "100k"
    base = dome_mesh(size)
    mesh = api.build_aaac(base)
    Hi, Hb, SL = workloads.marine_geometry(base, seed=20261208)
    ssa, _ = workloads.prepare_inputs(mesh, Hi, Hb, SL)
    lb = workloads.log_beta_field(mesh, std=1.0, ell=100e3, seed=20261209)
    lbo = lb + workloads.log_beta_field(mesh, std=0.3, ell=100e3, seed=20261210)
    torch.cuda.set_device(0)
    api.init(0)
    dm = api.DeviceMesh(mesh)
    # The SOR tolerance is absolute (m/yr); below ~1e-10 it is under the FP64 floor of the
    # defect for velocities of a few km/yr and would never be met.
    tight = dict(SSA_RN_tol=args.adj_rn_tol, SSA_max_residual_UV=max(args.adj_rn_tol / 10, 1e-10),
                 SSA_max_outer_loops=400, SSA_max_inner_loops=2000000)
    p64 = api.default_params(precision=nat.UFE_FP64, **tight)
    p32 = api.default_params(precision=nat.UFE_MIXED, **tight)

    def forward(lbeta, p, warm=None):
        f = dict(ssa)
        f["beta_sq_AaAc"] = np.exp(lbeta)
        rc, out, st = dm.solve_ssa(f, p, warm=warm, check=False)
        U = np.concatenate([out["U_SSA"], out["Ux_SSA_Ac"]])
        V = np.concatenate([out["V_SSA"], out["Uy_SSA_Ac"]])
        return U, V, out, st

    Uo, Vo, _, _ = forward(lbo, p32)
    res = {}
    for name, p in (("fp64", p64), ("mixed", p32)):
        U, V, out, st = forward(lb, p)
        print("forward %s: %.1f ms, %d Picard, %d sweeps, RN %.2e" % (name, st["device_ms"], st["picard_iterations"],
                                                                       st["total_sweeps"], st["last_RN"]),
              file=sys.stderr, flush=True)
        dJ = dict(U_SSA=out["U_SSA"] - Uo[:base.nV], V_SSA=out["V_SSA"] - Vo[:base.nV],
                  Ux_SSA_Ac=out["Ux_SSA_Ac"] - Uo[base.nV:], Uy_SSA_Ac=out["Uy_SSA_Ac"] - Vo[base.nV:])
        rc, g, vs = dm.ssa_vjp(dJ, p, geom_mesh=mesh, tol=args.adj_tol, check=False)
        res[name] = dict(forward_ms=st["device_ms"], forward_sweeps=st["total_sweeps"],
                         picard=st["picard_iterations"], vjp_ms=vs["device_ms"], vjp_sweeps=vs["sweeps"],
                         vjp_status=rc, vjp_rel_residual=vs["last_rel_update"],
                         vjp_over_forward=vs["device_ms"] / st["device_ms"], grad=g, U=U, V=V, out=out)
    # finite differences with the mixed forward (converged to the FP64 fixed point), every
    # perturbed solve from a cold start like the unperturbed one: the SOR's stopping rule
    # (an absolute update below the tolerance) leaves an error of about tolerance / (1 - rate)
    # in the slowest mode, which cancels in the difference only when both solves follow the
    # same path (warm starts from the unperturbed solution measured 1e-4 disagreement).
    rng = np.random.default_rng(20261211)
    g = res["mixed"]["grad"]
    warm = None
    J = lambda U, V: 0.5 * float(np.sum((U - Uo) ** 2 + (V - Vo) ** 2))
    fd = []
    t_fd = time.time()
    for k in range(args.fd_directions):
        d = rng.normal(size=mesh.nVAaAc)
        Up, Vp, _, stp = forward(lb + 1e-4 * d, p32, warm)
        Um, Vm, _, stm = forward(lb - 1e-4 * d, p32, warm)
        print("fd direction %d: %.1f + %.1f ms, %d + %d sweeps" % (k, stp["device_ms"], stm["device_ms"],
                                                                   stp["total_sweeps"], stm["total_sweeps"]),
              file=sys.stderr, flush=True)
        f = (J(Up, Vp) - J(Um, Vm)) / 2e-4
        a = float(g["dJ_dlogbeta_sq_AaAc"] @ d)
        fd.append(abs(f - a) / abs(a))
    g64, g32 = res["fp64"]["grad"], res["mixed"]["grad"]
    agree = float(np.linalg.norm(g64["dJ_dlogbeta_sq_AaAc"] - g32["dJ_dlogbeta_sq_AaAc"]) /
                  np.linalg.norm(g64["dJ_dlogbeta_sq_AaAc"]))
    line = {
        "metric": "adjoint ms (VJP of the converged marine solve)", "value": res["fp64"]["vjp_ms"], "unit": "ms",
        "n_gpus": 1, "higher_is_better": False, "dtype": "f64", "data": "synthetic (seeded marine setup)",
        "config": {"workload": "%s-vertex marine, gradient w.r.t. log beta^2 and Hi" % size, "nV": int(base.nV),
                   "nVAaAc": int(mesh.nVAaAc), "forward_rn_tol": args.adj_rn_tol, "vjp_tol": args.adj_tol},
        "vjp_over_forward_fp64": res["fp64"]["vjp_over_forward"],
        "vjp_over_forward_mixed": res["mixed"]["vjp_over_forward"],
        "forward": {k: {q: v[q] for q in ("forward_ms", "forward_sweeps", "picard", "vjp_ms", "vjp_sweeps",
                                          "vjp_status", "vjp_rel_residual")} for k, v in res.items()},
        "vjp_method": "GMRES(100), 8 transposed sweeps per iteration",
        "gradient_fp64_vs_mixed_forward_rel_l2": agree,
        "fd_directions": args.fd_directions, "fd_rel_err_max": max(fd) if fd else None, "fd_rel_err": fd,
        "fd_seconds": time.time() - t_fd,
    }
    print(json.dumps(line))
    dm.close()
    return 0


def step_bench(args):
    """One time step of the velocity path through the C-ABI, every input and output a host array:
    device geometry preparation from Hi, Hb, SL (update_general_ice_model_data) and the SSA
    upload -> SSA solve (mixed) -> SIA on the device geometry -> 3-D SIA -> frictional heating ->
    thickness update from the velocities left on the device. Each call is timed on the host
    (each returns after its device work); beside them the oracle's C restatements of the
    non-SSA steps timed on one host thread (the cpu_baseline leg)."""
    import torch
    from ufemism_gb300 import _native as nat
    from ufemism_gb300 import api, workloads
    from ufemism_gb300.meshgen import dome_mesh
    size = args.size
    base = dome_mesh(size)
    mesh = api.build_aaac(base)
    Hi, Hb, SL = workloads.dome_geometry(base)
    ssa, sia = workloads.prepare_inputs(mesh, Hi, Hb, SL)
    nV, nAc = base.nV, mesh.nAc
    Aw, Cw = workloads.areas_and_widths(base)
    A3 = np.full((nV, 15), workloads.A_FLOW, order="F")
    dHb_dt = np.zeros(nV)
    smb = np.full(nV, 0.3)
    bmb = np.zeros(nV)
    torch.cuda.set_device(0)
    api.init(0)
    dm = api.DeviceMesh(mesh)
    dm.geometry_attach(mesh)
    p = api.default_params(precision=nat.UFE_MIXED)
    names = ("geometry+upload", "ssa_solve", "ssa_download", "sia", "sia_3d", "frictional_heating", "thickness")

    def one_step():
        t = {}
        t0 = time.perf_counter()
        dm.ssa_upload_geometry(Hi, Hb, SL, ssa["A_flow_mean"], ssa["A_flow_mean_Ac"], p)
        t["geometry+upload"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        rc, st = dm.ssa_run(p, check=False)
        t["ssa_solve"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        dm.ssa_download()
        t["ssa_download"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        dm.solve_sia_geometry(sia["A_flow_Ac"], p)
        t["sia"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        dm.solve_sia_3d(A3, dHb_dt, p)
        t["sia_3d"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        dm.frictional_heating(ssa["mask_sheet"])
        t["frictional_heating"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        dm.thickness_update(Hi, Aw, Cw, smb, bmb, 10.0)
        t["thickness"] = time.perf_counter() - t0
        return t, st

    for _ in range(args.warmup):
        one_step()
    rows = []
    for _ in range(args.steps):
        t, st = one_step()
        rows.append(t)
    gpu_ms = {k: 1e3 * float(np.median([r[k] for r in rows])) for k in names}
    line = {
        "metric": "velocity time step through the C-ABI (ms)", "value": sum(gpu_ms.values()), "unit": "ms",
        "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "dtype": "f64 (SSA mixed)", "data": "synthetic (seeded dome geometry and mesh)",
        "config": {"workload": "%s-vertex dome, one velocity and thickness step" % size, "nV": int(nV),
                   "nAc": int(nAc), "ssa_sweeps": st["total_sweeps"]},
        "components_ms": gpu_ms,
    }
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc
        om = orc.build_aaac(base)
        cpu = {}
        t0 = time.perf_counter(); g = orc.update_geometry(om, Hi, Hb, SL); cpu["geometry"] = time.perf_counter() - t0
        sia_o = dict(sia)
        t0 = time.perf_counter(); so = orc.solve_sia(om, sia_o, orc.default_params()); cpu["sia"] = time.perf_counter() - t0
        o = dm.ssa_download()
        t0 = time.perf_counter()
        orc.solve_sia_3d(om, g, A3, dHb_dt, o["U_SSA"], o["V_SSA"])
        cpu["sia_3d"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        orc.frictional_heating(ssa["mask_sheet"], o["tau_c_AaAc"][:nV], o["U_SSA"], o["V_SSA"])
        cpu["frictional_heating"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        orc.thickness_change(om, Aw, Cw, so["Up_SIA_Ac"], o["Up_SSA_Ac"], smb, bmb, 10.0, Hi)
        cpu["thickness"] = time.perf_counter() - t0
        cpu_ms = {k: 1e3 * v for k, v in cpu.items()}
        line["cpu_baseline"] = {"components_ms": cpu_ms, "cores": 1, "kind": "port",
                                "sample": "the oracle's C restatements of the non-SSA steps, one call each"}
        gpu_cmp = {"geometry": gpu_ms["geometry+upload"], "sia": gpu_ms["sia"], "sia_3d": gpu_ms["sia_3d"],
                   "frictional_heating": gpu_ms["frictional_heating"], "thickness": gpu_ms["thickness"]}
        line["speedup_vs_cpu"] = {k: cpu_ms[k] / gpu_cmp[k] for k in cpu_ms}
    print(json.dumps(line))
    dm.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile-case", choices=["mixed", "fp64", "exact"], default=None,
                    help="run one capped solve (for profiler captures) instead of the benchmark")
    ap.add_argument("--profile-sweeps", type=int, default=60)
    ap.add_argument("--refold-sweeps", type=int, default=0, help="profile case: mixed refold interval (0: default)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", default="200k")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="leave out the adjoint keys of the default line")
    ap.add_argument("--ref-sample-sweeps", type=int, default=40)
    ap.add_argument("--adj-rn-tol", type=float, default=1e-10, help="adjoint: forward Picard tolerance")
    ap.add_argument("--adj-tol", type=float, default=1e-12, help="adjoint: VJP relative residual tolerance")
    ap.add_argument("--fd-directions", type=int, default=2)
    ap.add_argument("--workload", default="dome", choices=["dome", "ensemble", "marine", "adjoint", "step"],
                    help="dome: the 200k-vertex single solve; ensemble: the batched ensemble")
    ap.add_argument("--members", type=int, default=256)
    ap.add_argument("--autotune", action="store_true", help="ensemble: run the autotuner first")
    ap.add_argument("--rows-per-cta", type=int, default=16384)
    ap.add_argument("--block", type=int, default=1024)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_case:
        return profile_case(args)
    if args.workload == "ensemble":
        return ensemble_bench(args)
    if args.workload == "marine":
        return marine_bench(args)
    if args.workload == "step":
        return step_bench(args)
    if args.workload == "adjoint":
        return adjoint_bench(args)

    rank, world, local = dist_info()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    from ufemism_gb300 import _native as nat
    from ufemism_gb300 import api
    api.init(local)

    base, mesh, ssa, sia = make_workload(args.size)
    dm = api.DeviceMesh(mesh)
    counts = mesh_counts(mesh)
    p64 = api.default_params(precision=nat.UFE_FP64)
    p32 = api.default_params(precision=nat.UFE_MIXED)

    # results of both paths through the C-ABI, checked against the oracle's full solve below
    rc64, o64, s64 = dm.solve_ssa(ssa, p64)
    rc32, o32, s32 = dm.solve_ssa(ssa, p32)
    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))
    FIELDS = ("U_SSA", "V_SSA", "Ux_SSA_Ac", "Uy_SSA_Ac")
    l2 = max(rel(o32[k], o64[k]) for k in FIELDS)

    dm.ssa_upload(ssa, p64)
    stream_ptr = dm.stream
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t64, st64 = timed_runs(dm, p64, args.steps, args.warmup, stream_ptr)
        t32, st32 = timed_runs(dm, p32, args.steps, args.warmup, stream_ptr)
    clocks = clk.summary()
    torch.cuda.synchronize()
    ms32 = float(np.mean(t32))
    ms64 = float(np.mean(t64))
    if world > 1:
        tt = torch.tensor([ms32, ms64], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms32, ms64 = float(tt[0]), float(tt[1])
    value = world * 1000.0 / ms32
    fp64_value = world * 1000.0 / ms64

    # e2e: host buffers through ufe_ssa_solve (H2D inputs, solve, D2H results) each step
    h2d = sum(np.asarray(v).nbytes for k, v in ssa.items()
              if k in ("Hi", "Hb", "SL", "dHs_dx_shelf", "dHs_dy_shelf", "A_flow_mean", "mask_sheet", "Hi_Ac",
                       "Hb_Ac", "SL_Ac", "dHs_dx_shelf_Ac", "dHs_dy_shelf_Ac", "A_flow_mean_Ac"))
    h2d += 8 * (2 * base.nV + 2 * mesh.nAc + mesh.nVAaAc)   # warm start + Picard state
    d2h = 8 * (2 * base.nV + 4 * mesh.nAc + 5 * mesh.nVAaAc)
    # The host arrays are allocated once and reused every step, as a model's state arrays are
    # (fresh arrays each step would time the host's first-touch page faults, not the solve);
    # resetting the warm start to a cold start is inside the timed region.
    bufs = dm.ssa_buffers()
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in api.SSA_INOUT_FIELDS:
            bufs[k].fill(0.0)
        rc, out, st = dm.solve_ssa(ssa, p32, buffers=bufs)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_value = world * 1000.0 / float(np.mean(e2e_ms))

    adjoint = adjoint_summary(dm, mesh, ssa, p32, ms32) if not args.no_adjoint else None

    peak, peak_kind = load_peaks()
    bytes32, sweep32 = algorithmic_bytes(counts, st32, True)
    bytes64, sweep64 = algorithmic_bytes(counts, st64, False)
    ach32 = bytes32 / (ms32 * 1e-3) / 1e9
    ach64 = bytes64 / (ms64 * 1e-3) / 1e9
    # DRAM traffic per launch and L2 throughput of the kernel from an ncu capture of a capped
    # solve of this workload (profiles/), scaled to this launch's sweeps
    traffic = tprof = None
    prof = os.path.join(ROOT, "profiles", "ssa_persistent_traffic.json")
    if os.path.exists(prof):
        try:
            tprof = json.load(open(prof))
            traffic = tprof["dram_bytes_per_sweep"] * st32["total_sweeps"]
        except Exception:
            traffic = tprof = None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 sweeps / f64 defect", "data": "synthetic (seeded dome geometry and mesh)",
        "config": workload_config(args.size, base, mesh.nVAaAc, counts["nnz_all"]),
        "precision": "mixed", "parallelism": "replicas" if world > 1 else "1 GPU",
        "picard_iterations": st32["picard_iterations"], "sor_sweeps": st32["total_sweeps"],
        "working_set": {"mixed_sweep_mb": round(sweep32 / 1e6, 1), "fp64_sweep_mb": round(sweep64 / 1e6, 1),
                        "note": "the mixed sweep's arrays fit the 129 MB L2, the FP64 sweep's do not"},
        "fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": ms64, "sor_sweeps": st64["total_sweeps"],
                 "picard_iterations": st64["picard_iterations"],
                 "vertex_sweeps_per_s": counts["nA"] * st64["total_sweeps"] / (ms64 * 1e-3),
                 "achieved_gbs": ach64, "frac": ach64 / peak},
        "mixed_vs_fp64_speedup": fp64_value and value / fp64_value,
        "rel_l2_mixed_vs_fp64_gpu": l2,
        "vertex_sweeps_per_s": counts["nA"] * st32["total_sweeps"] / (ms32 * 1e-3),
        "roofline": {"bound": "hbm", "achieved": ach32, "peak": peak, "unit": "GB/s", "frac": ach32 / peak,
                     "traffic": traffic, "peak_kind": peak_kind, "kernel": "ssa_persistent<mixed>",
                     "dram_frac": None if traffic is None else traffic / (ms32 * 1e-3) / 1e9 / peak,
                     "l2_throughput_pct_ncu": None if tprof is None else tprof.get("lts_throughput_pct"),
                     "note": "achieved/frac: algorithmic bytes (each array once per sweep) over the launch time; "
                             "dram_frac: measured DRAM bytes over the same time; the mixed sweep's working set "
                             "lives in L2, so it is bound by L2 latency and synchronisation, not by HBM",
                     "algorithmic_bytes_per_launch": bytes32, "bytes_per_sweep": sweep32},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        # k_gather + ssa_persistent + k_scatter per mixed solve in the timed region
        "gpu_launches": 3 * args.steps,
        "clocks": clocks,
    }
    if adjoint:
        line["adjoint"] = adjoint
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb, rc_o, oout, ost = cpu_baseline(args.size)
        line["cpu_baseline"] = cb
        # accuracy against the oracle's FP64 solve of the same workload (the metric's rel-L2)
        line["accuracy_vs_oracle"] = {
            "rel_l2_mixed": max(rel(o32[k], oout[k]) for k in FIELDS),
            "rel_l2_fp64": max(rel(o64[k], oout[k]) for k in FIELDS),
            "fp64_same_sweep_counts": s64["sweeps"] == ost["sweeps"],
            "same_picard_iterations": s64["picard_iterations"] == s32["picard_iterations"] == ost["picard_iterations"],
            "oracle_status": rc_o, "oracle_sweeps": ost["total_sweeps"],
            "fields": "U_SSA, V_SSA, Ux_SSA_Ac, Uy_SSA_Ac (max over the four)"}
    dm.close()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
