#!/usr/bin/env python
"""Benchmark: beam-element assemblies per second on the 60×60×20 lattice frame.

One step is one complete assembly of the Newton system of the static lattice
frame (210,000 EulerBeam3D, 21,600 Hold, 205,200 DofLoad; 453,600 dofs,
17,776,800 nonzeros): every element's residual and exact tangent on the
device, then the deterministic scatter into Lλ and Lλx.nzval.

  value  beams × assemblies / s with the state resident in HBM; each timed
         assembly is preceded by a 512 MB write that flushes the L2
  e2e    the same through the C-ABI call a host caller makes (mgpu_assemble):
         host state in, host Lλ and nzval out, copies inside the timed region
  --impl reference   the CPU arm: the oracle (a C++ dual-number restatement
         of the reference's assembly) of the same lattice on the host cores

Launched as `python bench.py --gpus N ...` or under torch.distributed.run for
N>1; the lattice is a single model, so N>1 runs N independent replicas and the
value sums them (scaling "weak").  Prints one JSON line on rank 0.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "muscade.jl_gb300"))

import numpy as np  # noqa: E402

METRIC = "beam-element assemblies/s"
UNIT = "beam assemblies/s"
WORKLOAD = "lattice frame 60x60x20, SweepX{0} assembly (210000 EulerBeam3D, 21600 Hold, 205200 DofLoad)"
FLOPS_FILE = os.path.join(ROOT, "profiles", "beam_kernel_flops.json")
NCU_FILE = os.path.join(ROOT, "profiles", "beam_kernel_lattice_traffic.json")


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 0, 1, None
    import torch.distributed as dist

    dist.init_process_group("gloo")  # host-side coordination only: barrier and max-time reduction
    return dist.get_rank(), int(os.environ.get("LOCAL_RANK", "0")), ws, dist


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except OSError:
            rows = []
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and "Active" in r[5 + k] and "Not" not in r[5 + k]:
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def fp64_peak_tflops(device):
    """FP64 FMA throughput of this GPU, measured by the library (independent DFMA chains)."""
    import ctypes

    from muscade_gpu import _lib

    v = ctypes.c_double()
    rc = _lib.load().mgpu_measure_fp64_peak(device, ctypes.byref(v))
    return v.value if rc == 0 else None


def state_for(model, seed=2027):
    rng = np.random.Generator(np.random.PCG64(seed))
    return [rng.normal(size=model.ndof["X"]) * 1e-3]


class OracleAssembly:
    """The CPU leg: the oracle's restatement of the reference's assembly of the
    same lattice (prepare with asmmat!, then per step every element's R and K
    by nested duals on all host threads and the serial add_value!/add_∂!
    scatter into Lλ and Lλx.nzval, src/Assemble.jl:470-608).  It is both the
    timed CPU baseline and the checker of the device's pattern and values."""

    def __init__(self, model, dis):
        from oracle import lib as O
        from oracle import reference as REF

        O.build()
        self.REF, self.model = REF, model
        t0 = time.perf_counter()
        self.prep = REF.Prepared(model, dis)
        self.prepare_s = time.perf_counter() - t0

    def assemble(self, X, t):
        """One full assembly; returns (Lλ, nzval, seconds)."""
        REF = self.REF
        t0 = time.perf_counter()
        Ll, nz = REF.assemble(self.prep, tuple(X), (np.zeros(self.model.ndof["U"]),), t, "static",
                              REF.newmark_coefficients(0, 1.0, 0.25, 0.5))
        return Ll, nz, time.perf_counter() - t0

    def parity(self, dm, Ll, nz, X, t):
        """Pattern and asm maps bit-exact, Lλ and nzval relative to their largest entry."""
        prep = self.prep
        colptr, rowval = dm.pattern()
        pat = bool(dm.nnz == prep.nnz and np.array_equal(colptr, prep.colptr) and np.array_equal(rowval, prep.rowval))
        for ig in range(len(self.model.groups)):
            a1, a2 = dm.asm(ig)
            pat &= bool(np.array_equal(a1, prep.asm1[ig]) and np.array_equal(a2, prep.asm2[ig]))
        Lr, nr, dt = self.assemble(X, t)
        eL = float(np.max(np.abs(Ll - Lr)) / np.max(np.abs(Lr)))
        eK = float(np.max(np.abs(nz - nr)) / np.max(np.abs(nr)))
        return {"pattern_and_asm_bit_exact": pat, "Ll_max_rel_err": eL, "nzval_max_rel_err": eK, "tol": 1e-12,
                "pass": bool(pat and eL <= 1e-12 and eK <= 1e-12),
                "checked_against": "oracle assembly of the whole lattice (asmmat! pattern, nested-dual elements)"}, dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--grid", default="60,60,20")
    ap.add_argument("--ref-steps", type=int, default=int(os.environ.get("MGPU_REF_STEPS", "20")),
                    help="reference arm: at most this many timed whole assemblies")
    ap.add_argument("--config", default="lattice",
                    choices=["lattice", "lattice-solve", "risers", "cantilever", "batched", "adjoint"],
                    help="lattice: the headline assembly metric; lattice-solve: the lattice's 5 load steps of "
                         "SweepX{0} with the multifrontal device solver; risers/cantilever: whole SweepX solves; "
                         "batched: independent cantilevers and portal frames solved together; "
                         "adjoint: cost gradient of the stiffness identification beam")
    ap.add_argument("--adj-nel", type=int, default=5000)
    ap.add_argument("--adj-steps", type=int, default=500)
    ap.add_argument("--fd-params", type=int, default=50, help="adjoint: A-dofs checked by central differences")
    ap.add_argument("--fd-steps", type=int, default=50, help="adjoint: horizon of the finite-difference check")
    ap.add_argument("--models", type=int, default=4096, help="batched: number of models")
    ap.add_argument("--individual", type=int, default=16, help="batched: models also solved one by one")
    ap.add_argument("--oracle-models", type=int, default=4, help="batched: sampled models also solved by the oracle")
    ap.add_argument("--no-graph", action="store_true", help="risers: launch kernel by kernel instead of replaying "
                                                              "a captured CUDA graph per step")
    ap.add_argument("--autotune", action="store_true",
                    help="risers/batched: pick element block size and linear solver by timing them first")
    ap.add_argument("--risers", type=int, default=200)
    ap.add_argument("--linsolve", default="auto",
                    choices=["auto", "f32ir", "f64", "block", "torn", "torn32", "sparse", "sparse64"],
                    help="device linear solver of the whole-solve modes")
    args = ap.parse_args()
    rank, local_rank, ws, dist = dist_setup()
    if args.config == "batched":
        return bench_batched(args, rank, local_rank, ws, dist)
    if args.config == "adjoint":
        return bench_adjoint(args, rank, local_rank, ws, dist)
    if args.config == "lattice-solve":
        return bench_lattice_solve(args, rank, local_rank, ws, dist)
    if args.config != "lattice":
        return bench_solve(args, rank, local_rank, ws, dist)
    nx, ny, nz = (int(v) for v in args.grid.split(","))

    from muscade_gpu import workloads

    model, times = workloads.lattice(nx, ny, nz)
    st = model.initialize()
    model.initialize_cached = st.dis
    nbeam = model.groups[0].nele
    t = float(times[0])
    X = state_for(model)
    threads = os.cpu_count() or 1
    config = {"workload": WORKLOAD if (nx, ny, nz) == (60, 60, 20) else f"lattice frame {nx}x{ny}x{nz}",
              "beams": nbeam, "dofs": model.ndof["X"], "l2": "flushed between timed assemblies (512 MB write)"}

    if args.impl == "reference":
        if rank != 0:
            return
        ora = OracleAssembly(model, st.dis)
        per = []
        # each step is one whole assembly (about 2 s on 16 cores); the step count
        # is capped so that the arm ends within a few minutes
        nsteps = min(args.steps, args.ref_steps)
        nwarm = min(args.warmup, 1)
        for i in range(nwarm + nsteps):
            _, _, dt = ora.assemble(X, t)
            if i >= nwarm:
                per.append(dt)
        tstep = sum(per) / len(per)
        value = nbeam / tstep
        sample = (f"the whole lattice per step ({nbeam} beams: element R and K by nested duals on {threads} "
                  f"threads, serial add_value!/add_∂! into Lλ and nzval), {nsteps} steps after {nwarm} warm-up")
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
                "steps": nsteps, "warmup": nwarm, "ms_per_step": tstep * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                                 "prepare_s": ora.prepare_s},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    from muscade_gpu import _lib
    from muscade_gpu.device import DeviceModel

    _lib.build()
    device = local_rank
    fp64_peak = fp64_peak_tflops(device) if rank == 0 else None
    t_create = time.perf_counter()
    dm = DeviceModel(model, st.dis, device=device)
    t_create = time.perf_counter() - t_create
    dm.upload_state(X, t=t)
    # warm-up
    dm.time_assemble(reps=max(args.warmup, 1), t=t, flush_l2=True)
    if dist:
        dist.barrier()
    with Clocks(device) as ck:
        tt, tg, ts = dm.time_assemble(reps=args.steps, t=t, flush_l2=True)
    if dist:
        dist.barrier()
    clocks = ck.summary()
    tmax = reduce_max(dist, tt)
    value = ws * nbeam / (tmax * 1e-3)
    # e2e through the C-ABI with host buffers (the caller's output buffers are
    # page-locked once and reused, as a solver loop would).  Pipelined: every
    # step uploads its state and load values and copies Lλ and nzval back, the
    # copies of step k overlapping the kernels of step k+1
    # (mgpu_assemble_async / mgpu_assemble_wait); the synchronous call
    # (mgpu_assemble) is timed too and reported beside it.
    for _ in range(max(args.warmup, 1)):
        dm.assemble(X, t=t, reuse=True)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        Ll, nzv = dm.assemble(X, t=t, reuse=True)
    e2e_sync = reduce_max(dist, (time.perf_counter() - t0) / args.steps)
    for _ in range(max(args.warmup, 2)):
        dm.assemble_wait(dm.assemble_async(X, t=t)[0])
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    prev = None
    for _ in range(args.steps):
        tk = dm.assemble_async(X, t=t)[0]
        if prev is not None:
            dm.assemble_wait(prev)
        prev = tk
    dm.assemble_wait(prev)
    e2e_dt = (time.perf_counter() - t0) / args.steps
    e2e_dt = reduce_max(dist, e2e_dt)
    h2d = 8 * (model.ndof["X"] + dm.ntval + model.ndof["U"])
    d2h = 8 * (model.ndof["X"] + dm.nnz)
    if rank != 0:
        dm.close()
        return
    ngroup = len(model.groups)
    launches_per_step = ngroup + 2 + 1  # element kernels, two scatters, L2 flush
    # roofline of the beam element kernel (FP64-pipe bound)
    tbeam = float(tg[0])
    flops = None
    try:
        flops = json.load(open(FLOPS_FILE))["fp64_flops_per_beam_static"]
    except (OSError, KeyError, ValueError):
        pass
    traffic = None
    try:
        tr = json.load(open(NCU_FILE))
        traffic = tr["dram_bytes_per_beam"] * nbeam
    except (OSError, KeyError, ValueError):
        pass
    roof = {"bound": "fp64", "unit": "TFLOP/s", "kernel": "beam_kernel<false>", "ms_per_launch": tbeam,
            "peak_source": "measured on this GPU: DFMA throughput of independent FMA chains (mgpu_measure_fp64_peak)", "peak": fp64_peak,
            "traffic": traffic, "traffic_unit": "bytes per launch"}
    if flops:
        ach = flops * nbeam / (tbeam * 1e-3) / 1e12
        roof.update({"achieved": ach, "frac": ach / fp64_peak if fp64_peak else None,
                     "algorithmic_flops_per_beam": flops})
    else:
        roof.update({"achieved": None, "frac": None})
    # scatter kernels against HBM
    hbm_peak = None
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, KeyError, ValueError):
        hbm_peak = 6800.0
    ent = sum(g.nele * (len(g.etype.doflist(g.key)[0]) ** 2) for g in model.groups)
    vent = sum(g.nele * len(g.etype.doflist(g.key)[0]) for g in model.groups)
    sb = ent * (8 + 4) + dm.nnz * (8 + 4) + vent * (8 + 4) + model.ndof["X"] * (8 + 4)
    roof_scatter = {"bound": "hbm", "unit": "GB/s", "achieved": sb / (ts * 1e-3) / 1e9, "peak": hbm_peak,
                    "frac": sb / (ts * 1e-3) / 1e9 / hbm_peak, "bytes_per_launch": sb, "ms": ts}
    # CPU leg: the oracle's assembly of the same lattice, timed, and the parity
    # of this run's device assembly (the e2e call's outputs) against it
    ora = OracleAssembly(model, st.dis)
    parity, cpu_dt = ora.parity(dm, Ll, nzv, X, t)
    cpu_rate = nbeam / cpu_dt
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tmax, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded lattice frame, lognormal sections, Gaussian loads)", "config": config,
        "e2e": {"value": ws * nbeam / e2e_dt, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_dt * 1e3, "api": "mgpu_assemble_async + mgpu_assemble_wait (two in flight)",
                "synchronous": {"value": ws * nbeam / e2e_sync, "ms_per_step": e2e_sync * 1e3, "api": "mgpu_assemble"}},
        "roofline": roof, "roofline_scatter": roof_scatter,
        "kernel_ms": {"beam": tbeam, "other_elements": float(np.sum(tg[1:])), "scatter": ts},
        "cpu_baseline": {"value": cpu_rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"one whole assembly of the lattice ({nbeam} beams; oracle nested-dual R and K "
                                   f"on {threads} threads + serial scatter into Lλ and nzval)"},
        "parity": parity,
        "gpu_launches": args.steps * launches_per_step, "clocks": clocks,
        "create_s": t_create,
    }
    print(json.dumps(line), flush=True)
    dm.close()
    if dist:
        dist.destroy_process_group()


def lattice_solve_cpu_leg(grid=(12, 12, 6)):
    """CPU leg of lattice-solve: the oracle's SweepX{0} (nested-dual assembly,
    SuperLU factorisation) of a reduced lattice, timed per Newton iteration,
    and the device's states on the same lattice against it."""
    from muscade_gpu import workloads
    from muscade_gpu.device import DeviceModel
    from oracle import reference as REF

    m, times = workloads.lattice(*grid)
    st = m.initialize()
    niter = [0]
    assemble = REF.assemble

    def counted(*a, **k):
        niter[0] += 1
        return assemble(*a, **k)

    REF.assemble = counted
    try:
        t0 = time.perf_counter()
        ref = REF.sweepx(m, st.dis, st, times, OX=0, maxdx=1e-8, maxLl=1e-3)
        dt = time.perf_counter() - t0
    finally:
        REF.assemble = assemble
    dm = DeviceModel(m, st.dis)
    rc, states, _ = dm.sweepx(0, times, st.time, list(st.X), maxdx=1e-8, maxLl=1e-3)
    dm.close()
    lam = np.array([str(f).startswith("λ") for f in st.dis.fieldX])
    errs = {}
    if rc == 0:
        for name, sel in (("dofs", ~lam), ("multipliers", lam)):
            dev = max(np.max(np.abs(states[k, 0][sel] - Xr[0][sel])) for k, (_, Xr) in enumerate(ref))
            errs[name] = float(dev / max(np.max(np.abs(Xr[0][sel])) for _, Xr in ref))
    return {"ms_per_newton_iteration": dt / niter[0] * 1e3, "newton_iterations": niter[0], "seconds": dt,
            "dofs": m.ndof["X"], "parity": {"grid": list(grid), "rc": int(rc), "max_rel_state_err": errs,
                                            "tol": 1e-9, "pass": bool(rc == 0 and all(e <= 1e-9 for e in errs.values())),
                                            "checked_against": "oracle SweepX{0} (SuperLU) of the same lattice"}}


def bench_lattice_solve(args, rank, local_rank, ws, dist):
    """The lattice's Newton solve on the device: 5 load steps of SweepX{0} on
    the 60×60×20 frame (453,600 dofs), each Newton iteration an assembly, a
    multifrontal factorisation (FP32 factors in FP64 refinement) and a
    decrement.  One bench step is the whole 5-load-step solve.  Replicas only:
    one model per GPU."""
    from muscade_gpu import _lib, workloads
    from muscade_gpu.device import DeviceModel

    _lib.build()
    nx, ny, nz = (int(v) for v in args.grid.split(","))
    model, times = workloads.lattice(nx, ny, nz)
    st = model.initialize()
    # |Δx| includes the Hold reactions (about 1e4 N at this size); 1e-6 is well
    # above their rounding floor
    kw = dict(maxdx=1e-6, maxLl=1e-3)
    t0 = time.perf_counter()
    dm = DeviceModel(model, st.dis, device=local_rank, linsolve=args.linsolve)
    sp0 = dm.sparse_info()  # analysis (first use)
    t_create = time.perf_counter() - t0
    X0 = list(st.X)
    for _ in range(max(args.warmup, 1)):
        rc, _, _ = dm.sweepx(0, times[:1], st.time, X0, **kw)
        if rc != 0:
            raise SystemExit(dm.lib.mgpu_last_error(dm.ctx).decode())
    if dist:
        dist.barrier()
    nrep = max(1, min(args.steps, 3))
    nl0 = dm.launch_count()
    with Clocks(local_rank) as ck:
        t0 = time.perf_counter()
        for _ in range(nrep):
            rc, states, stats = dm.sweepx(0, times, st.time, X0, **kw)
            if rc != 0:
                raise SystemExit(dm.lib.mgpu_last_error(dm.ctx).decode())
        dt = (time.perf_counter() - t0) / nrep
    launches = (dm.launch_count() - nl0) // nrep
    clocks = ck.summary()
    dt = reduce_max(dist, dt)
    sp = dm.sparse_info()
    info = dm.linear_solver_info()
    dm.close()
    if rank != 0:
        return
    iters = stats.niter_total
    ms_iter = dt / iters * 1e3
    fl = sp["flops"]
    cpu = lattice_solve_cpu_leg()
    line = {"metric": "ms per Newton iteration (lattice 60x60x20, SweepX{0}, multifrontal device solve)",
            "value": ms_iter, "unit": "ms", "higher_is_better": False, "n_gpus": ws, "steps": nrep,
            "warmup": max(args.warmup, 1), "ms_per_step": dt * 1e3, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 (FP32 factors in FP64 refinement)" if not sp["fp64"] else "f64",
            "data": "synthetic (seeded lattice frame, lognormal sections, Gaussian loads)",
            "config": {"workload": f"lattice frame {nx}x{ny}x{nz}, SweepX{{0}}, {len(times)} load steps",
                       "dofs": model.ndof["X"], "newton_iterations": iters, "load_steps": stats.nstep_done,
                       "ms_per_load_step": dt / stats.nstep_done * 1e3, "linear_solver": info,
                       "multifrontal": sp0 | {k: sp[k] for k in ("fp64", "last_fallback", "last_sweeps",
                                                                  "last_perturbed", "last_factor_ms",
                                                                  "last_refine_ms")},
                       "l2": "inputs larger than L2 (the factors alone are tens of GB)"},
            "factorisation": {"ms": sp["last_factor_ms"], "flops": fl,
                              "achieved_tflops": fl / (sp["last_factor_ms"] * 1e-3) / 1e12
                              if sp["last_factor_ms"] > 0 else None,
                              "precision": "FP64" if sp["fp64"] else "FP32"},
            "e2e": {"value": ms_iter, "unit": "ms", "h2d_bytes_per_step": 8 * (model.ndof["X"] + len(times) * (dm.ntval + 1)),
                    "d2h_bytes_per_step": 8 * model.ndof["X"] * len(times),
                    "note": "the whole mgpu_sweepx call with host initial state, load values and states"},
            "cpu_baseline": {"value": cpu["ms_per_newton_iteration"], "unit": "ms per Newton iteration", "kind": "port",
                             "cores": os.cpu_count(),
                             "sample": f"oracle SweepX{{0}} of the 12x12x6 lattice ({cpu['dofs']} dofs, "
                                       f"{cpu['newton_iterations']} iterations, nested-dual assembly + SuperLU); "
                                       "the full lattice is out of the CPU's reach"},
            "parity": cpu["parity"], "create_s": t_create, "clocks": clocks,
            "gpu_launches": launches}
    print(json.dumps(line), flush=True)


def bench_solve(args, rank, local_rank, ws, dist):
    """Whole device SweepX runs: Newmark risers (3 Newton iterations per step) or the static cantilever."""
    from muscade_gpu import _lib, workloads
    from muscade_gpu.device import DeviceModel
    from oracle import reference as REF

    _lib.build()
    if args.config == "risers":
        # one fixed set of risers × ranks, split by muscade_gpu.shard: each rank
        # solves its own share (no collective on the data path)
        from muscade_gpu.shard import shard_bounds

        lo, hi = shard_bounds(np.ones(args.risers * ws), ws)[rank]
        model, times = workloads.risers(nriser=args.risers * ws, subset=(lo, hi))
        st = model.initialize(time=0.0)
        OX, kw = 2, dict(fixed_iter=3, graph=not args.no_graph)
        nstep_w, nstep = args.warmup, args.steps
        nbeam = model.groups[0].nele
    else:
        model, times = workloads.cantilever()
        st = model.initialize()
        OX, kw = 0, dict(maxdx=1e-9, maxLl=1e-5)
        nstep_w, nstep = 0, len(times)
        nbeam = model.groups[0].nele
    dm = DeviceModel(model, st.dis, device=local_rank, linsolve=args.linsolve)
    X0 = list(st.X)[: OX + 1]
    tune = None
    if args.autotune:
        nX = model.ndof["X"]
        dm.upload_state([st.X[0]] + [np.zeros(nX)] * OX, t=float(times[0]))
        nm = None
        if OX == 2:
            a1, b1 = 0.5 / (0.25 * 0.05), 1 / (0.25 * 0.05**2)
            nm = dict(a1=a1, a2=2.0, a3=0.0, b1=b1, b2=1 / (0.25 * 0.05), b3=2.0)
        tune = dm.autotune(2 if OX == 2 else 0, nm)
    T = np.asarray(times[: nstep_w + nstep], dtype=np.float64)
    if args.config == "risers" and nstep_w:
        dm.sweepx(OX, T[:nstep_w], st.time, X0, **kw)
    if dist:
        dist.barrier()
    nl0 = dm.launch_count()
    with Clocks(local_rank) as ck:
        t0 = time.perf_counter()
        rc, states, stats = dm.sweepx(OX, T if args.config == "cantilever" else T[:nstep], st.time, X0, **kw)
        dt = time.perf_counter() - t0
    clocks = ck.summary()
    # a replayed step graph is captured (and counted) once: its kernels run every step
    launches = dm.launch_count() - nl0
    if kw.get("graph") and kw.get("fixed_iter"):
        launches *= max(stats.nstep_done, 1)
    if rc != 0:
        raise SystemExit(dm.lib.mgpu_last_error(dm.ctx).decode())
    dt = reduce_max(dist, dt)
    host_loop_ms = None
    if args.config == "cantilever":
        # the same solve with the load steps and Newton iterations looped on the
        # device (one graph launch); it replaces the host loop when it is faster
        dm.sweepx(OX, T, st.time, X0, device_loop=True, **kw)
        t0 = time.perf_counter()
        rc_d, states_d, stats_d = dm.sweepx(OX, T, st.time, X0, device_loop=True, **kw)
        dt_d = reduce_max(dist, time.perf_counter() - t0)
        if rc_d == 0 and np.array_equal(states_d, states) and dt_d < dt:
            host_loop_ms = dt / max(stats.nstep_done, 1) * 1e3
            dt = dt_d
    if rank != 0:
        return
    steps_run = stats.nstep_done
    ms_step = dt / steps_run * 1e3
    iters = stats.niter_total
    value = ws * nbeam * iters / dt
    # CPU arm on a bounded sample: the oracle's SweepX on a reduced model of the same kind
    if args.config == "risers":
        sm, stimes = workloads.risers(nriser=2)
        sst = sm.initialize(time=0.0)
        c0 = time.perf_counter()
        try:
            REF.sweepx(sm, sst.dis, sst, stimes[:3], OX=2, maxiter=60, maxdx=1e-5)
        except Exception:
            pass
        cdt = time.perf_counter() - c0
        cpu_rate = sm.groups[0].nele * 3 * 3 / cdt
        sample = "2 risers x 3 Newmark steps (oracle assembly + SuperLU)"
    else:
        c0 = time.perf_counter()
        ref = REF.sweepx(model, st.dis, st, times, OX=0, maxdx=1e-9, maxLl=1e-5)
        cdt = time.perf_counter() - c0
        cpu_rate = None
        sample = f"whole cantilever solve: {cdt * 1e3:.1f} ms"
    line = {"metric": "ms per " + ("Newmark step (3 Newton iterations)" if args.config == "risers" else "load step"),
            "value": ms_step, "unit": "ms", "higher_is_better": False, "n_gpus": ws, "steps": steps_run,
            "warmup": nstep_w, "ms_per_step": ms_step, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.config, "beams": nbeam, "dofs": model.ndof["X"], "newton_iterations": iters,
                       "cuda_graph": bool(kw.get("graph", False)), "autotune": tune,
                       "device_loop": host_loop_ms is not None, "host_loop_ms_per_step": host_loop_ms,
                       "linear_solver": dm.linear_solver_info()},
            "beam_assemblies_per_s": value, "e2e": {"value": ms_step, "unit": "ms", "note": "whole solve incl. copies"},
            "cpu_baseline": {"value": cpu_rate, "unit": "beam assemblies/s", "kind": "port", "sample": sample,
                             "cores": os.cpu_count()},
            "gpu_launches": launches, "clocks": clocks}
    print(json.dumps(line), flush=True)
    dm.close()



def bench_batched(args, rank, local_rank, ws, dist):
    """Independent models (half cantilevers, half portal frames, 10-400 beams,
    8 load steps of SweepX{0}) solved together with per-model convergence.
    One bench step is one whole batched solve.  N ranks split one seeded set of
    N × --models models by cost, with no collective: weak scaling by models."""
    from muscade_gpu import _lib, workloads
    from muscade_gpu.device import DeviceModel

    _lib.build()
    # one fixed seeded set of models × ranks, split by cost (element counts)
    # with muscade_gpu.shard: each rank solves its share, no collective
    from muscade_gpu.shard import my_share

    allp = workloads.batched_params(args.models * ws, seed=2030)
    params, _ = my_share(allp, [p["nel"] for p in allp], rank, ws)
    model, offs, times = workloads.build_batched(params)
    st = model.initialize()
    nbeam = model.groups[0].nele
    # maxLλ = ∞ (the reference's default): with the finer meshes the residual
    # levels off near 1e-4 N from rounding, while Δx still reaches 1e-9
    kw = dict(maxdx=1e-9, maxLl=math.inf, per_component=True)
    t_create = time.perf_counter()
    dm = DeviceModel(model, st.dis, device=local_rank, linsolve=args.linsolve)
    t_create = time.perf_counter() - t_create
    X0 = list(st.X)
    tune = None
    if args.autotune:
        dm.upload_state([st.X[0]], t=float(times[0]))
        tune = dm.autotune(0)
    for _ in range(args.warmup):
        dm.sweepx(0, times, st.time, X0, **kw)
    if dist:
        dist.barrier()
    with Clocks(local_rank) as ck:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            rc, xb, stats = dm.sweepx(0, times, st.time, X0, **kw)
            if rc != 0:
                raise SystemExit(dm.lib.mgpu_last_error(dm.ctx).decode())
        dt = (time.perf_counter() - t0) / args.steps
    clocks = ck.summary()
    dt = reduce_max(dist, dt)
    iters = stats.niter_total
    info64 = dm.linear_solver_info()
    # the same sweep as one graph launch with the load steps and Newton
    # iterations looped on the device (no per-iteration host read-back)
    dm.sweepx(0, times, st.time, X0, device_loop=True, **kw)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rc_dl, x_dl, stats_dl = dm.sweepx(0, times, st.time, X0, device_loop=True, **kw)
    dt_dl = reduce_max(dist, (time.perf_counter() - t0) / args.steps)
    same_dl = rc_dl == 0 and bool(np.array_equal(x_dl, xb)) and stats_dl.niter_total == iters
    # the same batch with FP32 factors and FP64 refinement
    dm.set_linear_solver("f32ir")
    dm.sweepx(0, times, st.time, X0, **kw)
    t0 = time.perf_counter()
    rc32, x32, stats32 = dm.sweepx(0, times, st.time, X0, **kw)
    dt32 = time.perf_counter() - t0
    info32 = dm.linear_solver_info()
    dm.close()
    if rank != 0:
        return
    # per-model deviation of the FP32-refined states from the FP64 ones
    bounds = list(offs) + [model.nnod]
    worst = 0.0
    if rc32 == 0:
        for i in range(len(params)):
            d = workloads.node_dofs(model, np.arange(bounds[i] + 1, bounds[i + 1] + 1))
            d = d[d >= 0]
            ref = xb[:, 0, d]
            worst = max(worst, float(np.max(np.abs(x32[:, 0, d] - ref)) / max(np.max(np.abs(ref)), 1e-300)))
    # the plain per-model path: models solved one by one (FP64), same seeded sample
    pick = np.random.Generator(np.random.PCG64(7)).permutation(len(params))[: args.individual]
    tind, same = [], True
    for i in pick:
        mi, _, _ = workloads.build_batched([params[i]])
        si = mi.initialize()
        # the batch's linear solver (one model alone would be partitioned, another pivoting order)
        di = DeviceModel(mi, si.dis, device=local_rank, linsolve=info64["kind"])
        di.sweepx(0, times, si.time, list(si.X), maxdx=1e-9, maxLl=math.inf)  # warm
        t0 = time.perf_counter()
        rci, xi, _ = di.sweepx(0, times, si.time, list(si.X), maxdx=1e-9, maxLl=math.inf)
        tind.append(time.perf_counter() - t0)
        di.close()
        nodes = np.arange(1, mi.nnod + 1)
        a, b = workloads.node_dofs(mi, nodes), workloads.node_dofs(model, nodes + offs[i])
        sel = a >= 0
        same &= rci == 0 and bool(np.array_equal(xi[:, 0, a[sel]], xb[:, 0, b[sel]]))
    per_model = 1.0 / float(np.mean(tind))
    cpu = batched_cpu_leg(params, pick[: args.oracle_models], times, model, offs, xb, x32 if rc32 == 0 else None)
    value = len(allp) / dt  # all ranks' models over the slowest rank's time
    h2d = 8 * (model.ndof["X"] + len(times) * dm.ntval + len(times))
    d2h = 8 * model.ndof["X"] * len(times)
    launches_per_iter = len(model.groups) + 2 + 9  # element kernels, scatters, solver, decrement, convergence
    line = {"metric": "models/s (SweepX{0}, 8 load steps per model, per-model convergence)", "value": value,
            "unit": "models/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded cantilevers and portal frames, lognormal sections, Gumbel loads)",
            "config": {"workload": f"batched uneven models: {len(params)} models, {nbeam} beams, "
                                   f"{model.ndof['X']} dofs", "models": len(params), "beams": nbeam,
                       "dofs": model.ndof["X"], "newton_iterations": iters, "linear_solver": info64, "autotune": tune,
                       "l2": "inputs larger than L2 (nzval alone is several hundred MB)"},
            "beam_assemblies_per_s": ws * nbeam * iters / dt,
            "e2e": {"value": value, "unit": "models/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "note": "the whole mgpu_sweepx call with host initial state, load values and states"},
            "per_model_path": {"models_per_s": per_model, "sample": int(len(pick)), "speedup_of_batch": value / per_model,
                               "states_bitwise_equal_to_batch": same},
            "device_loop": {"models_per_s": len(allp) / dt_dl if rc_dl == 0 else None, "rc": rc_dl,
                            "states_bitwise_equal_to_host_loop": same_dl, "graph_launches_per_sweep": 1,
                            "note": "load steps and Newton iterations looped on the device by conditional graph nodes"},
            "fp32_refined": {"models_per_s": len(params) / dt32 if rc32 == 0 else None, "rc": rc32,
                             "max_rel_state_dev_vs_fp64": worst, "linear_solver": info32,
                             "newton_iterations": stats32.niter_total,
                             "max_rel_state_dev_vs_oracle": cpu["dev_fp32"]},
            "fp64_max_rel_state_dev_vs_oracle": cpu["dev_fp64"],
            "cpu_baseline": cpu["baseline"],
            "gpu_launches": args.steps * iters * launches_per_iter, "clocks": clocks, "create_s": t_create}
    print(json.dumps(line), flush=True)


def batched_cpu_leg(params, pick, times, model, offs, xb, x32):
    """CPU leg of the batched mode: the oracle's SweepX{0} (nested-dual
    assembly, SuperLU) of a few sampled models, timed, and the deviation of
    the device's FP64 and FP32-refined states from it, per dof class relative
    to that class's largest value over the trajectory."""
    from muscade_gpu import workloads
    from oracle import reference as REF

    dev64 = dev32 = 0.0
    tcpu = 0.0
    for i in pick:
        mi, _, _ = workloads.build_batched([params[i]])
        si = mi.initialize()
        t0 = time.perf_counter()
        ref = REF.sweepx(mi, si.dis, si, times, OX=0, maxdx=1e-9, maxLl=math.inf)
        tcpu += time.perf_counter() - t0
        nodes = np.arange(1, mi.nnod + 1)
        a, b = workloads.node_dofs(mi, nodes), workloads.node_dofs(model, nodes + offs[i])
        sel = a >= 0
        R = np.stack([Xr[0] for _, Xr in ref])[:, a[sel]]
        scale = max(float(np.max(np.abs(R))), 1e-300)
        dev64 = max(dev64, float(np.max(np.abs(xb[:, 0, b[sel]] - R))) / scale)
        if x32 is not None:
            dev32 = max(dev32, float(np.max(np.abs(x32[:, 0, b[sel]] - R))) / scale)
    return {"dev_fp64": dev64, "dev_fp32": dev32 if x32 is not None else None,
            "baseline": {"value": len(pick) / tcpu if tcpu > 0 else None, "unit": "models/s", "kind": "port",
                         "cores": 1, "sample": f"{len(pick)} sampled models solved one by one by the oracle "
                                               "(nested-dual assembly, SuperLU)"}}


def bench_adjoint(args, rank, local_rank, ws, dist):
    """Stiffness identification: the gradient of the identification cost with
    respect to one EI scale per beam by the discrete Newmark adjoint (one
    forward sweep, √N checkpoints, a reverse sweep of transposed solves).  The
    cost is built from elements, as a Muscade model states it: a
    SingleDofCost per sensor (quadratic misfit to its record) and a
    SingleAcost per A-dof (prior towards the nominal EI).  One bench step is
    one gradient.  Replicas only: one beam per GPU."""
    from muscade_gpu import _lib, workloads
    from muscade_gpu.device import DeviceModel

    _lib.build()
    d = workloads.adjoint_beam(nel=args.adj_nel, nstep=args.adj_steps)
    m = d["model"]
    st = m.initialize(time=0.0)
    dm = DeviceModel(m, st.dis, device=local_rank, linsolve=args.linsolve)
    X0 = list(st.X)
    tol = 1e-7
    dm.set_A(d["A_true"])
    rc, truth, _ = dm.sweepx(2, d["times"], st.time, X0, maxdx=tol)
    if rc != 0:
        raise SystemExit(dm.lib.mgpu_last_error(dm.ctx).decode())
    dm.close()
    y, sd = workloads.synthetic_measurements(truth, d["sensors"])
    w = 1.0 / sd**2
    a_weight = 1.0
    # the same beam with the identification cost as elements
    d = workloads.adjoint_beam(nel=args.adj_nel, nstep=args.adj_steps, measurements=(y, sd), a_weight=a_weight)
    m = d["model"]
    st = m.initialize(time=0.0)
    dm = DeviceModel(m, st.dis, device=local_rank, linsolve=args.linsolve)
    ncost = sum(g.nele for g in m.groups if g.key[0] in ("SingleDofCost", "SingleAcost"))
    tv = dm.time_values(d["times"])  # load values and sensor records, tabulated once
    A0 = np.ones(dm.nA)
    dm.set_A(A0)
    # one forward sweep alone (the unit of a finite-difference gradient)
    t0 = time.perf_counter()
    dm.sweepx(2, d["times"], st.time, X0, maxdx=tol)
    t_fwd = time.perf_counter() - t0
    for _ in range(args.warmup):
        dm.adjoint(2, d["times"], st.time, X0, maxdx=tol, tvals=tv)
    if dist:
        dist.barrier()
    with Clocks(local_rank) as ck:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            C, gA, _, stats = dm.adjoint(2, d["times"], st.time, X0, maxdx=tol, tvals=tv)
        dt = (time.perf_counter() - t0) / args.steps
    clocks = ck.summary()
    dt = reduce_max(dist, dt)
    if rank != 0:
        dm.close()
        return
    # central differences on the first fd_steps steps at fd_params random A-dofs
    nfd = min(args.fd_steps, len(d["times"]))
    tf, yf = d["times"][:nfd], y[:nfd]
    Cf, gf, _, _ = dm.adjoint(2, tf, st.time, X0, maxdx=tol, tvals=tv[:nfd])

    def cost(A):
        dm.set_A(A)
        rc, s, _ = dm.sweepx(2, tf, st.time, X0, maxdx=tol)
        r = s[:, 0, d["sensors"] - 1] - yf
        misfit = float(np.sum(np.diff(np.concatenate([[st.time], tf])) * np.sum(w * r * r, axis=1)))
        return misfit + a_weight * float(np.sum((A - 1.0) ** 2))

    idx = np.random.Generator(np.random.PCG64(2032)).choice(dm.nA, min(args.fd_params, dm.nA), replace=False)
    h = 1e-4
    fd = np.array([(cost(A0 + h * np.eye(1, dm.nA, i)[0]) - cost(A0 - h * np.eye(1, dm.nA, i)[0])) / (2 * h)
                   for i in idx])
    fd_err = float(np.max(np.abs(gf[idx] - fd)) / np.max(np.abs(fd)))
    dm.set_A(A0)
    info = dm.linear_solver_info()
    dm.close()
    nst = len(d["times"])
    line = {"metric": "adjoint gradients/s (dC/dA, stiffness identification)", "value": ws / dt,
            "unit": "gradients/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded GP loads, lognormal true EI scales, 1 % sensor noise)",
            "config": {"workload": f"simply supported beam, {args.adj_nel} EulerBeam3D with EI-scale A-dofs, "
                                   f"{nst} Newmark steps of 0.01 s", "beams": args.adj_nel, "dofs": m.ndof["X"],
                       "A_dofs": dm.nA, "sensors": int(len(d["sensors"])), "cost_elements": ncost,
                       "cost": "SingleDofCost per sensor (1/sd^2 (x - y(t))^2), SingleAcost per A-dof ((a - 1)^2)",
                       "checkpoints": "sqrt(N)", "newton_iterations_forward": stats.niter_total,
                       "linear_solver": info},
            "cost": C, "grad_norm": float(np.linalg.norm(gA)),
            "fd_check": {"params": int(len(idx)), "steps": int(nfd), "h": h, "max_rel_err": fd_err},
            "forward_sweep_s": t_fwd,
            "speedup_vs_finite_differences": 2 * dm.nA * t_fwd / dt,
            "e2e": {"value": ws / dt, "unit": "gradients/s", "h2d_bytes_per_step": 8 * (nst * (dm.ntval + 1) + dm.nA),
                    "d2h_bytes_per_step": 8 * (dm.nA + nst),
                    "note": "the whole mgpu_adjoint_sweepx call with the host table of load values and sensor "
                            "records (tabulated once before the timed region) and the gradient back"},
            # per Newton iteration ~20 launches (element kernels, scatters, partitioned solve,
            # decrement, norms), forward and recomputation; per reverse step ~31
            "gpu_launches": args.steps * (2 * stats.niter_total * 20 + nst * 31), "clocks": clocks}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
