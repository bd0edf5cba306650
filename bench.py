#!/usr/bin/env python
"""Benchmark: zone-updates/s of the Guacho timestep on GB300.

Workload (N=1): decaying MHD turbulence on a 256^3 periodic box (seeded
random-phase solenoidal velocity, E(k) ~ k^-2 on 2<=|k|<=8, RMS Mach 1;
B = (0.1,0,0) + solenoidal perturbation of RMS 0.05), HLLD, van Leer,
flux-CD, gamma = 5/3.  A step = get_timestep + tstep over the whole box.

  value  : FP32 + Kahan-pair zone-updates/s, state resident in HBM,
           CUDA-graph device loop, timed with CUDA events (max over ranks)
  e2e    : the same through the C ABI with the state in page-locked HOST
           memory (gch_step_host: u read over the host link, get_timestep,
           tstep, u written back over the link, every step)
  e2e_main_loop : the reference's main loop through the C ABI: upload once,
           per step gch_get_timestep (dt read back) + gch_tstep, download
           at the end, all timed
  extra  : FP32 with FP64 u and the plain FP64 path on the same box, their
           L1 distances, the batched boxes, the live roofline of the
           dominant kernel, the CPU oracle on a bounded sample, SM clocks
           sampled during the run.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
  python bench.py --configs      # the other configurations, one line each

Under torchrun every rank advances its own replica box on its own GPU
(the path does not shard: replicas only), timings are max-reduced.
"""
from __future__ import annotations

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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "zone-updates/s on 1 GB300: FP64 plain vs FP32-mixed vs batched, at stated L1 err"
UNIT = "zone-updates/s"
WORKLOAD = ("decaying MHD turbulence 256^3, periodic, HLLD + van Leer + flux-CD, "
            "seeded random-phase solenoidal velocity (E(k)~k^-2, 2<=|k|<=8, Mach 1)")


def bench_config(n: int, ws: int) -> dict:
    """The workload description both arms print (the same box and problem)."""
    return {"workload": WORKLOAD, "n": n,
            "precision": "fp32 + Kahan-compensated pair accumulation (GCH_FP32_KAHAN)",
            "parallelism": f"replicas x{ws}",
            "l2": "state 1.1 GB FP64 u + 0.56 GB FP32 up >> 129 MB L2 (no flush)"}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max-reduce across ranks (no-op at N=1)."""

    def __init__(self):
        self.ws, self.rank, self.local = _dist()
        self.pg = None
        if self.ws > 1:
            import torch
            import torch.distributed as td
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(0)  # one visible GPU per rank
            td.init_process_group(backend=backend)
            self.td, self.torch, self.backend = td, torch, backend

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.ws == 1:
            return x
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = self.torch.tensor([x], dtype=self.torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi samples during the timed region (SM clock, reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.out.flush()
        rows = [r.split(",") for r in Path(self.out.name).read_text().splitlines() if r.strip()]
        os.unlink(self.out.name)
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        rows = [r for r in rows if r[0].strip() == vis] or rows
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].strip().lower() == "active"})
        load = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(load) if load else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def peaks() -> dict:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


# ---------------------------------------------------------------------------
# algorithmic bytes per cell of the dominant kernel (stage-2 k_flux) and per
# zone-update of the whole step (two-sweep minimum 3 u + 2 up passes)
# ncu, 256^3 turbulence, one k_flux<PolKahan,4,8,2,0,2> launch:
# dram__bytes_read.sum 1277941760 + dram__bytes_write.sum 838390528
STAGE2_KAHAN_TRAFFIC_PER_CELL = (1277941760 + 838390528) / 256 ** 3


# The plain FP64 path is bound by the FP64 pipe, not by HBM.  ncu on the
# 64^3 turbulence box (smsp/sm__inst_executed_pipe_fp64.sum per launch over
# the 262,144 cells; sm__inst_executed_pipe_fp64.avg.pct_of_peak_sustained_active
# with sm__cycles_elapsed.avg gives the pipe's peak issue rate):
#   FP64-pipe warp instructions per zone-update of a whole step
#   k_flux stage 1 44.83 + stage 2 78.04 + k_cfl 1.62 (its square roots and
#   quotients on the integer pipes) + k_ct 0.91 + 0.90
FP64_PIPE_WARP_INST_PER_ZONE = 44.83 + 78.04 + 1.62 + 0.91 + 0.90
#   peak: 0.0530 FP64-pipe warp instructions per SM cycle (stage 2: 20,456,302
#   instructions over 152 SMs x 4,283,477 cycles at 59.27% of peak)
FP64_PIPE_PEAK_PER_SM_CYCLE = 20456302 / (152 * 4283477.11) / 0.5927
N_SM = 152


def fp64_pipe_record(zone_updates_per_s: float, sm_mhz) -> dict:
    """FP64-pipe utilisation of the plain FP64 step: the ncu instruction
    count per zone-update times the live zone-update rate, over the pipe's
    peak issue rate at the SM clock sampled during the run."""
    mhz = sm_mhz or 2070.0
    achieved = FP64_PIPE_WARP_INST_PER_ZONE * zone_updates_per_s / (N_SM * mhz * 1e6)
    return {"bound": "fp64 pipe", "warp_inst_per_zone_update": FP64_PIPE_WARP_INST_PER_ZONE,
            "achieved_per_sm_cycle": achieved, "peak_per_sm_cycle": FP64_PIPE_PEAK_PER_SM_CYCLE,
            "frac": achieved / FP64_PIPE_PEAK_PER_SM_CYCLE, "sm_mhz": mhz,
            "source": "FP64-pipe instruction counts per zone-update and the pipe's peak "
                      "issue rate from ncu on the 64^3 turbulence box; zone-update rate and "
                      "SM clock from this run"}


def kernel_bytes_per_cell(prec: int, neq: int = 8) -> int:
    tu = 8  # FP64 u, or a (hi, lo) FP32 pair
    ts = 8 if prec == 0 else 4
    # read up (neq), read u(1:5), write u(1:5), write E (3)
    return neq * ts + 5 * tu + 5 * tu + 3 * ts


def step_bytes_per_zone(prec: int, neq: int = 8) -> int:
    tu = 8
    ts = 8 if prec == 0 else 4
    return neq * (3 * tu + 2 * ts)


def prim_fields(p, u):
    """Interior primitives of a host-layout u (FP64), the reference's u2prim
    without floors: rho, p, v and (MHD) B."""
    import numpy as np
    ui = u[2:-2, 2:-2, 2:-2]
    rho = ui[..., 0]
    v = ui[..., 1:4] / rho[..., None]
    e = ui[..., 4] - 0.5 * rho * (v ** 2).sum(-1)
    out = {"rho": rho, "vx": v[..., 0], "vy": v[..., 1], "vz": v[..., 2]}
    if p.neq >= 8:
        if p.mhd:
            e = e - 0.5 * (ui[..., 5:8] ** 2).sum(-1)
        out.update(Bx=ui[..., 5], By=ui[..., 6], Bz=ui[..., 7])
    out["p"] = e / p.cv
    return out


def field_errors(p, u, uref) -> dict:
    """Per-field errors of u against uref over the interior: relative L1
    mean|x - x_ref| / mean|x_ref|, absolute Linf max|x - x_ref| and Linf
    relative to the field's scale max|x_ref|."""
    import numpy as np
    a, r = prim_fields(p, u), prim_fields(p, uref)
    out = {}
    for k in ("rho", "p", "vx", "vy", "vz", "Bx", "By", "Bz"):
        if k not in r:
            continue
        d = np.abs(a[k] - r[k])
        ref = np.abs(r[k])
        out[k] = {"l1": float(d.mean() / max(ref.mean(), 1e-300)),
                  "linf": float(d.max()), "linf_rel": float(d.max() / max(ref.max(), 1e-300))}
    return out


def max_divb(p, u) -> dict:
    """max |div B| over the interior with the centred formula of the
    reference's div B dump (src/Out_BIN_Module.f90:214-222), absolute and
    relative to max|B|/dx."""
    import numpy as np
    from guacho_gb300 import binio
    d = float(np.abs(binio.divb(u, p)).max())
    ui = u[2:-2, 2:-2, 2:-2]
    bmax = float(np.sqrt((ui[..., 5:8] ** 2).sum(-1)).max())
    return {"abs": d, "rel": d * min(p.dx, p.dy, p.dz) / max(bmax, 1e-300)}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


# ---------------------------------------------------------------------------
def _tuning_record(t: dict) -> dict:
    """The autotuner's choice and search for the JSON line: the stage
    kernels' z-march depth and launch form (blocks_per_sm: resident blocks
    per SM of the persistent work-queue grid, 0 = one block per work item),
    and the stage-1 time of every pair tried."""
    return {"grouped": t["grouped"], "kz": t["kz"], "blocks_per_sm": t["blocks_per_sm"],
            "tile": "32x8 cells", "stage1_ms": [
                {"kz": k, "blocks_per_sm": b, "ms": round(ms, 4)}
                for (k, b), ms in sorted(t["grid"].items())]}


def batched_run(args, precision: int) -> dict:
    """The batched configuration: nbox boxes of sizes drawn from
    {32,48,64,96}^3, each an Orszag-Tang box (B0 x U[0.5,2]) or a blast
    (pressure ratio log-uniform in [10,1000]), each with its own CFL dt,
    `batch_steps` steps; aggregate zone-updates/s (host wall clock around one
    gch_batch_advance of most of the steps, which runs them back to back on
    the device), p50/p99 of the batch step time (one synchronous
    gch_batch_advance per step), and the per-box L1 error against a per-box
    FP64 run."""
    import numpy as np

    from guacho_gb300 import params as P
    from guacho_gb300 import problems
    from guacho_gb300.domain import Batch
    boxes = problems.batch_boxes(nbox=args.batch_boxes, precision=precision)
    zones = sum(p.nx * p.ny * p.nz for p, _ in boxes)
    b = Batch([p for p, _ in boxes])
    for i, (_, u) in enumerate(boxes):
        b.upload(i, u)
    warm = 3
    n_single = max(1, (args.batch_steps - warm) * 3 // 10)
    n_run = args.batch_steps - warm - n_single
    if n_run < 1:
        raise SystemExit("--batch-steps must be at least 5")
    b.advance(warm)  # warm-up (kz tuning, graph capture)
    t0 = time.perf_counter()
    b.advance(n_run)
    total = time.perf_counter() - t0
    times = []
    for _ in range(n_single):
        t0 = time.perf_counter()
        b.advance(1)
        times.append(time.perf_counter() - t0)
    res = {"value": zones * n_run / total, "unit": UNIT, "boxes": len(boxes),
           "zones": zones, "steps": args.batch_steps, "timed_steps": n_run,
           "step_ms_p50": 1e3 * float(np.percentile(times, 50)),
           "step_ms_p99": 1e3 * float(np.percentile(times, 99)),
           "timing": (f"host wall clock around one advance of {n_run} steps; p50/p99 over "
                      f"{n_single} synchronous single-step advances"),
           "tuning": _tuning_record(b.tuning())}
    # per-box error against FP64 boxes advanced the same number of steps
    b64 = Batch([p.replace(precision=P.FP64) for p, _ in boxes])
    for i, (_, u) in enumerate(boxes):
        b64.upload(i, u)
    b64.advance(args.batch_steps)
    errs = []
    for i, (p, _) in enumerate(boxes):
        a = prim_fields(p, b.download(i))
        r = prim_fields(p, b64.download(i))
        bmag = np.sqrt(r["Bx"] ** 2 + r["By"] ** 2 + r["Bz"] ** 2).mean()
        errs.append(max(float(np.abs(a["rho"] - r["rho"]).mean() / np.abs(r["rho"]).mean()),
                        float(np.abs(a["p"] - r["p"]).mean() / np.abs(r["p"]).mean()),
                        float(np.abs(a["Bx"] - r["Bx"]).mean() / bmag)))
    res["l1_err_max_over_boxes"] = max(errs)
    res["l1_err_median_over_boxes"] = float(np.median(errs))
    b.close()
    b64.close()
    return res


def c2_errors(n: int, steps: int, warm: int = 3) -> tuple:
    """Decaying turbulence n^3 (HLLD, van Leer, flux-CD): `steps` steps from
    the initial state on the plain FP64 path and on both FP32 paths, each
    with its own dt; per-field L1/Linf of the FP32 states against the FP64
    state at equal step count, and max |div B| of all three.  The FP64 run
    is timed (CUDA events, device loop) over its last steps - warm steps;
    returns (errors, FP64 ms over those steps, their count)."""
    from guacho_gb300 import params as P
    from guacho_gb300 import problems
    from guacho_gb300.domain import Domain
    p, u0 = problems.turbulence(n)
    with Domain(p.replace(precision=P.FP64)) as d:
        d.init(u0)
        d.advance_timed(warm)
        ms64 = d.advance_timed(steps - warm)
        u64 = d.download()
    res = {"workload": f"decaying MHD turbulence {n}^3 (HLLD, van Leer, flux-CD)",
           "steps": steps, "compare": "equal step count, each precision with its own dt",
           "fp64": {"max_divb": max_divb(p, u64)}}
    for name, prec in (("fp32_kahan", P.FP32_KAHAN), ("fp32_mixed_fp64u", P.FP32_MIXED)):
        with Domain(p.replace(precision=prec)) as d:
            d.init(u0)
            d.advance_timed(steps)
            u = d.download()
        res[name] = {"errors": field_errors(p, u, u64), "max_divb": max_divb(p, u)}
        del u
    return res, ms64, steps - warm


def c3_errors(n: int, tmax: float) -> dict:
    """Low-beta blast n^3 (outflow, HLLD, minmod, flux-CD) run to t = tmax in
    FP64, FP32 with FP64 u and FP32 with Kahan pairs, host-driven steps
    (get_timestep + tstep, the last dt clipped to land on tmax as the
    reference clips to its output time): the pressure-floor hits of every
    step (cells whose recovered pressure fell below the 1e-16 floor of
    src/hydro_core.f90:78 when get_timestep formed the primitives of u),
    per-field L1/Linf of the FP32 states against FP64 at t = tmax, and
    max |div B|."""
    from guacho_gb300 import params as P
    from guacho_gb300 import problems
    from guacho_gb300.domain import Domain
    p, u0 = problems.blast(n)
    res = {"workload": f"low-beta MHD blast {n}^3 (outflow, HLLD, minmod, flux-CD), "
                       f"beta ~ 0.025 outside the sphere", "tmax": tmax,
           "floor_count": "cells of u below the pressure floor at each step's get_timestep"}
    ref = None
    for name, prec in (("fp64", P.FP64), ("fp32_mixed_fp64u", P.FP32_MIXED),
                       ("fp32_kahan", P.FP32_KAHAN)):
        with Domain(p.replace(precision=prec)) as d:
            d.init(u0)
            t, it, floors, bits = 0.0, 1, [], 0
            while it <= 100000:
                dt, dump = d.get_timestep(it, 10, t, tmax)
                d.tstep(dt)
                t += dt
                it += 1
                pf, err = d.step_info()
                floors.append(int(pf))
                bits |= err
                if dump or t >= tmax:
                    break
            u = d.download()
        e = {"steps": it - 1, "time": t, "floor_hits_total": sum(floors),
             "steps_with_floor_hits": sum(1 for x in floors if x),
             "floor_hits_max_step": max(floors) if floors else 0,
             "floor_hits_per_step": floors, "err_bits": bits, "max_divb": max_divb(p, u)}
        if ref is None:
            ref = u
        else:
            e["errors"] = field_errors(p, u, ref)
        res[name] = e
    return res


def c5_errors(n: int, steps: int) -> dict:
    """Hydro wind interaction with tabulated cooling n^3 (HLLC, outflow, two
    spheres re-imposed at every boundary call): `steps` steps from the
    initial state in FP64 and on both FP32 paths; per-field L1/Linf of the
    FP32 states against FP64 at equal step count, and the FP64 step time."""
    from guacho_gb300 import params as P
    from guacho_gb300 import problems
    from guacho_gb300.domain import Domain
    p, u0 = problems.wind_cooling(n)
    with Domain(p.replace(precision=P.FP64)) as d:
        d.init(u0)
        ms64 = d.advance_timed(steps)
        u64 = d.download()
    res = {"workload": f"hydro wind + table cooling {n}^3 (HLLC, outflow, 2 spheres)",
           "steps": steps, "compare": "equal step count, each precision with its own dt",
           "fp64_ms_per_step": ms64 / steps}
    for name, prec in (("fp32_kahan", P.FP32_KAHAN), ("fp32_mixed_fp64u", P.FP32_MIXED)):
        with Domain(p.replace(precision=prec)) as d:
            d.init(u0)
            ms = d.advance_timed(steps)
            u = d.download()
        res[name] = {"errors": field_errors(p, u, u64), "ms_per_step": ms / steps}
        del u
    return res


def cpu_oracle_rate(n: int, steps: int, threads: int) -> dict:
    """The oracle (the C restatement of the reference's CPU algorithm) on an
    n^3 sample of the same turbulence problem, FP64, all threads."""
    from guacho_gb300 import problems
    from oracle.oracle import Oracle
    p, u0 = problems.turbulence(n)
    o = Oracle(p, threads=threads)
    o.init(u0)
    t, it = 0.0, 1
    dt, _ = o.get_timestep(it, 10, t, 1e30)  # warm-up step
    o.tstep(dt)
    t += dt
    it += 1
    t0 = time.perf_counter()
    for _ in range(steps):
        dt, _ = o.get_timestep(it, 10, t, 1e30)
        o.tstep(dt)
        t += dt
        it += 1
    el = time.perf_counter() - t0
    return {"value": n ** 3 * steps / el, "seconds": el, "n": n, "steps": steps}


def run_reference(args, dist: Dist) -> None:
    if dist.rank != 0:
        dist.close()
        return
    threads = os.cpu_count() or 1
    from oracle.oracle import Oracle, build
    from guacho_gb300 import problems
    build()
    n = args.ref_size
    p, u0 = problems.turbulence(n)
    o = Oracle(p, threads=threads)
    o.init(u0)
    t, it = 0.0, 1
    for _ in range(args.warmup):
        dt, _ = o.get_timestep(it, 10, t, 1e30)
        o.tstep(dt)
        t += dt
        it += 1
    t0 = time.perf_counter()
    for _ in range(args.steps):
        dt, _ = o.get_timestep(it, 10, t, 1e30)
        o.tstep(dt)
        t += dt
        it += 1
    el = time.perf_counter() - t0
    rate = n ** 3 * args.steps / el
    sample = (f"the same {n}^3 turbulence box (same seed and spectrum), FP64, {args.steps} "
              f"steps after {args.warmup} warm-up, OpenMP over {threads} threads; the "
              f"reference Fortran+MPI build cannot be compiled here (no Fortran compiler), so "
              f"the C restatement of its algorithm (oracle/) runs instead")
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(n, dist.ws),
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                             "cpu": cpu_model(), "sample": sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    dist.close()


# ---------------------------------------------------------------------------
def run_ours(args, dist: Dist) -> None:
    import numpy as np

    from guacho_gb300 import build as gbuild
    if dist.rank == 0 or dist.ws == 1:
        gbuild.build(verbose=False)
    dist.barrier()
    from guacho_gb300 import params as P
    from guacho_gb300 import problems
    from guacho_gb300.domain import Domain

    n = args.size
    K, W = args.steps, args.warmup
    p, u0 = problems.turbulence(n)
    pk = peaks()
    out = {}

    # ---- FP32 paths, device resident ---------------------------------------
    # headline: FP32 state/fluxes with Kahan-compensated FP32-pair u;
    # also the variant with u in FP64 (FP64 accumulation and recovery)
    variants = {}
    headline = P.FP32_KAHAN
    for prec in (P.FP32_KAHAN, P.FP32_MIXED):
        d = Domain(p.replace(precision=prec))
        d.init(u0)
        # the z-march depth by the library's autotuner (stage-1 probes on
        # this state; results are the same for every depth)
        tuned = d.autotune()
        d.advance_timed(W)
        clocks = Clocks()
        dist.barrier()
        clocks.start()
        ms_v = d.advance_timed(K)
        clk_v = clocks.stop()
        ms_v = dist.max(ms_v)
        prof_v = {}
        if prec == headline:
            for _ in range(3):
                for name, t in d.profile_step():
                    prof_v.setdefault(name, []).append(t)
        variants[prec] = dict(ms=ms_v, clk=clk_v, prof=prof_v,
                              launches=d.launches_per_step(), kz=d.kz,
                              kz_probe_ms={k: round(v, 4) for k, v in tuned.items()})
        d.close()
    ms = variants[headline]["ms"]
    clk = variants[headline]["clk"]
    prof = variants[headline]["prof"]
    launches = variants[headline]["launches"]
    value = dist.ws * n ** 3 * K / (ms * 1e-3)

    # ---- plain FP64 on the same box, and the FP32 paths' errors against it ---
    # (C2: every precision advanced the same number of steps from the initial
    # state; the FP64 run's last steps are its timing)
    c2, ms64, k64 = c2_errors(n, args.err_steps)
    configs_err = {"C2": c2}
    if not args.no_config_errors and dist.rank == 0:
        configs_err["C3"] = c3_errors(args.blast_size, args.blast_tmax)
        configs_err["C5"] = c5_errors(args.wind_size, args.wind_steps)
    pm = p.replace(precision=headline)

    # ---- e2e through the C ABI with host buffers ----------------------------
    import torch
    host = torch.empty(p.shape, dtype=torch.float64, pin_memory=True).numpy()
    host[...] = u0
    de = Domain(pm)
    de.init(u0)
    t, it = 0.0, 1
    for _ in range(2):
        dt, _ = de.step_host(host, it, 10, t, 1e300)
        t += dt
        it += 1
    ke = max(2, args.e2e_steps)  # each step moves 2 x 1.12 GB over the host link
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        dt, _ = de.step_host(host, it, 10, t, 1e300)
        t += dt
        it += 1
    e2e_s = dist.max(time.perf_counter() - t0)
    de.close()
    e2e = {"value": dist.ws * n ** 3 * ke / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(host.nbytes), "d2h_bytes_per_step": int(host.nbytes),
           "steps": ke, "path": "gch_step_host: page-locked host u (reference layout, FP64) "
                                "read by the layout kernel over the host link -> "
                                "get_timestep + tstep -> written back over the link"}

    # ---- the reference's main loop through the C ABI (extra) -----------------
    # src/main.f90:73-125 with the drop-in, all timed: u uploaded from the
    # page-locked host array, boundaryI and calcprim, then every step
    # get_timestep (dt read back to the host) and tstep, and u downloaded into
    # the host array at the end (the output of the run).
    km = max(2, args.loop_steps)
    dm = Domain(pm)
    dm.init(u0)  # first-touch costs of the domain, outside the timed run
    dist.barrier()
    t0 = time.perf_counter()
    dm.upload(host)
    dm.boundaryI()
    dm.calcprim()
    t, it = 0.0, 1
    for _ in range(km):
        dt, _ = dm.get_timestep(it, 10, t, 1e300)
        dm.tstep(dt)
        t += dt
        it += 1
    dm.download(out=host)
    ml_s = dist.max(time.perf_counter() - t0)
    dm.close()
    e2e_loop = {"value": dist.ws * n ** 3 * km / ml_s, "unit": UNIT, "steps": km,
                "h2d_bytes": int(host.nbytes), "d2h_bytes": int(host.nbytes),
                "d2h_bytes_per_step": 12,
                "path": "gch_upload + gch_boundaryI + gch_calcprim, then per step "
                        "gch_get_timestep (dt and the dump flag read back) + gch_tstep, "
                        "then gch_download; host u page-locked, reference layout, FP64"}

    # ---- roofline of the dominant kernel -----------------------------------
    means = {k: sum(v) / len(v) for k, v in prof.items()}
    total = sum(sum(v) for v in prof.values())
    dom = max(means, key=lambda k: sum(prof[k]))
    cells = n ** 3
    bpc = kernel_bytes_per_cell(headline) if dom == "k_flux_stage2" else None
    roof = None
    if bpc:
        ach = bpc * cells / (means[dom] * 1e-3) / 1e9
        traffic = args.traffic
        if traffic is None and headline == P.FP32_KAHAN:
            # dram__bytes_read.sum + dram__bytes_write.sum of one stage-2
            # k_flux launch (FP32 + Kahan, HLLD, van Leer) measured by ncu on
            # the 256^3 box: 126.1 bytes per cell, scaled by the cell count
            traffic = STAGE2_KAHAN_TRAFFIC_PER_CELL * cells
        roof = {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"],
                "unit": "GB/s", "frac": ach / pk["hbm_gbs"], "traffic": traffic,
                "bytes_per_cell": bpc, "launch_ms": means[dom],
                "share_of_step": sum(prof[dom]) / total, "peak_source": pk["source"]}
    mixed_value = dist.ws * n ** 3 * K / (variants[P.FP32_MIXED]["ms"] * 1e-3)
    sbz = step_bytes_per_zone(headline)
    step_gbs = value / dist.ws * sbz / 1e9
    step_roof = {"bytes_per_zone_update": sbz, "achieved": step_gbs, "peak": pk["hbm_gbs"],
                 "unit": "GB/s", "frac": step_gbs / pk["hbm_gbs"],
                 # the compulsory bytes 2 neq w_u (u read once, written once),
                 # the bound of a temporally fused single-sweep step
                 "compulsory_bytes_per_zone_update": 2 * 8 * 8,
                 "compulsory_frac": value / dist.ws * 128 / 1e9 / pk["hbm_gbs"]}

    # ---- batched uneven boxes ----------------------------------------------
    batched = batched_run(args, headline) if args.batch_boxes > 0 else None
    if batched:
        batched["vs_single_box"] = batched["value"] / (value / dist.ws)
        # the same boxes with FP64 u (FP32 arithmetic, FP64 pressure recovery)
        bm = batched_run(args, P.FP32_MIXED)
        batched["fp32_mixed_fp64u"] = {
            k: bm[k] for k in ("value", "step_ms_p50", "step_ms_p99", "l1_err_max_over_boxes",
                               "l1_err_median_over_boxes")}
        batched["fp32_mixed_fp64u"]["vs_single_box"] = bm["value"] / (mixed_value / dist.ws)

    # ---- CPU baseline (rank 0, N=1 only) ------------------------------------
    cpu = None
    if dist.rank == 0 and dist.ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        r = cpu_oracle_rate(args.cpu_size, args.cpu_steps, threads)
        cpu = {"value": r["value"], "unit": UNIT, "cores": threads, "kind": "port",
               "cpu": cpu_model(),
               "sample": f"oracle (C restatement of the reference CPU algorithm, OpenMP over "
                         f"{threads} threads), {r['n']}^3 box of the same problem, "
                         f"{r['steps']} steps after 1 warm-up, FP64, {r['seconds']:.1f} s"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.ws, "steps": K,
        "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (u as Kahan-compensated f32 pairs; double-float pressure recovery; f64 dt)",
        "data": "synthetic (seeded turbulence initial state, no dataset)",
        "config": bench_config(n, dist.ws),
        # the z-march depth each timed FP32 box ran with, chosen by
        # gch_autotune from these stage-1 probe times (ms per launch)
        "z_march": {"fp32_kahan": {"kz": variants[P.FP32_KAHAN]["kz"],
                                   "stage1_probe_ms": variants[P.FP32_KAHAN]["kz_probe_ms"]},
                    "fp32_mixed_fp64u": {"kz": variants[P.FP32_MIXED]["kz"],
                                         "stage1_probe_ms":
                                             variants[P.FP32_MIXED]["kz_probe_ms"]}},
        "fp64_plain": {"value": dist.ws * n ** 3 * k64 / (ms64 * 1e-3),
                       "ms_per_step": ms64 / k64, "steps": k64,
                       "roofline": fp64_pipe_record(n ** 3 * k64 / (ms64 * 1e-3),
                                                    clk.get("sm_mhz"))},
        "fp32_mixed_fp64u": {"value": mixed_value, "ms_per_step": variants[P.FP32_MIXED]["ms"] / K,
                             "step_roofline": {
                                 "bytes_per_zone_update": step_bytes_per_zone(P.FP32_MIXED),
                                 "achieved": mixed_value / dist.ws
                                             * step_bytes_per_zone(P.FP32_MIXED) / 1e9,
                                 "peak": pk["hbm_gbs"], "unit": "GB/s",
                                 "frac": mixed_value / dist.ws * step_bytes_per_zone(P.FP32_MIXED)
                                         / 1e9 / pk["hbm_gbs"]}},
        "config_errors": configs_err,
        "batched": batched,
        "kernel_ms": {k: round(v, 4) for k, v in means.items()},
        "roofline": roof, "step_roofline": step_roof,
        "cpu_baseline": cpu, "e2e": e2e, "e2e_main_loop": e2e_loop, "clocks": clk,
        # get_timestep + tstep, and the loop-tail kernel of the device loop
        "gpu_launches": (launches + 1) * K,
    }
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


def run_ncu_case(args) -> None:
    """A short host-driven step sequence (no CUDA graphs) of the benchmark
    problem for profiler captures: --size, --precision, --steps; with
    --ncu-batch the batched set of boxes instead (grouped steps)."""
    from guacho_gb300 import build as gbuild
    gbuild.build(verbose=False)
    from guacho_gb300 import params as P
    from guacho_gb300 import problems
    from guacho_gb300.domain import Domain
    prec = {"kahan": P.FP32_KAHAN, "mixed": P.FP32_MIXED, "fp64": P.FP64}[args.precision]
    if args.ncu_batch:  # the batched set: 3 grouped warm-up steps (tuning), then --steps
        from guacho_gb300.domain import Batch
        boxes = problems.batch_boxes(nbox=args.batch_boxes, precision=prec)
        b = Batch([q for q, _ in boxes])
        for i, (_, u) in enumerate(boxes):
            b.upload(i, u)
        b.advance(3)
        b.advance(args.steps)
        print(json.dumps({"ncu_case": args.precision, "boxes": len(boxes), "steps": args.steps,
                          "zones": sum(q.nx * q.ny * q.nz for q, _ in boxes)}))
        b.close()
        return
    p, u0 = problems.turbulence(args.size)
    with Domain(p.replace(precision=prec)) as d:
        d.init(u0)
        t = 0.0
        for it in range(1, args.steps + 1):
            dt, _ = d.get_timestep(it, 10, t, 1e30)
            d.tstep(dt)
            t += dt
        print(json.dumps({"ncu_case": args.precision, "size": args.size, "steps": args.steps,
                          "time": t, "info": d.step_info()}))


def run_configs(args) -> None:
    """The benchmark's other configurations, one JSON line per configuration
    and precision (not the headline line): Orszag-Tang 128x128x4 (HLLD,
    minmod, flux-CD, periodic), the low-beta blast 192^3 (outflow; pressure
    floor hits reported) and the hydro wind + table cooling box 256^3 (HLLC,
    user spheres re-imposed at every boundary call).  Device loop, CUDA
    events, after `warmup` steps.  Then one line per configuration with the
    CPU oracle (all host threads) on the same box, a bounded number of steps
    after one warm-up step."""
    from guacho_gb300 import build as gbuild
    gbuild.build(verbose=False)
    from guacho_gb300 import params as P
    from guacho_gb300 import problems
    from guacho_gb300.domain import Domain
    from oracle.oracle import Oracle, build as obuild
    precs = {"fp64": P.FP64, "fp32_mixed_fp64u": P.FP32_MIXED, "fp32_kahan": P.FP32_KAHAN}
    # every precision runs the same steps, so the floor counts compare;
    # (name, problem, GPU steps, CPU oracle steps)
    cases = [
        ("orszag_tang 128x128x4", lambda: problems.orszag_tang(128, 128, 4), 200, 40),
        ("low-beta blast 192^3", lambda: problems.blast(192), 50, 5),
        ("wind + table cooling 256^3 (hydro)", lambda: problems.wind_cooling(256), 50, 4),
    ]
    for name, make, steps, _ in cases:
        p0, u0 = make()
        for pname, prec in precs.items():
            with Domain(p0.replace(precision=prec)) as d:
                d.init(u0)
                d.advance_timed(args.warmup)
                ms = d.advance_timed(steps)
                pfloor, err = d.step_info()
            cells = p0.nx * p0.ny * p0.nz
            print(json.dumps({"config": name, "precision": pname,
                              "value": cells * steps / (ms * 1e-3), "unit": UNIT,
                              "ms_per_step": ms / steps, "steps": steps,
                              "warmup": args.warmup, "pfloor_hits_last_step": pfloor,
                              "err_bits": err}), flush=True)
    obuild()
    threads = os.cpu_count() or 1
    for name, make, _, csteps in cases:
        p0, u0 = make()
        o = Oracle(p0, threads=threads)
        o.init(u0)
        t, it = 0.0, 1
        dt, _ = o.get_timestep(it, 10, t, 1e30)  # warm-up step
        o.tstep(dt)
        t += dt
        it += 1
        t0 = time.perf_counter()
        for _ in range(csteps):
            dt, _ = o.get_timestep(it, 10, t, 1e30)
            o.tstep(dt)
            t += dt
            it += 1
        el = time.perf_counter() - t0
        cells = p0.nx * p0.ny * p0.nz
        print(json.dumps({"config": name, "impl": "cpu oracle (FP64 C restatement)",
                          "value": cells * csteps / el, "unit": UNIT,
                          "ms_per_step": 1e3 * el / csteps, "steps": csteps,
                          "cores": threads, "cpu": cpu_model()}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--err-steps", type=int, default=200,
                    help="steps of the turbulence error comparison (the FP64 timing too)")
    ap.add_argument("--blast-size", type=int, default=192)
    ap.add_argument("--blast-tmax", type=float, default=0.02)
    ap.add_argument("--wind-size", type=int, default=256)
    ap.add_argument("--wind-steps", type=int, default=500)
    ap.add_argument("--no-config-errors", action="store_true",
                    help="skip the blast and wind error runs")
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--loop-steps", type=int, default=50)
    ap.add_argument("--cpu-size", type=int, default=256)
    ap.add_argument("--cpu-steps", type=int, default=8)
    ap.add_argument("--ref-size", type=int, default=256)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch-boxes", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=100)
    ap.add_argument("--traffic", type=float, default=None,
                    help="ncu dram bytes per launch of the dominant kernel, if known")
    ap.add_argument("--ncu-case", action="store_true",
                    help="run a short host-driven step sequence for profiler captures")
    ap.add_argument("--ncu-batch", action="store_true",
                    help="with --ncu-case: the batched set (--batch-boxes) instead of one box")
    ap.add_argument("--precision", default="kahan", choices=["kahan", "mixed", "fp64"])
    ap.add_argument("--configs", action="store_true",
                    help="time the other benchmark configurations (one line each)")
    args = ap.parse_args()
    if args.ncu_case:
        run_ncu_case(args)
        return
    if args.configs:
        run_configs(args)
        return
    ws, rank, local = _dist()
    if ws > 1 and args.impl == "ours":
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
    else:
        run_ours(args, dist)


if __name__ == "__main__":
    main()
