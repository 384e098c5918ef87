"""Benchmark: RK-stage DOF updates/s of the DGSEM Euler residual + SSP-RK3.

Workload (one "step" = one SSP-RK3 step = dt reduction + 3 stages):
  isentropic vortex on the periodic box [0,10]^3 meshed with 64^3 uniform
  Hex8 cells, DGSEM p = 3 (64 GLL nodes/cell), Rusanov flux, SSP-RK3,
  CFL 0.1, FP64 (plain form).  L = 83,886,080 DOFs; a step updates 3 L.

Arms
  default          the GPU library (libmcfd.so) through its C ABI.
                   value: device-resident stepping (mcfd_advance, dt on the
                   device, CUDA-graph replay), CUDA events on the handle stream.
                   e2e: per step the column in from pinned host memory, one
                   step, the column back to pinned host memory, streamed
                   (mcfd_stream_step: neighbouring steps' copies overlap the
                   compute); the sequential set/advance/get figure beside it.
  --impl reference the reference algorithm restated on the CPU (the oracle,
                   OpenMP over all host cores) on a bounded sample of the same
                   workload (the 16^3 mesh of the same case).

N > 1 GPUs run independent replicas (the path is single-GPU by design):
value = sum over ranks / max time over ranks ("scaling": "weak").
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
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "RK-stage DOF updates/s on 1 GB300: plain FP64 vs mixed, at stated L2 error"
UNIT = "DOF-updates/s"
N_CELLS_1D = 64
DEGREE = 3
CFL = 0.1
SAMPLE_1D = 16
VORTEX_ACCURACY_STEPS = 100  # SSP-RK3 steps of the convergence and accuracy runs
K = 5


def workload(n1d=N_CELLS_1D):
    return {
        "workload": f"isentropic vortex, periodic [0,10]^3, {n1d}^3 Hex8, DGSEM p={DEGREE}, Rusanov, SSP-RK3, CFL {CFL}",
        "cells": n1d ** 3,
        "dofs": n1d ** 3 * (DEGREE + 1) ** 3 * K,
        "form": "plain FP64",
        "step": "dt reduction + 3 RK stages",
        "l2_flush": "inputs larger than L2 (solution column 671 MB, geometry 1.3 GB)",
    }


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().splitlines() if r.strip()]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [c.strip() for c in r]
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak_tflops(torch, device) -> float:
    """cuBLAS DGEMM throughput (best of 3), the FP64 denominator."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=device)
    b = torch.randn(n, n, dtype=torch.float64, device=device)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def cpu_sample(steps_min=1, seconds=12.0, max_steps=200, threads=None, fixed_steps=None, n1d=SAMPLE_1D):
    """The oracle on n1d^3 cells of the workload (the 16^3 sample by
    default), all host cores."""
    import oracle.orc as orc
    from pvcriemannsolvers_gb300 import cases, mesh as meshlib
    orc.build()
    threads = threads or os.cpu_count() or 1
    orc.set_threads(threads)
    m = meshlib.box((n1d,) * 3, lengths=(10.0,) * 3, periodic=(True,) * 3)
    om = orc.Mesh(m, DEGREE)
    x = meshlib.node_coordinates(m, DEGREE).reshape(-1, 3)
    u = cases.vortex_ic(x).ravel()
    L = u.size
    t, n, t0 = 0.0, 0, time.perf_counter()
    while True:
        dt = om.time_step(u, 1e9, 3, CFL)
        u = om.rk_update(orc.RUSANOV, 3, t, dt, u)
        t += dt
        n += 1
        el = time.perf_counter() - t0
        if fixed_steps is not None:
            if n >= fixed_steps:
                break
        elif (n >= steps_min and el >= seconds) or n >= max_steps:
            break
    el = time.perf_counter() - t0
    return {"value": 3 * L * n / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n1d}^3 cells of the same case (L = {L} DOFs), {n} SSP-RK3 steps, "
                      f"{el:.1f} s, oracle (plain C restatement, OpenMP)", "seconds": el, "steps": n}


def density_l2_vs_exact(sol, mesh, t):
    """Relative L2 of density against the advected vortex, GLL-weighted."""
    from pvcriemannsolvers_gb300 import cases, mesh as meshlib
    q = DEGREE + 1
    x = meshlib.node_coordinates(mesh, DEGREE).reshape(-1, 3)
    rho_exact = cases.vortex_prim(x, t)[0]
    rho = sol.reshape(-1, K)[:, 0]
    w1 = {4: np.array([1 / 6, 5 / 6, 5 / 6, 1 / 6])}[q]
    w = np.einsum("i,j,k->ijk", w1, w1, w1).ravel()
    w = np.tile(w, mesh.n_cells)
    return float(math.sqrt(np.sum(w * (rho - rho_exact) ** 2) / np.sum(w * rho_exact ** 2)))


def convergence(forms, device, dt_cfl, n_steps, finest):
    """Density L2 against the exact vortex on 16^3, 32^3 and the timed mesh
    after the same number of steps of one fixed dt (half the finest mesh's
    CFL step, so every mesh runs the same times): the observed order of
    both forms."""
    from pvcriemannsolvers_gb300 import Lobatto, cases, mesh as meshlib
    dt = 0.5 * dt_cfl
    out = {"dt": dt, "steps": n_steps, "t_end": dt * n_steps}
    sizes = [n for n in (16, 32) if n < finest] + [finest]
    finest_rho = {}
    for form in forms:
        errs = []
        for n1d in sizes:
            m = meshlib.box((n1d,) * 3, lengths=(10.0,) * 3, periodic=(True,) * 3)
            s = Lobatto(m, DEGREE, "rusanov", cfl=CFL, device=device, precision=form)
            s.SetSolutionColumn(cases.vortex_ic(meshlib.node_coordinates(m, DEGREE).reshape(-1, 3)).ravel())
            t = s.advance(n_steps, dt, 3, 0.0)
            sol = s.GetSolutionColumn()
            errs.append(density_l2_vs_exact(sol, m, t))
            if n1d == finest:
                finest_rho[form] = sol.reshape(-1, K)[:, 0].copy()
            s.close()
        orders = [math.log2(errs[i] / errs[i + 1]) * math.log(2) / math.log(sizes[i + 1] / sizes[i])
                  for i in range(len(errs) - 1)]
        out[form] = {"cells_1d": sizes, "density_rel_l2_vs_exact": errs, "observed_order": orders}
    if "fp64" in finest_rho and "mixed" in finest_rho:
        a, b = finest_rho["mixed"], finest_rho["fp64"]
        out["mixed_vs_fp64_density_rel_l2_finest"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    return out


def run_reference(args, rank, world):
    """The reference algorithm (the oracle, all host cores) on the GPU arm's
    own configuration: the 64^3 mesh, every one of the W + K steps timed."""
    if rank != 0:
        return
    res = cpu_sample(threads=os.cpu_count(), fixed_steps=args.warmup + args.steps, n1d=args.cells)
    line = {
        "impl": "reference", "metric": METRIC, "value": res["value"], "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": res["seconds"] / res["steps"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload(args.cells),
        "cpu_baseline": {k: res[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def max_over_ranks(torch, dist, dev, x: float) -> float:
    """The maximum of a per-rank time over all ranks (the job's time)."""
    tt = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def whole_job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """value = the units all ranks processed / the max-over-ranks time."""
    return units_per_rank * world / seconds


def e2e_runs(torch, dev, sysm, sol, t, steps, dt_guess, dist=None):
    """End-to-end stepping through the C ABI from / to pinned host memory.

    streamed:   mcfd_stream_step per step (the upload of step k+1 and the
                download of step k-1 overlap step k's compute), closed by
                mcfd_stream_end, which waits for the last download.
    sequential: mcfd_set_solution + mcfd_advance(1) + mcfd_get_solution.
    Every step copies the whole column in from and back to pinned host
    memory in both.  Returns (streamed seconds, sequential seconds)."""
    L = sol.size
    host_in = torch.empty(L, dtype=torch.float64, pin_memory=True).numpy()
    host_out = torch.empty(L, dtype=torch.float64, pin_memory=True).numpy()
    host_in[:] = sol
    # set-up, untimed: the device staging and the two job graphs
    sysm.stream_begin()
    sysm.stream_step(host_in, host_out, t, 1, dt_guess, 3)
    sysm.stream_step(host_in, host_out, t, 1, dt_guess, 3)
    sysm.stream_end()
    out = []
    for mode in ("streamed", "sequential"):
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        if mode == "streamed":
            sysm.stream_begin()
            for _ in range(steps):
                sysm.stream_step(host_in, host_out, t, 1, dt_guess, 3)
            sysm.stream_end()
        else:
            te = t
            for _ in range(steps):
                sysm.SetSolutionColumn(host_in)
                te = sysm.advance(1, dt_guess, 3, te)
                sysm.get_solution_into(host_out)
        torch.cuda.synchronize(dev)
        el = time.perf_counter() - t0
        if dist:
            el = max_over_ranks(torch, dist, dev, el)
        out.append(el)
    return out[0], out[1]


E2E_PATH = ("mcfd_stream_step per step (pinned host column in, one SSP-RK3 step, pinned host column out; "
            "the copies of neighbouring steps overlap the compute), mcfd_stream_end")
E2E_SEQ_PATH = "mcfd_set_solution (pinned host) + mcfd_advance(1) + mcfd_get_solution (pinned host)"


def measure_form(args, torch, dist, dev, local_rank, m, u0, precision, contraction="simt", e2e=True):
    """Time one precision form: device-resident stepping, kernel times, e2e."""
    from pvcriemannsolvers_gb300 import Lobatto
    world = dist.get_world_size() if dist else 1
    sysm = Lobatto(m, DEGREE, "rusanov", cfl=CFL, device=local_rank, precision=precision,
                   contraction=contraction)
    stream = torch.cuda.Stream(device=dev)
    sysm.set_stream(stream.cuda_stream)
    L = u0.size
    sysm.SetSolutionColumn(u0)
    tune = sysm.autotune()
    t = sysm.advance(args.warmup, 1e9, 3, 0.0)
    sysm.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    launches0 = sysm.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        with torch.cuda.stream(stream):
            e0.record(stream)
            t = sysm.advance(args.steps, 1e9, 3, t)
            e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize(dev)
    launches = sysm.launch_count() - launches0
    ms = e0.elapsed_time(e1)
    if dist:
        ms = max_over_ranks(torch, dist, dev, ms)
    sol = sysm.GetSolutionColumn()
    kt = sysm.kernel_times(reps=5)
    # end to end through the C ABI with pinned host buffers
    e2e_s, seq_s = e2e_runs(torch, dev, sysm, sol, t, args.steps, 1e9, dist) if e2e else (1.0, 1.0)
    sysm.close()
    return {"value": 3 * L * args.steps * world / (ms * 1e-3), "ms_per_step": ms / args.steps,
            "e2e": 3 * L * args.steps * world / e2e_s, "e2e_sequential": 3 * L * args.steps * world / seq_s,
            "launches": launches, "kernel_ms": kt,
            "clocks": clocks.summary(), "solution": sol, "t": t, "autotune": tune}


# DRAM bytes (read + write) per launch measured by one ncu capture on the
# 40^3 p = 3 case (64 000 cells); scaled linearly with the cell count.  Mixed
# form: the traced face kernel and the cell kernel writing the node traces.
NCU_TRAFFIC_40 = {
    ("mixed", "face_flux"): 380.926720e6 + 50.025984e6,
    ("mixed", "cell_update"): 591.940608e6 + 229.314048e6,  # the RK3 last stage
}
NCU_CELLS = 40 ** 3


# Whole-step roofline (the fixed convention of the workload's algorithmic
# counts): T_roof = max(B / BW_HBM, F64 / P_FP64, F32 / P_FP32) for one SSP-RK3
# step of three stages, achieved = T_roof / T_measured.  The dt reduction and
# limiter passes add measured time but no algorithmic counts.  B: per stage
# 8 L (stage input) + 8 L (u_n, stages 2-3) + 8 L (output) + geometry (Hex8
# 192 B, Tet4 96 B, Wedge6 144 B, Pyra5 120 B per cell) + 4 B per face slot.
# FP64 / FP32 flops per the form: the plain form counts every flop as FP64;
# the mixed form moves the contractions (volume flux and contravariant
# transform, differentiation, lift) to FP32 and keeps the Riemann fluxes and
# the RK accumulation in FP64.  P_FP32 is the nominal SIMT rate (152 SMs x 128
# lanes x 2 flops x 2.07 GHz); the contractions run on the FP32 SIMT pipe.
FP32_SIMT_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
C_R = {"rusanov": 60, "hllc": 120, "roe": 200, "exact": 400, "ausm": 80}


def step_roofline(bytes_step, f64_step, f32_step, ms_per_step, hbm_peak, fp64_peak, peak_src):
    terms = {"hbm": bytes_step / (hbm_peak * 1e9), "fp64": f64_step / (fp64_peak * 1e12),
             "fp32": f32_step / (FP32_SIMT_PEAK_TFLOPS * 1e12)}
    bound = max(terms, key=terms.get)
    t_roof = terms[bound]
    return {"t_roof_ms": t_roof * 1e3, "t_measured_ms": ms_per_step, "achieved": t_roof / (ms_per_step * 1e-3),
            "bound": bound, "alg_bytes_per_step": bytes_step, "alg_fp64_flops_per_step": f64_step,
            "alg_fp32_flops_per_step": f32_step, "terms_ms": {k: v * 1e3 for k, v in terms.items()},
            "peaks": {"hbm_gbs": hbm_peak, "hbm_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                      "fp64_tflops": fp64_peak, "fp64_source": "cuBLAS DGEMM 4096^3 measured in this run",
                      "fp32_tflops": FP32_SIMT_PEAK_TFLOPS, "fp32_source": "nominal SIMT rate at 2070 MHz"}}


def nodal_step_counts(L, cells, degree, riemann, precision):
    """Algorithmic bytes and FP64 / FP32 flops of one SSP-RK3 step of DGSEM
    (Hex8 cells, the three stages)."""
    Q = degree + 1
    N = Q ** 3
    per_stage_bytes = 24 * L + (192 + 4 * 6) * cells
    bytes_step = 3 * per_stage_bytes - 8 * L  # stage 1 reads no u_n
    contraction = 130 / K + 6 * Q            # per DOF: volume flux + transform, differentiation
    riemann_f = 3 * Q * Q * C_R[riemann] / (N * K)
    if precision == "mixed":
        f64, f32 = riemann_f + 4, contraction
    else:
        f64, f32 = contraction + riemann_f + 4, 0.0
    return bytes_step, 3 * f64 * L, 3 * f32 * L


def roofline_of(kt, L, cells, hbm_peak, peak_src, fp64_peak, precision):
    """Roofline of the dominant kernel (algorithmic counts per launch)."""
    N = (DEGREE + 1) ** 3
    qf = (DEGREE + 1) ** 2
    dom = "cell_update" if kt["cell_update"] >= kt["face_flux"] else "face_flux"
    if dom == "cell_update":
        alg_bytes = 24 * L + (192 + 24) * cells
        alg_flops = (4 if precision == "mixed" else (130 / K + 6 * (DEGREE + 1) + 4)) * L
    else:
        alg_bytes = 2 * K * 8 * 3 * cells * qf + K * 8 * 3 * cells * qf
        alg_flops = 3 * qf * 60 / (N * K) * L
    t_dom = kt[dom] * 1e-3
    achieved = alg_bytes / t_dom / 1e9
    traffic = NCU_TRAFFIC_40.get((precision, dom))
    traffic = traffic * cells / NCU_CELLS if traffic is not None and DEGREE == 3 else None
    return {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": traffic, "traffic_source": "ncu dram__bytes_read+write on 40^3, scaled by cells",
            "alg_bytes_per_launch": alg_bytes, "launch_ms": kt[dom],
            "fp64": {"achieved": alg_flops / t_dom / 1e12, "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": alg_flops / t_dom / 1e12 / fp64_peak,
                     "peak_source": "measured in this run: cuBLAS DGEMM 4096^3",
                     "alg_flops_per_launch": alg_flops},
            "binding": "fp64 pipe", "pipe_utilisation": NCU_PIPE_40.get((precision, dom)),
            "kernel_ms": kt}


# FP64-pipe utilisation of the dominant kernels (ncu --set full on the 40^3
# p = 3 case, one capture per kernel): the mixed form's
# algorithmic FP64 flops (RK accumulation, 4 per DOF) understate the FP64
# instruction stream (conversions, node traces, positivity), which is what
# binds the kernel.
NCU_PIPE_40 = {
    ("mixed", "cell_update"): {"sm__pipe_fp64_cycles_active_pct": 80.1, "issue_active_pct": 50.4,
                               "source": "ncu --metrics, 40^3 p = 3 case, RK3 last stage"},
    ("mixed", "face_flux"): {"sm__pipe_fp64_cycles_active_pct": 89.4, "issue_active_pct": 17.0,
                             "source": "ncu --metrics, 40^3 p = 3 case"},
}


# ---------------------------------------------------------------------------
# Mixed hex + tet box: modal DG (dg::General over Projection), p = 2, HLLC.
# Two independent periodic unit-cube blocks: 100^3 Hex8 and 64^3 x 6 Tet4
# (Kuhn split), interior nodes jittered U(-0.1 h, 0.1 h), seed 0; 2,572,864
# cells, M = 10, L = 128,643,200.  rho = 1 + 0.2 sin(2 pi x) cos(2 pi y),
# u = (0.5, 0.3, 0.1), p = 1; CFL from the reference table (0.209).
MIXED_HEX_1D, MIXED_TET_1D, MIXED_DEGREE, MIXED_SAMPLE = 100, 64, 2, (12, 8)
C_HLLC = 120


def mixed_box_mesh(n_hex, n_tet):
    from pvcriemannsolvers_gb300 import cases
    return cases.mixed_box_mesh(n_hex, n_tet)


def mixed_box_ic(x):
    from pvcriemannsolvers_gb300 import cases
    return cases.mixed_box_ic(x)


def mixed_box_config(n_hex, n_tet):
    cells = n_hex ** 3 + 6 * n_tet ** 3
    m = (MIXED_DEGREE + 1) * (MIXED_DEGREE + 2) * (MIXED_DEGREE + 3) // 6
    return {"workload": f"mixed box: periodic unit cube {n_hex}^3 Hex8 + periodic unit cube {n_tet}^3 x 6 Tet4, "
                        f"jitter 0.1 h, modal DG p={MIXED_DEGREE} (dg::General + Projection), HLLC, SSP-RK3, "
                        f"CFL 0.209 (reference table)",
            "cells": cells, "dofs": cells * m * K, "form": "plain FP64",
            "quadrature": "Hex8 Gauss 3^3 / Quad4 3^2; Tet4 14 points / Tri3 6 points",
            "step": "dt reduction + 3 RK stages (3 kernels each)",
            "l2_flush": "inputs larger than L2 (solution column 1.03 GB)"}


# All four cell types of the modal scheme: independent periodic unit-cube
# blocks of Hex8, Tet4 (Kuhn split), Wedge6 (2 per hex) and Pyra5 (6 per hex,
# apex at the hex's centroid), jitter 0.1 h, the mixed box's initial state.
ALL_TYPES = (60, 32, 48, 32)
ALL_TYPES_SAMPLE = (8, 6, 8, 6)


def _wavy(eps):
    """x + eps (sin 2 pi y sin 2 pi z, ...): smooth and periodic on the unit cube"""
    def fn(x):
        s = np.sin(2 * np.pi * x)
        y = x.copy()
        y[:, 0] += eps * s[:, 1] * s[:, 2]
        y[:, 1] += eps * s[:, 2] * s[:, 0]
        y[:, 2] += eps * s[:, 0] * s[:, 1]
        return y
    return fn


def all_types_mesh(n_hex, n_tet, n_wedge, n_pyr, curved=False):
    """curved: every block quadratic (Hex27, Tet10, Wedge18, Pyra14) with its
    nodes moved by a smooth periodic deformation of amplitude 0.02."""
    from pvcriemannsolvers_gb300 import mesh as meshlib
    kw = dict(periodic=(True,) * 3, jitter=0.1, seed=0)
    m = meshlib.concat(meshlib.box((n_hex,) * 3, **kw), meshlib.tet_box((n_tet,) * 3, **kw),
                       meshlib.wedge_box((n_wedge,) * 3, **kw), meshlib.pyramid_box((n_pyr,) * 3, **kw))
    return meshlib.deform(meshlib.quadratic(m), _wavy(0.02)) if curved else m


def all_types_config(n_hex, n_tet, n_wedge, n_pyr, curved=False):
    cells = n_hex ** 3 + 6 * n_tet ** 3 + 2 * n_wedge ** 3 + 6 * n_pyr ** 3
    m = (MIXED_DEGREE + 1) * (MIXED_DEGREE + 2) * (MIXED_DEGREE + 3) // 6
    names = ("Hex27", "Tet10", "Wedge18", "Pyra14") if curved else ("Hex8", "Tet4", "Wedge6", "Pyra5")
    shape = ", quadratic nodes moved by a periodic deformation of amplitude 0.02" if curved else ""
    return {"workload": f"{'curved' if curved else 'all'} cell types: periodic unit cubes {n_hex}^3 {names[0]} + "
                        f"{n_tet}^3 x 6 {names[1]} + {n_wedge}^3 x 2 {names[2]} + {n_pyr}^3 x 6 {names[3]}, "
                        f"jitter 0.1 h{shape}, modal DG p={MIXED_DEGREE} "
                        f"(dg::General + Projection), HLLC, SSP-RK3, CFL 0.209 (reference table)",
            "cells": cells, "dofs": cells * m * K, "form": "plain FP64",
            "quadrature": "hexahedra Gauss 3^3; tetrahedra 14; wedges 6 x 3; pyramids 3^2 x Gauss-Jacobi 3; faces "
                          "3^2 / 6" + (" (curved: cell maps, pyramid faces on their own Triangle6 / Quadrangle9 maps)"
                                       if curved else ""),
            "step": "dt reduction + 3 RK stages (3 kernels each)",
            "l2_flush": f"inputs larger than L2 (solution column {8 * cells * m * K / 1e6:.0f} MB)"}


def mixed_box_cpu_sample(seconds=12.0, threads=None, fixed_steps=None, kind="mixed_box"):
    import oracle.orc as orc
    orc.build()
    threads = threads or os.cpu_count() or 1
    orc.set_threads(threads)
    m = mixed_box_mesh(*MIXED_SAMPLE) if kind == "mixed_box" else \
        all_types_mesh(*ALL_TYPES_SAMPLE, curved=kind == "curved_types")
    o = orc.Modal(m, MIXED_DEGREE)
    x, _ = o.points()
    u = o.project(mixed_box_ic(x))
    L = u.size
    t, n, t0 = 0.0, 0, time.perf_counter()
    while True:
        dt = o.time_step(u, 1e9, 3, 0.0)
        u = o.rk_update(orc.HLLC, 3, t, dt, u)
        t += dt
        n += 1
        el = time.perf_counter() - t0
        if (fixed_steps is not None and n >= fixed_steps) or (fixed_steps is None and el >= seconds):
            break
    el = time.perf_counter() - t0
    what = (f"mixed box {MIXED_SAMPLE[0]}^3 Hex8 + {MIXED_SAMPLE[1]}^3 x 6 Tet4" if kind == "mixed_box" else
            "all types {}^3 Hex8 + {}^3 x 6 Tet4 + {}^3 x 2 Wedge6 + {}^3 x 6 Pyra5".format(*ALL_TYPES_SAMPLE) +
            (", quadratic and deformed" if kind == "curved_types" else ""))
    return {"value": 3 * L * n / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{what} (L = {L} DOFs), {n} SSP-RK3 steps, {el:.1f} s, oracle (plain C restatement, OpenMP)",
            "seconds": el, "steps": n}


def modal_roofline(kt, m, L, fp64_peak, hbm_peak, peak_src):
    """Algorithmic counts of the modal kernels (per launch).
    cell kernel: volume 2 K 3 M per quadrature point (F . grad psi), lift
    2 K M per face point and side, stage 4 per DOF; bytes: 3 column
    accesses + Hex8 192 B / Tet4 96 B of geometry + 4 B per face slot.
    face kernel: 2 x 2 K M (both traces) + c_R per face point."""
    from pvcriemannsolvers_gb300 import mesh as meshlib
    M = (MIXED_DEGREE + 1) * (MIXED_DEGREE + 2) * (MIXED_DEGREE + 3) // 6
    Q = MIXED_DEGREE + 1
    # the quadratic types by their family (the kernels read the same
    # precomputed point data)
    ct = np.array([0, 1, 0, 1, 0, meshlib.WEDGE6, meshlib.PYRA5, meshlib.WEDGE6, meshlib.WEDGE6, meshlib.PYRA5,
                   meshlib.PYRA5])[m.cell_type]
    # per type: volume points, geometry bytes (3 doubles per corner), face slots
    per = {0: (Q ** 3, 192, 6), 1: (14, 96, 4), meshlib.WEDGE6: (6 * Q, 144, 5), meshlib.PYRA5: (Q ** 3, 120, 5)}
    counts = {t: int((ct == t).sum()) for t in per}
    nq = sum(counts[t] * per[t][0] for t in per)
    interior = m.face_cells[:, 1] >= 0
    hold = ct[m.face_cells[:, 0]]
    quad = np.array([meshlib.CELL_FACES[meshlib.family(t)][sd][3] >= 0
                     for t, sd in zip(hold, m.face_sides[:, 0])]) if (hold > 1).any() else hold == 0
    fq_face = np.where(quad, Q * Q, 6)
    face_pts = int(fq_face.sum())
    face_sides = int(fq_face.sum() + fq_face[interior].sum())
    cell_flops = 2 * K * 3 * M * nq + 2 * K * M * face_sides + 4 * L
    face_flops = face_pts * (4 * K * M + C_HLLC)
    cell_bytes = 24 * L + sum(counts[t] * per[t][1] for t in per) + 4 * sum(counts[t] * per[t][2] for t in per)
    if kt is None:  # the counts of one SSP-RK3 step for step_roofline: (bytes, FP64, FP32) per form
        f64_mixed = face_pts * C_HLLC + 4 * L
        return {"fp64": (3 * cell_bytes - 8 * L, 3 * (cell_flops + face_flops), 0.0),
                "mixed": (3 * cell_bytes - 8 * L, 3 * f64_mixed, 3 * (cell_flops + face_flops) - 3 * f64_mixed)}
    dom = "cell_update" if kt["cell_update"] >= kt["face_flux"] else "face_flux"
    flops = cell_flops if dom == "cell_update" else face_flops
    t = kt[dom] * 1e-3
    ach = flops / t / 1e12
    return {"bound": "fp64", "kernel": dom, "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
            "frac": ach / fp64_peak, "peak_source": "measured in this run: cuBLAS DGEMM 4096^3",
            "traffic": None, "alg_flops_per_launch": flops, "launch_ms": kt[dom],
            "hbm": {"alg_bytes_per_launch": cell_bytes, "achieved": cell_bytes / (kt["cell_update"] * 1e-3) / 1e9,
                    "peak": hbm_peak, "unit": "GB/s", "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)"},
            "kernel_ms": kt,
            "note": "face_flux includes the Taylor-coefficient kernel a = S^T c"}


def run_mixed_box(args, rank, world, local_rank, kind="mixed_box"):
    import torch
    from pvcriemannsolvers_gb300 import General, build
    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    n_hex, n_tet = args.mixed_cells
    m = mixed_box_mesh(n_hex, n_tet) if kind == "mixed_box" else \
        all_types_mesh(*ALL_TYPES, curved=kind == "curved_types")
    res = {}
    u0 = None
    for form in ("fp64", "mixed"):
        sysm = General(m, MIXED_DEGREE, "hllc", device=local_rank, precision=form)
        stream = torch.cuda.Stream(device=dev)
        sysm.set_stream(stream.cuda_stream)
        if u0 is None:
            sysm.project(mixed_box_ic(sysm.points()))
            u0 = sysm.GetSolutionColumn()
        else:
            sysm.SetSolutionColumn(u0)
        L = u0.size
        sysm.autotune()
        t = sysm.advance(args.warmup, 1e9, 3, 0.0)
        sysm.synchronize()
        torch.cuda.synchronize(dev)
        launches0 = sysm.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local_rank) as clocks:
            with torch.cuda.stream(stream):
                e0.record(stream)
                t = sysm.advance(args.steps, 1e9, 3, t)
                e1.record(stream)
            e1.synchronize()
        launches = sysm.launch_count() - launches0
        ms = e0.elapsed_time(e1)
        sol = sysm.GetSolutionColumn()
        kt = sysm.kernel_times(reps=3)
        e2e_steps = max(1, min(args.steps, 20))
        e2e_s, seq_s = e2e_runs(torch, dev, sysm, sol, t, e2e_steps, 1e9)
        sysm.close()
        res[form] = {"value": 3 * L * args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps,
                     "e2e": 3 * L * e2e_steps / e2e_s, "e2e_sequential": 3 * L * e2e_steps / seq_s,
                     "launches": launches, "kernel_ms": kt,
                     "clocks": clocks.summary(), "t": t, "solution": sol, "e2e_steps": e2e_steps}
    hbm_peak, peak_src = measured_peaks()
    fp64_peak = fp64_peak_tflops(torch, dev)
    cpu = None
    if not args.no_cpu:
        cpu = mixed_box_cpu_sample(kind=kind)
        cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    a = res["mixed"]["solution"].reshape(-1, K)[:, 0]
    b = res["fp64"]["solution"].reshape(-1, K)[:, 0]
    r = res["mixed"]
    L = u0.size
    cfg = mixed_box_config(n_hex, n_tet) if kind == "mixed_box" else \
        all_types_config(*ALL_TYPES, curved=kind == "curved_types")
    cfg["form"] = "mixed (FP32 contractions; FP64 face states, Riemann fluxes, RK)"
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
        "config": cfg,
        "accuracy": {"t_end": r["t"], "finite": bool(np.isfinite(r["solution"]).all()),
                     "mixed_vs_fp64_density_rel_l2": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                     "note": "density coefficients on each cell's orthonormal basis (their L2 is the field L2)"},
        "clocks": r["clocks"],
        "e2e": {"value": r["e2e"], "unit": UNIT, "h2d_bytes_per_step": 8 * L,
                "d2h_bytes_per_step": 8 * L, "steps": r["e2e_steps"], "path": E2E_PATH,
                "sequential": {"value": r["e2e_sequential"], "path": E2E_SEQ_PATH}},
        "gpu_launches": r["launches"],
        "plain_fp64": {k: res["fp64"][k] for k in ("value", "ms_per_step", "e2e", "e2e_sequential", "launches",
                                                   "kernel_ms", "clocks")},
        "roofline": modal_roofline(res["fp64"]["kernel_ms"], m, L, fp64_peak, hbm_peak, peak_src),
        "cpu_baseline": cpu,
    }
    line["roofline"]["note"] = ("FP64 form's dominant kernel (the mixed form moves the contractions "
                                "to FP32); face_flux includes the Taylor-coefficient kernel a = S^T c")
    line["roofline"]["mixed_kernel_ms"] = r["kernel_ms"]
    counts = modal_roofline(None, m, L, fp64_peak, hbm_peak, peak_src)
    line["roofline"]["step"] = step_roofline(*counts["mixed"], r["ms_per_step"], hbm_peak, fp64_peak, peak_src)
    line["plain_fp64"]["roofline_step"] = step_roofline(*counts["fp64"], res["fp64"]["ms_per_step"], hbm_peak,
                                                        fp64_peak, peak_src)
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Ensemble: 64 independent periodic unit-cube cases (numpy PCG64 seed 1):
# element counts log-uniform in [4k, 200k]; each case Hex8 or 6-tet-split
# (fair draw), p in {1, 2, 3} (uniform draw); Hex8 cases use DGSEM or modal
# DG (fair draw), Tet4 cases modal DG; Rusanov; rho = 1 + sum_{m=1..3}
# a_m sin(2 pi k_m . x + phi_m), a_m ~ U(0, 0.1), |k_m|_inf <= 3,
# phi_m ~ U(0, 2 pi); uniform velocity, direction on the sphere, magnitude
# U(0, 0.5); p = 1.  Cases of one (scheme, p) share a handle (mcfd_set_cases,
# own dt and t per case); the handles form one mcfd_ensemble (one CUDA graph
# per step, forked over the handles' streams).
ENSEMBLE_CASES = 64


def ensemble_spec(n_cases=ENSEMBLE_CASES, seed=1, scale=1.0):
    from pvcriemannsolvers_gb300 import cases
    return cases.ensemble_spec(n_cases, seed, scale)


def ensemble_state(x, spec):
    from pvcriemannsolvers_gb300 import cases
    return cases.ensemble_state(x, spec)


def ensemble_mesh(spec):
    from pvcriemannsolvers_gb300 import cases
    return cases.ensemble_mesh(spec)


def build_ensemble(specs, device=0, precision="fp64"):
    """Group the cases by (scheme, p); one handle per group with its cases."""
    from pvcriemannsolvers_gb300 import General, Lobatto, mesh as meshlib
    groups = {}
    for sp in specs:
        groups.setdefault((sp["scheme"], sp["p"]), []).append(sp)
    members = []
    for (scheme, p), sps in sorted(groups.items()):
        meshes = [ensemble_mesh(sp) for sp in sps]
        m = meshlib.concat(*meshes)
        sysm = General(m, p, "rusanov", device=device, precision=precision) if scheme == "modal" else \
            Lobatto(m, p, "rusanov", device=device, precision=precision)
        if scheme == "modal":
            # volume points come cell by cell; a case's cells are one type
            pts = sysm.points()
            vals, off = [], 0
            for q, sp in zip(meshes, sps):
                ppc = (p + 1) ** 3 if not sp["tet"] else (14 if p <= 2 else 24)
                n = q.n_cells * ppc
                vals.append(ensemble_state(pts[off:off + n], sp))
                off += n
            sysm.project(np.concatenate(vals))
        else:
            cols = [ensemble_state(meshlib.node_coordinates(q, p).reshape(-1, 3), sp).ravel()
                    for q, sp in zip(meshes, sps)]
            sysm.SetSolutionColumn(np.concatenate(cols))
        sysm.set_cases(np.concatenate([[0], np.cumsum([q.n_cells for q in meshes])]))
        members.append({"scheme": scheme, "p": p, "system": sysm, "cases": len(sps),
                        "cells": m.n_cells, "dofs": sysm.column_size})
    return members


def ensemble_cpu_sample(specs, seconds=12.0, threads=None):
    """The oracle on the smallest cases of the ensemble, one after another."""
    import oracle.orc as orc
    orc.build()
    threads = threads or os.cpu_count() or 1
    orc.set_threads(threads)
    from pvcriemannsolvers_gb300 import mesh as meshlib
    done, dofs_steps, t0 = 0, 0, time.perf_counter()
    for sp in sorted(specs, key=lambda s: s["n"] ** 3 * (6 if s["tet"] else 1)):
        q = ensemble_mesh(sp)
        if sp["scheme"] == "modal":
            o = orc.Modal(q, sp["p"])
            u = o.project(ensemble_state(o.points()[0], sp))
        else:
            o = orc.Mesh(q, sp["p"])
            u = ensemble_state(meshlib.node_coordinates(q, sp["p"]).reshape(-1, 3), sp).ravel()
        t = 0.0
        for _ in range(2):
            dt = o.time_step(u, 1e9, 3, 0.0)
            u = o.rk_update(orc.RUSANOV, 3, t, dt, u)
            t += dt
            dofs_steps += 3 * u.size
        done += 1
        if time.perf_counter() - t0 >= seconds:
            break
    el = time.perf_counter() - t0
    return {"value": dofs_steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"the {done} smallest ensemble cases, 2 SSP-RK3 steps each, {el:.1f} s, "
                      f"oracle (plain C restatement, OpenMP)"}


def ensemble_form(args, torch, dev, local_rank, specs, precision):
    """Time one precision form of the ensemble: device-resident steps, e2e."""
    from pvcriemannsolvers_gb300 import Ensemble
    members = build_ensemble(specs, device=local_rank, precision=precision)
    for mb in members:
        mb["system"].autotune()
    ens = Ensemble([mb["system"] for mb in members])
    stream = torch.cuda.Stream(device=dev)
    ens.set_stream(stream.cuda_stream)
    L = sum(mb["dofs"] for mb in members)
    ens.advance(args.warmup, 1e9, 3)
    torch.cuda.synchronize(dev)
    launches0 = sum(mb["system"].launch_count() for mb in members)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        with torch.cuda.stream(stream):
            e0.record(stream)
            ens.advance(args.steps, 1e9, 3)
            e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1)
    launches = sum(mb["system"].launch_count() for mb in members) - launches0
    solution = [mb["system"].GetSolutionColumn() for mb in members]
    # end to end: every member's column from / to pinned host memory each step
    hosts = []
    for mb, sol in zip(members, solution):
        n = mb["dofs"]
        hin = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
        hout = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
        hin[:] = sol
        hosts.append((hin, hout))
    e2e_steps = max(1, min(args.steps, 20))
    ins, outs = [h[0] for h in hosts], [h[1] for h in hosts]
    ens.stream_begin()  # staging allocation and the job set-up, untimed
    ens.stream_step(ins, outs, 1, 1e9, 3)
    ens.stream_end()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    ens.stream_begin()
    for _ in range(e2e_steps):
        ens.stream_step(ins, outs, 1, 1e9, 3)
    ens.stream_end()
    torch.cuda.synchronize(dev)
    e2e_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for mb, (hin, _) in zip(members, hosts):
            mb["system"].SetSolutionColumn(hin)
        ens.advance(1, 1e9, 3)
        for mb, (_, hout) in zip(members, hosts):
            mb["system"].get_solution_into(hout)
    torch.cuda.synchronize(dev)
    seq_s = time.perf_counter() - t0
    per_member = []
    for mb in members:
        kt = mb["system"].kernel_times(reps=3)
        t_cases, _ = mb["system"].case_times()
        per_member.append({"scheme": mb["scheme"], "p": mb["p"], "cases": mb["cases"], "cells": mb["cells"],
                           "dofs": mb["dofs"], "kernel_ms": kt, "case_t_min": float(t_cases.min()),
                           "case_t_max": float(t_cases.max())})
    ens.close()
    for mb in members:
        mb["system"].close()
    return {"value": 3 * L * args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps,
            "e2e": 3 * L * e2e_steps / e2e_s, "e2e_sequential": 3 * L * e2e_steps / seq_s,
            "e2e_steps": e2e_steps, "launches": launches,
            "clocks": clocks.summary(), "members": per_member, "solution": solution, "L": L}


def run_ensemble(args, rank, world, local_rank):
    import torch
    from pvcriemannsolvers_gb300 import build
    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    specs = ensemble_spec(scale=args.ensemble_scale)
    res = {f: ensemble_form(args, torch, dev, local_rank, specs, f) for f in ("fp64", "mixed")}
    r, pf = res["mixed"], res["fp64"]
    L = r["L"]
    # density of every member: nodal values (DGSEM) or the coefficients on the
    # orthonormal basis (modal), whose L2 is the field's L2
    a = np.concatenate([s.reshape(-1, K)[:, 0] for s in r["solution"]])
    b = np.concatenate([s.reshape(-1, K)[:, 0] for s in pf["solution"]])
    fp64_peak = fp64_peak_tflops(torch, dev)
    hbm_peak, peak_src = measured_peaks()
    dom = max(pf["members"], key=lambda m: m["kernel_ms"]["rk3_step"])
    cpu = None
    if not args.no_cpu:
        cpu = ensemble_cpu_sample(specs)
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
        "config": {"workload": f"ensemble of {len(specs)} periodic unit-cube cases (seed 1), counts log-uniform "
                               f"in [4k, 200k] x {args.ensemble_scale}, Hex8 DGSEM / Hex8 modal / Tet4 modal, "
                               f"p in 1..3, Rusanov, SSP-RK3, own dt per case",
                   "cases": len(specs), "cells": sum(m["cells"] for m in r["members"]), "dofs": L,
                   "handles": len(r["members"]),
                   "form": "mixed (FP32 contractions; FP64 Riemann fluxes and RK)",
                   "step": "one CUDA graph per step: every handle's dt reduction + 3 RK stages",
                   "l2_flush": f"inputs larger than L2 (all columns {8 * L / 1e9:.2f} GB)"},
        "accuracy": {"mixed_vs_fp64_density_rel_l2": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                     "finite": bool(np.isfinite(a).all())},
        "clocks": r["clocks"],
        "e2e": {"value": r["e2e"], "unit": UNIT, "h2d_bytes_per_step": 8 * L,
                "d2h_bytes_per_step": 8 * L, "steps": r["e2e_steps"],
                "path": "mcfd_ensemble_stream_step per step (every member's column in from pinned host memory, "
                        "one ensemble step, the columns out; neighbouring steps' copies overlap the compute)",
                "sequential": {"value": r["e2e_sequential"],
                               "path": "mcfd_set_solution per handle + mcfd_ensemble_advance(1) + "
                                       "mcfd_get_solution per handle"}},
        "gpu_launches": r["launches"],
        "members": r["members"],
        "plain_fp64": {"value": pf["value"], "ms_per_step": pf["ms_per_step"], "e2e": pf["e2e"],
                       "launches": pf["launches"], "clocks": pf["clocks"], "members": pf["members"]},
        "roofline": {"bound": "fp64", "kernel": f"step of the {dom['scheme']} p={dom['p']} handle (FP64 form)",
                     "achieved": None, "peak": fp64_peak, "unit": "TFLOP/s", "frac": None,
                     "traffic": None, "peak_source": "measured in this run: cuBLAS DGEMM 4096^3",
                     "hbm_peak": hbm_peak, "hbm_peak_source": peak_src,
                     "note": "per-kernel rooflines of these kernels: the vortex and mixed-box lines"},
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Four-quadrant Riemann problem (demo/euler/riemann2d.cpp:5-53): 256 x 256 x
# 16 Hex8 on [0,1]^2 x [0,0.0625], DGSEM p = 2, Roe, SSP-RK3 at the reference
# CFL table value (0.209), weno::Eigen limiter (jump detector + characteristic
# reconstruction) after every stage; walls on top/right/front/back, moving-
# shock smart states left/bottom.  Both precision forms; the troubled
# fraction is reconstructions per cell per limiter pass.
QUAD_DEGREE = 2
QUAD_SAMPLE = (32, 32, 2)


def quadrant_oracle_bcs():
    import oracle.orc as orc
    from pvcriemannsolvers_gb300 import MovingSplit, cases
    return {0: (orc.BC_SMART, MovingSplit(axis=1, position=0.8, speed=cases.SPEED_BC, a=cases.Q_C, b=cases.Q_B)),
            1: (orc.BC_INVISCID_WALL, None),
            2: (orc.BC_SMART, MovingSplit(axis=0, position=0.8, speed=cases.SPEED_CD, a=cases.Q_C, b=cases.Q_D)),
            3: (orc.BC_INVISCID_WALL, None), 4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_INVISCID_WALL, None)}


QUAD_FLOOR_STEPS = 200
# the forms of the four-quadrant workload: plain FP64 (the result), mixed,
# and mixed with the flagged cells and their neighbours in FP64
QUAD_FORMS = {"fp64": dict(precision="fp64"), "mixed": dict(precision="mixed"),
              "mixed_shock_fp64": dict(precision="mixed", shock_cells_fp64=1),
              "mixed_shock_fp64_2": dict(precision="mixed", shock_cells_fp64=2)}


def quadrant_cpu_sample(threads=None, steps=QUAD_FLOOR_STEPS, device=0):
    """The oracle on the 32 x 32 x 2 cells of the same case (all host cores)
    for the case's 200 steps, timed; the same steps on the GPU in both forms
    from the same initial state give the FP64 floor of the comparison: how far
    the FP64 GPU run drifts from the FP64 oracle (the same algorithm in
    another rounding order) on this limited shock problem, next to the mixed
    form's deviation."""
    import oracle.orc as orc
    from pvcriemannsolvers_gb300 import Lobatto, cases, mesh as meshlib
    orc.build()
    threads = threads or os.cpu_count() or 1
    orc.set_threads(threads)
    m = cases.quadrant_mesh(*QUAD_SAMPLE)
    u0 = cases.quadrant_ic(meshlib.node_coordinates(m, QUAD_DEGREE).reshape(-1, 3)).ravel()
    om = orc.Mesh(m, QUAD_DEGREE)
    om.set_bcs(quadrant_oracle_bcs())
    lim = orc.Limiter(om, orc.LIMITER_EIGEN)
    u, _ = lim.limit(u0)
    t, t0 = 0.0, time.perf_counter()
    for _ in range(steps):
        dt = om.time_step(u, 1.0, 3, 0.0)
        u = lim.rk_update(orc.ROE, 3, t, dt, u)
        t += dt
    el = time.perf_counter() - t0
    gpu = {}
    for form, kw in QUAD_FORMS.items():
        s = Lobatto(m, QUAD_DEGREE, "roe", device=device, limiter="eigen", **kw)
        cases.quadrant_bc(s)
        s.SetSolutionColumn(u0)
        s.advance(steps, 1.0, 3, 0.0)
        gpu[form] = s.GetSolutionColumn().reshape(-1, K)[:, 0]
        s.close()
    rho = u.reshape(-1, K)[:, 0]
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    floor = {"steps": steps, "mesh": "x".join(map(str, QUAD_SAMPLE)),
             "fp64_gpu_vs_fp64_oracle_density_rel_l2": rel(gpu["fp64"], rho),
             "mixed_gpu_vs_fp64_gpu_density_rel_l2": rel(gpu["mixed"], gpu["fp64"]),
             "mixed_gpu_vs_fp64_oracle_density_rel_l2": rel(gpu["mixed"], rho),
             "mixed_shock_fp64_gpu_vs_fp64_gpu_density_rel_l2": rel(gpu["mixed_shock_fp64"], gpu["fp64"]),
             "mixed_shock_fp64_2_gpu_vs_fp64_gpu_density_rel_l2": rel(gpu["mixed_shock_fp64_2"], gpu["fp64"])}
    return {"value": 3 * u.size * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{QUAD_SAMPLE[0]}x{QUAD_SAMPLE[1]}x{QUAD_SAMPLE[2]} cells of the same case "
                      f"(L = {u.size} DOFs), {steps} SSP-RK3 steps with the limiter, {el:.1f} s, oracle (OpenMP)",
            "floor": floor}


def run_quadrant(args, rank, world, local_rank):
    import torch
    from pvcriemannsolvers_gb300 import Lobatto, build, cases, mesh as meshlib
    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    nx, ny, nz = args.quadrant_cells
    m = cases.quadrant_mesh(nx, ny, nz)
    u0 = np.ascontiguousarray(cases.quadrant_ic(meshlib.node_coordinates(m, QUAD_DEGREE).reshape(-1, 3)).ravel())
    L = u0.size
    # --form fp64 / mixed times that form alone (profiling runs); the line
    # then carries no comparison between the forms
    forms = QUAD_FORMS if args.form == "both" else {args.form: QUAD_FORMS[args.form]}
    res = {}
    for form, kw in forms.items():
        sysm = Lobatto(m, QUAD_DEGREE, "roe", device=local_rank, limiter="eigen", **kw)
        cases.quadrant_bc(sysm)
        stream = torch.cuda.Stream(device=dev)
        sysm.set_stream(stream.cuda_stream)
        sysm.SetSolutionColumn(u0)
        sysm.autotune()
        t = sysm.advance(args.warmup, 1.0, 3, 0.0)
        sysm.troubled_cells()
        torch.cuda.synchronize(dev)
        launches0 = sysm.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local_rank) as clocks:
            with torch.cuda.stream(stream):
                e0.record(stream)
                t = sysm.advance(args.steps, 1.0, 3, t)
                e1.record(stream)
            e1.synchronize()
        ms = e0.elapsed_time(e1)
        troubled = sysm.troubled_cells()
        launches = sysm.launch_count() - launches0
        sol = sysm.GetSolutionColumn()
        kt = sysm.kernel_times(reps=3)
        e2e_steps = max(1, min(args.steps, 20))
        e2e_s, seq_s = e2e_runs(torch, dev, sysm, sol, t, e2e_steps, 1.0)
        sysm.close()
        res[form] = {"value": 3 * L * args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps,
                     "e2e": 3 * L * e2e_steps / e2e_s, "e2e_sequential": 3 * L * e2e_steps / seq_s,
                     "launches": launches, "kernel_ms": kt,
                     "clocks": clocks.summary(), "t": t, "solution": sol,
                     "troubled_fraction": troubled / (3.0 * args.steps * m.n_cells)}
    fp64_peak = fp64_peak_tflops(torch, dev)
    if args.form != "both":
        r = res[args.form]
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.form == "fp64" else "f64+f32",
                "data": "synthetic",
                "config": {"workload": f"four-quadrant Riemann problem, {nx}x{ny}x{nz} Hex8, DGSEM "
                                       f"p={QUAD_DEGREE}, Roe, weno::Eigen, {args.form} form alone",
                           "cells": m.n_cells, "dofs": L},
                "clocks": r["clocks"], "gpu_launches": r["launches"], "kernel_ms": r["kernel_ms"],
                "e2e": {"value": r["e2e"], "unit": UNIT, "h2d_bytes_per_step": 8 * L,
                        "d2h_bytes_per_step": 8 * L, "steps": min(args.steps, 20), "path": E2E_PATH},
                "troubled_fraction": r["troubled_fraction"]}
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    a, b = res["mixed"]["solution"].reshape(-1, K)[:, 0], res["fp64"]["solution"].reshape(-1, K)[:, 0]
    # the workload's stated step count on the full mesh: each form from the
    # initial state for 200 steps, densities against the FP64 form's
    long = {}
    for form, kw in QUAD_FORMS.items():
        sysm = Lobatto(m, QUAD_DEGREE, "roe", device=local_rank, limiter="eigen", **kw)
        cases.quadrant_bc(sysm)
        sysm.SetSolutionColumn(u0)
        t_long = sysm.advance(QUAD_FLOOR_STEPS, 1.0, 3, 0.0)
        long[form] = sysm.GetSolutionColumn().reshape(-1, K)[:, 0]
        sysm.close()
    ref_long = long["fp64"]
    accuracy_200 = {"steps": QUAD_FLOOR_STEPS, "t_end": t_long,
                    **{f"{form}_vs_fp64_density_rel_l2": float(np.linalg.norm(v - ref_long) / np.linalg.norm(ref_long))
                       for form, v in long.items() if form != "fp64"}}
    cpu = None
    floor = None
    if not args.no_cpu:
        cpu = quadrant_cpu_sample(device=local_rank)
        floor = cpu.pop("floor")
    # the plain FP64 form is the line's value: with the limiter switching on
    # shocks this case amplifies perturbations over the steps (mixed vs FP64
    # density 4.9e-7 after 53 steps, 4.7e-4 after 200), so the mixed form is
    # reported beside it with its deviation, not as the result
    r = res["fp64"]
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"four-quadrant Riemann problem, {nx}x{ny}x{nz} Hex8, DGSEM p={QUAD_DEGREE}, Roe, "
                               f"SSP-RK3, CFL 0.209, weno::Eigen limiter after every stage",
                   "cells": m.n_cells, "dofs": L,
                   "form": "plain FP64 (mixed beside it: FP32 volume flux + contraction, FP64 Riemann "
                           "fluxes, limiter smoothness and reconstruction, RK)",
                   "step": "dt reduction + 3 x (RK stage + limiter pass)",
                   "l2_flush": "inputs larger than L2 (solution column 1.13 GB)"},
        "accuracy": {"t_end": r["t"], "mixed_vs_fp64_density_rel_l2": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                     "troubled_fraction_mixed": res["mixed"]["troubled_fraction"],
                     "troubled_fraction_fp64": res["fp64"]["troubled_fraction"],
                     "full_mesh_200_steps": accuracy_200,
                     "fp64_floor": floor},
        "clocks": r["clocks"],
        "e2e": {"value": r["e2e"], "unit": UNIT, "h2d_bytes_per_step": 8 * L, "d2h_bytes_per_step": 8 * L,
                "steps": e2e_steps, "path": E2E_PATH,
                "sequential": {"value": r["e2e_sequential"], "path": E2E_SEQ_PATH}},
        "gpu_launches": r["launches"],
        "mixed": {k: res["mixed"][k] for k in ("value", "ms_per_step", "e2e", "e2e_sequential", "launches",
                                                   "kernel_ms", "clocks")},
        "mixed_shock_fp64": dict({k: res["mixed_shock_fp64"][k] for k in ("value", "ms_per_step", "launches",
                                                                          "kernel_ms", "clocks")},
                                 density_rel_l2_vs_fp64=float(np.linalg.norm(
                                     res["mixed_shock_fp64"]["solution"].reshape(-1, K)[:, 0] - b)
                                     / np.linalg.norm(b)),
                                 note="the mixed form with the cells of the last limiter pass's flags "
                                      "and their face neighbours through the FP64 cell update"),
        "mixed_shock_fp64_2": dict({k: res["mixed_shock_fp64_2"][k] for k in ("value", "ms_per_step", "launches",
                                                                              "kernel_ms", "clocks")},
                                   density_rel_l2_vs_fp64=float(np.linalg.norm(
                                       res["mixed_shock_fp64_2"]["solution"].reshape(-1, K)[:, 0] - b)
                                       / np.linalg.norm(b)),
                                   note="as mixed_shock_fp64 with two layers of neighbours"),
        "roofline": {"bound": "fp64", "kernel": "step", "kernel_ms": r["kernel_ms"], "peak": fp64_peak,
                     "unit": "TFLOP/s", "achieved": None, "frac": None, "traffic": None,
                     "peak_source": "measured in this run: cuBLAS DGEMM 4096^3",
                     "note": "per-kernel rooflines of the DGSEM kernels: the vortex line"},
        "cpu_baseline": cpu,
    }
    line["roofline"]["step"] = step_roofline(*nodal_step_counts(L, m.n_cells, QUAD_DEGREE, "roe", "fp64"),
                                             r["ms_per_step"], *measured_peaks()[:1], fp64_peak,
                                             measured_peaks()[1])
    line["mixed"]["roofline_step"] = step_roofline(
        *nodal_step_counts(L, m.n_cells, QUAD_DEGREE, "roe", "mixed"), res["mixed"]["ms_per_step"],
        *measured_peaks()[:1], fp64_peak, measured_peaks()[1])
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_gpu(args, rank, world, local_rank):
    import torch
    from pvcriemannsolvers_gb300 import build, cases, mesh as meshlib
    build.build()
    dist = None
    if world > 1:
        import torch.distributed as dist
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    m = meshlib.box((args.cells,) * 3, lengths=(10.0,) * 3, periodic=(True,) * 3)
    x = meshlib.node_coordinates(m, DEGREE).reshape(-1, 3)
    u0 = np.ascontiguousarray(cases.vortex_ic(x).ravel())
    del x
    L = u0.size
    forms = ["fp64", "mixed"] if args.form == "both" else [args.form]
    res = {f: measure_form(args, torch, dist, dev, local_rank, m, u0, f,
                           contraction="tensor" if (f == "mixed" and args.contraction == "tensor") else "simt")
           for f in forms}
    tensor = None
    if "mixed" in res and DEGREE == 3 and args.contraction == "both":
        # the same mixed form with the differentiation on the tensor cores
        # (TF32x3 mma.sync): timed beside the SIMT path, which stays the
        # headline unless the tensor path is faster
        tensor = measure_form(args, torch, dist, dev, local_rank, m, u0, "mixed", contraction="tensor",
                              e2e=False)
    head = "mixed" if "mixed" in res else "fp64"
    r = res[head]
    accuracy = {"density_rel_l2_vs_exact": density_l2_vs_exact(r["solution"], m, r["t"]), "t_end": r["t"],
                "steps": args.warmup + args.steps}
    if "fp64" in res and "mixed" in res:
        a, b = res["mixed"]["solution"].reshape(-1, K)[:, 0], res["fp64"]["solution"].reshape(-1, K)[:, 0]
        accuracy["mixed_vs_fp64_density_rel_l2"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
        accuracy["fp64_density_rel_l2_vs_exact"] = density_l2_vs_exact(res["fp64"]["solution"], m, res["fp64"]["t"])
    # the workload's stated 100 steps, at half the timed run's CFL step on
    # every mesh
    accuracy["convergence"] = convergence(forms, local_rank, r["t"] / (args.warmup + args.steps),
                                          VORTEX_ACCURACY_STEPS, args.cells)
    hbm_peak, peak_src = measured_peaks()
    fp64_peak = fp64_peak_tflops(torch, dev)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        full = cpu_sample()
        one = cpu_sample(seconds=6.0, threads=1)
        cpu = {k: full[k] for k in ("value", "unit", "cores", "kind", "sample")}
        cpu["single_core"] = {k: one[k] for k in ("value", "cores", "sample")}
    if rank == 0:
        cfg = workload(args.cells)
        cfg["form"] = "mixed (FP32 volume flux + contraction; FP64 Riemann fluxes, lift, RK)" if head == "mixed" \
            else "plain FP64"
        line = {
            "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64+f32" if head == "mixed" else "f64", "data": "synthetic",
            "config": cfg,
            "accuracy": accuracy,
            "clocks": r["clocks"],
            "e2e": {"value": r["e2e"], "unit": UNIT, "h2d_bytes_per_step": 8 * L, "d2h_bytes_per_step": 8 * L,
                    "steps": args.steps, "path": E2E_PATH,
                    "sequential": {"value": r["e2e_sequential"], "path": E2E_SEQ_PATH}},
            "gpu_launches": r["launches"],
            "autotune": r["autotune"],
            "roofline": roofline_of(r["kernel_ms"], L, m.n_cells, hbm_peak, peak_src, fp64_peak, head),
            "cpu_baseline": cpu,
        }
        line["roofline"]["step"] = step_roofline(*nodal_step_counts(L, m.n_cells, DEGREE, "rusanov", head),
                                                 r["ms_per_step"], hbm_peak, fp64_peak, peak_src)
        if tensor is not None:
            ta = tensor["solution"].reshape(-1, K)[:, 0]
            tb = (res["fp64"] if "fp64" in res else res["mixed"])["solution"].reshape(-1, K)[:, 0]
            line["mixed_tensor_contraction"] = {
                "value": tensor["value"], "ms_per_step": tensor["ms_per_step"], "kernel_ms": tensor["kernel_ms"],
                "gpu_launches": tensor["launches"], "clocks": tensor["clocks"],
                "density_rel_l2_vs_fp64": float(np.linalg.norm(ta - tb) / np.linalg.norm(tb)),
                "vs_simt": tensor["value"] / r["value"],
                "note": "DGSEM differentiation as TF32x3 mma.sync m16n8k8 products (FP32 accumulation); "
                        "the line's value is the FP32 SIMT path unless this one is faster"}
        if head == "mixed" and "fp64" in res:
            p = res["fp64"]
            line["plain_fp64"] = {"value": p["value"], "ms_per_step": p["ms_per_step"], "e2e": p["e2e"],
                                  "e2e_sequential": p["e2e_sequential"],
                                  "gpu_launches": p["launches"], "clocks": p["clocks"],
                                  "roofline": roofline_of(p["kernel_ms"], L, m.n_cells, hbm_peak, peak_src,
                                                          fp64_peak, "fp64")}
            line["plain_fp64"]["roofline"]["step"] = step_roofline(
                *nodal_step_counts(L, m.n_cells, DEGREE, "rusanov", "fp64"), p["ms_per_step"], hbm_peak,
                fp64_peak, peak_src)
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Sod shock tube, the reference's CPU-sized case (demo/euler/shock_tube.cpp):
# [0,1] x [0,0.04]^2 with 100 x 4 x 4 Hex8 (h = 0.01), DGSEM p = 2, Roe,
# weno::Lazy on every cell after every stage, SSP-RK3 at CFL 0.1, from t = 0
# to t = 0.2.  The whole run on the GPU (both forms, one CUDA graph per
# step) against the oracle on the same case (all host cores, bounded sample
# of the steps, the run's time extrapolated); parity of the first steps.

def run_sod(args, rank, world, local_rank):
    import torch
    import oracle.orc as orc
    from pvcriemannsolvers_gb300 import Lobatto, build, cases, mesh as meshlib
    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    p, t_end, cfl = 2, 0.2, 0.1
    m = cases.sod_mesh()
    u0 = np.ascontiguousarray(cases.sod_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel())
    L = u0.size
    res = {}
    for form in ("fp64", "mixed"):
        sysm = Lobatto(m, p, "roe", cfl=cfl, device=local_rank, precision=form, limiter="lazy")
        cases.sod_bc(sysm)
        stream = torch.cuda.Stream(device=dev)
        sysm.set_stream(stream.cuda_stream)
        sysm.SetSolutionColumn(u0)
        sysm.advance(args.warmup, 1.0, 3, 0.0)  # warm-up (graph capture), then restart
        sysm.SetSolutionColumn(u0)
        torch.cuda.synchronize(dev)
        launches0 = sysm.launch_count()
        t, n = 0.0, 0
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local_rank) as clocks:
            with torch.cuda.stream(stream):
                e0.record(stream)
                while t < t_end - 1e-12:
                    t = sysm.advance(10, t_end - t if t_end - t < 1.0 else 1.0, 3, t)
                    n += 10
                e1.record(stream)
            e1.synchronize()
        ms = e0.elapsed_time(e1)
        res[form] = {"steps": n, "t": t, "seconds": ms * 1e-3, "value": 3 * L * n / (ms * 1e-3),
                     "launches": sysm.launch_count() - launches0, "clocks": clocks.summary(),
                     "solution": sysm.GetSolutionColumn(), "kernel_ms": sysm.kernel_times(reps=3)}
        sysm.close()
    # the oracle: parity of the first steps, then a bounded timing sample
    orc.build()
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    om = orc.Mesh(m, p)
    om.set_bcs({0: (orc.BC_SMART, cases.SOD_LEFT), 1: (orc.BC_SMART, cases.SOD_RIGHT),
                2: (orc.BC_INVISCID_WALL, None), 3: (orc.BC_INVISCID_WALL, None),
                4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_INVISCID_WALL, None)})
    lim = orc.Limiter(om, orc.LIMITER_LAZY)
    u, _ = lim.limit(u0)
    chk = Lobatto(m, p, "roe", cfl=cfl, device=local_rank, limiter="lazy")
    cases.sod_bc(chk)
    chk.SetSolutionColumn(u0)
    t, n_cpu, t0 = 0.0, 0, time.perf_counter()
    parity = None
    while True:
        dt = om.time_step(u, 1.0, 3, cfl)
        u = lim.rk_update(orc.ROE, 3, t, dt, u)
        t += dt
        n_cpu += 1
        if n_cpu == 5:
            chk.advance(5, 1.0, 3, 0.0)
            g = chk.GetSolutionColumn()
            parity = float(np.linalg.norm(g - u) / np.linalg.norm(u))
            t0_cpu = time.perf_counter()
            n0 = n_cpu
        if n_cpu >= 5 and (time.perf_counter() - t0 >= 12.0 or n_cpu >= res["fp64"]["steps"]):
            break
    cpu_s = time.perf_counter() - t0_cpu
    chk.close()
    cpu_rate = 3 * L * (n_cpu - n0) / cpu_s
    # the plain FP64 form is the line's value: with weno::Lazy on every cell
    # this case amplifies perturbations exponentially (the FP64 GPU run and
    # the FP64 oracle drift apart from 1e-13 at 100 steps to 1e-8 at 400), so
    # the mixed form's FP32 rounding grows to percent-level differences by
    # t = 0.2 and is reported beside it, not as the result
    r, pm = res["fp64"], res["mixed"]
    a, b = pm["solution"].reshape(-1, K)[:, 0], r["solution"].reshape(-1, K)[:, 0]
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": r["steps"],
        "warmup": args.warmup, "ms_per_step": r["seconds"] * 1e3 / r["steps"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "Sod shock tube 100x4x4 Hex8 on [0,1]x[0,0.04]^2, DGSEM p=2, Roe, weno::Lazy "
                               "on every cell after every stage, SSP-RK3, CFL 0.1, t = 0 -> 0.2",
                   "cells": m.n_cells, "dofs": L, "form": "plain FP64 (mixed beside it)",
                   "l2_flush": "none: the whole case (1.7 MB) lives in L2, as it does on the CPU"},
        "time_to_solution_s": {"gpu_fp64": r["seconds"], "gpu_mixed": pm["seconds"],
                               "cpu_oracle_extrapolated": r["steps"] * (cpu_s / (n_cpu - n0))},
        "accuracy": {"gpu_fp64_vs_oracle_rel_l2_after_5_steps": parity,
                     "mixed_vs_fp64_density_rel_l2_at_t_end": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                     "t_end_fp64": r["t"], "t_end_mixed": pm["t"]},
        "clocks": r["clocks"], "gpu_launches": r["launches"],
        "mixed": {k: pm[k] for k in ("value", "steps", "seconds", "launches", "kernel_ms", "clocks")},
        "roofline": {"bound": "latency",
                     "note": "1,600 cells: each kernel fills few SMs; three weno::Lazy passes over every "
                             "cell (one 64-thread block per cell, dependent FP64 phases) take most of the "
                             "step; the step graph removes launch gaps", "kernel_ms": r["kernel_ms"]},
        "cpu_baseline": {"value": cpu_rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"the same case, steps 6..{n_cpu} of {r['steps']}, {cpu_s:.1f} s, oracle "
                                   f"(plain C restatement, OpenMP)"},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Energy-based artificial viscosity on fr::Lobatto (the reference's default
# shock capturing in its viscous demos: demo/euler/sourceless.hpp FR +
# VISCOSITY, Exact Riemann solver, DDG beta0 = 2, beta1 = 0.0833333333,
# time_scale = 0.05 from riemann2d.json / shock_tube_sod.json).
#   value: the four-quadrant demo (riemann2d, average initial limiter) on the
#          four-quadrant mesh, SSP-RK3 with the viscous time step
#   sod:   the Sod demo (majority initial limiter) on the 100x4x4 tube to
#          t = 0.2, GPU time to solution against the oracle's

VISC_BETA0, VISC_BETA1, VISC_TIME_SCALE = 2.0, 0.0833333333, 0.05
VISC_SAMPLE = (48, 48, 2)


def viscous_cpu_sample(seconds=12.0, threads=None):
    """The oracle (EnergyBasedViscosity on fr::Lobatto) on a slice of the
    four-quadrant demo; the damping matrices are built before the clock."""
    import oracle.orc as orc
    from pvcriemannsolvers_gb300 import cases, mesh as meshlib
    orc.build()
    threads = threads or os.cpu_count() or 1
    orc.set_threads(threads)
    m = cases.quadrant_mesh(*VISC_SAMPLE)
    om = orc.Mesh(m, QUAD_DEGREE, scheme="fr")
    om.set_bcs(quadrant_oracle_bcs())
    ov = orc.Viscosity(om, VISC_BETA0, VISC_BETA1, VISC_TIME_SCALE)
    u, _ = orc.initial_limiter(om, orc.INIT_AVERAGE,
                               cases.quadrant_ic(meshlib.node_coordinates(m, QUAD_DEGREE).reshape(-1, 3)).ravel())
    t, n, t0 = 0.0, 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds or n == 0:
        dt = ov.time_step(u, 1.0, 3)
        u = ov.rk_update(orc.EXACT, 3, t, dt, u)
        t += dt
        n += 1
    el = time.perf_counter() - t0
    return {"value": 3 * u.size * n / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{VISC_SAMPLE[0]}x{VISC_SAMPLE[1]}x{VISC_SAMPLE[2]} cells of the same case "
                      f"(L = {u.size} DOFs), {n} SSP-RK3 steps with viscous time steps, {el:.1f} s, "
                      f"oracle (OpenMP over cells; the damping matrices are built before the clock)"}


def run_viscous(args, rank, world, local_rank):
    import torch
    import oracle.orc as orc
    from pvcriemannsolvers_gb300 import Lobatto, build, cases, mesh as meshlib
    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    p = QUAD_DEGREE
    # ---- four-quadrant demo with the viscosity
    nx, ny, nz = args.quadrant_cells
    m = cases.quadrant_mesh(nx, ny, nz)
    u0 = np.ascontiguousarray(cases.quadrant_ic(meshlib.node_coordinates(m, p).reshape(-1, 3)).ravel())
    L = u0.size
    sysm = Lobatto(m, p, "exact", device=local_rank, scheme="fr")
    cases.quadrant_bc(sysm)
    sysm.SetViscosity(VISC_BETA0, VISC_BETA1, VISC_TIME_SCALE)
    stream = torch.cuda.Stream(device=dev)
    sysm.set_stream(stream.cuda_stream)
    sysm.SetSolutionColumn(u0)
    sysm.InitialLimiter("average")
    t = sysm.advance(args.warmup, 1.0, 3, 0.0)
    torch.cuda.synchronize(dev)
    launches0 = sysm.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        with torch.cuda.stream(stream):
            e0.record(stream)
            t = sysm.advance(args.steps, 1.0, 3, t)
            e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1)
    launches = sysm.launch_count() - launches0
    sol = sysm.GetSolutionColumn()
    nu = sysm.GetViscosity()
    kt = sysm.kernel_times(reps=3)
    e2e_steps = max(1, min(args.steps, 10))
    e2e_s, seq_s = e2e_runs(torch, dev, sysm, sol, t, e2e_steps, 1.0)
    sysm.close()
    value = 3 * L * args.steps / (ms * 1e-3)
    fp64_peak = fp64_peak_tflops(torch, dev)
    # ---- the Sod demo with the viscosity, to t = 0.2
    ms_ = cases.sod_mesh()
    us0 = np.ascontiguousarray(cases.sod_ic(meshlib.node_coordinates(ms_, p).reshape(-1, 3)).ravel())
    Ls = us0.size
    sod = Lobatto(ms_, p, "exact", device=local_rank, scheme="fr")
    cases.sod_bc(sod)
    sod.SetViscosity(VISC_BETA0, VISC_BETA1, VISC_TIME_SCALE)
    sstream = torch.cuda.Stream(device=dev)
    sod.set_stream(sstream.cuda_stream)
    sod.SetSolutionColumn(us0)
    sod.InitialLimiter("majority")
    start = sod.GetSolutionColumn()
    sod.advance(args.warmup, 1.0, 3, 0.0)
    sod.SetSolutionColumn(start)
    torch.cuda.synchronize(dev)
    t_end, ts, n_sod = 0.2, 0.0, 0
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(sstream):
        s0.record(sstream)
        while ts < t_end - 1e-12:
            ts = sod.advance(10, t_end - ts if t_end - ts < 1.0 else 1.0, 3, ts)
            n_sod += 10
        s1.record(sstream)
    s1.synchronize()
    sod_s = s0.elapsed_time(s1) * 1e-3
    # oracle: parity of the first 5 steps from the same start, then a timing sample
    orc.build()
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    om = orc.Mesh(ms_, p, scheme="fr")
    om.set_bcs({0: (orc.BC_SMART, cases.SOD_LEFT), 1: (orc.BC_SMART, cases.SOD_RIGHT),
                2: (orc.BC_INVISCID_WALL, None), 3: (orc.BC_INVISCID_WALL, None),
                4: (orc.BC_INVISCID_WALL, None), 5: (orc.BC_INVISCID_WALL, None)})
    ov = orc.Viscosity(om, VISC_BETA0, VISC_BETA1, VISC_TIME_SCALE)
    u = start.copy()
    tt, n_cpu, t0 = 0.0, 0, time.perf_counter()
    parity, n0, t0_cpu = None, 0, t0
    while True:
        dt = ov.time_step(u, 1.0, 3)
        u = ov.rk_update(orc.EXACT, 3, tt, dt, u)
        tt += dt
        n_cpu += 1
        if n_cpu == 5:
            sod.SetSolutionColumn(start)
            sod.advance(5, 1.0, 3, 0.0)
            g = sod.GetSolutionColumn()
            parity = float(np.linalg.norm(g - u) / np.linalg.norm(u))
            t0_cpu, n0 = time.perf_counter(), n_cpu
        if n_cpu >= 5 and (time.perf_counter() - t0 >= 12.0 or n_cpu >= n_sod):
            break
    cpu_sod_s = time.perf_counter() - t0_cpu
    sod.close()
    cpu = None
    if not args.no_cpu:
        cpu = viscous_cpu_sample()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"four-quadrant Riemann problem with energy-based artificial viscosity, "
                               f"{nx}x{ny}x{nz} Hex8, fr::Lobatto p={p} (Huynh g2), Exact Riemann solver, "
                               f"DDG beta0 = {VISC_BETA0}, beta1 = {VISC_BETA1}, time scale {VISC_TIME_SCALE}, "
                               f"average initial limiter, SSP-RK3 with the viscous time step",
                   "cells": m.n_cells, "dofs": L, "form": "plain FP64",
                   "step": "viscosity properties + viscous dt + 3 x (properties + face flux + cell update)",
                   "l2_flush": "inputs larger than L2 (solution column 1.13 GB)"},
        "accuracy": {"t_end": t, "cells_with_viscosity": int((nu.max(axis=1) > 0).sum()),
                     "max_viscosity": float(nu.max())},
        "clocks": clocks.summary(),
        "e2e": {"value": 3 * L * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 8 * L,
                "d2h_bytes_per_step": 8 * L, "steps": e2e_steps, "path": E2E_PATH,
                "sequential": {"value": 3 * L * e2e_steps / seq_s, "path": E2E_SEQ_PATH}},
        "gpu_launches": launches,
        "sod": {"workload": "Sod shock tube 100x4x4 Hex8, fr::Lobatto p=2, Exact, the same viscosity, majority "
                            "initial limiter, t = 0 -> 0.2",
                "steps": n_sod, "t_end": ts, "gpu_s": sod_s, "value": 3 * Ls * n_sod / sod_s,
                "cpu_oracle_extrapolated_s": n_sod * (cpu_sod_s / max(n_cpu - n0, 1)),
                "cpu_sample": f"steps 6..{n_cpu}, {cpu_sod_s:.1f} s, {threads} threads",
                "gpu_vs_oracle_rel_l2_after_5_steps": parity},
        "roofline": {"bound": "fp64", "kernel": "step", "kernel_ms": kt, "peak": fp64_peak, "unit": "TFLOP/s",
                     "achieved": None, "frac": None, "traffic": None,
                     "peak_source": "measured in this run: cuBLAS DGEMM 4096^3",
                     "note": "face_flux includes the viscosity properties pass of the stage"},
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Output and restart on the headline mesh (64^3 Hex8, DGSEM p = 3, 83.9 M
# values): the DataOnCells field transposition (Part::GatherSolutions /
# ScatterSolutions) against HBM, the VTK sampling (Writer::Prepare) and the
# restart file round trip through the C ABI.

def run_output(args, rank, world, local_rank):
    import torch
    from pvcriemannsolvers_gb300 import Lobatto, build, cases, mesh as meshlib
    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    m = meshlib.box((args.cells,) * 3, lengths=(10.0,) * 3, periodic=(True,) * 3)
    u0 = np.ascontiguousarray(cases.vortex_ic(meshlib.node_coordinates(m, DEGREE).reshape(-1, 3)).ravel())
    L = u0.size
    sysm = Lobatto(m, DEGREE, "rusanov", cfl=CFL, device=local_rank)
    stream = torch.cuda.Stream(device=dev)
    sysm.set_stream(stream.cuda_stream)
    sysm.SetSolutionColumn(u0)
    fields = torch.empty(L, dtype=torch.float64, device=dev)
    launches0 = sysm.launch_count()
    times = {}
    with ClockSampler(local_rank) as clocks:
        for name, fn in (("gather", sysm.gather_fields_device), ("scatter", sysm.scatter_fields_device)):
            for _ in range(args.warmup):
                fn(fields.data_ptr(), L)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                fn(fields.data_ptr(), L)
            e1.record(stream)
            e1.synchronize()
            times[name] = e0.elapsed_time(e1) / args.steps
    launches = sysm.launch_count() - launches0
    ok = bool(np.array_equal(sysm.GetSolutionColumn(), u0))
    t0 = time.perf_counter()
    xyz, values, types = sysm.vtk_sample()
    sample_s = time.perf_counter() - t0
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "state.rst")
        t0 = time.perf_counter()
        sysm.write_restart(path, 0.0)
        write_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        sysm.read_restart(path)
        read_s = time.perf_counter() - t0
    ok = ok and bool(np.array_equal(sysm.GetSolutionColumn(), u0))
    sysm.close()
    hbm_peak, peak_src = measured_peaks()
    gbs = 16.0 * L / (times["gather"] * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu:
        t0 = time.perf_counter()
        reps = 0
        while time.perf_counter() - t0 < 5.0:
            np.ascontiguousarray(u0.reshape(m.n_cells, -1).T)
            reps += 1
        el = time.perf_counter() - t0
        cpu = {"value": 16.0 * L * reps / el / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
               "sample": f"numpy transpose of the same column, {reps} reps, {el:.1f} s"}
    line = {
        "metric": "DataOnCells field gather (column -> fields) bandwidth", "value": gbs, "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": times["gather"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"output of the vortex {args.cells}^3 Hex8 DGSEM p={DEGREE} column",
                   "values": L, "cells": m.n_cells, "l2_flush": f"inputs larger than L2 ({8 * L / 1e9:.2f} GB)"},
        "clocks": clocks.summary(), "gpu_launches": launches, "round_trip_bit_exact": ok,
        "scatter_ms": times["scatter"], "scatter_gbs": 16.0 * L / (times["scatter"] * 1e-3) / 1e9,
        "roofline": {"bound": "hbm", "kernel": "fields_transpose_kernel<true>", "achieved": gbs,
                     "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak, "traffic": None,
                     "peak_source": peak_src, "algorithmic_bytes": 16 * L},
        "e2e": {"vtk_sample_s": sample_s, "vtk_points": len(xyz),
                "restart_write_s": write_s, "restart_read_s": read_s,
                "restart_write_gbs": 8 * L / write_s / 1e9, "restart_read_gbs": 8 * L / read_s / 1e9,
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Cell numbering: the headline step (mixed form) on the box's lexicographic
# numbering, on a random renumbering (seed 0) and on the Hilbert order of the
# random one (mesh.renumber_cells / mcfd_hilbert_order).

def run_reorder(args, rank, world, local_rank):
    import torch
    from pvcriemannsolvers_gb300 import Lobatto, build, cases, mesh as meshlib
    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    m = meshlib.box((args.cells,) * 3, lengths=(10.0,) * 3, periodic=(True,) * 3)
    u0 = np.ascontiguousarray(cases.vortex_ic(meshlib.node_coordinates(m, DEGREE).reshape(-1, 3)).ravel())
    L = u0.size
    rng = np.random.default_rng(0)
    shuffle = rng.permutation(m.n_cells)
    shuffled = meshlib.renumber_cells(m, shuffle)
    t0 = time.perf_counter()
    hil = meshlib.hilbert_order(shuffled)
    order_s = time.perf_counter() - t0
    variants = {"lexicographic": (m, np.arange(m.n_cells)), "random": (shuffled, shuffle),
                "hilbert_of_random": (meshlib.renumber_cells(shuffled, hil), shuffle[hil])}
    res = {}
    sols = {}
    for name, (mm, order) in variants.items():
        sysm = Lobatto(mm, DEGREE, "rusanov", cfl=CFL, device=local_rank, precision="mixed")
        stream = torch.cuda.Stream(device=dev)
        sysm.set_stream(stream.cuda_stream)
        sysm.SetSolutionColumn(np.ascontiguousarray(u0.reshape(m.n_cells, -1)[order].ravel()))
        sysm.autotune()
        t = sysm.advance(args.warmup, 1e9, 3, 0.0)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local_rank) as clocks:
            with torch.cuda.stream(stream):
                e0.record(stream)
                t = sysm.advance(args.steps, 1e9, 3, t)
                e1.record(stream)
            e1.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        back = np.empty_like(u0.reshape(m.n_cells, -1))
        back[order] = sysm.GetSolutionColumn().reshape(m.n_cells, -1)
        sols[name] = back.ravel()
        res[name] = {"ms_per_step": ms, "value": 3 * L / (ms * 1e-3), "kernel_ms": sysm.kernel_times(reps=3),
                     "clocks": clocks.summary()}
        sysm.close()
    ref = sols["lexicographic"]
    agree = {k: float(np.linalg.norm(v - ref) / np.linalg.norm(ref)) for k, v in sols.items()}
    # mesh ingest: the faces of the same mesh from its cells and boundary
    # elements, host builder against GPU builder (the same faces)
    open_mesh = meshlib.box((args.cells,) * 3, lengths=(10.0,) * 3)
    bn, bg = meshlib.boundary_elements(open_mesh)
    spec = [(2 * ax, 2 * ax + 1, tuple(-10.0 if e == ax else 0.0 for e in range(3))) for ax in range(3)]
    ingest = {}
    built = {}
    for name, device in (("host", None), ("gpu", local_rank)):
        times = []
        for _ in range(3):
            t0 = time.perf_counter()
            built[name] = meshlib.build(open_mesh.xyz, open_mesh.cell_nodes, None, bn, bg, spec, device=device)
            times.append(time.perf_counter() - t0)
        ingest[name + "_s"] = sorted(times)[1]
    ingest["same_faces"] = bool(all(np.array_equal(getattr(built["host"], f), getattr(built["gpu"], f))
                                    for f in ("face_cells", "face_sides", "face_group", "face_shift")))
    ingest["faces"] = built["gpu"].n_faces
    r = res["hilbert_of_random"]
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
        "config": {"workload": f"vortex {args.cells}^3 Hex8 DGSEM p={DEGREE} mixed, cells renumbered",
                   "numbering": "Hilbert order (mcfd_hilbert_order) of a random renumbering",
                   "l2_flush": f"inputs larger than L2 ({8 * L / 1e9:.2f} GB)"},
        "clocks": r["clocks"], "hilbert_order_s": order_s, "face_builder": ingest,
        "variants": res, "solution_rel_l2_vs_lexicographic": agree,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--cells", type=int, default=N_CELLS_1D, help="cells per direction (profiling runs a smaller case)")
    ap.add_argument("--form", default="both", choices=["both", "fp64", "mixed"],
                    help="precision form(s) to time; the line's value is the mixed form when timed")
    ap.add_argument("--contraction", default="both", choices=["both", "simt", "tensor"],
                    help="the mixed form's differentiation: FP32 SIMT, tensor cores (TF32x3), or both "
                         "(SIMT for the line's value, the tensor path timed beside it)")
    ap.add_argument("--workload", default="vortex",
                    choices=["vortex", "mixed_box", "all_types", "curved_types", "ensemble", "quadrant", "output",
                             "reorder", "sod", "viscous"],
                    help="vortex: the headline DGSEM case; mixed_box: modal DG on hex + tet blocks; "
                         "ensemble: 64 independent cases in one graph per step; output: field "
                         "gather/scatter, VTK sampling and restart on the headline column; viscous: fr::Lobatto "
                         "with the energy-based artificial viscosity (four-quadrant and Sod demos); all_types: "
                         "modal DG on Hex8, Tet4, Wedge6 and Pyra5 blocks; curved_types: the same blocks as "
                         "deformed Hex27, Tet10, Wedge18 and Pyra14 cells")
    ap.add_argument("--quadrant-cells", type=int, nargs=3, default=[256, 256, 16], metavar=("NX", "NY", "NZ"),
                    help="mesh of the four-quadrant workload")
    ap.add_argument("--ensemble-scale", type=float, default=1.0,
                    help="scale of the ensemble's element counts (profiling runs a smaller case)")
    ap.add_argument("--mixed-cells", type=int, nargs=2, default=[MIXED_HEX_1D, MIXED_TET_1D],
                    metavar=("HEX_1D", "TET_1D"), help="block sizes of the mixed box")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload in ("mixed_box", "all_types", "curved_types"):
        run_mixed_box(args, rank, world, local_rank, args.workload)
        return
    if args.workload == "ensemble":
        run_ensemble(args, rank, world, local_rank)
        return
    if args.workload == "quadrant":
        run_quadrant(args, rank, world, local_rank)
        return
    if args.workload == "output":
        run_output(args, rank, world, local_rank)
        return
    if args.workload == "reorder":
        run_reorder(args, rank, world, local_rank)
        return
    if args.workload == "sod":
        run_sod(args, rank, world, local_rank)
        return
    if args.workload == "viscous":
        run_viscous(args, rank, world, local_rank)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    run_gpu(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
