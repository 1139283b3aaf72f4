"""Throughput benchmark: D3Q19 channel 256x128x128 (inflow u_x = 0.04, pressure outflow rho = 1,
no-slip walls, solid sphere r = 16 at (64, 64, 64), omega = 1.8), populations stored as FP32
(the headline) and FP16 (shifted by w_q), one fused step kernel per time step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line. `value` is MLUPS over interior cells (xl*yl*zl*K / seconds) with the state
resident in HBM, timed with CUDA events on the library's stream; `e2e` is the same metric through
the C ABI over the workload's full 5000-step run, with the initial state uploaded from pinned host
memory, every step's FP64 mass and momentum copied to pinned host memory and the density and
velocity of every cell read back, all inside the timed region. The line carries one summary per
further workload (FP16 / FP64 storage, D3Q15 / D3Q27, errors against FP64, adjoint, Taylor-Green,
512^3 cavity); their full records go to gpurun_out/bench_detail.json. With --impl reference the
CPU solver of the reference (the C restatement under oracle/, or the reference's own build where
it exists) is timed on the host cores on the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
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

METRIC = "D3Q19 MLUPS & % HBM roofline, FP16-store vs FP32 at stated FP64 error"
WORKLOAD = "channel 256x128x128, sphere r16 at (64,64,64), u_in 0.04, omega 1.8"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", default="256,128,128")
    ap.add_argument("--quick", action="store_true", help="headline only (no stencil sweep / e2e / cpu)")
    ap.add_argument("--extra-only", action="store_true",
                    help="only the Taylor-Green, 512^3 cavity and cavity-adjoint workloads")
    ap.add_argument("--profile", choices=["fp64", "fp32", "fp16", "bf16", "adjoint"],
                    help="only step the headline workload (warmup + steps) in this storage, or run a "
                         "gradient of the adjoint channel (128x64x64, FP32, warmup + steps forward steps, "
                         "checkpoint every 10), with no timing and no JSON line: the command the "
                         "profiler runs")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(q: int, size):
    from lbm_gb300 import scenario as S
    xl, yl, zl = size
    return S.channel(xl, yl, zl, q=q, u_in=0.04, omega=1.8,
                     sphere=((xl // 4, yl // 2, zl // 2), max(1, yl // 8)))


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel_tag: str):
    """DRAM bytes per launch of the step kernel from the committed ncu summary, or None."""
    f = ROOT / "profiles" / "traffic.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel_tag:
            return float(parts[1])
    return None


class ClockSampler:
    """nvidia-smi clocks, utilisation and throttle reasons, sampled every 100 ms while running;
    the summary keeps the samples taken while the GPU was busy (utilisation >= 50 %)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, window: str = ""):
        sm, mx, reasons, total = [], [], set(), 0
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                clk, cmax, util = float(parts[1]), float(parts[2]), float(parts[9])
            except ValueError:
                continue
            total += 1
            if util < 50:
                continue
            sm.append(clk)
            mx.append(cmax)
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
               "reasons": sorted(reasons), "samples": total, "samples_under_load": len(sm)}
        if window:
            out["window"] = window
        return out


def time_steps(dom, steps: int, warmup: int):
    """Warm up, then time `steps` single-step launches with CUDA events on the library's stream.
    Returns seconds."""
    import torch
    dom.step(warmup)
    dom.sync()
    stream = torch.cuda.ExternalStream(dom.stream_handle())
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        dom.step(1)
    end.record(stream)
    end.synchronize()
    return start.elapsed_time(end) / 1e3


def sig(x, n: int = 4):
    """x rounded to n significant digits (numbers in nested dicts / lists too): keeps the line short."""
    if isinstance(x, float):
        return float(f"{x:.{n}g}")
    if isinstance(x, dict):
        return {k: sig(v, n) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [sig(v, n) for v in x]
    return x


def soak(dom, seconds: float):
    """Plain steps for about `seconds` (untimed): gives the clock sampler samples of this kernel
    under load, which a 20-step timed region (2 ms) is too short for."""
    dom.step(50)
    dom.sync()
    t0 = time.perf_counter()
    dom.step(50)
    dom.sync()
    per = max((time.perf_counter() - t0) / 50, 1e-6)
    dom.step(int(seconds / per))
    dom.sync()


DETAIL = ROOT / "gpurun_out" / "bench_detail.json"


def replica_barrier(world: int) -> None:
    """All ranks of the replica run meet here (no-op on one GPU)."""
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def replica_max(x: float, world: int) -> float:
    """The largest x over the ranks (the slowest replica's time): one all-reduce on the process
    group's device (CUDA for NCCL, the host for gloo)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_mlups(cells_per_rank: int, steps: int, seconds_max: float, world: int) -> float:
    """Whole-job MLUPS of `world` replicas, each updating cells_per_rank cells `steps` times, over
    the slowest rank's time (weak scaling: the work per GPU is fixed)."""
    return world * cells_per_rank * steps / seconds_max / 1e6


def run_ours(args, rank, world, local):
    import torch
    import torch.distributed as dist

    from lbm_gb300 import build_domain
    torch.cuda.set_device(local)
    size = tuple(int(v) for v in args.size.split(","))
    K, W = args.steps, args.warmup
    peak, peak_kind = measured_peak()

    def barrier():
        replica_barrier(world)
        torch.cuda.synchronize()

    def max_over_ranks(x: float) -> float:
        return replica_max(x, world)

    scn19 = workload(19, size)
    ncell = scn19.ninterior
    detail = {}

    def timed(prec, q=19):
        d = build_domain(scn19 if q == 19 else workload(q, size), prec)
        info = d.memory_info()
        barrier()
        sec = max_over_ranks(time_steps(d, K, W))
        return d, info, sec

    with ClockSampler(local) as clk:
        # headline: D3Q19 FP32; the sampler runs through its warm-up, the timed steps and a 1 s
        # run of the same step right after
        dom, info, sec = timed("fp32")
        soak(dom, 1.0)
        dom.close()
    clocks = clk.summary("headline warm-up, its timed steps and 1 s of the same step right after "
                         "(the timed steps alone last less than one 100 ms sampling period)")
    # FP16 and FP64 storage, same workload
    dom, info16, sec16 = timed("fp16")
    dom.close()
    dom, info64, sec64 = timed("fp64")
    dom.close()

    def mlups(sec_):
        return replica_mlups(ncell, K, sec_, world)

    def frac(info_, sec_):
        return info_["step_bytes"] / (sec_ / K) / 1e9 / peak

    ms = sec / K * 1e3
    achieved = info["step_bytes"] / (sec / K) / 1e9
    line = {
        "metric": METRIC, "value": mlups(sec), "unit": "MLUPS", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "lattice": "D3Q19", "size": list(size), "storage": "fp32 (f - w)",
                   "fluid_cells": info["fluid_cells"], "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (%.0f MB populations per step > 129 MB)" % (info["step_bytes"] / 2e6)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": ncu_traffic("step_kernel_d3q19_fp32"),
                     "algorithmic_bytes_per_launch": info["step_bytes"]},
        "gpu_launches": K * info["launches_per_step"],
        "clocks": clocks,
        "fp16": {"value": mlups(sec16), "speedup_vs_fp32": sec / sec16, "frac": frac(info16, sec16)},
        "fp64": {"value": mlups(sec64), "frac": frac(info64, sec64)},
    }
    if not args.quick:
        # error statement: FP32 / FP16 / BF16 storage against the FP64 run of the same workload
        n_err = 1000
        us = {}
        for prec in ("fp64", "fp32", "fp16", "bf16"):
            with build_domain(scn19, prec) as d:
                d.step(n_err)
                us[prec] = d.moments()[1]
        fl = scn19.fluid_mask_interior()

        def err(u):
            return float(np.linalg.norm(u[fl] - us["fp64"][fl]) / np.linalg.norm(us["fp64"][fl]))
        line["u_rel_l2_vs_fp64"] = {"fp32": err(us["fp32"]), "fp16": err(us["fp16"]), "bf16": err(us["bf16"]),
                                    "steps": n_err}
        del us
        # other stencils, FP32
        sten = {}
        for q in (15, 27):
            d, mi, s_ = timed("fp32", q)
            d.close()
            sten[f"D3Q{q}"] = {"mlups": mlups(s_), "frac": frac(mi, s_)}
        line["stencils_fp32"] = sten
        adj = detail["adjoint"] = run_adjoint()
        tg = detail["taylor_green"] = run_taylor_green()
        cav = detail["cavity512_d3q27"] = run_large_cavity()
        cadj = detail["cavity256_adjoint"] = run_cavity_adjoint()
        line["adjoint"] = {
            "channel128_fp32": {"bwd_over_fwd_per_step": adj["backward_over_forward"],
                                "call_over_fwd": adj["backward_call_over_forward"],
                                "fd_rel_err": adj["fd_check"]["max_rel_err_fp32_adjoint"],
                                "records_resident": {
                                    "bwd_over_fwd_per_step": adj["records_resident"]["backward_over_forward"],
                                    "call_over_fwd": adj["records_resident"]["backward_call_over_forward"]}},
            "cavity256_d3q27_fp16": {"bwd_over_fwd_per_step": cadj["backward_over_forward"],
                                     "call_over_fwd": cadj["backward_call_over_forward"],
                                     "fd_rel_err": cadj["fd_check"]["rel_err"]}}
        line["taylor_green384"] = {"mlups": {p_: tg[p_]["mlups"] for p_ in ("fp64", "fp32", "fp16", "bf16")},
                                   "u_rel_l2_vs_fp64": {p_: tg[p_]["u_rel_l2_vs_fp64"] for p_ in ("fp32", "fp16", "bf16")},
                                   "ke_decay_ratio_fp64": tg["fp64"]["ke_linear_decay_ratio"]}
        line["cavity512_d3q27"] = {p_: {"mlups": cav[p_]["mlups"], "frac": cav[p_]["hbm_frac"]} for p_ in ("fp16", "fp32")}
        line["e2e"] = run_e2e(scn19, W)
        if rank == 0:
            line["cpu_baseline"] = cpu_baseline(size, budget_s=12.0)
    if rank == 0 and detail:
        try:
            DETAIL.parent.mkdir(exist_ok=True)
            DETAIL.write_text(json.dumps(detail, indent=1))
            line["details"] = str(DETAIL.relative_to(ROOT))
        except OSError:
            pass
    return sig(line) if rank == 0 else None


def run_adjoint(xl=128, yl=64, zl=64, steps=2000, ckpt=100):
    """Gradient workload: D3Q19 channel 128x64x64, per-cell inlet profile u_x ~ U[0.02, 0.05] and 5 %
    random solids from seed 0, omega 1.7, 2000 steps, checkpoints every 100 steps, objective = kinetic
    energy in x in [96, 128) (interior cells 97..128). FP32 forward + adjoint, with checkpoints and
    recompute and with every step's record kept (ckpt_every = 1); plain FP32 steps timed beside it;
    the FP32 and FP64 adjoint gradients at three inlet cells against FP64 central finite
    differences (h = 1e-5)."""
    from lbm_gb300 import build_domain
    from lbm_gb300 import scenario as S
    scn = S.adjoint_channel(xl, yl, zl, omega=1.7, seed=0)
    box = (97, xl, 1, yl, 1, zl)
    with build_domain(scn, "fp32") as d:
        plain = time_steps(d, steps, 5)
    cost, (J32, (g32, _)) = _adjoint_costs(scn, "fp32", steps, ckpt, box)
    # a checkpoint every step: the forward keeps every step's record (4 values per cell and step,
    # 22 GB here) and the backward recomputes nothing
    cost_res, (_, (g32_res, _)) = _adjoint_costs(scn, "fp32", steps, 1, box)
    with build_domain(scn, "fp64") as d:
        d.adjoint_forward(steps, ckpt)
        J64 = d.objective_ke(box)
        g64, _ = d.adjoint_backward(box)
    h = 1e-5
    cells = [(32, 32), (10, 50), (60, 5)]
    errs32, errs64, fds = [], [], []
    for (y, z) in cells:
        k = (z * (yl + 2) + y) * (xl + 2)
        vals = []
        for sgn in (1, -1):
            s2 = S.adjoint_channel(xl, yl, zl, omega=1.7, seed=0)
            s2.boundaries[0].profile = s2.boundaries[0].profile.copy()
            s2.boundaries[0].profile[k, 0] += sgn * h
            with build_domain(s2, "fp64") as d:
                d.step(steps)
                vals.append(d.objective_ke(box))
        fd = (vals[0] - vals[1]) / (2 * h)
        fds.append(fd)
        errs32.append(abs(g32[k, 0] - fd) / abs(fd))
        errs64.append(abs(g64[k, 0] - fd) / abs(fd))
    n = scn.ninterior
    return {
        "workload": f"adjoint channel D3Q19 {xl}x{yl}x{zl}, inlet profile + 5% solids from seed 0, omega 1.7, "
                    f"{steps} steps, checkpoint every {ckpt}, J = KE in x in [96,{xl})",
        "storage": "fp32 (f - w)", "steps": steps, "ckpt_every": ckpt,
        "forward_plain_ms_per_step": plain / steps * 1e3,
        **_adjoint_report(cost, plain / steps),
        "records_resident": {**_adjoint_report(cost_res, plain / steps),
                             "grad_rel_l2_vs_ckpt": _rel_l2(g32_res, g32)},
        "forward_mlups": n * steps / plain / 1e6,
        "J_fp32": J32, "J_fp64": J64,
        "fd_check": {"param": "inlet u_x at (y, z)", "cells": cells, "fd_fp64": fds,
                     "max_rel_err_fp32_adjoint": max(errs32), "max_rel_err_fp64_adjoint": max(errs64),
                     "h": h},
    }


def _adjoint_costs(scn, prec, steps, ckpt, box):
    """Wall-clock seconds of adjoint_forward(n, ckpt) and of adjoint_backward (the faster of two
    calls) on fresh domains, for n = steps and n = steps // 2; and (J, gradients) of the full run.
    The difference of the two lengths is the cost per step without the costs of a call (allocations,
    the gradient download and its scaling on the host), which plain steps timed by CUDA events do
    not carry either."""
    import torch
    from lbm_gb300 import build_domain

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0, r

    out, first = {}, None
    for n in (steps, steps // 2):
        with build_domain(scn, prec) as d:
            d.step(0)
            d.sync()
            fwd, _ = timed(lambda: (d.adjoint_forward(n, ckpt), d.sync()))
            J = d.objective_ke(box)
            bwd, grads = timed(lambda: d.adjoint_backward(box))
            bwd2, _ = timed(lambda: d.adjoint_backward(box))
        out[n] = (fwd, min(bwd, bwd2))
        if first is None:
            first = (J, grads)
    return {"steps": steps, "half": steps // 2, "t": out}, first


def _adjoint_report(cost, plain_step):
    n, h = cost["steps"], cost["half"]
    (fwd, bwd), (fwd_h, bwd_h) = cost["t"][n], cost["t"][h]
    fwd_step = (fwd - fwd_h) / (n - h)
    bwd_step = (bwd - bwd_h) / (n - h)
    return {
        "forward_ckpt_ms_per_step": fwd_step * 1e3,
        "backward_ms_per_step": bwd_step * 1e3,
        "backward_over_forward": bwd_step / plain_step,
        "forward_plus_backward_over_forward": (fwd_step + bwd_step) / plain_step,
        "backward_call_ms": bwd * 1e3,
        "backward_call_over_forward": bwd / (n * plain_step),
        "backward_fixed_ms_per_call": (bwd - bwd_step * n) * 1e3,
        "timing": f"wall clock around synchronised calls; per step = difference of {n}- and {h}-step "
                  f"runs over {n - h} steps (a call's allocations, gradient download and host-side "
                  f"scaling cancel); backward_call_* = the whole {n}-step call; plain steps by CUDA events",
    }


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run_taylor_green(n=384, u0=0.03, omega=1.9, steps=2000):
    """Decaying Taylor-Green vortex, D3Q19 periodic n^3, f = feq(1, u_TG) at start: FP32 / BF16 /
    FP16 shifted storage against the FP64 GPU run of the same steps (relative L2 of u and of
    rho - 1), and the kinetic energy against the linear decay E0 exp(-6 nu k^2 t),
    nu = cs^2 (tau - 1/2), k = 2 pi / n (a low-Reynolds guide: Re = u0 / (nu k) here)."""
    from lbm_gb300 import build_domain
    from lbm_gb300 import scenario as S
    scn = S.taylor_green(n, u0, omega)
    out = {"workload": f"Taylor-Green D3Q19 {n}^3 periodic, u0 {u0}, omega {omega}, {steps} steps", "steps": steps}
    ref = None
    nu = (1.0 / omega - 0.5) / 3.0
    k = 2 * np.pi / n
    u_init = S.taylor_green_velocity(n, u0)
    ke0 = 0.5 * float((u_init ** 2).sum())
    del u_init
    for prec in ("fp64", "fp32", "bf16", "fp16"):
        with build_domain(scn, prec) as d:
            sec = time_steps(d, steps, 0)
            rho, u = d.moments()
        ke = 0.5 * float((rho * (u ** 2).sum(axis=-1)).sum())
        r = {"mlups": n ** 3 * steps / sec / 1e6, "ke_over_ke0": ke / ke0}
        if ref is None:
            ref = (rho, u)
            r["ke_linear_decay_ratio"] = ke / (ke0 * np.exp(-6 * nu * k * k * steps))
        else:
            r["u_rel_l2_vs_fp64"] = _rel_l2(u, ref[1])
            r["rho_rel_l2_vs_fp64"] = _rel_l2(rho - 1.0, ref[0] - 1.0)
        out[prec] = r
        del rho, u
    out["reynolds"] = u0 / (nu * k)
    return out


def run_large_cavity(n=512, q=27, omega=1.95, lid=0.1, steps=500, n_acc=128, omega_acc=1.8):
    """D3Q27 lid-driven cavity n^3 with FP16 shifted storage (AA in place) and, beside it, FP32:
    `steps` steps timed. At omega 1.95 (tau 0.513) and lid 0.1 the BGK cavity diverges within
    these steps in every precision, FP64 included (the reference's scheme, reproduced bit for bit
    in FP64, behaves the same), so the velocity errors are stated on an n_acc^3 cavity at
    omega_acc, where the same 500 steps stay stable: FP16 / BF16 / FP32 against FP64."""
    from lbm_gb300 import build_domain
    from lbm_gb300 import scenario as S
    peak, _ = measured_peak()
    out = {"workload": f"cavity D3Q{q} {n}^3, lid {lid}, omega {omega}, {steps} steps", "cells": n ** 3}
    for prec in ("fp16", "fp32"):
        with build_domain(S.cavity(n, q=q, lid=lid, tau=1.0 / omega), prec) as d:
            info = d.memory_info()
            sec = time_steps(d, steps, 0)
            rho, _ = d.moments()
        fin = np.isfinite(rho)
        out[prec] = {"mlups": n ** 3 * steps / sec / 1e6, "ms_per_step": sec / steps * 1e3,
                     "hbm_frac": info["step_bytes"] / (sec / steps) / 1e9 / peak,
                     "device_bytes": info["device_bytes"],
                     "final_rho_range": [float(rho[fin].min()), float(rho[fin].max())] if fin.any() else None,
                     "non_finite_cells": int((~fin).sum())}
        del rho
    acc = {"workload": f"cavity D3Q{q} {n_acc}^3, lid {lid}, omega {omega_acc}, {steps} steps"}
    us = {}
    for prec in ("fp64", "fp32", "fp16", "bf16"):
        with build_domain(S.cavity(n_acc, q=q, lid=lid, tau=1.0 / omega_acc), prec) as d:
            d.step(steps)
            rho, us[prec] = d.moments()
        if prec == "fp64":
            acc["fp64_rho_range"] = [float(rho.min()), float(rho.max())]
    for prec in ("fp32", "fp16", "bf16"):
        acc[f"u_rel_l2_{prec}_vs_fp64"] = _rel_l2(us[prec], us["fp64"])
    out["accuracy"] = acc
    return out


def run_cavity_adjoint(n=256, q=27, omega=1.8, lid=0.1, steps=500, ckpt=50, n_fd=128):
    """Gradient of the cavity's kinetic energy after `steps` steps with respect to the lid
    velocity, FP16 storage (FP32 adjoint arithmetic), checkpoints every `ckpt` steps, timed
    against plain FP16 steps on n^3. omega 1.8: at 1.95 the forward run itself diverges. dJ/du_x is
    checked on an n_fd^3 cavity against FP64 central differences (h = 1e-6)."""
    from lbm_gb300 import build_domain
    from lbm_gb300 import scenario as S

    def make(m, v):
        return S.cavity(m, q=q, lid=v, tau=1.0 / omega)
    box = (1, n, 1, n, 1, n)
    with build_domain(make(n, lid), "fp16") as d:
        plain = time_steps(d, steps, 0)
    cost, (_, (_, gw)) = _adjoint_costs(make(n, lid), "fp16", steps, ckpt, box)
    fbox = (1, n_fd, 1, n_fd, 1, n_fd)
    with build_domain(make(n_fd, lid), "fp16") as d:
        d.adjoint_forward(steps, ckpt)
        _, gw_fd = d.adjoint_backward(fbox)
    h = 1e-6
    vals = []
    for sgn in (1, -1):
        with build_domain(make(n_fd, lid + sgn * h), "fp64") as d:
            d.step(steps)
            vals.append(d.objective_ke(fbox))
    fd = (vals[0] - vals[1]) / (2 * h)
    return {"workload": f"cavity D3Q{q} {n}^3 adjoint wrt lid velocity, lid {lid}, omega {omega}, {steps} steps, "
                        f"checkpoint every {ckpt}, J = KE of the whole cavity",
            "storage": "fp16 (f - w), adjoint in fp32",
            "forward_plain_ms_per_step": plain / steps * 1e3,
            **_adjoint_report(cost, plain / steps),
            "dJ_du_lid": [float(x) for x in gw[1]],
            "fd_check": {"cells": n_fd ** 3, "fd_fp64_dJ_du_x": fd, "adjoint_fp16_dJ_du_x": float(gw_fd[1][0]),
                         "rel_err": abs(gw_fd[1][0] - fd) / abs(fd)}}


def run_e2e(scn, W, steps: int = 5000):
    """The same metric through the C ABI with host buffers, over the workload's full run (5000
    steps): the initial state uploaded from pinned host memory (lbm_set_populations), the steps
    through lbm_step_monitored, which copies every step's FP64 mass and momentum (32 bytes) to
    pinned host memory, and the density and velocity of every interior cell read back into pinned
    memory (lbm_moments); all inside the timed region. One untimed call of each before it, as a
    user's first call, allocates the handle's staging buffers."""
    import torch

    from lbm_gb300 import build_domain
    dom = build_domain(scn, "fp32")
    f0 = torch.empty((scn.ncells, scn.q), dtype=torch.float64).pin_memory()
    f0.numpy()[:] = np.tile(scn.model.weights, (scn.ncells, 1))
    totals = torch.empty((steps, 4), dtype=torch.float64).pin_memory()
    rho = torch.empty(scn.ninterior, dtype=torch.float64).pin_memory()
    u = torch.empty(3 * scn.ninterior, dtype=torch.float64).pin_memory()
    lib = dom._lib
    P = ctypes.c_void_p
    rc = lib.lbm_set_populations(dom._h, P(f0.data_ptr()))
    dom.step(W)
    rc |= lib.lbm_moments(dom._h, P(rho.data_ptr()), P(u.data_ptr()))
    t0 = time.perf_counter()
    rc |= lib.lbm_set_populations(dom._h, P(f0.data_ptr()))
    rc |= lib.lbm_step_monitored(dom._h, steps, P(totals.data_ptr()))
    rc |= lib.lbm_moments(dom._h, P(rho.data_ptr()), P(u.data_ptr()))
    t1 = time.perf_counter()
    mass = totals.numpy()[:, 0]
    dom.close()
    if rc:
        raise RuntimeError("e2e run failed")
    h2d = scn.ncells * scn.q * 8
    d2h = 32 * steps + 32 * scn.ninterior
    return {"value": scn.ninterior * steps / (t1 - t0) / 1e6, "unit": "MLUPS", "h2d_bytes_per_step": h2d / steps,
            "d2h_bytes_per_step": d2h / steps, "steps": steps, "seconds": t1 - t0,
            "mass_drift": float(abs(mass[-1] - mass[0]) / mass[0])}


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_run(size, steps: int, threads: int, kind: str):
    import oracle
    scn = workload(19, size)
    if kind == "reference":
        r = oracle.run_ref(scn, steps, threads=threads, fast=True, want_pops=False)
        return r["seconds"]
    c = oracle.Checker(scn)
    sec = c.step(steps, threads)
    c.close()
    return sec


def cpu_kind() -> str:
    import oracle
    return "reference" if oracle.checkers.REF_LIB_FAST.exists() else "port"


def cpu_baseline(size, budget_s: float):
    """The reference CPU solver on all host cores, on a bounded number of steps of the same
    workload (about `budget_s` seconds)."""
    import oracle
    oracle.build(with_ref=False) if not oracle.port_available() else None
    threads = cpu_threads()
    kind = cpu_kind()
    probe = cpu_run(size, 2, threads, kind) / 2
    steps = int(max(2, min(200, budget_s / max(probe, 1e-6))))
    sec = cpu_run(size, steps, threads, kind)
    ncell = size[0] * size[1] * size[2]
    return {"value": ncell * steps / sec / 1e6, "unit": "MLUPS", "cores": threads, "kind": kind,
            "sample": f"{steps} steps of the full {size[0]}x{size[1]}x{size[2]} D3Q19 channel (FP64, "
                      f"reference algorithm: AoS pull-stream + two-phase collide, OpenMP)"}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    size = tuple(int(v) for v in args.size.split(","))
    import oracle
    if not oracle.port_available():
        oracle.build(with_ref=False)
    threads = cpu_threads()
    kind = cpu_kind()
    ncell = size[0] * size[1] * size[2]
    probe = cpu_run(size, 1, threads, kind)
    K, W = args.steps, args.warmup
    # bound the run to about two minutes: each timed step is one full step of the workload
    k_run = int(max(1, min(K, 100.0 / max(probe, 1e-6))))
    w_run = int(max(0, min(W, 20.0 / max(probe, 1e-6))))
    if w_run:
        cpu_run(size, w_run, threads, kind)
    sec = cpu_run(size, k_run, threads, kind)
    mlups = ncell * k_run / sec / 1e6
    sample = (f"{k_run} timed steps (of {K} requested) after {w_run} warm-up steps of the full "
              f"{size[0]}x{size[1]}x{size[2]} D3Q19 channel, FP64")
    return {
        "impl": "reference", "metric": METRIC, "value": mlups, "unit": "MLUPS", "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": sec / k_run * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "lattice": "D3Q19", "size": list(size), "storage": "fp64 AoS, two fields"},
        "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if args.profile:
        import torch
        torch.cuda.set_device(local)
        from lbm_gb300 import build_domain
        from lbm_gb300 import scenario as S
        if args.profile == "adjoint":
            with build_domain(S.adjoint_channel(128, 64, 64, omega=1.7, seed=0), "fp32") as d:
                d.adjoint_forward(args.warmup + args.steps, 10)
                d.adjoint_backward((97, 128, 1, 64, 1, 64))
                d.sync()
            return
        with build_domain(workload(19, tuple(int(v) for v in args.size.split(","))), args.profile) as d:
            d.step(args.warmup + args.steps)
            d.sync()
        return
    if args.extra_only:
        import torch
        torch.cuda.set_device(local)
        line = {"adjoint": run_adjoint(), "taylor_green": run_taylor_green(), "cavity512_d3q27": run_large_cavity(),
                "cavity256_adjoint": run_cavity_adjoint()}
        print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    line = run_ours(args, rank, world, local)
    if line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
