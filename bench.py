#!/usr/bin/env python
"""Benchmark of the five-equation block timestep on GB300.

Workload (default): the 2D air-helium shock-bubble on a 3-level block AMR
(levels 4..6 of a 4x1 brick, 16x16 blocks, finest dx = 1/1024, refined from
the initial condition by the SIMPLE_GRADIENT flags), synthetic data with the
shape of the reference's shock-bubble deck.  One "step" is one solver step of
the whole mesh: dt = cfl / inv_dt, the fused timestep kernel (+ coarse/fine
reflux pass), the boundary fill and the fused CFL reduction, replayed from a
CUDA graph (g5_advance).  The L2 cache (129 MB) is flushed before every timed
step (the mesh state fits in L2), and steps are timed with CUDA events on the
launching stream.

value            mixed-precision cell-updates/s (all ranks, replicas)
fp64_plain       the same for the FP64 reference method
e2e              g5_step_host through the C ABI with pinned host buffers: H2D
                 of U (chunked DMA), the step, and U2's owned blocks stored
                 into host memory by the step kernels, all inside the timed
                 region (copies overlapped with the chunk steps)
roofline         fused step kernel: 128 B/cell-update (read U + write U2,
                 8 FP64 variables) / kernel time, against the measured HBM copy
                 bandwidth of MEASURED_PEAKS.json
cpu_baseline     the CPU oracle (FP64 restatement, OpenMP) on the host cores,
                 bounded sample of the same workload
workloads        the same measurements (value, FP64 value, L1, roofline, CPU
                 baseline) for the other benchmark configurations, by
                 default the 256 batched droplet-advection instances, the 3D
                 triple point, the air-R22 THINC shock-bubble and the
                 gas-water shock tube (--extra-workloads)

--impl reference times the CPU restatement of the reference method (the
reference's own Kokkos build cannot be built: its kalypsso core, Kokkos and
p4est dependencies are absent) with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s, 1 GB300: mixed vs FP64 plain at L1 err<=1e-5 vs FP64; %HBM peak"
BYTES_PER_CELL_2D = 2 * 8 * 8  # read U + write U2, 8 FP64 variables
BYTES_PER_CELL_3D = 2 * 9 * 8  # read U + write U2, 9 FP64 variables
L1_STEPS = {"shock_bubble": 500, "gas_water": 200, "droplets": 100, "droplets32": 100, "shock_bubble_r22_thinc": 500, "triple_point_3d": 300, "triple_point_3d_small": 50}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=list(L1_STEPS), default="shock_bubble")
    ap.add_argument("--no-l1", action="store_true", help="skip the 500-step accuracy run")
    ap.add_argument(
        "--extra-workloads",
        default="droplets,triple_point_3d,shock_bubble_r22_thinc,gas_water",
        help="comma-separated workloads measured after the headline and reported under 'workloads' ('none' to skip)",
    )
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape (no g5_tune before timing)")
    ap.add_argument(
        "--reflux-layout",
        type=int,
        choices=[0, 1, 2],
        default=None,
        help="FP32-bulk 2D reflux layout of --profile and --no-tune runs (0 separate pass, 8 lanes per cell; 1 separate pass, one thread per cell; 2 the step kernel's tail; default: the library's)",
    )
    ap.add_argument("--profile", action="store_true", help="one FP64 and one mixed step kernel launch, for ncu")
    ap.add_argument("--no-clocks", action="store_true", help="skip the nvidia-smi clock sampling (and its bracketing load)")
    ap.add_argument(
        "--amr-cycles",
        type=int,
        default=0,
        help="time N dynamic AMR cycles (10 steps + flags, adaptation, remap, table upload) instead of the benchmark",
    )
    ap.add_argument(
        "--prolongation",
        type=int,
        choices=[0, 1, 2, 3],
        default=0,
        help="ghost cells in coarser neighbours: 0 SIMPLE_COPY, 1 minmod extrapolation, 2/3 conservative order 2/4",
    )
    return ap.parse_args()


def build_workload(name, flag_fn, prolongation=0, with_mesh=False, mesh_cls=None):
    desc, t, p, U, mesh = _workload(name, flag_fn, mesh_cls)
    if prolongation:
        import dataclasses

        p = dataclasses.replace(p, prolongation=prolongation)
        desc += ("", "_minmod_prolongation", "_conservative_o2_prolongation", "_conservative_o4_prolongation")[prolongation]
    return (desc, t, p, U, mesh) if with_mesh else (desc, t, p, U)


def _workload(name, flag_fn, mesh_cls=None):
    from godunov_five_eq_gb300 import configs
    from godunov_five_eq_gb300.mesh import BlockMesh

    kw = {"mesh_cls": mesh_cls or BlockMesh}

    if name == "shock_bubble":
        mesh, t, p, U = configs.shock_bubble("helium", thinc=False, flag_fn=flag_fn, **kw)
        desc = "shock_bubble_air_helium_2d_amr_levels4-6_16x16"
    elif name == "shock_bubble_r22_thinc":
        mesh, t, p, U = configs.shock_bubble("r22", thinc=True, flag_fn=flag_fn, **kw)
        desc = "shock_bubble_air_r22_thinc_2d_amr_levels4-6_16x16"
    elif name == "triple_point_3d":
        mesh, t, p, U = configs.triple_point_3d(flag_fn=flag_fn, **kw)
        desc = "triple_point_3d_thinc_amr_levels0-3_8x8x8"
    elif name == "triple_point_3d_small":
        mesh, t, p, U = configs.triple_point_3d(level_min=0, level_max=2, flag_fn=flag_fn, **kw)
        desc = "triple_point_3d_thinc_amr_levels0-2_8x8x8"
    elif name == "gas_water":
        mesh, t, p, U = configs.gas_water_shock_tube(**kw)
        desc = "gas_water_shock_tube_2d_512x32_16x16"
    elif name == "droplets32":
        _, t, p, U, _ = configs.droplet_instances(n_inst=32, **kw)
        U = np.ascontiguousarray(U)
        mesh = None
        desc = "droplet_advection_2d_32_instances_16x16"
    else:
        _, t, p, U, _ = configs.droplet_instances(**kw)
        U = np.ascontiguousarray(U)
        mesh = None
        desc = "droplet_advection_2d_256_instances_16x16"
    return desc, t, p, U, mesh


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL,
                text=True,
            )
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# committed ncu summary of each workload's step kernel, and the cells of the captured case
PROFILE_OF = {
    "shock_bubble": ("ncu_step2d_shock_bubble.md", 431104),
    "droplets32": ("ncu_step2d_droplets32.md", 2244608),
    "droplets": ("ncu_step2d_droplets32.md", 2244608),
    "triple_point_3d": ("ncu_step3d_triple_point.md", 1720320),
    "triple_point_3d_small": ("ncu_step3d_triple_point.md", 1720320),
}


def ncu_traffic(workload, mode, cells):
    """Per-launch DRAM bytes of the step kernel from the committed ncu summary,
    scaled by cells when the capture was a smaller case of the same kernel."""
    if workload not in PROFILE_OF:
        return None
    name, captured = PROFILE_OF[workload]
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    m = re.search(rf"traffic_bytes_per_launch_{mode}:\s*([0-9.eE+]+)", open(path).read())
    return float(m.group(1)) * cells / captured if m else None


def cpu_baseline(t, p, U, max_seconds=20.0):
    from oracle.oracle import Oracle

    cores = os.cpu_count() or 1
    o = Oracle(t, p, nthreads=cores)
    A = U.copy()
    o.fill_outside(A)
    dt = o.dt(A)
    A = o.step(A, dt)  # warm-up (first-touch of the work arrays)
    n, t0 = 0, time.perf_counter()
    while True:
        o.fill_outside(A)
        A = o.step(A, o.dt(A))
        n += 1
        el = time.perf_counter() - t0
        if el > max_seconds / 4 or n >= 20:
            break
    cells = t.n_owned * t.ncell
    o.close()
    return {
        "value": cells * n / el,
        "unit": "cell-updates/s",
        "cores": cores,
        "kind": "port",
        "sample": f"{n} solver steps (fill outside, dt reduction, step) of the same mesh, {cells} cells, FP64 oracle with OpenMP",
    }


def run_reference(args):
    from godunov_five_eq_gb300.replicas import rank_env

    if rank_env()[1] != 0:
        return 0
    from oracle.forest_py import PyBlockMesh
    from oracle.oracle import Oracle, oracle_flag_fn

    # the mesh comes from the Python forest restatement and the refine flags
    # from the oracle: this arm loads no library of the GPU product
    desc, t, p, U = build_workload(args.workload, oracle_flag_fn(), args.prolongation, mesh_cls=PyBlockMesh)
    cores = os.cpu_count() or 1
    o = Oracle(t, p, nthreads=cores)
    A = U.copy()
    for _ in range(max(args.warmup, 1)):
        o.fill_outside(A)
        A = o.step(A, o.dt(A))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.fill_outside(A)
        A = o.step(A, o.dt(A))
    el = time.perf_counter() - t0
    cells = t.n_owned * t.ncell
    value = cells * args.steps / el
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "cell-updates/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": desc, "blocks": int(t.n_owned), "cells": int(cells), "parallelism": "host threads"},
        "cpu_baseline": {
            "value": value,
            "unit": "cell-updates/s",
            "cores": cores,
            "kind": "port",
            "sample": f"{args.steps} solver steps of the full mesh ({cells} cells); CPU restatement of the reference method (the reference's Kokkos build is unavailable: kalypsso core, Kokkos and p4est are absent)",
        },
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _load(impl, A, B, mode, seconds):
    """Untimed solver steps for about `seconds` (keeps the GPU under the timed load)."""
    import torch

    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for _ in range(20):
            impl.advance(A, B, mode)
            A, B = B, A
        torch.cuda.synchronize()
    return A, B


def time_steps(impl, A, B, mode, steps, flush, stream):
    """K solver steps, each timed alone after an L2 flush; returns (total ms, launches, A, B)."""
    import torch

    total, launches = 0.0, 0
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        impl.advance(A, B, mode, stream=stream)
        e1.record(stream)
        launches += impl.last_launch_count()
        e1.synchronize()
        total += e0.elapsed_time(e1)
        A, B = B, A
    return total, launches, A, B


def time_kernel(impl, A, B, d_dt, mode, steps, flush, stream):
    """The fused step kernel alone (g5_step_dev), L2 flushed before each launch."""
    import torch

    ts = []
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        impl.do_time_step_dev(A, B, d_dt, mode, stream=stream)
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.mean(ts))


def run_profile_case(args):
    """The step kernel launched once in FP64 and once in mixed mode (for ncu)."""
    import torch

    from godunov_five_eq_gb300 import GodunovImplemGB300, gpu_flag_fn

    desc, t, p, U = build_workload(args.workload, gpu_flag_fn(), args.prolongation)
    impl = GodunovImplemGB300(p, t)
    if args.reflux_layout is not None:
        impl.set_shape("mixed", reflux_layout=args.reflux_layout)
    A = torch.from_numpy(U.copy()).cuda()
    B = torch.zeros_like(A)
    impl.fill_outside_quadrants(A)
    dt = impl.compute_dt_local(A)
    impl.do_time_step_dev(A, B, dt, mode="fp64")
    impl.do_time_step_dev(A, B, dt, mode="mixed")
    torch.cuda.synchronize()
    st = impl.status()
    print(json.dumps({"profile_case": desc, "cells": int(t.n_owned * t.ncell), "status": st}))
    return 0 if st == 0 else 1


def run_amr_case(args):
    """Dynamic AMR: N cycles of 10 mixed steps (the decks' cycle_frequency)
    then SolverGodunovFiveEq::do_amr_cycle's phases, each timed on the host
    with the device synchronised: boundary fill + refine flags + flag copy,
    forest adaptation, block table build, remap, table upload, boundary fill."""
    import time

    import torch

    from godunov_five_eq_gb300 import GodunovImplemGB300, gpu_flag_fn

    desc, t, p, U, mesh = build_workload(args.workload, gpu_flag_fn(), args.prolongation, with_mesh=True)
    if mesh is None:
        raise SystemExit("--amr-cycles needs a single-mesh workload")
    impl = GodunovImplemGB300(p, t)
    A = torch.from_numpy(U.copy()).cuda()
    phases = {k: [] for k in ("steps", "flags", "adapt", "build", "remap", "set_mesh", "fill")}
    blocks = []

    def now():
        torch.cuda.synchronize()
        return time.perf_counter()

    for cycle in range(args.amr_cycles + 1):
        B = torch.empty_like(A)
        impl.begin(A)
        t0 = now()
        for _ in range(10):
            impl.advance(A, B, "mixed")
            A, B = B, A
        t1 = now()
        impl.fill_outside_quadrants(A)
        flags = impl.refine_flags(A, 0, 0.1, 0.0125, 0.02, mesh.level_min, mesh.level_max).cpu().numpy()
        t2 = now()
        rt = mesh.adapt(flags)
        t3 = now()
        table = mesh.build()
        t4 = now()
        A2 = torch.empty((table.n_total, table.nv, table.ncell), dtype=torch.float64, device="cuda")
        impl.remap(rt, A, A2)
        t5 = now()
        impl.resize_auxiliary_data(table)
        t6 = now()
        impl.fill_outside_quadrants(A2)
        t7 = now()
        A = A2
        if cycle == 0:
            continue  # warm-up cycle
        for k, v in zip(phases, (t1 - t0, t2 - t1, t3 - t2, t4 - t3, t5 - t4, t6 - t5, t7 - t6)):
            phases[k].append(v * 1e3)
        blocks.append(table.n_owned)
    st = impl.status()
    ms = {k: round(float(np.median(v)), 3) for k, v in phases.items()}
    print(
        json.dumps(
            {
                "amr_cycles": args.amr_cycles,
                "workload": desc,
                "median_ms": ms,
                "cycle_ms": round(sum(ms.values()) - ms["steps"], 3),
                "blocks": blocks,
                "status": st,
            }
        )
    )
    return 0 if st == 0 else 1


def measure(name, args, world, local, flush, stream, steps, clocks=True, want_l1=True):
    """Time one workload: K graph-replayed solver steps per precision form (L2
    flushed before each), the step kernel alone, and the mixed form's L1 error
    against the FP64 form after the config's step count."""
    import torch
    import torch.distributed as dist

    from godunov_five_eq_gb300 import GodunovImplemGB300, gpu_flag_fn
    from godunov_five_eq_gb300.replicas import max_over_ranks, whole_job_rate

    desc, t, p, U = build_workload(name, gpu_flag_fn(), args.prolongation)
    cells = t.n_owned * t.ncell
    res = {}
    for mode in ("fp64", "mixed"):
        impl = GodunovImplemGB300(p, t)
        A = torch.from_numpy(U.copy()).cuda()
        B = torch.zeros_like(A)
        # the autotuner picks the launch shape of this mesh (g5_tune, untimed)
        impl.fill_outside_quadrants(A)
        if args.no_tune and args.reflux_layout is not None:
            impl.set_shape(mode, reflux_layout=args.reflux_layout)
        shape = impl.tune(A, B, mode) if not args.no_tune else impl.tune_choice(mode)
        # the tuner's candidates, fastest first: [ctas_per_sm, claim, walk_cf_first,
        # reflux_layout, ms per step]
        report = [] if args.no_tune else sorted(
            ([s[k] for k in GodunovImplemGB300.SHAPE_KEYS] + [round(ms, 5)] for s, ms in impl.tune_report(mode)), key=lambda r: r[-1]
        )
        impl.begin(A)
        for _ in range(args.warmup):
            impl.advance(A, B, mode)
            A, B = B, A
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        sampler = ClockSampler(local) if (mode == "mixed" and clocks) else None
        if sampler:
            # nvidia-smi samples every 200 ms: the same load runs for ~0.5 s
            # before and after the timed steps so that the samples see it
            sampler.start()
            A, B = _load(impl, A, B, mode, 0.5)
        total_ms, launches, A, B = time_steps(impl, A, B, mode, steps, flush, stream)
        if sampler:
            A, B = _load(impl, A, B, mode, 0.4)
        clk = sampler.stop() if sampler else None
        total_ms = max_over_ranks(total_ms, device="cuda")
        d_dt = impl.compute_dt_local(A)
        kern_ms = time_kernel(impl, A, B, d_dt, mode, max(5, min(steps, 20)), flush, stream)
        res[mode] = dict(total_ms=total_ms, launches=launches, clocks=clk, kern_ms=kern_ms, impl=impl, shape=shape, report=report)
        del A, B
    out = dict(desc=desc, t=t, p=p, U=U, cells=cells, res=res)
    out["value"] = whole_job_rate(world, cells, steps, res["mixed"]["total_ms"])
    out["value64"] = whole_job_rate(world, cells, steps, res["fp64"]["total_ms"])

    # accuracy of the mixed path: L1 against the FP64 path after the config's step count
    l1 = None
    if want_l1:
        nst = L1_STEPS[name]
        outs = {}
        for mode in ("fp64", "mixed"):
            impl = res[mode]["impl"]
            A = torch.from_numpy(U.copy()).cuda()
            B = torch.zeros_like(A)
            impl.run(A, B, nst, mode)
            torch.cuda.synchronize()
            outs[mode] = A.cpu().numpy()
            del A, B
        from godunov_five_eq_gb300.metrics import interface_error, l1_relative, linf_relative

        errs = [float(e) for e in l1_relative(t, outs["mixed"], outs["fp64"])]
        linf = [float(e) for e in linf_relative(t, outs["mixed"], outs["fp64"])]
        l1 = {
            "steps": nst,
            "max": max(errs),
            "per_variable": errs,
            "norm": "volume-weighted relative L1 (momentum by |rho u|)",
            "linf_max": max(linf),
            "linf_per_variable": linf,
            "interface": interface_error(t, outs["mixed"], outs["fp64"]) if t.n_inst == 1 else None,
        }
    out["l1"] = l1

    peak, peak_kind = measured_peaks()
    kern_s = res["mixed"]["kern_ms"] * 1e-3
    bpc = BYTES_PER_CELL_2D if t.dim == 2 else BYTES_PER_CELL_3D
    achieved = cells * bpc / kern_s / 1e9
    traffic = ncu_traffic(name, "mixed", cells)
    # the coarse/fine record pass runs only where a face has a finer neighbour
    faces = [3, 5, 1, 7] if t.dim == 2 else [12, 14, 10, 16, 4, 22]
    has_records = bool((t.nbr_rel[: t.n_owned][:, faces] > 0).any())
    if t.dim == 2:
        kernel_label = "step2d_kernel<16,mixed>" + (
            ("" if not has_records else " (+reflux in its tail)" if res["mixed"]["shape"].get("reflux_layout") == 2 else " (+reflux2d)")
        )
    else:
        kernel_label = "step3d_kernel<mixed>" + (" (+reflux3d)" if has_records else "")
    out["roofline"] = {
        "bound": "hbm",
        "achieved": achieved,
        "peak": peak,
        "unit": "GB/s",
        "frac": achieved / peak,
        "traffic": traffic,
        "traffic_source": (f"committed ncu capture profiles/{PROFILE_OF[name][0]} (dram read + write bytes per launch), scaled by cells" if traffic else None),
        "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s",
        "kernel": kernel_label,
        "kernel_ms": res["mixed"]["kern_ms"],
        "algorithmic_bytes_per_launch": cells * bpc,
        "fp64_kernel_ms": res["fp64"]["kern_ms"],
        "fp64_frac": cells * bpc / (res["fp64"]["kern_ms"] * 1e-3) / 1e9 / peak,
    }
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile:
        return run_profile_case(args)
    if args.amr_cycles > 0:
        return run_amr_case(args)
    import torch
    import torch.distributed as dist

    from godunov_five_eq_gb300.replicas import max_over_ranks, rank_env, whole_job_rate

    world, rank, local = rank_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    stream = torch.cuda.current_stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float64, device="cuda")  # 512 MB > L2
    m = measure(args.workload, args, world, local, flush, stream, args.steps, clocks=not args.no_clocks, want_l1=not args.no_l1)
    desc, t, p, U, cells, res = m["desc"], m["t"], m["p"], m["U"], m["cells"], m["res"]
    value, value64 = m["value"], m["value64"]

    # end to end through the C ABI with host buffers: g5_step_host copies the
    # pinned host U (owned + outside blocks) to the device and the owned blocks
    # of U2 back, chunk by chunk, overlapped with the step
    impl = res["mixed"]["impl"]
    A = torch.from_numpy(U.copy()).cuda()
    impl.fill_outside_quadrants(A)
    hU = A.cpu().pin_memory()
    hO = torch.empty_like(hU).pin_memory()
    dt_host = impl.compute_dt_local(A).cpu().numpy()
    del A
    e2e_ms = 0.0
    for k in range(args.warmup + args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        impl.do_time_step_host(hU, hO, dt_host, mode="mixed", stream=stream)
        e1.record(stream)
        e1.synchronize()
        if k >= args.warmup:
            e2e_ms += e0.elapsed_time(e1)
    blk = t.nv * t.ncell * 8
    e2e = {
        "value": whole_job_rate(world, cells, args.steps, max_over_ranks(e2e_ms, device="cuda")),
        "unit": "cell-updates/s",
        "h2d_bytes_per_step": int(t.n_total * blk),
        "d2h_bytes_per_step": int(t.n_owned * blk),
        "api": "g5_step_host: pinned host U copied in chunks of about 3.5 MB (8 to 16), chunk steps on 8 streams as neighbours arrive, U2 stored by the kernels into pinned host memory (one CUDA graph)",
    }
    del hU, hO
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(t, p, U)
    for mode in ("fp64", "mixed"):
        res[mode]["impl"].close()

    # further workloads on the same line (not the headline): the batched
    # droplet instances (many uneven instances in one persistent launch), the
    # 3D triple point (8^3 blocks, THINC, levels 0..3), the air-R22 THINC
    # shock-bubble and the gas-water shock tube
    workloads = {}
    for extra in [w for w in args.extra_workloads.split(",") if w and w != "none" and w != args.workload]:
        mx = measure(extra, args, world, local, flush, stream, min(args.steps, 10), clocks=False, want_l1=not args.no_l1)
        tx = mx["t"]
        workloads[extra] = {
            "workload": mx["desc"],
            "instances": int(tx.n_inst),
            "blocks": int(tx.n_owned),
            "cells": int(mx["cells"]),
            "value": mx["value"],
            "unit": "cell-updates/s",
            "ms_per_step": mx["res"]["mixed"]["total_ms"] / min(args.steps, 10),
            "fp64_plain": {"value": mx["value64"], "unit": "cell-updates/s"},
            "speedup_mixed_vs_fp64": mx["value"] / mx["value64"],
            "l1_err_vs_fp64": mx["l1"],
            "roofline": mx["roofline"],
            "cpu_baseline": cpu_baseline(tx, mx["p"], mx["U"], max_seconds=12.0) if (rank == 0 and not args.no_cpu) else None,
            "gpu_launches": int(mx["res"]["mixed"]["launches"]),
            "launch_shape": {mode: mx["res"][mode]["shape"] for mode in ("fp64", "mixed")},
        }
        for mode in ("fp64", "mixed"):
            mx["res"][mode]["impl"].close()
        del mx
    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "cell-updates/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": res["mixed"]["total_ms"] / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32+f64",
            "data": "synthetic",
            "config": {
                "workload": desc,
                "blocks": int(t.n_owned),
                "outside_blocks": int(t.n_outside),
                "cells": int(cells),
                "blocks_per_level": {int(k): int(v) for k, v in enumerate(np.bincount(t.level[: t.n_owned])) if v},
                "l2": "flushed (512 MB write) before every timed step",
                "parallelism": "replicas" if world > 1 else "single GPU",
                "launch_shape": {mode: res[mode]["shape"] for mode in ("fp64", "mixed")},
                "tuner_candidates_mixed": res["mixed"]["report"][:8],
            },
            "fp64_plain": {"value": value64, "unit": "cell-updates/s", "ms_per_step": res["fp64"]["total_ms"] / args.steps},
            "speedup_mixed_vs_fp64": value / value64,
            "l1_err_vs_fp64": m["l1"],
            "roofline": m["roofline"],
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(res["mixed"]["launches"]),
            "clocks": res["mixed"]["clocks"],
            "workloads": workloads,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
