"""Benchmark: DG DOF-updates/s of the explicit SSP-RK3 time step on one GB300.

Workload (default): Euler isentropic vortex, periodic [0,10]^3, uniform
level 7 (128^3 = 2,097,152 hex), p1 Taylor basis (4 coefficients), 5
conserved variables, HLLC flux, no limiter, seeded +-1e-3 density noise.
One bench step = one full SSP-RK3 time step (3 stages) over the whole mesh.

  DOF-updates/s = E * V * B * 3 stages * steps / seconds

Lines printed (rank 0, one JSON object each run):
  * our arm: plain FP64 path (the drop-in) as `value`, with
      - `e2e`: the same metric through the C ABI with host buffers (state
        H2D + step + state D2H every step),
      - `mixed`: the FP32-residual / FP32 hi-lo-state form on the same steps
        with its error against the FP64 path; `double_word`: the FP32-pair
        form held to the drop-in's bar,
      - `roofline` (HBM, and the FP64 pipe's counted rate), `cpu_baseline`,
        `clocks`, `gpu_launches`, `parity` (the FP64 state vs the oracle),
      - summaries of the legs on the other configurations: `adjoint`
        (config 5), `reacting_ns` (config 4, p2), `blast_amr` (config 3),
        `p2_contraction` (tensor cores vs FMA) and `hex_sample` (the
        reference's sample case on its trilinear hexahedra); their full
        records are in `details`.
  * --impl reference: the reference's CPU algorithm (the oracle
    restatement, all host cores) on a bounded sample of the same workload.

Multi-GPU: the path is run as independent replicas (one per rank, weak
scaling); there is no data-path collective.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "DG DOF-updates/s (SSP-RK3 stage DOF updates per second)"
UNIT = "DOF-updates/s"
STAGES = 3
L2_BYTES = 129e6


# counted FP64 flops per face quadrature point of face_kernel<double, 1, HLLC>
# (profiles/face_kernel_fp64_instruction_mix_vortex_32k.md)
FP64_FLOPS_PER_FACE_POINT = 245.1


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return {"hbm_gbs": float(d["hbm_gbs"]), "src": "measured"}
    return {"hbm_gbs": 6800.0, "src": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"charm_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
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
            self.fh.close()

    def summary(self) -> dict:
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names[1:], parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def workload(level: int, brick: int = 1):
    """The vortex workload; brick > 1 stretches the box along x (profiling sizes)."""
    from charm_3d_gb300 import synthetic
    c = synthetic("vortex", level=level)
    if brick > 1:
        c.brick = (brick, 1, 1)
    return c


def dof_per_step(E: int, V: int) -> int:
    return E * V * 4 * STAGES


# ---------------------------------------------------------------------------
# CPU baseline (oracle restatement), used by our arm and by --impl reference
# ---------------------------------------------------------------------------

def _port_worker(args):
    level, seconds = args
    sys.path.insert(0, ROOT)
    from charm_3d_gb300.solver import Forest
    from oracle.port import Port
    case = workload(level)
    f = Forest(case)
    mesh = f.flatten()
    port = Port(case.config(), mesh)
    port.set_state(case.initial_state(mesh.center))
    steps, t0 = 0, time.perf_counter()
    while True:
        port.step(case.tau)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return mesh.n_elem, 4 + case.n_comp, steps, el


def cpu_sample_with_state(level: int, steps: int):
    """The oracle on the vortex at `level` for exactly `steps` steps from the
    seeded state, timed (one core): (cpu_baseline dict, mesh, u0, final state)."""
    from charm_3d_gb300.solver import Forest
    from oracle.port import Port
    case = workload(level)
    mesh = Forest(case).flatten()
    u0 = case.initial_state(mesh.center)
    port = Port(case.config(), mesh)
    port.set_state(u0)
    t0 = time.perf_counter()
    port.run(steps, case.tau)
    el = time.perf_counter() - t0
    u = port.get_state()
    port.close()
    E, V = mesh.n_elem, 4 + case.n_comp
    cpu = {"value": dof_per_step(E, V) * steps / el, "unit": UNIT, "cores": 1, "kind": "port",
           "sample": f"vortex level {level} ({E} hex), {steps} SSP-RK3 steps in {el:.1f} s, one process; "
                     f"oracle/charm_oracle.c -O2"}
    return cpu, case, mesh, u0, u


def parity_vs_oracle(level: int, steps: int, device: int):
    """cpu_baseline and the parity of the GPU's FP64 path with the oracle on
    the same sample (the bench workload at `level`, `steps` steps, outside
    the timed region)."""
    from charm_3d_gb300.solver import Solver
    cpu, case, mesh, u0, want = cpu_sample_with_state(level, steps)
    gpu = Solver(case, device)
    gpu.upload(mesh)
    gpu.set_state(u0)
    gpu.run(steps, case.tau)
    gpu.sync()
    got = gpu.get_state()
    gpu.close()
    par = {"oracle_rel_l2": float(np.linalg.norm(got - want) / np.linalg.norm(want)), "bar": 1e-12,
           "level": level, "elements": int(mesh.n_elem), "steps": steps,
           "what": "GPU FP64 state vs oracle/charm_oracle.c after the same steps from the same seeded state"}
    return cpu, par


def cpu_baseline(level: int, seconds: float, cores: int) -> dict:
    if cores <= 1:
        E, V, steps, el = _port_worker((level, seconds))
        rate = dof_per_step(E, V) * steps / el
    else:
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        with ctx.Pool(cores) as pool:
            res = pool.map(_port_worker, [(level, seconds)] * cores)
        rate = sum(dof_per_step(E, V) * s / el for E, V, s, el in res)
        E, V, steps, el = res[0]
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"vortex level {level} ({E} hex), {steps} SSP-RK3 steps per process in {el:.1f} s, "
                      f"{cores} independent process(es); oracle/charm_oracle.c -O2"}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def run_gpu(args, rank: int, world: int, device: int) -> dict | None:
    from charm_3d_gb300 import abi
    from charm_3d_gb300.solver import Forest, Solver

    case = workload(args.level, args.brick)
    t0 = time.perf_counter()
    forest = Forest(case)
    mesh = forest.flatten()
    u0 = case.initial_state(mesh.center)
    t_mesh = time.perf_counter() - t0
    E, V = mesh.n_elem, case.n_var
    state_bytes = u0.nbytes

    if args.only == "mixed":
        return run_mixed_only(args, case, mesh, u0, device, world)
    if args.only == "dw":
        case.precision = "DW"
        g = Solver(case, device)
        g.upload(mesh)
        g.set_state(u0)
        g.run(args.warmup, case.tau)
        g.sync()
        g.set_state(u0)
        g.reset_stats()
        g.set_timing(True)
        msd = g.time_run(args.steps, case.tau)
        g.set_timing(False)
        n_l, k_ms = g.kernel_stats()
        g.close()
        print(json.dumps({"only": "dw", "ms_per_step": msd / args.steps, "kernel_ms": k_ms.tolist(),
                          "launches": n_l.tolist()}))
        return None
    # ---- plain FP64 (drop-in) ----
    case.precision = "FP64"
    gpu = Solver(case, device)
    gpu.upload(mesh)
    gpu.set_state(u0)
    gpu.run(args.warmup, case.tau)
    gpu.sync()
    gpu.set_state(u0)
    gpu.reset_stats()
    gpu.set_timing(True)
    barrier(world)
    with ClockSampler(device) as clk:
        ms = gpu.time_run(args.steps, case.tau)
    gpu.set_timing(False)
    launches, kms = gpu.kernel_stats()
    ms = max_over_ranks(ms, world)
    u64 = gpu.get_state()
    value = dof_per_step(E, V) * args.steps * world / (ms * 1e-3)

    if args.only == "fp64":
        gpu.close()
        if rank == 0:
            print(json.dumps({"only": "fp64", "ms_per_step": ms / args.steps, "value": value,
                              "kernel_ms": kms.tolist(), "launches": launches.tolist()}))
        return None
    # ---- mixed form on the same steps ----
    case.precision = "MIXED"
    g32 = Solver(case, device)
    g32.upload(mesh)
    g32.set_state(u0)
    g32.run(args.warmup, case.tau)
    g32.sync()
    g32.set_state(u0)
    g32.reset_stats()
    barrier(world)
    ms32 = max_over_ranks(g32.time_run(args.steps, case.tau), world)
    u32 = g32.get_state()
    rho64, rho32 = u64[4:].sum(axis=0), u32[4:].sum(axis=0)
    mass64 = float(np.sum(rho64[0])) ; mass32 = float(np.sum(rho32[0]))
    mass0 = float(np.sum(u0[4:].sum(axis=0)[0]))
    mixed = {"value": dof_per_step(E, V) * args.steps * world / (ms32 * 1e-3), "unit": UNIT,
             "ms_per_step": ms32 / args.steps, "speedup_vs_fp64": ms / ms32,
             "rel_l2_density_vs_fp64": float(np.linalg.norm(rho32 - rho64) / np.linalg.norm(rho64)),
             "rel_l2_state_vs_fp64": float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64)),
             "mass_drift_fp64": (mass64 - mass0) / mass0, "mass_drift_mixed": (mass32 - mass0) / mass0,
             "dtype": "f32 residual, f32 hi/lo state pairs (float-float update), f64 dt"}
    g32.close()

    # ---- double-word form (FP64 state, FP32-pair residual) on the same steps ----
    dwf = None
    if not args.skip_dw:
        case.precision = "DW"
        gdw = Solver(case, device)
        gdw.upload(mesh)
        gdw.set_state(u0)
        gdw.run(args.warmup, case.tau)
        gdw.sync()
        gdw.set_state(u0)
        gdw.reset_stats()
        gdw.set_timing(True)
        barrier(world)
        msdw = max_over_ranks(gdw.time_run(args.steps, case.tau), world)
        gdw.set_timing(False)
        _, kdw = gdw.kernel_stats()
        udw = gdw.get_state()
        gdw.close()
        dwf = {"value": dof_per_step(E, V) * args.steps * world / (msdw * 1e-3), "unit": UNIT,
               "ms_per_step": msdw / args.steps, "speedup_vs_fp64": ms / msdw,
               "rel_l2_state_vs_fp64": float(np.linalg.norm(udw - u64) / np.linalg.norm(u64)),
               "kernel_ms_face_cell": [float(kdw[0]), float(kdw[1])],
               "dtype": "f64 state; fluxes and volume terms in double-word f32 pairs (~48-bit)"}
        case.precision = "FP64"

    # ---- e2e through the C ABI with host buffers ----
    if args.skip_e2e:
        e2e = None
        gpu.close()
        return finish(args, rank, world, device, case, mesh, E, V, state_bytes, t_mesh, value, ms, launches, kms,
                      mixed, e2e, clk, dwf)
    import torch
    pin_in = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True).numpy()
    pin_out = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True).numpy()
    pin_in[...] = u0
    n_e2e = max(1, min(args.steps, 5))
    gpu.set_state(pin_in)
    gpu.step(case.tau)
    gpu.get_state(pin_out)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        gpu.set_state(pin_in)
        gpu.step(case.tau)
        gpu.get_state(pin_out)
    t_e2e = max_over_ranks(time.perf_counter() - t0, world)
    e2e = {"value": dof_per_step(E, V) * n_e2e * world / t_e2e, "unit": UNIT, "h2d_bytes_per_step": state_bytes,
           "d2h_bytes_per_step": state_bytes, "steps": n_e2e,
           "path": "charm_gpu_set_state(host) + charm_gpu_step + charm_gpu_get_state(host), pinned buffers"}
    gpu.close()
    return finish(args, rank, world, device, case, mesh, E, V, state_bytes, t_mesh, value, ms, launches, kms, mixed,
                  e2e, clk, dwf)


def run_mixed_only(args, case, mesh, u0, device, world):
    from charm_3d_gb300.solver import Solver
    case.precision = "MIXED"
    g32 = Solver(case, device)
    g32.upload(mesh)
    g32.set_state(u0)
    g32.run(args.warmup, case.tau)
    g32.sync()
    g32.set_state(u0)
    g32.reset_stats()
    g32.set_timing(True)
    ms32 = g32.time_run(args.steps, case.tau)
    g32.set_timing(False)
    launches, kms = g32.kernel_stats()
    g32.close()
    print(json.dumps({"only": "mixed", "ms_per_step": ms32 / args.steps, "kernel_ms": kms.tolist(),
                      "launches": launches.tolist()}))
    return None


def finish(args, rank, world, device, case, mesh, E, V, state_bytes, t_mesh, value, ms, launches, kms, mixed, e2e,
           clk, dwf=None):
    from charm_3d_gb300 import abi
    if rank != 0:
        return None

    # ---- roofline for the dominant kernel ----
    pk = peaks()
    names = ["face", "cell", "limiter", "other"]
    dom = int(np.argmax(kms))
    per_launch_ms = kms[dom] / max(launches[dom], 1)
    F = mesh.n_face + mesh.n_bface
    # algorithmic bytes per launch (FP64): face kernel reads the stage state
    # once (V*B*8 per element) and the face records (9 B per face); the cell
    # kernel reads the stage state and u^n and writes the new state, plus the
    # element level byte.  Slot buffers are intermediate and not counted.
    alg = {"face": E * V * 4 * 8 + F * 9, "cell": E * (3 * V * 4 * 8 + 1), "limiter": E * (3 * V * 4 * 8 + 24),
           "other": E * V * 8}
    achieved = alg[names[dom]] / (per_launch_ms * 1e-3) / 1e9
    # DRAM bytes (read + write) of one face_kernel<double> launch on the
    # level-7 vortex (2,097,152 hex), from one ncu capture (dram__bytes_read /
    # _write, 1 pass) of this bench command: 1.111 GB read, 1.961 GB written
    # (the slot buffer: 2 sides x V x 4 coefficients x 8 B per face)
    traffic = 1111392000 + 1960973056 if (names[dom] == "face" and E == 2 ** 21 and V == 5) else None
    fp64_peak = probe(abi, device, 0)
    # FP64 flops of the face kernel (HLLC, one species) per face point, from
    # the thread-level DFMA / DADD / DMUL counts of one ncu capture of this
    # kernel on the level-5 vortex (an FMA counted as 2 flops):
    # 2 x 83.4 + 25.4 + 52.8 = 245.1 per point, 6 points per face record
    fp64 = {"peak_tflops_measured": fp64_peak, "flops_per_face_point_counted": FP64_FLOPS_PER_FACE_POINT}
    if names[dom] == "face" and V == 5 and case.flux == "HLLC":
        tf = FP64_FLOPS_PER_FACE_POINT * 6 * F / (per_launch_ms * 1e-3) / 1e12
        fp64.update({"achieved_tflops": tf, "frac": tf / fp64_peak if fp64_peak else None,
                     "note": "the plain FP64 path is bound by the FP64 pipe (profiles/)"})
    roofline = {"bound": "hbm", "kernel": names[dom] + "_kernel<double>", "achieved": achieved,
                "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": achieved / pk["hbm_gbs"],
                "peak_src": pk["src"], "traffic": traffic,
                "algorithmic_bytes_per_launch": alg[names[dom]], "launch_ms": per_launch_ms,
                "kernel_share": {n: float(kms[i] / kms.sum()) for i, n in enumerate(names)},
                "fp64_pipe": fp64}
    cpu, parity = parity_vs_oracle(args.cpu_level, args.parity_steps, device) if args.parity_steps > 0 else (None, None)
    adjoint = run_adjoint(args, device) if args.adjoint_steps > 0 else None
    flame = run_flame(args, device) if args.flame_steps > 0 else None
    blast = run_blast(args, device) if args.blast_steps > 0 else None
    blast_rel = run_blast(args, device, relative=0.1) if args.blast_steps > 0 else None
    tc = run_tc(args) if args.tc_reps > 0 else None
    hexs = run_hex(args, device) if args.hex_steps > 0 else None
    n_launch = int(launches.sum())
    # the full records first; the one-line summaries of the extra legs last,
    # where a reader of the end of the line finds them
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded isentropic vortex + 1e-3 density noise)",
            "config": bench_config(args, world, E, V, state_bytes, t_mesh),
            "details": {"mixed": mixed, "double_word": dwf, "adjoint": adjoint, "reacting_ns": flame,
                        "blast_amr": blast, "blast_amr_relative": blast_rel, "p2_contraction": tc,
                        "hex_sample": hexs},
            "e2e": e2e,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "gpu_launches": n_launch,
            "clocks": clk.summary(),
            "parity": parity,
            "mixed": summary_mixed(mixed), "double_word": summary_dw(dwf), "adjoint": summary_adjoint(adjoint),
            "reacting_ns": summary_flame(flame), "blast_amr": summary_blast(blast),
            "blast_amr_relative": summary_blast(blast_rel), "p2_contraction": summary_tc(tc),
            "hex_sample": summary_hex(hexs)}


def bench_config(args, world: int, E: int, V: int, state_bytes: int, t_mesh: float | None) -> dict:
    c = {"workload": f"Euler isentropic vortex, periodic [0,10]^3, level {args.level} ({E} hex), p1, HLLC, "
                     f"no limiter, SSP-RK3",
         "elements": E, "variables": V, "basis": 4, "stages_per_step": STAGES,
         "parallelism": f"replicas x{world}",
         "l2": f"inputs larger than L2 (state {state_bytes / 1e6:.0f} MB > 129 MB)"}
    if t_mesh is not None:
        c["mesh_build_s"] = t_mesh
    return c


def _r(x, n=4):
    return None if x is None else float(f"{x:.{n}g}")


def summary_mixed(m):
    if not m:
        return None
    return {"ms_per_step": _r(m["ms_per_step"]), "value": _r(m["value"]), "x_fp64": _r(m["speedup_vs_fp64"]),
            "rel_l2_density_vs_fp64": _r(m["rel_l2_density_vs_fp64"], 3), "mass_drift": _r(m["mass_drift_mixed"], 3)}


def summary_dw(d):
    if not d:
        return None
    return {"ms_per_step": _r(d["ms_per_step"]), "value": _r(d["value"]), "x_fp64": _r(d["speedup_vs_fp64"]),
            "rel_l2_state_vs_fp64": _r(d["rel_l2_state_vs_fp64"], 3)}


def summary_adjoint(a):
    if not a:
        return None
    out = {"x_forward": _r(a["adjoint_over_forward"]),
           "reverse_step_x_forward_step": _r(a["reverse_step_over_forward_step"]), "snapshots": a["n_snapshots"],
           "fd_max": _r(a["fd_check"]["max_rel_err"], 3), "fd_median": _r(a["fd_check"]["median_rel_err"], 3)}
    if a.get("revolve"):
        out["revolve_x_forward"] = _r(a["revolve"]["adjoint_over_forward"])
        out["revolve_snapshots"] = a["revolve"]["n_snapshots"]
    if a["fd_check"].get("smooth"):
        out["fd_smooth_max"] = _r(a["fd_check"]["smooth"]["max_rel_err"], 3)
    return out


def summary_flame(f):
    if not f:
        return None
    out = {"fp64_ms_per_step": _r(f["ms_per_step"])}
    if isinstance(f.get("mixed"), dict):
        out.update({"mixed_ms_per_step": _r(f["mixed"]["ms_per_step"]), "x_fp64": _r(f["mixed"]["speedup_vs_fp64"]),
                    "rel_l2_density": _r(f["mixed"]["rel_l2_density_vs_fp64"], 3)})
    return out


def summary_hex(x):
    if not x:
        return None
    return {"value": _r(x["value"]), "ms_per_step": _r(x["ms_per_step"]), "elements": x["elements"],
            "parity_rel_l2": _r(x["parity"]["oracle_rel_l2"])}


def summary_tc(t):
    if not t or "tcgen05_over_fma_time" not in t:
        return None
    return {"fma_ms": _r(t["fma"]["ms"]), "tcgen05_ms": _r(t["tcgen05"]["ms"]),
            "max_rel_diff": _r(t["max_rel_diff_values"], 3)}


def summary_blast(b):
    if not b:
        return None
    return {"fp64_value": _r(b["fp64"]["value"]), "mixed_value": _r(b["mixed"]["value"]),
            "mixed_e2e": _r(b["mixed"]["e2e_dof_updates_per_s"]), "mixed_adapt_share":
                _r(b["mixed"]["adapt_s"] / b["mixed"]["wall_s"], 3), "same_mesh": b["same_mesh"],
            "final_elements": b["mixed"]["final_elements"]}


def run_adjoint(args, device: int) -> dict:
    """Discrete adjoint of the vortex at level `adjoint_level`: J = integral of
    p over [4,6]^3 after `adjoint_steps` steps, gradient with respect to the
    initial state (checked against central differences in the density
    perturbation), its wall time against the forward run of the same steps."""
    from charm_3d_gb300.solver import Forest, Solver
    case = workload(args.adjoint_level)
    case.precision = "FP64"
    mesh = Forest(case).flatten()
    u0 = case.initial_state(mesh.center)
    n = args.adjoint_steps
    snaps = args.adjoint_snapshots if args.adjoint_snapshots > 0 else 3 * n
    blo, bhi = (float(x) for x in args.adjoint_box.split(","))
    obj = Solver.pressure_box((blo,) * 3, (bhi,) * 3)
    gpu = Solver(case, device)
    gpu.upload(mesh)
    gpu.set_state(u0)
    gpu.run(3, case.tau)
    gpu.sync()
    # forward run of the same steps (wall clock, synchronised), median of 3
    t_fwds = []
    for _ in range(3):
        gpu.set_state(u0)
        gpu.sync()
        t0 = time.perf_counter()
        gpu.run(n, case.tau)
        gpu.sync()
        t_fwds.append(time.perf_counter() - t0)
    t_fwd = float(np.median(t_fwds))
    J_fwd = gpu.objective(obj)
    # the first call allocates the checkpoint buffers; the next 3 are measured (median)
    gpu.set_state(u0)
    gpu.adjoint(n, snaps, obj)
    t_adjs = []
    for _ in range(3):
        gpu.set_state(u0)
        gpu.sync()
        t0 = time.perf_counter()
        grad, info = gpu.adjoint(n, snaps, obj)
        t_adjs.append(time.perf_counter() - t0)
    t_adj = float(np.median(t_adjs))
    # the same run with the checkpoints bounded (binomial schedule,
    # recomputation): the memory-bounded form long runs need
    revolve = None
    if args.adjoint_revolve_snapshots > 0:
        rs = args.adjoint_revolve_snapshots
        gpu.set_state(u0)
        grad_r, info_r = gpu.adjoint(n, rs, obj)      # allocates the buffers
        t_revs = []
        for _ in range(2):
            gpu.set_state(u0)
            gpu.sync()
            t0 = time.perf_counter()
            gpu.adjoint(n, rs, obj)
            t_revs.append(time.perf_counter() - t0)
        t_rev = float(np.median(t_revs))
        revolve = {"n_snapshots": rs, "adjoint_s": t_rev, "adjoint_over_forward": t_rev / t_fwd,
                   "forward_steps_in_adjoint": int(info_r.forward_steps), "snapshots_held": int(info_r.snapshots),
                   "state_bytes_per_snapshot": int(u0.nbytes),
                   "gradient_equal_to_full_storage": bool(np.array_equal(grad_r, grad))}
    # central differences along random density perturbations (variable rc_0, coefficient 0)
    rng = np.random.default_rng(2024)
    eps = args.adjoint_fd_eps
    # the same run with J over the whole box: no zero region of the adjoint to skip
    gpu.set_state(u0)
    gpu.sync()
    t0 = time.perf_counter()
    gpu.adjoint(n, snaps, Solver.pressure_box((0.0, 0.0, 0.0), (10.0, 10.0, 10.0)))
    t_dense = time.perf_counter() - t0
    # the same directions also at eps / 10: white-noise directions move some
    # face points across HLLC's case switches, where a difference quotient
    # mixes the two one-sided derivatives; that part of the error shrinks
    # with the step, down to the round-off of J
    # besides the relative error of each directional derivative, its size
    # and the error normalised by |dJ/du restricted to the perturbed
    # coefficients| * |d| (Cauchy-Schwarz bound of the derivative): a
    # direction nearly orthogonal to the gradient has a small derivative, and
    # the round-off of J / eps then dominates its relative error
    gsub = grad[4, 0]
    fd_abs, fd_norm = {}, {}

    def fd_err(d, h, key=None):
        ad = float((grad * d).sum())
        Js = []
        for sgn in (1.0, -1.0):
            gpu.set_state(u0 + sgn * h * d)
            gpu.run(n, case.tau)
            Js.append(gpu.objective(obj))
        fd = (Js[0] - Js[1]) / (2 * h)
        if key is not None:
            fd_abs.setdefault(key, []).append(float(f"{abs(fd):.3g}"))
            fd_norm.setdefault(key, []).append(
                float(f"{abs(ad - fd) / (np.linalg.norm(gsub) * np.linalg.norm(d[4, 0])):.3g}"))
        return abs(ad - fd) / max(abs(fd), 1e-300)

    errs, errs10 = [], []
    for k in range(args.adjoint_fd):
        d = np.zeros_like(u0)
        d[4, 0] = rng.uniform(-1.0, 1.0, mesh.n_elem)
        errs.append(fd_err(d, eps, "white"))
        if k < 4:
            errs10.append(fd_err(d, 0.1 * eps))
    # smooth random directions: a few random Fourier modes of the element
    # centres (the seeded perturbation's variable and coefficient), which
    # move far fewer face points across HLLC's case switches than white noise
    errs_s = []
    L = 10.0
    for _ in range(args.adjoint_fd):
        d = np.zeros_like(u0)
        field = np.zeros(mesh.n_elem)
        for _m in range(3):
            kv = rng.integers(1, 4, 3)
            ph = rng.uniform(0, 2 * np.pi)
            field += rng.uniform(-1, 1) * np.sin(2 * np.pi * (kv @ mesh.center) / L + ph)
        d[4, 0] = field
        errs_s.append(fd_err(d, eps, "smooth"))
    gpu.close()
    return {"workload": f"vortex level {args.adjoint_level} ({mesh.n_elem} hex), HLLC, no limiter, FP64, "
                        f"J = integral of p over [{args.adjoint_box}]^3 at step {n}",
            "n_steps": n, "n_snapshots": snaps, "J": info.J, "J_forward": J_fwd,
            "forward_s": t_fwd, "adjoint_s": t_adj, "adjoint_over_forward": t_adj / t_fwd,
            # the reverse step alone (the adjoint's own forward sweep runs the
            # forward run's kernels, so it takes the forward run's time)
            "reverse_step_over_forward_step": (t_adj - t_fwd) / t_fwd,
            "forward_s_runs": t_fwds, "adjoint_s_runs": t_adjs,
            "adjoint_whole_domain_J_over_forward": t_dense / t_fwd,
            "forward_steps_in_adjoint": int(info.forward_steps), "snapshots_held": int(info.snapshots),
            "revolve": revolve,
            "fd_check": {"directions": args.adjoint_fd, "eps": eps, "max_rel_err": max(errs) if errs else None,
                         "median_rel_err": float(np.median(errs)) if errs else None,
                         "per_direction": [float(f"{x:.3g}") for x in errs],
                         "abs_fd_per_direction": fd_abs.get("white"),
                         "err_over_gradnorm_times_dnorm": fd_norm.get("white"),
                         "eps_over_10": {"eps": 0.1 * eps, "directions": len(errs10),
                                         "per_direction": [float(f"{x:.3g}") for x in errs10]},
                         "direction": "uniform(-1, 1) on the density mean of every element (the seeded "
                                      "noise's variable and coefficient)",
                         "smooth": {"directions": len(errs_s), "eps": eps,
                                    "max_rel_err": max(errs_s) if errs_s else None,
                                    "median_rel_err": float(np.median(errs_s)) if errs_s else None,
                                    "per_direction": [float(f"{x:.3g}") for x in errs_s],
                                    "abs_fd_per_direction": fd_abs.get("smooth"),
                                    "err_over_gradnorm_times_dnorm": fd_norm.get("smooth"),
                                    "direction": "sum of 3 random Fourier modes (wave numbers 1..3 per axis, "
                                                 "random phase and amplitude) on the density mean"}}}


def _flame_run(case, mesh, u0, steps: int, device: int, precision: str):
    """Warm-up, then `steps` timed steps (CUDA events on the solver's stream)
    from u0; returns (ms, per-class kernel ms, final state)."""
    from charm_3d_gb300.solver import Solver
    case.precision = precision
    gpu = Solver(case, device)
    gpu.upload(mesh)
    gpu.set_state(u0)
    gpu.run(3, case.tau)
    gpu.sync()
    gpu.set_state(u0)
    gpu.reset_stats()
    gpu.set_timing(True)
    ms = gpu.time_run(steps, case.tau)
    gpu.set_timing(False)
    _, kms = gpu.kernel_stats()
    u = gpu.get_state()
    gpu.close()
    return ms, kms, u


def run_flame(args, device: int) -> dict:
    """Reacting 2-species Navier-Stokes (viscous terms, species diffusion,
    Arrhenius chemistry every stage): DOF-updates/s of the FP64 step and of
    the mixed form (p2 only), the mixed form's error against FP64."""
    from charm_3d_gb300 import synthetic
    from charm_3d_gb300.solver import Forest
    case = synthetic("flame", level=args.flame_level, p_order=args.flame_order)
    mesh = Forest(case).flatten()
    u0 = case.initial_state(mesh.center)
    E, V, B = mesh.n_elem, case.n_var, case.n_basis
    dofs = E * V * B * STAGES * args.flame_steps
    ms, kms, u = _flame_run(case, mesh, u0, args.flame_steps, device, "FP64")
    names = ["face (convective + viscous)", "cell", "limiter", "chemistry, diffusion coefficients, lifting, viscous volume"]
    out = {"workload": f"reacting 2-species NS, unit cube level {args.flame_level} ({E} hex), p{args.flame_order} "
                       f"({B} basis functions, {'27/9' if B == 10 else '8/6'}-point rules), HLLC, MIX EOS, "
                       f"Sutherland mu/kappa, species diffusion, A->B Arrhenius",
           "value": dofs / (ms * 1e-3), "unit": UNIT, "dtype": "f64",
           "ms_per_step": ms / args.flame_steps, "steps": args.flame_steps,
           "kernel_share": {n: float(kms[i] / kms.sum()) for i, n in enumerate(names)},
           "finite": bool(np.isfinite(u).all())}
    if B != 10:
        out["mixed"] = "not built for the viscous/reacting terms at p1 (FP64 only)"
        return out
    ms32, kms32, u32 = _flame_run(case, mesh, u0, args.flame_steps, device, "MIXED")
    rho = lambda x: x[4:V].sum(axis=0)
    # reference-box mass matrix of the 10 Taylor functions (3-point Gauss per
    # axis): the L2 norm of a p2 field on the uniform mesh is sqrt(sum c^T M c)
    gx, gw = np.array([-0.5 * np.sqrt(0.6), 0.0, 0.5 * np.sqrt(0.6)]), np.array([5.0, 8.0, 5.0]) / 18.0
    X, Y, Z = [a.ravel() for a in np.meshgrid(gx, gx, gx, indexing="ij")]
    W = (gw[:, None, None] * gw[None, :, None] * gw[None, None, :]).ravel()
    P = np.stack([np.ones_like(X), X, Y, Z, X * X, Y * Y, Z * Z, X * Y, X * Z, Y * Z])
    M = (P * W) @ P.T

    def field_l2(a, b):
        d, r = (a - b).reshape(-1, B, E), b.reshape(-1, B, E)
        return float(np.sqrt(np.einsum("vke,kl,vle->", d, M, d) / np.einsum("vke,kl,vle->", r, M, r)))

    def mass(x):   # cell mean of a p2 field on a box: c0 + (c4 + c5 + c6) / 12
        vol = np.prod([mesh.tree_len[d] * 2.0 ** (-mesh.level.astype(np.float64)) for d in range(3)], axis=0)
        r = rho(x)
        return float((vol * (r[0] + (r[4] + r[5] + r[6]) / 12.0)).sum())

    out["mixed"] = {"dtype": "f32 residual, f32 hi/lo state, f64 chemistry",
                    "value": dofs / (ms32 * 1e-3), "ms_per_step": ms32 / args.flame_steps,
                    "speedup_vs_fp64": ms / ms32,
                    "kernel_share": {n: float(kms32[i] / kms32.sum()) for i, n in enumerate(names)},
                    "rel_l2_density_vs_fp64": field_l2(rho(u32), rho(u)),
                    "rel_l2_state_vs_fp64": field_l2(u32, u),
                    "norm": "L2 of the fields over the domain (coefficients weighted by the mass matrix)",
                    "rel_l2_density_coefficients_vs_fp64": float(np.linalg.norm(rho(u32) - rho(u)) /
                                                                 np.linalg.norm(rho(u))),
                    "total_mass_vs_fp64": abs(mass(u32) - mass(u)) / mass(u),
                    "finite": bool(np.isfinite(u32).all())}
    return out


def _blast_run(case, steps: int, device: int, precision: str, relative: float = 0.0):
    """The AMR time loop of charm_model_ns_timestep_single on the GPU: the
    reference criterion (charm_gpu_refine_flags; or, with relative > 0, the
    configuration's |grad rho| h / rho > relative, charm_gpu_refine_flags_relative)
    and the host octree's adapt with projection every refine_period steps,
    then upload and continue."""
    from charm_3d_gb300.solver import Forest, Solver
    case.precision = precision
    forest = Forest(case)
    mesh = forest.flatten()
    u = case.initial_state(mesh.center)
    mass0 = _mass(mesh, u)
    gpu = Solver(case, device)
    gpu.upload(mesh)
    gpu.set_state(u)
    dev_ms, dofs, t_adapt, step = 0.0, 0, 0.0, 0
    parts = {"flags_s": 0.0, "plan_s": 0.0, "flatten_s": 0.0, "upload_s": 0.0}
    t0 = time.perf_counter()
    while step < steps:
        if step and step % case.refine_period == 0:
            # the state stays on the device: the host plans the adapt from the
            # gradient estimate and the densities, the device projects
            ta = time.perf_counter()
            if relative > 0.0:
                flags, _ = gpu.refine_flags_relative(relative, True)
                tb = time.perf_counter()
                _, plan = forest.adapt_plan_flags(flags, case.min_level, case.max_level)
            else:
                _, grad = gpu.refine_flags(case.max_err)
                rho = gpu.density_means()
                tb = time.perf_counter()
                _, plan = forest.adapt_plan(grad, rho, case.max_err, case.min_level, case.max_level)
            tc = time.perf_counter()
            mesh = forest.flatten()
            td = time.perf_counter()
            gpu.adapt_upload(plan, mesh)
            te = time.perf_counter()
            parts["flags_s"] += tb - ta
            parts["plan_s"] += tc - tb
            parts["flatten_s"] += td - tc
            parts["upload_s"] += te - td
            t_adapt += te - ta
        n = min(case.refine_period - step % case.refine_period, steps - step)
        dev_ms += gpu.time_run(n, case.tau)
        dofs += dof_per_step(mesh.n_elem, case.n_var) * n
        step += n
    gpu.sync()
    wall = time.perf_counter() - t0
    u = gpu.get_state()
    gpu.close()
    return forest, mesh, u, dev_ms, dofs, wall, t_adapt, (_mass(mesh, u) - mass0) / mass0, parts


def _mass(mesh, u) -> float:
    """Total mass: density means times leaf volumes."""
    vol = np.prod([np.asarray(mesh.tree_len[d]) * 2.0 ** (-mesh.level.astype(np.float64)) for d in range(3)], axis=0)
    return float((u[4:, 0].sum(axis=0) * vol).sum())


def _shock_radius(mesh, u, gam):
    """Largest centre distance from the blast centre where p > 2 x ambient."""
    r = np.sqrt(((mesh.center - 0.5) ** 2).sum(axis=0))
    rho = u[4:, 0].sum(axis=0)
    vel = u[:3, 0] / rho
    p = (u[3, 0] - 0.5 * rho * (vel ** 2).sum(axis=0)) * (gam - 1.0)
    hot = p > 0.2
    return float(r[hot].max()) if hot.any() else 0.0


def run_blast(args, device: int, relative: float = 0.0) -> dict:
    """Spherical blast on AMR (base level 5, max 8, refine every 10 steps),
    HLLC + BJ limiter: FP64 and the mixed form on the same loop; the
    reference's refine criterion, or with relative > 0 the configuration's
    |grad rho| h / rho > relative per cell."""
    from charm_3d_gb300 import synthetic
    crit = (f"|grad rho| h / rho > {relative} per cell (coarsen below half of it)" if relative > 0.0
            else "reference refine criterion")
    out = {"workload": f"blast p=1 in r<0.1, p=0.1 outside, rho=1 +-1% noise; levels 5..8, {crit} "
                       f"every 10 steps, HLLC, BJ limiter, {args.blast_steps} steps"}
    res = {}
    for prec in ("FP64", "MIXED"):
        case = synthetic("blast")
        _, gam = case.gas_constants()
        forest, mesh, u, dev_ms, dofs, wall, t_adapt, drift, parts = _blast_run(case, args.blast_steps, device, prec,
                                                                                relative)
        q, lv = forest.leaves()
        res[prec] = (q, lv, u, mesh)
        out[prec.lower()] = {"value": dofs / (dev_ms * 1e-3), "unit": UNIT, "device_ms": dev_ms,
                             "e2e_dof_updates_per_s": dofs / wall, "wall_s": wall, "adapt_s": t_adapt,
                             "adapt_parts_s": parts,
                             "final_elements": int(mesh.n_elem), "levels": [int(lv.min()), int(lv.max())],
                             "shock_radius": _shock_radius(mesh, u, gam), "mass_drift": drift,
                             "finite": bool(np.isfinite(u).all())}
    q0, l0, u0, m0 = res["FP64"]
    q1, l1, u1, _ = res["MIXED"]
    same = q0.shape == q1.shape and np.array_equal(q0, q1) and np.array_equal(l0, l1)
    out["same_mesh"] = bool(same)
    if same:
        rho0, rho1 = u0[4:].sum(axis=0), u1[4:].sum(axis=0)
        out["rel_l2_density_mixed_vs_fp64"] = float(np.linalg.norm(rho1 - rho0) / np.linalg.norm(rho0))
    out["speedup_mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def run_hex(args, device: int) -> dict:
    """The reference's sample case (samples/klin_amr: Euler, HLLC, BJ,
    inlet / outlet / slip walls) on its 800-hexahedron ramp geometry, the
    trees refined uniformly to --hex-level, on the general-hexahedron
    kernels (FP64): device time of --hex-steps steps, kernel shares, and
    the state against the oracle after 10 steps at level 0."""
    from charm_3d_gb300.hexmesh import ramp_channel
    from charm_3d_gb300.solver import Solver
    from oracle.port import Port
    case, _, mesh, u0 = ramp_channel(args.hex_level, 10)
    g = Solver(case, device)
    g.upload(mesh)
    g.set_state(u0)
    g.run(args.warmup, case.tau)
    g.sync()
    g.set_state(u0)
    g.reset_stats()
    g.set_timing(True)
    ms = g.time_run(args.hex_steps, case.tau)
    g.set_timing(False)
    n_l, k_ms = g.kernel_stats()
    u = g.get_state()
    g.close()
    E, V = mesh.n_elem, case.n_var
    # parity on the sample's own size: 10 steps, GPU vs oracle
    c0, _, m0, v0 = ramp_channel(0, 10)
    gp = Solver(c0, device)
    gp.upload(m0)
    gp.set_state(v0)
    gp.run(10, c0.tau)
    gp.sync()
    port = Port(c0.config(), m0)
    port.set_state(v0)
    port.run(10, c0.tau)
    a, b = gp.get_state(), port.get_state()
    gp.close()
    names = ["face", "cell", "limiter", "other"]
    # Euler model: one stage per step
    dofs = E * V * 4 * args.hex_steps
    return {"workload": f"samples/klin_amr geometry (800 trilinear hexahedra, ramp 10 deg) at level {args.hex_level} "
                        f"({E} elements), Euler, HLLC, BJ, inlet/outlet/slip, FP64, forward Euler steps",
            "value": dofs / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / args.hex_steps, "elements": E,
            "kernel_share": {n: float(k_ms[i] / k_ms.sum()) for i, n in enumerate(names)},
            "finite": bool(np.isfinite(u).all()),
            "parity": {"oracle_rel_l2": float(np.linalg.norm(a - b) / np.linalg.norm(b)), "elements": int(m0.n_elem),
                       "steps": 10}}


def run_tc(args) -> dict:
    """The p2 basis contraction of config 4 (64^3 = 262,144 elements, 6
    variables, 10 coefficients at 27 cell Gauss points) on the tensor cores
    (tcgen05, 3-term BF16 splits, six products, FP32 accumulation) and on
    FP32 FMAs: time per launch (CUDA events, median of the event-timed
    repetitions) and the largest difference of the two."""
    import ctypes as C
    from charm_3d_gb300 import abi
    lib = abi.load()
    E, V = 64 ** 3, 6
    rng = np.random.default_rng(4)
    coef = (rng.normal(size=(V, 10, E)) * 0.1 + np.eye(1, 10)[0][None, :, None]).astype(np.float32)
    out = {"workload": f"p2 basis at the 27 cell Gauss points, {E} elements x {V} variables "
                       f"(interpolation of the p2 cell stage; reduced to one number per element)"}
    sums, vals = {}, {}
    for method, name in ((0, "fma"), (1, "tcgen05")):
        s = np.empty(E)
        v = np.empty((E, V, 27), np.float32)
        ms = C.c_double()
        rc = lib.charm_gpu_p2_interp(method, E, V, coef.ctypes.data, s.ctypes.data, v.ctypes.data,
                                     args.tc_reps, C.byref(ms))
        if rc != 0:
            out[name] = {"error": lib.charm_gpu_last_error().decode()}
            continue
        sums[name], vals[name] = s, v
        out[name] = {"ms": ms.value, "elements_per_s": E / (ms.value * 1e-3)}
    if len(vals) == 2:
        out["tcgen05_over_fma_time"] = out["tcgen05"]["ms"] / out["fma"]["ms"]
        out["max_rel_diff_values"] = float(np.abs(vals["tcgen05"] - vals["fma"]).max() / np.abs(vals["fma"]).max())
    return out


def probe(abi, device: int, which: int) -> float | None:
    import ctypes as C
    lib = abi.load()
    v = C.c_double()
    return v.value if lib.charm_gpu_probe_peak(device, which, C.byref(v)) == 0 else None


# ---------------------------------------------------------------------------
# distributed plumbing (replicas; only barrier and max-reduce of times)
# ---------------------------------------------------------------------------

_DIST = {"on": False}


def init_dist(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        gpu = torch.cuda.is_available() and args.impl != "reference"
        if gpu:
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if gpu else "gloo")
        _DIST["on"] = True
    return rank, world, local


def barrier(world: int):
    if world > 1 and _DIST["on"]:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world > 1 and _DIST["on"]:
        import torch
        import torch.distributed as dist
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return x


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--level", type=int, default=7)
    ap.add_argument("--cpu-level", type=int, default=5)
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="--impl reference: seconds per process")
    ap.add_argument("--parity-steps", type=int, default=20,
                    help="oracle steps on the level --cpu-level sample (cpu_baseline and parity; 0 skips both)")
    ap.add_argument("--brick", type=int, default=1, help="trees along x (profiling sizes)")
    ap.add_argument("--only", default="both",
                    choices=["both", "fp64", "mixed", "dw", "adjoint", "flame", "blast", "tc", "hex"])
    ap.add_argument("--blast-steps", type=int, default=200, help="0 skips the AMR blast leg")
    ap.add_argument("--flame-level", type=int, default=6)
    ap.add_argument("--flame-order", type=int, default=2, choices=[1, 2], help="basis order of the reacting leg")
    ap.add_argument("--flame-steps", type=int, default=5, help="0 skips the reacting-NS leg")
    ap.add_argument("--adjoint-level", type=int, default=6)
    ap.add_argument("--adjoint-box", default="4,6", help="J = integral of p over [lo,hi]^3 (lo,hi)")
    ap.add_argument("--adjoint-steps", type=int, default=200, help="0 skips the adjoint leg")
    ap.add_argument("--adjoint-snapshots", type=int, default=0,
                    help="checkpoint buffers (0: every stage state of the run, 3 per step)")
    ap.add_argument("--adjoint-fd", type=int, default=16, help="finite-difference directions")
    ap.add_argument("--adjoint-revolve-snapshots", type=int, default=20,
                    help="checkpoints of the memory-bounded adjoint timing (0 skips it)")
    ap.add_argument("--adjoint-fd-eps", type=float, default=1e-6, help="central-difference step")
    ap.add_argument("--tc-reps", type=int, default=20, help="timed launches of the p2 contraction leg (0 skips it)")
    ap.add_argument("--hex-level", type=int, default=3, help="uniform level of the sample-geometry leg")
    ap.add_argument("--hex-steps", type=int, default=20, help="timed steps of the sample-geometry leg (0 skips it)")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-dw", action="store_true", help="skip the double-word form's leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        if rank != 0:
            return
        cores = os.cpu_count() or 1
        res = cpu_baseline(args.cpu_level, max(2.0, args.cpu_seconds / 2), cores)
        out = {"metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
               "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f64", "data": "synthetic (seeded isentropic vortex + 1e-3 density noise)",
               "impl": "reference",
               "config": bench_config(args, args.gpus, 8 ** args.level, 5, 8 ** args.level * 5 * 4 * 8, None),
               "cpu_baseline": res,
               "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
               "note": "reference CPU algorithm = oracle/charm_oracle.c, the C restatement pinned to the "
                       "reference's own sources (the reference's MPI build cannot be built here: no p4est/MPI); "
                       f"each step of the workload is sampled on level {args.cpu_level} (per-element rate)"}
        print(json.dumps(out))
        return

    rank, world, local = init_dist(args)
    if args.only == "adjoint":
        if rank == 0:
            print(json.dumps({"only": "adjoint", "adjoint": run_adjoint(args, local)}))
        return
    if args.only == "blast":
        if rank == 0:
            print(json.dumps({"only": "blast", "blast_amr": run_blast(args, local),
                              "blast_amr_relative": run_blast(args, local, relative=0.1)}))
        return
    if args.only == "hex":
        if rank == 0:
            print(json.dumps({"only": "hex", "hex_sample": run_hex(args, local)}))
        return
    if args.only == "tc":
        if rank == 0:
            print(json.dumps({"only": "tc", "p2_contraction": run_tc(args)}))
        return
    if args.only == "flame":
        if rank == 0:
            print(json.dumps({"only": "flame", "reacting_ns": run_flame(args, local)}))
        return
    res = run_gpu(args, rank, world, local)
    if rank == 0 and res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
