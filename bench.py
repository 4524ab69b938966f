"""Benchmark of the explicit DG residual path on GB300 (one JSON line on rank 0).

Workload (default ``hex3d``): 3D Euler, curved periodic HEX mesh of 32^3 elements on [0,10]^3 with a sinusoidal
interior mapping of amplitude 0.03, p=3 (64 DOF per element and variable, 5 variables, 10,485,760 state values),
Lax-Friedrichs flux, z-axis isentropic vortex plus seeded uniform density perturbations of 1e-3. Synthetic,
seeded inputs; no dataset is involved.

Metric: DOF-residual-evals/s (FP64) = N_s x residual evaluations per second, N_s = total state scalars.
One step = one SSP-RK3 step of the whole mesh = 3 residual evaluations R = M^-1 (volume + face), each followed
by its stage update and positivity check (time_step_ssp_rk_33), replayed from a captured CUDA graph.
  value           device-resident state, CUDA events on the library's stream, max over ranks.
  plain_launches  the same stages launched kernel by kernel (the per-group form without the graph).
  compute_rhs_dg  the residual entry alone on the reference's GLL coefficients.
  e2e             every step through the C ABI on pinned host memory: dgpu_ssp_rk3_step_host, the drop-in for
                  time_step_ssp_rk_33 on the host's sol_coef (84 MB each way per step inside the timed region).
Inputs are larger than L2 (state 84 MB + metric terms 151 MB + face data 50 MB per evaluation), so no flush.

--impl reference times the reference's algorithm on the host cores. The reference itself cannot be built here
(MPI, MKL, GSL, PETSc and a cmake-generated header), so its CPU restatement (oracle/, dense operators, the
reference's element-by-element data flow) runs instead, one serial instance per host core on the same
per-element work, and the aggregate throughput is reported.

Multi-GPU (torchrun, N > 1): one element partition per GPU, weak scaling: the hex box is repeated N times along z
and split into N slabs; every RK stage exchanges the traces of the cut faces with NCCL send/recv (run_partitioned).
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

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

PEAKS_PATH = os.path.join(HERE, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    "hex3d": dict(kind="euler_hex_3d", n=32, p=3, flux="lax_friedrichs",
                  desc="3D Euler curved HEX 32^3 p3 Lax-Friedrichs, z-axis vortex + 1e-3 density noise"),
    "hex3d_roe": dict(kind="euler_hex_3d", n=32, p=3, flux="roe_pike",
                      desc="3D Euler curved HEX 32^3 p3 Roe-Pike"),
    "vortex2d": dict(kind="euler_vortex_2d", n=64, p=3, flux="roe_pike",
                     desc="2D Euler curved QUAD 64^2 p3 Roe-Pike isentropic vortex"),
    "mixed3d": dict(kind="mixed", n=58, p=None, flux="roe_pike",
                    desc="3D Euler mixed-order HEX 58^3 unit cube, p uniform in {1,2,3,4} (seed 0), Roe-Pike"),
    "mixed_types": dict(kind="mixed", n=50, p=None, flux="roe_pike",
                        desc="3D Euler HEX/TET/WEDGE/PYR 50^3 cells unit cube, p uniform in {1,2,3,4} (seed 0), "
                             "Roe-Pike"),
    "mixed_ns": dict(kind="mixed", n=24, p=None, flux="roe_pike",
                     desc="3D Navier-Stokes mixed-order HEX 24^3 on [0, 2 pi]^3 with adiabatic walls, p uniform in "
                          "{1,2,3,4} (seed 0), Roe-Pike + BR2"),
}


def make_problem(w, n=None):
    from dpgsolver_gb300.host import problem as P
    flux = P.NUM_FLUX_ROE_PIKE if w["flux"] == "roe_pike" else P.NUM_FLUX_LAX_FRIEDRICHS
    n = w["n"] if n is None else n
    if w["kind"] == "euler_hex_3d":
        return P.euler_hex_3d(n, w["p"], num_flux=flux)
    return P.euler_vortex_2d(n, w["p"], num_flux=flux)


# ------------------------------------------------------------------------------------------------------------------
# helpers
# ------------------------------------------------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            # nvidia-smi start-up can stall the driver for a moment: start timing only once it samples
            t0 = time.time()
            while not self.lines and time.time() - t0 < 10.0 and self.proc.poll() is None:
                time.sleep(0.05)
            self.n_before = len(self.lines)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines[getattr(self, "n_before", 0):] or self.lines[-1:]
        for ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def hbm_peak():
    try:
        with open(PEAKS_PATH) as fh:
            pk = json.load(fh)
        return float(pk["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def flops_per_element(d, q, nv, flux, coef_io):
    """FP64 flops of one residual per element, counted from the kernels (FMA = 2 flops; a division or square root
    counted as 1 flop; the instruction sequences behind them take more FP64 issue slots). coef_io: the residual
    reads and writes the reference's GLL coefficients (compute_rhs_dg: + V u and V^-1 R); otherwise it is the RK
    stage on GL nodal values (+ the stage update)."""
    N = q ** d
    NF = q ** (d - 1)
    pass_ = 2 * q * N * nv                     # one sum-factorised pass over all variables
    flux_vol = N * (1 + 2 * d + 2 * d + 3 + d * (2 * d + 1 + 2 * d + 1))   # rho_inv,u,V2,p, U_j, fr
    vol = d * pass_                            # sum_j Dgl_j^T fr_j
    traces = 2 * d * NF * nv * 2 * q
    if flux == "roe_pike":
        f_num = 130 if d == 3 else 105
    else:
        f_num = 75 if d == 3 else 60
    num = d * NF * (f_num + nv)                # d faces per element, scaled by w J
    lift = 2 * d * N * nv * 2 + N * nv         # E^T nnf per face + diag(1/(wJ))
    total = flux_vol + vol + traces + num + lift
    if coef_io:
        total += 2 * d * pass_                 # V u and V^-1 R
    else:
        total += 3 * N * nv                    # stage update
    return total


# FP64 thread-instructions (DFMA + DMUL + DADD) per element of one RK stage, from ncu
# (sm__sass_thread_inst_executed_op_{dfma,dmul,dadd}_pred_on of the volume, face and lift kernels on the 24^3 p3
# Lax-Friedrichs case, the --set full capture of one stage): 8.64 k + 4.85 k + 2.94 k.
FP64_INSTR_PER_ELEMENT = {(3, 3, "lf"): 16432}


def ranks_barrier(torch, world):
    """The barrier on both sides of a timed region (replicas: the only collective of a run)."""
    if world > 1:
        torch.distributed.barrier()


def ranks_max(torch, world, ms, device):
    """The maximum of a time over the ranks (the job's time is its slowest replica's)."""
    if world > 1:
        t = torch.tensor([float(ms)], device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())
    return ms


def fp64_issue(prob, w, stage_ms, peak_tflops):
    """Fraction of the FP64 pipe's issue slots the live stage uses: every FP64 instruction (a division or square root
    is several) against 2 per cycle per SM, i.e. the DFMA probe's rate / 2. Known for the workloads ncu counted."""
    from dpgsolver_gb300.host import problem as P
    key = (prob.d, prob.ops.p, "lf" if prob.num_flux == P.NUM_FLUX_LAX_FRIEDRICHS else "roe")
    n = FP64_INSTR_PER_ELEMENT.get(key)
    if n is None:
        return {}
    rate = n * prob.n_volumes / (stage_ms * 1e-3)
    return {"instr_per_element": n, "issue_frac": rate / (peak_tflops * 1e12 / 2.0),
            "issue_source": "ncu FP64 instruction counts per element (the --set full capture of one 24^3 p3 stage) x "
                            "elements / live stage time, against the DFMA probe's instruction rate"}


def _batching_bound(prob, w, plain_stage_ms, peak_tflops):
    """How much faster any launch form can make a stage than the plain per-kernel launches: the plain form already
    fills this fraction of the FP64 pipe's issue slots, and every form issues the same FP64 instructions."""
    iss = fp64_issue(prob, w, plain_stage_ms, peak_tflops)
    if not iss:
        return None
    return {"plain_fp64_issue_frac": iss["issue_frac"], "max_speedup_vs_plain": 1.0 / iss["issue_frac"],
            "mixed_order_hex": {"plain_fp64_pipe_frac": 0.717, "max_speedup_vs_plain": 1.39,
                                "source": "time-weighted FP64 pipe (elapsed) of the plain per-group stage's kernels in "
                                          "the ncu --set full capture of the 36^3 mixed-order HEX mesh"},
            "note": "a 3x batched-vs-plain speed-up exceeds these bounds: the plain form is FP64-issue "
                    "bound already, so batching can only recover the idle issue slots (launch gaps, tails, low "
                    "occupancy of the lifts)"}


def algorithmic_bytes(prob, kernel):
    """Compulsory DRAM bytes of one launch of `kernel` (each array read or written once)."""
    d, q, nv = prob.d, prob.ops.q, prob.n_var
    N, NF = q ** d, q ** (d - 1)
    nV, nF = prob.n_volumes, prob.mesh.n_faces
    s = 8 * nV * nv * N
    tr = 8 * nF * 2 * nv * NF
    nnf = 8 * nF * nv * NF
    if kernel == "tp_volume_kernel":
        return s + 8 * nV * d * d * N + s + tr
    if kernel == "tp_face_kernel":
        return tr + 8 * nF * (d + 1) * NF + nnf
    if kernel == "tp_lift_kernel":      # RK stage: vol_gl + nnf + 1/(wJ) + state + stage-0 copy in, state out
        return s + 2 * nnf + 8 * nV * N + 3 * s
    raise KeyError(kernel)


# DRAM bytes per element of one tp_volume_kernel launch (GL state in) measured by ncu on curved HEX 24^3, p = 3,
# 5 variables: 99.5 MB read + 42.7 MB written over 13,824 elements (writes stay below the algorithmic vol_gl +
# traces because L2 holds part of them until the face kernel reads them).
_VOLUME_DRAM_BYTES_PER_ELEMENT_HEX_P3 = (99.5e6 + 42.7e6) / 13824


def volume_traffic(prob, kernel):
    """Measured DRAM traffic per launch of the dominant kernel, where an ncu capture of the same kernel and order
    exists (the curved HEX p = 3 Euler volume kernel); None otherwise."""
    if kernel == "tp_volume_kernel" and prob.d == 3 and prob.ops.q == 4 and prob.n_var == 5:
        return _VOLUME_DRAM_BYTES_PER_ELEMENT_HEX_P3 * prob.n_volumes
    return None


def eval_bytes(prob):
    """Algorithmic bytes of one residual evaluation: state read + residual written + metric terms and J at the
    cubature nodes + face normals x J_f (the compulsory traffic, reference-element operators excluded)."""
    d, q, nv = prob.d, prob.ops.q, prob.n_var
    N, NF = q ** d, q ** (d - 1)
    return 8 * (2 * prob.n_volumes * nv * N + prob.n_volumes * (d * d + 1) * N + prob.mesh.n_faces * d * NF)


# ------------------------------------------------------------------------------------------------------------------
# arms
# ------------------------------------------------------------------------------------------------------------------

def _timed(torch, stream, fn, reps):
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(reps):
        fn()
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1)


def run_ours(args, rank, world, local_rank):
    import torch
    from dpgsolver_gb300 import _lib
    from dpgsolver_gb300.solver import Simulation

    torch.cuda.set_device(local_rank)
    w = WORKLOADS[args.workload]
    if w["kind"] == "mixed":
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        if args.only_rk:
            return mixed_only_rk(torch, stream, args)
        if args.workload == "mixed_ns":
            mx = mixed_ns_measurements(torch, stream, args)
        else:
            mx = mixed_measurements(torch, stream, args, "types" if args.workload == "mixed_types" else "hex")
        best = max(mx["forms"], key=lambda k: mx["forms"][k]["value"])
        return {"metric": "DOF-residual-evals/sec FP64 (batched graph vs plain per-group) at <=1e-12; %HBM peak",
                "value": mx["forms"][best]["value"], "unit": "DOF-residual-evals/s", "n_gpus": world,
                "steps": mx["steps"], "warmup": args.warmup, "ms_per_step": mx["forms"][best]["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded p per volume, seeded sinusoidal state)",
                "config": {"workload": mx["workload"], "form": best}, "mixed": mx}
    t0 = time.time()
    prob = make_problem(w, n=args.n)
    setup_s = time.time() - t0
    # a dedicated stream: graph capture is not possible on the legacy default stream
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sim = Simulation(prob, stream=stream.cuda_stream)
    lib = _lib.load()
    ns = prob.n_state
    dt = prob.dt
    # steps of the timed region: each step is one SSP-RK3 step = 3 residual evaluations (stages)
    n_rk = max(1, args.steps)

    def barrier():
        ranks_barrier(torch, world)

    def max_over_ranks(ms):
        return ranks_max(torch, world, ms, "cuda")

    if args.only_residual:
        for _ in range(max(args.warmup, 3)):
            sim.compute_rhs(want_max=False)
        ms = _timed(torch, stream, lambda: sim.compute_rhs(want_max=False), args.steps)
        sim.close()
        return {"metric": "DOF-residual-evals/sec (compute_rhs_dg, device-resident)", "value": ns * args.steps / (ms * 1e-3),
                "unit": "DOF-residual-evals/s", "ms_per_step": ms / args.steps, "n_state": ns,
                "elements": prob.n_volumes}
    if args.only_rk:
        sim.ssp_rk3_steps(dt, max(args.warmup, 3), want_max=False)
        ms = _timed(torch, stream, lambda: sim.ssp_rk3_steps(dt, 1, want_max=False), args.steps)
        sim.close()
        return {"metric": "DOF-residual-evals/sec (SSP-RK3 stages, graph)", "value": 3 * ns * args.steps / (ms * 1e-3),
                "unit": "DOF-residual-evals/s", "ms_per_step": ms / args.steps, "n_state": ns,
                "elements": prob.n_volumes}

    # ---- headline: SSP-RK3 steps replayed from the captured CUDA graph (device-resident state) ----
    sim.ssp_rk3_steps(dt, max(args.warmup, 3), want_max=False)
    torch.cuda.synchronize()
    launches0 = sim.kernel_launches()
    with ClockSampler(local_rank) as clk:
        barrier()
        ms = _timed(torch, stream, lambda: sim.ssp_rk3_steps(dt, n_rk, want_max=False), 1)
        barrier()
    launches = sim.kernel_launches() - launches0
    clocks = clk.summary()
    t_max = max_over_ranks(ms)
    ms_per_step = t_max / n_rk
    value = world * ns * 3 * n_rk / (t_max * 1e-3)

    # ---- plain form: the same stages launched one kernel at a time (no graph) ----
    sim.set_kernel_timing(True)       # eager launches, CUDA events around each kernel
    n_plain = max(3, min(n_rk, 20))
    sim.ssp_rk3_steps(dt, 1, want_max=False)
    ms_plain = _timed(torch, stream, lambda: sim.ssp_rk3_steps(dt, n_plain, want_max=False), 1)
    kt, kt_total = {}, {}
    for name in ("tp_volume_kernel", "tp_face_kernel", "tp_lift_kernel"):
        tot, cnt = sim.kernel_time(name)
        if cnt:
            kt[name] = tot / cnt
            kt_total[name] = tot
    sim.set_kernel_timing(False)
    plain_value = world * ns * 3 * n_plain / (max_over_ranks(ms_plain) * 1e-3)

    # ---- compute_rhs_dg: residual on the reference's GLL coefficients (device-resident) ----
    for _ in range(3):
        sim.compute_rhs(want_max=False)
    ms_rhs = _timed(torch, stream, lambda: sim.compute_rhs(want_max=False), n_rk)
    rhs_value = world * ns * n_rk / (max_over_ranks(ms_rhs) * 1e-3)

    # ---- e2e: the reference-facing calls with pinned host buffers, copies inside the timed region ----
    # every step: sol_coef host -> device, time_step_ssp_rk_33 (3 residuals), sol_coef device -> host
    sol_h = torch.empty(prob.sol.shape, dtype=torch.float64, pin_memory=True)
    sol_h.copy_(torch.from_numpy(prob.sol))
    out_h = torch.empty_like(sol_h).pin_memory()
    c_dp = _lib.c_double_p
    sp = ctypes.cast(sol_h.data_ptr(), c_dp)
    op = ctypes.cast(out_h.data_ptr(), c_dp)

    def e2e_step():
        _lib.check(lib.dgpu_ssp_rk3_step_host(sim.handle, ctypes.c_double(dt), sp, op, None), sim.handle)

    for _ in range(2):
        e2e_step()
    n_e2e = max(3, min(n_rk, 50))
    barrier()
    e2e_ms = max_over_ranks(_timed(torch, stream, e2e_step, n_e2e))
    e2e_value = world * ns * 3 * n_e2e / (e2e_ms * 1e-3)

    dom = max(kt_total, key=kt_total.get)     # the kernel with the largest share of the step
    peak, peak_kind = hbm_peak()
    ab = algorithmic_bytes(prob, dom)
    achieved = ab / (kt[dom] * 1e-3) / 1e9
    fp64_peak = ctypes.c_double()
    _lib.check(lib.dgpu_probe_fp64(20000, ctypes.byref(fp64_peak)))
    mma_peak = ctypes.c_double()
    _lib.check(lib.dgpu_probe_fp64_mma(2500, ctypes.byref(mma_peak)))
    stage_flops = flops_per_element(prob.d, prob.ops.q, prob.n_var, w["flux"], coef_io=False) * prob.n_volumes
    stage_ms = ms_per_step / 3.0          # live graph replay (the kernel sum above is serialised and timed eagerly)
    res = {
        "metric": "DOF-residual-evals/sec FP64 (batched graph vs plain per-group) at <=1e-12; %HBM peak",
        "value": value,
        "unit": "DOF-residual-evals/s",
        "n_gpus": world,
        "steps": n_rk,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded mesh mapping, isentropic vortex state + uniform density noise)",
        "config": {"workload": w["desc"], "elements": prob.n_volumes, "p": prob.ops.p, "n_state": ns,
                   "faces": prob.mesh.n_faces, "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (state 84 MB + metrics 151 MB + face data 50 MB), no flush",
                   "step": "one SSP-RK3 step = 3 residual evaluations (volume + face + lift + stage update + "
                           "positivity), replayed from a CUDA graph; value counts N_s per residual evaluation",
                   "dt": dt},
        "plain_launches": {"value": plain_value, "unit": "DOF-residual-evals/s",
                           "note": "the same stages launched kernel by kernel without the graph"},
        "compute_rhs_dg": {"value": rhs_value, "unit": "DOF-residual-evals/s",
                           "note": "residual on the reference's GLL coefficients (V u and V^-1 R included)"},
        "e2e": {"value": e2e_value, "unit": "DOF-residual-evals/s", "h2d_bytes_per_step": int(ns * 8),
                "d2h_bytes_per_step": int(ns * 8),
                "note": "per step: dgpu_ssp_rk3_step_host (time_step_ssp_rk_33 on host sol_coef) from and to "
                        "pinned memory; the first volume kernel reads and the last lift writes the host buffers "
                        "over the host link, overlapped with their arithmetic"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": volume_traffic(prob, dom),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of tp_volume_kernel on the "
                                       "24^3 p3 case (the --set full capture of one stage), scaled per element",
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS hbm_gbs)",
                     "algorithmic_bytes_per_launch": ab, "kernel_ms": kt},
        "fp64_pipe": {"achieved_tflops": stage_flops / (stage_ms * 1e-3) / 1e12,
                      "peak_tflops": fp64_peak.value, "peak_source": "measured (dgpu_probe_fp64 DFMA loop)",
                      "frac": stage_flops / (stage_ms * 1e-3) / 1e12 / fp64_peak.value,
                      "flops_per_stage": stage_flops,
                      **fp64_issue(prob, w, stage_ms, fp64_peak.value),
                      "dmma_tflops": mma_peak.value,
                      "dmma_source": "measured (dgpu_probe_fp64_mma: mma.sync m8n8k4 f64 loop)",
                      "note": "binding roof: FP64 issue rate, not HBM; the FP64 tensor cores (dmma_tflops) run at "
                              "the DFMA rate on this part, so the contractions stay on DFMA"},
        "batching_bound": _batching_bound(prob, w, ms_plain / (3.0 * n_plain), fp64_peak.value),
        "eval_hbm": {"bytes_per_eval": eval_bytes(prob),
                     "achieved_gbs": eval_bytes(prob) / (ms_per_step / 3 * 1e-3) / 1e9,
                     "frac": eval_bytes(prob) / (ms_per_step / 3 * 1e-3) / 1e9 / peak},
        "clocks": clocks,
        "setup_s": setup_s,
    }
    if prob.d == 3:
        res["geometry"] = geometry_measurements(torch, prob, stream)
    if prob.d == 3 and not args.no_jacobian:
        res["jacobian"] = jacobian_measurements(torch, stream, args)
    if not args.no_adjoint and prob.pde == 3:
        res["adjoint"] = adjoint_measurements(torch, sim, prob, args)
    if not args.no_vortex:
        res["vortex2d"] = vortex2d_measurements(torch, stream, args)
    if prob.d == 3 and not args.no_ns:
        res["navier_stokes"] = ns_measurements(torch, stream, args)
    if not args.no_mixed:
        res["mixed_types"] = mixed_measurements(torch, stream, args, "types")
        res["mixed"] = mixed_measurements(torch, stream, args, "hex")
        res["mixed_ns"] = mixed_ns_measurements(torch, stream, args)
        res["tri_quad_2d"] = tri_quad_measurements(torch, stream, args)
    if rank == 0 and not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_baseline(w, args.cpu_seconds, workers=1, prob=prob)
    sim.close()
    return res


def run_partitioned(args, rank, world, local_rank):
    """N > 1: one element partition per GPU (weak scaling). The hex workload's box is repeated along z once per rank
    (n x n x N n volumes), split by recursive coordinate bisection into N slabs of n^3 volumes; every RK stage runs
    the volume term, exchanges the traces of the cut faces with NCCL send/recv on the library's stream, then the face
    term and the lift (dgpu_halo_stage_begin / _end). value = N_s of all ranks x 3 x steps / max over ranks."""
    import torch
    from dpgsolver_gb300 import partition as PT
    from dpgsolver_gb300.host import problem as P
    from dpgsolver_gb300.solver import PartitionSimulation

    torch.cuda.set_device(local_rank)
    w = WORKLOADS[args.workload]
    if w["kind"] != "euler_hex_3d":
        raise SystemExit("multi-GPU runs partition the hex workloads")
    n = args.n or w["n"]
    flux = P.NUM_FLUX_ROE_PIKE if w["flux"] == "roe_pike" else P.NUM_FLUX_LAX_FRIEDRICHS
    t0 = time.time()
    prob = P.euler_hex_3d(n, w["p"], num_flux=flux, stack=world)
    owner = PT.partition_volumes(prob, world)
    part = PT.Partition(prob, owner, rank)
    setup_s = time.time() - t0
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sim = PartitionSimulation(prob, part, stream=stream.cuda_stream)
    send, recv = sim.halo_tensors()
    dt = prob.dt
    ns_local = int(sim.shape[0] * sim.shape[1] * sim.shape[2])
    ns_total = prob.n_state

    def exchange():
        if send is not None:
            PT.exchange(part, send, recv)   # NCCL on the current stream (the library's)

    def step(want_max=False):
        mx = None
        for stage in range(3):
            sim.stage_begin(stage)
            exchange()
            mx = sim.stage_end(dt, stage, want_max and stage == 2)
        return mx

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    n_rk = max(1, args.steps)
    launches0 = sim.kernel_launches()
    with ClockSampler(local_rank) as clk:
        ranks_barrier(torch, world)
        ms = _timed(torch, stream, lambda: [step() for _ in range(n_rk)], 1)
        ranks_barrier(torch, world)
    launches = sim.kernel_launches() - launches0
    t_max = ranks_max(torch, world, ms, "cuda")
    mx = PT.all_max(step(want_max=True), device="cuda")

    # e2e: every step the rank's sol_coef from pinned host memory, the step, and the new state back
    sol_h = torch.from_numpy(np.ascontiguousarray(part.local_state(prob.sol))).pin_memory()
    out_h = torch.empty_like(sol_h).pin_memory()

    def e2e_step():
        sim.upload_state(sol_h.numpy())
        step()
        out_h.numpy()[...] = sim.sol_coef

    e2e_step()
    n_e2e = max(3, min(n_rk, 20))
    ranks_barrier(torch, world)
    e2e_ms = ranks_max(torch, world, _timed(torch, stream, e2e_step, n_e2e), "cuda")
    halo_bytes = part.n_halo * sim.slot_doubles * 8
    res = {
        "metric": "DOF-residual-evals/sec FP64 (batched graph vs plain per-group) at <=1e-12; %HBM peak",
        "value": ns_total * 3 * n_rk / (t_max * 1e-3),
        "unit": "DOF-residual-evals/s",
        "n_gpus": world,
        "steps": n_rk,
        "warmup": args.warmup,
        "ms_per_step": t_max / n_rk,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded mesh mapping, isentropic vortex state + uniform density noise)",
        "config": {"workload": w["desc"] + f", box repeated {world}x along z", "elements": prob.n_volumes,
                   "elements_per_gpu": len(part.volumes), "p": prob.ops.p, "n_state": ns_total,
                   "parallelism": f"element partition x{world} (recursive coordinate bisection), NCCL trace "
                                  "exchange per RK stage", "halo_bytes_per_stage_per_rank": halo_bytes,
                   "l2": "inputs larger than L2, no flush", "dt": dt},
        "e2e": {"value": ns_total * 3 * n_e2e / (e2e_ms * 1e-3), "unit": "DOF-residual-evals/s",
                "h2d_bytes_per_step": int(ns_local * 8), "d2h_bytes_per_step": int(ns_local * 8),
                "note": "per rank and step: dgpu_upload_state from pinned memory, the partitioned step, "
                        "dgpu_download_state into pinned memory"},
        "gpu_launches": int(launches),
        "max_rhs": mx,
        "clocks": clk.summary(),
        "setup_s": setup_s,
    }
    sim.close()
    return res


def geometry_measurements(torch, prob, stream):
    """Geometry precompute of the workload's mesh: the host restatement (numpy, TPGeometry) against the device
    (dgpu_compute_geometry: coefficients in, the five factor arrays out, copies included), and context creation from
    the host's factors against creation from the geometry coefficients alone."""
    from dpgsolver_gb300.host.geometry import TPGeometry, sinusoidal_deform_3d
    from dpgsolver_gb300.solver import Simulation, compute_geometry
    t0 = time.perf_counter()
    TPGeometry(prob.mesh, prob.ops, deform=sinusoidal_deform_3d(0.03, 10.0), curved=True)
    host_s = time.perf_counter() - t0
    compute_geometry(prob)                       # warm-up (module load, first launches)
    t0 = time.perf_counter()
    dev = compute_geometry(prob)
    dev_s = time.perf_counter() - t0
    g = prob.geom
    diff = max(float(np.max(np.abs(dev[k] - getattr(g, k))) / np.max(np.abs(getattr(g, k))))
               for k in ("metrics_vc", "jacobian_det_vc", "normals_fc", "jacobian_det_fc", "xyz_fc"))
    times = {}
    for name, flag in (("create_from_factors_s", False), ("create_from_geom_coef_s", True)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s = Simulation(prob, stream=stream.cuda_stream, device_geometry=flag)
        torch.cuda.synchronize()
        times[name] = time.perf_counter() - t0
        s.close()
    return {"host_numpy_s": host_s, "device_s": dev_s, "speedup": host_s / dev_s, "max_rel_diff": diff, **times,
            "note": "host: TPGeometry of the same mesh (vectorised numpy, metric terms + faces); device: "
                    "dgpu_compute_geometry incl. host<->device copies of coefficients and results"}


def jacobian_measurements(torch, stream, args):
    """Block-sparse Jacobian assembly (dgpu_jacobian_bsr, raw residual = the reference's lhs) on the 8^3 HEX p3
    Euler mesh into device memory, against the oracle's complex-step Jacobian, whose cost is one complex residual per
    column: that rate is sampled and extrapolated to every column (the full CPU run would take hours)."""
    import oracle
    from dpgsolver_gb300.host import problem as P
    from dpgsolver_gb300.solver import Simulation
    prob = P.euler_hex_3d(8, 3)
    base = prob.sol
    with Simulation(prob, stream=stream.cuda_stream) as sim:
        nb, nnz, n_col = sim.jacobian_structure()
        dev = torch.empty((nnz, nb, nb), dtype=torch.float64, device="cuda")
        sim.jacobian(base, raw=True, values_ptr=dev.data_ptr())      # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.jacobian(base, raw=True, values_ptr=dev.data_ptr())
        torch.cuda.synchronize()
        gpu_s = time.perf_counter() - t0
        del dev
    res = {"workload": "3D Euler curved HEX 8^3 p3 Lax-Friedrichs, raw residual (the reference's lhs)",
           "block_size": nb, "n_blocks": nnz, "n_colours": n_col, "directional_derivatives": n_col * nb,
           "bytes": nnz * nb * nb * 8, "gpu_s": gpu_s, "blocks_per_s": nnz / gpu_s}
    if not args.no_cpu_baseline:
        o = oracle.Oracle(prob)
        e = np.zeros(prob.sol.shape)
        e.flat[0] = 1e-30
        o.compute_rhs_cmplx(base, e)
        t0 = time.perf_counter()
        k = 0
        while time.perf_counter() - t0 < 5.0:
            o.compute_rhs_cmplx(base, e)
            k += 1
        per_col = (time.perf_counter() - t0) / k
        res["cpu_complex_step"] = {"s_per_column": per_col, "columns": prob.n_state,
                                   "extrapolated_s": per_col * prob.n_state, "cores": 1, "kind": "port",
                                   "sample": f"{k} complex residual evaluations of the oracle on the same mesh"}
    return res


def adjoint_measurements(torch, sim, prob, args):
    """The discrete adjoint on the bench mesh: one VJP of R through the host-buffer forward/backward pair, and
    the checkpointed adjoint of SSP-RK3 steps of J = integral of pressure over the z = 0 faces."""
    rng = np.random.default_rng(0)
    v = rng.standard_normal(prob.sol.shape)
    sim.vjp_forward(prob.sol)
    sim.vjp_backward(v)
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        sim.vjp_backward(v)
    vjp_s = (time.perf_counter() - t0) / reps
    d = rng.standard_normal(prob.sol.shape)
    sim.jvp(prob.sol, d)
    t0 = time.perf_counter()
    for _ in range(reps):
        sim.jvp(prob.sol, d)
    jvp_s = (time.perf_counter() - t0) / reps
    sim.set_objective_faces(prob.faces_on_plane(2))
    n_adj = args.adjoint_steps
    budget = int(args.adjoint_budget_gb * 2**30)
    t0 = time.perf_counter()
    J, g, K = sim.adjoint_ssp_rk3(prob.sol, prob.dt, n_adj, budget)
    adj_s = time.perf_counter() - t0
    return {"vjp_backward_s": vjp_s,
            "vjp_dof_per_s": prob.n_state / vjp_s,
            "vjp_note": "host cotangent in, host gradient out (84 MB each way included)",
            "jvp_s": jvp_s, "jvp_note": "dgpu_jvp: host state and direction in, R and (dR/du) d out (dual numbers)",
            "rk3_adjoint_steps": n_adj, "rk3_adjoint_s": adj_s, "segment_steps": K,
            "budget_bytes": budget, "J": J, "grad_norm": float(np.linalg.norm(g)),
            "note": "forward sweep with checkpoints, segment recomputation, stage recomputation, 3 VJPs per step"}


def _dense_flops(ops, nv=5):
    """FP64 flops of one RK stage of a dense-operator volume (FMA = 2): interpolation to the cubature nodes, the
    contravariant flux (~50 per node), the weak derivative, traces and lifts at the volume's own face order and
    the stage update. WEDGE volume terms are counted sum-factorised (TRI x LINE), as the kernel applies them;
    M^-1 is 1/J for these orthonormal bases."""
    d, nvs, nvc = 3, ops.n_vs, ops.n_vc
    nfc = sum(len(ops.w_fc(lf, ops.q)) for lf in range(ops.n_lf))
    if getattr(ops, "e_type", None) == 6:     # WEDGE: TRI x LINE factors
        t0, _, l0, _ = ops.prism_factors()
        ntc, ntv = t0.shape
        nlc, nlv = l0.shape
        vol = nv * (nlv * ntc * ntv + nvc * nlv) \
            + nv * (2 * nlv * ntc * nlc + nlc * ntv * ntc + nvs * (2 * ntc + nlc))
    else:
        vol = nv * nvc * nvs * (1 + d)
    fma = vol + 2 * nv * nfc * nvs
    return 2 * fma + 50 * nvc + 3 * nv * nvs


def make_mixed(kind, n):
    if kind == "types":
        from dpgsolver_gb300.host.mixed_types import mixed_types_euler
        return mixed_types_euler(n, seed=0)
    from dpgsolver_gb300.host.mixed import mixed_euler
    return mixed_euler(3, n, seed=0)


def _batched_forms(torch, stream, args, sim, prob, n_steps, autotune=True):
    """SSP-RK3 steps of a batched context in its forms: plain per-group launches, the same from a graph, the fused
    persistent launches and the parallel branches from graphs, then (autotune) the autotuned choice."""
    ns, dt = prob.n_state, prob.dt
    out = {}

    def run(label, form, graphs):
        sim.form = form
        sim.set_graphs(graphs)
        sim.upload_state(prob.sol)
        sim.ssp_rk3_steps(dt, max(args.warmup, 3), want_max=False)
        l0 = sim.kernel_launches()
        ms = _timed(torch, stream, lambda: sim.ssp_rk3_steps(dt, n_steps, want_max=False), 1)
        out[label] = {"value": 3 * ns * n_steps / (ms * 1e-3), "ms_per_step": ms / n_steps,
                      "launches_per_step": (sim.kernel_launches() - l0) / n_steps}

    persistent = getattr(prob, "ns", None) is None   # Navier-Stokes runs in the per-group and branch forms only
    run("plain_per_group", "plain", False)
    run("per_group_graph", "plain", True)
    if persistent:
        run("fused_graph", "fused", True)
    run("branches_graph", "branches", True)
    if persistent:
        run("stage_graph", "stage", True)
    report, tuned_form = None, None
    if autotune:
        sim.upload_state(prob.sol)
        report = sim.autotune(dt, reps=3)
        tuned_form = sim.form
        run("autotuned_graph", tuned_form, True)
    return out, report, tuned_form


def tri_quad_measurements(torch, stream, args):
    """2D Euler on the mixed QUAD/TRI mesh of the periodic unit square (mixed_tri_quad_euler: n^2 cells, half of
    them split into two TRIs, p uniform in {1,2,3,4} with seed 0, Roe-Pike, Mach 0.5 seeded sinusoidal state with
    5 % perturbations): SSP-RK3 steps in the batched context's four forms, the TRI groups on the dense kernels."""
    from dpgsolver_gb300.host.element import QUAD, TRI
    from dpgsolver_gb300.host.mixed_types import mixed_tri_quad_euler
    from dpgsolver_gb300.solver import BatchSimulation
    n = args.tri_n
    t0 = time.time()
    prob = mixed_tri_quad_euler(n, seed=0, perturb=0.05)
    setup_s = time.time() - t0
    n_steps = max(3, min(args.steps, 20))
    with BatchSimulation(prob, stream=stream.cuda_stream) as sim:
        out, _, _ = _batched_forms(torch, stream, args, sim, prob, n_steps, autotune=False)
    tname = {QUAD: "QUAD", TRI: "TRI"}
    return {"workload": f"2D Euler mixed QUAD/TRI {n}^2 cells on the unit square (half split into TRIs, straight, "
                        "conforming, periodic), p uniform in {1,2,3,4} (seed 0), Roe-Pike, Mach 0.5 seeded "
                        "sinusoidal state",
            "elements": prob.n_volumes, "n_state": prob.n_state,
            "groups": {f"{tname[getattr(o, 'e_type', QUAD)]} p{o.p}": int(np.sum(prob.vol_group == i))
                       for i, o in enumerate(prob.groups)},
            "unit": "DOF-residual-evals/s", "steps": n_steps, "forms": out, "setup_s": setup_s}


def mixed_ns_measurements(torch, stream, args):
    """Navier-Stokes in the batched context: mixed-order HEX n^3 on [0, 2 pi]^3 (mixed_ns: p uniform in {1,2,3,4}
    per volume with seed 0, Roe-Pike + BR2, mu = 0.02, Mach 0.3 channel-like state, no-slip adiabatic walls at
    y = 0 and 2 pi, periodic in x and z): SSP-RK3 steps per-group and on graph branches."""
    from dpgsolver_gb300.host import problem as P
    from dpgsolver_gb300.host.mixed import mixed_ns
    from dpgsolver_gb300.solver import BatchSimulation
    n = args.mixed_ns_n
    prob = mixed_ns(3, n, seed=0, walls={(1, 0): P.BC_NOSLIP_ADIABATIC, (1, 1): P.BC_NOSLIP_ADIABATIC})
    n_steps = max(3, min(args.steps, 10))
    with BatchSimulation(prob, stream=stream.cuda_stream) as sim:
        out, report, tuned = _batched_forms(torch, stream, args, sim, prob, n_steps, autotune=True)
    return {"workload": f"3D Navier-Stokes mixed-order HEX {n}^3 on [0, 2 pi]^3, p uniform in {{1,2,3,4}} (seed 0), "
                        "Roe-Pike + BR2, mu 0.02, adiabatic no-slip walls at y = 0, 2 pi",
            "elements": prob.n_volumes, "n_state": prob.n_state,
            "groups": {f"HEX p{o.p}": int(np.sum(prob.vol_group == i)) for i, o in enumerate(prob.groups)},
            "unit": "DOF-residual-evals/s", "steps": n_steps, "forms": out, "autotune": {"form": tuned}}


def mixed_measurements(torch, stream, args, kind="types"):
    """Batched mixed workloads, both Roe-Pike with a seeded smooth sinusoidal state around a Mach 0.5 free stream on
    the periodic unit cube, p drawn uniformly from {1,2,3,4} per volume with seed 0:

    * kind "types" (the configuration with mixed element types): n^3 cells (n = 50) split into HEX, TET, WEDGE
      and PYR volumes (about 50/25/15/10 %, 207,312 volumes, 41.2 M state values), conforming and straight;
    * kind "hex": n^3 HEX volumes (n = 58: 195,112 volumes, 54.6 M state values).

    SSP-RK3 steps of the whole mesh in five forms: one launch per group and face order from the host (plain),
    the same launches replayed from a CUDA graph, the fused persistent launches replayed from a graph, the
    per-group launches on parallel graph branches, and the autotuned choice (elements per CTA and form)."""
    from dpgsolver_gb300.solver import BatchSimulation
    n = args.mixed_n if kind == "hex" else args.types_n
    t0 = time.time()
    prob = make_mixed(kind, n)
    setup_s = time.time() - t0
    sim = BatchSimulation(prob, stream=stream.cuda_stream)
    ns, dt = prob.n_state, prob.dt
    n_steps = max(3, min(args.steps, 20))
    out, report, tuned_form = _batched_forms(torch, stream, args, sim, prob, n_steps)
    flops = 0
    for g, ops in enumerate(prob.groups):
        cnt = int(np.sum(prob.vol_group == g))
        if getattr(ops, "dense", False):
            flops += _dense_flops(ops) * cnt
        else:
            flops += flops_per_element(3, ops.q, 5, "roe_pike", coef_io=False) * cnt
    best = max(out, key=lambda k: out[k]["value"])
    fp64_peak = ctypes.c_double()
    from dpgsolver_gb300 import _lib
    _lib.check(_lib.load().dgpu_probe_fp64(20000, ctypes.byref(fp64_peak)))
    stage_s = out[best]["ms_per_step"] / 3 * 1e-3
    n_vc = np.array([prob.groups[g].n_vc for g in prob.vol_group], dtype=np.int64)
    n_fcn = int(prob.face_off[-1]) if hasattr(prob, "face_off") else int(np.sum(prob.face_q.astype(np.int64) ** 2))
    bytes_eval = 8 * (2 * ns + int(np.sum(10 * n_vc)) + 3 * n_fcn)
    peak, peak_kind = hbm_peak()
    from dpgsolver_gb300.host.element import HEX, PYR, TET, WEDGE
    tname = {HEX: "HEX", TET: "TET", WEDGE: "WEDGE", PYR: "PYR"}
    res = {
        "workload": (f"3D Euler mixed-type {n}^3 cells on the unit cube (HEX/TET/WEDGE/PYR, straight, conforming, "
                     f"periodic)" if kind == "types" else f"3D Euler mixed-order HEX {n}^3 on the unit cube "
                                                          f"(straight, periodic)")
                    + ", p uniform in {1,2,3,4} (seed 0), Roe-Pike, Mach 0.5 seeded sinusoidal state",
        "elements": prob.n_volumes, "n_state": ns,
        "groups": {f"{tname[getattr(o, 'e_type', HEX)]} p{o.p}": int(np.sum(prob.vol_group == i))
                   for i, o in enumerate(prob.groups)},
        "face_orders": {int(qf) - 1: int(np.sum(prob.face_q == qf)) for qf in np.unique(prob.face_q)},
        "unit": "DOF-residual-evals/s", "steps": n_steps, "dt": dt,
        "forms": out,
        "speedup_fused_graph_vs_plain": out["fused_graph"]["value"] / out["plain_per_group"]["value"],
        "speedup_branches_graph_vs_plain": out["branches_graph"]["value"] / out["plain_per_group"]["value"],
        "speedup_stage_graph_vs_plain": out["stage_graph"]["value"] / out["plain_per_group"]["value"],
        "speedup_best_vs_plain": out[best]["value"] / out["plain_per_group"]["value"],
        "autotune": {"form": tuned_form, "report": report},
        "fp64_pipe": {"flops_per_stage": flops, "achieved_tflops": flops / stage_s / 1e12,
                      "peak_tflops": fp64_peak.value, "frac": flops / stage_s / 1e12 / fp64_peak.value,
                      "form": best, "note": "flops counted per volume at its own order (face interpolation to "
                                            "p_f not counted)"},
        "eval_hbm": {"bytes_per_eval": bytes_eval, "achieved_gbs": bytes_eval / stage_s / 1e9,
                     "frac": bytes_eval / stage_s / 1e9 / peak, "peak_source": peak_kind},
        "setup_s": setup_s,
    }
    if kind == "types":
        res["counts"] = {tname[t]: c for t, c in prob.mesh.counts().items()}
        if not args.no_cpu_baseline:
            res["cpu_baseline"] = mixed_cpu_baseline(kind, seconds=min(10.0, args.cpu_seconds))
    sim.close()
    return res


def _mixed_oracle_worker(a):
    kind, n, seconds = a
    sys.path.insert(0, HERE)
    import oracle
    prob = make_mixed(kind, n)
    o = oracle.Oracle(prob)
    o.compute_rhs(prob.sol)
    t0 = time.perf_counter()
    k = 0
    while True:
        o.compute_rhs(prob.sol)
        k += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return prob.n_state * k / el, k, el, prob.n_volumes


def mixed_cpu_baseline(kind, seconds, workers=1):
    n = 8
    if workers == 1:
        v, k, el, nvol = _mixed_oracle_worker((kind, n, seconds))
        vals, ks = [v], k
    else:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(workers) as pool:
            outs = pool.map(_mixed_oracle_worker, [(kind, n, seconds)] * workers)
        vals, ks, nvol = [o[0] for o in outs], sum(o[1] for o in outs), outs[0][3]
    return {"value": float(sum(vals)), "unit": "DOF-residual-evals/s", "cores": workers, "kind": "port",
            "sample": f"the same generator at n = {n} ({nvol} volumes), {ks} residual evaluations over ~{seconds:.0f} s "
                      f"per core with the C oracle (dense operators, reference data flow)"}


def mixed_only_rk(torch, stream, args):
    """One form of the mixed stages, graph-replayed RK steps only (profiling)."""
    from dpgsolver_gb300.solver import BatchSimulation
    if args.workload == "mixed_ns":
        from dpgsolver_gb300.host import problem as P
        from dpgsolver_gb300.host.mixed import mixed_ns
        prob = mixed_ns(3, args.mixed_ns_n, seed=0, walls={(1, 0): P.BC_NOSLIP_ADIABATIC,
                                                           (1, 1): P.BC_NOSLIP_ADIABATIC})
    else:
        kind = "types" if args.workload == "mixed_types" else "hex"
        prob = make_mixed(kind, args.types_n if kind == "types" else args.mixed_n)
    sim = BatchSimulation(prob, stream=stream.cuda_stream)
    sim.form = {"plain": "plain", "per_group_graph": "plain", "fused": "fused",
                "branches": "branches", "stage": "stage"}[args.mixed_form]
    sim.set_graphs(args.mixed_form != "plain")
    sim.ssp_rk3_steps(prob.dt, max(args.warmup, 3), want_max=False)
    ms = _timed(torch, stream, lambda: sim.ssp_rk3_steps(prob.dt, 1, want_max=False), args.steps)
    sim.close()
    return {"metric": f"DOF-residual-evals/sec (mixed-order SSP-RK3 stages, {args.mixed_form})",
            "value": 3 * prob.n_state * args.steps / (ms * 1e-3), "unit": "DOF-residual-evals/s",
            "ms_per_step": ms / args.steps, "n_state": prob.n_state, "elements": prob.n_volumes}


def vortex2d_measurements(torch, stream, args):
    """The 2D isentropic vortex workload: curved QUAD 64^2, p = 3, Roe-Pike, 1000 graph-replayed SSP-RK3 steps; the
    L2 entropy error (compute_error_euler.c:135-180) of the initial and final states."""
    from dpgsolver_gb300.host.errors import l2_entropy_error
    from dpgsolver_gb300.host.problem import euler_vortex_2d
    from dpgsolver_gb300.solver import Simulation
    prob = euler_vortex_2d(64, 3)
    sim = Simulation(prob, stream=stream.cuda_stream)
    n = args.vortex_steps
    sim.ssp_rk3_steps(prob.dt, 1, want_max=False)     # capture the step graph
    sim.upload_state(prob.sol)
    ms = _timed(torch, stream, lambda: sim.ssp_rk3_steps(prob.dt, n, want_max=False), 1)
    final = sim.sol_coef
    res = {"workload": "2D Euler curved QUAD 64^2 p3 Roe-Pike isentropic vortex (strength 5 at (5,5) on (1,1,1,1))",
           "n_state": prob.n_state, "steps": n, "dt": prob.dt, "t_final": n * prob.dt,
           "value": 3 * prob.n_state * n / (ms * 1e-3), "unit": "DOF-residual-evals/s", "ms_per_step": ms / n,
           "l2_entropy_error": {"initial": l2_entropy_error(prob, prob.sol), "final": l2_entropy_error(prob, final)},
           "note": "state (2.1 MB) stays in L2 between steps; positivity checked every stage"}
    sim.close()
    return res


def ns_measurements(torch, stream, args):
    """Navier-Stokes: the Taylor-Green vortex at Re = 1600, Mach 0.1 on HEX 32^3, p = 3 (Roe-Pike + BR2), graph-
    replayed SSP-RK3 steps and plain residuals; the kinetic energy before and after (it must decay); the CPU oracle
    on a 6^3 sample of the same element work."""
    import oracle
    from dpgsolver_gb300.host.errors import kinetic_energy
    from dpgsolver_gb300.host.problem import ns_taylor_green
    from dpgsolver_gb300.solver import Simulation
    prob = ns_taylor_green(32, 3, Re=1600.0, mach=0.1)
    sim = Simulation(prob, stream=stream.cuda_stream)
    n = args.ns_steps
    sim.ssp_rk3_steps(prob.dt, 1, want_max=False)     # capture the step graph
    sim.upload_state(prob.sol)
    ms = _timed(torch, stream, lambda: sim.ssp_rk3_steps(prob.dt, n, want_max=False), 1)
    final = sim.sol_coef
    sim.upload_state(prob.sol)
    k = 20
    ms_rhs = _timed(torch, stream, lambda: [sim.compute_rhs(want_max=False) for _ in range(k)], 1) / k
    # end to end: dgpu_ssp_rk3_step_host on pinned buffers (a Navier-Stokes context runs upload + step + download)
    from dpgsolver_gb300 import _lib
    lib = _lib.load()
    sol_h = torch.from_numpy(np.ascontiguousarray(prob.sol)).pin_memory()
    out_h = torch.empty_like(sol_h).pin_memory()
    sp, op = (ctypes.cast(t.data_ptr(), _lib.c_double_p) for t in (sol_h, out_h))

    def e2e_step():
        _lib.check(lib.dgpu_ssp_rk3_step_host(sim.handle, ctypes.c_double(prob.dt), sp, op, None), sim.handle)
    e2e_step()
    n_e2e = 10
    ms_e2e = _timed(torch, stream, lambda: [e2e_step() for _ in range(n_e2e)], 1) / n_e2e
    # the end-to-end step's result against upload + graph-replayed step + download from the same input, bit for bit
    e2e_step()
    torch.cuda.synchronize()
    sim.upload_state(prob.sol)
    sim.ssp_rk3_steps(prob.dt, 1, want_max=False)
    e2e_bitwise = bool(np.array_equal(out_h.numpy(), sim.sol_coef))
    # the discrete adjoint: one VJP of R through the host-buffer forward/backward pair
    v = np.random.default_rng(0).standard_normal(prob.sol.shape)
    sim.vjp_forward(prob.sol)
    sim.vjp_backward(v)
    t0 = time.perf_counter()
    for _ in range(3):
        sim.vjp_backward(v)
    vjp_s = (time.perf_counter() - t0) / 3
    sim.close()
    res = {"workload": "3D Navier-Stokes Taylor-Green vortex, Re 1600, Mach 0.1, HEX 32^3 p3, Roe-Pike + BR2",
           "n_state": prob.n_state, "steps": n, "dt": prob.dt,
           "value": 3 * prob.n_state * n / (ms * 1e-3), "unit": "DOF-residual-evals/s", "ms_per_step": ms / n,
           "rhs_value": prob.n_state / (ms_rhs * 1e-3), "rhs_ms": ms_rhs,
           "e2e": {"value": 3 * prob.n_state / (ms_e2e * 1e-3), "unit": "DOF-residual-evals/s", "ms_per_step": ms_e2e,
                   "h2d_bytes_per_step": int(prob.n_state * 8), "d2h_bytes_per_step": int(prob.n_state * 8),
                   "note": "dgpu_ssp_rk3_step_host on pinned buffers (upload, graph-replayed step, download)",
                   "bitwise_equal_to_upload_step_download": e2e_bitwise},
           "kinetic_energy": {"initial": kinetic_energy(prob, prob.sol), "final": kinetic_energy(prob, final)},
           "launches_per_stage": 4,
           "vjp_backward_s": vjp_s,
           "vjp_note": "dgpu_vjp_backward: host cotangent in, host gradient out (84 MB each way included)"}
    if not args.no_cpu_baseline:
        sample = ns_taylor_green(6, 3, Re=1600.0, mach=0.1)
        o = oracle.Oracle(sample)
        o.compute_rhs(sample.sol)
        t0, cnt = time.perf_counter(), 0
        while time.perf_counter() - t0 < 5.0:
            o.compute_rhs(sample.sol)
            cnt += 1
        el = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": sample.n_state * cnt / el, "unit": "DOF-residual-evals/s", "cores": 1,
                               "kind": "port", "sample": f"HEX 6^3 p3 Taylor-Green, {cnt} oracle residuals in {el:.1f} s"}
    return res


_REF_WORKER = {}


def _ref_worker_init(sub, remote):
    """Pool initializer: the worker's share of the mesh (an element partition) and its oracle."""
    sys.path.insert(0, HERE)
    import oracle
    _REF_WORKER["o"] = oracle.Oracle(sub)
    _REF_WORKER["sol"] = np.ascontiguousarray(sub.sol)
    _REF_WORKER["remote"] = remote
    _REF_WORKER["o"].compute_rhs_remote(_REF_WORKER["sol"], remote)   # first touch


def _ref_worker_eval(_):
    t0 = time.perf_counter()
    _REF_WORKER["o"].compute_rhs_remote(_REF_WORKER["sol"], _REF_WORKER["remote"])
    return time.perf_counter() - t0


class PartitionedOracle:
    """The full workload's residual on `workers` host cores: the mesh split into element partitions
    (dpgsolver_gb300.partition, as on the GPUs), one oracle process per partition, the traces of the cut faces taken
    from the state once (the exchange itself is not timed). One evaluation = every process evaluates its partition's
    residual; its time is the slowest process's."""

    def __init__(self, prob, workers):
        import multiprocessing as mp

        import oracle
        from dpgsolver_gb300 import partition as PT
        self.n_state = prob.n_state
        self.workers = workers
        if workers == 1:
            self.pool = None
            self.o = oracle.Oracle(prob)
            self.sol = prob.sol
            return
        full = oracle.Oracle(prob)
        owner = PT.partition_volumes(prob, workers)
        jobs = []
        for r in range(workers):
            part = PT.Partition(prob, owner, r)
            sub = part.local_problem(prob)
            remote = np.zeros((len(part.faces), prob.n_var, prob.ops.n_fc))
            if part.n_halo:
                g = 2 * part.faces[part.recv_slots // 2] + part.recv_slots % 2
                remote[part.recv_slots // 2] = full.face_traces(prob.sol, g)
            jobs.append((sub, remote))
        del full
        ctx = mp.get_context("spawn")
        self.pool = [ctx.Pool(1, initializer=_ref_worker_init, initargs=job) for job in jobs]

    def evaluate(self) -> float:
        """Seconds of one full-mesh residual evaluation."""
        if self.pool is None:
            t0 = time.perf_counter()
            self.o.compute_rhs(self.sol)
            return time.perf_counter() - t0
        t0 = time.perf_counter()
        outs = [p.apply_async(_ref_worker_eval, (0,)) for p in self.pool]
        [o.get() for o in outs]
        return time.perf_counter() - t0

    def close(self):
        for p in self.pool or []:
            p.terminate()
            p.join()


def cpu_baseline(w, seconds, workers=1, prob=None):
    """The C oracle (dense operators, the reference's element-by-element data flow) on the bench's own mesh."""
    prob = make_problem(w) if prob is None else prob
    po = PartitionedOracle(prob, workers)
    try:
        po.evaluate()
        ts = []
        t0 = time.perf_counter()
        while not ts or time.perf_counter() - t0 < seconds:
            ts.append(po.evaluate())
    finally:
        po.close()
    return {"value": float(prob.n_state / statistics.median(ts)), "unit": "DOF-residual-evals/s", "cores": workers,
            "kind": "port",
            "sample": f"the GPU arm's own mesh ({prob.n_volumes} volumes, p{prob.ops.p}, {prob.n_state} state values), "
                      f"{len(ts)} residual evaluations, median time"
                      + (f"; split into {workers} element partitions, one oracle process each" if workers > 1 else
                         ", one core")}


def run_reference(args, rank, world):
    """The reference's algorithm on every host core, on the GPU arm's own mesh (rank 0 only). The reference itself is
    compiled in oracle/_ref only on the build host (from its sources, x86); the GPU host is an Arm machine without
    the reference tree, so its C restatement (oracle/, pinned to oracle/_ref's residuals by the tests) runs here,
    the mesh split into one element partition per core."""
    if rank != 0:
        return None
    w = WORKLOADS[args.workload]
    cores = os.cpu_count() or 1
    if w["kind"] == "mixed":
        per_step = []
        secs = max(1.0, min(10.0, 120.0 / max(1, args.steps + args.warmup)))
        for i in range(args.warmup + args.steps):
            cb = mixed_cpu_baseline("types" if args.workload == "mixed_types" else "hex", secs, workers=cores)
            if i >= args.warmup:
                per_step.append(cb["value"])
        value = statistics.median(per_step)
        cb["value"] = value
        config = {"workload": w["desc"]}
    else:
        prob = make_problem(w, n=args.n)
        po = PartitionedOracle(prob, cores)
        try:
            for _ in range(max(args.warmup, 1)):
                po.evaluate()
            # each step one full-mesh residual on all cores, bounded to about two minutes in all
            times = []
            t0 = time.perf_counter()
            for _ in range(max(1, args.steps)):
                times.append(po.evaluate())
                if time.perf_counter() - t0 > 120.0:
                    break
        finally:
            po.close()
        value = prob.n_state / statistics.median(times)
        cb = {"value": value, "unit": "DOF-residual-evals/s", "cores": cores, "kind": "port",
              "sample": f"the full mesh of the GPU arm ({prob.n_state} state values) split into {cores} element "
                        f"partitions, one oracle process per core; {len(times)} residual evaluations, median"}
        config = {"workload": w["desc"], "elements": prob.n_volumes, "p": prob.ops.p, "n_state": prob.n_state}
    return {
        "metric": "DOF-residual-evals/sec FP64 (batched graph vs plain per-group) at <=1e-12; %HBM peak",
        "impl": "reference", "value": value, "unit": "DOF-residual-evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
        "cpu_baseline": cb,
        "e2e": {"value": value, "unit": "DOF-residual-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference compiles here only on the build host (oracle/_ref, x86, from its own sources); on the "
                "GPU host its C restatement runs, which the tests pin to oracle/_ref's residuals and RK states",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="hex3d")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n", type=int, default=None, help="elements per direction (profiling of smaller cases)")
    ap.add_argument("--only-residual", action="store_true",
                    help="time compute_rhs_dg only (device-resident; profiling)")
    ap.add_argument("--only-rk", action="store_true", help="time graph-replayed SSP-RK3 steps only (profiling)")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint measurements")
    ap.add_argument("--no-jacobian", action="store_true", help="skip the block-sparse Jacobian assembly")
    ap.add_argument("--no-ns", action="store_true", help="skip the Navier-Stokes Taylor-Green measurements")
    ap.add_argument("--ns-steps", type=int, default=100, help="timed SSP-RK3 steps of the Taylor-Green run")
    ap.add_argument("--adjoint-steps", type=int, default=200)
    ap.add_argument("--adjoint-budget-gb", type=float, default=4.0)
    ap.add_argument("--no-mixed", action="store_true", help="skip the batched mixed-order measurements")
    ap.add_argument("--no-vortex", action="store_true", help="skip the 2D vortex run (1000 steps, entropy error)")
    ap.add_argument("--vortex-steps", type=int, default=1000)
    ap.add_argument("--mixed-n", type=int, default=58, help="volumes per direction of the mixed-order HEX mesh")
    ap.add_argument("--types-n", type=int, default=50, help="cells per direction of the mixed-type mesh (even)")
    ap.add_argument("--mixed-ns-n", type=int, default=24, help="volumes per direction of the mixed-order NS mesh")
    ap.add_argument("--tri-n", type=int, default=384, help="cells per direction of the 2D QUAD/TRI mesh")
    ap.add_argument("--mixed-form", choices=["plain", "per_group_graph", "fused", "branches", "stage"], default="fused",
                    help="form of the mixed-order stages for --workload mixed3d --only-rk")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        res = run_reference(args, rank, world)
        if rank == 0 and res is not None:
            print(json.dumps(res))
        return

    import dpgsolver_gb300
    dpgsolver_gb300.build()
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    res = run_partitioned(args, rank, world, local_rank) if world > 1 else run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
