"""Benchmark of the method-of-lines hot path on GB300.

Headline workload: the 3-D advection-diffusion-reaction system at 256^3 unknowns
(16,777,216), Float64, one fixed SSPRK33 step per bench step:
    u_t = div(K grad u) + 0.3 u_xy - (1, 0.5, 0) . grad u - 0.5 u^2
on [0,1]^3, x and y periodic, z Dirichlet 0, K a seeded log-normal field at the faces,
second-order centered diffusion and mixed terms, first-order upwind advection.  Metric:
Mcell-updates/s, a cell-update being one unknown advanced by one full step.  Inputs are
synthetic (seeded), resident in HBM when timing starts; the state (134 MB) and the per-cell
coefficient arrays (6 or 7 x 134 MB) are larger than L2, so no flush is needed.
`--stencil-form` picks the coefficient stencils' difference (default) or expanded form.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--full]

`--impl reference` times the CPU restatement of the reference's discretisation of the same
workload (C/OpenMP, oracle/c/adr_oracle.c, on every host core); the reference itself is
Julia and cannot run on this machine.  Secondary workloads (every other configuration at
its size) follow in `workloads`; `--full` lengthens the Tsit5 horizon.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "methodoflines.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Mcell-updates/s + %HBM roofline; batched & adjoint vs plain, 1 GPU, 1e-10 rel"
UNIT = "Mcell-updates/s"
HEADLINE = {"N": 256, "nz_pts": 258}
# algorithmic bytes per unknown and SSPRK33 step: 64 (u -> u1 16, (u, u1) -> u2 24,
# (u, u2) -> u' 24) plus 8 per per-cell coefficient array read once per stage: the three
# face-diffusivity arrays of the face form, or the plan's coefficient-stencil arrays
# (6 in the difference form, 7 expanded)


def adr_bytes_per_unknown_step(coef_arrays: int) -> int:
    return 64 + 3 * 8 * (coef_arrays if coef_arrays > 0 else 3)


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _profile_numbers():
    """Per-step DRAM traffic and FP64 flop counts taken from ncu captures (profiles/)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            return json.load(fh)
    except Exception:
        return {}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return rank, world


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed work runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.out = None
        self.gpu = gpu_index

    def start(self):
        try:
            self.out = open(os.path.join("/tmp", f"molgpu_clocks_{os.getpid()}.csv"), "w+")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        res = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.proc:
            return res
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.seek(0)
        rows = [r.split(",") for r in self.out.read().strip().splitlines() if r.strip()]
        self.out.close()
        try:
            os.remove(self.out.name)
        except OSError:
            pass
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        res.update(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=max(mx) if mx else None,
                   reasons=sorted(reasons), samples=len(rows))
        return res


def adr_problem():
    from molgpu import lower, problems
    sys_, disc, ex = problems.adr3d(**HEADLINE)
    return lower(sys_.to_spec(disc)), ex


def headline_config(lw, ex, world):
    """The workload description both arms print (identical dicts)."""
    return {"workload": "adr3d_256^3_ssprk33_step", "unknowns": int(lw.n_unknowns), "fields": 1,
            "grid": [256, 256, 256], "dt": float(ex["dt"]), "integrator": "SSPRK33 (fixed step)",
            "equation": "u_t = div(K grad u) + 0.3 u_xy - (1, 0.5, 0).grad u - 0.5 u^2",
            "bcs": "x, y periodic; z Dirichlet 0",
            "discretisation": "approx_order 2, nonlinear Laplacian with K at the faces, UpwindScheme(1)",
            "l2": "no flush: the state (134 MB) and the per-cell coefficient arrays (134 MB each) exceed L2",
            "parallelism": "replicas only" if world > 1 else "single GPU"}


def brusselator_plan(N):
    from molgpu import Plan, lower, problems
    sys_, disc, ex = problems.brusselator(N=N)
    lw = lower(sys_.to_spec(disc))
    return Plan(lw), lw, ex


def fp64_peak_live():
    """FP64 pipe peak on this GPU, measured now (eight independent DFMA chains per thread)."""
    import ctypes as C
    from molgpu import _lib as L
    w, t = C.c_double(), C.c_double()
    if L.lib().mol_diag_fp64_rate(32, C.byref(w), C.byref(t)) != 0:
        return None
    return t.value


# ---------------------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------------------

def run_ours(args, rank, world):
    import numpy as np
    import torch
    from molgpu import Plan
    from molgpu import _lib as L

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    hbm_peak, peak_kind = _peaks()
    t_setup = time.perf_counter()
    lw, ex = adr_problem()
    plan = Plan(lw, expand_stencils=args.stencil_form == "expanded")
    plan.set_stream(stream.cuda_stream)
    setup_s = time.perf_counter() - t_setup
    bytes_per_unknown = adr_bytes_per_unknown_step(plan.coef_arrays)
    n = lw.n_unknowns
    dt = ex["dt"]
    p = torch.tensor(lw.param_values, device=dev)
    u0 = torch.tensor(lw.u0, device=dev)
    u = u0.clone()
    fp64_peak = fp64_peak_live()
    t = 0.0
    for _ in range(max(3, args.warmup)):
        plan.step_ssprk33(u, dt, 1, t0=t, p=p)
        t += dt
    # The configuration's 0.3 u_xy exceeds 2 K (K ~ 0.01): its diffusion tensor is indefinite and
    # the discretisation grows modes near kx dx = ky dx = pi/2 by ~8 % per step, so from the
    # initial state a trajectory reaches O(1) growth, and -lambda u^2 then a blow-up, within
    # ~500 steps (the C/OpenMP restatement of the reference's discretisation does the same).  The
    # state is reset to u0 outside the timed events every RESET steps; the time of a step does not
    # depend on the values.
    RESET = 100
    u.copy_(u0)
    t = 0.0
    torch.cuda.synchronize()
    sampler = ClockSampler(dev.index)
    sampler.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = L.lib().mol_launch_count()
    evs = []
    wall0 = time.perf_counter()
    reps = max(1, args.steps)
    for k in range(reps):
        if k and k % RESET == 0:
            u.copy_(u0)
            t = 0.0
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.step_ssprk33(u, dt, 1, t0=t, p=p)
        e1.record(stream)
        evs.append((e0, e1))
        t += dt
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    wall = time.perf_counter() - wall0
    launches = L.lib().mol_launch_count() - launches0
    # keep the GPU busy a little longer so the clock sampler sees the kernels under load
    tl = time.perf_counter()
    u.copy_(u0)
    t, done = 0.0, 0
    while time.perf_counter() - tl < 1.0:
        if done >= RESET:
            u.copy_(u0)
            t, done = 0.0, 0
        plan.step_ssprk33(u, dt, 16, t0=t, p=p)
        t += 16 * dt
        done += 16
        torch.cuda.synchronize()
    clocks = sampler.stop()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms_total = sum(step_ms)
    if world > 1:
        tt = torch.tensor([ms_total], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(tt.item())
    ms_per_step = ms_total / reps
    value = world * n * reps / (ms_total * 1e-3) / 1e6
    prof = _profile_numbers().get(f"adr3d_256_{args.stencil_form}", {})
    bytes_per_step = float(bytes_per_unknown) * n
    achieved = bytes_per_step / (ms_per_step * 1e-3) / 1e9
    traffic = prof.get("step_bytes")
    fp64_per_unknown = prof.get("fp64_flops_per_unknown_step")
    fp64_achieved = fp64_per_unknown * n / (ms_per_step * 1e-3) / 1e12 if fp64_per_unknown else None
    # e2e: the public C-ABI call with pinned host buffers (H2D + step + D2H in every call)
    host = torch.empty(n, dtype=torch.float64, pin_memory=True)
    host.copy_(torch.from_numpy(lw.u0))
    hnp = host.numpy()
    pnp = lw.param_values.copy()
    for _ in range(2):
        plan.step_ssprk33(hnp, dt, 1, t0=0.0, p=pnp)
    e2e_reps = max(3, min(reps, 30))
    te = time.perf_counter()
    for k in range(e2e_reps):
        plan.step_ssprk33(hnp, dt, 1, t0=k * dt, p=pnp)
    te = time.perf_counter() - te
    e2e_value = world * n * e2e_reps / te / 1e6
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": reps,
        "warmup": max(3, args.warmup),
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: seeded log-normal diffusivity (64 random Fourier modes, correlation length 0.1) "
                "and a Gaussian initial blob, 256^3 unknowns",
        "config": headline_config(lw, ex, world),
        "codegen": bool(plan.uses_codegen),
        "stencil_form": args.stencil_form,
        "setup_s": setup_s,
        "gpu_launches": int(launches),
        "wall_s_timed_loop": wall,
        "step_ms_min_median": [min(step_ms), statistics.median(step_ms)],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": traffic,
                     "peak_source": peak_kind,
                     "kernel": "one SSPRK33 step: k_ssprk_t per stage (coefficient stencil, "
                               f"{plan.coef_arrays} per-cell coefficient arrays, no face pass)",
                     "algorithmic_bytes_per_unknown_step": bytes_per_unknown,
                     "traffic_source": prof.get("source") if traffic else None,
                     "note": "FP64-pipe bound on GB300 (FP64 = 1/64 of FP32); see fp64"},
        "fp64": {"peak_tflops_measured_now": fp64_peak,
                 "flops_per_unknown_step": fp64_per_unknown,
                 "achieved_tflops": fp64_achieved,
                 "frac": fp64_achieved / fp64_peak if (fp64_achieved and fp64_peak) else None},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                "path": "mol_step_ssprk33 with pinned host buffers, one step per call"},
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"], out["parity"] = cpu_baseline(lw, ex, plan, args.stencil_form, dev, stream)
    if rank == 0 and not args.headline_only:
        out["workloads"] = workloads(args, dev, stream, (plan, lw, ex))
    plan.close()
    return out


def cpu_baseline(lw, ex, plan, form, dev, stream):
    """The C/OpenMP restatement of the reference discretisation and SSPRK33 (oracle/c) on the
    host cores: SSPRK33 steps of the same 256^3 system on every core until at least 10 s have
    passed (at most 400 steps, restarted from u0 every 100: the configuration blows up near
    step 450), then one step on one core.  The same restatement checks the GPU right-hand side of
    both stencil forms on u0 (the parity bar is 1e-12 relative, norm-wise)."""
    import numpy as np
    import torch
    from molgpu import Plan
    from oracle.c_port import ADR3D, max_threads
    a = ADR3D(lw)
    dt = ex["dt"]
    ref_rhs = a.rhs(lw.u0)
    parity = {"reference": "oracle/c/adr_oracle.c right-hand side at u0", "bar": 1e-12}
    for f in ("difference", "expanded"):
        fp = plan if f == form else Plan(lw, expand_stencils=f == "expanded")
        fp.set_stream(stream.cuda_stream)
        uf = torch.tensor(lw.u0, device=dev)
        duf = torch.zeros_like(uf)
        fp.rhs(duf, uf, None, 0.0)
        torch.cuda.synchronize()
        parity[f"rhs_rel_err_{f}"] = float(np.linalg.norm(duf.cpu().numpy() - ref_rhs) / np.linalg.norm(ref_rhs))
        if fp is not plan:
            fp.close()
    s = np.array(lw.u0, copy=True)
    a.ssprk33(s, dt, 1, out=s)                     # warm (pages, threads)
    steps, el = 0, 0.0
    while el < 10.0 and steps < 400:
        if steps and steps % 100 == 0:
            s[...] = lw.u0
        t0 = time.perf_counter()
        a.ssprk33(s, dt, 2, out=s)
        el += time.perf_counter() - t0
        steps += 2
    cores = max_threads()
    t0 = time.perf_counter()
    a.ssprk33(lw.u0, dt, 1, 1)
    one = lw.n_unknowns / (time.perf_counter() - t0) / 1e6
    return {"value": lw.n_unknowns * steps / el / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} SSPRK33 steps of the 256^3 ADR system (16,777,216 unknowns) in {el:.1f} s, "
                      f"C/OpenMP restatement of the reference discretisation on {cores} threads; "
                      f"one thread: {one:.1f} Mcell-updates/s"}, parity


# ---------------------------------------------------------------------------------------
# secondary workloads (every configuration at its size)
# ---------------------------------------------------------------------------------------

def _time(fn, stream, reps, warm=True):
    import torch
    if warm:
        fn()  # first call may compile a kernel group (NVRTC) and capture graphs
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def workloads(args, dev, stream, adr):
    import numpy as np
    import torch
    from molgpu import Plan, lower, problems
    hbm_peak, _ = _peaks()
    res = {}
    full = args.full

    # config 1: heat, Tsit5 1e-10 to t=0.1
    sys_, disc, _ = problems.heat1d(101)
    lw = lower(sys_.to_spec(disc))
    plan = Plan(lw)
    plan.set_stream(stream.cuda_stream)
    u = lw.u0.copy()
    t0 = time.perf_counter()
    st = plan.solve_tsit5(u, 0.0, 0.1, 1e-10, 1e-10)
    el = time.perf_counter() - t0
    lam = -(4 / 0.01 ** 2) * math.sin(math.pi * 0.01 / 2) ** 2
    res["heat1d_n101_tsit5"] = {"wall_s": el, "naccept": st["naccept"], "nreject": st["nreject"],
                                "max_err_vs_semidiscrete_exact": float(np.max(np.abs(u - math.exp(lam * 0.1) * lw.u0)))}
    plan.close()

    # config 2: Brusselator RHS at 256^2 and 1024^2, SSPRK33 step, Tsit5 (short horizon unless --full)
    for N in (256, 1024):
        plan, lw, ex = brusselator_plan(N)
        plan.set_stream(stream.cuda_stream)
        n = lw.n_unknowns
        ud = torch.tensor(lw.u0, device=dev)
        du = torch.zeros_like(ud)
        ms = _time(lambda: plan.rhs(du, ud, None, 0.5), stream, 20)
        ms_step = _time(lambda: plan.step_ssprk33(ud, ex["dt_ssprk"], 16), stream, 3) / 16
        u32 = torch.tensor(lw.u0, device=dev, dtype=torch.float32)
        du32 = torch.zeros_like(u32)
        ms32 = _time(lambda: plan.rhs(du32, u32, None, 0.5), stream, 20)
        row = {"unknowns": n, "rhs_ms": ms, "rhs_Mcell_s": n / ms / 1e3,
               "rhs_hbm_frac": 16 * n / (ms * 1e-3) / 1e9 / hbm_peak,
               "ssprk33_step_ms": ms_step, "ssprk33_Mcell_s": n / ms_step / 1e3,
               "ssprk33_hbm_frac": 64 * n / (ms_step * 1e-3) / 1e9 / hbm_peak,
               "f32state_rhs_ms": ms32, "f32state_rhs_hbm_frac": 8 * n / (ms32 * 1e-3) / 1e9 / hbm_peak}
        if N == 256:
            # explicit Tsit5 on this stiff system is step-size limited by diffusion (dt ~ 6.6e-7):
            # t = 11.5 needs ~1.7e7 steps, so the timed run covers a short horizon
            uh = lw.u0.copy()
            t_end = 0.02 if full else 0.002
            t0 = time.perf_counter()
            st = plan.solve_tsit5(uh, 0.0, t_end, 1e-8, 1e-8)
            row["tsit5"] = {"t_end": t_end, "wall_s": time.perf_counter() - t0,
                            "naccept": st["naccept"], "nreject": st["nreject"]}
        else:
            # end to end through mol_step_ssprk33 on pinned host buffers, and the C/OpenMP
            # restatement on the host cores, one step per call / per sample step
            from oracle.c_port import Brusselator, max_threads
            host = torch.empty(n, dtype=torch.float64, pin_memory=True)
            host.copy_(torch.from_numpy(lw.u0))
            hnp = host.numpy()
            for _ in range(2):
                plan.step_ssprk33(hnp, ex["dt_ssprk"], 1)
            te = time.perf_counter()
            for k in range(30):
                plan.step_ssprk33(hnp, ex["dt_ssprk"], 1, t0=k * ex["dt_ssprk"])
            row["e2e_Mcell_s"] = n * 30 / (time.perf_counter() - te) / 1e6
            b = Brusselator(lw)
            s = b.ssprk33(lw.u0, 0.0, ex["dt_ssprk"], 2)
            steps, el = 0, 0.0
            while el < 3.0:
                t0 = time.perf_counter()
                s = b.ssprk33(s, steps * ex["dt_ssprk"], ex["dt_ssprk"], 20)
                el += time.perf_counter() - t0
                steps += 20
            row["cpu_port_Mcell_s"] = n * steps / el / 1e6
            row["cpu_port_cores"] = max_threads()
        res[f"brusselator_{N}"] = row
        plan.close()

    # config 3: Burgers WENO5, SSPRK33 for 20000 steps and the discrete adjoint
    sys_, disc, ex = problems.burgers()
    lw = lower(sys_.to_spec(disc))
    plan = Plan(lw)
    plan.set_stream(stream.cuda_stream)
    n = lw.n_unknowns
    nsteps = 20000
    ud = torch.tensor(lw.u0, device=dev)
    plan.step_ssprk33(ud, ex["dt"], 32)
    torch.cuda.synchronize()
    fwd_ms = _time(lambda: plan.step_ssprk33(ud, ex["dt"], nsteps), stream, 1, warm=False)
    tgt = torch.tensor(ex["target"], device=dev)
    g = torch.zeros(n, dtype=torch.float64, device=dev)
    gp = torch.zeros(1, dtype=torch.float64, device=dev)
    u0d = torch.tensor(lw.u0, device=dev)
    plan.adjoint_ssprk33(u0d, ex["dt"], 2, tgt, nsnap=2, dLdu0=g, dLdp=gp)   # warm: compiles the VJP
    torch.cuda.synchronize()
    # each schedule once untimed first: its checkpoint storage (31 GB with every state kept) is
    # allocated by the first call and reused by later ones
    plan.adjoint_ssprk33(u0d, ex["dt"], nsteps, tgt, nsnap=64, dLdu0=g, dLdp=gp)
    torch.cuda.synchronize()
    ta = time.perf_counter()
    loss, nfw = plan.adjoint_ssprk33(u0d, ex["dt"], nsteps, tgt, nsnap=64, dLdu0=g, dLdp=gp)
    torch.cuda.synchronize()
    adj_s = time.perf_counter() - ta
    plan.adjoint_ssprk33(u0d, ex["dt"], nsteps, tgt, nsnap=0, dLdu0=g, dLdp=gp)
    torch.cuda.synchronize()
    ta = time.perf_counter()
    plan.adjoint_ssprk33(u0d, ex["dt"], nsteps, tgt, nsnap=0, dLdu0=g, dLdp=gp)
    torch.cuda.synchronize()
    adj_all_s = time.perf_counter() - ta
    res["burgers_65536_weno5"] = {"unknowns": n, "steps": nsteps, "ssprk33_ms_per_step": fwd_ms / nsteps,
                                  "ssprk33_Mcell_s": n * nsteps / fwd_ms / 1e3,
                                  "adjoint_64_snapshots_s": adj_s, "adjoint_vs_forward": adj_s / (fwd_ms * 1e-3),
                                  "adjoint_forward_steps_recomputed": nfw,
                                  "adjoint_all_steps_stored_s": adj_all_s,
                                  "adjoint_all_stored_vs_forward": adj_all_s / (fwd_ms * 1e-3),
                                  "loss": loss, "dLdnu": float(gp.item())}
    plan.close()

    # config 5 beyond the headline step: RHS, Float32 state, adjoint dL/dK over 500 steps
    plan, lw, ex = adr
    n = lw.n_unknowns
    ud = torch.tensor(lw.u0, device=dev)
    du = torch.zeros_like(ud)
    ms = _time(lambda: plan.rhs(du, ud, None, 0.1), stream, 5)
    u32 = torch.tensor(lw.u0, device=dev, dtype=torch.float32)
    du32 = torch.zeros_like(u32)
    ms32 = _time(lambda: plan.rhs(du32, u32, None, 0.1), stream, 5)
    # 400 of the configuration's 500 steps: its 0.3 u_xy makes the system ill-posed (indefinite
    # diffusion tensor), and from u0 the reference's discretisation itself (the C/OpenMP
    # restatement) leaves O(1) between steps 400 (max |u| 1.03) and 450 (2.95) and overflows before
    # step 500, where the gradient is no longer finite
    adj_steps = 400
    tgt = torch.tensor(np.random.default_rng(12).standard_normal(n) * 1e-3, device=dev)
    u0d = torch.tensor(lw.u0, device=dev)
    gaux = torch.zeros(sum(a.size for a in lw.aux), dtype=torch.float64, device=dev)
    fwd = _time(lambda: plan.step_ssprk33(u0d.clone(), ex["dt"], adj_steps), stream, 1)
    plan.adjoint_ssprk33(u0d, ex["dt"], 2, tgt, nsnap=2, dLdaux=gaux)   # warm: compiles the VJP
    torch.cuda.synchronize()
    plan.adjoint_ssprk33(u0d, ex["dt"], adj_steps, tgt, nsnap=64, dLdaux=gaux)   # allocates the slots
    torch.cuda.synchronize()
    ta = time.perf_counter()
    _, nfw64 = plan.adjoint_ssprk33(u0d, ex["dt"], adj_steps, tgt, nsnap=64, dLdaux=gaux)
    torch.cuda.synchronize()
    adj_s = time.perf_counter() - ta
    plan.adjoint_ssprk33(u0d, ex["dt"], adj_steps, tgt, nsnap=0, dLdaux=gaux)    # allocates 54 GB of states
    torch.cuda.synchronize()
    ta = time.perf_counter()
    _, nfw0 = plan.adjoint_ssprk33(u0d, ex["dt"], adj_steps, tgt, nsnap=0, dLdaux=gaux)
    torch.cuda.synchronize()
    adj_all_s = time.perf_counter() - ta
    # both stencil forms' step (the headline plan's and the other one)
    forms = {}
    for form in ("difference", "expanded"):
        fp = plan if form == args.stencil_form else Plan(lw, expand_stencils=form == "expanded")
        fp.set_stream(stream.cuda_stream)
        uf = torch.tensor(lw.u0, device=dev)
        step = _time(lambda: fp.step_ssprk33(uf, ex["dt"], 1), stream, 10)
        forms[form] = {"ssprk33_step_ms": step, "ssprk33_Mcell_s": n / step / 1e3, "coef_arrays": fp.coef_arrays}
        if fp is not plan:
            fp.close()
    res["adr3d_256^3"] = {"unknowns": n, "rhs_ms": ms, "rhs_Mcell_s": n / ms / 1e3,
                          "rhs_hbm_frac": (16 + 8 * max(plan.coef_arrays, 3)) * n / (ms * 1e-3) / 1e9 / hbm_peak,
                          "stencil_forms": forms,
                          "f32state_rhs_ms": ms32,
                          "f32state_rhs_hbm_frac": (8 + 4 * max(plan.coef_arrays, 3)) * n / (ms32 * 1e-3) / 1e9
                          / hbm_peak,
                          "forward_steps_ms": fwd,
                          "adjoint_steps": adj_steps, "adjoint_dLdK_64_snapshots_s": adj_s,
                          "adjoint_64_snapshots_vs_forward": adj_s / (fwd * 1e-3),
                          "adjoint_64_snapshots_forward_steps": nfw64,
                          "adjoint_dLdK_states_kept_s": adj_all_s,
                          "adjoint_states_kept_vs_forward": adj_all_s / (fwd * 1e-3),
                          "adjoint_states_kept_forward_steps": nfw0}

    # config 4: batched ensemble of uneven nonlinear-diffusion problems vs sequential plain solves
    res["batched_nonlinear_diffusion"] = batched(args, dev, stream)
    return res


def batched(args, dev, stream):
    """The configuration's 4096 members for its 1000 SSPRK33 steps, FP64 and Float32 state
    from the same initial states (the Float32 error is taken between the two runs), against
    sequential plain solves of a stratified sample of the members for the same 1000 steps."""
    import numpy as np
    import torch
    from molgpu import Batch, Plan, lower, problems
    count = 4096
    members = problems.ensemble_members(4096)[:count]
    t0 = time.perf_counter()
    lws, dts = [], []
    for (n, k, seed) in members:
        sys_, disc, _ = problems.nonlinear_diffusion(n, k, seed)
        lw = lower(sys_.to_spec(disc))
        lws.append(lw)
        dx = 1.0 / (n - 1)
        dts.append(0.125 * dx * dx / float(np.max(lw.u0)) ** 2)
    dts = np.array(dts)
    batch = Batch(lws)
    batch.set_stream(stream.cuda_stream)
    setup = time.perf_counter() - t0
    total = int(batch.offsets[-1])
    steps = 1000
    packed = batch.pack([lw.u0 for lw in lws])
    w = torch.tensor(packed, device=dev)
    batch.step_ssprk33(w, dts, 2)          # autotune + warm
    w32 = w.float()
    batch.step_ssprk33(w32, dts, 2)
    del w, w32
    u = torch.tensor(packed, device=dev)
    u32 = u.float()
    torch.cuda.synchronize()
    ms = _time(lambda: batch.step_ssprk33(u, dts, steps), stream, 1, warm=False)
    ms32 = _time(lambda: batch.step_ssprk33(u32, dts, steps), stream, 1, warm=False)
    batch.check()
    f32err = float(torch.linalg.norm(u32.double() - u) / torch.linalg.norm(u))
    # sequential plain solves (one plan per instance, same steps) on a stratified sample
    idx = list(range(0, count, max(1, count // 64)))
    seq_ms = 0.0
    for i in idx:
        p = Plan(lws[i])
        p.set_stream(stream.cuda_stream)
        ui = torch.tensor(lws[i].u0, device=dev)
        p.step_ssprk33(ui, dts[i], 2)
        seq_ms += _time(lambda: p.step_ssprk33(ui, dts[i], steps), stream, 1, warm=False)
        p.close()
    seq_ms *= count / len(idx)
    sched = batch.config
    batch.close()
    return {"instances": count, "unknowns": total, "steps": steps, "setup_s": setup,
            "batched_ms": ms, "batched_Mcell_s": total * steps / ms / 1e3,
            "f32state_batched_ms": ms32, "f32state_rel_err_vs_f64": f32err,
            "schedule": sched,
            "sequential_plain_ms_estimated": seq_ms,
            "sequential_sample": f"{len(idx)} of {count} instances ({steps} steps each), scaled by "
                                 f"{count / len(idx):.1f}",
            "batched_vs_sequential": seq_ms / ms}


# ---------------------------------------------------------------------------------------
# reference arm: the reference's discretisation on the host (C/OpenMP restatement)
# ---------------------------------------------------------------------------------------

def run_reference(args, rank, world):
    """The reference's CPU path for the headline workload: the reference itself is Julia and
    cannot run on this machine, so its discretisation and SSPRK33 are timed through the
    C/OpenMP restatement (oracle/c/adr_oracle.c) on every host core: W warm-up steps, then
    at least K steps and at least one second."""
    if rank != 0:
        return None
    import numpy as np
    from oracle.c_port import ADR3D, max_threads
    lw, ex = adr_problem()
    a = ADR3D(lw)
    dt = ex["dt"]
    w = max(0, args.warmup)
    s = np.array(lw.u0, copy=True)
    if w:
        a.ssprk33(s, dt, w, out=s)
    reps = max(1, args.steps)
    steps, el = 0, 0.0
    while steps < reps or el < 1.0:
        if steps and steps % 100 == 0:
            s[...] = lw.u0          # outside the timed call: the configuration blows up near step 450
        t0 = time.perf_counter()
        a.ssprk33(s, dt, 1, out=s)
        el += time.perf_counter() - t0
        steps += 1
    value = lw.n_unknowns * steps / el / 1e6
    cores = max_threads()
    sample = (f"{steps} SSPRK33 steps of the 256^3 ADR system (16,777,216 unknowns) after {w} warm-up steps, "
              f"{el:.2f} s; C/OpenMP restatement of the reference discretisation on {cores} threads (the "
              "reference is Julia and is not runnable here)")
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": w,
            "ms_per_step": el / steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": headline_config(lw, ex, world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------------------
# small single-path cases, the commands the ncu summaries under profiles/ were taken with

def run_case(name, args):
    import numpy as np
    import torch
    from molgpu import Batch, Plan, lower, problems
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    out = {"case": name}
    if name == "burgers_adjoint":
        # Burgers WENO5 (65,536 unknowns): 30-step adjoint, every state and stage kept
        sys_, disc, ex = problems.burgers()
        lw = lower(sys_.to_spec(disc))
        plan = Plan(lw)
        plan.set_stream(stream.cuda_stream)
        u0 = torch.tensor(lw.u0, device=dev)
        tgt = torch.tensor(ex["target"], device=dev)
        g = torch.zeros_like(u0)
        gp = torch.zeros(1, dtype=torch.float64, device=dev)
        for _ in range(2):
            loss, nfw = plan.adjoint_ssprk33(u0, ex["dt"], 30, tgt, nsnap=0, dLdu0=g, dLdp=gp)
        torch.cuda.synchronize()
        out.update(loss=loss, dLdnu=float(gp.item()))
        plan.close()
    elif name == "burgers_steps":
        # Burgers WENO5 (65,536 unknowns): 64 SSPRK33 steps
        sys_, disc, ex = problems.burgers()
        lw = lower(sys_.to_spec(disc))
        plan = Plan(lw)
        plan.set_stream(stream.cuda_stream)
        u = torch.tensor(lw.u0, device=dev)
        for _ in range(4):
            plan.step_ssprk33(u, ex["dt"], 16)
        torch.cuda.synchronize()
        out.update(norm=float(torch.linalg.norm(u)))
        plan.close()
    elif name == "ensemble":
        # the first 512 ensemble members, 5 steps of the tiled persistent kernel with the
        # schedule the autotuner picks for all 4096 (256 threads, 3 CTAs per SM, 65536-cell tiles)
        lws, dts = [], []
        for (n, k, seed) in problems.ensemble_members(4096)[:512]:
            sys_, disc, _ = problems.nonlinear_diffusion(n, k, seed)
            lw = lower(sys_.to_spec(disc))
            lws.append(lw)
            dts.append(0.125 / (n - 1) ** 2 / float(np.max(lw.u0)) ** 2)
        batch = Batch(lws)
        batch.set_stream(stream.cuda_stream)
        batch.tune(256, 3, 65536)
        u = torch.tensor(batch.pack([lw.u0 for lw in lws]), device=dev)
        for _ in range(3):
            batch.step_ssprk33(u, np.array(dts), 5)
        batch.check()
        out.update(unknowns=int(batch.offsets[-1]), norm=float(torch.linalg.norm(u)))
        batch.close()
    elif name in ("brusselator_rhs_generated", "brusselator_rhs_interpreted", "brusselator_steps"):
        # one RHS (or SSPRK33 steps) of the 1024^2 Brusselator through the generated cell or
        # the interpreter
        if name.endswith("interpreted"):
            os.environ["MOL_DISABLE_CODEGEN"] = "1"
        sys_, disc, ex = problems.brusselator(N=1024)
        lw = lower(sys_.to_spec(disc))
        plan = Plan(lw)
        plan.set_stream(stream.cuda_stream)
        u = torch.tensor(lw.u0, device=dev)
        du = torch.zeros_like(u)
        for _ in range(5):
            if name == "brusselator_steps":
                plan.step_ssprk33(u, ex["dt_ssprk"], 1)
            else:
                plan.rhs(du, u, None, 0.5)
        torch.cuda.synchronize()
        out.update(codegen=plan.uses_codegen, norm=float(torch.linalg.norm(du)))
        plan.close()
    elif name == "fp64_lanes":
        # the FP64 pipe: warp FMA instructions per second with 32..1 active lanes per warp
        import ctypes as C
        from molgpu import _lib as L
        rows = []
        for act in (32, 16, 8, 4, 2, 1):
            w, t = C.c_double(), C.c_double()
            L.check(L.lib().mol_diag_fp64_rate(act, C.byref(w), C.byref(t)))
            rows.append({"active_lanes": act, "warp_fma_G_per_s": w.value / 1e9, "lane_tflops": t.value})
        out.update(rows=rows)
    elif name in ("adr3d_rhs", "adr3d_steps", "adr3d_vjp"):
        # five RHS evaluations, SSPRK33 steps or vector-Jacobian products (into dL/du and
        # dL/daux, as the adjoint accumulates them) of the 3-D ADR problem at N^3 (--case-n,
        # 128 by default)
        N = args.case_n or 128
        sys_, disc, ex = problems.adr3d(N=N, nz_pts=N + 2)
        lw = lower(sys_.to_spec(disc))
        plan = Plan(lw, expand_stencils=args.stencil_form == "expanded")
        plan.set_stream(stream.cuda_stream)
        # --state f32: the Float32-state kernels (RHS and steps)
        u = torch.tensor(lw.u0, device=dev, dtype=torch.float32 if args.state == "f32" else torch.float64)
        du = torch.zeros_like(u)
        lam = torch.tensor(np.random.default_rng(3).standard_normal(u.numel()), device=dev)
        gaux = torch.zeros(sum(a.size for a in lw.aux), dtype=torch.float64, device=dev)
        for _ in range(5):
            if name == "adr3d_steps":
                plan.step_ssprk33(u, ex["dt"], 1)
            elif name == "adr3d_vjp":
                plan.vjp(lam, u, None, 0.1, lam_u=du, lam_aux=gaux)
            else:
                plan.rhs(du, u, None, 0.1)
        torch.cuda.synchronize()
        out.update(norm=float(torch.linalg.norm(u if name == "adr3d_steps" else du)))
        plan.close()
    else:
        raise SystemExit(f"unknown case {name}")
    print(json.dumps(out), flush=True)


CASES = ["burgers_adjoint", "burgers_steps", "ensemble", "brusselator_rhs_generated", "brusselator_rhs_interpreted",
         "brusselator_steps", "adr3d_rhs", "adr3d_steps", "adr3d_vjp", "fp64_lanes"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--full", action="store_true", help="longer Tsit5 horizon")
    ap.add_argument("--headline-only", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--case", default=None, choices=CASES,
                    help="run one small single-path case (for profiling) and exit")
    ap.add_argument("--case-n", type=int, default=0, help="grid side of the adr3d cases")
    ap.add_argument("--state", default="f64", choices=["f64", "f32"], help="state precision of the adr3d cases")
    ap.add_argument("--stencil-form", default="expanded", choices=["difference", "expanded"],
                    help="coefficient stencils of the 3-D ADR plan (MOL_FLAG_EXPAND_STENCILS for expanded)")
    args = ap.parse_args()
    if args.case:
        run_case(args.case, args)
        return
    rank, world = _dist()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    out = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
