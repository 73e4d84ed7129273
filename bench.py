"""Benchmark: integrating-factor RK4 steps/s of the forced 512^3 DNS on GB300.

Workload (the reference's forced-DNS configuration at 512^3): incompressible
Navier-Stokes in rotational form on [0, 2 pi]^3, 2/3 dealiasing, constant-power
forcing eps = 0.1 on k2 < 2.5^2, nu = 1.5e-3, dt = 5e-4, initial field seeded
by ran1 (seed 1) with E(k) ~ k^4 exp(-2 (k/4)^2) and energy 0.5.  One "step"
is one full IF-RK4 step (4 right-hand sides).  The headline arm is the FP32-bulk
mode; the plain-FP64 mode is timed beside it.

`value`: steps/s with the state resident in HBM (CUDA events on the launch
stream).  `e2e`: steps/s through the C ABI with host buffers, each step
uploading the state from pinned host memory, stepping and downloading it.
Every field (539 MB in FP32) is larger than L2 (129 MB), so no flush is
needed between steps.

`--impl reference` times the reference algorithm on the host cores instead:
whole IF-RK4 steps of the same 512^3 workload from the same seeded field, in
the reference's single-precision build (constant_sp.f90), computed by the
threaded restatement oracle/cpu_step.py on every host core (the reference's
Fortran + FFTW sources cannot be compiled here or on the GPU host).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 512
NU, DT, EPS, FKMAX = 1.5e-3, 5e-4, 0.1, 2.5
AKP, U0, SEED = 4.0, 1.0 / 3.0 ** 0.5, 1
METRIC = "RK4 steps/s, 512^3 forced DNS (FP32 bulk; plain FP64 alongside)"
UNIT = "steps/s"


def workload_config(n, world):
    """The workload both arms report (the reference arm samples it on the CPU)."""
    return {"workload": "forced DNS %d^3 IF-RK4, FP32 bulk" % n, "grid": n,
            "nu": NU, "dt": DT, "eps": EPS, "fkmax": FKMAX,
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "inputs larger than L2 (%d MB per field)" % round((n // 2 + 1) * n * n * 8 / 1e6)}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N)
    ap.add_argument("--ny", type=int, default=0, help="non-cubic grid (profiling runs)")
    ap.add_argument("--nz", type=int, default=0, help="non-cubic grid (profiling runs)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-les", action="store_true")
    ap.add_argument("--cpu-configs", action="store_true",
                    help="only time the CPU port on the other configurations (forced DNS 128^3 FP64, LES "
                         "256^3 Smagorinsky and dynamic, the 2D ensemble members one at a time) and print "
                         "one JSON line")
    ap.add_argument("--no-schemes", action="store_true",
                    help="skip timing the rotating solver, its passive scalar and the variable-step IF-AB2 "
                         "(passes per second on the same grid and initial field)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler over the timed region (SM clock, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(5)
            except Exception:
                self.p.kill()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        except Exception:
            rows = []
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = max(float(r[2]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max(float(r[3]) for r in rows)}


# algorithmic bytes per launch, in fields F = (nx/2+1) ny nz complex elements
# (exact reads + writes of each pass; RK stage averages).  Unfused, zfwd runs
# all four stages (12, 15, 15, 9 F: stage 4 reads the Lamb vector and the
# accumulator, which stage 3 left holding E^2 v + its partial sum, and
# writes the state).  With stages 1-3 fused into zfwd_zinv (15, 18, 18 F:
# the RHS, v, acc read; acc and the next u, w written) zfwd runs stage 4
# only (9 F); zinv runs once per step and zinv_kx0 covers one kx tile (not
# counted).
KERNELS = ["zinv", "ypass_inv", "xpass", "ypass_fwd", "zfwd", "zfwd_zinv", "zinv_kx0", "fixup"]


def kernel_fields(fused):
    return {"zinv": 9.0, "ypass_inv": 12.0, "xpass": 9.0, "ypass_fwd": 6.0,
            "zfwd": 9.0 if fused else 12.75, "zfwd_zinv": 17.0, "zinv_kx0": 0.0, "fixup": 0.0}


def traffic_from_profiles(kernel):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic_512.txt")
    try:
        for line in open(path):
            m = re.match(r"\s*%s\s+([0-9.eE+]+)\s*$" % re.escape(kernel), line)
            if m:
                return float(m.group(1))
    except OSError:
        pass
    return None


def seeded_field(n):
    """The workload's initial field as the reference generates it
    (initialize.f90:284-371, ran1 seed 1), from the oracle."""
    import numpy as np
    from oracle import spectral_ref as R
    return R.initialize_dealiased(n, n, n, SEED, AKP, U0, 2.0 * (n // 2) / 3.0)


def cpu_stepper(n, workers, precision):
    """The threaded CPU restatement of the 512^3 IF-RK4 step
    (oracle/cpu_step.py); precision "f32" is the reference's single build
    (constant_sp.f90), "f64" its double build (constant.f90)."""
    import numpy as np
    from oracle import spectral_ref as R
    from oracle.cpu_step import CpuRK4
    R.WORKERS = workers
    g = R.Grid(R.Params(nx=n, nu=NU, dt=DT, eps=EPS, fkmax=FKMAX))
    return CpuRK4(g, workers, np.complex64 if precision == "f32" else np.complex128)


def cpu_time_steps(st, v, k):
    t0 = time.perf_counter()
    for _ in range(k):
        st.step(v)
    return (time.perf_counter() - t0) / k


def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np
    workers = len(os.sched_getaffinity(0))
    n = a.n
    v0 = seeded_field(n)
    st = cpu_stepper(n, workers, "f32")
    v = [np.array(x, np.complex64) for x in v0]
    del v0
    for _ in range(max(a.warmup, 0)):
        st.step(v)
    t_step = cpu_time_steps(st, v, a.steps)
    st.close()
    val = 1.0 / t_step
    sample = ("%d whole IF-RK4 steps (4 right-hand sides each) of the %d^3 forced DNS from the ran1 "
              "seed-1 field after %d warm-up steps, single-precision build (constant_sp.f90) restated by "
              "oracle/cpu_step.py: scipy.fft with %d workers and the pointwise passes threaded over "
              "z-slabs" % (a.steps, n, a.warmup, workers))
    out = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
           "impl": "reference",
           "config": workload_config(n, world),
           "cpu_baseline": {"value": val, "unit": UNIT, "cores": workers, "kind": "port",
                            "sample": sample},
           "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


def cpu_baseline_leg(n):
    """The bounded CPU samples beside the GPU number (rank 0, N = 1): one
    whole RK4 step on every core in each build of the reference, and one
    right-hand side on one core (the reference's single-threaded FFTW plans,
    fftwplan.f90:11-14), reported per step as 4 right-hand sides."""
    import numpy as np
    workers = len(os.sched_getaffinity(0))
    v0 = seeded_field(n)
    out = {}
    for prec, dt in (("f32", np.complex64), ("f64", np.complex128)):
        st = cpu_stepper(n, workers, prec)
        v = [np.array(x, dt) for x in v0]
        st.step(v)                       # warm-up: allocation, transform plans
        t = cpu_time_steps(st, v, 1)
        st.close()
        out[prec] = {"steps_per_s": 1.0 / t, "s_per_step": t, "workers": workers,
                     "sample": "1 whole RK4 step after 1 warm-up step"}
        del st, v
    st = cpu_stepper(n, 1, "f32")
    v = [np.array(x, np.complex64) for x in v0]
    st.rhs(v)
    t0 = time.perf_counter()
    st.rhs(v)
    t_rhs = time.perf_counter() - t0
    st.close()
    out["f32_one_core"] = {"steps_per_s": 1.0 / (4.0 * t_rhs), "s_per_step": 4.0 * t_rhs, "workers": 1,
                           "sample": "1 right-hand side after 1 warm-up right-hand side, x4 per step"}
    return {"value": out["f32"]["steps_per_s"], "unit": UNIT, "cores": workers, "kind": "port",
            "sample": "one whole IF-RK4 step of the %d^3 forced DNS from the ran1 seed-1 field, "
                      "single-precision build (constant_sp.f90) restated by oracle/cpu_step.py on %d "
                      "cores; the double build and one core beside it" % (n, workers),
            "by_build": out}


def run_ours(a):
    import numpy as np
    import torch
    import speccodelib_gb300 as S
    from speccodelib_gb300 import specns as SP

    rank, world, local = dist_env()
    dist = world > 1
    if dist:
        import torch.distributed as td
        td.init_process_group("nccl")
    torch.cuda.set_device(local)
    SP._check(SP.lib().sc_set_device(local))
    n = a.n
    stream = torch.cuda.Stream()

    def make(prec):
        p = S.default_params(n, prec, nu=NU, dt=DT, eps=EPS, fkmax=FKMAX,
                             ny=a.ny or n, nz=a.nz or n)
        h = S.SpectralNS(p)
        h.set_stream(stream.cuda_stream)
        h.init_field(seed=SEED, akp=AKP, u0=U0)
        return h

    def barrier():
        if dist:
            td.barrier()

    def max_over_ranks(x):
        if not dist:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        td.all_reduce(t, op=td.ReduceOp.MAX)
        return float(t.item())

    def time_steps(h, k):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        h.rk4_steps(k)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return e0.elapsed_time(e1)

    # ---- FP32 bulk: the headline ----
    h = make(S.SC_FP32)
    init32 = h.get_state()
    h.rk4_steps(a.warmup)
    torch.cuda.synchronize()
    with Clocks(local) as ck:
        ms = time_steps(h, a.steps)
    clocks = ck.summary()
    ms = max_over_ranks(ms)
    # per-kernel times: the same K steps again, with CUDA events around every launch
    h.profile_enable(True)
    time_steps(h, a.steps)
    prof = {}
    launches = 0
    for name in KERNELS:
        cnt, tot = h.profile_read(name)
        if cnt:
            prof[name] = (cnt, tot)
        launches += cnt
    KERNEL_FIELDS = kernel_fields("zfwd_zinv" in prof)
    h.profile_enable(False)
    value = world * a.steps / (ms / 1e3)
    ms_step = ms / a.steps

    F = (n // 2 + 1) * (a.ny or n) * (a.nz or n) * 8.0
    dom = max(prof, key=lambda k: prof[k][1])
    cnt, tot = prof[dom]
    avg_ms = tot / max(cnt, 1)
    alg = KERNEL_FIELDS[dom] * F
    hbm, peak_kind = peaks()
    achieved = alg / (avg_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_source": peak_kind,
                "traffic": traffic_from_profiles(dom),
                "algorithmic_bytes_per_launch": alg, "avg_launch_ms": avg_ms}
    step_bytes = h.step_bytes()
    tot_all = max(sum(x[1] for x in prof.values()), 1e-9)
    kernels = {k: {"launches": c, "ms_total": t, "avg_ms": t / max(c, 1), "share": t / tot_all,
                   "achieved_gbs": (KERNEL_FIELDS[k] * F / (t / c / 1e3) / 1e9)
                   if c and KERNEL_FIELDS[k] else None}
               for k, (c, t) in prof.items()}

    # ---- e2e through the C ABI with host buffers ----
    e2e = None
    if not a.no_e2e:
        shape = (n, n, n // 2 + 1)
        host = [torch.empty(shape, dtype=torch.complex64, pin_memory=True) for _ in range(3)]
        hv = [x.numpy() for x in host]
        for dst, src in zip(hv, init32):
            dst[...] = src
        ke = min(a.steps, 5)
        SP._check(SP.lib().sc_set_state(h.h, *[SP._ptr(x) for x in hv]))
        h.rk4_steps(1)
        SP._check(SP.lib().sc_get_state(h.h, *[SP._ptr(x, True) for x in hv]))
        barrier()
        t0 = time.perf_counter()
        for _ in range(ke):
            SP._check(SP.lib().sc_set_state(h.h, *[SP._ptr(x) for x in hv]))
            h.rk4_steps(1)
            SP._check(SP.lib().sc_get_state(h.h, *[SP._ptr(x, True) for x in hv]))
        torch.cuda.synchronize()
        te = max_over_ranks(time.perf_counter() - t0)
        nbytes = 3 * (n // 2 + 1) * n * n * 8
        e2e = {"value": world * ke / te, "unit": UNIT, "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes, "steps": ke,
               "path": "sc_set_state(pinned host) + sc_rk4_steps(1) + sc_get_state(pinned host)"}
        del host, hv

    # FP32 diagnostics after 2 steps from the seeded field (compared with FP64 below)
    h.set_state(*init32)
    h.rk4_steps(2)
    d32, e32 = h.diagnostics()
    h.close()
    del h, init32
    torch.cuda.empty_cache()

    # ---- plain FP64 beside it, and the FP32 error against it ----
    fp64 = None
    if not a.no_fp64:
        k64 = 2
        h64 = make(S.SC_FP64)
        h64.rk4_steps(2)
        d64, e64 = h64.diagnostics()
        h64.rk4_steps(1)
        ms64 = time_steps(h64, k64)
        h64.close()
        del h64
        fp64 = {"steps_per_s": k64 / (ms64 / 1e3), "ms_per_step": ms64 / k64,
                "speedup_fp32_over_fp64": (value / world) / (k64 / (ms64 / 1e3))}
        # compute ceiling: the FFT flop model (9 real 3D transforms per right-hand side,
        # 2.5 N log2 N flops each, 4 right-hand sides per step) against the measured FP64 FMA rate
        npts = float(n) * (a.ny or n) * (a.nz or n)
        flops = 4 * 9 * 2.5 * npts * np.log2(npts)
        peak64 = S.fp64_peak_probe()
        ach64 = flops / (ms64 / k64 / 1e3) / 1e12
        fp64["roofline"] = {"bound": "fp64", "achieved": ach64, "peak": peak64, "unit": "TFLOP/s",
                            "frac": ach64 / peak64,
                            "peak_source": "measured: sc_fp64_peak_probe (FP64 FMA loop, 8 chains per thread)",
                            "flop_model": "4 RHS x 9 real 3D FFTs x 2.5 N^3 log2 N^3 per step (%.3g flop)" % flops}
        b64 = 4 * 51 * 2.0 * F
        fp64["hbm_roofline"] = {"bound": "hbm", "achieved": b64 / (ms64 / k64 / 1e3) / 1e9, "peak": hbm,
                                "unit": "GB/s", "frac": b64 / (ms64 / k64 / 1e3) / 1e9 / hbm,
                                "bytes_model": "4 x 51 F per step, F = %.3g B (FP64)" % (2.0 * F)}
        # shells holding energy above the FP32 round-off floor of the total
        m = e64 > 1e-10 * float(np.sum(e64))
        fp64["fp32_vs_fp64_after_2_steps"] = {
            "Ek_max_rel_err": float(np.max(np.abs(e32[m] - e64[m]) / e64[m])),
            "Ek_shells_compared": int(np.sum(m)),
            "Ek_max_abs_err_over_total": float(np.max(np.abs(e32 - e64)) / float(np.sum(e64))),
            "dissipation_rel_err": abs(d32["dissipation"] - d64["dissipation"]) / d64["dissipation"],
            "energy_rel_err": abs(d32["energy"] - d64["energy"]) / d64["energy"],
            "max_div_fp32": d32["max_div"], "max_div_fp64": d64["max_div"]}

    # ---- discrete adjoint cost (FP32, T = 200, checkpoints every 20; 256^3 and 128^3) ----
    adjoint = None
    if not a.no_adjoint:
        import ctypes

        def adjoint_cost(na, Ta=200, Ka=20, host_gradient=False):
            p = S.default_params(na, S.SC_FP32, nu=NU, dt=DT, eps=EPS, fkmax=FKMAX)
            ha = S.SpectralNS(p)
            ha.set_stream(stream.cuda_stream)
            ha.init_field(seed=SEED, akp=AKP, u0=U0)
            init_a = ha.get_state()
            ha.rk4_steps(3)
            ha.set_state(*init_a)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ha.rk4_steps(Ta)
            torch.cuda.synchronize()
            t_fwd = time.perf_counter() - t0
            schedules = {}
            Ja = None

            def adj_device(nsteps, k):
                """sc_adjoint_rk4 with the gradient left in HBM (null host outputs)."""
                J = ctypes.c_double(0)
                SP._check(SP.lib().sc_adjoint_rk4(ha.h, nsteps, k, 8, 16, None, None, None, ctypes.byref(J)))
                return J.value

            for mode, budget in (("stage_inputs_kept", -1.0), ("checkpoint_recompute", 0.0)):
                ha.set_adjoint_budget(budget)
                ha.set_state(*init_a)
                adj_device(Ta, Ka)   # warm-up (allocates the store; the next call replays a graph)
                ha.set_state(*init_a)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                Ja = adj_device(Ta, Ka)
                torch.cuda.synchronize()
                t_adj = time.perf_counter() - t0
                schedules[mode] = {"kept_segments": ha.adjoint_kept_segments(),
                                   "adjoint_call_ms_per_step": 1e3 * t_adj / Ta,
                                   "cost_ratio": t_adj / t_fwd}
            if host_gradient:
                # the same call returning dJ/dv0 in host arrays (pageable memory)
                ha.set_adjoint_budget(-1.0)
                ha.set_state(*init_a)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                ha.adjoint(Ta, Ka, kmin=8, kmax=16)
                t_host = time.perf_counter() - t0
                schedules["stage_inputs_kept"]["with_host_gradient_ms_per_step"] = 1e3 * t_host / Ta
            ha.close()
            del ha, init_a
            torch.cuda.empty_cache()
            return {"grid": na, "steps": Ta, "checkpoint_every": Ka, "J": Ja,
                    "forward_ms_per_step": 1e3 * t_fwd / Ta, "schedules": schedules}

        adjoint = adjoint_cost(256, host_gradient=True)
        adjoint["grid_128"] = adjoint_cost(128)
        adjoint["note"] = ("cost_ratio = adjoint call through the C ABI, J returned and the gradient "
                           "left in HBM (forward sweep + any segment recompute + backward "
                           "sweep) / plain forward of the same steps; stage_inputs_kept: the default "
                           "memory budget keeps every segment's stage inputs (12 fields per step) from "
                           "the forward sweep; checkpoint_recompute: budget 0, state checkpoints every "
                           "K steps, the last segment's stage inputs recorded by the forward sweep and "
                           "every other segment recomputed; grid_128: the same at 128^3")

    # ---- LES at 256^3 FP32: Smagorinsky (c1 = 0.17^2) and dynamic (update every 10) ----
    les = None
    if not a.no_les:
        les = {"grid": 256, "nu": 1e-4, "dt": 1e-3, "init": "E(k) ~ k^-5/3 on 2 <= k <= 85, E = 0.5"}
        for sgs, name in ((S.SC_SGS_SMAG, "smagorinsky"), (S.SC_SGS_DYNSMAG, "dynamic")):
            p = S.default_params(256, S.SC_FP32, nu=1e-4, dt=1e-3, sgs=sgs, c1=0.17 ** 2)
            hl = S.SpectralNS(p)
            hl.set_stream(stream.cuda_stream)
            hl.init_field(seed=SEED, kind=1, u0=U0, kmin=2.0, kmax=85.0)
            hl.rk4_steps(3)
            kl = 20   # two dynamic-coefficient updates
            ms_l = time_steps(hl, kl)
            d_l, _ = hl.diagnostics()
            hl.close()
            del hl
            les[name] = {"steps_per_s": kl / (ms_l / 1e3), "ms_per_step": ms_l / kl,
                         "energy_after": d_l["energy"], "cs2": d_l["cs2"]}
            # field-pass model: P = 3 + 4 n_i + 4 n_f + 12 with 12 inverse and 9 forward
            # transforms (P = 99); the dynamic procedure adds 42 transforms (168 F) on one
            # step in ten
            Fl = 129 * 256 * 256 * 8.0
            bl = 4 * 99 * Fl + (168 * Fl / 10 if sgs == S.SC_SGS_DYNSMAG else 0.0)
            gbs = bl / (ms_l / kl / 1e3) / 1e9
            les[name]["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                                     "frac": gbs / hbm, "bytes_per_step": bl,
                                     "bytes_model": "4 x 99 F per step%s, F = %.3g B" %
                                     (" + 168 F / 10" if sgs == S.SC_SGS_DYNSMAG else "", Fl)}
        torch.cuda.empty_cache()

    # ---- batched 2D ensemble: 24 x 256^2, 24 x 512^2, 16 x 1024^2 ----
    ensemble = None
    if not a.no_ensemble:
        sizes = [256] * 24 + [512] * 24 + [1024] * 16
        dts, nus = [], []
        for n2 in sizes:
            kmax = 2.0 * (n2 // 2) / 3.0
            dt2 = 0.5 / n2                      # CFL ~0.5 at |u| ~ 1 (E = 0.5)
            dts.append(dt2)
            nus.append(1.0 / (kmax ** 8 * dt2))  # nu8 kmax^8 dt = 1
        ens = S.Ensemble2D(sizes, dts, nus, 0.01, S.SC_FP32)
        ens.set_stream(stream.cuda_stream)
        ens.init([-(i + 1) for i in range(len(sizes))], kpeak=6.0, energy=0.5)
        ens.rk4_steps(5, 0)   # the first call runs the launch-shape autotuner
        var, shape, tune_ms = ens.variant()
        torch.cuda.synchronize()
        ke = 1000
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ens.rk4_steps(ke, 0)
        e1.record(stream)
        torch.cuda.synchronize()
        t_b = e0.elapsed_time(e1) / 1e3
        k1 = 50
        e0.record(stream)
        ens.rk4_steps(k1, 2)
        e1.record(stream)
        torch.cuda.synchronize()
        t_1 = e0.elapsed_time(e1) / 1e3
        ensemble = {"members": len(sizes), "sizes": "24x256^2 + 24x512^2 + 16x1024^2", "alpha": 0.01,
                    "dt": "0.5/N", "nu8": "1/(kmax^8 dt), kmax = N/3",
                    "graph": ens.uses_graph(), "steps": ke,
                    "autotuner": {"variant": var, "shape": shape,
                                  "ms_per_step_by_variant": [round(t, 4) for t in tune_ms]},
                    "ensemble_steps_per_s": ke / t_b,
                    "one_at_a_time_steps_per_s": k1 / t_1,
                    "speedup_vs_one_at_a_time": (ke / t_b) / (k1 / t_1)}
        # field-pass model of the 2D step: per RHS P = 1 + 2 n_i + 2 n_f + 4 with the
        # inverse transforms of u, v, w (n_i = 3) and the forward ones of (u w, v w) (n_f = 2)
        F2 = sum((m // 2 + 1) * m * 8.0 for m in sizes)
        b2 = 4 * 15 * F2
        gb2 = b2 * ke / t_b / 1e9
        ensemble["roofline"] = {"bound": "hbm", "achieved": gb2, "peak": hbm, "unit": "GB/s",
                                "frac": gb2 / hbm, "bytes_per_step": b2,
                                "bytes_model": "4 x 15 F per step summed over the members, sum F = %.3g B "
                                               "(the whole ensemble's fields fit in the 129 MB L2)" % F2}
        ens.close()
        del ens

    # ---- opt-in: the other steppers on the headline grid ----
    schemes = None
    if not a.no_schemes:
        schemes = {"grid": n, "dtype": "f32", "om": 5.0, "band": [1.0, 2.5], "pr": 0.7,
                   "note": "passes through the public API; the rotating pass sums force_rot's band on the "
                           "device and replays passes >= 2 as one captured graph; the rotating-scalar pass "
                           "reads its band sums on the host; ab2v_pass checks its status every call"}

        def time_calls(fn, k):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            barrier()
            torch.cuda.synchronize()
            e0.record(stream)
            fn(k)
            e1.record(stream)
            torch.cuda.synchronize()
            barrier()
            return e0.elapsed_time(e1)

        hs = make(S.SC_FP32)
        start = hs.get_state()
        ks = max(a.steps, 4)
        hs.rot_steps(2, om=5.0, fk1=1.0, fk2=2.5)   # Euler half step and restart
        ms_r = time_calls(lambda k: hs.rot_steps(k, om=5.0, fk1=1.0, fk2=2.5), ks)
        hs.set_state(*start)
        hs.set_scalar(start[0])
        hs.rot_scalar_steps(2, om=5.0, fk1=1.0, fk2=2.5, pr=0.7, scalarforced=True, epsphi=0.05)
        ms_s = time_calls(lambda k: hs.rot_scalar_steps(k, om=5.0, fk1=1.0, fk2=2.5, pr=0.7,
                                                        scalarforced=True, epsphi=0.05), ks)
        hs.set_state(*start)
        hs.ab2v_pass(DT)
        hs.ab2v_pass(DT)

        def ab2v(k):
            for _ in range(k):
                hs.ab2v_pass(DT)

        ms_v = time_calls(ab2v, ks)
        hs.close()
        del hs
        torch.cuda.empty_cache()
        for name, ms_x in (("rotating", ms_r), ("rotating_scalar", ms_s), ("ab2_variable_step", ms_v)):
            schemes[name] = {"passes": ks, "passes_per_s": ks / (ms_x / 1e3), "ms_per_pass": ms_x / ks}

    cpu = None
    if not a.no_cpu and rank == 0 and world == 1:
        cpu = cpu_baseline_leg(n)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
               "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (ran1 seed 1 initial field, as the reference generates it)",
               "config": workload_config(n, world),
               "gpu_launches": launches,
               "roofline": roofline,
               "step_model_bytes": step_bytes,
               "step_model_gbs": step_bytes / (ms_step / 1e3) / 1e9,
               "kernels": kernels,
               "clocks": clocks,
               "e2e": e2e,
               "fp64": fp64,
               "adjoint": adjoint,
               "les256": les,
               "ensemble2d": ensemble,
               "cpu_baseline": cpu}
        if schemes is not None:
            out["schemes"] = schemes
        print(json.dumps(out), flush=True)
    if dist:
        td.destroy_process_group()
    return 0


def run_cpu_configs(a):
    """CPU seconds per step of the oracle port on the configurations beside
    the headline, on every host core: forced DNS 128^3 (the threaded step,
    double build), LES 256^3 (the oracle's rk4_run, transforms on every core,
    pointwise work on one), the 2D ensemble (each member's Lawson RK4 step in
    turn).  A bounded sample of each, stated in the output."""
    import numpy as np
    from oracle import spectral_ref as R
    workers = len(os.sched_getaffinity(0))
    R.WORKERS = workers
    out = {"cores": workers, "kind": "port"}
    # C1: forced DNS 128^3, nu 0.01, dt 2e-3, double build
    v = R.initialize_dealiased(128, 128, 128, SEED, AKP, U0, 2.0 * 64 / 3.0)
    from oracle.cpu_step import CpuRK4
    st = CpuRK4(R.Grid(R.Params(nx=128, nu=0.01, dt=2e-3)), workers, np.complex128)
    vv = [np.array(x) for x in v]
    st.step(vv)
    t = cpu_time_steps(st, vv, 5)
    st.close()
    out["dns128_fp64"] = {"s_per_step": t, "sample": "5 whole RK4 steps after 1 warm-up, threaded port"}
    # C3: LES 256^3, nu 1e-4, dt 1e-3, c1 = 0.17^2
    v = R.initialize_dealiased(256, 256, 256, SEED, AKP, U0, 2.0 * 128 / 3.0, spectrum_kind="kolmogorov",
                               kmin=2.0, kmax=85.0)
    for sgs in ("smag", "dynsmag"):
        g = R.Grid(R.Params(nx=256, nu=1e-4, dt=1e-3, sgs=sgs, c1=0.17 ** 2))
        state = {"cs2": 0.0, "update": True} if sgs == "dynsmag" else None
        t0 = time.perf_counter()
        R.rk4_step(v, g, state, dyn_update=True)
        out["les256_" + sgs] = {"s_per_step": time.perf_counter() - t0,
                                "sample": "1 RK4 step (dynamic: its coefficient refreshed, one step in ten "
                                          "does this), oracle restatement"}
    # C5: 24 x 256^2, 24 x 512^2, 16 x 1024^2, members one at a time
    tot = 0.0
    for n2, count in ((256, 24), (512, 24), (1024, 16)):
        kmax = 2.0 * (n2 // 2) / 3.0
        dt2 = 0.5 / n2
        p2 = R.Params2D(n=n2, alpha=0.01, nu8=1.0 / (kmax ** 8 * dt2), dt=dt2)
        w = R.initialize2d(n2, 1)
        R.rk4_step2d(w, p2)
        t0 = time.perf_counter()
        R.rk4_step2d(w, p2)
        tot += count * (time.perf_counter() - t0)
    out["ensemble2d"] = {"s_per_step": tot, "sample": "one RK4 step of one member of each size, times the "
                                                      "member count, oracle restatement"}
    print(json.dumps(out), flush=True)
    return 0


def main():
    a = parse()
    if a.cpu_configs:
        return run_cpu_configs(a)
    if a.impl == "reference":
        return run_reference(a)
    return run_ours(a)


if __name__ == "__main__":
    sys.exit(main())
