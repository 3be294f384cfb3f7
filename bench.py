"""Benchmark of the FSIBE_2D fluid step + flexible-beam coupling on GB300.

Workload (the precision configuration): periodic box 4 x 4, nx = ny = 1024, ns = 256 beam
nodes, Re = 500, dt = 5e-5, clamped flexible beam (length 1, thickness 4 dx, leading edge
(1, 2), EI = 0.1, density ratio 1), penalization 1e-3 over a 2-cell smoothed mask, initial
vorticity = seeded N(0, 1e-3) noise low-passed to |k| <= 8.  Inputs are seeded synthetic
fields of exactly that shape (there is no dataset).

One step = one full time step of the reference's loop (mask -> vorticity AB2 step with the
pressure solve -> beam forces -> beam Newton solve).  `value` is the FP32-compensated form's
throughput in Mcell-steps/s with the state resident in HBM; the FP64 plain form is measured
on the same workload and reported beside it, with the FP32 form's relative L2 vorticity error
against the FP64 form after a fixed number of steps.  `e2e` runs through the C ABI with
host buffers (initial field upload, a per-step beam_data read-back, the final field read).

--impl reference times the CPU restatement of the reference (oracle/, FP64, OpenMP on every
host core): the reference's own Fortran/FFTW/MKL build cannot be built on this machine
(no Fortran compiler, FFTW, MKL or LAPACK).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

NX = NY = 1024
NS = 256
RE = 500.0
DT = 5.0e-5
L2_BYTES = 129 * 1024 * 1024
METRIC = "Mcell-steps/s at 1024^2 (FP32-compensated form; FP64 plain form beside it)"


def seeded_vorticity(n, K=8, sigma=1e-3, seed=0):
    rng = np.random.default_rng(seed)
    w = rng.normal(0.0, sigma, (n, n))
    wk = np.fft.rfft2(w)
    kx = np.fft.rfftfreq(n, 1.0 / n)
    ky = np.fft.fftfreq(n, 1.0 / n)
    wk[(kx[None, :] ** 2 + ky[:, None] ** 2) > K * K] = 0.0
    return np.fft.irfft2(wk, s=(n, n))


def bench_config(world):
    """The workload's `config`, identical in both arms (the reference arm runs the same
    workload on the host cores)."""
    return {"workload": "precision form: 1024^2 box 4x4, ns=256, Re=500, dt=5e-5, clamped flexible beam EI=0.1, mu=1, eta=1e-3",
            "nx": NX, "ny": NY, "ns": NS, "parallelism": f"replicas x{world}" if world > 1 else "single run",
            "l2": "GPU arm: flushed between timed steps (256 MB write outside the event pair)"}


def params(precision):
    from fsibe_2d_gb300 import make_params
    return make_params(nx=NX, ny=NY, ns=NS, Re=RE, dt=DT, precision=precision)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def start(self):
        def run():
            q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap")
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                         timeout=5).stdout.strip()
                    if out:
                        self.samples.append([v.strip() for v in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 3 + i and s[3 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# Fields each fused fluid kernel reads + writes once per launch, FP32-compensated form with the
# split launches of fsibe_step.  One real field of nx*ny values, or one half spectrum of
# nx/2*ny complex values, is one pass; a spectrum touched only on its rows kx < kcut (every
# row above is zero after the 2/3 rule) counts f = kcut / (nx/2) of a pass:
#   nl_y      R A, B, W, Wlo, M (f)      W W, Wlo, M (1), Tu, Tv, Tw, Tdx, Tdy, Tsa, Tsb (f)
#   nl_adv    R Tdx, Tdy (f), u, v       W A, B (f)
#   nl_x      R Tdx, Tdy (f), u, v, mask, mvx, mvy      W A, B (f)   (one launch, FSIBE_NL_SPLIT=0)
#   press_x   R Tu, Tv, Tw (f), mask, mvx, mvy, vor_mean      W u, v, vor_mean, P1, P2
#   press_y   R P1, P2                   W Tq
#   press_fin R Tq, u, v                 W press
# (nl_pen and stress_x touch only the rows near the beam.)
# (k_press_fin has no line: in the step it forms only the rows the forces' stencils reach, so
# its bytes depend on where the beam is)
# k_nl_y (FP32C): reads A, B, W, W_lo, M (f), writes W, W_lo, M and the five spectra Tu, Tv,
# Tw, T dy(omega), T sigma_b (f); the readers form i kx Tw and i kx Tu as they load
PASSES = {"nl_y": lambda f: 10 * f + 3, "nl_adv": lambda f: 4 * f + 2, "nl_x": lambda f: 4 * f + 5,
          "press_x": lambda f: 3 * f + 9, "press_y": lambda f: 3}


def kcut_fraction(nx, ny):
    """kcut / (nx/2): the first kx whose modes the 2/3 rule removes for every ky
    (dealiase_mask.f90:9-26, kx^2/kxt^2 >= 1 with kxt = 2/3 (nx/2 - 1))."""
    kxt = 2.0 / 3.0 * (nx // 2 - 1)
    kcut = next((kx for kx in range(nx // 2) if kx * kx / (kxt * kxt) >= 1.0), nx // 2)
    return kcut / (nx // 2)


def algorithmic_bytes(kernel, nx, ny, rbytes):
    """Bytes one launch must move: the fields it reads and writes, each once."""
    if kernel not in PASSES:
        return 0
    return int(round(PASSES[kernel](kcut_fraction(nx, ny)) * nx * ny * rbytes))


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return json.load(open(p)), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def ncu_traffic(kernel, precision):
    p = os.path.join(HERE, "profiles", "roofline_traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    return d.get(f"{kernel}:{precision}")


def gpu_arm(args):
    import torch
    import fsibe_2d_gb300 as F
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)  # a capturable (non-legacy) stream for the library and the events
    torch.cuda.set_stream(stream)
    w0 = seeded_vorticity(NX)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)

    def timed_steps(run, K):
        """K steps, each bracketed by CUDA events on the run's stream, L2 flushed between."""
        ms = 0.0
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        for k in range(K):
            flush.add_(1.0)
            ev[k][0].record(stream)
            st = run._lib.fsibe_step(run._ctx)
            ev[k][1].record(stream)
            if st:
                raise RuntimeError(f"fsibe_step status {st}")
        torch.cuda.synchronize(dev)
        for a, b in ev:
            ms += a.elapsed_time(b)
        return ms

    results = {}
    for prec, tag in ((F.FSIBE_FP32C, "fp32c"), (F.FSIBE_FP64, "fp64")):
        run = F.Run(params(prec))
        run.set_stream(stream.cuda_stream)
        run.use_graph(True)
        run.init_fields(w0)
        for _ in range(args.warmup):
            run.step()
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        sampler = ClockSampler(local) if tag == "fp32c" else None
        if sampler:
            sampler.start()
        ms = timed_steps(run, args.steps)
        clocks = sampler.stop() if sampler else None
        if world > 1:
            t = torch.tensor([ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        s = run.scalars()
        if s.status:
            raise RuntimeError(f"device status {s.status}")
        kt = kernel_times(run, 3)
        results[tag] = {"ms": ms, "clocks": clocks, "kernels": kt, "launches": run.launches_per_step(),
                        "newton_iters": s.newton_iters, "tiles": run.tiles()}
        run.close()

    # FP32-compensated vs FP64 on the GPU from the same seed (relative L2 of vorticity)
    err_steps = args.err_steps
    r64, r32 = F.Run(params(F.FSIBE_FP64)), F.Run(params(F.FSIBE_FP32C))
    r64.init_fields(w0)
    r32.init_fields(w0)
    d64, d32 = r64.time_step(err_steps), r32.time_step(err_steps)
    v64, v32 = r64.vort(), r32.vort()
    rel_err = float(np.linalg.norm(v32 - v64) / np.linalg.norm(v64))
    drag_err = float(np.abs(d32[:, 10] - d64[:, 10]).max() / np.abs(d64[:, 10]).max())
    r64.close()
    r32.close()

    # end to end through the C ABI with host buffers
    e2e_steps = args.steps
    r = F.Run(params(F.FSIBE_FP32C))
    r.use_graph(True)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    r.init_fields(w0)
    for _ in range(e2e_steps):
        r.step()
        r.scalars()  # per-step device->host read of the beam_data row
    vfin = r.vort()
    t1 = time.perf_counter()
    r.close()
    e2e_val = NX * NY * e2e_steps / (t1 - t0) / 1e6
    del vfin

    ens = ensemble_c4(F, args, rank, world)
    adj = adjoint_c3(F) if rank == 0 else None
    large = large_run_c5(F, measured_peaks()[0]) if rank == 0 and not args.no_large else None

    cells = NX * NY * world
    val32 = cells * args.steps / (results["fp32c"]["ms"] * 1e-3) / 1e6
    val64 = cells * args.steps / (results["fp64"]["ms"] * 1e-3) / 1e6
    peaks, which = measured_peaks()
    kt = results["fp32c"]["kernels"]
    top = max((k for k in kt if k in PASSES), key=lambda k: kt[k])
    top_ms = kt[top]
    ab = algorithmic_bytes(top, NX, NY, 4)
    achieved = ab / (top_ms * 1e-3) / 1e9
    traffic = ncu_traffic(top, "fp32c")
    roof = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / peaks["hbm_gbs"], 3), "traffic": traffic, "peak_source": which,
            "algorithmic_bytes_per_launch": ab, "avg_launch_ms": round(top_ms, 5)}
    flops = measure_gemm_peaks(dev)
    cpu = cpu_baseline_sample() if rank == 0 else None
    if cpu is not None and os.environ.get("FSIBE_CPU_CONFIGS", "1") != "0":
        cpu["configs_median_of_3"] = cpu_baseline_configs()
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(val32, 2), "unit": "Mcell-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(results["fp32c"]["ms"] / args.steps, 5),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (seeded N(0,1e-3) vorticity, |k|<=8)",
            "config": bench_config(world), "cuda_graph": True,
            "fp64_value": round(val64, 2), "fp64_ms_per_step": round(results["fp64"]["ms"] / args.steps, 5),
            "fp32_over_fp64": round(val32 / val64, 3),
            "fp32_rel_l2_vorticity_vs_fp64": rel_err, "fp32_drag_rel_err_vs_fp64": drag_err, "error_steps": err_steps,
            "newton_iters_last_step": results["fp32c"]["newton_iters"],
            "kernel_ms_per_step_fp32c": {k: round(v, 5) for k, v in kt.items()},
            "kernel_ms_per_step_fp64": {k: round(v, 5) for k, v in results["fp64"]["kernels"].items()},
            "adjoint_over_forward": adj["ratio_40_snapshots"] if adj else None,
            "adjoint": adj,
            "measured_gemm_tflops": flops,
            "roofline": roof,
            "roofline_4096": large_roofline(large),
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_val, 2), "unit": "Mcell-steps/s", "h2d_bytes_per_step": int(8 * NX * NY / e2e_steps),
                    "d2h_bytes_per_step": int(8 * 21 + 8 * NX * NY / e2e_steps)},
            "gpu_launches": results["fp32c"]["launches"] * args.steps,
            "clocks": results["fp32c"]["clocks"],
            "ensemble": ens,
            "large_run": large,
            "autotuned_x_tiles": {tag: dict(zip(("nl_x", "press_x", "press_fin"), results[tag]["tiles"]))
                                  for tag in ("fp32c", "fp64")},
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def large_roofline(large):
    """The 4096^2 run's dominant fused kernel against the HBM peak: there the fields exceed L2,
    so its algorithmic bytes over its live time is an HBM fraction."""
    if not large or not large.get("hbm_roofline"):
        return None
    hr = large["hbm_roofline"]
    k = max(hr, key=lambda q: hr[q]["us"])
    peaks, which = measured_peaks()
    return {"bound": "hbm", "kernel": k, "achieved": hr[k]["GB/s"], "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": hr[k]["frac"], "traffic": ncu_traffic(k, "fp32c_4096"), "peak_source": which,
            "algorithmic_bytes_per_launch": hr[k]["bytes"], "avg_launch_ms": round(hr[k]["us"] * 1e-3, 5),
            "workload": "4096^2 large run, FP32-compensated"}


def large_run_c5(F, peaks, err_steps=1000):
    """The large single run: 4096^2, box 8x8, Re=2000, clamped beam ns=1024, EI=0.05, mu=2,
    eta=1e-4, dt=1e-5, seeded |k|<=32 noise of amplitude 1e-3, FP32-compensated form.  Cell-steps/s
    from the CUDA graph (the working set, about 2 GB, exceeds L2: no flush is needed), each
    fused fluid kernel's algorithmic bytes over its live time against the HBM peak, and the
    drag/lift error against an FP64 run over the first err_steps steps."""
    n = 4096
    kw = dict(nx=n, ny=n, ns=1024, xl=8.0, yl=8.0, Re=2000.0, dt=1e-5, EI=0.05, mu=2.0, eps=1e-4, x0=2.0, y0=4.0)
    w = seeded_vorticity(n, K=32, sigma=1e-3, seed=2)
    g32 = F.Run(F.make_params(precision=F.FSIBE_FP32C, **kw))
    g32.init_fields(w)
    r32 = g32.time_step(err_steps)
    kt = kernel_times(g32, 10)
    g32.use_graph(True)
    g32.time_step(3)
    K = 50
    ms = g32.time_steps(K) / K
    g32.close()
    g64 = F.Run(F.make_params(precision=F.FSIBE_FP64, **kw))
    g64.init_fields(w)
    r64 = g64.time_step(err_steps)
    g64.close()
    drag_err = float(np.linalg.norm(r32[:, 10] - r64[:, 10]) / np.linalg.norm(r64[:, 10]))
    lift_err = float(np.linalg.norm(r32[:, 11] - r64[:, 11]) / np.linalg.norm(r64[:, 10:12]))
    roof = {}
    for k, v in kt.items():
        ab = algorithmic_bytes(k, n, n, 4)
        if ab:
            gbs = ab / (v * 1e-3) / 1e9
            roof[k] = {"us": round(v * 1e3, 1), "bytes": ab, "GB/s": round(gbs, 1), "frac": round(gbs / peaks["hbm_gbs"], 3)}
    return {"workload": "4096^2 box 8x8, Re=2000, ns=1024, EI=0.05, mu=2, eta=1e-4, dt=1e-5, FP32-compensated",
            "ms_per_step": round(ms, 4), "value": round(n * n / (ms * 1e-3) / 1e6, 1), "unit": "Mcell-steps/s",
            "kernel_ms_per_step": {k: round(v, 4) for k, v in kt.items()},
            "hbm_roofline": roof, "error_steps": err_steps,
            "drag_rel_err_vs_fp64": drag_err, "lift_rel_err_at_force_scale_vs_fp64": lift_err}


def adjoint_c3(F):
    """The adjoint configuration: flat plate of length 1 at 10 degrees incidence, 512^2 box
    4x4, Re=200, eta=1e-3, dt=1e-4, 2000 steps, mean drag over the last 1000, seeded
    band-limited initial vorticity (amplitude 1e-2).  Wall time of the gradient (with respect
    to the initial vorticity, the mask field and nu) over the wall time of the forward run."""
    n, steps, avg_from = 512, 2000, 1001
    p = F.make_params(nx=n, ny=n, ns=n // 4, Re=200.0, dt=1e-4, eps=1e-3, cfl=10.0, precision=F.FSIBE_FP64,
                      angle_beam=10.0, iFLUSI=0, iSaveBeam=0, iMotion=0)
    r = F.Run(p)
    w0 = seeded_vorticity(n, K=8, sigma=1e-2, seed=1)
    r.init_fields(w0)
    r.drag_objective(w0, 20, 11)
    t0 = time.perf_counter()
    J = r.drag_objective(w0, steps, avg_from)
    t_fwd = time.perf_counter() - t0
    out = {"workload": "512^2 flat plate at 10 deg, Re=200, eta=1e-3, dt=1e-4, 2000 steps, mean drag of the last 1000",
           "forward_s": round(t_fwd, 4), "J": J}
    for snaps, key in ((40, "40_snapshots"), (steps, "all_states")):
        t0 = time.perf_counter()
        Jg, gv, gm, gnu, info = r.drag_gradient(w0, steps, avg_from, snapshots=snaps)
        t = time.perf_counter() - t0
        out[f"gradient_s_{key}"] = round(t, 4)
        out[f"ratio_{key}"] = round(t / t_fwd, 3)
        out[f"forward_steps_{key}"] = info.forward_steps
    r.close()
    return out


def ensemble_c4(F, args, rank=0, world=1):
    """The batched configuration: 48 runs at 256^2, 12 at 512^2 and 4 at 1024^2, ns = nx/4,
    FP32-compensated, seeded parameters (Re uniform in [100, 1000], EI log-uniform in [0.01, 1],
    density ratio uniform in [0.5, 5]); one graph launch advances a rank's runs by one step.
    With several ranks the runs are shared out by cost (fsibe_2d_gb300.sharding, no exchange
    on the data path) and the step time is the slowest rank's."""
    from fsibe_2d_gb300.sharding import ShardedEnsemble
    rng = np.random.default_rng(4)
    ps = []
    for n, count in ((256, 48), (512, 12), (1024, 4)):
        for _ in range(count):
            ps.append(F.make_params(nx=n, ny=n, ns=n // 4, precision=F.FSIBE_FP32C, dt=5e-5,
                                    Re=float(rng.uniform(100, 1000)), EI=float(10 ** rng.uniform(-2, 0)),
                                    mu=float(rng.uniform(0.5, 5))))
    ens = ShardedEnsemble(ps, rank, world)
    ens.init_fields(lambda i: seeded_vorticity(ps[i].nx, seed=100 + i))
    ens.step(max(args.warmup, 3))
    K = max(args.steps // 2, 5)
    ms = ens.ens.time_steps(K) if ens.ens else 0.0
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX, group=dist.new_group(backend="gloo"))
        ms = float(t.item())
    cells = sum(p.nx * p.ny for p in ps)
    ens.close()
    return {"workload": "48 x 256^2 + 12 x 512^2 + 4 x 1024^2 runs, ns=nx/4, FP32-compensated, seeded parameters",
            "runs": len(ps), "ranks": world, "steps": K, "ms_per_step": round(ms / K, 5),
            "value": round(cells * K / (ms * 1e-3) / 1e6, 2), "unit": "Mcell-steps/s"}


def measure_gemm_peaks(dev):
    """FP64 (DGEMM 4096^3) and FP32 (SGEMM 8192^3, TF32 off) throughput through cuBLAS, the
    denominators for the FP64 form's compute roofline."""
    import torch
    out = {}
    torch.backends.cuda.matmul.allow_tf32 = False
    for dt, n, tag in ((torch.float64, 4096, "fp64"), (torch.float32, 8192, "fp32")):
        a = torch.randn(n, n, dtype=dt, device=dev)
        b = torch.randn(n, n, dtype=dt, device=dev)
        for _ in range(2):
            torch.matmul(a, b)
        torch.cuda.synchronize(dev)
        best = 1e30
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize(dev)
            best = min(best, e0.elapsed_time(e1))
        out[tag] = round(2.0 * n ** 3 / (best * 1e-3) / 1e12, 2)
        del a, b
    return out


def kernel_times(run, nsteps):
    import ctypes as C
    from fsibe_2d_gb300 import library
    lib = library()

    class KT(C.Structure):
        _fields_ = [("name", C.c_char * 32), ("ms_total", C.c_float), ("launches", C.c_int32)]
    lib.fsibe_kernel_times.argtypes = [C.c_void_p, C.c_int, C.POINTER(KT), C.c_int, C.POINTER(C.c_int)]
    out = (KT * 32)()
    n = C.c_int()
    st = lib.fsibe_kernel_times(run._ctx, nsteps, out, 32, C.byref(n))
    if st:
        raise RuntimeError(f"fsibe_kernel_times status {st}")
    return {out[i].name.decode(): out[i].ms_total / nsteps for i in range(n.value)}


def oracle_steps(nsteps, threads, p=None, w=None):
    """Wall time of nsteps AB2 steps of the oracle (after the start-up step), default the
    headline workload."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import pyoracle
    from fsibe_2d_gb300 import FSIBE_FP64
    used = pyoracle.set_threads(threads)
    r = pyoracle.OracleRun(p if p is not None else params(FSIBE_FP64))
    r.init_fields(w if w is not None else seeded_vorticity(NX))
    r.time_step(1)  # start-up step outside the timing
    t0 = time.perf_counter()
    r.time_step(nsteps)
    dt = time.perf_counter() - t0
    r.close()
    return dt, used


def cpu_baseline_sample():
    threads = os.cpu_count() or 1
    n = int(os.environ.get("FSIBE_CPU_SAMPLE_STEPS", "8"))
    dt, used = oracle_steps(n, threads)
    return {"value": round(NX * NY * n / dt / 1e6, 3), "unit": "Mcell-steps/s", "cores": used, "kind": "port",
            "sample": f"{n} FP64 AB2 steps of the same 1024^2 workload (after the start-up step), oracle/ C++ OpenMP"}


# The benchmark table's single-run workloads for the CPU samples: (name, make_params keywords,
# seed field (n, K, seed), AB2 steps a sample)
CPU_CONFIGS = (
    ("C1 256^2 plain FP64", dict(nx=256, ny=256, ns=64, Re=100.0, dt=2e-4), (256, 8, 0), 60),
    ("C2 1024^2 precision form", dict(nx=NX, ny=NY, ns=NS, Re=RE, dt=DT), (NX, 8, 0), 8),
    ("C5 4096^2 large run", dict(nx=4096, ny=4096, ns=1024, xl=8.0, yl=8.0, Re=2000.0, dt=1e-5, EI=0.05,
                                 mu=2.0, eps=1e-4, x0=2.0, y0=4.0), (4096, 32, 2), 2),
)


def cpu_baseline_configs(repeats=3):
    """The oracle's throughput on the host cores at C1, C2 and C5: the median of `repeats`
    samples each (a bounded sample: a few seconds of CPU work per configuration)."""
    from fsibe_2d_gb300 import make_params, FSIBE_FP64
    threads = os.cpu_count() or 1
    out = {}
    for name, kw, (n, K, seed), steps in CPU_CONFIGS:
        p = make_params(precision=FSIBE_FP64, **kw)
        w = seeded_vorticity(n, K=K, seed=seed)
        vals, used = [], 1
        for _ in range(repeats):
            dt, used = oracle_steps(steps, threads, p, w)
            vals.append(kw["nx"] * kw["ny"] * steps / dt / 1e6)
        out[name] = {"value": round(statistics.median(vals), 3), "unit": "Mcell-steps/s", "samples": [round(v, 3) for v in vals],
                     "steps_per_sample": steps, "cores": used}
    return out


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    total_dt = 0.0
    # a bounded sample: at most 200 CPU steps (about 10 s on 16 cores) whatever --steps says
    K = min(args.steps, int(os.environ.get("FSIBE_REF_MAX_STEPS", "200")))
    for _ in range(min(args.warmup, 3)):
        oracle_steps(1, threads)
    dt, used = oracle_steps(K, threads)
    total_dt += dt
    val = NX * NY * K / total_dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(val, 3), "unit": "Mcell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total_dt / K, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded N(0,1e-3) vorticity, |k|<=8)",
        "config": bench_config(world),
        "cpu_baseline": {"value": round(val, 3), "unit": "Mcell-steps/s", "cores": used, "kind": "port",
                         "sample": f"{K} FP64 AB2 steps at 1024^2 (CPU restatement; the Fortran/FFTW/MKL build is unavailable here)"},
        "e2e": {"value": round(val, 3), "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# The workloads of --profile-case: (make_params keywords, seed field (n, K, seed))
PROFILE_CASES = {
    "c2": (dict(nx=NX, ny=NY, ns=NS, Re=RE, dt=DT), (NX, 8, 0)),
    "c5": (dict(nx=4096, ny=4096, ns=1024, xl=8.0, yl=8.0, Re=2000.0, dt=1e-5, EI=0.05, mu=2.0, eps=1e-4,
                x0=2.0, y0=4.0), (4096, 32, 2)),
}


def profile_case(name, precision, steps):
    """A short run of one workload with the CUDA graph off (every kernel its own launch, the
    start-up step first), for ncu captures: `python bench.py --profile-case c5 --precision 1
    --steps 3`.  Prints the status and the autotuned tile heights."""
    import fsibe_2d_gb300 as F
    kw, (n, K, seed) = PROFILE_CASES[name]
    r = F.Run(F.make_params(precision=precision, **kw))
    r.init_fields(seeded_vorticity(n, K=K, seed=seed))
    r.time_step(steps)
    print("status", r.scalars().status, "tiles", r.tiles())
    r.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 1000 steps keep the timed region (about 0.5 s) long enough for the clock sampler
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--err-steps", type=int, default=2000)
    ap.add_argument("--no-large", action="store_true", help="skip the 4096^2 large-run report")
    ap.add_argument("--profile-case", choices=sorted(PROFILE_CASES), help="run --steps steps of a workload for ncu")
    ap.add_argument("--precision", type=int, default=1, help="with --profile-case: 0 FP64, 1 FP32-compensated")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args.profile_case, args.precision, args.steps)
        return
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
