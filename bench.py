#!/usr/bin/env python
"""Krylov time-propagation benchmark on one GB300: state-steps/s.

A step is one TDSE.update of a state vector (H0 half-phases + the field-dressed
Krylov exponential); state-steps/s = vectors x steps / time.

Headline (``value``): the batched mixed-precision form on the thermal-ensemble
configuration — asymmetric top (A, B, C = 9.0, 5.0, 3.2 cm^-1, Watson A,
D2), J = 0..30 (dim 39,711), the T = 5 K ensemble (states with Boltzmann
weight >= 1e-5, padded to 4096 vectors), DC 20 kV/cm + 1e12 W/cm^2 FWHM 500 fs
pulse at 35 deg, dt = 10 fs, per-vector Krylov tolerance 1e-8. Beside it the
plain FP64 path on the same workload (the ratio the metric names), the
observable error of the batched form against FP64, and the plain FP64 drop-in
configuration (J <= 40, dim 91,881, one vector, dt = 5 fs). Synthetic molecule
and fields are built in-process.

``--impl reference`` times the CPU restatement of the reference algorithm (the
oracle, numpy/scipy) on the host cores, one process per core, for the same
workload and metric.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Krylov state-steps/s: batched FP32/FP64 vs plain FP64, 1 GB300, err<=1e-6; p99 ms"
UNIT = "state-steps/s"


def parse(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50, help="timed steps of the batched ensemble")
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--jmax", type=int, default=30, help="J range of the ensemble workload")
    p.add_argument("--nvec", type=int, default=4096)
    p.add_argument("--jmax-plain", type=int, default=40, help="J range of the plain FP64 drop-in workload")
    p.add_argument("--plain-steps", type=int, default=400)
    p.add_argument("--acc-steps", type=int, default=0,
                   help="steps of the configured run with the FP64 check (0: the whole time grid, 3000 steps)")
    p.add_argument("--acc-every", type=int, default=10,
                   help="observables compared every this many steps (every step inside the pulse's FWHM)")
    p.add_argument("--acc-padded", type=int, default=7, help="padding vectors in the FP64 sample")
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="bound of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true", help="headline measurement only")
    p.add_argument("--plain-only", action="store_true",
                   help="only the plain drop-in step (FP64 and double-float products; for profiling)")
    p.add_argument("--widek-only", action="store_true",
                   help="only the wide-K (C1, KP = 32 tiles) batched mat-vec of every kind (for profiling)")
    p.add_argument("--matvec", choices=["auto", "tensor", "tensor_tmem", "fp32", "fp32_reg"], default="auto",
                   help="batched mat-vec kind: tensor-core K contraction (split TF32; A operands in shared "
                        "or tensor memory) or FP32 FMAs; auto: every kind timed on the first step's operator, "
                        "the fastest kept (richmol_gb300.tune)")
    p.add_argument("--serve-rate", type=float, default=2.0, help="requests per second of the serving sample")
    p.add_argument("--serve-duration", type=float, default=3.0, help="seconds of arrivals of the serving sample")
    p.add_argument("--serve-jmax", type=int, nargs=2, default=[10, 50], help="Jmax range of the requests")
    p.add_argument("--serve-tend", type=float, default=5.0, help="ps propagated per request (dt 10 fs)")
    p.add_argument("--serve-budget-gb", type=float, default=150.0)
    p.add_argument("--serve-load", type=float, default=0.7,
                   help="sustained serving sample: arrival rate as a fraction of the capacity the burst measured")
    p.add_argument("--serve-sustained-n", type=int, default=10,
                   help="requests of the sustained serving sample (0: skip it)")
    p.add_argument("--uneven-n", type=int, default=256, help="molecules of the uneven-size batch")
    p.add_argument("--uneven-jmax", type=int, nargs=2, default=[10, 50])
    p.add_argument("--uneven-steps", type=int, default=5)
    return p.parse_args(argv)


def dist_info():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def job_throughput(local_seconds, units_per_rank, ws, device="cpu"):
    """Whole-job rate: the units of all ranks over the slowest rank's time (max
    over ranks, one all-reduce when ws > 1). Returns (rate, max seconds)."""
    t = float(local_seconds)
    if ws > 1:
        import torch
        import torch.distributed as dist
        x = torch.tensor([t], dtype=torch.float64, device=device)
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        t = float(x.item())
    return ws * units_per_rank / t, t


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append(dict(sm=float(f[1]), smax=float(f[2]), hw=f[5], hwt=f[6], swt=f[7], pcap=f[8]))
            except ValueError:
                continue
        if not rows:
            return None
        reasons = set()
        for r in rows:
            for k, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"), ("swt", "sw_thermal_slowdown"),
                            ("pcap", "sw_power_cap")):
                if r[k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in rows), "sm_max_mhz": max(r["smax"] for r in rows),
                "reasons": sorted(reasons), "samples": len(rows)}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def load_traffic():
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


# ---------------------------------------------------------------------------
# CPU restatement (oracle) of the reference algorithm on the same workload
# ---------------------------------------------------------------------------
def to_oracle(T):
    from oracle.fixtures import from_cartens
    return from_cartens(T)


def cpu_reference_rate(wl, seconds, max_steps=None, warmup=1, vec=None):
    """State-steps/s of the oracle (reference algorithm in numpy/scipy, one
    host thread) on the first steps of the workload for one vector."""
    from oracle.cartens import add_cartens
    from oracle.tdse import OTDSE
    from richmol_gb300.convert_units import AUdip_x_Vm_to_invcm
    oh0 = to_oracle(wl.h0)
    oHac = to_oracle(wl.Hac)
    oHdc = None
    if wl.Hdc is not None:
        oHdc = to_oracle(wl.dip) * list(wl.dc)
        oHdc = oHdc * (-1 * AUdip_x_Vm_to_invcm())
    td = OTDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    v = td.init_state(oh0, temp=0) if vec is None else vec.reshape(1, -1).astype(np.complex128)
    n, t_run, i = 0, 0.0, 0
    while True:
        oHac.field(wl.field(tc[i]))
        H = oHac if oHdc is None else add_cartens(oHdc, oHac)
        t0 = time.perf_counter()
        v, _ = td.update(H, v, H0=oh0)
        dtm = time.perf_counter() - t0
        i += 1
        if i > warmup:
            n += 1
            t_run += dtm
        if t_run >= seconds or (max_steps is not None and n >= max_steps) or i >= len(tc):
            break
    return v.shape[0] * n / t_run, n, t_run


SINGLE_THREAD_ENV = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS", "BLIS_NUM_THREADS",
                     "VECLIB_MAXIMUM_THREADS", "NUMEXPR_NUM_THREADS")


def _reference_worker(args):
    """One host process: one vector of the ensemble workload (spawned; its
    BLAS thread pools are limited to one thread by the environment the parent
    set before starting the pool, which a spawned child reads when it imports
    numpy)."""
    jmax, nvec, idx, seconds, max_steps, warmup = args
    sys.path.insert(0, ROOT)
    from richmol_gb300 import workloads
    wl, ens = workloads.thermal_asym_top(Jmax=jmax, nvec=nvec)
    v = np.zeros(wl.dim, np.complex128)
    v[ens.index[idx % nvec]] = 1.0
    rate, n, t = cpu_reference_rate(wl, seconds, max_steps=max_steps, warmup=warmup, vec=v)
    return n, t, {k: os.environ.get(k) for k in SINGLE_THREAD_ENV}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, ws, rank, local):
    import ctypes
    import torch
    from richmol_gb300 import TDSE, _native, workloads
    from richmol_gb300.batch import Ensemble
    from richmol_gb300.device import context

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    ctx = context(local)
    fp64, fp32 = ctypes.c_double(), ctypes.c_double()
    _native.check(_native.lib().kr_probe_fp64(ctx, ctypes.byref(fp64)), ctx)
    _native.check(_native.lib().kr_probe_fp32(ctx, ctypes.byref(fp32)), ctx)
    peaks, peak_kind = load_peaks()
    if args.widek_only:
        return {"metric": "wide-K batched mat-vec only (--widek-only)", "unit": "ms",
                "wide_k_matvec": run_widek(args)}
    if args.plain_only:
        out = {"metric": "plain drop-in step only (--plain-only)", "unit": UNIT}
        out["plain_fp64_drop_in"] = run_plain(args, dev, peaks, peak_kind, fp64.value)
        out["plain_fp64_drop_in"]["df_products"] = run_plain(args, dev, peaks, peak_kind, fp64.value, products="df")
        return out

    # ---- batched ensemble: the headline --------------------------------------
    note("headline")
    t_build = time.time()
    wl, ensd = workloads.thermal_asym_top(Jmax=args.jmax, nvec=args.nvec)
    t_build = time.time() - t_build
    nvec, dim = args.nvec, wl.dim
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    nsteps = len(tc)
    ens = Ensemble(td, wl.h0, nvec, tol=1e-8, matvec=args.matvec, tune_cache=False)
    ens.load(ensd.vectors(dim))
    for i in range(args.warmup):
        ens.step(wl.hamiltonian(tc[i]))
    torch.cuda.synchronize()
    K = args.steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    l0 = ens.launches()
    plan_l0 = wl.Hac._plan().launches()
    kmax_seen = []
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for j in range(K):
            i = (args.warmup + j) % nsteps
            H = wl.hamiltonian(tc[i])
            ev[j][0].record()
            ens.step(H)
            ev[j][1].record()
            kmax_seen.append(ens.last_kmax)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    launches = (ens.launches() - l0) + (wl.Hac._plan().launches() - plan_l0)
    value, total_s = job_throughput(sum(step_ms) / 1e3, nvec * K, ws, dev)
    korder = np.bincount(ens.korder(), minlength=1)

    # dominant kernel (batched complex64 mat-vec) alone
    plan = wl.hamiltonian(tc[args.warmup]).device_operator()

    note("mat-vec kinds")

    def time_matvec(kind):
        _native.check(_native.lib().kr_batch_set_matvec(ens.handle, kind), ctx)
        em = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(6)]
        for a, b in em:
            a.record()
            _native.check(_native.lib().kr_batch_matvec(ens.handle, plan.op, ctypes.c_void_p(
                torch.cuda.current_stream().cuda_stream)), ctx)
            b.record()
        torch.cuda.synchronize()
        return statistics.median(a.elapsed_time(b) for a, b in em[1:]) / 1e3

    kinds = {"tensor": _native.KR_MATVEC_TENSOR, "tensor_tmem": _native.KR_MATVEC_TENSOR_TMEM,
             "fp32": _native.KR_MATVEC_FP32, "fp32_reg": _native.KR_MATVEC_FP32_REG}
    kind_s = {k: time_matvec(code) for k, code in kinds.items()}
    kind = ens.matvec  # the kind the ensemble steps with (picked by the autotuner with "auto")
    _native.check(_native.lib().kr_batch_set_matvec(ens.handle, kinds[kind]), ctx)
    mv_s = kind_s[kind]
    fma_mv, bytes_mv = plan.work()
    mv_flops = 2.0 * fma_mv * nvec
    mv_bytes = 8.0 * 2 * dim * nvec  # complex64 X in + Y out (factors are shared by all vectors)
    # ncu DRAM bytes of one launch at 4096 vectors (profiles/traffic.json), in proportion to the vectors
    tkey = {"fp32": "kb_matvec_per_launch_bytes_4096", "fp32_reg": "kb_matvec_zr_per_launch_bytes_4096",
            "tensor_tmem": "kb_matvec_tcp_tmem_per_launch_bytes_4096"}.get(kind, "kb_matvec_tc_per_launch_bytes_4096")
    t4096 = load_traffic().get(tkey)
    traffic = None if t4096 is None else int(round(t4096 * nvec / 4096))
    gbs = mv_bytes / mv_s / 1e9
    roofline = {
        "bound": "hbm", "achieved": round(gbs, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
        "frac": round(gbs / peaks["hbm_gbs"], 4), "traffic": traffic,
        "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
        "kernel": {"tensor": "kb_matvec_tcp (complex64 batched mat-vec, K contraction on tcgen05, A in shared memory)",
                   "tensor_tmem": "kb_matvec_tcp (complex64 batched mat-vec, K contraction on tcgen05, A in TMEM)",
                   "fp32": "kb_matvec (complex64 batched mat-vec, FP32 FMAs)",
                   "fp32_reg": "kb_matvec_zr (complex64 batched mat-vec, FP32 FMAs, register-tiled)"}[kind],
        "kind_choice": ({"tuned_ms": {k: round(v, 3) for k, v in ens.tuned.items()}}
                        if ens.tuned else {"fixed": kind}),
        "kernel_ms": round(mv_s * 1e3, 3),
        "kernel_ms_by_kind": {k: round(t * 1e3, 3) for k, t in kind_s.items()},
        "alg_bytes_per_launch": mv_bytes,
        "fp32": {"achieved_tflops": round(mv_flops / mv_s / 1e12, 2), "peak_tflops": round(fp32.value, 1),
                 "frac": round(mv_flops / mv_s / 1e12 / fp32.value, 4),
                 "peak_source": "measured FP32 FMA probe (kr_probe_fp32)", "flops_per_launch": mv_flops},
    }
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": args.warmup,
        "ms_per_step": round(total_s * 1e3 / K, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": ("c64 mat-vec (FP32 FMAs)" if kind.startswith("fp32") else
                                       "c64 mat-vec (K contraction as split-TF32 tcgen05 MMAs, FP32 accumulate)")
        + " / f64 Lanczos scalars, double-float state",
        "data": "synthetic",
        "config": {"workload": f"batched thermal ensemble: asymmetric top D2 Watson-A J=0..{args.jmax} "
                               f"(dim {dim}), T=5 K ensemble of {ensd.n_natural} states with weight>=1e-5 padded "
                               f"to {nvec} vectors, DC 20 kV/cm + 1e12 W/cm^2 FWHM 500 fs pulse at 35 deg, "
                               f"dt 10 fs, per-vector Krylov tolerance 1e-8",
                   "dim": dim, "nvec": nvec, "n_natural": ensd.n_natural, "jmax": args.jmax, "dt_fs": 10.0,
                   "tol": 1e-8, "l2": "inputs larger than L2 (state 2.6 GB, basis complex64)",
                   "parallelism": f"replicas x{ws}", "factor_build_s": round(t_build, 2),
                   "krylov_orders": {str(k): int(c) for k, c in enumerate(korder) if c},
                   "timed_window_ps": [float(tc[args.warmup % nsteps]), float(tc[(args.warmup + K - 1) % nsteps])]},
        "roofline": roofline,
        "gpu_launches": int(launches),
        "step_ms_p50": round(statistics.median(step_ms), 3),
        "step_ms_p99": round(float(np.percentile(step_ms, 99)), 3),
        "peaks_probe": {"fp64_tflops": round(fp64.value, 3), "fp32_tflops": round(fp32.value, 2)},
    }
    clocks = clk.summary()
    if clocks:
        out["clocks"] = clocks

    # ---- the same K steps through the pulse maximum (where the Krylov orders rise)
    note("pulse window")
    ip = int(np.argmin(np.abs(np.asarray(tc) - wl.pulse[0])))
    i_lo = max(args.warmup, ip - K // 2)
    ens.load(ensd.vectors(dim))
    for i in range(i_lo - args.warmup, i_lo):
        ens.step(wl.hamiltonian(tc[i]))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    kp = {}
    torch.cuda.synchronize()
    for j in range(K):
        H = wl.hamiltonian(tc[(i_lo + j) % nsteps])
        ev[j][0].record()
        ens.step(H)
        ev[j][1].record()
        kp[ens.last_kmax] = kp.get(ens.last_kmax, 0) + 1
    torch.cuda.synchronize()
    pms = [a.elapsed_time(b) for a, b in ev]
    out["pulse_window"] = {
        "value": round(nvec * K / (sum(pms) / 1e3), 1), "unit": UNIT, "steps": K,
        "ms_per_step": round(sum(pms) / K, 3),
        "timed_window_ps": [float(tc[i_lo % nsteps]), float(tc[(i_lo + K - 1) % nsteps])],
        "largest_krylov_order_per_step": {str(k): v for k, v in sorted(kp.items())},
        "sample": f"{K} steps centred on the pulse maximum ({wl.pulse[0]} ps) after {args.warmup} untimed steps, "
                  "from the ensemble's initial vectors; CUDA events around each step"}

    if not args.no_extras:
        # ---- e2e: public API, per step the field in and the observable out ----
        note("e2e")
        K2 = args.e2e_steps
        from richmol_gb300._native import FIELD_COEF_BYTES
        # the thermal average: Boltzmann weights of the states above the
        # ensemble's threshold, zero on the padding vectors
        wnat = np.zeros(nvec)
        wnat[: ensd.n_natural] = ensd.weights[: ensd.n_natural]
        wdev = torch.from_numpy(wnat).to(dev)
        obs = torch.zeros(1, dtype=torch.float64, device=dev)
        host = torch.zeros(1, dtype=torch.float64).pin_memory()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        trace = []
        for j in range(K2):
            H = wl.hamiltonian(tc[(args.warmup + K + j) % nsteps])
            ens.step(H)
            ens.expect_into(wl.cos2, obs, wdev)         # the weighted <cos^2> on the device
            host.copy_(obs)                              # synchronises: the result on the host
            trace.append(float(host[0]) + 1.0 / 3.0)
        e2e_s = time.perf_counter() - t0
        # the same loop with every vector's <cos^2> read back (Ensemble.expect)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for j in range(K2):
            H = wl.hamiltonian(tc[(args.warmup + K + K2 + j) % nsteps])
            ens.step(H)
            e = ens.expect(wl.cos2)
            trace.append(float(np.dot(wnat, e.real)) + 1.0 / 3.0)
        e2e_all_s = time.perf_counter() - t0
        # the first loop pipelined: each step queued without waiting for it
        # (sync=False), its weighted <cos^2> copied to pinned host memory in stream
        # order without blocking the host, which meanwhile prepares the next
        # step; the copies and any step error are waited for once at the end
        obs_k = torch.zeros(K2, dtype=torch.float64, device=dev)
        host_k = torch.zeros(K2, dtype=torch.float64).pin_memory()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for j in range(K2):
            H = wl.hamiltonian(tc[(args.warmup + K + 2 * K2 + j) % nsteps])
            ens.step(H, sync=False)
            ens.expect_into(wl.cos2, obs_k[j:j + 1], wdev)
            host_k[j:j + 1].copy_(obs_k[j:j + 1], non_blocking=True)
        torch.cuda.synchronize()
        ens.sync()
        e2e_pipe_s = time.perf_counter() - t0
        trace.extend((host_k.numpy() + 1.0 / 3.0).tolist())
        out["e2e"] = {"value": round(ws * nvec * K2 / e2e_s, 1), "unit": UNIT,
                      "h2d_bytes_per_step": FIELD_COEF_BYTES, "d2h_bytes_per_step": 8, "steps": K2,
                      "api": "Ensemble.step(H(t)) + Ensemble.expect_into(cos^2, weights) each step (field in, the "
                             "Boltzmann-weighted <cos^2> out; the observable's mat-vec runs on the vector groups of "
                             "non-zero weight)",
                      "includes_observable": True,
                      "every_vector_observable": {
                          "value": round(ws * nvec * K2 / e2e_all_s, 1), "unit": UNIT,
                          "d2h_bytes_per_step": 16 * nvec,
                          "api": "Ensemble.step(H(t)) + Ensemble.expect(cos^2) each step (<cos^2> of all vectors out)"},
                      "pipelined": {
                          "value": round(ws * nvec * K2 / e2e_pipe_s, 1), "unit": UNIT,
                          "h2d_bytes_per_step": FIELD_COEF_BYTES, "d2h_bytes_per_step": 8,
                          "api": "Ensemble.step(H(t), sync=False) + Ensemble.expect_into(cos^2, weights) + a "
                                 "non-blocking copy of that step's result to pinned host memory each step; one wait "
                                 "for the copies and the step errors at the end (the host prepares step j + 1 while "
                                 "the GPU runs step j)"}}

        # ---- the configured run: every step, batched beside plain FP64 ----
        note("configured run")
        full = run_full(args, wl, ensd, ens, dev)
        out["full_run"] = full.pop("rates")
        out["accuracy_vs_fp64"] = full.pop("accuracy")

        # ---- plain FP64 drop-in configuration (J <= 40, one vector, dt 5 fs) ----
        note("plain drop-in")
        out["plain_fp64_drop_in"] = run_plain(args, dev, peaks, peak_kind, fp64.value)
        note("plain step, double-float products")
        out["plain_fp64_drop_in"]["df_products"] = run_plain(args, dev, peaks, peak_kind, fp64.value, products="df")

        # ---- serving: a Poisson stream of requests, continuous batching ----
        note("serving")
        if ws == 1:
            del ens
            torch.cuda.empty_cache()
            out["serving"] = run_serving(args)
            note("uneven batch")
            out["uneven_batch"] = run_uneven(args)
            note("wide-K mat-vec")
            out["wide_k_matvec"] = run_widek(args)

    if rank == 0 and not args.no_cpu_baseline:
        rate, nst, tt = cpu_reference_rate(wl, args.cpu_seconds, vec=ensd.vectors(dim)[0])
        out["cpu_baseline"] = {"value": round(rate, 4), "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"{nst} steps of 1 vector of the ensemble workload in {tt:.1f} s "
                                         f"(oracle restatement of tdse.py/field.py, numpy/scipy, 1 thread)"}
    if ws > 1:
        torch.distributed.destroy_process_group()
    return out


def run_full(args, wl, ensd, ens, dev):
    """The configured run of the batched ensemble (every step of the time grid:
    3000 x 10 fs from t = 0 at the default size) with the plain FP64 path (the
    one pinned to the reference and the oracle) beside it on a sample of the
    vectors: every vector with Boltzmann weight >= 1e-5 and ``--acc-padded``
    padding vectors spread over the rest. Both arms take the same steps from
    the same start. Per step, CUDA events time each arm's step; the
    observables <cos^2>, <cos> and the J-populations of both arms are compared
    every ``--acc-every`` steps and at every step inside the pulse's FWHM.
    Returns the rates (the batched form over all vectors, the plain path over
    the sample, their ratio on the same steps, and the same over the pre-pulse
    window and the pulse window) and the largest errors against FP64."""
    import torch
    from richmol_gb300 import TDSE
    nvec, dim = ens.nvec, wl.dim
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    nsteps = len(tc) if args.acc_steps <= 0 else min(args.acc_steps, len(tc))
    nat = min(ensd.n_natural, nvec)
    pad = sorted(set(np.linspace(nat, nvec - 1, args.acc_padded).astype(int).tolist())) if nvec > nat else []
    sample = list(range(nat)) + [i for i in pad if i >= nat]
    natural = np.array([i < nat for i in sample])
    w = ensd.weights[sample]
    V0 = ensd.vectors(dim)
    ens.load(V0)
    ref = torch.from_numpy(V0[sample]).to(dev)
    tdp = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tdp.time_grid()
    # J of every element (populations of the FP64 states on the device)
    basis = wl.h0._parts[0].src.basis("1")
    Js = sorted({b[0] for b in basis})
    jidx = torch.cat([torch.full((b[2] * b[3],), Js.index(b[0]), dtype=torch.long) for b in basis]).to(dev)
    t0, fwhm = wl.pulse[0], wl.pulse[1]
    names = ("cos2", "cos", "pops")
    err = {n: {"weighted": 0.0, "per_vector": 0.0, "per_vector_padded": 0.0} for n in names}
    b_ev, p_ev, orders, checked = [], [], {}, 0
    for i in range(nsteps):
        H = wl.hamiltonian(tc[i])
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        e[0].record()
        ens.step(H)
        e[1].record()
        e[2].record()
        ref, _ = tdp.update(H, H0=wl.h0, vecs=ref, inplace=True, check=False)
        e[3].record()
        b_ev.append((e[0], e[1]))
        p_ev.append((e[2], e[3]))
        orders[ens.last_kmax] = orders.get(ens.last_kmax, 0) + 1
        if i % args.acc_every == args.acc_every - 1 or abs(tc[i] - t0) <= fwhm or i == nsteps - 1:
            checked += 1
            vals = {"cos2": (ens.expect(wl.cos2).real[sample], ens_expect_plain(ref, wl.cos2)),
                    "cos": (ens.expect(wl.cos).real[sample], ens_expect_plain(ref, wl.cos))}
            pj = ens.populations()
            pb = np.stack([pj[J][sample] for J in Js], axis=1)
            pp = torch.zeros((len(sample), len(Js)), dtype=torch.float64, device=dev)
            pp.index_add_(1, jidx, (ref.real ** 2 + ref.imag ** 2))
            vals["pops"] = (pb, pp.cpu().numpy())
            for n, (a, b) in vals.items():
                d = np.asarray(a) - np.asarray(b)
                dv = np.abs(d) if d.ndim == 1 else np.abs(d).max(axis=1)
                wd = np.abs(np.tensordot(w[natural], d[natural], axes=(0, 0))).max()
                err[n]["weighted"] = max(err[n]["weighted"], float(wd))
                err[n]["per_vector"] = max(err[n]["per_vector"], float(dv[natural].max()))
                if (~natural).any():
                    err[n]["per_vector_padded"] = max(err[n]["per_vector_padded"], float(dv[~natural].max()))
    torch.cuda.synchronize()
    b_ms = np.array([a.elapsed_time(b) for a, b in b_ev])
    p_ms = np.array([a.elapsed_time(b) for a, b in p_ev])

    def window(lo, hi):
        sel = [(lo <= tc[i] <= hi) for i in range(nsteps)]
        if not any(sel):
            return None
        sel = np.array(sel)
        rb = nvec * sel.sum() / (b_ms[sel].sum() / 1e3)
        rp = len(sample) * sel.sum() / (p_ms[sel].sum() / 1e3)
        return {"t_ps": [float(lo), float(hi)], "steps": int(sel.sum()), "batched": round(float(rb), 1),
                "plain_fp64": round(float(rp), 1), "speedup_batched_vs_plain": round(float(rb / rp), 2)}

    rb = nvec * nsteps / (b_ms.sum() / 1e3)
    rp = len(sample) * nsteps / (p_ms.sum() / 1e3)
    rates = {
        "unit": UNIT, "steps": nsteps, "t_ps": [float(tc[0]), float(tc[nsteps - 1])],
        "batched": round(float(rb), 1), "batched_vectors": nvec,
        "plain_fp64": round(float(rp), 1), "plain_vectors": len(sample),
        "speedup_batched_vs_plain": round(float(rb / rp), 2),
        "batched_step_ms_p50": round(float(np.median(b_ms)), 3),
        "batched_step_ms_p99": round(float(np.percentile(b_ms, 99)), 3),
        "windows": {"pre_pulse": window(tc[0], t0 - fwhm - 1e-9), "pulse": window(t0 - fwhm, t0 + fwhm),
                    "after_pulse": window(t0 + fwhm + 1e-9, tc[nsteps - 1])},
        "largest_krylov_order_per_step": {str(k): v for k, v in sorted(orders.items())},
        "sample": ("every step of the time grid from t = 0, both arms from the same vectors; the plain FP64 path "
                   f"on {len(sample)} of the vectors (all {nat} with Boltzmann weight >= 1e-5 and "
                   f"{len(sample) - nat} padding vectors); CUDA events around each arm's step"),
    }
    acc = {
        "bound": 1e-6, "steps": nsteps, "steps_compared": checked, "vectors": len(sample),
        "vectors_natural": nat, "vectors_padded": len(sample) - nat, "padded_indices": [i for i in sample if i >= nat],
        "max_abs_err": err,
        "within_bound": bool(all(err[n][k] <= 1e-6 for n in names for k in err[n])),
        "reference": "plain FP64 GPU path (parity-tested against the reference's own propagation and the oracle)",
        "observables": "cos2: <cos^2 theta> - 1/3 per vector; cos: <cos theta>; pops: J-populations (max over J); "
                       "weighted: Boltzmann-weighted sum over the natural vectors",
    }
    return {"rates": rates, "accuracy": acc}


def run_serving(args):
    """Requests from the uneven-size distributions (C1 asymmetric tops, Jmax
    uniform in the given range, random polarizability, pulse and temperature,
    thermal ensembles of at most 512 vectors) arriving as a Poisson stream,
    served with continuous batching under an HBM budget; p50/p99 latency from
    arrival to the finished <cos^2> trace, aggregate state-steps/s, and the
    trace of the smallest request against the plain FP64 path."""
    import torch
    from richmol_gb300 import TDSE, serve
    reqs = serve.poisson_requests(2024, args.serve_rate, args.serve_duration, jmax_range=tuple(args.serve_jmax),
                                  t_end=args.serve_tend, dt=0.01, max_vectors=512)
    srv = serve.Server(budget_bytes=args.serve_budget_gb * 1e9, max_active=16)
    results, stats = srv.serve(reqs, realtime=True)
    s = stats.summary()
    failed = [rid for rid, r in results.items() if isinstance(r, Exception)]
    # FP64 check of the smallest request (the plain path, vector by vector)
    small = min(reqs, key=lambda r: serve.c1_dim(r.jmax))
    job = serve.Job(small)
    job.build()
    td = TDSE(t_start=0.0, t_end=small.t_end, dt=small.dt)
    tc = td.time_grid()
    v = np.zeros((job.nvec, job.dim), np.complex128)
    v[np.arange(job.nvec), job.index] = 1.0
    ref = torch.from_numpy(v).cuda()
    worst = 0.0
    trace = results.get(small.rid)
    ncheck = min(len(tc), 100)  # the first 1 ps of the trace (the FP64 path runs vector by vector)
    if trace is not None and not isinstance(trace, Exception):
        for i, t in enumerate(tc[:ncheck]):
            ref, _ = td.update(job.wl.hamiltonian(t), H0=job.wl.h0, vecs=ref, inplace=True, check=False)
            if not job.wl.cos2._parts[0].prods:
                job.wl.cos2.field([0, 0, 1])
            e = ens_expect_plain(ref, job.wl.cos2)
            worst = max(worst, abs(float(job.weights @ e) + 1.0 / 3.0 - float(trace[i])))
    else:
        worst = None
    # a sustainable stream: Poisson arrivals at a fraction of the capacity the
    # burst above measured (its aggregate state-steps/s over its mean state-steps
    # per request), so that the queue stays bounded and the latency is the
    # steady-state one
    sustained = None
    if args.serve_sustained_n > 0 and s["requests"] and stats.state_steps > 0:
        cap = s["state_steps_per_s"] / (stats.state_steps / s["requests"])
        rate = args.serve_load * cap
        n2 = args.serve_sustained_n
        reqs2 = serve.poisson_requests(2025, rate, 10.0 * n2 / rate, jmax_range=tuple(args.serve_jmax),
                                       t_end=args.serve_tend, dt=0.01, max_vectors=512)[:n2]
        if reqs2:
            first = reqs2[0].arrival  # the stream starts with its first arrival
            for r in reqs2:
                r.arrival -= first
            res2, st2 = serve.Server(budget_bytes=args.serve_budget_gb * 1e9, max_active=16).serve(reqs2, realtime=True)
            s2 = st2.summary()
            sustained = {
                "rate_per_s": round(rate, 4), "load": args.serve_load, "capacity_per_s": round(cap, 4),
                "p50_ms": round(s2["p50_ms"], 1), "p99_ms": round(s2["p99_ms"], 1),
                "state_steps_per_s": round(s2["state_steps_per_s"], 1), "unit": UNIT, "requests": s2["requests"],
                "failed": sum(isinstance(r, Exception) for r in res2.values()), "wall_s": round(s2["wall_s"], 2),
                "max_concurrent": s2["max_concurrent"],
                "arrivals_s": round(reqs2[-1].arrival, 1),
                "sample": (f"the first {n2} arrivals of a Poisson stream at {args.serve_load} x the capacity the "
                           "burst measured (its state-steps/s over its mean state-steps per request); requests "
                           "drawn as in the burst, latency from arrival to finished trace"),
            }
    return {
        "sustained": sustained,
        "p50_ms": round(s["p50_ms"], 1), "p99_ms": round(s["p99_ms"], 1),
        "state_steps_per_s": round(s["state_steps_per_s"], 1), "unit": UNIT,
        "requests": s["requests"], "failed": len(failed), "wall_s": round(s["wall_s"], 2),
        "max_concurrent": s["max_concurrent"], "peak_admitted_gb": round(s["peak_admitted_bytes"] / 1e9, 1),
        "sample": (f"Poisson {args.serve_rate}/s for {args.serve_duration} s, Jmax {args.serve_jmax[0]}-"
                   f"{args.serve_jmax[1]} (C1, n_k up to {2 * args.serve_jmax[1] + 1}), <=512 vectors per "
                   f"request, {args.serve_tend} ps at 10 fs each, HBM budget {args.serve_budget_gb:.0f} GB; "
                   "latency = arrival to finished trace, incl. queueing and the factor build (started at "
                   "arrival on the builder thread)"),
        "fp64_check": {"rid": small.rid, "jmax": small.jmax, "vectors": job.nvec, "steps": ncheck,
                       "max_abs_err_cos2": worst, "bound": 1e-6},
    }


def run_widek(args, jmax=40, nvec=512):
    """The batched mat-vec of one served-size request with wide K blocks: a C1
    molecule (no symmetry, n_k = 2J + 1 up to 81, slabs cut into column chunks
    of 32) at J <= 40, 512 vectors, every kernel kind; CUDA events over 5
    launches after 2."""
    import torch
    from richmol_gb300 import TDSE, _native, rot, workloads
    from richmol_gb300.batch import Ensemble
    from richmol_gb300.device import stream_ptr
    from richmol_gb300.serve import draw_request
    L = _native.lib()
    req = draw_request(np.random.default_rng(7), 0, 0.0, jmax_range=(jmax, jmax), t_end=5.0, dt=0.01)
    mol = rot.Molecule(B=req.abc, sym="C1", pol=req.pol)
    wl = workloads.Workload("c1_j%d" % jmax, mol, jmax, 0.0, 5.0, 0.01, None, req.pulse)
    td = TDSE(t_start=0.0, t_end=5.0, dt=0.01)
    tc = td.time_grid()
    res = {}
    for kind in ("tensor_tmem", "tensor", "fp32", "fp32_reg"):
        ens = Ensemble(td, wl.h0, nvec, tol=1e-8, matvec=kind)
        v = np.zeros((nvec, wl.dim), np.complex128)
        v[np.arange(nvec), np.arange(nvec)] = 1.0
        ens.load(v)
        ens.step(wl.hamiltonian(tc[250]))
        plan = wl.hamiltonian(tc[251]).device_operator(split=ens.split)
        for _ in range(2):
            _native.check(L.kr_batch_matvec(ens.handle, plan.op, stream_ptr()), ens.ctx)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(5):
            _native.check(L.kr_batch_matvec(ens.handle, plan.op, stream_ptr()), ens.ctx)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / 5
        fma, _ = plan.work()
        res[kind] = {"ms": round(ms, 3), "alg_gbs": round(16.0 * wl.dim * nvec / ms / 1e6, 1),
                     "fp32_tflops": round(2.0 * fma * nvec / ms / 1e9, 1)}
        del ens
        torch.cuda.empty_cache()
    return {"workload": f"C1 asymmetric top J=0..{jmax} (dim {wl.dim}, n_k up to {2 * jmax + 1}, column chunks "
                        f"of 32), {nvec} vectors, one batched mat-vec", "by_kind": res}


def run_uneven(args):
    """The uneven-size batch: molecules drawn from the seeded distributions (C1,
    Jmax uniform in the range, own pulse each) joined in one block-diagonal
    operator; a time step is one field launch and one persistent segmented step
    launch over the ragged block table of all molecules (per-molecule Lanczos,
    stopping test and Krylov order). Both arithmetic forms run on the same
    molecules and steps through the pulse maxima: "f64" (every product FP64,
    as the reference) and "mixed" (the mat-vec products in FP32, states,
    Krylov vectors and Lanczos scalars FP64). The first three molecules are
    checked against their own TDSE.update propagation (FP64)."""
    import torch
    from richmol_gb300 import TDSE, workloads
    from richmol_gb300.molecules import MoleculeSet
    t0 = time.time()
    wls = workloads.uneven_molecules(args.uneven_n, seed=2025, jmax_range=tuple(args.uneven_jmax), t_end=20.0)
    build_s = time.time() - t0
    td = TDSE(t_start=0.0, t_end=20.0, dt=0.01)
    tc = td.time_grid()
    v0 = [workloads.ground_state(w) for w in wls]
    i0 = len(tc) // 2 - 2
    out = {"molecules": len(wls), "unit": "molecule-steps/s", "factor_build_s": round(build_s, 1)}
    for prec in ("f64", "mixed"):
        ms = MoleculeSet(td, [w.h0 for w in wls], [w.Hac for w in wls], precision=prec)
        state = ms.join(v0)
        for i in range(i0, i0 + 2):  # warm-up
            for w in wls:
                w.hamiltonian(tc[i])
            ms.step(state)
        torch.cuda.synchronize()
        ev, korders = [], []
        l0 = ms.launches()
        for i in range(i0 + 2, i0 + 2 + args.uneven_steps):
            for w in wls:
                w.hamiltonian(tc[i])
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            ms.step(state)
            b.record()
            ev.append((a, b))
            korders.append([int(ms.last_korder.min()), int(ms.last_korder.max())])
        torch.cuda.synchronize()
        launches = ms.launches() - l0
        ms_step = statistics.median(a.elapsed_time(b) for a, b in ev)
        # the first three molecules alone (FP64 TDSE.update), same steps from the same start
        chk = wls[:3]
        ms2 = MoleculeSet(td, [w.h0 for w in chk], [w.Hac for w in chk], precision=prec)
        st2 = ms2.join(v0[:3])
        alone = [torch.from_numpy(v).cuda().reshape(1, -1) for v in v0[:3]]
        tds = [TDSE(t_start=0.0, t_end=20.0, dt=0.01) for _ in chk]
        for t_ in tds:
            t_.time_grid()
        for i in range(i0, i0 + 2 + args.uneven_steps):
            for w in chk:
                w.hamiltonian(tc[i])
            ms2.step(st2)
            for m, w in enumerate(chk):
                alone[m], _ = tds[m].update(w.hamiltonian(tc[i]), H0=w.h0, vecs=alone[m], inplace=True, check=False)
        worst = max(float((v - alone[m].reshape(-1)).abs().max()) for m, v in enumerate(ms2.split(st2)))
        c2a = ms2.expect([w.cos2 for w in chk], st2)
        c2b = np.array([ens_expect_plain(alone[m], w.cos2)[0] for m, w in enumerate(chk)])
        out[prec] = {
            "value": round(len(wls) / (ms_step / 1e3), 1), "ms_per_step": round(ms_step, 3),
            "total_dim": ms.dim, "dims_min_max": [int(min(ms.dims)), int(max(ms.dims))],
            "krylov_order_min_max_per_step": korders, "gpu_launches_per_step": launches / max(1, args.uneven_steps),
            "dtype": ("f64 (segmented step: mat-vec, per-molecule Lanczos, state)" if prec == "f64" else
                      "f32 mat-vec products / f64 states, Krylov vectors, Lanczos scalars"),
            "check_vs_alone": {"molecules": 3, "steps": 2 + args.uneven_steps, "max_abs_err_state": worst,
                               "max_abs_err_cos2": float(np.abs(c2a - c2b).max()),
                               "bound": 1e-10 if prec == "f64" else 1e-6},
        }
        del ms, ms2, state, st2
        torch.cuda.empty_cache()
    out["value"] = out["mixed"]["value"]
    out["speedup_mixed_vs_f64"] = round(out["mixed"]["value"] / out["f64"]["value"], 2)
    out["sample"] = (f"{len(wls)} molecules (C1, Jmax {args.uneven_jmax[0]}-{args.uneven_jmax[1]}, seed 2025), "
                     f"{args.uneven_steps} steps of 10 fs through the pulse maxima after 2 untimed; CUDA events")
    return out


def ens_expect_plain(ref, O):
    """<v|O|v> of FP64 states (rows of a CUDA tensor) through the FP64 mat-vec."""
    import torch
    plan = O.device_operator()
    y = torch.empty_like(ref)
    plan.matvec(ref, y)
    return torch.sum(torch.conj(ref) * y, dim=1).real.cpu().numpy()


def run_plain(args, dev, peaks, peak_kind, fp64_peak, products="f64"):
    """The plain FP64 drop-in configuration: J <= 40 (dim 91,881), one vector,
    dt = 5 fs, L2 flushed before every step; kernel roofline on the FP64 pipe.
    products="df": the same steps with double-float mat-vec products (FP32
    pipes), with their largest state difference from the FP64 products' over
    the timed steps."""
    import torch
    from richmol_gb300 import TDSE, workloads
    wl = workloads.asym_top(Jmax=args.jmax_plain)
    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    v0 = td.init_state(wl.h0, temp=0)
    v = torch.from_numpy(v0).to(dev)
    phase = td._h0_phase(wl.h0, td.exp_fac, dev)
    fac = td.exp_fac
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for i in range(5):
        pl = wl.hamiltonian(tc[i]).device_operator()
        pl.set_precision(products)
        pl.step(v, phase, fac, 1e-15)
    K = args.plain_steps
    vref = v.clone() if products != "f64" else None
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    ek = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    torch.cuda.synchronize()
    for j in range(K):
        flush.zero_()
        ev[j][0].record()
        plan = wl.hamiltonian(tc[5 + j]).device_operator()
        ek[j][0].record()
        plan.step(v, phase, fac, 1e-15)
        ek[j][1].record()
        ev[j][1].record()
    torch.cuda.synchronize()
    plan.sync_status()
    df_err = None
    if vref is not None:  # the same K steps with FP64 products, untimed
        for j in range(K):
            pl = wl.hamiltonian(tc[5 + j]).device_operator()
            pl.set_precision("f64")
            pl.step(vref, phase, fac, 1e-15)
            pl.set_precision(products)
        torch.cuda.synchronize()
        df_err = float((v - vref).abs().max() / vref.abs().max())
    step_ms = [a.elapsed_time(b) for a, b in ev]
    kern_s = statistics.mean(a.elapsed_time(b) for a, b in ek) / 1e3
    kord = np.zeros(1, np.int32)
    ks = []
    vp = v.clone()
    for j in range(0, K, max(1, K // 20)):
        wl.hamiltonian(tc[5 + j]).device_operator().step(vp, phase, fac, 1e-15, korder=kord)
        ks.append(int(kord[0]))
    kavg = float(np.mean(ks))
    fma_mv, bytes_mv = plan.work()
    n = wl.dim
    flops = 2.0 * kavg * fma_mv + n * sum(8.0 * (k + 1) + 40.0 for k in range(1, int(round(kavg))))
    alg_bytes = 16.0 * n * (3 * kavg + 1) + (bytes_mv - 32.0 * n)
    gbs = alg_bytes / kern_s / 1e9
    # the same steps recorded once as a CUDA graph (field + step launches per
    # step, L2 flush recorded ahead of each) and replayed with one launch
    from richmol_gb300.graph import StepGraph
    sg = StepGraph(td, wl.h0, v, wl.hamiltonian, tc[5 + K:5 + 2 * K], before_step=flush.zero_, products=products)
    ga, gb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ga.record()
    sg.replay()
    gb.record()
    torch.cuda.synchronize()
    graph_ms = ga.elapsed_time(gb) / K
    fa, fb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fa.record()
    for _ in range(20):
        flush.zero_()
    fb.record()
    torch.cuda.synchronize()
    flush_ms = fa.elapsed_time(fb) / 20
    # e2e through the reference-facing API with host (numpy) buffers
    td2 = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc2 = td2.time_grid()
    vh, _ = td2.update(wl.hamiltonian(tc2[0]), v0, H0=wl.h0, products=products)
    torch.cuda.synchronize()
    K2 = 100
    t0 = time.perf_counter()
    for j in range(1, K2 + 1):
        vh, _ = td2.update(wl.hamiltonian(tc2[j]), vh, H0=wl.h0, products=products)
    e2e = K2 / (time.perf_counter() - t0)
    out = {
        "value": round(K / (sum(step_ms) / 1e3), 1), "unit": UNIT, "steps": K,
        "workload": f"asymmetric top D2 J=0..{args.jmax_plain} (dim {n}), 1 vector, dt 5 fs, L2 flushed per step",
        "step_ms_p50": round(statistics.median(step_ms), 4), "kernel": "kr_step_kernel",
        "graph": {"value": round(1e3 / (graph_ms - flush_ms), 1), "unit": UNIT,
                  "step_ms": round(graph_ms - flush_ms, 4), "step_ms_with_flush": round(graph_ms, 4),
                  "flush_ms": round(flush_ms, 4),
                  "sample": f"{K} further steps recorded as one CUDA graph (field + step launches, "
                            "L2 flush ahead of each), one replay; the flush's own time subtracted"},
        "kernel_ms": round(kern_s * 1e3, 4), "krylov_order_avg": kavg,
        # the step's working set stays in L2 and its FP64 work binds before HBM
        # does (GB300's FP64 rate is 1/58 of its FP32 rate): bound = the FP64 pipe
        "roofline": {"bound": "fp64", "achieved": round(flops / kern_s / 1e12, 4), "peak": round(fp64_peak, 4),
                     "unit": "TFLOP/s", "frac": round(flops / kern_s / 1e12 / fp64_peak, 4),
                     "peak_source": "measured FP64 FMA probe (kr_probe_fp64)",
                     "traffic": load_traffic().get("kr_step_kernel_per_launch_bytes"),
                     "hbm": {"achieved_gbs": round(gbs, 2), "peak_gbs": peaks["hbm_gbs"],
                             "frac": round(gbs / peaks["hbm_gbs"], 5)}},
        "e2e": {"value": round(e2e, 1), "unit": UNIT, "h2d_bytes_per_step": int(v0.nbytes),
                "d2h_bytes_per_step": int(v0.nbytes), "api": "TDSE.update(H, numpy vecs, H0=h0)"},
        "products": products,
    }
    if df_err is not None:
        out["max_rel_state_diff_vs_fp64_products"] = df_err
        out["sample_diff"] = f"{K} timed steps from the same state, FP64 products run beside them untimed"
        # the FP64 pipe no longer carries the products: report the kernel
        # against the HBM roofline only, with the FP64-equivalent rate beside it
        out["roofline"] = {"bound": "latency", "achieved_fp64_equiv_tflops": out["roofline"]["achieved"],
                           "hbm": out["roofline"]["hbm"],
                           "note": "double-float products on the FP32 pipes; grid barriers and the "
                                   "row-task tail bound the step"}
    return out


def run_reference(args, ws, rank, local):
    """CPU restatement of the reference algorithm (the reference itself does not
    install: numpy.distutils / Fortran), one process per host core, each
    propagating one vector of the ensemble workload."""
    if rank != 0:
        return None
    import multiprocessing as mp
    ncores = os.cpu_count() or 1
    nproc = max(1, min(ncores, 64))
    per_steps = max(1, min(args.steps, 20))
    warm = max(1, min(args.warmup, 10))  # untimed steps per process (bounded: each is ~0.5 s of CPU)
    budget = 60.0
    ctxm = mp.get_context("spawn")
    # one thread per process: the children import numpy (and its BLAS) at
    # start-up, before any code of theirs runs, so the limit goes into the
    # environment they inherit
    saved = {k: os.environ.get(k) for k in SINGLE_THREAD_ENV}
    os.environ.update({k: "1" for k in SINGLE_THREAD_ENV})
    t0 = time.perf_counter()
    try:
        with ctxm.Pool(nproc) as pool:
            res = pool.map(_reference_worker,
                           [(args.jmax, args.nvec, i, budget, per_steps, warm) for i in range(nproc)])
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    wall = time.perf_counter() - t0
    steps = sum(r[0] for r in res)
    busy = max(r[1] for r in res)
    rate = steps / busy
    threads = sorted({str(r[2].get("OMP_NUM_THREADS")) for r in res})
    return {
        "impl": "reference", "metric": METRIC, "value": round(rate, 3), "unit": UNIT, "n_gpus": ws,
        "steps": per_steps, "warmup": warm, "ms_per_step": round(busy * 1e3 / per_steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64)",
        "data": "synthetic",
        "config": {"workload": f"batched thermal ensemble: asymmetric top D2 Watson-A J=0..{args.jmax}, "
                               f"{args.nvec} vectors (sampled: {nproc} vectors x {per_steps} steps)",
                   "jmax": args.jmax, "nvec": args.nvec},
        "cpu_baseline": {"value": round(rate, 3), "unit": UNIT, "cores": nproc, "kind": "port",
                         "threads_per_process": threads,
                         "sample": f"{nproc} processes x {per_steps} steps, one vector each, one BLAS/OpenMP "
                                   f"thread per process, wall {wall:.0f} s "
                                   "(incl. factor build); the reference does not install here "
                                   "(numpy.distutils, Fortran extensions), its algorithm runs as the numpy/scipy "
                                   "restatement"},
        "e2e": {"value": round(rate, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def note(msg):
    """Progress of the run on stderr (stdout carries the JSON line only)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def main():
    import faulthandler
    faulthandler.enable()  # a crash prints the Python stacks of all threads on stderr
    args = parse()
    ws, rank, local = dist_info()
    out = run_reference(args, ws, rank, local) if args.impl == "reference" else run_ours(args, ws, rank, local)
    if out is not None and rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
