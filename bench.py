#!/usr/bin/env python
"""Krylov time-propagation benchmark: state-steps/s on one GB300.

One step is one TDSE.update of the state (H0 half-phases + the field-dressed
Lanczos exponential). Default workload: the plain FP64 drop-in configuration,
an asymmetric top (A, B, C = 9.0, 5.0, 3.2 cm^-1, Watson A, D2) with J = 0..40
(dim 91,881), one state vector, DC 20 kV/cm + 1e12 W/cm^2 FWHM 500 fs pulse at
35 deg, dt = 5 fs; synthetic molecule and fields built in-process.

Prints ONE JSON line (rank 0). ``--impl reference`` times the CPU
restatement of the reference algorithm (numpy/scipy, the oracle) on the host
cores for the same workload and metric.
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


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--jmax", type=int, default=40)
    p.add_argument("--e2e-steps", type=int, default=300)
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="bound of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


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
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
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
    from oracle.cartens import OCarTens
    src = T._parts[0].src
    o = OCarTens()
    for k in ("Jlist1", "Jlist2", "symlist1", "symlist2", "dim_m1", "dim_m2", "dim_k1", "dim_k2", "dim1", "dim2",
              "mmat", "rank"):
        setattr(o, k, getattr(src, k))
    # own copy of the K dictionaries: mul() replaces their entries
    o.kmat = {Jp: {sp: dict(kS) for sp, kS in kJ.items()} for Jp, kJ in src.kmat.items()}
    o.cart = src.carts
    if T._parts[0].kscale != 1:
        o.mul(T._parts[0].kscale)
    return o


def cpu_reference_rate(wl, seconds, max_steps=None, warmup=1):
    """State-steps/s of the oracle (reference algorithm in numpy/scipy, one
    host thread) on the first steps of the workload, bounded by ``seconds``."""
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
    v = td.init_state(oh0, temp=0)
    n = 0
    t_run = 0.0
    i = 0
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


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, ws, rank, local):
    import torch
    from richmol_gb300 import TDSE, _native, workloads
    from richmol_gb300.device import context

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    t_build = time.time()
    wl = workloads.asym_top(Jmax=args.jmax)
    t_build = time.time() - t_build

    td = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc = td.time_grid()
    nsteps = len(tc)
    v0 = td.init_state(wl.h0, temp=0)
    nvec = v0.shape[0]
    v = torch.from_numpy(v0).to(dev)
    phase = td._h0_phase(wl.h0, td.exp_fac, dev)
    fac = td.exp_fac
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MiB > L2

    def step(i):
        H = wl.hamiltonian(tc[i % nsteps])
        plan = H.device_operator()
        plan.step(v, phase, fac, 1e-15)
        return plan

    for i in range(args.warmup):
        plan = step(i)
    torch.cuda.synchronize()
    plan.sync_status()

    # ---- value: device-resident state, L2 flushed before every step -----------
    K = args.steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    ek = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    launches0 = plan.launches()
    korders = []
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for j in range(K):
            i = args.warmup + j
            flush.zero_()
            ev[j][0].record()
            H = wl.hamiltonian(tc[i % nsteps])
            plan = H.device_operator()
            ek[j][0].record()
            plan.step(v, phase, fac, 1e-15)
            ek[j][1].record()
            ev[j][1].record()
        torch.cuda.synchronize()
    plan.sync_status()
    launches = plan.launches() - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    kern_ms = [a.elapsed_time(b) for a, b in ek]
    total_s = sum(step_ms) / 1e3
    if ws > 1:
        t = torch.tensor([total_s], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_s = float(t.item())
        torch.distributed.barrier()
    value = ws * nvec * K / total_s

    # Krylov orders of the timed steps (one checked step per 50 to read them)
    kord = np.zeros(1, np.int32)
    ks = []
    v_probe = v.clone()
    for j in range(0, K, max(1, K // 20)):
        H = wl.hamiltonian(tc[(args.warmup + j) % nsteps])
        H.device_operator().step(v_probe, phase, fac, 1e-15, korder=kord)
        ks.append(int(kord[0]))
    kavg = float(np.mean(ks))

    # ---- e2e: TDSE.update with host (numpy) buffers ---------------------------
    K2 = min(args.e2e_steps, nsteps)
    td2 = TDSE(t_start=wl.t_start, t_end=wl.t_end, dt=wl.dt)
    tc2 = td2.time_grid()
    vh = v0.copy()
    Hs = wl.hamiltonian(tc2[0])
    vh, _ = td2.update(Hs, vh, H0=wl.h0)  # warm-up (H0 phase set-up)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for j in range(1, K2 + 1):
        vh, _ = td2.update(wl.hamiltonian(tc2[j]), vh, H0=wl.h0)
    e2e_s = time.perf_counter() - t0
    e2e_value = ws * nvec * K2 / e2e_s

    # ---- roofline of the dominant kernel (kr_step_kernel) ----------------------
    fma_mv, bytes_mv = plan.work()
    n = wl.dim
    kern_s = statistics.mean(kern_ms) / 1e3
    # FLOPs: k mat-vecs + the Lanczos vector work of each iteration
    flops_step = 2.0 * kavg * fma_mv + n * sum(8.0 * (k + 1) + 40.0 for k in range(1, int(round(kavg))))
    # algorithmic bytes (no re-orthogonalisation): s n (3m + 1) + factors
    alg_bytes = 16.0 * n * (3 * kavg + 1) + (bytes_mv - 32.0 * n)
    peaks, peak_kind = load_peaks()
    ctx = context(local)
    import ctypes
    fp64 = ctypes.c_double()
    _native.check(_native.lib().kr_probe_fp64(ctx, ctypes.byref(fp64)), ctx)
    traffic = load_traffic().get("kr_step_kernel_per_launch_bytes")
    achieved_gbs = alg_bytes / kern_s / 1e9
    roofline = {
        "bound": "hbm", "achieved": round(achieved_gbs, 2), "peak": peaks["hbm_gbs"], "unit": "GB/s",
        "frac": round(achieved_gbs / peaks["hbm_gbs"], 5), "traffic": traffic,
        "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
        "kernel": "kr_step_kernel", "kernel_ms": round(kern_s * 1e3, 4),
        "alg_bytes_per_launch": alg_bytes, "krylov_order_avg": kavg,
        "fp64": {"achieved_tflops": round(flops_step / kern_s / 1e12, 4),
                 "peak_tflops": round(fp64.value, 4), "frac": round(flops_step / kern_s / 1e12 / fp64.value, 4),
                 "peak_source": "measured FMA probe (kr_probe_fp64)",
                 "flops_per_launch": flops_step},
    }

    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": args.warmup,
        "ms_per_step": round(total_s * 1e3 / K, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128 (f64)", "data": "synthetic",
        "config": {"workload": f"plain FP64 drop-in: asymmetric top D2 Watson-A, J=0..{args.jmax}, dim {n}, "
                               f"{nvec} vector, DC 20 kV/cm + 1e12 W/cm^2 FWHM 500 fs pulse at 35 deg, dt 5 fs",
                   "dim": n, "nvec": nvec, "jmax": args.jmax, "dt_fs": 5.0, "tol": 1e-15,
                   "l2": "flushed (256 MiB write) before every timed step", "parallelism": f"replicas x{ws}",
                   "factor_build_s": round(t_build, 2)},
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": int(v0.nbytes),
                "d2h_bytes_per_step": int(v0.nbytes), "steps": K2,
                "api": "richmol_gb300.TDSE.update(H, numpy vecs, H0=h0)"},
        "roofline": roofline,
        "gpu_launches": int(launches),
        "step_ms_p50": round(statistics.median(step_ms), 4),
        "step_ms_p99": round(float(np.percentile(step_ms, 99)), 4),
    }
    clocks = clk.summary()
    if clocks:
        out["clocks"] = clocks
    if rank == 0 and not args.no_cpu_baseline:
        rate, nst, tt = cpu_reference_rate(wl, args.cpu_seconds)
        out["cpu_baseline"] = {"value": round(rate, 4), "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"{nst} steps x {nvec} vector of the same workload in {tt:.1f} s "
                                         f"(oracle restatement of tdse.py/field.py, numpy/scipy, 1 thread)"}
    if ws > 1:
        torch.distributed.destroy_process_group()
    return out


def run_reference(args, ws, rank, local):
    if rank != 0:
        return None
    from richmol_gb300 import workloads
    wl = workloads.asym_top(Jmax=args.jmax)
    budget = min(120.0, max(10.0, args.cpu_seconds * 4))
    rate, nst, tt = cpu_reference_rate(wl, budget, max_steps=args.steps, warmup=min(args.warmup, 1))
    return {
        "impl": "reference", "metric": METRIC, "value": round(rate, 4), "unit": UNIT, "n_gpus": ws,
        "steps": nst, "warmup": min(args.warmup, 1), "ms_per_step": round(tt * 1e3 / max(nst, 1), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64)",
        "data": "synthetic",
        "config": {"workload": f"plain FP64 drop-in: asymmetric top D2 Watson-A, J=0..{args.jmax}, dim {wl.dim}, "
                               f"1 vector, DC 20 kV/cm + 1e12 W/cm^2 FWHM 500 fs pulse at 35 deg, dt 5 fs",
                   "dim": wl.dim, "nvec": 1, "jmax": args.jmax},
        "cpu_baseline": {"value": round(rate, 4), "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"{nst} steps of 1 vector in {tt:.1f} s (time budget {budget:.0f} s); the "
                                   "reference itself does not install (numpy.distutils, Fortran), its algorithm "
                                   "runs as the numpy/scipy restatement; one vector leaves no parallel work "
                                   "for more host threads"},
        "e2e": {"value": round(rate, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    ws, rank, local = dist_info()
    if args.impl == "reference":
        out = run_reference(args, ws, rank, local)
    else:
        out = run_ours(args, ws, rank, local)
    if out is not None and rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
