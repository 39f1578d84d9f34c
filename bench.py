#!/usr/bin/env python
"""Shell-to-shell benchmark: 512^3 D=3 32-shell T(n,m) per second on GB300.

One step = one full T(n,m) matrix (32 linear shells, dk = 14, Orszag 2/3) of a seeded Hermitian
solenoidal 512^3 field (k^-5/3 on 4 <= k <= 170, k^4 rise below 4), computed by libfit_gb300 in the
FP32-batched form (FP32 transforms/products, FP64 shell sums, CUDA-graph replay). The JSON line
also carries: the plain FP64 form (one nonlinear term per mediator, FP64 everywhere) and its
relative difference from the FP32 result, the end-to-end figure through the host-buffer C ABI
(host->device copy of the input and device->host copy of T inside the timed region), the dominant
kernel's achieved DRAM bandwidth from CUDA events around its launches, SM clocks sampled during
the timed region, and the CPU oracle timed on a bounded sample.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica (no collective on the data path);
the value is the units all ranks processed divided by the slowest rank's time.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "512³ shell-to-shell T(n,m)/s & HBM GB/s: FP32-batched vs FP64 plain, rel err 1e-5"
UNIT = "T(n,m)/s"
FALLBACK_BF16_TFLOPS = 1900.0
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--dk", type=float, default=14.0)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--oracle-column", type=int, default=8,
                    help="1-based mediator shell whose full column the oracle computes for the headline's "
                         "error line (0: skip)")
    ap.add_argument("--no-cufft", action="store_true", help="skip the cuFFT comparison")
    ap.add_argument("--config", default="s2s", choices=["s2s", "closure", "batch", "partial", "padded", "m2m", "band", "frontend", "xpass", "ypass", "zbin"],
                    help="s2s: the 512^3 shell-to-shell headline; closure: learned closure vs exact "
                         "coarse-graining flux on a forced 256^3 field; batch: 64 uneven spectral-flux "
                         "instances per graph launch; partial: 512^3 helical partial fluxes of kinetic energy "
                         "and helicity (16 channels) in one graph launch; padded: 256^3 32-shell shell-to-shell "
                         "with the exact 3/2 rule; m2m: 32^3 resolved mode-to-mode S(k|p); band: 512^3 smooth "
                         "band-to-band T(K,Q) over 7 log-Gaussian bands; frontend: 512^3 u_hat = fft(u)/Np of three "
                         "real fields")
    ap.add_argument("--decomp", default="helical", choices=["helical", "toroidal_poloidal"],
                    help="partial config: the decomposition of the velocity into two components")
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--lines", type=int, default=65536, help="xpass config: x lines of the one-mediator slice")
    ap.add_argument("--planes", type=int, default=128, help="ypass config: z planes of the one-mediator slice")
    ap.add_argument("--mediators", type=int, default=1, help="zbin config: mediators of the z-forward + binning pass")
    ap.add_argument("--branches", type=int, default=8, help="batch config: concurrent graph branches")
    ap.add_argument("--closure-n", type=int, default=256)
    ap.add_argument("--closure-nsteps", type=int, default=200)
    ap.add_argument("--train-steps", type=int, default=1500)
    ap.add_argument("--train-batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--mixed", type=int, default=1, help="closure network as a residual over the gradient model")
    return ap.parse_args()


# ---------------------------------------------------------------------------------------------
def dist_setup():
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, x):
    """Maximum of x over the ranks (on the device for NCCL, on the host for gloo)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(ws, units_per_rank, ms):
    """Whole-job throughput of ws independent replicas: the units all ranks processed divided by the
    slowest rank's time. Returns (units/s, slowest ms)."""
    ms_max = allmax(ws, ms)
    return ws * units_per_rank * 1000.0 / ms_max, ms_max


def make_field(N, seed, device, spectrum="kolmogorov"):
    """û = fft(u)/Np of real Gaussian noise per component, scaled by sqrt(E(|k|)/|k|^2), with
    E = k^-5/3 on [4, 170], (k/4)^4 4^-5/3 below 4, 0 above ("kolmogorov") or
    E = k^4 exp(-2 (k/8)^2) ("k4exp8"); Leray-projected, mean removed.
    Returned as a (3, N, N, N) complex64 CUDA tensor, i.e. the column-major (N, N, N, 3) layout."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    k1 = torch.fft.fftfreq(N, d=1.0 / N, device=device, dtype=torch.float32)
    kz, ky, kx = k1.view(N, 1, 1), k1.view(1, N, 1), k1.view(1, 1, N)
    k2 = kx * kx + ky * ky + kz * kz
    km = torch.sqrt(k2)
    if spectrum == "k4exp8":
        E = km ** 4 * torch.exp(-2 * (km / 8) ** 2)
    else:
        E = torch.where(km < 4, (km / 4) ** 4 * 4.0 ** (-5 / 3),
                        torch.where(km <= 170, km.clamp_min(1e-30) ** (-5 / 3), torch.zeros_like(km)))
    amp = torch.where(k2 > 0, torch.sqrt(E / k2.clamp_min(1e-30)), torch.zeros_like(km))
    del E, km
    u = torch.empty((3, N, N, N), dtype=torch.complex64, device=device)
    for c in range(3):
        r = torch.randn((N, N, N), generator=g, device=device, dtype=torch.float32)
        u[c] = torch.fft.fftn(r) * (amp / float(N) ** 3)
        del r
    div = (kx * u[0] + ky * u[1] + kz * u[2]) / torch.where(k2 > 0, k2, torch.ones_like(k2))
    u[0] -= kx * div
    u[1] -= ky * div
    u[2] -= kz * div
    del div, amp, k2
    u[:, 0, 0, 0] = 0
    torch.cuda.synchronize()
    return u


class Clocks:
    """nvidia-smi sampling of SM clock, power and throttle reasons during the timed region."""
    Q = ("index,pci.bus_id,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, bus_id=None):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.bus = bus_id
        self.p = None

    def start(self):
        try:
            cmd = ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"]
            if self.bus:
                cmd += ["-i", self.bus]
            self.p = subprocess.Popen(cmd, stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = [l.split(",") for l in open(self.f.name).read().strip().splitlines() if l.strip()]
        os.unlink(self.f.name)
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 10:
                continue
            try:
                sm.append(float(r[2])); mx.append(float(r[3])); pw.append(float(r[4]))
            except ValueError:
                continue
            for i, n in enumerate(names):
                if r[6 + i].lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "power_w_max": max(pw),
                "samples": len(sm), "reasons": sorted(reasons)}


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def read_bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["bf16_tflops"]), "measured (burst)"
    except Exception:
        return FALLBACK_BF16_TFLOPS, "fallback"


def prof_roofline(F, fn, sync):
    """Per-kernel CUDA-event breakdown of one eager call of ``fn`` (the library's per-launch events):
    the dominant kernel's algorithmic bytes over its measured time against the HBM peak."""
    F._lib.prof_enable(True)
    fn()
    sync()
    prof = F._lib.prof_read_all()
    F._lib.prof_enable(False)
    if not prof:
        return None
    prof_ms = sum(v[0] for v in prof.values())
    dname, (dms, dbytes, dn) = max(prof.items(), key=lambda kv: kv[1][0])
    peak, peak_kind = read_peaks()
    achieved = dbytes / (dms / 1e3) / 1e9
    return {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "launches_per_step": dn,
            "algorithmic_bytes_per_launch": dbytes / dn, "avg_launch_ms": dms / dn,
            "share_of_step": dms / prof_ms, "traffic": None,
            "all_kernels": {k: {"ms": v[0], "GBps": v[1] / (v[0] / 1e3) / 1e9 if v[0] > 0 else None,
                                "launches": v[2]} for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
            "step_alg_bytes_GB": sum(v[1] for v in prof.values()) / 1e9}


def read_traffic(kernel):
    """Per-launch DRAM bytes of ``kernel`` from the committed ncu summary (``profiles/``), or None."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def host_field(u):
    """(3,N,N,N) complex64 CUDA tensor -> (N,N,N,3) complex128 numpy array (column-major data)."""
    a = u.cpu().numpy()
    return np.transpose(a, (3, 2, 1, 0)).astype(np.complex128)


def cpu_sample(u_np, ks, dk, reps=1):
    """Time the oracle (the reference algorithm restated, FP64, scipy.fft with all host threads)
    on a bounded sample: the mediator-independent setup, then one advected component of one
    mediator column. A full T(n,m) is setup + 32 mediators x 3 components."""
    import oracle as O
    cores = os.cpu_count() or 1
    O.set_fft_workers(cores)
    t0 = time.perf_counter()
    st = O.s2s_setup(u_np, ks, ("linear", dk), "two_thirds")
    t_setup = time.perf_counter() - t0
    nsh = st["nsh"]
    times = []
    for r in range(reps):
        m, c = (7 + r) % nsh, r % 3
        t0 = time.perf_counter()
        O.s2s_column(st, m, comps=[c])
        times.append(time.perf_counter() - t0)
    t_piece = float(np.mean(times))
    t_matrix = t_setup + nsh * 3 * t_piece
    return t_setup, t_piece, t_matrix, cores, nsh, st


def julia_probe():
    """Whether a Julia toolchain exists on this host (the reference's own CPU path needs one, plus
    FlowInvariantTransfer.jl and FFTW.jl installed for it)."""
    import shutil
    exe = shutil.which("julia")
    if not exe:
        return {"found": False}
    try:
        v = subprocess.run([exe, "--version"], capture_output=True, text=True, timeout=60).stdout.strip()
    except Exception as e:
        v = f"failed: {e}"
    return {"found": True, "path": exe, "version": v}


# ---------------------------------------------------------------------------------------------
def run_reference(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import torch
    import oracle as O
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    N = args.n
    u = make_field(N, args.seed, "cuda")
    u_np = host_field(u)
    del u
    torch.cuda.empty_cache()
    ks = O.wavenumber_grid((N, N, N), (2 * np.pi,) * 3)
    cores = os.cpu_count() or 1
    O.set_fft_workers(cores)
    t0 = time.perf_counter()
    st = O.s2s_setup(u_np, ks, ("linear", args.dk), "two_thirds")
    t_setup = time.perf_counter() - t0
    nsh = st["nsh"]
    for w in range(args.warmup):
        O.s2s_column(st, (7 + w) % nsh, comps=[w % 3])
    times = []
    for s in range(args.steps):
        t0 = time.perf_counter()
        O.s2s_column(st, (7 + s) % nsh, comps=[s % 3])
        times.append(time.perf_counter() - t0)
    t_piece = float(np.mean(times))
    t_matrix = t_setup + nsh * 3 * t_piece
    v = 1.0 / t_matrix
    sample = (f"oracle restatement of _shell_to_shell_fft! (FP64, scipy.fft {cores} threads): setup once "
              f"({t_setup:.1f} s) + {args.steps} timed pieces of one advected component of one mediator "
              f"({t_piece:.2f} s each); T(n,m) time = setup + {nsh}x3 pieces")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_piece * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{N}^3 D=3 {nsh}-shell shell-to-shell, LinearBinning({args.dk}), 2/3",
                       "seed": args.seed},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "julia": julia_probe(),
            "note": "the reference is Julia (FFTW+OhMyThreads) and is not installed on this box, so the timed "
                    "CPU implementation is the FP64 oracle restatement of its algorithm"}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    ws, rank, local = dist_setup()
    dev = torch.device("cuda", local)
    import __graft_entry__
    F = __graft_entry__.load_package()
    N = args.n
    ns = (N, N, N)
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    edges = np.asarray(F.shell_edges(F.LinearBinning(args.dk), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    dmask = F.dims_mask(F.IsotropicShells(), 3)
    u = make_field(N, args.seed, dev)
    stream = torch.cuda.Stream(device=dev)
    plan = F.Plan(ns, 3, 3, "two_thirds", 32, False, ks)
    plan.set_stream(stream.cuda_stream)
    T = torch.zeros((nsh, nsh), dtype=torch.float64, device=dev)
    net = torch.zeros(nsh, dtype=torch.float64, device=dev)
    asym = torch.zeros(1, dtype=torch.float64, device=dev)

    def step():
        plan.shell_to_shell_device(u.data_ptr(), 0, edges, dmask, 0, 0, F._lib.S2S_BATCHED, T.data_ptr(),
                                   net.data_ptr(), asym.data_ptr())

    bus = None
    try:
        pr = torch.cuda.get_device_properties(dev)
        bus = "%08X:%02X:%02X.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
    except Exception:
        bus = None
    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            step()
        torch.cuda.synchronize()
        barrier(ws)
        clk = Clocks(bus)
        clk.start()
        l0 = F.launch_count()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        launches = F.launch_count() - l0
        clocks = clk.stop()
        barrier(ws)
    ms = e0.elapsed_time(e1) / args.steps
    value, ms_max = replica_throughput(ws, 1.0, ms)
    T32 = T.cpu().numpy().copy()
    net32 = net.cpu().numpy().copy()

    # ---- dominant kernel from per-launch CUDA events (one eager step) ----
    F._lib.prof_enable(True)
    with torch.cuda.stream(stream):
        step()
    torch.cuda.synchronize()
    prof = F._lib.prof_read_all()
    F._lib.prof_enable(False)
    prof_ms = sum(v[0] for v in prof.values())
    dom = max(prof.items(), key=lambda kv: kv[1][0])
    dname, (dms, dbytes, dn) = dom
    peak, peak_kind = read_peaks()
    achieved = dbytes / (dms / 1e3) / 1e9
    traffic = read_traffic(dname)
    roofline = {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "launches_per_step": dn,
                "algorithmic_bytes_per_launch": dbytes / dn, "avg_launch_ms": dms / dn,
                "traffic": traffic, "share_of_step": dms / prof_ms,
                "all_kernels": {k: {"ms": v[0], "GBps": v[1] / (v[0] / 1e3) / 1e9 if v[0] > 0 else None,
                                    "launches": v[2]} for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])},
                "step_alg_bytes_GB": sum(v[1] for v in prof.values()) / 1e9}

    # ---- end to end through the host-buffer C ABI ----
    host = torch.empty((3, N, N, N), dtype=torch.complex64, pin_memory=True)
    host.copy_(u)
    host_np = np.transpose(host.numpy(), (3, 2, 1, 0))
    for _ in range(3):   # warm the host path: eager run, capture of its graph, first replay (graph upload)
        plan.shell_to_shell(host_np, edges, dmask, False, 0, F._lib.S2S_BATCHED)
    torch.cuda.synchronize()
    h2d0 = plan.info()[8]
    call_ms = []
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        t1 = time.perf_counter()
        Th, _, _ = plan.shell_to_shell(host_np, edges, dmask, False, 0, F._lib.S2S_BATCHED)
        call_ms.append(round((time.perf_counter() - t1) * 1e3, 2))
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    e2e_s = allmax(ws, e2e_s)
    # the library copies only the 2/3-kept slabs of the host field (the path reads nothing else)
    h2d = (plan.info()[8] - h2d0) / args.e2e_steps
    e2e = {"value": ws / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(nsh * nsh * 8), "host_field_bytes": int(host.numel() * 8),
           "steps": args.e2e_steps, "call_ms": call_ms}
    del host, host_np

    # ---- cuFFT beside, as a comparison only: the library's 3D real transforms at this size, and
    # what the reference algorithm's transform count for one T(n,m) (3 + 12 N_sh unpruned real 3D
    # transforms) would take on them alone ----
    cufft = None
    if not args.no_cufft:
        x = torch.randn((N, N, N), dtype=torch.float32, device=dev)
        X = torch.fft.rfftn(x)
        t_f = _timed_ms(lambda: torch.fft.rfftn(x), stream, 5, warm=2)
        t_i = _timed_ms(lambda: torch.fft.irfftn(X, s=(N, N, N)), stream, 5, warm=2)
        per = 0.5 * (t_f + t_i)
        n_t = 3 + 12 * nsh
        cufft = {"library": "cuFFT (torch.fft, %s)" % torch.version.cuda, "rfftn_ms": t_f, "irfftn_ms": t_i,
                 "GBps_per_transform_model": 6.0 * N ** 3 * 4 / (per / 1e3) / 1e9,
                 "unpruned_transforms_per_T": n_t, "transforms_only_ms_per_T": n_t * per,
                 "ours_ms_per_T": ms, "ours_vs_cufft_transforms_only": n_t * per / ms}
        del x, X
        torch.cuda.empty_cache()

    # ---- plain FP64 form (one nonlinear term per mediator) ----
    fp64 = None
    T64n = None
    oracle_col = None
    if not args.no_fp64:
        del plan
        F.clear_plans()
        torch.cuda.empty_cache()
        u64 = u.to(torch.complex128)
        p64 = F.Plan(ns, 3, 3, "two_thirds", 64, True, ks)
        p64.set_stream(stream.cuda_stream)
        T64 = torch.zeros((nsh, nsh), dtype=torch.float64, device=dev)
        with torch.cuda.stream(stream):
            # warm: allocate the workspace and build the shell table with one FP64 nonlinear term
            p64.shell_to_shell_device(u64.data_ptr(), 0, edges[:2], dmask, 0, 0, F._lib.S2S_PLAIN, T64.data_ptr(),
                                      0, 0)
            torch.cuda.synchronize()
            e0.record(stream)
            p64.shell_to_shell_device(u64.data_ptr(), 0, edges, dmask, 0, 0, F._lib.S2S_PLAIN, T64.data_ptr(),
                                      0, 0)
            e1.record(stream)
            torch.cuda.synchronize()
        s64 = allmax(ws, e0.elapsed_time(e1) / 1e3)
        T64n = T64.cpu().numpy()
        rel = float(np.max(np.abs(T32 - T64n)) / np.max(np.abs(T64n)))
        Tanti = 0.5 * (T32 - T32.T)
        fp64 = {"value": ws / s64, "unit": UNIT, "s_per_matrix": s64, "speedup_fp32_batched": value / (ws / s64),
                "rel_err_fp32_vs_fp64_maxnorm": rel,
                "conservation_fp32": float(abs(net32.sum()) / np.abs(T32).sum()),
                "conservation_fp64": float(abs(T64n.sum()) / np.abs(T64n).sum()),
                "conservation_fp32_antisymmetrized": float(abs(Tanti.sum()) / np.abs(Tanti).sum()),
                "rel_err_fp32_antisymmetrized_vs_fp64": float(np.max(np.abs(Tanti - T64n)) / np.max(np.abs(T64n))),
                "max_asym_fp64": float(np.max(np.abs(T64n + T64n.T)))}
        del u64, p64

    # ---- CPU oracle baseline (rank 0, single GPU only) ----
    cpu = None
    if not args.no_cpu and ws == 1:
        try:
            import oracle as O
            u_np = host_field(u)
            ksd = O.wavenumber_grid(ns, (2 * np.pi,) * 3)
            t_setup, t_piece, t_matrix, cores, _, st = cpu_sample(u_np, ksd, args.dk)
            cpu = {"value": 1.0 / t_matrix, "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": f"oracle restatement (FP64, scipy.fft x{cores} threads) of the same 512^3 field: "
                             f"setup {t_setup:.1f} s + one advected component of one mediator {t_piece:.1f} s; "
                             f"T(n,m) = setup + {nsh}x3 pieces"}
            if args.oracle_column >= 1:
                # one full column of the headline matrix from the oracle: the FP32 and FP64 GPU
                # results against the FFT-based FP64 restatement of the reference on the same field
                m = args.oracle_column - 1
                t0 = time.perf_counter()
                col = O.s2s_column(st, m)
                # errors in max-norm relative to max|T| over the whole matrix
                sc = float(np.max(np.abs(T64n if T64n is not None else T32)))
                oracle_col = {"m": m + 1, "seconds": time.perf_counter() - t0,
                              "max_abs_T_column": float(np.max(np.abs(col))), "max_abs_T": sc,
                              "rel_err_fp32_maxnorm": float(np.max(np.abs(T32.T[:, m] - col)) / sc)}
                if T64n is not None:
                    oracle_col["rel_err_fp64_maxnorm"] = float(np.max(np.abs(T64n.T[:, m] - col)) / sc)
            del st
        except Exception as e:   # the baseline never blocks the GPU line
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {e}"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": max(3, args.warmup), "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"{N}^3 D=3 {nsh}-shell shell-to-shell T(n,m), LinearBinning({args.dk}), "
                                       "OrszagTwoThirds, FP32-batched (FP64 sums)",
                           "grid": N, "shells": nsh, "spectrum": "k^-5/3 on [4,170], k^4 rise below 4, solenoidal",
                           "seed": args.seed, "parallelism": f"replicas x{ws}",
                           "l2": "inputs 3.2 GB per step >> 129 MB L2; no flush needed"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches / args.steps),
                "gpu_launches_timed_region": int(launches), "clocks": clocks, "fp64_plain": fp64,
                "oracle_column": oracle_col, "cufft_comparison": cufft}
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_closure(args):
    """Learned closure vs exact coarse-graining flux: a seeded k^4 exp(-2(k/8)^2) field at N^3 is
    evolved by SSP-RK3 forced Navier-Stokes on the GPU (nu = 2e-3, forcing of 0 < |k| <= 2 at
    constant power 0.1, dt = 5e-3); for each Gaussian filter k_c in {8, 16, 32} (ell = pi/k_c) the
    exact path gives A = grad ū, tau and Pi_ell; the MLP trains on the half z < N/2 and is scored on
    the other half against Pi_ell, beside the gradient (Clark) model and no closure."""
    import torch
    import __graft_entry__
    F = __graft_entry__.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    N = args.closure_n
    ns = (N, N, N)
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = make_field(N, args.seed, dev, spectrum="k4exp8")
    u *= math.sqrt(0.5 / (0.5 * float((u.abs() ** 2).sum())))
    nu, dt, kf, power = 2e-3, 5e-3, 2.0, 0.1
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    F.evolve_forced_navier_stokes_device(u, ks, 1, dt, nu, kf, power)    # workspace + first step
    l0 = F.launch_count()
    e0.record()
    F.evolve_forced_navier_stokes_device(u, ks, args.closure_nsteps - 1, dt, nu, kf, power)
    e1.record()
    torch.cuda.synchronize()
    evolve_ms = e0.elapsed_time(e1) / max(1, args.closure_nsteps - 1)
    evolve_launches = (F.launch_count() - l0) / max(1, args.closure_nsteps - 1)
    energy = 0.5 * float((u.abs() ** 2).sum())
    n = N ** 3
    half = n // 2
    flop_pt = 2 * (9 * 64 + 64 * 64 + 64 * 6)
    results = {}
    for kc in (8, 16, 32):
        ell = math.pi / kc
        F.closure_data(u, ks, ell)                     # warm the coarse-graining plan
        torch.cuda.synchronize()
        e0.record()
        d = F.closure_data(u, ks, ell)
        e1.record()
        torch.cuda.synchronize()
        exact_ms = e0.elapsed_time(e1)
        m = F.SubfilterStressMLP(seed=args.seed, mixed=args.mixed)
        t0 = time.perf_counter()
        hist = m.train(d, 0, half, steps=args.train_steps, batch=args.train_batch, lr=args.lr,
                       log_every=max(1, args.train_steps // 5))
        torch.cuda.synchronize()
        train_s = time.perf_counter() - t0
        ev = m.evaluate(d, half, n)
        for _ in range(3):
            m.predict(d.A, n, n, want_tau=False)
        torch.cuda.synchronize()
        reps = 10
        e0.record()
        for _ in range(reps):
            m.predict(d.A, n, n, want_tau=False)
        e1.record()
        torch.cuda.synchronize()
        inf_ms = e0.elapsed_time(e1) / reps
        results[str(kc)] = {"ell": ell, "exact_path_ms": exact_ms, "exact_points_per_s": n / (exact_ms / 1e3),
                            "train_s": train_s, "train_steps": args.train_steps, "train_points_per_step": args.train_batch,
                            "loss_history": hist, "inference_ms": inf_ms,
                            "inference_points_per_s": n / (inf_ms / 1e3),
                            "inference_tflops": n * flop_pt / (inf_ms / 1e3) / 1e12,
                            "mean_flux_exact": d.mean_flux, **ev}
        del d, m
        torch.cuda.empty_cache()
    headline = results["16"]
    bf16, bf16_kind = read_bf16_peak()
    hbm, hbm_kind = read_peaks()
    tfl = headline["inference_tflops"]
    io_gbs = n * (9 * 4 + 4) / (headline["inference_ms"] / 1e3) / 1e9   # 9 FP32 inputs, 1 FP32 flux per point
    roofline = {"bound": "tensor", "kernel": "mlp_forward (tcgen05, BF16 operands, FP32 accumulation)",
                "achieved": tfl, "peak": bf16, "unit": "TFLOP/s", "frac": tfl / bf16, "peak_source": bf16_kind,
                "flop_per_point": flop_pt, "traffic": None,
                "hbm": {"achieved": io_gbs, "peak": hbm, "unit": "GB/s", "frac": io_gbs / hbm,
                        "bytes_per_point": 40, "peak_source": hbm_kind}}
    line = {"metric": "learned closure: inference points/s, Pi_ell correlation and rel L2 vs exact coarse-graining "
                      "flux (256^3 forced NS, Gaussian k_c = 16)",
            "value": headline["inference_points_per_s"], "unit": "points/s", "n_gpus": 1, "steps": 10,
            "warmup": 3, "ms_per_step": headline["inference_ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 (FP32 accumulation)", "data": "synthetic",
            "config": {"workload": f"{N}^3 D=3 forced SSP-RK3 NS ({args.closure_nsteps} steps, nu={nu}, dt={dt}, "
                                   f"forcing 0<|k|<={kf} at power {power}) from k^4 exp(-2(k/8)^2); Gaussian filter "
                                   "k_c in {8,16,32}, ell = pi/k_c; MLP 9-64-64-6 (homogeneous form" +
                                   (", residual over the gradient model" if args.mixed else "") +
                                   ") trained on z < N/2, scored on z >= N/2",
                       "seed": args.seed},
            "roofline": roofline,
            "evolve": {"ms_per_rk3_step": evolve_ms, "launches_per_step": evolve_launches, "energy": energy},
            "flop_per_point": flop_pt, "results": results}
    print(json.dumps(line), flush=True)
    return 0


def make_field_nd(ns, seed, device, spectrum, ncomp=None, project=True, dtype=None):
    """Seeded Hermitian random-phase field û = fft(u)/Np on grid ns (any nd), shell spectrum
    ``spectrum(|k|)`` (torch function), Leray-projected when ncomp == nd, mean removed. Returned as a
    contiguous (ncomp, *reversed(ns)) CUDA tensor: the column-major (ns..., ncomp) layout."""
    import torch
    nd = len(ns)
    ncomp = nd if ncomp is None else ncomp
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    shape = tuple(reversed(ns))
    kk = []
    for d in range(nd):
        k1 = torch.fft.fftfreq(ns[d], d=1.0 / ns[d], device=device, dtype=torch.float64)
        view = [1] * nd
        view[nd - 1 - d] = ns[d]
        kk.append(k1.view(view))
    k2 = sum(k * k for k in kk)
    km = torch.sqrt(k2)
    amp = torch.where(km > 0, torch.sqrt(spectrum(km) / km.clamp_min(1e-30) ** (nd - 1)), torch.zeros_like(km))
    Np = float(np.prod(ns))
    u = torch.empty((ncomp,) + shape, dtype=torch.complex128, device=device)
    for c in range(ncomp):
        r = torch.randn(shape, generator=g, device=device, dtype=torch.float64)
        u[c] = torch.fft.fftn(r) * (amp / Np)
    if project and ncomp == nd:
        div = sum(kk[d] * u[d] for d in range(nd)) / torch.where(k2 > 0, k2, torch.ones_like(k2))
        for d in range(nd):
            u[d] -= kk[d] * div
    u[(slice(None),) + (0,) * nd] = 0
    return u.to(dtype or torch.complex64).contiguous()


def draw_batch_instances(F, seed, n_instances, dev):
    """The uneven batch drawn from ``seed``: instance i is 2D (64^2..1024^2) when i % 4 < 2, else 3D
    (64^3..192^3), sizes 2^n and 3*2^n; odd instances carry a passive scalar; shell geometry drawn
    from isotropic / perpendicular / parallel. Returns the FP32 and FP64 instance specs (device
    fields), a description per instance and the FP32 input bytes."""
    import torch
    rng = np.random.default_rng(seed)
    sizes2 = [64, 96, 128, 192, 256, 384, 512, 768, 1024]
    sizes3 = [64, 96, 128, 192]
    e_vel = lambda k: k ** 4 * torch.exp(-2 * (k / 4) ** 2)          # noqa: E731
    e_sca = lambda k: k ** 2 * torch.exp(-(k / 6) ** 2)              # noqa: E731
    geos = ["isotropic", "perpendicular", "parallel"]
    specs32, specs64, desc = [], [], []
    h2d = 0
    for i in range(n_instances):
        nd = 2 if i % 4 < 2 else 3
        n = int(rng.choice(sizes2 if nd == 2 else sizes3))
        ns = (n,) * nd
        ks = F.wavenumber_grid(ns, (2 * np.pi,) * nd)
        scalar = i % 2 == 1
        gname = geos[int(rng.integers(0, 3))]
        geo = {"isotropic": F.IsotropicShells(), "perpendicular": F.PerpendicularShells(),
               "parallel": F.ParallelShells(dims=(nd,))}[gname]
        u = make_field_nd(ns, seed * 1000 + 2 * i, dev, e_vel, dtype=torch.complex128)
        th = make_field_nd(ns, seed * 1000 + 2 * i + 1, dev, e_sca, ncomp=1, project=False,
                           dtype=torch.complex128) if scalar else None
        base = {"ks": ks, "ns": ns, "geometry": geo, "binning": F.LinearBinning(1.0)}
        specs64.append(dict(base, velocity_dev=u.view(-1), scalar_dev=th.view(-1) if scalar else None))
        u32 = u.to(torch.complex64).view(-1)
        th32 = th.to(torch.complex64).view(-1) if scalar else None
        specs32.append(dict(base, velocity_dev=u32, scalar_dev=th32))
        h2d += u32.numel() * 8 + (th32.numel() * 8 if scalar else 0)
        desc.append(f"{'x'.join(map(str, ns))}:{'scalar' if scalar else 'ke'}:{gname}")
    return specs32, specs64, desc, h2d


def run_batch(args):
    """64 uneven spectral-flux instances (half kinetic energy, half passive scalar; 2D 64^2..1024^2 and
    3D 64^3..192^3, sizes 2^n and 3*2^n; isotropic / perpendicular / parallel shells) as ONE graph
    launch in FP32 (FP64 shell sums), against the same set in FP64 for the per-instance error."""
    import torch
    import __graft_entry__
    F = __graft_entry__.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    specs32, specs64, desc, h2d = draw_batch_instances(F, args.seed, args.instances, dev)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed(fn, reps):
        for _ in range(max(3, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    F.autotune_clear()
    b32 = F.SpectralFluxBatch(specs32, precision=32, n_branches=args.branches, autotune=True)
    t0 = time.perf_counter()
    b32.run()                                      # eager: allocation + autotuning
    torch.cuda.synchronize()
    tune_s = time.perf_counter() - t0
    tune = F.autotune_summary()
    b32.run()                                      # capture + launch
    bus = None
    try:
        pr = torch.cuda.get_device_properties(dev)
        bus = "%08X:%02X:%02X.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
    except Exception:
        pass
    clk = Clocks(bus)
    clk.start()
    l0 = F.launch_count()
    ms_graph = timed(b32.run, args.steps)
    launches = (F.launch_count() - l0) / (args.steps + max(3, args.warmup))
    clocks = clk.stop()
    ms_eager = timed(b32.run_eager, args.steps)
    roofline = prof_roofline(F, b32.run_eager, torch.cuda.synchronize)
    r32 = b32.results()
    info = b32.info()
    # same set, default kernels (autotuner off), graph
    F.autotune_enable(False)
    bnt = F.SpectralFluxBatch(specs32, precision=32, n_branches=args.branches, autotune=False)
    bnt.run()
    bnt.run()
    ms_graph_untuned = timed(bnt.run, args.steps)
    bnt.close()
    del bnt
    # FP64 reference set (eager, plain FP64 path)
    b64 = F.SpectralFluxBatch(specs64, precision=64, n_branches=1, autotune=False)
    b64.run()
    torch.cuda.synchronize()
    ms64 = timed(b64.run_eager, 1)
    r64 = b64.results()
    b64.close()
    errs = []
    for a, b in zip(r32, r64):
        errs.append(float(np.max(np.abs(a.transfer_spectrum.astype(np.float64) - b.transfer_spectrum)) /
                         max(np.max(np.abs(b.transfer_spectrum)), 1e-300)))
    # end to end: pinned host inputs -> device, one graph launch, T back to the host
    hosts = [(s["velocity_dev"].cpu().pin_memory(), s["scalar_dev"].cpu().pin_memory() if s["scalar_dev"] is not None
              else None) for s in specs32]
    d2h = sum(int(it["T"].numel()) * 8 for it in b32.items)

    def e2e_step():
        for (hv, hs), it in zip(hosts, b32.items):
            if hs is not None:
                it["a"].copy_(hv, non_blocking=True)
                it["f"].copy_(hs, non_blocking=True)
            else:
                it["f"].copy_(hv, non_blocking=True)
        b32.run()
        outs = [it["T"].to("cpu", non_blocking=True) for it in b32.items]
        torch.cuda.synchronize()
        return outs

    for _ in range(2):
        e2e_step()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    n = len(specs32)
    modes = sum(int(np.prod(s["ns"])) for s in specs32)
    line = {"metric": f"uneven batch: {n} spectral-flux instances per graph launch (FP32, FP64 sums), instances/s",
            "value": n / (ms_graph / 1e3), "unit": "instances/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms_graph, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{n} instances: 2D 64^2-1024^2 and 3D 64^3-192^3 (2^n, 3*2^n), half KE flux "
                                   "(E ~ k^4 exp(-2(k/4)^2)) and half passive-scalar flux (k^2 exp(-(k/6)^2)); "
                                   "isotropic / perpendicular / parallel shells, LinearBinning(1), 2/3 rule",
                       "seed": args.seed, "instances": desc, "modes_total": modes,
                       "l2": "inputs cycle through ~%.1f GB per launch (> 129 MB L2)" % (h2d / 1e9)},
            "roofline": roofline, "modes_per_s": modes / (ms_graph / 1e3),
            "graph": {"kernels": info["graph_kernels"], "branches": info["branches"]},
            "ms_sequential_eager_autotuned": ms_eager, "ms_graph_default_kernels": ms_graph_untuned,
            "speedup_graph_vs_sequential": ms_eager / ms_graph,
            "speedup_autotuned_vs_default_graph": ms_graph_untuned / ms_graph,
            "autotune": {"entries": tune["entries"], "runtime_engine_chosen": tune["runtime_engine_chosen"],
                         "tuning_s": tune_s, "sum_ms_default": tune["ms_default_sum"],
                         "sum_ms_best": tune["ms_best_sum"]},
            "fp64_plain_ms": ms64, "speedup_fp32_graph_vs_fp64": ms64 / ms_graph,
            "rel_err_vs_fp64": {"max": max(errs), "median": float(np.median(errs))},
            "e2e": {"value": n / e2e_s, "unit": "instances/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": args.e2e_steps},
            "gpu_launches": int(launches), "clocks": clocks}
    print(json.dumps(line), flush=True)
    b32.close()
    return 0


def run_partial(args):
    """512^3 helical partial fluxes Pi^{s_k s_p s_q}(K) of kinetic energy AND helicity (2 x 8 channels,
    DyadicBinning(2): 8 bands [2,4)..[256,512), 2/3 rule) from one pass (four shared nonlinear
    terms), replayed as one CUDA graph: FP32 transforms and products, FP64 shell sums. Compared with
    the per-invariant plain path in FP32 and in FP64 (the error reference)."""
    import torch
    import __graft_entry__
    F = __graft_entry__.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    N = args.n
    ns = (N, N, N)
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    edges = np.asarray(F.shell_edges(F.DyadicBinning(2.0), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    u = make_field(N, args.seed, dev)
    stream = torch.cuda.Stream(device=dev)
    plan = F.Plan(ns, 3, 3, "two_thirds", 32, False, ks)
    plan.set_stream(stream.cuda_stream)
    T = torch.zeros(2 * 8 * nsh, dtype=torch.float64, device=dev)
    invs = [F.KineticEnergy().code, F.Helicity().code]
    dcode = 1 if args.decomp == "helical" else 3   # decomposition codes of the C ABI
    dname_ = "HelicalDecomposition" if dcode == 1 else "ToroidalPoloidalDecomposition"

    def step():
        plan.partial_fluxes_batched_device(u.data_ptr(), dcode, invs, edges, 7, False, T.data_ptr())

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    bus = None
    try:
        pr = torch.cuda.get_device_properties(dev)
        bus = "%08X:%02X:%02X.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
    except Exception:
        pass
    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            step()
        torch.cuda.synchronize()
        clk = Clocks(bus)
        clk.start()
        l0 = F.launch_count()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        launches = (F.launch_count() - l0) / args.steps
        clocks = clk.stop()
    ms = e0.elapsed_time(e1) / args.steps
    T32 = T.cpu().numpy().reshape(2, 8, nsh).copy()

    def eager():   # per-kernel breakdown of one eager pass (CUDA events around each launch)
        with torch.cuda.stream(stream):
            step()

    roofline = prof_roofline(F, eager, torch.cuda.synchronize)
    # plain per-invariant path, FP32 (one call per invariant, four nonlinear terms each)
    Tp = torch.zeros(8 * nsh, dtype=torch.float64, device=dev)
    with torch.cuda.stream(stream):
        for inv in invs:
            plan.partial_fluxes_device(u.data_ptr(), dcode, inv, edges, 7, False, Tp.data_ptr())
        torch.cuda.synchronize()
        e0.record(stream)
        for inv in invs:
            plan.partial_fluxes_device(u.data_ptr(), dcode, inv, edges, 7, False, Tp.data_ptr())
        e1.record(stream)
        torch.cuda.synchronize()
    ms_plain32 = e0.elapsed_time(e1)
    del plan
    F.clear_plans()
    torch.cuda.empty_cache()
    # plain FP64 reference
    u64 = u.to(torch.complex128)
    p64 = F.Plan(ns, 3, 3, "two_thirds", 64, True, ks)
    p64.set_stream(stream.cuda_stream)
    T64 = np.zeros((2, 8, nsh))
    Tq = torch.zeros(8 * nsh, dtype=torch.float64, device=dev)
    with torch.cuda.stream(stream):
        torch.cuda.synchronize()
        e0.record(stream)
        for j, inv in enumerate(invs):
            p64.partial_fluxes_device(u64.data_ptr(), dcode, inv, edges, 7, False, Tq.data_ptr())
            torch.cuda.synchronize()
            T64[j] = Tq.cpu().numpy().reshape(8, nsh)
        e1.record(stream)
        torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1)
    del p64, u64
    rel = [float(np.max(np.abs(T32[j] - T64[j])) / np.max(np.abs(T64[j]))) for j in range(2)]
    cons = [float(abs(T32[j].sum()) / np.abs(T32[j]).sum()) for j in range(2)]
    kind = "helical" if dcode == 1 else "toroidal/poloidal"
    line = {"metric": f"{N}^3 {kind} partial fluxes, KE + helicity (16 channels), one graph launch: sets/s",
            "value": 1000.0 / ms, "unit": "sets/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{N}^3 D=3 {dname_} 8 channels x (KineticEnergy, Helicity), "
                                   f"DyadicBinning(2) ({nsh} bands), OrszagTwoThirds, complex64 fields, FP64 sums",
                       "spectrum": "k^-5/3 on [4,170], k^4 rise below 4, solenoidal", "seed": args.seed,
                       "l2": "inputs 3.2 GB per step >> 129 MB L2"},
            "roofline": roofline, "ms_plain_fp32_two_calls": ms_plain32, "speedup_vs_plain_fp32": ms_plain32 / ms,
            "ms_plain_fp64_two_calls": ms64, "speedup_vs_plain_fp64": ms64 / ms,
            "rel_err_vs_fp64_maxnorm": {"ke": rel[0], "helicity": rel[1]},
            "sum_over_channels_and_bands_rel": {"ke": cons[0], "helicity": cons[1]},
            "gpu_launches": int(launches), "clocks": clocks}
    print(json.dumps(line), flush=True)
    return 0


def _timed_ms(fn, stream, reps, warm=1):
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def run_padded(args):
    """256^3 D=3 32-shell shell-to-shell with the exact 3/2 rule (384^3 transforms), field
    E ~ k^4 exp(-2 (k/8)^2): FP32-batched vs plain FP64; antisymmetry and per-shell error."""
    import torch
    import __graft_entry__
    F = __graft_entry__.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    N = 256
    ns = (N, N, N)
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    edges = np.asarray(F.shell_edges(F.LinearBinning(7.0), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    u = make_field(N, args.seed, dev, spectrum="k4exp8")
    stream = torch.cuda.Stream(device=dev)
    plan = F.Plan(ns, 3, 3, "three_halves", 32, False, ks)
    plan.set_stream(stream.cuda_stream)
    T = torch.zeros((nsh, nsh), dtype=torch.float64, device=dev)
    net = torch.zeros(nsh, dtype=torch.float64, device=dev)
    asym = torch.zeros(1, dtype=torch.float64, device=dev)

    def step():
        plan.shell_to_shell_device(u.data_ptr(), 0, edges, 7, 0, 0, F._lib.S2S_BATCHED, T.data_ptr(),
                                   net.data_ptr(), asym.data_ptr())

    l0 = F.launch_count()
    ms = _timed_ms(step, stream, args.steps, warm=max(3, args.warmup))
    launches = (F.launch_count() - l0) / (args.steps + max(3, args.warmup))
    T32 = T.cpu().numpy().copy()
    net32 = net.cpu().numpy().copy()

    def eager():
        with torch.cuda.stream(stream):
            step()

    roofline = prof_roofline(F, eager, torch.cuda.synchronize)
    del plan
    F.clear_plans()
    torch.cuda.empty_cache()
    u64 = u.to(torch.complex128)
    p64 = F.Plan(ns, 3, 3, "three_halves", 64, True, ks)
    p64.set_stream(stream.cuda_stream)
    T64 = torch.zeros((nsh, nsh), dtype=torch.float64, device=dev)
    ms64 = _timed_ms(lambda: p64.shell_to_shell_device(u64.data_ptr(), 0, edges, 7, 0, 0, F._lib.S2S_PLAIN,
                                                        T64.data_ptr(), 0, 0), stream, 1, warm=1)
    T64n = T64.cpu().numpy()
    scale = np.max(np.abs(T64n))
    line = {"metric": "256^3 3/2-padded 32-shell shell-to-shell T(n,m)/s: FP32-batched vs FP64 plain",
            "value": 1000.0 / ms, "unit": "T(n,m)/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"256^3 D=3 {nsh}-shell shell-to-shell, LinearBinning(7), PaddedThreeHalves "
                                   "(384^3 transforms), E ~ k^4 exp(-2(k/8)^2), FP32-batched with FP64 sums",
                       "seed": args.seed},
            "roofline": roofline, "fp64_plain_ms": ms64, "speedup_vs_fp64_plain": ms64 / ms,
            "rel_err_vs_fp64_maxnorm": float(np.max(np.abs(T32 - T64n)) / scale),
            "per_shell_rel_err_max_over_shells_with_transfer": float(np.max(
                (np.abs(T32 - T64n).max(axis=0) / np.maximum(np.abs(T64n).max(axis=0), 1e-300))[
                    np.abs(T64n).max(axis=0) > 1e-3 * scale])),
            "antisymmetry_fp32_rel": float(np.max(np.abs(T32 + T32.T)) / scale),
            "antisymmetry_fp64_rel": float(np.max(np.abs(T64n + T64n.T)) / scale),
            "conservation_fp32": float(abs(net32.sum()) / np.abs(T32).sum()),
            "gpu_launches": int(launches)}
    print(json.dumps(line), flush=True)
    return 0


def run_m2m(args):
    """32^3 D=3 resolved mode-to-mode S(k|p) (32768^2 = 1.07e9 pairs, FP64 sums, 8.6 GB output),
    E ~ k^4 exp(-2 (k/8)^2), 2/3 rule; shell sums of S against T(n,m) of the shell-to-shell path."""
    import torch
    import __graft_entry__
    F = __graft_entry__.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    N = 32
    ns = (N, N, N)
    nm = N ** 3
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    u = make_field(N, args.seed, dev, spectrum="k4exp8").to(torch.complex128).contiguous()
    stream = torch.cuda.Stream(device=dev)
    plan = F.Plan(ns, 3, 3, "two_thirds", 64, True, ks)
    plan.set_stream(stream.cuda_stream)
    S = torch.empty((nm, nm), dtype=torch.float64, device=dev)
    net = torch.empty(nm, dtype=torch.float64, device=dev)
    res = {}
    for fp64 in (True, False):
        ms = _timed_ms(lambda: plan.mode_to_mode_device(u.data_ptr(), 0, fp64, S.data_ptr(), net.data_ptr()),
                       stream, max(1, args.steps), warm=2)
        res["fp64_products" if fp64 else "fp32_products"] = {
            "ms": ms, "pairs_per_s": nm * nm / (ms / 1e3), "GBps_S_write": 8.0 * nm * nm / (ms / 1e3) / 1e9}
    # shell sums of S (FP64 products) against T(n,m)
    plan.mode_to_mode_device(u.data_ptr(), 0, True, S.data_ptr(), net.data_ptr())
    edges = np.asarray(F.shell_edges(F.LinearBinning(1.0), F.kmax(ks)), dtype=np.float64)
    nsh = len(edges) - 1
    idx = torch.from_numpy(plan.assign_shells(edges, 7, False).ravel(order="F")).to(dev)
    valid = idx > 0
    oh = torch.zeros((nsh, nm), dtype=torch.float64, device=dev)
    oh[idx[valid] - 1, torch.nonzero(valid).squeeze(1)] = 1.0
    # S is [k, p] column-major (k fastest): Tsum[n, m] = sum_{k in n, p in m} S(k|p)
    Sm = S.view(nm, nm).t()            # Sm[k, p]
    Tsum = (oh @ Sm @ oh.t()).cpu().numpy()
    T = np.zeros((nsh, nsh))
    p2 = F.Plan(ns, 3, 3, "two_thirds", 64, True, ks)
    Tt = torch.zeros((nsh, nsh), dtype=torch.float64, device=dev)
    with torch.cuda.stream(stream):
        p2.shell_to_shell_device(u.data_ptr(), 0, edges, 7, 0, 0, F._lib.S2S_PLAIN, Tt.data_ptr(), 0, 0)
    torch.cuda.synchronize()
    T = Tt.cpu().numpy().T            # the library writes T(n, m) column-major
    scale = np.max(np.abs(T))
    head = res["fp64_products"]
    hbm, hbm_kind = read_peaks()
    roofline = {"bound": "hbm", "kernel": "mode_to_mode (FP64 products)", "achieved": head["GBps_S_write"],
                "peak": hbm, "unit": "GB/s", "frac": head["GBps_S_write"] / hbm, "peak_source": hbm_kind,
                "algorithmic_bytes_per_launch": 8.0 * nm * nm, "traffic": None,
                "note": "bytes = the FP64 S matrix written once; the kernel is bound by its triad products "
                        "(FP64 arithmetic), not by that write"}
    line = {"metric": "32^3 resolved mode-to-mode S(k|p): pairs/s (FP64 sums)", "value": head["pairs_per_s"],
            "unit": "pairs/s", "n_gpus": 1, "steps": max(1, args.steps), "warmup": 2, "ms_per_step": head["ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "32^3 D=3 S(k|p) over all 32768^2 mode pairs, OrszagTwoThirds, E ~ k^4 exp(-2(k/8)^2)",
                       "seed": args.seed},
            "roofline": roofline, "forms": res, "shell_sum_vs_shell_to_shell_rel": float(np.max(np.abs(Tsum - T)) / scale),
            "S_antisymmetry_rel": float((S + S.t()).abs().max().item() / S.abs().max().item()),
            "net_sum_rel": float(abs(net.sum().item()) / net.abs().sum().item())}
    print(json.dumps(line), flush=True)
    return 0


def run_band(args):
    """512^3 smooth band-to-band T(K,Q) over 7 log-Gaussian bands (centres 2..128, logwidth 0.6),
    kinetic energy, 2/3 rule, complex64 field: every band's nonlinear term through the live-box
    passes (weighted copies of the field, weighted carriers binned in one pass) against the plan's
    plain per-band path in FP32 and in FP64 (the error reference)."""
    import os
    import torch
    import __graft_entry__
    F = __graft_entry__.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    N = args.n
    ns = (N, N, N)
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    centers = [2.0 ** j for j in range(1, 8)]
    lw = 0.6
    nb = len(centers)
    u = make_field(N, args.seed, dev)
    stream = torch.cuda.Stream(device=dev)
    T = torch.zeros((nb, nb), dtype=torch.float64, device=dev)
    net = torch.zeros(nb, dtype=torch.float64, device=dev)
    asym = torch.zeros(1, dtype=torch.float64, device=dev)
    ke = F.KineticEnergy().code

    def run(plan, uu, TT):
        plan.band_to_band_device(uu.data_ptr(), 0, centers, lw, 7, False, ke, TT.data_ptr(), net.data_ptr(),
                                 asym.data_ptr())

    plan = F.Plan(ns, 3, 3, "two_thirds", 32, False, ks)
    plan.set_stream(stream.cuda_stream)
    bus = None
    try:
        pr = torch.cuda.get_device_properties(dev)
        bus = "%08X:%02X:%02X.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
    except Exception:
        pass
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for _ in range(max(3, args.warmup)):
            run(plan, u, T)
        torch.cuda.synchronize()
        clk = Clocks(bus)
        clk.start()
        l0 = F.launch_count()
        e0.record(stream)
        for _ in range(args.steps):
            run(plan, u, T)
        e1.record(stream)
        torch.cuda.synchronize()
        launches = (F.launch_count() - l0) / args.steps
        clocks = clk.stop()
    ms = e0.elapsed_time(e1) / args.steps
    T32 = T.cpu().numpy().T.copy()   # T(n, m) column-major on the device
    asym32 = float(asym.item())
    def eager():
        with torch.cuda.stream(stream):
            run(plan, u, T)

    roofline = prof_roofline(F, eager, torch.cuda.synchronize)
    del plan
    F.clear_plans()
    torch.cuda.empty_cache()
    ms_plain32 = ms64 = None
    T64n = T32
    if not args.no_fp64:
        # the plain per-band path in FP32 (live box switched off for this plan)
        os.environ["FIT_NO_FUSED"] = "1"
        try:
            pp = F.Plan(ns, 3, 3, "two_thirds", 32, False, ks)
            pp.set_stream(stream.cuda_stream)
            Tp = torch.zeros((nb, nb), dtype=torch.float64, device=dev)
            ms_plain32 = _timed_ms(lambda: run(pp, u, Tp), stream, 1, warm=1)
            del pp
        finally:
            del os.environ["FIT_NO_FUSED"]
        F.clear_plans()
        torch.cuda.empty_cache()
        u64 = u.to(torch.complex128)
        p64 = F.Plan(ns, 3, 3, "two_thirds", 64, True, ks)
        p64.set_stream(stream.cuda_stream)
        T64 = torch.zeros((nb, nb), dtype=torch.float64, device=dev)
        ms64 = _timed_ms(lambda: run(p64, u64, T64), stream, 1, warm=1)
        T64n = T64.cpu().numpy().T.copy()
        del p64, u64
        F.clear_plans()
    scale = float(np.max(np.abs(T64n)))
    line = {"metric": f"{N}^3 smooth band-to-band T(K,Q), {nb} bands: matrices/s", "value": 1000.0 / ms,
            "unit": "matrices/s", "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"{N}^3 D=3 SmoothBands(2^1..2^7, logwidth {lw}), KineticEnergy, OrszagTwoThirds, "
                                   "complex64 field, FP64 sums",
                       "spectrum": "k^-5/3 on [4,170], k^4 rise below 4, solenoidal", "seed": args.seed,
                       "l2": "field 3.2 GB per step >> 129 MB L2"},
            "roofline": roofline, "ms_plain_fp32": ms_plain32,
            "speedup_vs_plain_fp32": None if ms_plain32 is None else ms_plain32 / ms,
            "ms_plain_fp64": ms64, "speedup_vs_plain_fp64": None if ms64 is None else ms64 / ms,
            "rel_err_vs_fp64_maxnorm": None if ms64 is None else float(np.max(np.abs(T32 - T64n)) / scale),
            "antisymmetry_fp32_rel": asym32 / scale,
            "conservation_fp32": float(abs(T32.sum()) / np.abs(T32).sum()),
            "gpu_launches": int(launches), "clocks": clocks}
    print(json.dumps(line), flush=True)
    return 0


def run_frontend(args):
    """Physical-space front end at 512^3: u_hat = fft(u)/Np of three real FP32 fields on the device
    (the full N-grid spectrum in the user layout), against cuFFT (torch.fft.fftn) on the same fields."""
    import torch
    import __graft_entry__
    F = __graft_entry__.load_package()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    N = args.n
    ns = (N, N, N)
    ks = F.wavenumber_grid(ns, (2 * np.pi,) * 3)
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed)
    u = torch.randn((3, N, N, N), device=dev, dtype=torch.float32, generator=g)   # x fastest, component last
    out = torch.empty((3, N, N, N), device=dev, dtype=torch.complex64)
    stream = torch.cuda.Stream(device=dev)
    plan = F.Plan(ns, 3, 3, "two_thirds", 32, False, ks)
    plan.set_stream(stream.cuda_stream)

    def step():
        plan.forward_spectrum_device(u.data_ptr(), out.data_ptr())

    l0 = F.launch_count()
    ms = _timed_ms(step, stream, args.steps, warm=max(3, args.warmup))
    launches = (F.launch_count() - l0) / (args.steps + max(3, args.warmup))
    inv = 1.0 / float(N) ** 3
    with torch.cuda.stream(stream):
        ref = torch.fft.fftn(u, dim=(1, 2, 3)) * inv
    torch.cuda.synchronize()
    err = float((out - ref).abs().max().item() / ref.abs().max().item())
    del ref
    torch.cuda.empty_cache()
    res = torch.empty_like(out)

    def cufft_step():
        torch.mul(torch.fft.fftn(u, dim=(1, 2, 3)), inv, out=res)

    ms_cufft = _timed_ms(cufft_step, stream, args.steps, warm=max(3, args.warmup))

    def eager():
        with torch.cuda.stream(stream):
            step()

    passes = prof_roofline(F, eager, torch.cuda.synchronize)
    alg = 3.0 * N ** 3 * (4 + 8)
    peak, peak_kind = read_peaks()
    line = {"metric": f"{N}^3 physical-space front end u_hat = fft(u)/Np, 3 real FP32 fields: fields/s",
            "value": 1000.0 / ms, "unit": "fields/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{N}^3 x 3 real FP32 fields (Gaussian noise) -> full complex64 spectrum",
                       "seed": args.seed, "l2": "inputs 1.6 GB per step >> 129 MB L2"},
            "roofline": {"bound": "hbm", "kernel": "whole call", "achieved": alg / (ms / 1e3) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": alg / (ms / 1e3) / 1e9 / peak, "peak_source": peak_kind,
                         "algorithmic_bytes": alg, "traffic": None},
            "passes": None if passes is None else passes["all_kernels"],
            "cufft_fftn_ms": ms_cufft, "speedup_vs_cufft": ms_cufft / ms,
            "rel_err_vs_cufft_maxnorm": err, "gpu_launches": int(launches)}
    print(json.dumps(line), flush=True)
    return 0


def run_pass(args):
    """One kernel of the fused shell-to-shell pipeline alone on a slice of the 512^3 workload, on
    synthetic device data: the x pass (``--config xpass``, one mediator of full x extent over
    ``--lines`` x lines, about 2.3 GB at the default 65536; both forms of the kernel), the
    y-inverse pass (``--config ypass``, one mediator over ``--planes`` z planes, 4.6 GB) or the
    z-forward + binning pass (``--config zbin``, ``--mediators`` mediators over all pencils, 1.2 GB
    + 0.7 GB per mediator). These are the small cases the kernel-level profiles are taken on; the
    per-unit bytes scale to full launches."""
    import ctypes as C
    import torch
    import __graft_entry__
    F = __graft_entry__.load_package()
    lib = F._lib.load()
    torch.cuda.set_device(0)
    xpass = args.config == "xpass"
    pass_ = {"xpass": 0, "ypass": 1, "zbin": 2}[args.config]
    units = {"xpass": args.lines, "ypass": args.planes, "zbin": args.mediators}[args.config]
    forms = (("column_groups", None), ("block_register", "1")) if xpass else (("default", None),)
    out = {}
    for form, env in forms:
        if env:
            os.environ["FIT_XMIX_REG"] = env
        else:
            os.environ.pop("FIT_XMIX_REG", None)
        ms, by = C.c_double(), C.c_double()
        F._lib.check(lib.fit_bench_fused_pass(pass_, args.n, units, max(1, args.steps), C.byref(ms), C.byref(by)))
        out[form] = {"ms": ms.value, "GBps": by.value / (ms.value / 1e3) / 1e9, "alg_bytes": by.value}
    os.environ.pop("FIT_XMIX_REG", None)
    peak, kind = read_peaks()
    head = out[forms[0][0]]
    what = {0: "x pass", 1: "y-inverse pass", 2: "z-forward + binning pass"}[pass_]
    kern = {0: "s2s_xmix", 1: "s2s_yinv", 2: "s2s_zfwd_bin"}[pass_]
    slice_ = {0: f"one mediator, {units} x lines", 1: f"one mediator, {units} z planes",
              2: f"{units} mediators, all pencils"}[pass_]
    line = {"metric": f"{args.n}-point {what} of the fused shell-to-shell pipeline: algorithmic GB/s",
            "value": head["GBps"], "unit": "GB/s", "n_gpus": 1, "steps": max(1, args.steps), "warmup": 1,
            "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"{slice_} of a {args.n}^3 grid, 2/3 rule, full extent",
                       "l2": "inputs %.1f GB per launch > 129 MB L2" % (head["alg_bytes"] / 1e9)},
            "roofline": {"bound": "hbm", "kernel": kern, "achieved": head["GBps"],
                         "peak": peak, "unit": "GB/s", "frac": head["GBps"] / peak, "peak_source": kind,
                         "algorithmic_bytes_per_launch": head["alg_bytes"], "traffic": None},
            "forms": out}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "closure":
        return run_closure(args)
    if args.config == "batch":
        return run_batch(args)
    if args.config == "partial":
        return run_partial(args)
    if args.config == "padded":
        return run_padded(args)
    if args.config == "m2m":
        return run_m2m(args)
    if args.config == "band":
        return run_band(args)
    if args.config == "frontend":
        return run_frontend(args)
    if args.config in ("xpass", "ypass", "zbin"):
        return run_pass(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
