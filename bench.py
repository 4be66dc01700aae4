#!/usr/bin/env python
"""Benchmark: AFQMC sweeps/s of ALF's finite-temperature sweep on a GB300.

Workload (default): Hubbard model on a 16x16 square lattice, N_dim = 256,
t = 1, U = 4, mu = 0, beta = 10, dtau = 0.1 (Ltrot = 100), Nwrap = 10, Mz
decoupling with four-valued fields, one Markov chain.  A step is one full
sequential sweep (up pass, down pass, 2*Nstm stabilisations).

value: sweeps/s with all state resident on the device, timed with CUDA events
       on the library's stream (device draw stream, no host traffic).
mixed: (FP64 runs, one GPU) the same measurements for the mixed form on the same
       workload, and max |G_mixed - G_fp64| after one sweep on identical fields and draws.
e2e:   the same metric through the C ABI with host buffers: each step copies
       the host draws in (6*M*Ltrot doubles) and reads G back (N^2*N_FL complex),
       both inside the timed region.
--impl reference: ALF's algorithm on the host cores (the CPU restatement that
       calls the same LAPACK; the Fortran reference cannot be built here), one
       chain, all host threads given to its BLAS, each step a bounded sample of
       a sweep (a fixed number of time slices with their stabilisations) scaled
       to sweeps/s.
Multi-GPU (torchrun): every rank runs an independent chain (replicas); value is
the total sweeps of all ranks / the max over ranks of the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "AFQMC sweeps/s (per chain & aggregate), mixed vs FP64 GPU at max|dG|<=1e-5"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
# FP64 peak of a GB300: a register-only loop of independent mma.sync m8n8k4 f64 accumulators
# (608 CTAs x 256 threads) measured 1.048 TFLOP/s; DFMA gives 1.006.
FP64_DMMA_TFLOPS = 1.048
# DRAM bytes (read + write) of one G-wrap GEMM launch (N_dim = 256, two flavours), from
# an ncu capture of the 16x16 workload (dram__bytes_read.sum + dram__bytes_write.sum)
HOP_TRAFFIC_BYTES = 3.30e6


def measured_bf16_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["bf16_tflops"]), "MEASURED_PEAKS.json bf16_tflops (burst, cuBLAS)"
    except Exception:
        return 1900.0, "fallback 1.9 PFLOP/s bf16 burst"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="hubbard16x16",
                    choices=["hubbard4x4", "hubbard16x16", "honeycomb12x12", "kondo12x12", "batch128"],
                    help="hubbard16x16: one 16x16 chain; honeycomb12x12: 12x12 honeycomb, beta 20, TAU_M every "
                         "sweep; kondo12x12: Kondo bilayer (ham_Uf = 0), TAU_M every sweep; batch128: 128 Hubbard "
                         "chains with per-chain L, beta, U, one handle per (N_dim, Ltrot) group")
    ap.add_argument("--ltau", type=int, default=-1, help="TAU_M every sweep (default: the config's)")
    ap.add_argument("--drift-bound", type=float, default=1e-5,
                    help="batch128: Nwrap of a group is halved until its Precision Green is below this")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--flags", type=int, default=0, help="dims.reserved[0] flag bits (include/alfgpu.h)")
    ap.add_argument("--pivoting", default="default", choices=["default", "exact", "norms", "norms-cgr", "norms-decompose"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--chains", type=int, default=1, help="independent chains per GPU (batched)")
    ap.add_argument("--no-tune", dest="tune", action="store_false", help="keep the default delay depth")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", dest="compare", action="store_false",
                    help="FP64 runs: skip the mixed-form measurement reported beside the headline")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                parts = [x.strip() for x in out.stdout.strip().split(",")]
                if len(parts) >= 8:
                    self.samples.append(parts)
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._th:
            self._th.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def algorithmic_flops(m, phase: str, launches: int, n_acc: int) -> float:
    """Algorithmic FLOPs of one phase over `launches` launch groups (real-flop convention:
    complex MAC = 8, real x complex MAC = 4; LAPACK counts for QR)."""
    N, F = m.ndim, m.n_fl
    if phase == "hop":        # 2 real x complex N^3 products per flavour per group
        return launches * 2 * F * 4.0 * N ** 3
    if phase == "propagate":  # per group: Nwrap (or fewer) slices of one real x complex product per flavour
        return None
    if phase in ("qr", "orgqr"):
        return launches * F * (16.0 / 3.0) * N ** 3
    if phase == "solve":
        return launches * F * 4.0 * N ** 3
    if phase == "flush":
        return 8.0 * N * N * n_acc * 1.0  # rank-1 equivalents, both flavours counted in n_acc per flavour
    return None


def roofline(args, m, prof):
    """Roofline object of the G-wrap GEMM, the largest consumer of the complex products with a
    clean algorithmic count (2 real x complex N^3 products per flavour per slice, 2 L slices
    per sweep).  FP64 form: k_zgemm against the measured FP64 MMA rate.  Mixed form:
    k_oz_slice + k_oz_gemm (digit-sliced BF16 on tcgen05) against the measured BF16 peak; the
    algorithmic count is the same as FP64's, the BF16 products actually executed are
    reported beside it (tensor_op_tflops)."""
    hop_ms, hop_n = prof.get("hop", (0.0, 0))
    flops = algorithmic_flops(m, "hop", hop_n, 0) * args.chains
    if args.precision == "fp64":
        roof = {"bound": "tensor", "kernel": "k_zgemm (G wraps, FP64 mma.sync)", "achieved": None,
                "peak": FP64_DMMA_TFLOPS, "unit": "TFLOP/s", "frac": None,
                "traffic": HOP_TRAFFIC_BYTES if m.ndim == 256 else None,
                "algorithmic_flops_per_launch": args.chains * m.n_fl * 4.0 * m.ndim ** 3,
                "peak_source": "FP64 mma.sync m8n8k4 throughput measured on a GB300 with a register-only "
                               "loop; MEASURED_PEAKS.json has no FP64 figure"}
    else:
        peak, src = measured_bf16_peak()
        N, F = m.ndim, m.n_fl
        kpad = (N + 63) // 64 * 64
        bits, S = next((b, (54 + b - 1) // b) for b in range(7, 3, -1)
                       if ((54 + b - 1) // b) * kpad * ((1 << b) - 1) ** 2 < 2 ** 24)
        pairs = S * (S + 1) // 2 + (S - 1)  # digit pairs of the S + 1 accumulated diagonals
        roof = {"bound": "tensor", "kernel": "k_oz_slice + k_oz_gemm (G wraps, digit-sliced BF16 on tcgen05)",
                "achieved": None, "peak": peak, "unit": "TFLOP/s", "frac": None, "traffic": None,
                "algorithmic_flops_per_launch": args.chains * F * 4.0 * N ** 3,
                "bf16_products_per_algorithmic_product": pairs,
                "peak_source": src + "; of measured"}
    if flops and hop_ms > 0:
        roof["achieved"] = flops / (hop_ms / 1e3) / 1e12
        roof["frac"] = roof["achieved"] / roof["peak"]
        if args.precision != "fp64":
            roof["tensor_op_tflops"] = roof["achieved"] * roof["bf16_products_per_algorithmic_product"]
    return roof


def sweep_flops(m, n_acc: float, ltau: int) -> dict:
    """Algorithmic FLOPs of one sweep of one chain by phase (real-flop convention, LAPACK
    counts): per flavour G wraps 16 L N^3, UDV propagation 8 L N^3, decompose_UDV_state
    2 Nstm x 14.7 N^3, CGR 2 Nstm x 44 N^3, rank-1 updates 8 N^2 per accepted flip; with
    TAU_M also its wraps 16 L N^3, WRAPUR 4 L N^3 and Nstm CGR2_2 on 2N (~161.7 N^3)."""
    N, F, L = m.ndim, m.n_fl, m.ltrot
    nstm = -(-L // m.nwrap)
    n3 = float(N) ** 3
    out = {"wraps": F * 16.0 * L * n3, "propagate": F * 8.0 * L * n3,
           "decompose": F * 2.0 * nstm * 14.7 * n3, "cgr": F * 2.0 * nstm * 44.0 * n3,
           "rank1": F * 8.0 * N * N * float(n_acc)}
    if ltau:
        out["tau_wraps"] = F * 20.0 * L * n3
        out["tau_cgr2_2"] = F * nstm * (14.7 + 147.0) * n3
    return out


# phases whose products the mixed form runs on the tensor cores; the rest stay FP64
_TENSOR_PHASES = ("wraps", "propagate", "rank1", "tau_wraps")


def _reported(fn, *args):
    """An optional object of the JSON line: its failure is reported in the line, never fatal."""
    try:
        return fn(*args)
    except Exception as e:  # the line must still print
        return {"failed": f"{type(e).__name__}: {e}"}


def sweep_roofline(m, n_acc: float, ltau: int, chains: int, ms_per_step: float, precision: str,
                   p_fp64: float, p_bf16: float) -> dict:
    """Whole-sweep roofline: t_roof = sum over phases of FLOPs / peak for one step (one sweep of
    every chain).  FP64 form: every phase at the FP64 rate.  Mixed form: the wraps,
    propagation and rank-k flushes at the BF16 tensor peak, the QR / CGR phases at the FP64
    rate.  frac = t_roof / measured step time."""
    return sweep_roofline_groups([(m, n_acc, ltau, chains)], ms_per_step, precision, p_fp64, p_bf16)


def sweep_roofline_groups(groups, ms_per_step: float, precision: str, p_fp64: float, p_bf16: float) -> dict:
    """The same over several handles run one after the other in a step: groups of
    (model, accepted flips per chain and sweep, ltau, chains)."""
    if isinstance(groups, Exception):
        raise groups
    fl = {}
    for m, n_acc, ltau, chains in groups:
        for k, v in sweep_flops(m, n_acc, ltau).items():
            fl[k] = fl.get(k, 0.0) + v * chains
    t = 0.0
    for k, v in fl.items():
        peak = p_bf16 if (precision != "fp64" and k in _TENSOR_PHASES) else p_fp64
        t += v / (peak * 1e12)
    total = sum(fl.values())
    return {"flops_per_step": total, "flops_by_phase": fl, "t_roof_ms": 1e3 * t, "ms_per_step": ms_per_step,
            "frac": 1e3 * t / ms_per_step if ms_per_step > 0 else None,
            "achieved_tflops": total / (ms_per_step / 1e3) / 1e12 if ms_per_step > 0 else None,
            "peaks_tflops": {"fp64": p_fp64, "bf16": p_bf16},
            "basis": "FP64 phases at the measured FP64 MMA rate" + (
                "" if precision == "fp64" else "; wraps, propagation and flushes at the measured BF16 peak")}


def workload_model(name: str):
    """(model, ltau) of a named workload.  Kondo: the library runs the J_K vertices in their
    shared eigenbasis and rejects U_f vertices, so ham_Uf = 0."""
    from alf_gb300 import model as mdl
    if name == "kondo12x12":
        return mdl.kondo(12, 12, JK=1.5, Uf=0.0, beta=10.0, dtau=0.1, nwrap=10), 1
    if name == "honeycomb12x12":
        return mdl.config(name), 1
    if name == "batch128":
        return mdl.config("hubbard16x16"), 0
    return mdl.config(name), 0


def batch128_groups(seed: int, n: int = 128):
    """The 128-chain batch grouped by (N_dim, Ltrot) (alf_gb300.model.batch_groups)."""
    from alf_gb300 import model as mdl
    return mdl.batch_groups(seed, n)


def run_batch(args, ws, rank, local):
    """Config batch128: one handle per (N_dim, Ltrot) group with per-chain U; a step is one
    sweep of every chain (groups one after the other on the GPU)."""
    import torch
    from alf_gb300 import model as mdl, rng, replicas
    from alf_gb300.sweep import Chains
    torch.cuda.set_device(local)
    groups = batch128_groups(replicas.replica_seed(args.seed, rank))
    hs = []
    for (L, beta), members in sorted(groups.items()):
        models = [mdl.hubbard("square", L, L, U=U, beta=beta, dtau=0.1, nwrap=10) for _, U in members]
        ch = Chains(models[0], n_chains=len(members), precision=args.precision, device=local,
                    pivoting=args.pivoting, flags=args.flags, models=models)
        for k, (c, _) in enumerate(members):
            s = replicas.replica_seed(args.seed, rank, c)
            ch.set_fields(k, rng.initial_fields(s, k, models[0].n_op, models[0].ltrot))
        ch.init_state()
        for k, (c, _) in enumerate(members):
            ch.set_rng(k, replicas.replica_seed(args.seed, rank, c), rng.sweep_counter_base(models[0].n_op, models[0].ltrot, 0))
        hs.append((ch, models[0], members))
    nchains = sum(len(x[2]) for x in hs)
    streams = [torch.cuda.ExternalStream(ch.L.alfgpu_stream(ch.h), device=local) for ch, _, _ in hs]
    for _ in range(args.warmup):
        for ch, m, mem in hs:
            try:
                ch.sweep(None)
            except Exception as e:
                raise RuntimeError(f"group L={m.params.get('L1')} Ltrot={m.ltrot} chains={len(mem)}: {e}") from e
    # drift control: per group, halve Nwrap until Precision Green <= the bound (untimed sweeps)
    nwraps = []
    for ch, m, mem in hs:
        nw, worst = ch.adapt_nwrap(bound=args.drift_bound)
        nwraps.append((nw, worst))
    for ch, _, _ in hs:
        ch.reset_stats()
    torch.cuda.synchronize()
    n0 = sum(ch.L.alfgpu_launch_count(ch.h) for ch, _, _ in hs)
    ms = 0.0
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            for (ch, _, _), st in zip(hs, streams):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                ch.sweep(None)
                e1.record(st)
                e1.synchronize()
                ms += e0.elapsed_time(e1)
    n_launch = sum(ch.L.alfgpu_launch_count(ch.h) for ch, _, _ in hs) - n0
    # per group for the whole-sweep roofline: the adapted Nwrap, accepted flips per chain and sweep
    import dataclasses
    try:
        rgroups = [(dataclasses.replace(m, nwrap=ch.nwrap()),
                    sum(ch.stats(k).n_acc for k in range(len(mem))) / float(args.steps * len(mem)), 0, len(mem))
                   for ch, m, mem in hs]
    except Exception as e:  # only the roofline object depends on it
        rgroups = e
    h2d = d2h = 0
    t0 = time.perf_counter()
    for i in range(args.steps):
        for ch, m, members in hs:
            u = np.stack([rng.sweep_uniforms(replicas.replica_seed(args.seed, rank, c), k, m.n_op, m.ltrot, 1000 + i)
                          for k, (c, _) in enumerate(members)])
            ch.sweep(u)
            g = ch.green(0)
            if i == 0:
                h2d += u.nbytes
                d2h += g.nbytes
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    xmax = max(ch.stats(k).xmaxG for ch, _, mem in hs for k in range(len(mem)))
    out = dict(t_dev=ms / 1e3, t_e2e=e2e_s, clocks=clk.summary(), launches=n_launch, h2d=h2d, d2h=d2h,
               nchains=nchains, groups=[{"L": m.params.get("L1"), "Ltrot": m.ltrot, "chains": len(mem),
                                        "nwrap": nw, "xmaxG_at_adapt": worst}
                                       for (_, m, mem), (nw, worst) in zip(hs, nwraps)], xmaxG=xmax,
               rgroups=rgroups)
    for ch, _, _ in hs:
        ch.close()
    return out


def run_ours(args, ws, rank, local):
    import torch
    from alf_gb300 import model as mdl, rng
    from alf_gb300 import replicas
    from alf_gb300.sweep import Chains

    torch.cuda.set_device(local)
    m, ltau = workload_model(args.config)
    if args.ltau >= 0:
        ltau = args.ltau
    C = args.chains
    seed = replicas.replica_seed(args.seed, rank)
    ch = Chains(m, n_chains=C, precision=args.precision, device=local, pivoting=args.pivoting, flags=args.flags,
                ltau=ltau)
    for c in range(C):
        ch.set_fields(c, rng.initial_fields(replicas.replica_seed(args.seed, rank, c), c, m.n_op, m.ltrot))
    ch.init_state()
    for c in range(C):
        ch.set_rng(c, replicas.replica_seed(args.seed, rank, c), rng.sweep_counter_base(m.n_op, m.ltrot, 0))
    delay = ch.tune_delay(1) if args.tune else ch.delay()  # untimed (thermalisation) sweeps
    stream = torch.cuda.ExternalStream(ch.L.alfgpu_stream(ch.h), device=local)
    l2 = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")  # > 129 MB L2

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        ch.sweep(None)
    ch.reset_stats()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    n0 = ch.L.alfgpu_launch_count(ch.h)
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            l2.add_(1.0)  # flush L2 between timed steps (outside the timed region)
            torch.cuda.synchronize()
            ev[i][0].record(stream)
            ch.sweep(None)
            ev[i][1].record(stream)
        barrier()
    n_launch = ch.L.alfgpu_launch_count(ch.h) - n0
    ms = sum(a.elapsed_time(b) for a, b in ev)
    st = ch.stats(0)
    n_acc = st.n_acc
    # e2e through the C ABI with host buffers
    u_host = [np.stack([rng.sweep_uniforms(replicas.replica_seed(args.seed, rank, c), c, m.n_op, m.ltrot, 1000 + i)
                        for c in range(C)]) for i in range(args.steps)]
    G_host = np.zeros((m.n_fl, m.ndim, m.ndim), np.complex128)
    h2d = u_host[0].nbytes
    d2h = G_host.nbytes
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        ch.sweep(u_host[i])
        G_host = ch.green(0)
    barrier()
    e2e_s = time.perf_counter() - t0
    # phase profile of two sweeps (separate pass; events on the library stream)
    ch.set_profiling(True)
    for _ in range(2):
        ch.sweep(None)
    prof = ch.profile()
    ch.set_profiling(False)
    # launch count per sweep from the profile pass
    t_dev, t_e2e = replicas.max_over_ranks([ms / 1e3, e2e_s], device=f"cuda:{local}")
    return dict(m=m, t_dev=t_dev, t_e2e=t_e2e, clocks=clk.summary(), prof=prof, n_acc=n_acc, h2d=h2d, d2h=d2h,
                stats=st, chains=ch, launches=n_launch, delay=delay, ltau=ltau)


def mixed_vs_fp64(m, seed: int, local: int, flags: int):
    """max |G_mixed - G_fp64| over both flavours after one sweep from the same fields and
    the same host draws (the accept sequences agree unless a draw falls within rounding of
    its Metropolis weight), and the mixed form's own Precision Green of that sweep."""
    from alf_gb300 import rng
    from alf_gb300.sweep import Chains
    f0 = rng.initial_fields(seed, 0, m.n_op, m.ltrot)
    u = rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 0)[None, :]
    gs = []
    for prec in ("fp64", "mixed"):
        ch = Chains(m, n_chains=1, precision=prec, device=local, flags=flags)
        ch.set_fields(0, f0)
        ch.init_state()
        ch.sweep(u)
        gs.append((ch.green(0), ch.fields(0), ch.stats(0).xmaxG))
        ch.close()
    same = bool(np.array_equal(gs[0][1], gs[1][1]))
    return {"max_abs_dG_vs_fp64": float(np.max(np.abs(gs[1][0] - gs[0][0]))), "same_fields": same,
            "xmaxG_mixed": gs[1][2], "xmaxG_fp64": gs[0][2], "sweeps": 1}


def cpu_oracle_rate(m, seed: int, threads: int, slices: int, ltau: int = 0):
    """Sweeps/s of the CPU restatement on a bounded sample (slices time slices incl. stabilisations)."""
    import oracle
    from alf_gb300 import rng
    o = oracle.Oracle(m, ltau=ltau, threads=threads)
    o.set_fields(rng.initial_fields(seed, 0, m.n_op, m.ltrot))
    o.init_state()
    u = rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 0)
    t0 = time.perf_counter()
    o.sweep_chunk(u, slices)
    dt = time.perf_counter() - t0
    return (slices / (2.0 * m.ltrot)) / dt, dt


def batch_cpu_baseline(seed: int, slices: int = 10):
    """One host core on the batch: per (L, beta) group a bounded oracle sample (``slices`` time
    slices of one chain, by default Nwrap of them with the one stabilisation they end in, so
    the sample holds the sweep's own mix; scaled to a sweep); a step costs the sum
    over all chains, so the aggregate rate is chains / sum of per-chain sweep times."""
    from alf_gb300 import model as mdl
    groups = batch128_groups(seed)
    t_step, t_sample, n = 0.0, 0.0, 0
    for (L, beta), members in sorted(groups.items()):
        m = mdl.hubbard("square", L, L, U=members[0][1], beta=beta, dtau=0.1, nwrap=10)
        rate, dt = cpu_oracle_rate(m, seed, 1, min(slices, 2 * m.ltrot), 0)
        t_step += len(members) / rate
        t_sample += dt
        n += len(members)
    return {"value": n / t_step, "unit": "sweeps/s", "cores": 1, "kind": "port",
            "sample": f"{slices} time slices (with their stabilisations) of one chain per (L, beta) group, "
                      f"scaled to a sweep and summed over the {n} chains ({t_sample:.1f} s); CPU restatement "
                      f"of ALF's sweep with single-threaded OpenBLAS"}


def main():
    args = parse()
    ws, rank, local = dist_env()
    if ws > 1:
        import torch
        torch.distributed.init_process_group("nccl" if args.impl == "ours" else "gloo")
    m, ltau0 = workload_model(args.config)
    ltau = ltau0 if args.ltau < 0 else args.ltau
    if args.config == "batch128":
        desc = ("batch128: 128 Hubbard chains on square L x L lattices, per chain from its own seed L in "
                "{6,...,16}, beta in {4,6,8,10}, dtau 0.1, U in [2,8], Nwrap 10 (halved per group until Precision "
                f"Green <= {args.drift_bound:g}), Mz fields; one handle per (N_dim, Ltrot) group")
    elif args.config == "kondo12x12":
        desc = (f"kondo12x12: Kondo bilayer square 12x12, N_dim={m.ndim}, J_K=1.5, ham_Uf=0, beta={m.beta}, "
                f"dtau={m.dtau}, Ltrot={m.ltrot}, Nwrap={m.nwrap}, N_SUN=2, N_FL=1, four-valued fields, "
                f"TAU_M every sweep: {bool(ltau)}, "
                + ("one chain per GPU" if args.chains == 1 else f"{args.chains} independent chains per GPU"))
    else:
        desc = (f"{args.config}: {m.params.get('lattice')} {m.params.get('L1')}x{m.params.get('L2')}, "
                f"N_dim={m.ndim}, U={m.params.get('U')}, beta={m.beta}, dtau={m.dtau}, Ltrot={m.ltrot}, "
                f"Nwrap={m.nwrap}, Mz four-valued fields, TAU_M every sweep: {bool(ltau)}, "
                + ("one chain per GPU" if args.chains == 1 else f"{args.chains} independent chains per GPU"))
    workload = {"workload": desc,
                "chains_per_gpu": args.chains, "precision": args.precision, "pivoting": args.pivoting, "flags": args.flags, "l2": "flushed between timed steps (256 MB write)",
                "draws": "device counter stream (value); host arrays through the C ABI (e2e)"}
    if args.impl == "reference":
        if rank != 0:
            return
        cores = os.cpu_count() or 1
        slices = 20 if m.ndim >= 200 else 2 * m.ltrot
        rates = []
        for i in range(args.warmup + args.steps):
            r, dt = cpu_oracle_rate(m, args.seed, cores, slices, ltau)
            if i >= args.warmup:
                rates.append(r)
        v = float(np.mean(rates))
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "sweeps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded fields and draws)",
                "config": dict(workload, chains_per_gpu=1, parallelism="host cores",
                               l2="not applicable (host run; the sample's working set is the chain's own state)",
                               draws="host arrays of the same counter stream"),
                "cpu_baseline": {"value": v, "unit": "sweeps/s", "cores": cores, "kind": "port",
                                 "sample": f"{slices} time slices of one sweep (with their stabilisations"
                          + ("; TAU_M, which runs after the down pass, is outside the sample" if ltau else "")
                          + ") per step, "
                                           f"CPU restatement of ALF's default-STAB sweep calling OpenBLAS LAPACK "
                                           f"with {cores} threads; the Fortran reference has no compiler here"},
                "e2e": {"value": v, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if args.config == "batch128":
        rb = run_batch(args, ws, rank, local)
        if rank != 0:
            return
        from alf_gb300 import replicas
        t_dev, t_e2e = rb["t_dev"], rb["t_e2e"]
        cpu = None
        if not args.no_cpu_baseline:
            try:
                cpu = batch_cpu_baseline(replicas.replica_seed(args.seed, rank))
            except Exception as e:  # the baseline is reported, never required
                cpu = {"value": None, "unit": "sweeps/s", "cores": 1, "kind": "port", "sample": f"failed: {e}"}
        value = ws * rb["nchains"] * args.steps / t_dev
        line = {"metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "c128" if args.precision == "fp64" else "c128 state, digit-sliced bf16 tensor products, df64 visits",
                "data": "synthetic (seeded fields and draws)",
                "config": dict(workload, chains_per_gpu=rb["nchains"], groups=rb["groups"],
                               parallelism=f"replicas x{ws}", delay_depth="default"),
                "e2e": {"value": ws * rb["nchains"] * args.steps / t_e2e, "unit": "sweeps/s",
                        "h2d_bytes_per_step": rb["h2d"], "d2h_bytes_per_step": rb["d2h"]},
                "roofline": None, "cpu_baseline": cpu, "clocks": rb["clocks"], "gpu_launches": int(rb["launches"]),
                "precision_green": {"xmaxG": rb["xmaxG"]},
                "sweep_roofline": _reported(sweep_roofline_groups, rb["rgroups"], 1e3 * t_dev / args.steps,
                                            args.precision, FP64_DMMA_TFLOPS, measured_bf16_peak()[0])}
        print(json.dumps(line))
        return

    r = run_ours(args, ws, rank, local)
    if rank != 0:
        return
    m = r["m"]
    from alf_gb300 import replicas
    value = replicas.whole_job_rate(ws, args.chains, args.steps, r["t_dev"])
    e2e = replicas.whole_job_rate(ws, args.chains, args.steps, r["t_e2e"])
    prof = r["prof"]
    # Roofline of the dominant kernel: the complex GEMM (k_zgemm on FP64 DMMA; k_dfgemm in
    # the mixed form) carries the largest share of the launch list, and its largest
    # consumer with a clean algorithmic count is the G wrap (2 real x complex N^3
    # products per flavour per slice, 2 L slices per sweep).
    roof = roofline(args, m, prof)
    phases = {k: {"ms_per_sweep": v[0] / 2.0, "launch_groups_per_sweep": v[1] / 2.0} for k, v in prof.items()}
    launches = int(r["launches"])
    cpu = None
    if not args.no_cpu_baseline:
        try:
            ns = 2 * m.ltrot if m.ndim <= 256 else 40  # one full sweep (~6 s for 16x16 on one core)
            rate, dt = cpu_oracle_rate(m, args.seed, 1, ns, r.get("ltau", 0))
            cpu = {"value": rate, "unit": "sweeps/s", "cores": 1, "kind": "port",
                   "sample": f"{ns} time slices with their stabilisations ({dt:.1f} s), CPU restatement of ALF's "
                             f"sweep with single-threaded OpenBLAS"}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "sweeps/s", "cores": 1, "kind": "port", "sample": f"failed: {e}"}
    st = r["stats"]
    mixed = None
    if args.precision == "fp64" and args.compare and ws == 1:
        import copy
        a2 = copy.copy(args)
        a2.precision = "mixed"
        r2 = run_ours(a2, ws, rank, local)
        st2 = r2["stats"]
        mixed = {"value": replicas.whole_job_rate(ws, args.chains, args.steps, r2["t_dev"]), "unit": "sweeps/s",
                 "e2e": replicas.whole_job_rate(ws, args.chains, args.steps, r2["t_e2e"]),
                 "ms_per_step": 1e3 * r2["t_dev"] / args.steps, "gpu_launches": int(r2["launches"]),
                 "delay_depth": r2["delay"], "clocks": r2["clocks"],
                 "phases": {k: {"ms_per_sweep": v[0] / 2.0} for k, v in r2["prof"].items()},
                 "precision_green": {"xmaxG": st2.xmaxG, "xmeanG": st2.xmeanG_sum / max(st2.ncg, 1),
                                     "xmaxP": st2.xmaxP},
                 "roofline": roofline(a2, m, r2["prof"]),
                 "sweep_roofline": _reported(sweep_roofline, m, st2.n_acc / max(args.steps, 1), r2.get("ltau", 0),
                                             args.chains, 1e3 * r2["t_dev"] / args.steps, "mixed",
                                             FP64_DMMA_TFLOPS, measured_bf16_peak()[0]),
                 "dtype": "c128 state; G wraps and UDV propagation (and the flushes of batched grids) as "
                          "FP64-accurate digit-sliced BF16 tensor-core products; per-visit arithmetic and "
                          "single-chain flushes in double-float; QR / CGR in FP64"}
        r2["chains"].close()
        try:
            mixed["vs_fp64"] = mixed_vs_fp64(m, args.seed, local, args.flags)
        except Exception as e:
            mixed["vs_fp64"] = {"failed": str(e)}
    line = {
        "metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * r["t_dev"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "c128" if args.precision == "fp64" else "c128 state, digit-sliced bf16 tensor products, df64 visits",
        "data": "synthetic (seeded fields and draws)",
        "config": dict(workload, parallelism=f"replicas x{ws}", delay_depth=r["delay"],
                       delay_depth_source="autotuned (alfgpu_tune_delay)" if args.tune else "default"),
        "e2e": {"value": e2e, "unit": "sweeps/s", "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"]},
        "roofline": roof, "cpu_baseline": cpu, "clocks": r["clocks"], "gpu_launches": launches,
        "phases": phases,
        "precision_green": {"xmaxG": st.xmaxG, "xmeanG": st.xmeanG_sum / max(st.ncg, 1), "xmaxP": st.xmaxP},
        "acceptance": st.n_acc / max(st.n_prop, 1),
        "sweep_roofline": _reported(sweep_roofline, m, st.n_acc / max(args.steps, 1), r.get("ltau", 0), args.chains,
                                    1e3 * r["t_dev"] / args.steps, args.precision, FP64_DMMA_TFLOPS,
                                    measured_bf16_peak()[0]),
    }
    if mixed is not None:
        line["mixed"] = mixed
    print(json.dumps(line))
    r["chains"].close()


if __name__ == "__main__":
    main()
