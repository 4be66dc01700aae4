#!/usr/bin/env python
"""Benchmark: AFQMC sweeps/s of ALF's finite-temperature sweep on a GB300.

Default workload: Hubbard model on a 16x16 square lattice, N_dim = 256, t = 1, U = 4,
mu = 0, beta = 10, dtau = 0.1 (Ltrot = 100), Nwrap = 10, Mz decoupling with four-valued
fields; independent Markov chains, aggregate sweeps/s.  A step is one full sequential
sweep (up pass, down pass, 2*Nstm stabilisations) of every chain.

value:     aggregate sweeps/s of the batched mixed form: C chains (16 by default) in one
           handle, all state resident on the device, timed with CUDA events on the
           library's stream (device draw stream, L2 flushed between steps).
fp64:      the same for the plain FP64 form on the same workload and chain count, and
           mixed_over_fp64 = value / fp64.value (the spec ratio).
per_chain: one chain per handle in both forms (the single-chain rate).
vs_fp64:   max |G_mixed - G_fp64| after one sweep on identical fields and draws.
e2e:       the headline through the C ABI with host buffers: each step copies every
           chain's host draws in (6*M*Ltrot doubles per chain) and reads G of chain 0 back,
           both inside the timed region.
--impl reference: ALF's own use of a host (Documentation/performance.tex:29-37): one
           single-threaded walker per host core, each an independent chain on its own
           seed, running the CPU restatement of ALF's sweep (the same LAPACK calls; the
           Fortran reference has no compiler here).  A step is one whole sweep of every
           walker; value = walkers x steps / time.  The rate of one chain with all host
           threads given to its BLAS is measured beside it.
--config batch128: 128 chains with per-chain L, beta, U in one handle per (N_dim, Ltrot)
           group; the groups sweep concurrently from one host thread each.
Multi-GPU (torchrun): every rank runs its own chains (replicas); value is the total
sweeps of all ranks / the max over ranks of the timed region.
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
# DRAM bytes (read + write) of one G-wrap GEMM launch (N_dim = 256, two flavours, one chain),
# from an ncu capture of the 16x16 workload (dram__bytes_read.sum + dram__bytes_write.sum)
HOP_TRAFFIC_BYTES = 3.28e6
# the same for the mixed form's G-wrap k_oz_gemm launch of the 16-chain handle (78.1 MB read,
# 8.3 MB written: the digit slices of G and the output), per chain
OZ_HOP_TRAFFIC_BYTES_PER_CHAIN = 86.5e6 / 16
# default chains per GPU of each workload (the batched forms of the benchmark configurations)
DEFAULT_CHAINS = {"hubbard4x4": 1, "hubbard16x16": 16, "honeycomb12x12": 8, "kondo12x12": 32, "batch128": 128}
L2_NOTE = "GPU arm: L2 flushed between timed steps (256 MB write); host arm: not applicable"


def measured_bf16_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["bf16_tflops"]), "MEASURED_PEAKS.json bf16_tflops (burst, cuBLAS)"
    except Exception:
        return 1900.0, "fallback 1.9 PFLOP/s bf16 burst"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="hubbard16x16",
                    choices=["hubbard4x4", "hubbard16x16", "honeycomb12x12", "kondo12x12", "batch128"],
                    help="hubbard16x16: 16x16 Hubbard chains; honeycomb12x12: 12x12 honeycomb, beta 20, TAU_M every "
                         "sweep; kondo12x12: Kondo bilayer (ham_Uf = 0), TAU_M every sweep; batch128: 128 Hubbard "
                         "chains with per-chain L, beta, U, one handle per (N_dim, Ltrot) group")
    ap.add_argument("--ltau", type=int, default=-1, help="TAU_M every sweep (default: the config's)")
    ap.add_argument("--drift-bound", type=float, default=1e-5,
                    help="batch128: Nwrap of a group is halved until its Precision Green is below this")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"], help="the headline form")
    ap.add_argument("--flags", type=int, default=0, help="dims.reserved[0] flag bits (include/alfgpu.h)")
    ap.add_argument("--pivoting", default="default", choices=["default", "exact", "norms", "norms-cgr", "norms-decompose"])
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--chains", type=int, default=-1, help="independent chains per GPU (default: the config's)")
    ap.add_argument("--no-tune", dest="tune", action="store_false", help="keep the default delay depth")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serial-groups", action="store_true", help="batch128: sweep the groups one after another")
    ap.add_argument("--no-compare", dest="compare", action="store_false",
                    help="skip the other form and the one-chain runs reported beside the headline")
    ap.add_argument("--walkers", type=int, default=-1, help="--impl reference: host walkers (default: all cores)")
    ap.add_argument("--wrap-bits", type=int, default=0,
                    help="mixed form: target bits of the G-wrap / TAU_M tensor-core products (0: full)")
    ap.add_argument("--propagate-bits", type=int, default=0,
                    help="mixed form: target bits of the UDV-propagation tensor-core products (0: full)")
    a = ap.parse_args(argv)
    if a.chains < 1:
        a.chains = DEFAULT_CHAINS[a.config]
    return a


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
    """Algorithmic FLOPs of one phase over `launches` launch groups of one chain (real-flop
    convention: complex MAC = 8, real x complex MAC = 4; LAPACK counts for QR)."""
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


def digit_pairs(n: int):
    """(bits, slices, digit-pair products per algorithmic product) of the digit-sliced
    tensor-core GEMM at inner dimension n, as the library picks them (ozaki.cuh oz_pick)."""
    kpad = (n + 63) // 64 * 64
    bits, S = next((b, (54 + b - 1) // b) for b in range(7, 3, -1)
                   if ((54 + b - 1) // b) * kpad * ((1 << b) - 1) ** 2 < 2 ** 24)
    return bits, S, S * (S + 1) // 2 + (S - 1)


def roofline(precision: str, chains: int, m, prof):
    """Roofline object of the G-wrap GEMM, the largest consumer of the complex products with a
    clean algorithmic count (2 real x complex N^3 products per flavour per slice, 2 L slices
    per sweep).  FP64 form: k_zgemm against the measured FP64 MMA rate.  Mixed form:
    k_oz_slice + k_oz_gemm (digit-sliced BF16 on tcgen05) against the measured BF16 peak; the
    algorithmic count is the same as FP64's, the BF16 products actually executed are
    reported beside it (tensor_op_tflops)."""
    hop_ms, hop_n = prof.get("hop", (0.0, 0))
    flops = algorithmic_flops(m, "hop", hop_n, 0) * chains
    if precision == "fp64":
        roof = {"bound": "tensor", "kernel": "k_zgemm (G wraps, FP64 mma.sync)", "achieved": None,
                "peak": FP64_DMMA_TFLOPS, "unit": "TFLOP/s", "frac": None,
                "traffic": HOP_TRAFFIC_BYTES * chains if m.ndim == 256 else None,
                "algorithmic_flops_per_launch": chains * m.n_fl * 4.0 * m.ndim ** 3,
                "peak_source": "FP64 mma.sync m8n8k4 throughput measured on a GB300 with a register-only "
                               "loop; MEASURED_PEAKS.json has no FP64 figure"}
    else:
        peak, src = measured_bf16_peak()
        _, _, pairs = digit_pairs(m.ndim)
        roof = {"bound": "tensor", "kernel": "k_oz_slice + k_oz_gemm (G wraps, digit-sliced BF16 on tcgen05)",
                "achieved": None, "peak": peak, "unit": "TFLOP/s", "frac": None,
                "traffic": OZ_HOP_TRAFFIC_BYTES_PER_CHAIN * chains if m.ndim == 256 else None,
                "algorithmic_flops_per_launch": chains * m.n_fl * 4.0 * m.ndim ** 3,
                "bf16_products_per_algorithmic_product": pairs,
                "peak_source": src + "; of measured"}
    if flops and hop_ms > 0:
        roof["achieved"] = flops / (hop_ms / 1e3) / 1e12
        roof["frac"] = roof["achieved"] / roof["peak"]
        if precision != "fp64":
            # the BF16 digit products the tensor cores execute, against the same BF16 peak, and the
            # FP64-accurate algorithmic rate against the FP64 rate it replaces
            roof["tensor_op_tflops"] = roof["achieved"] * roof["bf16_products_per_algorithmic_product"]
            roof["tensor_op_frac"] = roof["tensor_op_tflops"] / roof["peak"]
            roof["achieved_over_fp64_peak"] = roof["achieved"] / FP64_DMMA_TFLOPS
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
    """The same over several handles swept in one step: groups of (model, accepted flips per
    chain and sweep, ltau, chains)."""
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
    """(model, ltau) of a named workload.  Kondo: the configuration leaves ham_Uf open; the bench
    runs the J_K vertices alone (ham_Uf = 0).  The library also runs the reference default
    ham_Uf = 2 (U_f as vector vertices in the J_K eigenbasis, parity-tested)."""
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


def bench_config(args, m, ltau) -> dict:
    """The `config` object of both arms' lines (identical by construction: the workload and
    how the aggregate is formed; how each arm runs it is in its `arm` object)."""
    if args.config == "batch128":
        desc = ("batch128: 128 Hubbard chains on square L x L lattices, per chain from its own seed L in "
                "{6,...,16}, beta in {4,6,8,10}, dtau 0.1, U in [2,8], Nwrap 10 (halved per group until Precision "
                f"Green <= {args.drift_bound:g}), Mz four-valued fields")
    elif args.config == "kondo12x12":
        desc = (f"kondo12x12: Kondo bilayer square 12x12, N_dim={m.ndim}, J_K=1.5, ham_Uf=0, beta={m.beta}, "
                f"dtau={m.dtau}, Ltrot={m.ltrot}, Nwrap={m.nwrap}, N_SUN=2, N_FL=1, four-valued fields, "
                f"TAU_M every sweep: {bool(ltau)}")
    else:
        desc = (f"{args.config}: {m.params.get('lattice')} {m.params.get('L1')}x{m.params.get('L2')}, "
                f"N_dim={m.ndim}, U={m.params.get('U')}, beta={m.beta}, dtau={m.dtau}, Ltrot={m.ltrot}, "
                f"Nwrap={m.nwrap}, Mz four-valued fields, TAU_M every sweep: {bool(ltau)}")
    return {"workload": desc, "aggregate": "independent Markov chains on their own seeds; sweeps/s summed over chains",
            "step": "one full sweep of every chain", "l2": L2_NOTE}


# ---------------------------------------------------------------------------------------------
# the host arm: ALF's one walker per core
# ---------------------------------------------------------------------------------------------
def _host_walker(conn, config: str, seed: int, chain: int):
    """One host walker: a single-threaded chain of the CPU restatement of ALF's sweep."""
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    try:
        import oracle
        from alf_gb300 import replicas, rng
        m, ltau = workload_model(config)
        s = replicas.replica_seed(seed, 0, chain)
        o = oracle.Oracle(m, ltau=ltau, threads=1)
        o.set_fields(rng.initial_fields(s, chain, m.n_op, m.ltrot))
        o.init_state()
        conn.send("ready")
        k = 0
        while conn.recv() == "sweep":
            o.sweep(rng.sweep_uniforms(s, chain, m.n_op, m.ltrot, k))
            k += 1
            conn.send(k)
    except Exception as e:  # reported by the parent
        conn.send(f"error: {type(e).__name__}: {e}")
    finally:
        conn.close()


def host_walkers_rate(config: str, seed: int, walkers: int, steps: int, warmup: int) -> dict:
    """Aggregate sweeps/s of `walkers` independent single-threaded host walkers (spawned
    processes, each on its own chain): every step sends one whole sweep to every walker and
    waits for all; value = walkers x steps / time of the timed steps."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    pipes, procs = [], []
    try:
        for c in range(walkers):
            a, b = ctx.Pipe()
            p = ctx.Process(target=_host_walker, args=(b, config, seed, c), daemon=True)
            p.start()
            pipes.append(a)
            procs.append(p)
        for a in pipes:
            r = a.recv()
            if r != "ready":
                raise RuntimeError(r)
        times = []
        for i in range(warmup + steps):
            t0 = time.perf_counter()
            for a in pipes:
                a.send("sweep")
            for a in pipes:
                r = a.recv()
                if isinstance(r, str):
                    raise RuntimeError(r)
            if i >= warmup:
                times.append(time.perf_counter() - t0)
        t = float(sum(times))
        return {"value": walkers * steps / t, "walkers": walkers, "steps": steps, "seconds": t,
                "s_per_step": times}
    finally:
        for a in pipes:
            try:
                a.send("stop")
            except Exception:
                pass
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.kill()


def one_chain_all_threads_rate(m, ltau: int, seed: int, threads: int, sweeps: int = 1) -> dict:
    """Sweeps/s of one chain of the CPU restatement with `threads` BLAS threads, whole sweeps
    after one untimed sweep."""
    import oracle
    from alf_gb300 import replicas, rng
    s = replicas.replica_seed(seed, 0, 0)
    o = oracle.Oracle(m, ltau=ltau, threads=threads)
    o.set_fields(rng.initial_fields(s, 0, m.n_op, m.ltrot))
    o.init_state()
    o.sweep(rng.sweep_uniforms(s, 0, m.n_op, m.ltrot, 0))
    t0 = time.perf_counter()
    for k in range(sweeps):
        o.sweep(rng.sweep_uniforms(s, 0, m.n_op, m.ltrot, 1 + k))
    dt = time.perf_counter() - t0
    return {"value": sweeps / dt, "threads": threads, "sweeps": sweeps, "seconds": dt}


def host_baseline(args, m, ltau, steps: int, warmup: int) -> dict:
    """cpu_baseline object: the host walkers' aggregate (ALF's model) with the one-chain
    all-threads figure beside it."""
    cores = os.cpu_count() or 1
    walkers = args.walkers if args.walkers > 0 else cores
    agg = host_walkers_rate(args.config, args.seed, walkers, steps, warmup)
    one = one_chain_all_threads_rate(m, ltau, args.seed, cores)
    return {"value": agg["value"], "unit": "sweeps/s", "cores": walkers, "kind": "port",
            "sample": f"{walkers} single-threaded walkers (one per host core, own seeds), {steps} whole sweeps "
                      f"each after {warmup} untimed ({agg['seconds']:.1f} s timed); CPU restatement of ALF's "
                      "default-STAB sweep calling OpenBLAS LAPACK; the Fortran reference has no compiler here",
            "walkers": walkers, "s_per_step": agg["s_per_step"],
            "one_chain_all_threads": {"value": one["value"], "unit": "sweeps/s", "threads": one["threads"],
                                      "sample": f"{one['sweeps']} whole sweep(s) of one chain after one untimed"}}


# ---------------------------------------------------------------------------------------------
# the GPU arm
# ---------------------------------------------------------------------------------------------
def run_ours(args, ws, rank, local, precision: str, chains: int, steps: int, warmup: int, e2e: bool = True,
             measure: bool = False):
    """One handle of `chains` chains in `precision`: delay autotune (untimed), warm-up, the
    device-timed steps, optionally the e2e steps through host buffers, and a two-sweep phase
    profile.  Returns the measurements."""
    import torch
    from alf_gb300 import replicas, rng
    from alf_gb300.sweep import Chains

    torch.cuda.set_device(local)
    m, ltau = workload_model(args.config)
    if args.ltau >= 0:
        ltau = args.ltau
    C = chains
    seeds = [replicas.replica_seed(args.seed, rank, c) for c in range(C)]
    ch = Chains(m, n_chains=C, precision=precision, device=local, pivoting=args.pivoting, flags=args.flags,
                ltau=ltau, wrap_bits=args.wrap_bits, propagate_bits=args.propagate_bits)
    for c in range(C):
        ch.set_fields(c, rng.initial_fields(seeds[c], c, m.n_op, m.ltrot))
    ch.init_state()
    for c in range(C):
        ch.set_rng(c, seeds[c], rng.sweep_counter_base(m.n_op, m.ltrot, 0))
    delay = ch.tune_delay(1) if args.tune else ch.delay()  # untimed (thermalisation) sweeps
    stream = torch.cuda.ExternalStream(ch.L.alfgpu_stream(ch.h), device=local)
    l2 = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")  # > 129 MB L2

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(warmup):
        ch.sweep(None)
    ch.reset_stats()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    barrier()
    n0 = ch.L.alfgpu_launch_count(ch.h)
    with ClockSampler(local) as clk:
        for i in range(steps):
            l2.add_(1.0)  # flush L2 between timed steps (outside the timed region)
            torch.cuda.synchronize()
            ev[i][0].record(stream)
            ch.sweep(None)
            ev[i][1].record(stream)
        barrier()
    n_launch = ch.L.alfgpu_launch_count(ch.h) - n0
    ms = sum(a.elapsed_time(b) for a, b in ev)
    st = [ch.stats(c) for c in range(C)]
    n_acc = sum(s.n_acc for s in st) / float(C * steps)
    h2d = d2h = 0
    e2e_s = None
    if e2e:  # through the C ABI with host buffers
        u_host = [np.stack([rng.sweep_uniforms(seeds[c], c, m.n_op, m.ltrot, 1000 + i) for c in range(C)])
                  for i in range(steps)]
        G_host = np.zeros((m.n_fl, m.ndim, m.ndim), np.complex128)
        h2d = u_host[0].nbytes
        d2h = G_host.nbytes
        barrier()
        t0 = time.perf_counter()
        for i in range(steps):
            ch.sweep(u_host[i])
            G_host = ch.green(0)
        barrier()
        e2e_s = time.perf_counter() - t0
    # a measuring sweep: ham%Obser's scalar (Kin, Pot, Part, Ener) and lattice (Green, SpinZ, SpinXY,
    # SpinT, Den) observables accumulated on the device at every slice, no G copies (graph replay)
    meas = None
    if measure and args.config in ("hubbard16x16", "hubbard4x4"):
        from alf_gb300 import lattice_obs as lo, model as mdl
        L1 = int(m.params.get("L1", 16))
        ch.set_scalar_obs(np.stack([mdl.hopping_matrix("square", L1, L1, t=1.0).real] * m.n_fl),
                          np.full(m.ndim, float(m.params.get("U", 4.0))))
        ch.set_lattice_obs(lo.Lattice("square", L1, L1))
        ch.sweep(None)  # capture
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            ch.sweep(None)
        e1.record(stream)
        barrier()
        tm = e0.elapsed_time(e1) / 1e3
        cnt = ch.scalar_obs(0)["count"]
        meas = {"value": C * steps / tm, "unit": "sweeps/s", "measurements_per_chain": cnt,
                "observables": "Kin, Pot, Part, Ener; Green, SpinZ, SpinXY, SpinT, Den (equal time, every slice)"}
        ch.set_scalar_obs()
        ch.set_lattice_obs(None)
    # phase profile of two sweeps (separate pass; events on the library stream)
    ch.set_profiling(True)
    for _ in range(2):
        ch.sweep(None)
    prof = ch.profile()
    ch.set_profiling(False)
    t = replicas.max_over_ranks([ms / 1e3] + ([e2e_s] if e2e else []), device=f"cuda:{local}")
    out = dict(m=m, t_dev=t[0], t_e2e=t[1] if e2e else None, clocks=clk.summary(), prof=prof, n_acc=n_acc, meas=meas,
               h2d=h2d, d2h=d2h, launches=n_launch, delay=delay, ltau=ltau, steps=steps, chains=C,
               precision=precision, acceptance=sum(s.n_acc for s in st) / max(sum(s.n_prop for s in st), 1),
               precision_green={"xmaxG": max(s.xmaxG for s in st),
                                "xmeanG": sum(s.xmeanG_sum for s in st) / max(sum(s.ncg for s in st), 1),
                                "xmaxP": max(s.xmaxP for s in st)})
    if ltau:
        out["precision_green"]["xmax_tau"] = max(s.xmax_tau for s in st)
    ch.close()
    return out


def form_summary(ws, r) -> dict:
    """The measurements of one run_ours result as a JSON object."""
    from alf_gb300 import replicas
    m = r["m"]
    ms_step = 1e3 * r["t_dev"] / r["steps"]
    d = {"value": replicas.whole_job_rate(ws, r["chains"], r["steps"], r["t_dev"]), "unit": "sweeps/s",
         "chains_per_gpu": r["chains"], "steps": r["steps"], "ms_per_step": ms_step,
         "per_chain_sweeps_per_s": 1e3 / ms_step, "gpu_launches": int(r["launches"]), "delay_depth": r["delay"],
         "clocks": r["clocks"],
         "phases": {k: {"ms_per_sweep": v[0] / 2.0, "launch_groups_per_sweep": v[1] / 2.0}
                    for k, v in r["prof"].items()},
         "precision_green": r["precision_green"], "acceptance": r["acceptance"],
         "roofline": _reported(roofline, r["precision"], r["chains"], m, r["prof"]),
         "sweep_roofline": _reported(sweep_roofline, m, r["n_acc"], r["ltau"], r["chains"], ms_step, r["precision"],
                                     FP64_DMMA_TFLOPS, measured_bf16_peak()[0])}
    if r["t_e2e"]:
        d["e2e"] = replicas.whole_job_rate(ws, r["chains"], r["steps"], r["t_e2e"])
    return d


def mixed_vs_fp64(m, seed: int, local: int, flags: int, ltau: int, wrap_bits: int = 0, propagate_bits: int = 0):
    """max |G_mixed - G_fp64| over both flavours after one sweep from the same fields and
    the same host draws (the accept sequences agree unless a draw falls within rounding of
    its Metropolis weight), and the mixed form's own Precision Green of that sweep."""
    from alf_gb300 import rng
    from alf_gb300.sweep import Chains
    f0 = rng.initial_fields(seed, 0, m.n_op, m.ltrot)
    u = rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 0)[None, :]
    gs = []
    for prec in ("fp64", "mixed"):
        ch = Chains(m, n_chains=1, precision=prec, device=local, flags=flags, ltau=ltau, wrap_bits=wrap_bits,
                    propagate_bits=propagate_bits)
        ch.set_fields(0, f0)
        ch.init_state()
        ch.sweep(u)
        gs.append((ch.green(0), ch.fields(0), ch.stats(0).xmaxG))
        ch.close()
    same = bool(np.array_equal(gs[0][1], gs[1][1]))
    return {"max_abs_dG_vs_fp64": float(np.max(np.abs(gs[1][0] - gs[0][0]))), "same_fields": same,
            "xmaxG_mixed": gs[1][2], "xmaxG_fp64": gs[0][2], "sweeps": 1}


def run_batch(args, ws, rank, local, precision: str, steps: int, warmup: int, e2e: bool = True):
    """Config batch128: one handle per (N_dim, Ltrot) group with per-chain U; a step is one
    sweep of every chain.  By default the groups sweep concurrently through alfgpu_sweep_many
    (one host thread; each handle's launches on its own stream), and the step is timed on the
    device from an event that every group stream waits for to an event that waits for every
    group's end."""
    import concurrent.futures as cf
    import dataclasses
    import torch
    from alf_gb300 import model as mdl, rng, replicas
    from alf_gb300.sweep import Chains, sweep_many
    torch.cuda.set_device(local)
    groups = batch128_groups(replicas.replica_seed(args.seed, rank))
    hs = []
    for (L, beta), members in sorted(groups.items()):
        models = [mdl.hubbard("square", L, L, U=U, beta=beta, dtau=0.1, nwrap=10) for _, U in members]
        ch = Chains(models[0], n_chains=len(members), precision=precision, device=local,
                    pivoting=args.pivoting, flags=args.flags, models=models, wrap_bits=args.wrap_bits,
                    propagate_bits=args.propagate_bits)
        for k, (c, _) in enumerate(members):
            s = replicas.replica_seed(args.seed, rank, c)
            ch.set_fields(k, rng.initial_fields(s, k, models[0].n_op, models[0].ltrot))
        ch.init_state()
        for k, (c, _) in enumerate(members):
            ch.set_rng(k, replicas.replica_seed(args.seed, rank, c),
                       rng.sweep_counter_base(models[0].n_op, models[0].ltrot, 0))
        hs.append((ch, models[0], members))
    nchains = sum(len(x[2]) for x in hs)
    streams = [torch.cuda.ExternalStream(ch.L.alfgpu_stream(ch.h), device=local) for ch, _, _ in hs]
    pool = cf.ThreadPoolExecutor(max_workers=len(hs))

    def each(fn):
        if args.serial_groups:
            return [fn(i) for i in range(len(hs))]
        return list(pool.map(fn, range(len(hs))))

    def sweep_group(i):
        ch, m, mem = hs[i]
        try:
            ch.sweep(None)
        except Exception as e:
            raise RuntimeError(f"group L={m.params.get('L1')} Ltrot={m.ltrot} chains={len(mem)}: {e}") from e

    def sweep_all(us=None):
        """One sweep of every group: alfgpu_sweep_many (one host thread, each handle's launches on
        its own stream), or one group after another with --serial-groups."""
        if args.serial_groups:
            for i in range(len(hs)):
                if us is None:
                    sweep_group(i)
                else:
                    hs[i][0].sweep(us[i])
        else:
            sweep_many([h[0] for h in hs], us)

    for _ in range(warmup):
        sweep_all()
    # drift control: per group, halve Nwrap until Precision Green <= the bound (untimed sweeps)
    nwraps = each(lambda i: hs[i][0].adapt_nwrap(bound=args.drift_bound))
    for ch, _, _ in hs:
        ch.reset_stats()
    torch.cuda.synchronize()
    n0 = sum(ch.L.alfgpu_launch_count(ch.h) for ch, _, _ in hs)
    ms = 0.0
    cur = torch.cuda.current_stream(local)
    with ClockSampler(local) as clk:
        for i in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ends = [torch.cuda.Event() for _ in hs]
            e0.record(cur)

            for k in range(len(hs)):
                streams[k].wait_event(e0)
            sweep_all()
            for k in range(len(hs)):
                ends[k].record(streams[k])
            for e in ends:
                cur.wait_event(e)
            e1.record(cur)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
    n_launch = sum(ch.L.alfgpu_launch_count(ch.h) for ch, _, _ in hs) - n0
    # per group for the whole-sweep roofline: the adapted Nwrap, accepted flips per chain and sweep
    try:
        rgroups = [(dataclasses.replace(m, nwrap=ch.nwrap()),
                    sum(ch.stats(k).n_acc for k in range(len(mem))) / float(steps * len(mem)), 0, len(mem))
                   for ch, m, mem in hs]
    except Exception as e:  # only the roofline object depends on it
        rgroups = e
    xmax = max(ch.stats(k).xmaxG for ch, _, mem in hs for k in range(len(mem)))
    h2d = d2h = 0
    e2e_s = None
    if e2e:
        us = [[np.stack([rng.sweep_uniforms(replicas.replica_seed(args.seed, rank, c), k, m.n_op, m.ltrot, 1000 + i)
                         for k, (c, _) in enumerate(members)]) for ch, m, members in hs] for i in range(steps)]
        h2d = sum(u.nbytes for u in us[0])
        d2h = sum(m.n_fl * m.ndim * m.ndim * 16 for _, m, _ in hs)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(steps):
            sweep_all(us[i])
            for ch, _, _ in hs:
                ch.green(0)
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
    pool.shutdown()
    out = dict(t_dev=ms / 1e3, t_e2e=e2e_s, clocks=clk.summary(), launches=n_launch, h2d=h2d, d2h=d2h,
               nchains=nchains, groups=[{"L": m.params.get("L1"), "Ltrot": m.ltrot, "chains": len(mem),
                                        "nwrap": nw, "xmaxG_at_adapt": worst}
                                       for (_, m, mem), (nw, worst) in zip(hs, nwraps)], xmaxG=xmax,
               rgroups=rgroups, steps=steps)
    for ch, _, _ in hs:
        ch.close()
    return out


def batch_summary(ws, rb, precision) -> dict:
    ms_step = 1e3 * rb["t_dev"] / rb["steps"]
    d = {"value": ws * rb["nchains"] * rb["steps"] / rb["t_dev"], "unit": "sweeps/s", "chains_per_gpu": rb["nchains"],
         "steps": rb["steps"], "ms_per_step": ms_step, "gpu_launches": int(rb["launches"]), "clocks": rb["clocks"],
         "groups": rb["groups"], "precision_green": {"xmaxG": rb["xmaxG"]},
         "sweep_roofline": _reported(sweep_roofline_groups, rb["rgroups"], ms_step, precision, FP64_DMMA_TFLOPS,
                                     measured_bf16_peak()[0])}
    if rb["t_e2e"]:
        d["e2e"] = ws * rb["nchains"] * rb["steps"] / rb["t_e2e"]
    return d


def batch_cpu_baseline(seed: int, slices: int = 10):
    """One host core on the batch: per (L, beta) group a bounded oracle sample (``slices`` time
    slices of one chain, by default Nwrap of them with the one stabilisation they end in, so
    the sample holds the sweep's own mix; scaled to a sweep); a step costs the sum
    over all chains, so the aggregate rate is chains / sum of per-chain sweep times."""
    import oracle
    from alf_gb300 import model as mdl, rng
    groups = batch128_groups(seed)
    t_step, t_sample, n = 0.0, 0.0, 0
    for (L, beta), members in sorted(groups.items()):
        m = mdl.hubbard("square", L, L, U=members[0][1], beta=beta, dtau=0.1, nwrap=10)
        o = oracle.Oracle(m, threads=1)
        o.set_fields(rng.initial_fields(seed, 0, m.n_op, m.ltrot))
        o.init_state()
        u = rng.sweep_uniforms(seed, 0, m.n_op, m.ltrot, 0)
        ns = min(slices, 2 * m.ltrot)
        t0 = time.perf_counter()
        o.sweep_chunk(u, ns)
        dt = time.perf_counter() - t0
        t_step += len(members) * dt * (2.0 * m.ltrot / ns)
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
    from alf_gb300 import replicas
    m, ltau0 = workload_model(args.config)
    ltau = ltau0 if args.ltau < 0 else args.ltau
    common = {"metric": METRIC, "unit": "sweeps/s", "steps": args.steps, "warmup": args.warmup,
              "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
              "data": "synthetic (seeded fields and draws)", "config": bench_config(args, m, ltau)}

    if args.impl == "reference":
        if rank != 0:
            return
        if args.config == "batch128":
            cpu = batch_cpu_baseline(args.seed)
            arm = {"parallelism": "one host core", "sample": cpu["sample"]}
        else:
            cpu = host_baseline(args, m, ltau, args.steps, args.warmup)
            arm = {"parallelism": f"{cpu['walkers']} host walkers (single-threaded processes, one chain each)",
                   "draws": "host arrays of the counter stream", "one_chain_all_threads": cpu["one_chain_all_threads"]}
        v = cpu["value"]
        line = dict(common, impl="reference", value=v, n_gpus=args.gpus,
                    ms_per_step=1e3 * cpu.get("walkers", 1) / v, dtype="c128", arm=arm, cpu_baseline=cpu,
                    e2e={"value": v, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
        print(json.dumps(line))
        return

    other = "fp64" if args.precision == "mixed" else "mixed"
    cmp_steps, cmp_warm = min(args.steps, 5), min(args.warmup, 3)
    if args.config == "batch128":
        rb = run_batch(args, ws, rank, local, args.precision, args.steps, args.warmup)
        if rank != 0:
            return
        head = batch_summary(ws, rb, args.precision)
        line = dict(common, value=head["value"], n_gpus=ws, ms_per_step=head["ms_per_step"])
        other_sum = None
        if args.compare and ws == 1:
            ro = run_batch(args, ws, rank, local, other, cmp_steps, cmp_warm, e2e=False)
            other_sum = batch_summary(ws, ro, other)
        cpu = None
        if not args.no_cpu_baseline:
            cpu = _reported(batch_cpu_baseline, replicas.replica_seed(args.seed, rank))
        line.update({
            "dtype": "c128" if args.precision == "fp64" else "c128 state, digit-sliced bf16 tensor products",
            "arm": {"precision": args.precision, "chains_per_gpu": head["chains_per_gpu"], "groups": head["groups"],
                    "parallelism": f"replicas x{ws}; groups " + ("one after another" if args.serial_groups else
                                                                  "concurrent through alfgpu_sweep_many (one host thread, a stream per handle)"),
                    "draws": "device counter stream (value); host arrays through the C ABI (e2e)"},
            "e2e": {"value": head.get("e2e"), "unit": "sweeps/s", "h2d_bytes_per_step": rb["h2d"],
                    "d2h_bytes_per_step": rb["d2h"]},
            "roofline": None, "cpu_baseline": cpu, "clocks": head["clocks"], "gpu_launches": head["gpu_launches"],
            "precision_green": head["precision_green"], "sweep_roofline": head["sweep_roofline"]})
        if other_sum is not None:
            line[other] = other_sum
            line["mixed_over_fp64"] = (head["value"] / other_sum["value"] if args.precision == "mixed"
                                       else other_sum["value"] / head["value"])
        print(json.dumps(line))
        return

    r = run_ours(args, ws, rank, local, args.precision, args.chains, args.steps, args.warmup, e2e=True,
                 measure=args.compare)
    if rank != 0:
        return
    head = form_summary(ws, r)
    line = dict(common, value=head["value"], n_gpus=ws, ms_per_step=head["ms_per_step"])
    extra = {}
    if args.compare and ws == 1:
        ro = run_ours(args, ws, rank, local, other, args.chains, cmp_steps, cmp_warm, e2e=False)
        extra[other] = form_summary(ws, ro)
        extra["mixed_over_fp64"] = (head["value"] / extra[other]["value"] if args.precision == "mixed"
                                    else extra[other]["value"] / head["value"])
        if args.chains > 1:
            pc = {}
            for prec in ("fp64", "mixed"):
                s1 = form_summary(ws, run_ours(args, ws, rank, local, prec, 1, cmp_steps, cmp_warm, e2e=False))
                pc[prec] = {k: s1[k] for k in ("value", "unit", "ms_per_step", "delay_depth", "clocks", "phases",
                                               "roofline", "sweep_roofline", "precision_green")}
            pc["mixed_over_fp64"] = pc["mixed"]["value"] / pc["fp64"]["value"]
            extra["per_chain"] = pc
        extra["vs_fp64"] = _reported(mixed_vs_fp64, m, args.seed, local, args.flags, ltau, args.wrap_bits,
                                     args.propagate_bits)
    cpu = None
    if not args.no_cpu_baseline:
        cpu = _reported(host_baseline, args, m, ltau, 1, 1)
    line.update({
        "dtype": "c128" if args.precision == "fp64" else
        "c128 state; G wraps, UDV propagation, stabilisation products (and batched flushes / explicit Q) as "
        "FP64-accurate digit-sliced BF16 tensor-core products; per-visit determinants in double-float with FP64 "
        "ratio and phase accumulation; pivoted QR, solves and phases FP64",
        "arm": {"precision": args.precision, "chains_per_gpu": args.chains, "pivoting": args.pivoting,
                "flags": args.flags, "wrap_bits": args.wrap_bits, "propagate_bits": args.propagate_bits,
                "delay_depth": r["delay"],
                "delay_depth_source": "autotuned (alfgpu_tune_delay)" if args.tune else "default",
                "parallelism": f"replicas x{ws}, {args.chains} chains per GPU in one handle",
                "draws": "device counter stream (value); host arrays through the C ABI (e2e)"},
        "e2e": {"value": head["e2e"], "unit": "sweeps/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"]},
        "roofline": head["roofline"], "cpu_baseline": cpu, "clocks": head["clocks"],
        "gpu_launches": head["gpu_launches"], "phases": head["phases"], "precision_green": head["precision_green"],
        "acceptance": head["acceptance"], "per_chain_sweeps_per_s": head["per_chain_sweeps_per_s"],
        "sweep_roofline": head["sweep_roofline"]})
    if r.get("meas"):
        line["measuring_sweeps"] = r["meas"]
    line.update(extra)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
