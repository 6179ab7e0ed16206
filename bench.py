#!/usr/bin/env python3
"""Benchmark of the Holstein TDVP hot path (one JSON line on rank 0).

A step is one TDVP time step (a full left-to-right plus right-to-left sweep)
of the configured chain.  Default workload ``holstein-2site-L32``: 32
molecules x 2 modes (omega 0.2 / 1.2, g 0.5 / 1.0), phonon cutoff 16, J = -1,
N_ex = 1 charge sectors, seeded random MPS at D = 128, two-site TDVP with
dt = 0.05, Krylov maxIter 11 (dimension <= 10), tolExp 1e-8, SVD cutoff 1e-8.
Inputs are synthetic: a seeded random right-canonical U(1) MPS and the
Holstein Hamiltonian as an MPO, generated on the host.

value      algorithmic TFLOP/s: 8*M*N*K summed over every complex GEMM the
           reference algorithm issues in the timed sweeps (Lanczos iterations
           as actually run), divided by the device time of those sweeps
           (CUDA events on the library's stream), MPS and environments already
           resident in HBM; L2 is flushed between steps.
e2e        the same metric through the public C ABI with host buffers: every
           step uploads the MPS and MPO from pinned host memory, builds the
           environments, sweeps and downloads the MPS.
roofline   the grouped block-sparse GEMM on the tensor cores: reference flops
           of its block pairs / the event-timed duration of the GEMM calls
           (operand slicing launch and GEMM launch together), against the
           measured dense FP16/BF16 tensor peak (the digit GEMM runs on the
           FP16 pipe); traffic from the committed ncu summary.
roofline_lanczos, roofline_mix  the Lanczos step and the MPO mixing kernels:
           algorithmic bytes / event-timed duration against the measured HBM
           copy rate (bytes_roofline).
fp64_compare  the mixed path against the plain FP64 GPU path on the same
           chain over --compare-steps steps (default 1): time per step and the
           largest site-population and energy differences.
cpu_baseline  the CPU oracle (restatement of the reference on OpenBLAS, all
           host threads) on the same chain: one molecule's five two-site local
           updates (sites 20-24) timed after the pass is advanced there, the
           full step extrapolated (2 x 159 updates).

batched    (N = 1, default config) the 64-chain disordered ensemble of
           --config holstein-1site-batch64 advanced by kv_sweep_batched: one
           untimed and one timed one-site step (batched_leg); --no-batched
           skips it.
--impl reference  runs only the CPU oracle sample (rank 0) and prints its line,
           with a one-thread measurement of the same sample beside it.
--config holstein-1site-batch64  the batched disordered ensemble instead
           (run_batched); under torchrun its chains are split across ranks.
--config holstein-1site-L24-grad  the differentiation workload: gradients
           through 10 one-site steps of the L = 24, D = 96 chain (run_gradient).
N > 1 (torchrun): each rank evolves its own replica chain (a single chain's
sweep is sequential), value = total flops / max time over ranks.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
METRIC = "TDVP sweep s & H_eff TFLOP/s, mixed vs plain FP64 on GB300 at <=1e-6 pop err"
DEFAULT_CONFIG = "holstein-2site-L32"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default=DEFAULT_CONFIG)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-compare", action="store_true", help="skip the mixed-vs-FP64 comparison leg")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched-ensemble leg of the default run (its own config: --config "
                         "holstein-1site-batch64)")
    ap.add_argument("--compare-steps", type=int, default=1,
                    help="time steps of the mixed-vs-FP64 comparison leg (on the benchmark chain itself)")
    ap.add_argument("--compare-against", default="fp64", choices=["fp64", "fp64-contractions"],
                    help="reference of the comparison leg: the plain FP64 path, or FP64 contractions with the "
                         "mixed SVD (KV_MIXED_SVD, whose L32 steps match the CPU oracle to 5e-10; 18x faster)")
    ap.add_argument("--chains", type=int, default=64,
                    help=f"{BATCH_CONFIG}: members of the disordered ensemble advanced together")
    ap.add_argument("--max-streams", type=int, default=0, help=f"{BATCH_CONFIG}: worker streams (0: library default)")
    ap.add_argument("--molecules", type=int, default=None,
                    help="shorter chain with the same local structure (profiling runs)")
    ap.add_argument("--cpu-only-json", action="store_true", help=argparse.SUPPRESS)
    return ap.parse_args()


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.f.read())) if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


BATCH_CONFIG = "holstein-1site-batch64"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["bf16_tflops"]), float(d["hbm_gbs"]), "measured"
    return 1900.0, 6800.0, "fallback"


def traffic_per_launch(config: str):
    """DRAM bytes per grouped-GEMM launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"k_gemm_tc_{config}.md")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    return None


def build_workload(config: str, seed: int, n_mol: int | None = None):
    import __graft_entry__ as ge

    ge.load_package()
    from kylin_v_gb300 import holstein as H

    chain, D, d = H.config_chain(config)
    if n_mol is not None:
        chain = H.HolsteinChain(n_mol, chain.omega, chain.g[:n_mol], chain.cutoff, chain.J, chain.eps[:n_mol])
    return chain, D, d, H.random_mps(chain, D, seed=seed), H.hamiltonian_mpo(chain)


CPU_WINDOW_SITE, CPU_WINDOW_UPDATES = 20, 5  # one molecule (sites 20-24) of the two-site L->R pass


def cpu_baseline(config: str, samples: int = 1, warm: int = 0):
    """The CPU oracle (restatement of the reference on OpenBLAS, the threads
    OPENBLAS_NUM_THREADS allows, default all host cores) on the same chain as
    the GPU: its two-site left-to-right pass is advanced once to site 20, then
    each sample times the 5 local updates of sites 20-24 (one molecule: the
    exciton site and both modes' phonon and auxiliary sites) on a copy of that
    state.  value = reference flops of the sample / its time; the full step
    (2 x 159 local updates) is extrapolated from it."""
    cores = int(os.environ.get("OPENBLAS_NUM_THREADS", "0")) or (os.cpu_count() or 1)
    os.environ["OPENBLAS_NUM_THREADS"] = str(cores)
    chain, D, d, mps, mpo = build_workload(config, 1234)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O  # CPU baseline leg only

    t = O.Tdvp(mps, mpo, d["tol_svd"], d["tol_exp"], D, d["max_iter"], d["dt"])
    i0, n = CPU_WINDOW_SITE, CPU_WINDOW_UPDATES
    for _ in range(max(1, warm)):  # the first call also advances the pass to site 20 (untimed)
        t.window(i0, n)
    O.flops(True)
    secs = [t.window(i0, n) for _ in range(samples)]
    f = O.flops(True)
    tot = sum(secs)
    updates_per_step = 2 * (chain.n_sites - 1)
    return {"value": f / tot / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
            "sample": f"{n} two-site local updates (sites {i0}-{i0 + n - 1}, one molecule) of the left-to-right pass "
                      f"of the {chain.n_sites}-site chain, same inputs and tolerances as the GPU run; {samples} "
                      f"sample(s), {f / samples / 1e9:.1f} GFLOP in {tot / samples:.2f} s each",
            "ms_per_step": 1e3 * tot / samples * updates_per_step / n,
            "ms_per_step_note": f"extrapolated: {updates_per_step} local updates per step / {n} per sample"}


def cpu_single_thread(config: str, samples: int = 2):
    """The same CPU sample with one OpenBLAS thread (a child process, so the
    thread count is set before the library loads)."""
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--impl", "reference", "--cpu-only-json",
                        "--config", config, "--steps", str(samples), "--warmup", "0"],
                       env=env, capture_output=True, text=True, timeout=1800)
    if r.returncode != 0:
        return {"unavailable": (r.stderr.strip().splitlines() or ["failed"])[-1]}
    return json.loads(r.stdout.strip().splitlines()[-1])


def run_reference(args):
    ws, rank, _ = dist()
    if rank != 0:
        return
    cb = cpu_baseline(args.config, samples=args.steps, warm=args.warmup)
    if args.cpu_only_json:
        print(json.dumps(cb), flush=True)
        return
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": cb["ms_per_step"],
            "ms_per_step_note": cb["ms_per_step_note"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": args.config, "same_config": True, "window": cb["sample"]},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    one = cpu_single_thread(args.config)
    line["single_thread"] = {k: one[k] for k in ("value", "unit", "cores", "ms_per_step") if k in one} if "value" in one \
        else one
    print(json.dumps(line), flush=True)


def run_ours(args):
    ws, rank, local = dist()
    import numpy as np
    import torch

    import __graft_entry__ as ge

    ge.load_package()
    from kylin_v_gb300 import kvgpu as G

    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    G.init(local)
    prec = G.KV_MIXED_TF32 if args.precision == "mixed" else G.KV_FP64
    chain, D, d, mps, mpo = build_workload(args.config, 1234 + rank, n_mol=args.molecules)
    mode = d["mode"]
    t = G.TDVP(mps, mpo, d["tol_svd"], d["tol_exp"], D, d["max_iter"], d["dt"], prec)
    sweep = t.two_site if mode == 2 else t.one_site
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)
    for _ in range(args.warmup):
        sweep()

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    dev_ms, flops, gemm_flops = 0.0, 0.0, 0.0
    modules, host_modules = {}, {}
    host_sweep_ms, plans_built, plan_ms = 0.0, 0, 0.0
    barrier()
    n0 = G.launches()
    G.svd_stats(reset=True)
    G.krylov_stats(reset=True)
    G.profile(True)
    with Clocks(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            sweep()
            st = t.stats()
            dev_ms += st["sweep_ms"]
            flops += st["ref_flops"]
            gemm_flops += st["gemm_ref_flops"]
            for k, v in st["modules_ms"].items():
                modules[k] = modules.get(k, 0.0) + v
            hs = t.host_stats()
            for k, v in hs["modules_ms"].items():
                host_modules[k] = host_modules.get(k, 0.0) + v
            host_sweep_ms += hs["sweep_ms"]
            plans_built += hs["plans_built"]
            plan_ms += hs["plan_ms"]
    barrier()
    prof = G.profile_read()
    lz = G.profile_read_lanczos()
    mx = G.profile_read_mix()
    G.profile(False)
    launches = G.launches() - n0
    svd = G.svd_stats(reset=True)
    kry = G.krylov_stats(reset=True)
    clocks = clk.summary()
    tot_flops, max_ms = flops, dev_ms
    if ws > 1:
        x = torch.tensor([flops, dev_ms], dtype=torch.float64, device="cuda")
        y = x.clone()
        torch.distributed.all_reduce(x[:1], op=torch.distributed.ReduceOp.SUM)
        torch.distributed.all_reduce(y[1:], op=torch.distributed.ReduceOp.MAX)
        tot_flops, max_ms = float(x[0]), float(y[1])
    value = tot_flops / (max_ms / 1e3) / 1e12

    # ---- end to end through the public API with pinned host buffers
    e2e = None
    steps_e2e = max(1, min(args.steps, 2))
    host = []
    for tns in mps + mpo:
        data = np.concatenate([a.ravel() for _, a in tns.blocks]).astype(np.complex128)
        pin = torch.from_numpy(data.view(np.float64)).pin_memory()
        host.append((tns, pin))
    h2d = sum(p.numel() * 8 for _, p in host)
    d2h = sum(a.size * 16 for tns in mps for _, a in tns.blocks)
    barrier()
    t0 = time.perf_counter()
    e2e_flops = 0.0
    for _ in range(steps_e2e):
        dev = []
        for tns, pin in host:
            dev.append(G.Tensor.from_pinned(tns, pin.data_ptr()))
        te = G.TDVP(dev[:len(mps)], dev[len(mps):], d["tol_svd"], d["tol_exp"], D, d["max_iter"], d["dt"], prec)
        te.two_site() if mode == 2 else te.one_site()
        e2e_flops += te.stats()["ref_flops"]
        out = te.sites()
        _ = [s.to_host() for s in out]
        del te
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": e2e_flops / e2e_s / 1e12, "unit": "TFLOP/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "steps": steps_e2e}

    if rank != 0:
        return
    bf16, hbm, src = peaks()
    # the grouped GEMM runs on the FP16 tensor pipe (dense FP16 = dense BF16 rate);
    # its 3M digit scheme issues 45 FP16 MMAs per complex K-step (11.25 tensor
    # flops per algorithmic flop), so frac cannot exceed ~0.09 on this pipe
    f16_peak = bf16
    achieved = prof["gemm_ref_flops"] / max(1e-9, prof["gemm_ms"]) / 1e9  # TFLOP/s
    per_launch = prof["gemm_ref_flops"] / max(1, prof["gemm_launches"])
    tr = traffic_per_launch(args.config)
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": ("c128 values; contractions as 3M FP16 digit products (5 x 8-bit digits of 38-bit fixed point) "
                  "with exact FP32 accumulation; c128 Lanczos, FP32 QR+Jacobi SVD + c128 polish") if prec else "c128",
        "data": "synthetic (seeded random right-canonical U(1) MPS, Holstein FSM MPO)",
        "config": {"workload": args.config + (f" ({args.molecules} molecules)" if args.molecules else ""),
                   "n_sites": chain.n_sites, "D": D, "mode": f"{mode}-site TDVP",
                   "dt": d["dt"], "max_iter": d["max_iter"], "precision": args.precision, "l2_flush": True,
                   "replicas_per_gpu": 1},
        "modules_ms_per_step": {k: v / args.steps for k, v in modules.items()},
        "host": {"modules_ms_per_step": {k: v / args.steps for k, v in host_modules.items()},
                 "sweep_ms_per_step": host_sweep_ms / args.steps, "heff_plans_built_per_step": plans_built / args.steps,
                 "plan_ms_per_step": plan_ms / args.steps},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": f16_peak, "unit": "TFLOP/s",
                     "frac": achieved / f16_peak, "traffic": tr,
                     "kernel": "k_gemm_tc" if prec else "k_gemm_fp64",
                     "flops_per_launch": per_launch, "launches": prof["gemm_launches"],
                     "peak_source": f"dense FP16/BF16 tensor rate, {src} ({bf16:.1f} TFLOP/s bf16); "
                                    "achieved counts the reference's 8MNK flops of the block pairs"},
        "roofline_lanczos": bytes_roofline(lz, "k_lanczos_step", hbm, src),
        "roofline_mix": bytes_roofline(mx, "k_mix", hbm, src),
        "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
        "svd_sectors": {"per_step": svd["sectors"] / args.steps, "mean_columns": svd["mean_columns"],
                        "mean_rank": svd["mean_rank"], "mean_jacobi_sweeps": svd["mean_sweeps"],
                        "max_jacobi_sweeps": svd["max_sweeps"]},
        "krylov": {"calls_per_step": kry["calls"] / args.steps, "iterations_issued_per_call": kry["issued_per_call"],
                   "mean_dimension": kry["mean_dimension"]},
        "gpu_launches_per_step": launches / args.steps,
    }
    if ws == 1 and not args.no_batched and args.molecules is None and args.config == DEFAULT_CONFIG:
        line["batched"] = batched_leg(G, prec, max_streams=args.max_streams)
    # the side legs report their own failure instead of losing the line
    if not args.no_compare:
        try:
            line["fp64_compare"] = compare_fp64(args, G)
        except Exception as e:
            line["fp64_compare"] = {"error": f"{type(e).__name__}: {e}"}
    if not args.no_cpu:
        try:
            cb = cpu_baseline(args.config)
            line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
            line["cpu_baseline"]["ms_per_step"] = cb["ms_per_step"]
        except Exception as e:
            line["cpu_baseline"] = {"error": f"{type(e).__name__}: {e}"}
    print(json.dumps(line), flush=True)


def bytes_roofline(rec, kernel, hbm, src):
    """A streaming kernel's algorithmic bytes over its event-timed duration,
    against the measured HBM copy rate.  k_lanczos_step: the two overlaps,
    two subtractions, norm and normalisation of one Lanczos iteration (16 B
    per complex element moved); k_mix: the MPO mixings of the H_eff applies
    and environment updates (per output element 16 B written and 16 B read
    per contracted index of each active term).  Their inputs were written by
    the launch just before, so at these sizes much of the traffic is served
    from L2 and frac can pass 1."""
    if not rec["launches"] or rec["ms"] <= 0.0:
        return None
    achieved = rec["bytes"] / (rec["ms"] / 1e3) / 1e9
    return {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "bytes_per_launch": rec["bytes"] / rec["launches"], "launches": rec["launches"],
            "us_per_launch": rec["ms"] * 1e3 / rec["launches"], "peak_source": f"HBM copy, {src}"}


def compare_fp64(args, G):
    """Mixed vs plain FP64 GPU path on the benchmark chain itself (same seeded
    inputs) over --compare-steps time steps: device time per step of each and
    the largest site-population and energy differences after every step."""
    import numpy as np

    import __graft_entry__ as ge

    ge.load_package()
    from kylin_v_gb300 import holstein as H

    chain, D, d, mps, mpo = build_workload(args.config, 1234, n_mol=args.molecules)
    # populations: every exciton site's density from one left and one right pass (kv_local_expectations)
    ident = [G.Tensor.from_host(x) for x in H.identity_mpo(chain)]
    dens = [(j, G.Tensor.from_host(H.density_mpo(chain, j)[j])) for j in chain.exciton_sites()]
    hm = [G.Tensor.from_host(x) for x in mpo]
    ref = G.KV_FP64 if args.compare_against == "fp64" else G.KV_MIXED_SVD
    runs = {p: G.TDVP(mps, mpo, d["tol_svd"], d["tol_exp"], D, d["max_iter"], d["dt"], p)
            for p in (ref, G.KV_MIXED_TF32)}
    ms = {p: 0.0 for p in runs}
    modules = {p: {} for p in runs}
    perr = eerr = 0.0
    per_step = []
    nsteps = args.compare_steps
    for _ in range(nsteps):
        obs = {}
        for p, t in runs.items():
            t.two_site() if d["mode"] == 2 else t.one_site()
            st = t.stats()
            ms[p] += st["sweep_ms"]
            for k, v in st["modules_ms"].items():
                modules[p][k] = modules[p].get(k, 0.0) + v / nsteps
            s = t.sites()
            obs[p] = (np.array([v.real for v in G.local_expectations(s, ident, dens)]), G.expectation(s, hm, s).real)
        pe = float(np.abs(obs[ref][0] - obs[G.KV_MIXED_TF32][0]).max())
        per_step.append(float("%.3g" % pe))
        perr = max(perr, pe)
        eerr = max(eerr, abs(obs[ref][1] - obs[G.KV_MIXED_TF32][1]))
    return {"sample": f"{chain.n_sites}-site benchmark chain, {nsteps} step(s), same inputs",
            "reference_mode": args.compare_against,
            "fp64_ms_per_step": ms[ref] / nsteps, "mixed_ms_per_step": ms[G.KV_MIXED_TF32] / nsteps,
            "speedup_mixed_vs_fp64": ms[ref] / max(1e-9, ms[G.KV_MIXED_TF32]),
            "fp64_modules_ms_per_step": modules[ref],
            "max_pop_err": perr, "max_energy_err": eerr, "pop_err_by_step": per_step,
            "energy_fp64": float(obs[ref][1])}


def batched_leg(G, prec, chains: int = 64, steps: int = 1, warmup: int = 1, max_streams: int = 0) -> dict:
    """The batched ensemble (run_batched's workload, 64 disordered chains,
    one-site TDVP) measured inside the default run at N = 1: `warmup` untimed
    and `steps` timed time steps of all chains advanced together by
    kv_sweep_batched (device ms).  Returns its figures, or the error that
    stopped it; the headline line is printed either way."""
    try:
        import __graft_entry__ as ge

        ge.load_package()
        from kylin_v_gb300 import holstein as H

        members = [H.disordered_chain(i) for i in range(chains)]
        host = [(H.random_mps(ch, D, seed=1234 + i), H.hamiltonian_mpo(ch), D) for i, (ch, D) in enumerate(members)]
        bat = [G.TDVP([G.Tensor.from_host(x) for x in m], [G.Tensor.from_host(x) for x in w], 1e-8, 1e-8, D, 11,
                      0.05, prec) for m, w, D in host]
        G.sweep_batched(bat, 1, warmup, max_streams)
        n0 = G.launches()
        ms, flops = 0.0, 0.0
        for _ in range(steps):
            ms += G.sweep_batched(bat, 1, 1, max_streams)
            flops += sum(t.stats()["ref_flops"] for t in bat)
        launches = G.launches() - n0
        del bat
        return {"workload": BATCH_CONFIG, "chains": chains, "mode": "1-site TDVP", "steps": steps,
                "warmup": warmup, "ms_per_step": ms / steps, "value": flops / (ms / 1e3) / 1e12, "unit": "TFLOP/s",
                "sites": sum(ch.n_sites for ch, _ in members), "gpu_launches_per_step": launches / steps,
                "note": f"device time of kv_sweep_batched; the full leg with the one-after-another timing is "
                        f"bench.py --config {BATCH_CONFIG}"}
    except Exception as e:  # the leg must not cost the headline line
        return {"workload": BATCH_CONFIG, "error": f"{type(e).__name__}: {e}"}


def run_batched(args):
    """The batched ensemble: --chains members of the disordered ensemble
    (holstein.disordered_chain: L in [8, 48], D in {32, 64, 128, 256},
    eps ~ N(0, 0.5^2), omega = 1, g in [0.5, 1.5], cutoff 8), one-site TDVP at
    dt = 0.05, advanced together by kv_sweep_batched.  Under torchrun the
    chains are split across the ranks (ensemble.shard: no data-path
    collective; the total is fixed, so scaling is strong).  At N = 1 the same
    chains advanced one after another by kv_tdvp_sweep are timed beside it."""
    import torch

    import __graft_entry__ as ge

    ge.load_package()
    from kylin_v_gb300 import ensemble as E
    from kylin_v_gb300 import holstein as H
    from kylin_v_gb300 import kvgpu as G

    ws, rank, local = dist()
    torch.cuda.set_device(local)
    if ws > 1:
        torch.distributed.init_process_group("nccl")
    G.init(local)
    prec = G.KV_MIXED_TF32 if args.precision == "mixed" else G.KV_FP64
    members = [H.disordered_chain(i) for i in range(args.chains)]
    mine = E.shard([E.chain_cost(ch.n_sites, D) for ch, D in members], ws)[rank]
    host = [(H.random_mps(members[i][0], members[i][1], seed=1234 + i), H.hamiltonian_mpo(members[i][0]),
             members[i][1]) for i in mine]

    def make():
        return [G.TDVP([G.Tensor.from_host(x) for x in m], [G.Tensor.from_host(x) for x in w], 1e-8, 1e-8, D, 11,
                       0.05, prec) for m, w, D in host]

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    bat = make()
    G.sweep_batched(bat, 1, args.warmup, args.max_streams)
    n0 = G.launches()
    bat_ms, flops = 0.0, 0.0
    barrier()
    t0 = time.perf_counter()
    with Clocks(local) as clk:
        for _ in range(args.steps):
            bat_ms += G.sweep_batched(bat, 1, 1, args.max_streams)
            flops += sum(t.stats()["ref_flops"] for t in bat)
    barrier()
    wall = time.perf_counter() - t0
    launches = G.launches() - n0
    tot_flops, max_ms = flops, bat_ms
    if ws > 1:
        x = torch.tensor([flops, bat_ms], dtype=torch.float64, device="cuda")
        y = x.clone()
        torch.distributed.all_reduce(x[:1], op=torch.distributed.ReduceOp.SUM)
        torch.distributed.all_reduce(y[1:], op=torch.distributed.ReduceOp.MAX)
        tot_flops, max_ms = float(x[0]), float(y[1])
    line = {"metric": METRIC, "value": tot_flops / (max_ms / 1e3) / 1e12, "unit": "TFLOP/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "c128" if not prec else "mixed (as the main workload)",
            "data": "synthetic (seeded disordered ensemble, random right-canonical U(1) MPS)",
            "config": {"workload": BATCH_CONFIG, "chains": args.chains, "mode": "1-site TDVP", "dt": 0.05,
                       "max_iter": 11, "precision": args.precision, "max_streams": args.max_streams or 8,
                       "sites": sum(ch.n_sites for ch, _ in members), "D": [D for _, D in members],
                       "chains_per_rank": len(mine)},
            "wall_ms_per_step": 1e3 * wall / args.steps, "gpu_launches": launches, "clocks": clk.summary()}
    if ws == 1:
        seq, seq_ms = make(), 0.0
        for t in seq:
            for _ in range(args.warmup):
                t.one_site()
        for _ in range(args.steps):
            for t in seq:
                t.one_site()
                seq_ms += t.stats()["sweep_ms"]
        line["sequential_ms_per_step"] = seq_ms / args.steps
        line["batch_speedup"] = seq_ms / max(1e-9, bat_ms)
    if rank == 0:
        print(json.dumps(line), flush=True)


WINDOW_CONFIGS = {"holstein-2site-L64": (9, 9)}  # first site, local updates: one molecule (9 sites)


def run_window(args):
    """A chain too long to sweep inside a benchmark run (the large single
    chain: 64 molecules x 4 modes, 576 sites, D = 512): its two-site
    left-to-right pass is advanced to the second molecule (untimed), then
    --steps windows of one molecule's 9 local updates each are timed on the
    device (--warmup windows before them untimed); the full step (2 x 575
    local updates) is extrapolated from the timed windows."""
    import torch

    import __graft_entry__ as ge

    ge.load_package()
    from kylin_v_gb300 import kvgpu as G

    ws, rank, local = dist()
    torch.cuda.set_device(local)
    G.init(local)
    prec = G.KV_MIXED_3M_DIGITS if args.precision == "mixed" else G.KV_FP64
    t_host = time.perf_counter()
    chain, D, d, mps, mpo = build_workload(args.config, 1234 + rank)
    t = G.TDVP(mps, mpo, d["tol_svd"], d["tol_exp"], D, d["max_iter"], d["dt"], prec)
    setup_s = time.perf_counter() - t_host
    i0, n = WINDOW_CONFIGS[args.config]
    t.window(i0, 0)
    at = i0
    for _ in range(args.warmup):
        t.window(at, n)
        at += n
    G.svd_stats(reset=True)
    G.profile(True)
    G.profile_read()
    dev_ms, flops, modules = 0.0, 0.0, {}
    n0 = G.launches()
    with Clocks(local) as clk:
        for _ in range(args.steps):
            t.window(at, n)
            at += n
            st = t.stats()
            dev_ms += st["sweep_ms"]
            flops += st["ref_flops"]
            for k, v in st["modules_ms"].items():
                modules[k] = modules.get(k, 0.0) + v / args.steps
    prof = G.profile_read()
    G.profile(False)
    launches = G.launches() - n0
    svd = G.svd_stats(reset=True)
    bf16, hbm, src = peaks()
    updates_per_step = 2 * (chain.n_sites - 1)
    per_update_ms = dev_ms / (args.steps * n)
    achieved = prof["gemm_ref_flops"] / max(1e-9, prof["gemm_ms"]) / 1e9
    line = {
        "metric": METRIC, "value": flops / (dev_ms / 1e3) / 1e12, "unit": "TFLOP/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_update_ms * updates_per_step,
        "ms_per_step_note": f"extrapolated: {updates_per_step} local updates per step from {args.steps} window(s) "
                            f"of {n} (one molecule)",
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 values; contractions as 3M FP16 digit products (38-bit fixed point)" if prec else "c128",
        "data": "synthetic (seeded random right-canonical U(1) MPS, Holstein FSM MPO)",
        "config": {"workload": args.config, "n_sites": chain.n_sites, "D": D, "mode": "2-site TDVP window",
                   "window_first_site": i0, "window_updates": n, "dt": d["dt"], "max_iter": d["max_iter"],
                   "tol_svd": d["tol_svd"], "precision": args.precision},
        "modules_ms_per_window": modules, "window_ms": dev_ms / args.steps, "host_setup_s": setup_s,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s", "frac": achieved / bf16,
                     "traffic": None, "kernel": "k_gemm_tc" if prec else "k_gemm_fp64",
                     "flops_per_launch": prof["gemm_ref_flops"] / max(1, prof["gemm_launches"]),
                     "launches": prof["gemm_launches"], "peak_source": f"dense FP16/BF16 tensor rate, {src}"},
        "gpu_launches": launches, "clocks": clk.summary(),
        "svd_sectors": {"per_window": svd["sectors"] / args.steps, "mean_columns": svd["mean_columns"],
                        "mean_rank": svd["mean_rank"], "mean_jacobi_sweeps": svd["mean_sweeps"],
                        "max_jacobi_sweeps": svd["max_sweeps"]},
    }
    print(json.dumps(line), flush=True)


GRAD_CONFIG = "holstein-1site-L24-grad"


def run_gradient(args):
    """The differentiation workload: L = 24, one mode (omega = 1, g = 1, J = 1),
    cutoff 12, D = 96, one-site TDVP at dt = 0.05 without truncation, 10 steps.
    Gradients of msd = sum_t sum_i i P_i(t) and of <H> with respect to (J,
    omega, g): central differences with the 7 chains (theta, theta +- h e_k)
    advanced together (gradient.fd_gradient), and the reverse-mode <H>
    gradient through the parameter-linear MPO (gradient.energy_gradient_adjoint,
    on the base chain's state).  value = wall seconds per gradient evaluation
    (both quantities, all three parameters).  FP64 throughout: central
    differences need a map that is smooth in theta, and the mixed SVD's
    resolution floor (singular values below 1e-6 of a sector's largest read as
    zero) is not."""
    import numpy as np
    import torch

    import __graft_entry__ as ge

    ge.load_package()
    from kylin_v_gb300 import gradient as Gr
    from kylin_v_gb300 import holstein as H
    from kylin_v_gb300 import kvgpu as G

    _, _, local = dist()
    torch.cuda.set_device(local)
    G.init(local)
    prec = G.KV_FP64
    n_mol, cutoff, D, steps = 24, 12, 96, 10
    theta = {"J": 1.0, "omega": 1.0, "g": 1.0}
    for _ in range(max(0, args.warmup)):
        Gr.fd_gradient(n_mol, cutoff, D, theta, steps=1, precision=prec)
    torch.cuda.synchronize()
    walls, dev = [], []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            r = Gr.fd_gradient(n_mol, cutoff, D, theta, steps=steps, precision=prec)
            torch.cuda.synchronize()
            walls.append(time.perf_counter() - t0)
            dev.append(r["device_ms"])
    # reverse mode for <H> on the base chain's state (energy_gradient_adjoint)
    ch = Gr.holstein_chain(n_mol, cutoff, theta)
    mps = [G.Tensor.from_host(x) for x in H.random_mps(ch, D, seed=1234)]
    t0 = time.perf_counter()
    adj = Gr.energy_gradient_adjoint(ch, mps, precision=prec)
    torch.cuda.synchronize()
    adj_s = time.perf_counter() - t0
    fd_e = Gr.fd_gradient(n_mol, cutoff, D, theta, steps=0, precision=prec)["grad"]["energy"]
    line = {"metric": "wall seconds per (msd, <H>) gradient w.r.t. (J, omega, g) through 10 1TDVP steps",
            "value": float(np.median(walls)), "unit": "s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * float(np.median(walls)) / steps, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded random right-canonical U(1) MPS, Holstein FSM MPO)",
            "config": {"workload": GRAD_CONFIG, "n_mol": n_mol, "cutoff": cutoff, "D": D, "tdvp_steps": steps,
                       "chains": 7, "h": 1e-5, "precision": "fp64"},
            "device_ms_per_gradient": float(np.median(dev)),
            "grad_fd": r["grad"], "value_fd": r["value"],
            "adjoint_energy": {"seconds": adj_s, "grad": adj["grad"], "fd_grad_same_state": fd_e},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == BATCH_CONFIG:
        run_batched(args)
    elif args.config == GRAD_CONFIG:
        run_gradient(args)
    elif args.config in WINDOW_CONFIGS:
        run_window(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
