"""Benchmark of the Wilson-clover Dirac operator and its MG solve path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W]
                    [--workload mg|mg2|dslash|smoother|cg|coarse|hmc|batch] [--impl ours|reference]

Prints ONE JSON line (rank 0).  A step is one pass of the hot path over one
batch of seeded synthetic input (links U = exp(i theta), theta ~ N(0, 1/beta);
Gaussian complex sources), timed with CUDA events on the library's stream
(smg_timer_begin/end) between a barrier and a synchronize; the max over ranks
is reported.  Workloads:

* mg (default) — the multi-RHS MG-GCR solve on a 512 x 512 lattice, beta = 6,
  m = -0.05, c_sw = 1; three levels (4 x 4 then 2 x 2 aggregates, 16 null
  vectors per level = 16 coarse dofs, V-cycle); 32 right-hand sides solved
  together to a true FP64 residual of 1e-10 by an FP32 GCR (truncation 6)
  preconditioned with the FP32 hierarchy, whose fine smoother and coarsest CG
  keep their work vectors in FP16 with per-site scales, inside FP64 defect
  correction.  The
  hierarchy is built once before timing.  value = solves/s.  The plain FP64
  single-RHS MG on the same inputs is measured beside it
  (detail.plain_fp64_mg_solves_per_s).
* mg2 — two-level MG-GCR at L = 256, beta = 6, m = -0.05, c_sw = 1; 4 x 4
  aggregates with 8 null vectors split by chirality (16 coarse dofs), 2
  inverse iterations, 4 MR steps; one source; the FP32 hierarchy inside FP64
  defect correction against the plain FP64 MG on the same inputs.
* dslash — FP32 D on 32 right-hand sides at L = 512; value = algorithmic GB/s.
* smoother — the fine smoother's three kernels of one MR step on the FP16
  work vectors of the mg workload's hierarchy (L = 512, 32 RHS); value =
  algorithmic GB/s of the stencil with the fused MR reductions.  A small
  process for kernel profiles.
* coarse — the level-1 coarse operator of the mg workload alone (128 x 128
  sites, 16 dofs, 32 RHS); value = algorithmic GB/s.  A small case for
  kernel profiles.
* hmc — differentiated HMC at L = 128 (beta = 4, m = 0.1, c_sw = 1): nested
  Omelyan with 10 fermion-force steps and 4 gauge-force substeps per inner
  integration, mixed-precision solves to 1e-10, 20 trajectories;
  value = trajectories/s, with dH, acceptance and plaquette in detail.
* batch — 64 independent lattices, L drawn from {64, 96, 128, 192, 256, 384},
  beta ~ U[2, 8], m ~ U[-0.05, 0.2], c_sw = 1, 8 Gaussian RHS each; every
  lattice runs a 2-level MG (4 x 4, 8 null vectors) mixed GCR to a true FP64
  residual of 1e-10 plus its pseudofermion force; one stream per lattice, a
  pool of host workers over one largest-first queue; value = solves/s.
* cg — the small single-RHS case (L = 32, beta = 2, m = 0.1, c_sw = 1) FP64 CG;
  value = solves/s.

`--impl reference` times the reference's CPU implementation of the same
workload on this machine's host cores, with every core: the C restatement in
oracle/ (the reference tree is not present where the benchmark runs), which
makes its own inputs and builds its own hierarchy on the CPU; nothing of the
GPU library is loaded.  The same code gives the GPU arm's cpu_baseline.
`--gpus N` without a torchrun environment relaunches itself under
torch.distributed.run with N ranks.
"""
from __future__ import annotations

import argparse
import atexit
import ctypes as Cc
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Dslash HBM GB/s; MG-GCR solves/s to 1e-10, mixed+batched vs plain FP64"
DP = Cc.POINTER(Cc.c_double)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """One nvidia-smi process per benchmark process sampling SM clocks, power and throttle reasons
    every 200 ms with a timestamp, started before any timed work so that its start-up (NVML
    initialisation) never falls inside a timed region."""

    def __init__(self):
        self.proc = None
        self.path = None
        self.f = None

    def start(self, device: int):
        if self.proc is not None:
            return
        self.path = Path(tempfile.gettempdir()) / f"smg_clocks_{os.getpid()}.csv"
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(device),
                 "--query-gpu=timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
            t_end = time.monotonic() + 5.0  # first sample before anything is timed
            while time.monotonic() < t_end and self.proc.poll() is None and self.path.stat().st_size == 0:
                time.sleep(0.02)
        except (OSError, FileNotFoundError):
            self.proc = None

    def rows(self, t0: float, t1: float):
        """Samples taken between the wall-clock times t0 and t1 (seconds since the epoch).  The sampler
        stops here (nvidia-smi writes its samples out when it ends) and the next timed region starts
        another one before its timing begins."""
        if self.proc is None or self.path is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        self.proc = None
        if not self.path.exists():
            return None
        text = self.path.read_text()
        try:
            self.path.unlink()
        except OSError:
            pass
        out = []
        for line in text.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                ts = time.mktime(time.strptime(parts[0].split(".")[0], "%Y/%m/%d %H:%M:%S"))
                ts += float("0." + parts[0].split(".")[1]) if "." in parts[0] else 0.0
                out.append((ts, float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except (ValueError, IndexError):
                continue
        return [r for r in out if t0 <= r[0] <= t1]

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()
            try:
                self.path.unlink()
            except OSError:
                pass
            self.proc = None


SAMPLER = ClockSampler()
atexit.register(SAMPLER.stop)


class Clocks:
    """The clock samples that fall inside one timed region (the process-wide sampler, started at the
    first use if the workload did not start it earlier)."""

    def __init__(self, device: int):
        self.device = device
        self.t0 = self.t1 = 0.0

    def __enter__(self):
        SAMPLER.start(self.device)
        self.t0 = time.time()
        return self

    def __exit__(self, *a):
        self.t1 = time.time()
        time.sleep(0.25)  # the sample that covers the region's end

    def summary(self):
        rows = SAMPLER.rows(self.t0 - 0.1, self.t1 + 0.25)
        if rows is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for *_, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[1] for r in rows])), "sm_max_mhz": max(r[2] for r in rows),
                "power_w_max": max(r[3] for r in rows), "reasons": reasons, "samples": len(rows)}


def dist_env():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(v: float, ws: int) -> float:
    if ws == 1:
        return v
    import torch

    dev = "cuda" if torch.distributed.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def shard(items: list, rank: int, ws: int) -> list:
    """The batch's lattices of one rank: every ws-th one from position rank (independent lattices, no
    data exchange between ranks)."""
    return items[rank::ws]


# ------------------------------------------------------------------ workloads
MG = dict(L=512, beta=6.0, m=-0.05, r=1.0, csw=1.0, mu=0.0, seed=20240, nrhs=32, levels=3, blocks=[(4, 4), (2, 2)],
          n_vec=16, chiral=False, w_cycle=False, null_iters=6, pre=4, post=4, coarse_max_iter=20, coarse_tol=5e-2,
          tol=1e-10, max_iter=500, trunc=6)
MG2 = dict(L=256, beta=6.0, m=-0.05, r=1.0, csw=1.0, mu=0.0, seed=2025, nrhs=1, levels=2, blocks=[(4, 4)], n_vec=8,
           chiral=True, w_cycle=False, null_iters=2, pre=4, post=4, coarse_max_iter=50, coarse_tol=5e-2, tol=1e-10,
           max_iter=1000, trunc=20)
DSLASH = dict(L=512, nrhs=32, beta=6.0, m=-0.05, r=1.0, csw=1.0, mu=0.0, seed=20240)
CG = dict(L=32, beta=2.0, m=0.1, r=1.0, csw=1.0, mu=0.0, seed=31, tol=1e-10, max_iter=10000)
HMC = dict(L=128, beta=4.0, m=0.1, r=1.0, csw=1.0, seed=2024, rng_seed=4048, tau=1.0, n_outer=10, n_inner=4,
           tol=1e-10, n_traj=20)
BATCH = dict(n_lat=64, sizes=[64, 96, 128, 192, 256, 384], seed=5005, nrhs=8, r=1.0, csw=1.0, levels=2,
             blocks=[(4, 4)], n_vec=8, chiral=False, w_cycle=False, null_iters=4, pre=4, post=4, coarse_max_iter=10,
             coarse_tol=5e-2, tol=1e-10, max_iter=500, trunc=10, workers=8, smoother_half=True)


def batch_lattices(c):
    """The uneven batch: L from the size list, beta ~ U[2, 8], m ~ U[-0.05, 0.2], drawn from one seed."""
    rng = np.random.default_rng(c["seed"])
    out = []
    for i in range(c["n_lat"]):
        L = int(rng.choice(c["sizes"]))
        beta = float(rng.uniform(2.0, 8.0))
        m = float(rng.uniform(-0.05, 0.2))
        out.append((L, beta, m, c["seed"] + 1 + i))
    return out


def dslash_bytes_f32(L, nrhs):
    """Compulsory HBM bytes of one FP32 D application to nrhs right-hand sides:
    spinor in + out (2 x 16 B per site per rhs), 2 complex64 links (16 B) and
    the clover shift (4 B) per site."""
    return L * L * (32 * nrhs + 20)


def dslash_bytes_f16(L, nrhs):
    """Compulsory HBM bytes of one FP16-field D application: spinor in + out (2 x 8 B per site per
    rhs) plus the two per-site scales (8 B), 2 complex64 links (16 B), the clover shift (4 B)."""
    return L * L * (16 * nrhs + 28)


def dslash_bytes_f64_single(L):
    """13 x 8 B per site for one FP64 single-RHS application (in 32, out 32, links 32, clover 8)."""
    return L * L * 104


def sized(base: dict, args) -> dict:
    """A workload's configuration with the --L / --nrhs overrides (smaller cases for profiles)."""
    c = dict(base)
    if args.L:
        c["L"] = args.L
    if args.nrhs:
        c["nrhs"] = args.nrhs
    return c


def workload_config(workload: str, args) -> tuple[dict, dict]:
    """(parameters, the `config` object of the JSON line): the same for both arms of the benchmark."""
    if workload in ("mg", "mg2", "smoother", "coarse"):
        c = sized(MG2 if workload == "mg2" else MG, args)
        if args.trunc:
            c["trunc"] = args.trunc
        if args.coarse_iters:
            c["coarse_max_iter"] = args.coarse_iters
        c["smoother_half"] = args.smoother == "f16" and workload != "mg2"
        c["coarse_half"] = args.coarse_prec == "f16" and workload != "mg2"
        L, nrhs = c["L"], c["nrhs"]
        blk = ", ".join(f"{a}x{b}" for a, b in c["blocks"])
        vecs = f"{c['n_vec']} null vectors{' split by chirality' if c['chiral'] else ''}"
        name = (f"MG-GCR, L={L} (beta={c['beta']:g}, m={c['m']:g}, c_sw={c['csw']:g}), {nrhs} RHS, {c['levels']} levels "
                f"({blk}; {vecs}, {c['null_iters']} inverse iterations), {'W' if c['w_cycle'] else 'V'}-cycle, "
                f"{c['pre']}+{c['post']} MR steps, coarsest CG <= {c['coarse_max_iter']} iterations to "
                f"{c['coarse_tol']:g}, GCR truncation {c['trunc']}, true FP64 residual {c['tol']:g}")
        if workload == "smoother":
            name = f"fine smoother kernels of one MR step on FP16 work vectors, L={L}, {nrhs} RHS"
        if workload == "coarse":
            name = (f"level-1 coarse operator apply, {L // 4}x{L // 4} sites x {c['n_vec']} dof, {nrhs} RHS "
                    f"(L={L} fine, 4x4 aggregates)")
        cfg = {"workload": name, "L": L, "nrhs": nrhs, "levels": c["levels"], "aggregates": [list(b) for b in c["blocks"]],
               "null_vectors": c["n_vec"], "chiral_split": c["chiral"], "null_iters": c["null_iters"],
               "mr_steps": [c["pre"], c["post"]], "coarse_cg": [c["coarse_max_iter"], c["coarse_tol"]],
               "gcr_truncation": c["trunc"], "tol": c["tol"]}
        return c, cfg
    if workload == "dslash":
        c = sized(DSLASH, args)
        prec = args.dslash_prec
        name = (f"FP32 Wilson-clover D on {c['nrhs']} RHS, L={c['L']} (beta=6, m=-0.05, c_sw=1)" if prec == "f32"
                else f"Wilson-clover D on FP16 fields (per-site scales, FP32 arithmetic), {c['nrhs']} RHS, "
                     f"L={c['L']} (beta=6, m=-0.05, c_sw=1)")
        return c, {"workload": name, "L": c["L"], "nrhs": c["nrhs"], "precision": prec}
    if workload == "hmc":
        c = sized(HMC, args)
        name = (f"HMC, L={c['L']} (beta={c['beta']}, m={c['m']}, c_sw={c['csw']}), two flavours, tau={c['tau']}, "
                f"nested Omelyan: {c['n_outer']} fermion-force steps, {c['n_inner']} gauge-force substeps per inner "
                "integration, mixed-precision CG to a true FP64 residual of 1e-10")
        return c, {"workload": name, "L": c["L"], "trajectories": c["n_traj"]}
    if workload == "batch":
        c = dict(BATCH)
        c["smoother_half"] = args.smoother == "f16"
        if args.trunc:
            c["trunc"] = args.trunc
        if args.coarse_iters:
            c["coarse_max_iter"] = args.coarse_iters
        if args.nrhs:
            c["nrhs"] = args.nrhs
        if args.L:
            c["n_lat"] = args.L  # --L N: the first N lattices of the batch (a small case)
        if args.workers:
            c["workers"] = args.workers
        name = (f"uneven batch of {c['n_lat']} lattices (L in {c['sizes']}, beta~U[2,8], m~U[-0.05,0.2], c_sw=1), "
                f"{c['nrhs']} RHS each, 2-level MG (4x4, 8 null vectors), mixed FP32/FP64 GCR to a true FP64 "
                "residual of 1e-10, plus each lattice's pseudofermion force")
        return c, {"workload": name, "lattices": c["n_lat"], "rhs_per_lattice": c["nrhs"]}
    c = dict(CG)
    return c, {"workload": f"FP64 CG on D^dag D, L={c['L']} (beta={c['beta']:g}, m={c['m']:g}, c_sw={c['csw']:g}) "
                           f"to {c['tol']:g}", "L": c["L"]}


def mg_params(smg, c, precision):
    return smg.mg_params(c["levels"], c["blocks"][0][0], c["n_vec"], blocks=c["blocks"], chiral_split=c["chiral"],
                         null_iters=c["null_iters"], pre_smooth=c["pre"], post_smooth=c["post"], w_cycle=c["w_cycle"],
                         coarse_max_iter=c["coarse_max_iter"], coarse_tol=c["coarse_tol"], precision=precision,
                         seed=c["seed"], smoother_half=c.get("smoother_half", False) and precision == "f32",
                         coarse_half=c.get("coarse_half", False) and precision == "f32")


def kernel_trace(step, ctx, path: str, what: str) -> None:
    """One extra step under the CUPTI kernel tracer (schwinger_mg_gb300/profiling/kernel_trace.cpp):
    launches, device time and share per kernel, written as a table to `path`."""
    import shutil

    so = ROOT / "schwinger_mg_gb300" / "libsmg_ktrace.so"
    if not so.exists():
        from schwinger_mg_gb300.build import build_kernel_trace

        if build_kernel_trace() is None:
            raise RuntimeError("--kernel-trace needs CUPTI")
    kt = Cc.CDLL(str(so))
    ctx.synchronize()
    if kt.smg_ktrace_start() != 0:
        raise RuntimeError("CUPTI activity tracing could not start")
    step()
    ctx.synchronize()
    raw = path + ".raw"
    kt.smg_ktrace_stop(raw.encode())
    lines = Path(raw).read_text().splitlines()
    span = float(lines[0].split()[2])
    rows = [l.split(" ", 3) for l in lines[1:]]
    names = [r[3] for r in rows]
    if shutil.which("c++filt"):
        names = subprocess.run(["c++filt"], input="\n".join(names), capture_output=True, text=True).stdout.splitlines()
    agg = {}
    for r, nm in zip(rows, names):
        nm = nm.replace("(anonymous namespace)::", "")
        key = nm.split("(")[0] if "<" not in nm.split("(")[0] else nm[: nm.find(">(") + 1] if ">(" in nm else nm
        key = (key, r[2])
        n, t = agg.get(key, (0, 0.0))
        agg[key] = (n + int(r[0]), t + float(r[1]))
    tot = sum(t for _, t in agg.values())
    out = [f"# CUPTI kernel trace: {what}", f"# kernel time {tot / 1e6:.2f} ms, span {span / 1e6:.2f} ms", "",
           "| launches | total ms | avg us | share | kernel | grid |", "|---:|---:|---:|---:|---|---|"]
    for (k, grid), (n, t) in sorted(agg.items(), key=lambda kv: -kv[1][1]):
        out.append(f"| {n} | {t / 1e6:.2f} | {t / n / 1e3:.1f} | {100 * t / tot:.1f}% | `{k}` | {grid} |")
    Path(path).write_text("\n".join(out) + "\n")


# DRAM read + write bytes per launch at L = 512, 32 RHS, from one ncu capture each
# (profiles/coarse_apply_tc_L512_level1_32rhs.md, profiles/dslash_f32_L512_32rhs.md,
# profiles/smoother_f16_L512_32rhs.md)
TC_LEVEL1_L512_DRAM_BYTES = 226.540288e6 + 42.035968e6
DSLASH_F32_L512_DRAM_BYTES = 140.034048e6 + 98.370048e6
SMOOTHER_D_L512_DRAM_BYTES = 74.627072e6 + 31.32672e6
# the persistent coarsest CG of the same workload (one solve of 20 iterations): ncu dram read + write and
# lts__t_bytes (profiles/coarsest_cg_tc_L512_64x64_32rhs.md)
CCG_L512_DRAM_BYTES = 338.875904e6 + 417.792768e6
CCG_L512_L2_BYTES = 5.71516448e9


def coarse_kernel_name(c, L, nrhs):
    lc = L // c["blocks"][0][0]
    if nrhs % 32 == 0 and lc % 8 == 0:
        return f"k_coarse_apply_tc<0> (tcgen05 BF16, level 1, {lc}x{lc}x16, {nrhs} RHS)"
    return f"k_coarse_apply_tiled<float,0,16> (level 1, {lc}x{lc}x16, {nrhs} RHS)"


def smoother_times(smg, lib, ctx, mg32, lat, B, reps=20):
    """The fine smoother's three kernels on the hierarchy's FP16 work vectors (smg_mg_time_smoother)."""
    f32 = smg.Field(lat, B.shape[0], "f32", ctx, data=B)
    ms, by = (Cc.c_double * 4)(), (Cc.c_double * 4)()
    smg._lib.check(lib.smg_mg_time_smoother(mg32.h, f32.h, reps, ms, by), "smg_mg_time_smoother", ctx.h)
    names = ["k_dslash_h32<D, fused ||t||^2> (FP16 in/out, 32 RHS)",
             "k_dslash_h32<D^dag, fused ||Ar||^2> (+ 2 kernels finishing the MR scalars)",
             "k_mr_rupdate_h (r' = r - omega Ar, FP16)", "k_mr_xupdate_h (x += sum_k omega_k r_k, one per smoothing)"]
    return [{"kernel": n, "ms_per_launch": ms[k], "bytes_per_launch": by[k],
             "achieved_gbs": by[k] / (ms[k] * 1e-3) / 1e9} for k, n in enumerate(names)]


def run_ours(args, ws, rank, local):
    import torch

    import schwinger_mg_gb300 as smg

    torch.cuda.set_device(local)
    ctx = smg.Context(local)
    lib = smg.lib()
    SAMPLER.start(local)  # clock sampling from before any set-up or timed work
    peak, peak_kind = peaks()
    c, cfg = workload_config(args.workload, args)
    out = {"metric": METRIC, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "scaling": "weak",
           "vs_baseline": None, "data": "synthetic (seeded theta ~ N(0,1/beta) links, Gaussian complex sources)",
           "config": cfg}

    def timed(step, n):
        """Device milliseconds per step on the library's stream, max over ranks."""
        ctx.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        ctx.timer_begin()
        for _ in range(n):
            step()
        ms = ctx.timer_end() / n
        return max_over_ranks(ms, ws)

    def pinned_io(B):
        host_in = torch.empty(B.size * 2, dtype=torch.float64).pin_memory()
        host_in.numpy()[:] = B.reshape(-1).view(np.float64)
        host_out = torch.empty_like(host_in).pin_memory()
        return host_in, host_out, Cc.cast(host_in.data_ptr(), DP), Cc.cast(host_out.data_ptr(), DP)

    if args.workload in ("mg", "mg2"):
        L, nrhs = c["L"], c["nrhs"]
        U = smg.gauge_normal(L, c["beta"], c["seed"])
        lat = smg.Lattice(L)
        g = smg.GaugeField(lat, U, ctx)
        D = smg.DiracOp(lat, g, c["m"], c["r"], c["csw"], c["mu"])
        t0 = time.perf_counter()
        mg32 = smg.MGHierarchy(D, mg_params(smg, c, "f32"))
        ctx.synchronize()
        setup_s = time.perf_counter() - t0
        B = np.stack([smg.random_vec(lat.ndof, c["seed"] + 1 + j) for j in range(nrhs)])
        fb = smg.Field(lat, nrhs, "f64", ctx, data=B)
        fx = smg.Field(lat, nrhs, "f64", ctx)
        res = smg._lib.SolveResult()

        def solve(mg, b, x):
            st = lib.smg_gcr_solve(D.h, mg.h, b.h, x.h, c["max_iter"], c["tol"], c["trunc"], 0, Cc.byref(res))
            smg._lib.check(st, "smg_gcr_solve", ctx.h)

        step = lambda: solve(mg32, fb, fx)  # noqa: E731
        for _ in range(args.warmup):
            step()
        l0 = ctx.kernel_launches
        with Clocks(local) as clk:
            ms = timed(step, args.steps)
        launches = (ctx.kernel_launches - l0) // args.steps
        iters, true_res = res.iterations, res.true_residual
        value = ws * nrhs / (ms * 1e-3)

        # end to end through the C ABI: pinned host rhs in, solve, solutions out, every timed step
        host_in, host_out, pin, pout = pinned_io(B)

        def e2e_step():
            smg._lib.check(lib.smg_field_upload_async(fb.h, pin), "upload", ctx.h)
            step()
            smg._lib.check(lib.smg_field_download_async(fx.h, pout), "download", ctx.h)

        e2e_step()
        e2e_ms = timed(e2e_step, args.steps)
        sol = host_out.numpy().view(np.complex128).reshape(nrhs, -1)
        hb = B.size * 16

        # plain FP64 single-RHS MG on the same inputs (the comparison point of the mixed batched solve)
        mg64 = smg.MGHierarchy(D, mg_params(smg, c, "f64"))
        b1 = smg.Field(lat, 1, "f64", ctx, data=B[0])
        x1 = smg.Field(lat, 1, "f64", ctx)
        solve(mg64, b1, x1)
        ms64 = timed(lambda: solve(mg64, b1, x1), 2)
        it64, res64 = res.iterations, res.true_residual
        detail = {"gcr_iterations": iters, "true_residual": true_res, "setup_s": setup_s,
                  "smoother_work_vectors": "FP16, per-site scales" if c["smoother_half"] and nrhs >= 8 else "FP32",
                  "coarse_work_vectors": ("FP16, scales per coarse site and rhs half (coarsest CG, level-1 MR)"
                                          if c["coarse_half"] and nrhs == 32 else "FP32"),
                  "plain_fp64_mg_solves_per_s": 1e3 / ms64, "plain_fp64_mg_iterations": it64,
                  "plain_fp64_mg_true_residual": res64, "mixed_batched_over_plain_fp64": value / ws / (1e3 / ms64),
                  "launches_before_timed": int(l0)}
        kernels = []
        # the coarse-operator apply at level 1, timed alone
        cms, cbytes = Cc.c_double(), Cc.c_double()
        smg._lib.check(lib.smg_mg_time_coarse_apply(mg32.h, 1, nrhs, 20, Cc.byref(cms), Cc.byref(cbytes)),
                       "smg_mg_time_coarse_apply", ctx.h)
        kernels.append({"kernel": coarse_kernel_name(c, L, nrhs), "ms_per_launch": cms.value,
                        "bytes_per_launch": cbytes.value, "achieved_gbs": cbytes.value / (cms.value * 1e-3) / 1e9,
                        "traffic": TC_LEVEL1_L512_DRAM_BYTES if (L, nrhs) == (512, 32) else None})
        # fine operator: FP32 D on the workload's right-hand sides
        f32s = smg.Field(lat, nrhs, "f32", ctx, data=B)
        f32d = smg.Field(lat, nrhs, "f32", ctx)
        dms = timed(lambda: smg._lib.check(lib.smg_dirac_apply(D.h, 0, f32s.h, f32d.h), "dirac", ctx.h), 20)
        dgbs = dslash_bytes_f32(L, nrhs) / (dms * 1e-3) / 1e9
        kernels.append({"kernel": f"k_dslash<float> (FP32 D, {nrhs} RHS)", "ms_per_launch": dms,
                        "bytes_per_launch": dslash_bytes_f32(L, nrhs), "achieved_gbs": dgbs,
                        "traffic": DSLASH_F32_L512_DRAM_BYTES if (L, nrhs) == (512, 32) else None})
        detail["fine_dslash_f32_gbs"] = dgbs
        detail["fine_dslash_frac_of_hbm"] = dgbs / peak
        if c["smoother_half"] and nrhs >= 8:
            sm = smoother_times(smg, lib, ctx, mg32, lat, B)
            sm[0]["traffic"] = SMOOTHER_D_L512_DRAM_BYTES if (L, nrhs) == (512, 32) else None
            kernels = sm + kernels
        # the coarsest solve of a cycle: with FP16 coarse vectors at 32 RHS one cooperative launch
        # (k_ccg_tc), L2-resident, so no HBM roofline applies; its DRAM and L2 traffic are from ncu
        sms, sit = Cc.c_double(), Cc.c_int()
        smg._lib.check(lib.smg_mg_time_coarse_solve(mg32.h, 10, Cc.byref(sms), Cc.byref(sit)),
                       "smg_mg_time_coarse_solve", ctx.h)
        ccg = {"kernel": "coarsest CG (k_ccg_tc: one cooperative launch per solve)" if sit.value >= 0
               else "coarsest CG (per-iteration kernels)", "ms_per_solve": sms.value,
               "iterations": sit.value if sit.value >= 0 else None, "bound": "L2 / latency"}
        if (L, nrhs) == (512, 32) and sit.value >= 0:
            ccg["dram_bytes_per_solve"] = CCG_L512_DRAM_BYTES
            ccg["l2_bytes_per_solve"] = CCG_L512_L2_BYTES
        detail["coarsest_solve"] = ccg
        # the step's largest kernel (profiles/mg_gcr_L512_32rhs_kernel_shares.md): the FP16 stencil with the
        # fused MR reductions when the smoother runs on FP16 work vectors, else the level-1 coarse apply
        top = next((k for k in kernels if "fused" in k["kernel"]), kernels[0])
        for k in kernels:
            k["frac_of_hbm"] = k["achieved_gbs"] / peak
        detail["kernels"] = kernels
        detail["l2"] = (f"fine fields of {nrhs} RHS ({16 * L * L * nrhs / 1e6:.0f} MB FP32) "
                        f"{'exceed' if 16 * L * L * nrhs > 129e6 else 'fit in'} the 129 MB L2; no flush")
        # the untimed traced step comes after every timed region: CUPTI stays attached once enabled
        if args.kernel_trace and rank == 0:
            kernel_trace(step, ctx, args.kernel_trace, f"one step of the {args.workload} workload (L={L}, {nrhs} RHS, "
                                                       f"{iters} GCR iterations)")
        out.update({
            "value": value, "unit": "solves/s", "ms_per_step": ms, "higher_is_better": True, "dtype": "f32+f16+f64",
            "detail": detail,
            "e2e": {"value": ws * nrhs / (e2e_ms * 1e-3), "unit": "solves/s", "h2d_bytes_per_step": hb,
                    "d2h_bytes_per_step": hb, "ms_per_step": e2e_ms, "timed_steps": args.steps,
                    "finite": bool(np.isfinite(sol).all())},
            "roofline": {"bound": "hbm", "achieved": top["achieved_gbs"], "peak": peak, "unit": "GB/s",
                         "frac": top["achieved_gbs"] / peak, "traffic": top.get("traffic"),
                         "traffic_unit": "bytes per launch (ncu dram read + write)", "kernel": top["kernel"],
                         "bytes_per_launch": top["bytes_per_launch"], "ms_per_launch": top["ms_per_launch"],
                         "peak_source": peak_kind},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
        })
    elif args.workload == "smoother":
        L, nrhs = c["L"], c["nrhs"]
        U = smg.gauge_normal(L, c["beta"], c["seed"])
        lat = smg.Lattice(L)
        D = smg.DiracOp(lat, smg.GaugeField(lat, U, ctx), c["m"], c["r"], c["csw"], c["mu"])
        mg32 = smg.MGHierarchy(D, mg_params(smg, c, "f32"))
        B = np.stack([smg.random_vec(lat.ndof, c["seed"] + 1 + j) for j in range(nrhs)])
        l0 = ctx.kernel_launches
        with Clocks(local) as clk:
            ks = smoother_times(smg, lib, ctx, mg32, lat, B, reps=max(args.steps, 50))
        launches = ctx.kernel_launches - l0
        top = ks[0]
        top["traffic"] = SMOOTHER_D_L512_DRAM_BYTES if (L, nrhs) == (512, 32) else None
        for k in ks:
            k["frac_of_hbm"] = k["achieved_gbs"] / peak
        out.update({
            "value": ws * top["achieved_gbs"], "unit": "GB/s", "ms_per_step": top["ms_per_launch"],
            "higher_is_better": True, "dtype": "f16 storage, f32 arithmetic",
            "detail": {"kernels": ks, "l2": "FP16 fields of 32 RHS (67 MB each) with their neighbours exceed L2"},
            "e2e": None,
            "roofline": {"bound": "hbm", "achieved": top["achieved_gbs"], "peak": peak, "unit": "GB/s",
                         "frac": top["achieved_gbs"] / peak, "traffic": top["traffic"], "kernel": top["kernel"],
                         "bytes_per_launch": top["bytes_per_launch"], "peak_source": peak_kind},
            "gpu_launches": int(launches), "clocks": clk.summary(),
        })
    elif args.workload == "dslash":
        L, nrhs = c["L"], c["nrhs"]
        U = smg.gauge_normal(L, c["beta"], c["seed"])
        lat = smg.Lattice(L)
        g = smg.GaugeField(lat, U, ctx)
        D = smg.DiracOp(lat, g, c["m"], c["r"], c["csw"], c["mu"])
        srcs = np.stack([smg.random_vec(lat.ndof, c["seed"] + 1 + j) for j in range(nrhs)])
        prec = args.dslash_prec
        fs = smg.Field(lat, nrhs, prec, ctx, data=srcs)
        fd = smg.Field(lat, nrhs, prec, ctx)
        bytes_step = dslash_bytes_f32(L, nrhs) if prec == "f32" else dslash_bytes_f16(L, nrhs)

        def step():
            smg._lib.check(lib.smg_dirac_apply(D.h, 0, fs.h, fd.h), "dirac_apply", ctx.h)

        for _ in range(args.warmup):
            step()
        n_timed = max(args.steps, 500)
        l0 = ctx.kernel_launches
        with Clocks(local) as clk:
            ms = timed(step, n_timed)
        launches = (ctx.kernel_launches - l0) // n_timed
        value = ws * bytes_step / (ms * 1e-3) / 1e9
        achieved = bytes_step / (ms * 1e-3) / 1e9
        host_in, host_out, pin, pout = pinned_io(srcs)

        def e2e_step():
            smg._lib.check(lib.smg_field_upload_async(fs.h, pin), "upload", ctx.h)
            step()
            smg._lib.check(lib.smg_field_download_async(fd.h, pout), "download", ctx.h)

        e2e_step()
        e2e_ms = timed(e2e_step, args.steps)
        hb = srcs.size * 16
        out.update({
            "value": value, "unit": "GB/s", "ms_per_step": ms, "higher_is_better": True, "dtype": prec,
            "detail": {"bytes_per_step": bytes_step, "timed_steps": n_timed,
                       "l2": f"inputs and outputs ({bytes_step / 1e6:.0f} MB) exceed the 129 MB L2; no flush"},
            "e2e": {"value": ws * bytes_step / (e2e_ms * 1e-3) / 1e9, "unit": "GB/s",
                    "h2d_bytes_per_step": hb, "d2h_bytes_per_step": hb, "ms_per_step": e2e_ms},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": DSLASH_F32_L512_DRAM_BYTES if (L, nrhs, prec) == (512, 32, "f32") else None,
                         "traffic_unit": "bytes per launch (ncu, profiles/dslash_f32_L512_32rhs.md)",
                         "kernel": ("k_dslash<float,false,0,r=1> (autotuned row kernel)" if prec == "f32"
                                    else "k_dslash_h<false,true,true,r=1> (FP16 fields)"),
                         "peak_source": peak_kind},
            "gpu_launches": int(launches), "clocks": clk.summary(),
        })
    elif args.workload == "hmc":
        # differentiated HMC: nested Omelyan (fermion force outside, gauge force inside), mixed solves
        L = c["L"]
        U = smg.gauge_normal(L, c["beta"], c["seed"])
        lat = smg.Lattice(L)
        g = smg.GaugeField(lat, U, ctx)
        p = smg.hmc_params(c["beta"], tau=c["tau"], n_steps=c["n_outer"], omelyan=True, n_inner=c["n_inner"],
                           cg_tol=c["tol"], c_sw=c["csw"], mixed_precision=True)
        rng = smg.Rng(c["rng_seed"])
        results = []

        def step():
            results.append(smg.hmc_trajectory(g, c["m"], c["r"], p, rng))

        for _ in range(args.warmup):
            step()
        n_timed = max(args.steps, c["n_traj"] - args.warmup)
        l0 = ctx.kernel_launches
        with Clocks(local) as clk:
            ms = timed(step, n_timed)
        launches = (ctx.kernel_launches - l0) // n_timed
        acc = [r.accepted for r in results]
        out.update({
            "value": ws * 1e3 / ms, "unit": "trajectories/s", "ms_per_step": ms, "higher_is_better": True,
            "dtype": "f64+f32",
            "detail": {"trajectories": len(results), "timed_trajectories": n_timed,
                       "acceptance": float(np.mean(acc)),
                       "dH": [round(r.dH, 6) for r in results],
                       "mean_exp_minus_dH": float(np.mean([np.exp(-r.dH) for r in results])),
                       "plaquette": [round(r.plaquette, 6) for r in results],
                       "solves_per_trajectory": results[-1].solves,
                       "cg_iterations_per_trajectory": float(np.mean([r.total_cg_iters for r in results])),
                       "l2": "gauge, momenta and fields (a few MB) are L2-resident; no flush"},
            "e2e": {"value": ws * 1e3 / ms, "unit": "trajectories/s", "h2d_bytes_per_step": 12 * lat.V * 8,
                    "d2h_bytes_per_step": 0, "ms_per_step": ms,
                    "note": "the trajectory runs through the C ABI; its host inputs (momenta, eta) are copied in"},
            "gpu_launches": int(launches), "clocks": clk.summary(),
        })
    elif args.workload == "batch":
        # uneven multi-lattice batch: every lattice's RHS by mixed MG-GCR to 1e-10 plus its pseudofermion force
        lats_all = batch_lattices(c)
        lats = shard(lats_all, rank, ws)  # several GPUs: the 64 lattices are split across the ranks
        nrhs = c["nrhs"]
        batch = smg.LatticeBatch(n_workers=c["workers"], device=local)
        sources = []
        for i, (L, beta, m, gseed) in enumerate(lats):
            batch.add(L, smg.gauge_normal(L, beta, gseed), m, c_sw=c["csw"], wilson_r=c["r"], nrhs=nrhs)
            B = np.stack([smg.random_vec(2 * L * L, gseed * 100 + j) for j in range(nrhs)])
            sources.append(B)
        t0 = time.perf_counter()
        batch.setup(mg_params(smg, c, "f32"))
        setup_s = time.perf_counter() - t0
        for i, B in enumerate(sources):
            batch.bind(i, B)

        def step():
            st, sec = batch.solve(c["max_iter"], c["tol"], c["trunc"], with_force=True)
            smg._lib.check(st, "smg_batch_solve")
            return sec

        for _ in range(args.warmup):
            step()
        l0 = batch.kernel_launches
        if ws > 1:
            torch.distributed.barrier()
        with Clocks(local) as clk:
            torch.cuda.synchronize()
            secs = [step() for _ in range(args.steps)]
            torch.cuda.synchronize()
        launches = (batch.kernel_launches - l0) // args.steps
        ms = max_over_ranks(1e3 * float(np.mean(secs)), ws)
        n_solves = len(lats_all) * nrhs  # all ranks together
        worst_res, iters = 0.0, []
        for i in range(len(lats)):
            st, r, _ = batch.result(i)
            smg._lib.check(st, "batch lattice")
            worst_res = max(worst_res, r.true_residual)
            iters.append(r.iterations)
        # end to end: host right-hand sides in, solutions and forces out, inside the timed call
        host = []
        for i, (L, beta, m, gseed) in enumerate(lats):
            xin = torch.from_numpy(sources[i].reshape(-1).view(np.float64)).pin_memory()
            xo = torch.empty(nrhs * 4 * L * L, dtype=torch.float64).pin_memory()
            fo = torch.empty(2 * L * L, dtype=torch.float64).pin_memory()
            host.append((xin, xo, fo))
            smg._lib.check(lib.smg_batch_bind_host(batch.h, i, Cc.cast(xin.data_ptr(), DP), Cc.cast(xo.data_ptr(), DP),
                                                   Cc.cast(fo.data_ptr(), DP)), "bind")
        st, _ = batch.solve(c["max_iter"], c["tol"], c["trunc"], with_force=True, host_io=True)
        smg._lib.check(st, "batch e2e")
        e2e_secs = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            st, sec = batch.solve(c["max_iter"], c["tol"], c["trunc"], with_force=True, host_io=True)
            smg._lib.check(st, "batch e2e")
            e2e_secs.append(sec)
        e2e_ms = max_over_ranks(1e3 * float(np.mean(e2e_secs)), ws)
        hb = sum(B.size * 16 for B in sources)
        db = hb + sum(2 * L * L * 8 for (L, _, _, _) in lats)
        # roofline kernel: FP32 D of the largest lattice on its 8 RHS, timed alone; one field of that size
        # fits in L2, so the launches rotate over enough source/destination pairs that together exceed it
        Lmax = max(L for (L, _, _, _) in lats)
        jmax = [L for (L, _, _, _) in lats].index(Lmax)
        latm = smg.Lattice(Lmax)
        Dm = smg.DiracOp(latm, smg.GaugeField(latm, smg.gauge_normal(Lmax, lats[jmax][1], lats[jmax][3]), ctx),
                         lats[jmax][2], c["r"], c["csw"], 0.0)
        field_bytes = 16 * Lmax * Lmax * nrhs
        nfields = max(2, int(np.ceil(2 * 129e6 / (2 * field_bytes))))
        f32s = [smg.Field(latm, nrhs, "f32", ctx, data=sources[jmax]) for _ in range(nfields)]
        f32d = [smg.Field(latm, nrhs, "f32", ctx) for _ in range(nfields)]
        turn = [0]

        def dstep():
            i = turn[0] % nfields
            turn[0] += 1
            smg._lib.check(lib.smg_dirac_apply(Dm.h, 0, f32s[i].h, f32d[i].h), "dirac", ctx.h)

        for _ in range(nfields):
            dstep()
        dms = timed(dstep, 10 * nfields)
        dgbs = dslash_bytes_f32(Lmax, nrhs) / (dms * 1e-3) / 1e9
        if args.kernel_trace and rank == 0:  # untimed, after the timed regions (CUPTI stays attached)
            kernel_trace(step, ctx, args.kernel_trace, f"one step of the batch workload ({len(lats)} lattices, "
                                                       f"{nrhs} RHS each)")
        sizes = {}
        for (L, _, _, _) in lats:
            sizes[L] = sizes.get(L, 0) + 1
        out.update({
            "value": n_solves / (ms * 1e-3), "unit": "solves/s", "ms_per_step": ms, "higher_is_better": True,
            "dtype": "f32+f16+f64", "scaling": "strong",
            "detail": {"lattices_rank0": len(lats), "sizes_rank0": sizes,
                       "smoother_work_vectors": "FP16, per-site scales" if c["smoother_half"] else "FP32",
                       "coarsest_cg_iterations": c["coarse_max_iter"],
                       "sites_total": int(sum(L * L for (L, _, _, _) in lats)),
                       "worst_true_residual": max_over_ranks(worst_res, ws),
                       "gcr_iterations_min_max": [min(iters), max(iters)],
                       "host_workers": c["workers"], "setup_s": setup_s,
                       "timing": "wall time of smg_batch_solve between device synchronisations (one stream per "
                                 "lattice, so no single stream brackets the work)",
                       "l2": "the batch's fields (several GB) exceed the 129 MB L2; no flush"},
            "e2e": {"value": n_solves / (e2e_ms * 1e-3), "unit": "solves/s", "h2d_bytes_per_step": hb,
                    "d2h_bytes_per_step": db, "ms_per_step": e2e_ms},
            "roofline": {"bound": "hbm", "achieved": dgbs, "peak": peak, "unit": "GB/s", "frac": dgbs / peak,
                         "traffic": None, "kernel": f"FP32 D (autotuned launch shape), L={Lmax}, {nrhs} RHS",
                         "ms_per_launch": dms, "peak_source": peak_kind,
                         "l2": f"launches rotate over {nfields} field pairs ({2 * nfields * field_bytes / 1e6:.0f} MB)"},
            "gpu_launches": int(launches), "clocks": clk.summary(),
        })
        batch.close()
    elif args.workload == "coarse":
        # the level-1 coarse operator alone: (L/4)^2 sites, 16 dofs, 32 RHS, 9-point stencil
        L, nrhs = c["L"], c["nrhs"]
        U = smg.gauge_normal(L, c["beta"], c["seed"])
        lat = smg.Lattice(L)
        g = smg.GaugeField(lat, U, ctx)
        D = smg.DiracOp(lat, g, c["m"], c["r"], c["csw"], c["mu"])
        mg32 = smg.MGHierarchy(D, mg_params(smg, c, "f32"))
        cms, cbytes = Cc.c_double(), Cc.c_double()
        reps = max(args.steps, 200)
        l0 = ctx.kernel_launches
        with Clocks(local) as clk:
            smg._lib.check(lib.smg_mg_time_coarse_apply(mg32.h, 1, nrhs, reps, Cc.byref(cms), Cc.byref(cbytes)),
                           "smg_mg_time_coarse_apply", ctx.h)
        launches = (ctx.kernel_launches - l0) // 2  # warm-up pass + timed pass
        gbs = cbytes.value / (cms.value * 1e-3) / 1e9
        out.update({
            "value": gbs * ws, "unit": "GB/s", "ms_per_step": cms.value, "higher_is_better": True, "dtype": "f32",
            "detail": {"bytes_per_launch": cbytes.value, "timed_launches": reps,
                       "l2": "links and vectors exceed the 129 MB L2 at L=512; no flush"},
            "e2e": None,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "traffic": TC_LEVEL1_L512_DRAM_BYTES if (L, nrhs) == (512, 32) else None,
                         "traffic_unit": "bytes per launch (ncu)", "kernel": coarse_kernel_name(c, L, nrhs),
                         "bytes_per_launch": cbytes.value, "peak_source": peak_kind},
            "gpu_launches": int(launches), "clocks": clk.summary(),
        })
    else:
        L = c["L"]
        U = smg.gauge_normal(L, c["beta"], c["seed"])
        lat = smg.Lattice(L)
        g = smg.GaugeField(lat, U, ctx)
        D = smg.DiracOp(lat, g, c["m"], c["r"], c["csw"], c["mu"])
        b = smg.random_vec(lat.ndof, c["seed"] + 1)
        fb = smg.Field(lat, 1, "f64", ctx, data=b)
        fx = smg.Field(lat, 1, "f64", ctx)
        res = smg._lib.SolveResult()

        def step():
            smg._lib.check(lib.smg_cg_solve(D.h, fb.h, fx.h, c["max_iter"], c["tol"], Cc.byref(res)), "cg", ctx.h)

        for _ in range(args.warmup):
            step()
        l0 = ctx.kernel_launches
        with Clocks(local) as clk:
            ms = timed(step, args.steps)
        launches = (ctx.kernel_launches - l0) // args.steps
        bh = b.copy()
        xh = np.empty_like(bh)
        pb, px = bh.view(np.float64).ctypes.data_as(DP), xh.view(np.float64).ctypes.data_as(DP)

        def e2e_step():
            smg._lib.check(lib.smg_field_upload(fb.h, pb), "upload", ctx.h)
            step()
            smg._lib.check(lib.smg_field_download(fx.h, px), "download", ctx.h)

        e2e_ms = timed(e2e_step, args.steps)
        out.update({"value": ws * 1e3 / ms, "unit": "solves/s", "ms_per_step": ms, "higher_is_better": True,
                    "dtype": "f64",
                    "detail": {"iterations": res.iterations, "true_residual": res.true_residual,
                               "l2": "working set is L2-resident within a solve"},
                    "e2e": {"value": ws * 1e3 / e2e_ms, "unit": "solves/s", "h2d_bytes_per_step": bh.nbytes,
                            "d2h_bytes_per_step": xh.nbytes, "ms_per_step": e2e_ms},
                    "gpu_launches": int(launches), "clocks": clk.summary()})
    if rank == 0 and not args.no_cpu_baseline and args.workload not in ("coarse", "smoother"):
        base = cpu_reference(args.workload, c, steps=1, warmup=0)
        out["cpu_baseline"] = {k: base[k] for k in ("value", "unit", "cores", "kind", "sample", "seconds")}
    return out


# ------------------------------------------------------------------ the reference's CPU path
def cpu_reference(workload: str, c: dict, steps: int, warmup: int, threads: int | None = None) -> dict:
    """The reference's CPU path for `workload` on this host's cores: the oracle's C restatement
    (oracle/smg_oracle.c), which makes its own seeded inputs (oracle/inputs.cpp) and builds its own
    hierarchy on the CPU; nothing of the GPU library is used.  Times `steps` bounded samples after
    `warmup` untimed ones; returns value, unit, ms_per_step and a description of the sample."""
    from oracle import oracle as O

    port = O.port()
    n_threads = threads or os.cpu_count() or 1
    port.set_threads(n_threads)
    if workload in ("mg", "mg2"):
        L = c["L"]
        U = port.gauge_normal(L, c["beta"], c["seed"])
        nl = c["levels"] - 1
        t0 = time.perf_counter()
        bvs, links, _ = port.mgN_setup(L, U, c["m"], c["r"], c["csw"], c["mu"], c["blocks"][:nl], [c["n_vec"]] * nl,
                                       c["null_iters"], c["seed"], chiral_split=c["chiral"])
        setup_s = time.perf_counter() - t0
        ncs = [2 * c["n_vec"] if c["chiral"] else c["n_vec"]] * nl
        p = port.mgN_params(L, c["m"], c["r"], c["csw"], c["mu"], c["blocks"][:nl], ncs, bvs, links, c["pre"],
                            c["post"], c["w_cycle"], c["coarse_max_iter"], c["coarse_tol"])
        secs, its, ress = [], [], []
        for i in range(warmup + steps):
            b = port.random_vec(2 * L * L, c["seed"] + 1 + (i % c["nrhs"]))
            _, it, res, sec = port.mgN_gcr(p, U, b, c["max_iter"], c["tol"], c["trunc"])
            if i >= warmup:
                secs.append(sec)
                its.append(it)
                ress.append(res)
        sec = float(np.mean(secs))
        return {"value": 1.0 / sec, "unit": "solves/s", "ms_per_step": 1e3 * sec, "cores": n_threads, "kind": "port",
                "sample": f"{len(secs)} one-RHS FP64 solve(s) of the workload's right-hand sides (the reference "
                          f"solves one at a time) on a hierarchy built on the CPU in {setup_s:.1f} s: GCR iterations "
                          f"{its}, final residuals {max(ress):.1e}, {sec:.2f} s per solve",
                "seconds": float(np.sum(secs)), "iterations": its, "setup_s": setup_s}
    if workload in ("dslash", "smoother", "coarse"):
        cc = DSLASH
        L, nrhs = cc["L"], 8
        U = port.gauge_normal(L, cc["beta"], cc["seed"])
        srcs = np.stack([port.random_vec(2 * L * L, cc["seed"] + 1 + j) for j in range(nrhs)])
        t1, _ = port.time_dirac(U, cc["m"], cc["r"], cc["csw"], cc["mu"], 0, srcs[:1], 1)
        reps = max(2, int(10.0 / max(t1 * nrhs, 1e-6)))  # about 10 s of CPU work per step
        ts = []
        for i in range(warmup + steps):
            t, _ = port.time_dirac(U, cc["m"], cc["r"], cc["csw"], cc["mu"], 0, srcs, reps)
            if i >= warmup:
                ts.append(t)
        t = float(np.mean(ts))
        gbs = reps * nrhs * dslash_bytes_f64_single(L) / t / 1e9
        return {"value": gbs, "unit": "GB/s", "ms_per_step": 1e3 * t, "cores": n_threads, "kind": "port",
                "sample": f"FP64 D on {nrhs} RHS x {reps} reps at L={L} per step (the reference computes one RHS at "
                          "a time in FP64; 104 B/site per application)", "seconds": float(np.sum(ts))}
    if workload == "batch":
        # one right-hand side of one sampled lattice (L = 128) through a 2-level hierarchy of the batch's
        # parameters built on the CPU, scaled to the whole batch by site count
        lats = batch_lattices(c)
        L, beta, m, gseed = next(t for t in lats if t[0] == 128)
        U = port.gauge_normal(L, beta, gseed)
        bvs, links, _ = port.mgN_setup(L, U, m, c["r"], c["csw"], 0.0, c["blocks"], [c["n_vec"]], c["null_iters"],
                                       c["seed"])
        p = port.mgN_params(L, m, c["r"], c["csw"], 0.0, c["blocks"], [c["n_vec"]], bvs, links, c["pre"], c["post"],
                            c["w_cycle"], c["coarse_max_iter"], c["coarse_tol"])
        secs, its = [], []
        for i in range(warmup + steps):
            b = port.random_vec(2 * L * L, gseed * 100 + (i % c["nrhs"]))
            _, it, res, sec = port.mgN_gcr(p, U, b, c["max_iter"], c["tol"], c["trunc"])
            if i >= warmup:
                secs.append(sec)
                its.append(it)
        sec = float(np.mean(secs))
        total_sites = sum(t[0] ** 2 for t in lats)
        est = sec * c["nrhs"] * total_sites / (L * L)
        return {"value": c["n_lat"] * c["nrhs"] / est, "unit": "solves/s", "ms_per_step": 1e3 * est, "cores": n_threads,
                "kind": "port",
                "sample": f"one-RHS solves of an L={L} lattice of the batch (GCR iterations {its}, {sec:.2f} s each), "
                          f"scaled by site count to the {c['n_lat']} x {c['nrhs']} solves (forces excluded)",
                "seconds": float(np.sum(secs))}
    if workload == "hmc":
        # one fermion-force evaluation (CG to 1e-10 + force) and one gauge force on the CPU; a nested
        # Omelyan trajectory makes 2 n_outer + 1 of them plus the two Hamiltonian solves
        L = c["L"]
        U = port.gauge_normal(L, c["beta"], c["seed"]).reshape(-1)
        phi = port.random_vec(2 * L * L, c["seed"] + 7)
        ts = []
        for i in range(warmup + steps):
            t0 = time.perf_counter()
            X, it, _ = port.cg(U, c["m"], c["r"], c["csw"], 0.0, phi, 100000, c["tol"])
            port.fermion_force(U, c["m"], c["r"], c["csw"], 0.0, X)
            port.gauge_force(U, c["beta"])
            if i >= warmup:
                ts.append(time.perf_counter() - t0)
        t_force = float(np.mean(ts))
        n_solves = 2 * c["n_outer"] + 3
        return {"value": 1.0 / (n_solves * t_force), "unit": "trajectories/s", "ms_per_step": 1e3 * n_solves * t_force,
                "cores": n_threads, "kind": "port",
                "sample": f"force evaluations at L={L} (FP64 CG, {it} iterations, to 1e-10, fermion + gauge force) "
                          f"in {t_force:.2f} s each, times the {n_solves} solves of one trajectory",
                "seconds": float(np.sum(ts))}
    U = port.gauge_normal(c["L"], c["beta"], c["seed"])
    b = port.random_vec(2 * c["L"] ** 2, c["seed"] + 1)
    ts, it = [], 0
    for i in range(warmup + steps):
        reps, tot = 0, 0.0
        while tot < 2.0 and reps < 100:
            t, _, it = port.time_cg(U, c["m"], c["r"], c["csw"], c["mu"], b, c["max_iter"], c["tol"])
            tot += t
            reps += 1
        if i >= warmup:
            ts.append(tot / reps)
    t = float(np.mean(ts))
    return {"value": 1.0 / t, "unit": "solves/s", "ms_per_step": 1e3 * t, "cores": n_threads, "kind": "port",
            "sample": f"FP64 CG solves at L={c['L']} ({it} iterations each), about 2 s of repeats per step",
            "seconds": float(np.sum(ts))}


def run_reference(args, ws, rank):
    """The reference's CPU path on every host core, same workload, metric and config as the GPU arm.
    Bounded: at most 5 timed steps after at most 1 warm-up (each MG step is one full solve)."""
    if rank != 0:
        return None
    c, cfg = workload_config(args.workload, args)
    steps, warmup = max(1, min(args.steps, 5)), min(args.warmup, 1)
    base = cpu_reference(args.workload, c, steps=steps, warmup=warmup)
    val = base["value"]
    return {"metric": METRIC, "impl": "reference", "value": val, "unit": base["unit"], "n_gpus": ws,
            "steps": steps, "warmup": warmup, "ms_per_step": base["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": cfg,
            "cpu_baseline": {"kind": base["kind"], "cores": base["cores"], "sample": base["sample"], "value": val},
            "e2e": {"value": val, "unit": base["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}


def relaunch_distributed(n: int) -> int:
    """`--gpus N` outside torchrun: run this script under torch.distributed.run with N ranks on this node."""
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr=127.0.0.1", f"--master-port={port}", str(Path(__file__).resolve()), *sys.argv[1:]]
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="mg",
                    choices=["mg", "mg2", "dslash", "smoother", "cg", "coarse", "hmc", "batch"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--L", type=int, default=0, help="lattice size override (smaller cases for profiles)")
    ap.add_argument("--nrhs", type=int, default=0, help="right-hand-side count override")
    ap.add_argument("--smoother", default="f16", choices=["f32", "f16"],
                    help="mg workload: precision of the fine smoother's work vectors (f16: per-site scaled FP16)")
    ap.add_argument("--coarse-prec", default="f16", choices=["f32", "f16"],
                    help="mg workload: precision of the coarsest CG's residual and search direction (f16: per-site "
                         "scaled FP16)")
    ap.add_argument("--trunc", type=int, default=0, help="mg / batch workloads: GCR truncation override")
    ap.add_argument("--coarse-iters", type=int, default=0, help="mg / batch workloads: coarsest-CG iteration cap override")
    ap.add_argument("--workers", type=int, default=0, help="batch workload: host worker threads override")
    ap.add_argument("--dslash-prec", default="f32", choices=["f32", "f16"],
                    help="dslash workload: field precision (f16 = FP16 storage with per-site scales)")
    ap.add_argument("--kernel-trace", default="", help="mg and batch workloads: write a CUPTI per-kernel summary of "
                                                         "one extra (untimed) step to this path")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        sys.exit(relaunch_distributed(args.gpus))
    ws, rank, local = dist_env()
    if ws != args.gpus:
        raise SystemExit(f"--gpus {args.gpus} but WORLD_SIZE={ws}: launch one rank per GPU")
    if args.impl == "reference":
        line = run_reference(args, ws, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if ws > 1:
        import torch

        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    line = run_ours(args, ws, rank, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
