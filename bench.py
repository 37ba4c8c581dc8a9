#!/usr/bin/env python3
"""Benchmark of the exact-diagonalisation hot path (one JSON line on stdout).

Workload (the batched multi-sector grid): 1D periodic Bose-Hubbard chain,
m = 10 sites, particle-number sectors n = 8..12 (D = 24,310 / 48,620 /
92,378 / 167,960 / 293,930), 64 hopping values J_b = 0.3 (b + 1) / 64 with
U = 1, the 10 lowest eigenvalues of each (J, n) point = 320 eigensolves per
step, then the 64-point mu grid on [0, 3] applied as the -mu n shift to
compose the density / compressibility map on the device.  One step = that
whole grid.  Inputs are synthetic by construction (the Hamiltonian is
determined by (m, n, J, U)); the seeded start block is Spectra's
SimpleRandom stream.

Our arm: batched mixed-precision solver (FP32 Krylov vectors and SpMM, FP64
coefficients / tridiagonal solve / final Rayleigh-Ritz) through the C ABI; one
call (bh_eigsh_batch_sectors) solves the five sectors, which run concurrently
on the device.
  value        eigensolves/s with the sector Hamiltonians resident in HBM
  e2e          the same through the public API from host arrays: device basis
               + Hamiltonian build, batched solve, phase map, results to host
  plain_fp64   the plain FP64 single-point path (one solve per call) on a
               sample of the grid, for the batched-vs-plain ratio
  accuracy     max relative eigenvalue error of the mixed results vs FP64
  roofline     dominant kernel, algorithmic bytes / CUDA-event duration
  whole_solver every kernel's algorithmic bytes of one step over the summed
               kernel time and over the step time
  spmm_gather  the sparse product against the bytes it must gather
  cpu_baseline the CPU oracle's restatement of the reference's IRLM
               (OpenMP over points) on a bounded sample of the grid
Reference arm (--impl reference): the CPU restatement alone, timed per step
on a bounded sample, on all host cores (the reference's own compiled code is
x86-only here and cannot run on the GPU host).
"""
from __future__ import annotations

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
M = 10
SECTORS = [8, 9, 10, 11, 12]
NJ = 64
JS = 0.3 * (np.arange(NJ) + 1) / NJ
U = 1.0
NEV = 10
MU = np.linspace(0.0, 3.0, 64)
WORKLOAD_NAME = ("1D periodic Bose-Hubbard chain m=10, sectors n=8..12 (D=24310..293930), "
                 "64 J in (0,0.3] x 5 sectors = 320 eigensolves (lowest 10), U=1, 64-point mu map")
METRIC = "eigensolves/s (batched mixed-precision, lowest 10, <=1e-8 rel err vs FP64)"
# the workload's description, shared by both arms' lines
def workload_config(ws: int) -> dict:
    """The `config` of both arms' lines (the same dict, so that the lines
    compare like with like)."""
    return {"workload": WORKLOAD_NAME, "m": M, "sectors": SECTORS, "j_points": NJ, "nev": NEV,
            "mu_points": len(MU), "precision": "mixed (FP32 vectors and products, FP64 coefficients)",
            "parallelism": ("one GPU" if ws == 1 else
                            f"{ws} ranks, each solving its 64 points of a {NJ * ws}-point J grid "
                            "(points r, r + N, ...), no exchange between ranks"),
            "l2": "256 MB buffer written between timed steps; Krylov basis (up to 9 GB) > L2"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched",
                    choices=["batched", "mixed-large", "matrix-free-2d", "mean-field", "plain-m12"],
                    help="batched (default): the m=10 multi-sector grid; the others are "
                         "the larger single-sector configurations, the mean-field sweep and "
                         "the plain FP64 single-point solve at m=n=12")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(kernel: str, algorithmic_bytes_per_launch: float | None = None):
    """Per-launch DRAM traffic of `kernel`: the DRAM/algorithmic byte ratio of
    its committed ncu capture (profiles/traffic.json) times this run's
    algorithmic bytes per launch."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        ratio = d[kernel]["dram_over_algorithmic"]
        if algorithmic_bytes_per_launch is None:
            return None
        return round(ratio * algorithmic_bytes_per_launch)
    except Exception:
        return None


# ---------------------------------------------------------------------------
# CPU restatement of the reference path (oracle)
# ---------------------------------------------------------------------------
class CpuReference:
    """The CPU restatement of the reference's path (oracle): Op::IRLM_eigen
    (Spectra GenEigsSolver, ncv = 2 nev + 1, SimpleRandom(0) start) on the
    model Hamiltonian of each sector of the grid, FP64, with the reference's
    own parallelism -- OpenMP over grid points (analysis.cpp:302), one solve
    per thread -- on every host core.  The five sector Hamiltonians are built
    once (untimed).  A sample is one wave of concurrent solves of one sector:
    as many points as there are cores, one thread each; in the sectors above
    5 10^4 states a quarter as many points with four threads on each solve's
    row loops (a wave of single-threaded solves there takes up to a minute)."""

    def __init__(self, threads: int = 0):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc_mod

        self.orc = orc_mod.Oracle()
        self.threads = threads or (os.cpu_count() or 1)
        off = np.zeros(M + 1, np.int32)
        flat = []
        for i in range(M):  # the periodic chain (Neighbours::chain_neighbours)
            nb = ([i - 1] if i > 0 else []) + ([i + 1] if i < M - 1 else [])
            nb += [M - 1] if i == 0 else ([0] if i == M - 1 else [])
            flat += nb
            off[i + 1] = len(flat)
        flat = np.array(flat, np.int32)
        self.ops = {}
        for n in SECTORS:
            occ = self.orc.lex_states(M, n)
            col_of_lex, lex_of_col = self.orc.reference_order(occ)
            rp, ci, tv = self.orc.build_T(occ, off, flat, lex_of_col, col_of_lex)
            self.ops[n] = (rp, ci, tv, self.orc.diag_V(occ, lex_of_col))

    def shape(self, n: int):
        """(concurrent solves, threads per solve) of a wave in sector n."""
        inner = 4 if len(self.ops[n][3]) > 50000 and self.threads >= 8 else 1
        return max(1, self.threads // inner), inner

    def points(self, k: int):
        """Wave k: sector SECTORS[k mod 5], J indices 8 + (7 + 13 i) mod 56 for
        the wave's consecutive sample numbers i, so that waves spread over J.
        The eight smallest J (b < 8, J < 0.042) are left out: there the
        reference's IRLM (ncv = 21) does not reach 10 converged values within
        its 1000 restarts at some points and would throw."""
        n = SECTORS[k % len(SECTORS)]
        groups, _ = self.shape(n)
        return n, [8 + (7 + 13 * (k * 16 + i)) % (NJ - 8) for i in range(groups)]

    def wave(self, k: int) -> tuple[int, int, float]:
        """Runs wave k: (sector, solves, seconds)."""
        n, bs = self.points(k)
        groups, inner = self.shape(n)
        rp, ci, tv, vd = self.ops[n]
        t0 = time.perf_counter()
        ev, nc = self.orc.irlm_wave(rp, ci, tv, vd, n, JS[bs], U, 0.0, nev=NEV, groups=groups, inner=inner)
        dt = time.perf_counter() - t0
        if nc.min() < NEV:
            raise RuntimeError(f"CPU reference did not converge (n={n})")
        return n, len(bs), dt

    @staticmethod
    def rate(per_solve: dict) -> float:
        """Eigensolves/s of the full grid (equal numbers of points in every
        sector) from each sector's seconds per solve (wave time / solves)."""
        return len(SECTORS) / sum(float(np.mean(per_solve[n])) for n in SECTORS)


def cpu_sample_rate():
    """One cycle of five waves (one per sector): (rate, cores, seconds)."""
    ref = CpuReference()
    per_solve, tot = {}, 0.0
    for k in range(len(SECTORS)):
        n, cnt, dt = ref.wave(k)
        per_solve.setdefault(n, []).append(dt / cnt)
        tot += dt
    return ref.rate(per_solve), ref.threads, tot


def cpu_sample_rate_subprocess():
    """cpu_sample_rate in a fresh process: in the GPU arm's process (CUDA
    runtime and solver host threads alive) the same waves ran 2.6x slower."""
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-sample"],
                       capture_output=True, text=True, timeout=900)
    if r.returncode != 0:
        raise RuntimeError("CPU sample failed: " + r.stderr[-2000:])
    d = json.loads(r.stdout.strip().splitlines()[-1])
    return d["rate"], d["cores"], d["seconds"]


CPU_SAMPLE = ("waves of concurrent solves, one sector per wave, the five sectors in turn: per wave one "
              "solve per host core (sectors n=8,9) or a quarter as many with four threads on each solve's "
              "row loops (n=10..12, above 5e4 states); J indices 8 + (7 + 13 i) mod 56 (the reference's "
              "IRLM fails to converge at some of the eight smallest J); rate = 5 / (sum over sectors of "
              "wave seconds / solves in the wave), i.e. the full grid's eigensolves/s with every sector "
              "weighted as in the grid; FP64 restatement of Op::IRLM_eigen (Spectra GenEigsSolver, "
              "ncv=2nev+1), OpenMP over points as analysis.cpp:302")


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev: int):
        self.dev = dev
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.dev)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def j_shard(pkg, ws: int, rank: int) -> np.ndarray:
    """J values of this rank: points rank, rank + ws, ... of the 64 ws-point
    grid J_b = 0.3 (b + 1) / (64 ws); one rank gets the 64-point grid JS."""
    return 0.3 * (pkg.shard_indices(NJ * ws, ws, rank) + 1) / (NJ * ws)


def max_over_ranks(x: float, ws: int, device: str) -> float:
    """The largest x over the ranks of the default process group."""
    if ws <= 1:
        return float(x)
    import torch

    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def run_ours(args):
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    sys.path.insert(0, ROOT)
    import __graft_entry__ as g

    pkg = g.load_package()
    pkg.load()
    nb = pkg.Neighbours(M)
    nb.chain_neighbours()
    lists = nb.getNeighbours()
    # N ranks: a 64 N-point J grid on (0, 0.3], rank r solving points r, r + N, ...
    # (64 per rank, the same spread as the one-GPU grid; no exchange between ranks)
    js = j_shard(pkg, ws, rank)

    # sector Hamiltonians resident in HBM (untimed setup for `value`)
    hams = [pkg.Hamiltonian(pkg.Basis(M, n), lists) for n in SECTORS]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def step_resident(prec=pkg.PREC_MIXED):
        # all five sectors in one call; they run concurrently on the device
        ev, rs, nc, info = pkg.eigsh_sectors(hams, js, U, 0.0, nev=NEV, precision=prec)
        if nc.min() < NEV:
            raise RuntimeError("a sector did not converge")
        e0 = ev[:, :, 0]
        dens, kap = pkg.Analysis.phase_map(M, SECTORS[0], e0, MU)
        return [ev[k] for k in range(len(SECTORS))], info.launches + 2

    def step_e2e():
        hs = [pkg.Hamiltonian(pkg.Basis(M, n), lists) for n in SECTORS]
        ev, rs, nc, info = pkg.eigsh_sectors(hs, js, U, 0.0, nev=NEV, precision=pkg.PREC_MIXED)
        dens, kap = pkg.Analysis.phase_map(M, SECTORS[0], ev[:, :, 0], MU)
        del hs
        return info.launches

    def timed(fn, steps):
        ts = []
        out = None
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            if ws > 1:
                torch.distributed.barrier()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            out = fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) / 1e3)
        return max_over_ranks(sum(ts), ws, "cuda"), out

    for _ in range(args.warmup):
        step_resident()
    clocks = ClockSampler(local)
    clocks.start()
    t_val, (evs_mixed, launches_step) = timed(step_resident, args.steps)
    clk = clocks.stop()
    solves_per_step = len(SECTORS) * NJ
    value = solves_per_step * args.steps * ws / t_val

    # end to end through the public API from host arrays
    step_e2e()
    t_e2e, _ = timed(step_e2e, args.steps)
    e2e_value = solves_per_step * args.steps * ws / t_e2e
    nbr_bytes = (M + 1) * 4 + 2 * M * 4
    h2d = len(SECTORS) * (nbr_bytes + 3 * NJ * 8) + len(SECTORS) * NJ * 8 + len(MU) * 8
    d2h = len(SECTORS) * NJ * (NEV * 8 * 2 + 4) + 2 * NJ * len(MU) * 8

    out = {"metric": METRIC,
           "value": round(value, 3), "unit": "eigensolves/s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(1e3 * t_val / args.steps, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
           "data": "synthetic (Hamiltonian determined by m, n, J, U; seeded start block)",
           "config": workload_config(ws),
           "e2e": {"value": round(e2e_value, 3), "unit": "eigensolves/s",
                   "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
           "gpu_launches": int(launches_step * args.steps),
           "clocks": clk}

    if rank == 0:
        # accuracy of the mixed results against the FP64 batched path (untimed):
        # eigenvalues, and the density / compressibility maps composed from
        # each path's ground-state energies
        ev64 = np.stack([h.eigsh_batch(js, U, 0.0, nev=NEV, precision=pkg.PREC_FP64)[0] for h in hams])
        evm = np.stack(evs_mixed)
        d_m, k_m = pkg.Analysis.phase_map(M, SECTORS[0], evm[:, :, 0], MU)
        d_d, k_d = pkg.Analysis.phase_map(M, SECTORS[0], ev64[:, :, 0], MU)
        out["accuracy"] = {
            "max_rel_err_vs_fp64": float(np.max(np.abs(evm - ev64) / np.abs(ev64))),
            "definition": "|E_mixed - E_fp64| / |E_fp64| over all 3200 eigenvalues",
            "max_rel_err_floored": float(np.max(np.abs(evm - ev64) / (np.abs(ev64) + 1e-2))),
            "floored_definition": "|E_mixed - E_fp64| / (|E_fp64| + 1e-2)",
            "density_map_max_abs_diff": float(np.max(np.abs(d_m - d_d))),
            "compressibility_map_max_abs_diff": float(np.max(np.abs(k_m - k_d))),
            "maps": f"{NJ} J x {len(MU)} mu, rho = n*/m and its finite-difference d rho / d mu"}

        # plain FP64 path: one solve per call, sample of 4 J per sector
        sample_b = [7, 23, 39, 55]
        t0 = time.perf_counter()
        for h in hams:
            for b in sample_b:
                h.eigsh(js[b], U, 0.0, nev=NEV)
        torch.cuda.synchronize()
        tp = time.perf_counter() - t0
        plain_rate = len(sample_b) * len(hams) / tp
        out["plain_fp64"] = {"value": round(plain_rate, 3), "unit": "eigensolves/s",
                             "sample": "J_b, b in {7,23,39,55}, all 5 sectors (20 solves)",
                             "batched_mixed_over_plain": round(value / ws / plain_rate, 2)}

        # roofline of the dominant kernel from one profiled step
        pkg.profile_reset()
        pkg.profile_enable(True)
        step_resident()
        pkg.profile_enable(False)
        prof = pkg.profile_read()
        tot_ms = sum(v["ms"] for v in prof.values())
        dom = max(prof.items(), key=lambda kv: kv[1]["ms"])
        name, rec = dom
        per_launch_bytes = rec["bytes"] / rec["launches"]
        per_launch_s = rec["ms"] / rec["launches"] / 1e3
        achieved = per_launch_bytes / per_launch_s / 1e9
        peak, peak_kind = measured_peaks()
        out["roofline"] = {"kernel": name, "bound": "hbm", "achieved": round(achieved, 1),
                           "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                           "frac": round(achieved / peak, 4),
                           "traffic": profile_traffic(name, per_launch_bytes),
                           "share_of_kernel_time": round(rec["ms"] / tot_ms, 4),
                           "algorithmic_bytes_per_launch": round(per_launch_bytes)}
        out["kernel_time_shares"] = {k: round(v["ms"] / tot_ms, 4)
                                     for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])}
        # the whole solver against the same roofline: every kernel's
        # algorithmic bytes of one step over the summed kernel time, and over
        # the timed step (the sectors overlap on the device)
        tot_bytes = sum(v["bytes"] for v in prof.values())
        out["whole_solver"] = {
            "algorithmic_bytes_per_step": round(tot_bytes),
            "kernel_ms_per_step": round(tot_ms, 1),
            "gbs_over_kernel_time": round(tot_bytes / (tot_ms * 1e6), 1),
            "gbs_over_step_time": round(tot_bytes / (t_val / args.steps * 1e9), 1),
            "peak": peak, "peak_kind": peak_kind,
            "frac_over_step_time": round(tot_bytes / (t_val / args.steps * 1e9) / peak, 4)}
        out["kernel_gbs"] = {k: round(v["bytes"] / (v["ms"] * 1e6), 1)
                             for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"]) if v["ms"] > 0}

        # the sparse product against the bytes it must gather (every entry
        # pulls a whole row of X), on the largest sector solved alone, whose
        # D and entry count fix the bytes of each launch
        pkg.profile_reset()
        pkg.profile_enable(True)
        hams[-1].eigsh_batch(js, U, 0.0, nev=NEV, precision=pkg.PREC_MIXED)
        pkg.profile_enable(False)
        gather = _spmm_gather(pkg.profile_read(), hams[-1], False)
        if gather:
            gather["sector"] = f"n={SECTORS[-1]} alone (D={hams[-1].D}), {len(js)} J"
        out["spmm_gather"] = gather

        # launch shapes the autotuner chose for the unfused products of the
        # bench's sectors (timed during the first warm-up step, while the five
        # sectors run concurrently)
        dims = {h.D for h in hams}
        tuned = [e for e in pkg.spmm_tuning_table() if e["dim"] in dims and e["elem_bytes"] == 4]
        if tuned:
            out["spmm_tuning"] = {
                "width_classes": len(tuned),
                "non_default_shape": int(sum(e["shape"] != pkg.spmm_candidates(e["ncols"], e["matrix_free"])[0]
                                             for e in tuned))}

        rate, cores, secs = cpu_sample_rate_subprocess()
        out["cpu_baseline"] = {"value": round(rate, 4), "unit": "eigensolves/s", "cores": cores,
                               "kind": "port", "sample": "one cycle of five waves: " + CPU_SAMPLE,
                               "seconds": round(secs, 2), "cpu": cpu_model()}
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------
# reference arm: the CPU restatement of the reference's path
# ---------------------------------------------------------------------------
def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as f:
            txt = f.read()
        for key in ("model name", "Model", "CPU part"):
            for ln in txt.splitlines():
                if ln.startswith(key):
                    return ln.split(":", 1)[1].strip() + f" ({os.cpu_count()} cores, {os.uname().machine})"
    except OSError:
        pass
    return f"{os.uname().machine}, {os.cpu_count()} cores"


def run_reference(args):
    """One step = one wave of CpuReference (one sector, the sectors in turn);
    value = the full grid's eigensolves/s from every sector's seconds per
    solve (CpuReference.rate).  Only rank 0 runs."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    ref = CpuReference()
    for k in range(args.warmup):
        ref.wave(k)
    per_solve, tot, solves = {}, 0.0, 0
    steps = max(args.steps, len(SECTORS))  # every sector at least once
    for k in range(args.warmup, args.warmup + steps):
        n, cnt, dt = ref.wave(k)
        per_solve.setdefault(n, []).append(dt / cnt)
        tot += dt
        solves += cnt
    value = ref.rate(per_solve)
    out = {"impl": "reference", "metric": METRIC,
           "value": round(value, 4), "unit": "eigensolves/s", "n_gpus": ws, "steps": steps,
           "warmup": args.warmup, "ms_per_step": round(1e3 * tot / steps, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (Hamiltonian determined by m, n, J, U; seeded start vector)",
           "config": workload_config(ws),
           "cpu_baseline": {"value": round(value, 4), "unit": "eigensolves/s", "cores": ref.threads,
                            "kind": "port", "sample": "one wave per step: " + CPU_SAMPLE,
                            "solves": solves,
                            "seconds_per_solve": {str(n): round(float(np.mean(v)), 3) for n, v in per_solve.items()},
                            "cpu": cpu_model()},
           "e2e": {"value": round(value, 4), "unit": "eigensolves/s",
                   "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
# the other configurations (not the default line)
# ---------------------------------------------------------------------------
EXTRA = {
    "mixed-large": dict(m=14, n=14, lattice="chain", J=np.linspace(0.02, 0.2, 8), U=1.0, mu=0.0,
                        nev=6, ncv=80, block=2, matrix_free=False, fp64_sample=[0, 7],
                        name="1D periodic chain m=14, n=14 (D=20058300, stored CSR), 8 J in "
                             "[0.02,0.2], U=1, lowest 6, 80-vector Krylov basis"),
    "matrix-free-2d": dict(m=16, n=12, lattice="square", J=np.linspace(0.02, 0.1, 16), U=1.0,
                           mu=0.4, nev=4, ncv=60, block=4, matrix_free=True, fp64_sample=[0, 15],
                           name="4x4 periodic square lattice, n=12 (D=17383860, matrix-free), 16 J "
                                "in [0.02,0.1], U=1, mu=0.4, lowest 4, 60-vector Krylov basis, "
                                "block 4 (the torus has four-fold levels)"),
}


def _profile_summary(pkg, prof):
    tot_ms = sum(v["ms"] for v in prof.values())
    name, rec = max(prof.items(), key=lambda kv: kv[1]["ms"])
    per_b = rec["bytes"] / rec["launches"]
    per_s = rec["ms"] / rec["launches"] / 1e3
    peak, kind = measured_peaks()
    achieved = per_b / per_s / 1e9
    return ({"kernel": name, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
             "peak_kind": kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
             "traffic": profile_traffic(name, per_b),
             "share_of_kernel_time": round(rec["ms"] / tot_ms, 4),
             "algorithmic_bytes_per_launch": round(per_b)},
            {k: round(v["ms"] / tot_ms, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])})


def run_extra(args):
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    sys.path.insert(0, ROOT)
    import __graft_entry__ as g

    pkg = g.load_package()
    pkg.load()
    if args.workload == "mean-field":
        return run_mean_field(args, pkg, torch)
    if args.workload == "plain-m12":
        return run_plain(args, pkg, torch)
    c = EXTRA[args.workload]
    nb = pkg.Neighbours(c["m"])
    if c["lattice"] == "chain":
        nb.chain_neighbours()
    else:
        nb.square_neighbours(True)
    h = pkg.Hamiltonian(pkg.Basis(c["m"], c["n"]), nb.getNeighbours(), matrix_free=c["matrix_free"])
    opts = dict(nev=c["nev"], ncv=c["ncv"], block=c["block"])
    S = len(c["J"])

    def solve(prec, J=c["J"]):
        return h.eigsh_batch(J, c["U"], c["mu"], precision=prec, **opts)

    for _ in range(max(0, args.warmup)):
        solve(pkg.PREC_MIXED, c["J"][:2])
    clocks = ClockSampler(local)
    clocks.start()
    ts = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        ev, rs, nc, info = solve(pkg.PREC_MIXED)
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b) / 1e3)
    clk = clocks.stop()
    value = S * args.steps / sum(ts)
    # FP64 plain path on a sample of the points: accuracy and the ratio
    smp = c["fp64_sample"]
    t0 = time.perf_counter()
    e64 = np.stack([h.eigsh(c["J"][k], c["U"], c["mu"], block=c["block"], ncv=c["ncv"], nev=c["nev"])[0]
                    for k in smp])
    t64 = time.perf_counter() - t0
    rel = np.abs(ev[smp] - e64) / np.abs(e64)
    # kernel shares and the dominant kernel's roofline from one profiled run on 4 points
    pkg.profile_reset()
    pkg.profile_enable(True)
    solve(pkg.PREC_MIXED, c["J"][:4])
    pkg.profile_enable(False)
    prof = pkg.profile_read()
    roof, shares = _profile_summary(pkg, prof)
    gather = _spmm_gather(prof, h, c["matrix_free"])
    out = {"metric": "eigensolves/s (batched mixed-precision, <=1e-8 rel err vs FP64)",
           "value": round(value, 4), "unit": "eigensolves/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(1e3 * sum(ts) / args.steps, 1),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
           "data": "synthetic (Hamiltonian determined by the lattice, n, J, U)",
           "config": {"workload": c["name"], "D": h.D, "nnz_offdiag": h.nnz_offdiag,
                      "matrix_free": c["matrix_free"], "restarts": info.restarts,
                      "matvecs": info.matvecs, "min_nconv": int(nc.min())},
           "accuracy": {"max_rel_err_vs_fp64": float(rel.max()),
                        "definition": "|E_mixed - E_fp64| / |E_fp64|, every eigenvalue of the points",
                        "points": [int(k) for k in smp]},
           "plain_fp64": {"value": round(len(smp) / t64, 5), "unit": "eigensolves/s",
                          "batched_mixed_over_plain": round(value / (len(smp) / t64), 2)},
           "roofline": roof, "spmm_gather": gather, "kernel_time_shares": shares, "clocks": clk}
    print(json.dumps(out), flush=True)


def _spmm_gather(prof, h, matrix_free):
    """The sparse product against the bandwidth of the bytes it must gather.
    The algorithmic count reads X once per product; every stored (or
    regenerated) entry gathers one whole row of X (ncols values), so the
    product moves  op + Z B s + 2 D B s  bytes (op: CSR pattern, values and
    diagonal, or the packed occupations; Z off-diagonal entries; B columns;
    s bytes per value), most of it from DRAM when X does not fit in L2.
    The total B over the product's launches follows from its algorithmic
    bytes, which are linear in B."""
    name = "k_spmm_mf" if matrix_free else "k_spmm"
    rec = prof.get(name)
    if not rec or not rec["launches"]:
        return None
    s_val, D, Z, L = 4.0, float(h.D), float(h.nnz_offdiag), rec["launches"]
    op = D * 8.0 if matrix_free else Z * (4.0 + s_val) + (D + 1.0) * 8.0 + D * s_val
    sumB = (rec["bytes"] - L * op) / (2.0 * D * s_val)
    gbytes = L * op + (Z + 2.0 * D) * s_val * sumB
    peak, kind = measured_peaks()
    achieved = gbytes / (rec["ms"] / 1e3) / 1e9
    return {"kernel": name, "gather_bytes_per_launch": round(gbytes / L), "achieved": round(achieved, 1),
            "peak": peak, "peak_kind": kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
            "mean_columns": round(sumB / L, 1),
            "definition": "(operator bytes + entries x columns x 4 B + 2 x D x columns x 4 B) / CUDA-event time"}


# E0 of the m=n=12 chain at J=0.05, U=1, mu=0.6 from the reference's Op::IRLM_eigen
# (Spectra GenEigsSolver) on the model Hamiltonian, 13 significant digits
PLAIN_E0 = -7.319694388230


def run_plain(args, pkg, torch):
    """One FP64 solve per step through the single-point call that replaces
    Op::IRLM_eigen (operator.cpp:22-33): m=n=12 chain (D=1352078), J=0.05,
    U=1, mu=0.6, lowest 10."""
    m, n, J, U, mu, nev = 12, 12, 0.05, 1.0, 0.6, 10
    nb = pkg.Neighbours(m)
    nb.chain_neighbours()
    lists = nb.getNeighbours()
    t0 = time.perf_counter()
    h = pkg.Hamiltonian(pkg.Basis(m, n), lists)
    t_build = time.perf_counter() - t0
    for _ in range(max(0, args.warmup)):
        h.eigsh(J, U, mu, nev=nev)
    local = dist_env()[2]
    clocks = ClockSampler(local)
    clocks.start()
    ts = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        ev, rs, _, info = h.eigsh(J, U, mu, nev=nev)
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b) / 1e3)
    clk = clocks.stop()
    value = args.steps / sum(ts)
    # end to end through the public API: basis, Hamiltonian, solve, results on the host
    te = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        h2 = pkg.Hamiltonian(pkg.Basis(m, n), lists)
        ev2, _, _, _ = h2.eigsh(J, U, mu, nev=nev)
        te.append(time.perf_counter() - t0)
        del h2
    pkg.profile_reset()
    pkg.profile_enable(True)
    h.eigsh(J, U, mu, nev=nev)
    pkg.profile_enable(False)
    prof = pkg.profile_read()
    roof, shares = _profile_summary(pkg, prof)
    # the FP64 rotation is bound by the FP64 FMA rate, not by HBM: 2 D kc nout
    # flops per launch (automatic basis kc = 7 nev = 70 vectors, nout = 40 kept)
    rot = prof.get("k_rotate")
    if rot and rot["launches"]:
        per_s = rot["ms"] / rot["launches"] / 1e3
        tflops = 2.0 * h.D * 70 * 40 / per_s / 1e12
        roof["fp64_rotation"] = {"achieved": round(tflops, 3), "unit": "TFLOP/s",
                                 "flops": "2 D x 70 x 40 per launch (every launch counted as a restart rotation)",
                                 "peak": 1.25, "peak_kind": "nominal GB300 FP64 (no measured FP64 peak)",
                                 "frac": round(tflops / 1.25, 3)}
    out = {"metric": "eigensolves/s (plain FP64 single-point solve, lowest 10)",
           "value": round(value, 4), "unit": "eigensolves/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(1e3 * sum(ts) / args.steps, 1),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (Hamiltonian determined by m, n, J, U; seeded start block)",
           "config": {"workload": "1D periodic chain m=12, n=12 (D=1352078), J=0.05, U=1, mu=0.6, "
                                  "lowest 10, FP64, one solve per call (the Op::IRLM_eigen drop-in)",
                      "D": h.D, "nnz_offdiag": h.nnz_offdiag, "restarts": info.restarts,
                      "matvecs": info.matvecs, "basis_and_hamiltonian_build_s": round(t_build, 3)},
           "e2e": {"value": round(len(te) / sum(te), 4), "unit": "eigensolves/s",
                   "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 2 * nev * 8,
                   "includes": "basis + Hamiltonian build on the device, solve, eigenvalues to host"},
           "accuracy": {"E0": float(ev[0]), "E0_reference_irlm": PLAIN_E0,
                        "abs_err": abs(float(ev[0]) - PLAIN_E0), "max_resid": float(np.max(rs))},
           "roofline": roof, "kernel_time_shares": shares, "clocks": clk}
    print(json.dumps(out), flush=True)


def run_mean_field(args, pkg, torch):
    n, prec, q = 1000, 6, 1
    pkg.Analysis.mean_field_parameters(50, prec, q=q)
    ts = []
    for s in range(args.steps):
        t0 = time.perf_counter()
        mu, J, psi = pkg.Analysis.mean_field_parameters(n, prec, q=q, seed=s + 1)
        ts.append(time.perf_counter() - t0)
    value = psi.size * args.steps / sum(ts)
    # the oracle on a random sample of the same grid points and seeds
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc_mod

    orc = orc_mod.Oracle()
    rng = np.random.RandomState(0)
    idx = rng.choice(psi.size, 20000, replace=False)
    M, JJ = np.meshgrid(mu, J, indexing="ij")
    psi0 = rng.uniform(0.0, 1.0, len(idx))
    pg, _ = pkg.Analysis.SCMF(M.ravel()[idx], JJ.ravel()[idx], q, psi0, prec)
    t0 = time.perf_counter()
    po, _ = orc.scmf_batch(M.ravel()[idx], JJ.ravel()[idx], q, psi0, prec)
    tc = time.perf_counter() - t0
    out = {"metric": "mean-field points/s (self-consistent psi to 1e-6)", "value": round(value, 1),
           "unit": "points/s", "n_gpus": 1, "steps": args.steps, "warmup": 1,
           "ms_per_step": round(1e3 * sum(ts) / args.steps, 1), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic grid",
           "config": {"workload": "mean-field sweep, 1001 x 1001 (mu, J) grid on [0,4) x [0,0.25), "
                                  "q=1, eps=1e-6 (the reference's README run)"},
           "accuracy": {"max_abs_psi_diff_vs_oracle": float(np.max(np.abs(pg - po))),
                        "sample_points": len(idx)},
           "cpu_baseline": {"value": round(len(idx) / tc, 1), "unit": "points/s",
                            "cores": os.cpu_count() or 1, "kind": "port",
                            "sample": "20000 random points of the grid, OpenMP over points"}}
    print(json.dumps(out), flush=True)


def main():
    if "--cpu-sample" in sys.argv:
        rate, cores, secs = cpu_sample_rate()
        print(json.dumps({"rate": rate, "cores": cores, "seconds": secs}), flush=True)
        return
    args = parse()
    if args.workload != "batched":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm covers the default "
                              "batched workload; the CPU oracle figure is in this workload's "
                              "cpu_baseline"}))
            return
        run_extra(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
