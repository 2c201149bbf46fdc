"""Benchmark: Fock builds/s (one J and one K build) on the Kr benchmark basis.

Workload (the reference's Kr Fock-build kernel configuration): Z = 36,
40 radial elements with boundaries r_i = 61^(i/40) - 1 bohr (exponential
grid, zexp = 1, Rmax = 60), 15-node LIP elements, l = 0..2 with m = -2..2
(Nang = 9, Nrad = 559, Nbf = 5031), multipoles L = 0..4. The density is
P = C C^T from 18 columns with entries drawn from N(0,1) (seed 12345),
Loewdin-orthonormalised against the FEM overlap. One step = J(P) + K(P),
plain FP64. P is 202 MB, larger than L2 (129 MB), so no L2 flush is needed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0). Under torchrun (N > 1) every rank runs an
independent replica (atoms do not shard: replicas only) and the value is the
whole-job throughput over the slowest rank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Fock builds/s (J+K)"
UNIT = "builds/s"
WORKLOAD = ("Kr (Z=36) J+K Fock build: 40 elements r_i=61^(i/40)-1, 15-node LIP, l<=2, m<=2, "
            "Nbf=5031, L<=4, P=CC^T (18 cols, N(0,1), seed 12345, Loewdin in S)")
KERNELS_PER_STEP = 5  # profiler marks per step: J contract, J scatter, K norms, K tiles, K fix-up
# kernel launches per step: j_contract, j_scatter, k_block_norms, k_flags, then
# k_tiles_tc + k_diag_tc (split form) or k_tiles (plain form), k_fixup
LAUNCHES_PER_STEP = {"split": 7, "plain": 6}
# what the timed K form computes in (the dtype key names the arithmetic, the
# form key the scheme)
FORMS = {
    "plain": {"dtype": "f64", "form": "plain FP64"},
    "split": {"dtype": "bf16 digits (7 x 8-bit slices, exact FP32 level sums on the tensor cores, FP64 recombination)",
              "form": "split precision on the tensor cores: density tiles recoupled in float pairs, radial tables "
                      "and density as balanced base-256 digit planes (bf16), tcgen05 MMAs form exact FP32 level "
                      "sums in tensor memory, carried and recombined to FP64 once per output element; J in float "
                      "pairs (hi + lo, error-free products) with one FP64 conversion per output element"},
}


def kr_basis():
    """The benchmark basis through the product's own grid and angular-basis
    entry points (hfg_grid, hfg_angular_basis)."""
    import helfem_gb300 as hg
    bval = hg.get_grid(60.0, 40, 4, 1.0)
    lval, mval = hg.angular_basis(2, 2)
    return 36, bval, lval, mval


def kr_basis_oracle():
    """The same basis for the CPU legs, from the oracle alone (the reference
    arm loads nothing of the product)."""
    from oracle import tabulate as tab
    bval = tab.get_grid(60.0, 40, 4, 1.0)
    lval, mval = tab.angular_basis(2, 2)
    return 36, bval, lval, mval


def kr_density(S: np.ndarray, nocc: int = 18, seed: int = 12345) -> np.ndarray:
    rng = np.random.default_rng(seed)
    C = rng.standard_normal((S.shape[0], nocc))
    M = C.T @ S @ C
    w, v = np.linalg.eigh(M)
    C = C @ (v @ np.diag(w ** -0.5) @ v.T)
    return C @ C.T


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


# --------------------------------------------------------------------------
# CPU side: the oracle (C++/OpenMP restatement of the reference's path)
# --------------------------------------------------------------------------

_CPU = {}


def cpu_reference_builds(min_seconds: float, max_builds: int, min_builds: int = 1, threads: int = 0):
    """Time full-size oracle J+K builds on the host cores (threads = 0: all
    of them); returns (builds/s, builds, seconds, threads)."""
    import oracle
    from oracle import tabulate as tab
    oracle.lib().ora_set_threads(threads)
    if not _CPU:
        Z, bval, lval, mval = kr_basis_oracle()
        A = tab.build_atom(Z, 15, bval, 2, 2)
        _CPU["P"] = kr_density(A.S)
        _CPU["F"] = oracle.FockOracle(A)
        _CPU["F"].coulomb(_CPU["P"])  # warm-up (page-in, thread pool)
    F, P = _CPU["F"], _CPU["P"]
    n, t0 = 0, time.perf_counter()
    while n < max_builds and (n < min_builds or time.perf_counter() - t0 < min_seconds):
        F.coulomb(P)
        F.exchange(P)
        n += 1
    dt = time.perf_counter() - t0
    return n / dt, n, dt, oracle.lib().ora_num_threads()


# --------------------------------------------------------------------------
# clocks sampled during the timed region
# --------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        try:
            rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        except OSError:
            rows = []
        finally:
            try:
                os.unlink(self.f.name)
            except OSError:
                pass
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "samples": len(sm), "reasons": sorted(reasons)}


def fp64_peak_tflops(torch) -> float:
    """cuBLAS DGEMM throughput, the FP64 denominator (not among the
    measured peaks)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


def fp32_peak_tflops(torch) -> float:
    """cuBLAS SGEMM with TF32 disabled: the FP32-pipe denominator."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, dtype=torch.float32, device="cuda")
        b = torch.randn(n, n, dtype=torch.float32, device="cuda")
        a @ b
        torch.cuda.synchronize()
        best = 0.0
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            a @ b
            e1.record()
            torch.cuda.synchronize()
            best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
        return best
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


# --------------------------------------------------------------------------

def dist_setup(n_gpus):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch.distributed as dist
    rank, local = int(os.environ["RANK"]), int(os.environ.get("LOCAL_RANK", "0"))
    return rank, ws, local, dist


def run_reference(args):
    rank, ws, local, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    per_step = []
    threads = None
    for i in range(args.warmup + args.steps):
        rate, n, dt, threads = cpu_reference_builds(0.0, 1, 1)
        if i >= args.warmup:
            per_step.append(dt / n)
    mean = sum(per_step) / len(per_step)
    val = 1.0 / mean
    out = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "inputs_vs_l2": "host run (no GPU)"},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full-size Kr J+K builds, one per step"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def host_link_rates(torch, Ph, Kh, reps=3):
    """Copy rates of the host link for one density-sized transfer between
    the pinned host buffers of the e2e leg and a device buffer: each way
    alone and both at once (GB/s, best of reps). The e2e step moves P in
    and K out unhidden, so these bound it."""
    hp = torch.from_numpy(Ph.T)  # the same pinned memory
    hk = torch.from_numpy(Kh.T)
    d1, d2 = torch.empty_like(hp, device="cuda"), torch.empty_like(hp, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    nbytes = hp.numel() * 8

    def timed(h2d, d2h):
        best = 1e30
        for _ in range(reps + 1):
            torch.cuda.synchronize()
            t = time.perf_counter()
            if h2d:
                with torch.cuda.stream(s1):
                    d1.copy_(hp, non_blocking=True)
            if d2h:
                with torch.cuda.stream(s2):
                    hk.copy_(d2, non_blocking=True)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t)
        return nbytes * (int(h2d) + int(d2h)) / best / 1e9

    out = {"h2d": timed(True, False), "d2h": timed(False, True), "both": timed(True, True)}
    del d1, d2
    return out


def n2_summary(hg, torch, builds=2):
    """The N2 diatomic Fock build beside the headline (split and plain K,
    J, the split error): seconds of work, reported as an object of the main
    line."""
    d, P, act = n2_setup(hg)
    Pd = torch.from_numpy(P.ravel(order="F")).cuda()
    Pa = 0.5 * Pd
    Jd, Kd = torch.empty_like(Pd), torch.empty_like(Pd)
    st = torch.cuda.current_stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)
    d.coulomb(Pd, Jd, stream=st)
    d.exchange(Pa, Kd, symmetric=True, stream=st, split=True)  # warm-up
    torch.cuda.synchronize()
    e0, e1, e2 = ev(), ev(), ev()
    e0.record(st)
    for _ in range(builds):
        d.coulomb(Pd, Jd, stream=st)
    e1.record(st)
    for _ in range(builds):
        d.exchange(Pa, Kd, symmetric=True, stream=st, split=True)
    e2.record(st)
    torch.cuda.synchronize()
    j_ms, k_ms = e0.elapsed_time(e1) / builds, e1.elapsed_time(e2) / builds
    K32 = Kd.clone()
    p0, p1 = ev(), ev()
    p0.record(st)
    d.exchange(Pa, Kd, symmetric=True, stream=st)
    p1.record(st)
    torch.cuda.synchronize()
    dK = K32 - Kd
    out = {"workload": N2_WORKLOAD, "nbf": d.nbf, "coulomb_ms": j_ms, "exchange_split_ms": k_ms,
           "exchange_plain_ms": p0.elapsed_time(p1),
           "builds_per_s_split": 1e3 / (j_ms + k_ms), "builds_per_s_plain": 1e3 / (j_ms + p0.elapsed_time(p1)),
           "split_error_vs_fp64": {"k_max_rel": float(dK.abs().max() / Kd.abs().max()),
                                   "exchange_energy_abs_eh": abs(float((Pa * dK).sum()))},
           "form": "split: float-pair diatomic tiles (the atomic tensor-core path does not cover the "
                   "diatomic four-channel kernel)", "builds": builds}
    del Pd, Pa, Jd, Kd, K32, dK
    d.close()
    torch.cuda.empty_cache()
    return out


def run_ours(args):
    import torch

    rank, ws, local, dist = dist_setup(args.gpus)
    if dist is not None:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    import helfem_gb300 as hg

    Z, bval, lval, mval = kr_basis()
    atom = hg.Atom(Z, bval, lval, mval, nnodes=15)
    S = atom.overlap()
    P = kr_density(S)
    nbf = atom.nbf
    Pd = torch.from_numpy(np.ascontiguousarray(P.T)).cuda()
    Jd, Kd = torch.empty_like(Pd), torch.empty_like(Pd)
    stream = torch.cuda.current_stream()

    split = not args.plain
    tuned = atom.autotune(symmetric=True, split=split)  # work partition, outside the timed region

    def step(split_k=split):
        # J on the handle's second stream, concurrent with K (hfg_jk); P = C C^T is symmetric
        atom.jk(Pd, Jd, Kd, stream=stream, symmetric=True, split=split_k, split_j=split_k)

    # plain FP64 beside the split form: rate and the split error on this density
    plain = None
    if split:
        K64 = torch.empty_like(Pd)
        for _ in range(args.warmup):
            step(False)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(args.steps):
            step(False)
        p1.record(stream)
        torch.cuda.synchronize()
        K64.copy_(Kd)
        J64 = Jd.clone()
        step(True)
        torch.cuda.synchronize()
        dK = Kd - K64
        dJ = Jd - J64
        plain = {"value": args.steps / (p0.elapsed_time(p1) * 1e-3), "unit": UNIT,
                 "ms_per_step": p0.elapsed_time(p1) / args.steps,
                 "split_error_vs_fp64": {
                     "k_max_rel": float(dK.abs().max() / K64.abs().max()),
                     "j_max_rel": float(dJ.abs().max() / J64.abs().max()),
                     "coulomb_energy_abs_eh": abs(0.5 * float((Pd * dJ).sum())),
                     "exchange_energy_abs_eh": abs(0.5 * float((Pd * dK).sum())),
                     "exchange_energy_eh": 0.5 * float((Pd * K64).sum())}}
        del K64, dK, J64, dJ

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # the tile stage (the roofline's kernel) bracketed by events on its
    # launch stream inside the timed region; the other classes are timed in
    # an extra pass after it (fewer events between the timed launches)
    atom.profile_enable(KERNELS_PER_STEP * args.steps + 16)
    atom.profile_classes(["k_tiles"])
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
    ms = e0.elapsed_time(e1)
    prof = atom.profile_read(reset=True)
    atom.profile_classes(None)
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    prof_all = atom.profile_read(reset=True)
    atom.profile_enable(0)
    clocks = clk.summary()
    if dist is not None:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = ws * args.steps / (ms * 1e-3)

    # end to end through the host-pointer drop-ins (pinned host buffers)
    def pinned():
        return torch.empty((nbf, nbf), dtype=torch.float64, pin_memory=True).numpy().T
    Ph, Jh, Kh = pinned(), pinned(), pinned()
    Ph[...] = P
    atom.jk_host(Ph, J=Jh, K=Kh, symmetric=True, split=split, split_j=split)
    ne = args.e2e_steps
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(ne):
        atom.jk_host(Ph, J=Jh, K=Kh, symmetric=True, split=split, split_j=split)
    te = max(time.perf_counter() - t0, 1e-30)
    if dist is not None:
        t = torch.tensor([te], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        te = float(t.item())
    h2d, d2h = atom.host_copy_bytes()  # counted by the library from the copies it issued
    e2e = {"value": ws * ne / te if ne else None, "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "steps": ne,
           "path": "hfg_jk_host (pinned host P, J, K; P symmetric, so its lower column blocks cross the "
                   "link and the device mirrors the rest; J copied back while K builds; same J and K "
                   "forms as value)",
           "host_link_gbs": host_link_rates(torch, Ph, Kh)}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    work = atom.work()
    n_off, ms_off = prof["k_tiles"]
    off_ms = ms_off / max(n_off, 1)
    kflops = work["k_offdiag_sym_flops"] + work["k_diag_sym_flops"]
    achieved = kflops / (off_ms * 1e-3) / 1e12  # FP64-equivalent algorithmic FLOPs
    peak = fp64_peak_tflops(torch)
    fp32 = fp32_peak_tflops(torch)
    hbm_peak = measured_peaks().get("hbm_gbs")
    kernel_ms = {k: (v[1] / max(v[0], 1)) for k, v in prof_all.items()}
    if split:
        # executed tensor work: the bf16 digit-plane MMAs of one exchange
        mma = atom.tc_work(symmetric=True)
        tc_rate = mma / (off_ms * 1e-3) / 1e12
        mp = measured_peaks()
        if mp.get("bf16_tflops"):
            tpeak, tsrc = float(mp["bf16_tflops"]), "MEASURED_PEAKS.json bf16_tflops (cuBLAS bf16 GEMM, burst)"
        else:
            tpeak = hg.tc_peak(2, 4096)["tflops"]
            tsrc = "measured in this run: this library's tcgen05 bf16 MMA loop (hfg_tc_peak)"
        roofline = {
            "bound": "tensor", "kernel": "k_tiles_tc + k_diag_tc (the exchange tile stage)", "achieved": tc_rate,
            "peak": tpeak, "unit": "TFLOP/s", "frac": tc_rate / tpeak if tpeak else None,
            "peak_source": tsrc,
            "mma_flops_per_launch": mma,
            "achieved_fp64_equivalent_tflops": achieved,
            "fp64_peak_tflops": peak, "fp32_peak_tflops": fp32,
            "achieved_note": "tensor FLOPs actually issued (digit-plane products, 55 per batch of 8 output blocks) "
                             "over the tile stage's time; the stage is bound by the digit conversions on the CUDA "
                             "cores (about half of the issue slots busy in ncu), not by the tensor pipe",
        }
    else:
        roofline = {"bound": "fp64", "kernel": "k_tiles", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                    "frac": achieved / peak if peak else None,
                    "peak_source": "measured in this run: cuBLAS DGEMM 4096^3 (no FP64 figure in MEASURED_PEAKS.json)"}
    roofline.update({
        "flops_per_launch": kflops, "ms_per_launch": off_ms,
        "traffic": None,
        "traffic_note": "DRAM bytes are not measurable inside this run; the ncu captures of the tile kernel "
                        "(profiles/) give them per launch",
        "hbm": {"achieved_gbs": (work["k_bytes"] / 2) / (off_ms * 1e-3) / 1e9, "peak_gbs": hbm_peak,
                "note": "the tile kernel reads P once; HBM is not its bound"},
        "kernel_ms_per_launch": kernel_ms,
        "kernel_ms_note": "per-class event brackets from an extra pass of the same steps after the timed region "
                          "(the timed region brackets the tile stage only); J runs on a second stream beside K, "
                          "so its brackets include the overlap",
    })
    cpu1 = None
    if args.cpu_seconds > 0:
        cpu_rate, cpu_n, cpu_dt, cpu_threads = cpu_reference_builds(args.cpu_seconds, 1000)
        # one thread, the reference's own test setting (OMP_NUM_THREADS=1)
        r1, n1, dt1, _ = cpu_reference_builds(0.0, 1, 1, threads=1)
        cpu_reference_builds(0.0, 0, 0, threads=0)  # restore every core
        cpu1 = {"value": r1, "unit": UNIT, "cores": 1, "kind": "port",
                "sample": f"{n1} full-size Kr J+K build in {dt1:.1f} s (oracle, one OpenMP thread)"}
    else:
        cpu_rate, cpu_n, cpu_dt, cpu_threads = None, 0, 0.0, host_cores()
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": FORMS["split" if split else "plain"]["dtype"], "data": "synthetic",
        "config": {"workload": WORKLOAD, "nbf": nbf, "parallelism": f"replicas x{ws}",
                   "autotune": tuned,
                   "inputs_vs_l2": "P is 202 MB > 129 MB L2: no flush needed"},
        "roofline": roofline,
        "form": FORMS["split" if split else "plain"]["form"],
        "plain_fp64": plain,
        "cpu_baseline": {"value": cpu_rate, "unit": UNIT, "cores": cpu_threads, "kind": "port",
                         "sample": f"{cpu_n} full-size Kr J+K builds in {cpu_dt:.1f} s (oracle, OpenMP)"},
        "cpu_baseline_1thread": cpu1,
        "e2e": e2e,
        "clocks": clocks,
        "gpu_launches": LAUNCHES_PER_STEP["split" if split else "plain"] * args.steps,
    }
    if args.n2:
        del Pd, Jd, Kd
        atom.close()
        torch.cuda.empty_cache()
        out["n2_diatomic"] = n2_summary(hg, torch)
    print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def _percentile(v, q):
    v = sorted(v)
    if not v:
        return None
    k = (len(v) - 1) * q
    lo, hi = int(np.floor(k)), int(np.ceil(k))
    return v[lo] + (v[hi] - v[lo]) * (k - lo)


def run_engine_batch(jobs, n_workers, budget_gb, split):
    """Submit every job at once; returns (wall_s, results)."""
    import helfem_gb300 as hg
    eng = hg.Engine(n_workers=n_workers, hbm_budget_gb=budget_gb)
    t0 = time.perf_counter()
    ids = [eng.submit(j["Z"], j["bval"], j["lval"], j["mval"], j["nela"], j["nelb"], j["method"], j["restricted"],
                      nnodes=j["nnodes"], symmetry=2, split=split, l_occ=j["l_occ"]) for j in jobs]
    res = [eng.wait(i) for i in ids]
    wall = time.perf_counter() - t0
    eng.close()
    return wall, res


def run_scf_batch(args):
    """Batched atomic SCF (seeded synthetic atoms after the 512-atom batch
    configuration, scaled by --atoms / --nel-max): solves/s of the engine
    (concurrent workers, split-precision exchange) against the plain path
    (one solve at a time, FP64 exchange) on the same atoms."""
    import torch
    torch.cuda.set_device(0)
    from helfem_gb300 import workloads as wl
    jobs = wl.batch_atoms(args.atoms, seed=2024, zmax=86, nel_range=(10, args.nel_max))
    warm = wl.batch_atoms(2, seed=1, zmax=10, nel_range=(10, 10))
    run_engine_batch(warm, 2, 180.0, True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        wall, res = run_engine_batch(jobs, args.workers, 180.0, True)
    wall_p, res_p = run_engine_batch(jobs, 1, 180.0, False)
    ok = [r for r in res if r["status"] == 2 and r["converged"]]
    both = [(a, b) for a, b in zip(res, res_p) if a["status"] == 2 and b["status"] == 2]
    dE = max((abs(a["Etot"] - b["Etot"]) for a, b in both), default=None)
    # the largest energy differences against the plain path, with the atom
    top = sorted(((abs(a["Etot"] - b["Etot"]), j) for j, (a, b) in zip(jobs, zip(res, res_p))
                  if a["status"] == 2 and b["status"] == 2), key=lambda x: -x[0])[:5]
    lat = [r["total_ms"] for r in res]
    svc = [r["setup_ms"] + r["scf_ms"] for r in res]
    out = {
        "metric": "atom-SCF solves/s (batched)", "value": len(jobs) / wall, "unit": "solves/s", "n_gpus": 1,
        "steps": 1, "warmup": 1, "ms_per_step": wall * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{len(jobs)} seeded atoms: Z 1-86, {10}-{args.nel_max} elements, nodes "
                               "{10,13,15,17}, Rmax 40-80, lmax by occupied shells, HF / LDA(Slater+PW92) 50/50, "
                               "restricted, Madelung occupations per l (spherically averaged), per-(l,m) blocks, to 1e-10 Eh",
                   "workers": args.workers, "hbm_budget_gb": 180.0},
        "converged": len(ok), "failed": len(res) - len(ok),
        "failures": sorted(set(f"Z={j['Z']}: {r['error']}" for j, r in zip(jobs, res) if r["status"] != 2)),
        "iterations_mean": float(np.mean([r["iterations"] for r in res])),
        "latency_ms": {"p50": _percentile(lat, 0.5), "p99": _percentile(lat, 0.99)},
        "service_ms": {"p50": _percentile(svc, 0.5), "p99": _percentile(svc, 0.99)},
        "setup_ms": {"p50": _percentile([r["setup_ms"] for r in res], 0.5),
                     "p99": _percentile([r["setup_ms"] for r in res], 0.99),
                     "sum": float(sum(r["setup_ms"] for r in res)),
                     "form": "host tables + device tabulation and upload, per solve"},
        "scf_phase_ms_sum": {k: float(sum(r["phase_ms"][k] for r in res)) for k in res[0]["phase_ms"]},
        "plain_path": {"value": len(jobs) / wall_p, "unit": "solves/s", "form": "one solve at a time, FP64 exchange",
                       "latency_ms_p99": _percentile([r["total_ms"] for r in res_p], 0.99)},
        "speedup_vs_plain": wall_p / wall,
        "max_abs_dE_vs_plain_eh": dE,
        "largest_dE_vs_plain": [{"dE_eh": d, "Z": j["Z"], "method": j["method"], "nnodes": j["nnodes"],
                                 "elements": len(j["bval"]) - 1} for d, j in top],
        "clocks": clk.summary(),
    }
    print(json.dumps(out), flush=True)


def run_fock_batch(args):
    """Fock builds (J + K) over the seeded batch atoms (the 512-atom batch
    draws, scaled by --atoms / --nel-max): per atom a density P = C C^T from
    min(18, nbf) orthonormalised N(0,1) columns, every build timed alone with
    CUDA events after an L2 flush (256 MB written), split and plain FP64 forms
    on the same handle; builds/s = builds / summed build time, and the split
    J and K errors against the plain ones per atom."""
    import torch
    torch.cuda.set_device(0)
    import helfem_gb300 as hg
    from helfem_gb300 import workloads as wl
    jobs = wl.batch_atoms(args.atoms, seed=2024, zmax=86, nel_range=(10, args.nel_max))
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(2024)
    reps = max(1, args.steps)
    t = {"split": 0.0, "plain": 0.0}
    nb = 0
    worst = {"k_max_rel": 0.0, "j_max_rel": 0.0, "exchange_energy_abs_eh": 0.0}
    per_size = []
    with ClockSampler(torch.cuda.current_device()) as clk:
        for j in jobs:
            atom = hg.Atom(j["Z"], j["bval"], j["lval"], j["mval"], nnodes=j["nnodes"])
            n = atom.nbf
            C = torch.randn(n, min(18, n), dtype=torch.float64, device="cuda", generator=gen)
            C, _ = torch.linalg.qr(C)
            P = (C @ C.T).contiguous()
            del C
            out = {f: (torch.empty_like(P), torch.empty_like(P)) for f in t}
            ms_atom = {}
            for f in ("plain", "split"):
                Jd, Kd = out[f]
                sp = f == "split"
                for _ in range(max(1, args.warmup)):
                    atom.coulomb(P, Jd, stream, split=sp)
                    atom.exchange(P, Kd, stream, symmetric=True, split=sp)
                ms = 0.0
                for _ in range(reps):
                    flush.zero_()
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    atom.coulomb(P, Jd, stream, split=sp)
                    atom.exchange(P, Kd, stream, symmetric=True, split=sp)
                    e1.record(stream)
                    torch.cuda.synchronize()
                    ms += e0.elapsed_time(e1)
                t[f] += ms
                ms_atom[f] = ms / reps
            nb += reps
            (J64, K64), (Js, Ks) = out["plain"], out["split"]
            worst["k_max_rel"] = max(worst["k_max_rel"], float((Ks - K64).abs().max() / K64.abs().max()))
            worst["j_max_rel"] = max(worst["j_max_rel"], float((Js - J64).abs().max() / J64.abs().max()))
            worst["exchange_energy_abs_eh"] = max(worst["exchange_energy_abs_eh"],
                                                  abs(0.5 * float((P * (Ks - K64)).sum())))
            per_size.append((n, ms_atom["plain"], ms_atom["split"]))
            del P, out, J64, K64, Js, Ks
            atom.close()
    torch.cuda.empty_cache()
    per_size.sort()
    big = per_size[len(per_size) // 2:]
    res = {
        "metric": "Fock builds/s (J+K, batched atoms)", "value": nb / (t["split"] * 1e-3), "unit": "builds/s",
        "n_gpus": 1, "steps": reps, "warmup": args.warmup, "ms_per_step": t["split"] / nb,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": FORMS["split"]["dtype"],
        "data": "synthetic",
        "config": {"workload": f"{len(jobs)} seeded atoms (the batch draws): Z 1-86, 10-{args.nel_max} elements, "
                               "nodes {10,13,15,17}, Rmax 40-80, lmax by occupied shells; P = C C^T, "
                               "min(18, nbf) orthonormal columns",
                   "timing": "each build alone, CUDA events, L2 flushed (256 MB) before every build"},
        "plain": {"value": nb / (t["plain"] * 1e-3), "unit": "builds/s", "form": "plain FP64 J and K"},
        "split_over_plain": t["plain"] / t["split"],
        "split_over_plain_larger_half": sum(p for _, p, _ in big) / sum(q for _, _, q in big),
        "nbf_range": [per_size[0][0], per_size[-1][0]],
        "split_error_vs_fp64_worst": worst,
        "form": FORMS["split"]["form"],
        "clocks": clk.summary(),
    }
    print(json.dumps(res), flush=True)


def run_serve(args):
    """Streaming atomic SCF requests with Poisson arrivals (seeded): p50/p99
    latency from submission to result and completed solves/s."""
    import torch
    torch.cuda.set_device(0)
    import helfem_gb300 as hg
    from helfem_gb300 import workloads as wl
    rng = np.random.default_rng(11)
    jobs = wl.stream_atoms(args.requests, seed=7, zmax=86, nel_range=(10, args.nel_max))
    gaps = rng.exponential(1.0 / args.rate, size=len(jobs))

    def serve(n_workers, split):
        eng = hg.Engine(n_workers=n_workers, hbm_budget_gb=180.0)
        t0 = time.perf_counter()
        ids, t_next = [], t0
        for j, g in zip(jobs, gaps):
            t_next += g
            dt = t_next - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            ids.append(eng.submit(j["Z"], j["bval"], j["lval"], j["mval"], j["nela"], j["nelb"], j["method"],
                                  j["restricted"], nnodes=j["nnodes"], symmetry=2, split=split, l_occ=j["l_occ"]))
        res = [eng.wait(i) for i in ids]
        wall = time.perf_counter() - t0
        eng.close()
        return wall, res

    warm = wl.batch_atoms(2, seed=1, zmax=10, nel_range=(10, 10))
    run_engine_batch(warm, 2, 180.0, True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        wall, res = serve(args.workers, True)
    wall_p, res_p = serve(1, False) if args.plain_serve else (None, None)
    lat = [r["total_ms"] for r in res]
    lat_p = [r["total_ms"] for r in res_p] if res_p else []
    out = {
        "metric": "atom-SCF solves/s (streaming, Poisson arrivals)", "value": len(jobs) / wall, "unit": "solves/s",
        "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": wall * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{len(jobs)} requests at {args.rate}/s: Z 1-86, charge -1..+3, RHF/UHF, "
                               f"HF/LDA/PBE, 10-{args.nel_max} elements of 15 nodes",
                   "workers": args.workers, "hbm_budget_gb": 180.0},
        "latency_ms": {"p50": _percentile(lat, 0.5), "p99": _percentile(lat, 0.99)},
        "setup_ms": {"p50": _percentile([r["setup_ms"] for r in res], 0.5),
                     "p99": _percentile([r["setup_ms"] for r in res], 0.99)},
        "failed": sum(1 for r in res if r["status"] != 2),
        "converged": sum(1 for r in res if r["status"] == 2 and r["converged"]),
        "plain_path": None if not res_p else {
            "value": len(jobs) / wall_p, "unit": "solves/s",
            "form": "same request stream, one solve at a time, FP64 exchange",
            "latency_ms": {"p50": _percentile(lat_p, 0.5), "p99": _percentile(lat_p, 0.99)}},
        "speedup_vs_plain": wall_p / wall if res_p else None,
        "max_abs_dE_vs_plain_eh": max((abs(a["Etot"] - b["Etot"]) for a, b in zip(res, res_p)
                                       if a["status"] == 2 and b["status"] == 2), default=None) if res_p else None,
        "failures": sorted(set(r["error"] for r in res if r["status"] != 2)),
        "failed_requests": [{"Z": j["Z"], "electrons": j["nela"] + j["nelb"], "method": j["method"],
                             "restricted": j["restricted"], "elements": len(j["bval"]) - 1,
                             "iterations": r["iterations"]}
                            for j, r in zip(jobs, res) if r["status"] != 2][:24],
        "clocks": clk.summary(),
    }
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------- N2 diatomic
N2_WORKLOAD = ("N2 diatomic J+K Fock build: R=2.074 bohr, 30 mu-elements to mu_max=arccosh(40/Rhalf) "
               "(exponential grid), 15-node LIP, l<=12 for m=0..3 (Nang=79, Nrad=420, Nbf=33114), L<=26; "
               "P from 7 seeded N(0,1) doubly occupied orbitals drawn inside m-blocks (5 sigma, 1 pi+, 1 pi-), "
               "Loewdin-orthonormal in the block overlap; K from the spin density P/2")


def n2_setup(hg, host_only=False, nelem=30, lmax=12):
    d = hg.Diatomic.from_grid(7, 7, 2.074, nelem, [lmax] * 4, host_only=host_only)
    idx = d.pure_indices()
    mv = d.mval[idx // d.nrad]
    rng = np.random.default_rng(12345)
    P = np.zeros((d.nbf, d.nbf), order="F")
    act = np.zeros(d.nang * d.nang, np.uint8)
    for m, nocc in ((0, 5), (1, 1), (-1, 1)):
        sel = np.where(mv == m)[0]
        S = d.one_electron_block("S", m)
        C = rng.standard_normal((len(sel), nocc))
        w, v = np.linalg.eigh(C.T @ S @ C)
        C = C @ (v @ np.diag(w ** -0.5) @ v.T)
        P[np.ix_(sel, sel)] = 2.0 * (C @ C.T)
        shells = np.where(d.mval == m)[0]
        for i in shells:
            for l in shells:
                act[i + l * d.nang] = 1
    return d, P, act


def n2_oracle(d):
    """The oracle's exchange (the reference's loop structure) fed with the
    product's tables of the diatomic handle d: (DiatomicOracle, tables)."""
    import oracle
    from oracle import diatomic as dia
    nel, nn = d.dims["nel"], d.dims["nnodes"]
    nlm = d.dims["nlm"]
    lm, P0, P2, Q0, Q2, cdB, cds = [], [], [], [], [], [], []
    ni = [nn] * (nel - 1) + [nn - 1]
    for i in range(nlm):
        rows = {k: [] for k in range(4)}
        fB, fS = [], []
        for e in range(nel):
            for which in range(4):
                L, M, t = d.tables(which, i, e)
                rows[which].append(np.asarray(t[:ni[e], :ni[e]]))
            _, _, B, s = d.tables(4, i, e)
            keep = np.array([a + b * nn for b in range(ni[e]) for a in range(ni[e])])
            fB.append(np.asarray(B[np.concatenate([keep, nn * nn + keep])]))
            fS.append(s)
        lm.append((L, M))
        P0.append(rows[0]); P2.append(rows[1]); Q0.append(rows[2]); Q2.append(rows[3])
        cdB.append(fB); cds.append(fS)
    _, LM = dia.lm_maps(d.lval, d.mval)
    first = np.array([e * (nn - 1) for e in range(nel)])
    D = dia.DiatomicTables(d.Z1, d.Z2, d.Rhalf, nn, np.zeros(nel + 1), np.asarray(d.lval, int),
                           np.asarray(d.mval, int), d.nrad, first, np.array(ni), lm, LM, P0, P2, Q0, Q2, cdB, cds)
    return oracle.DiatomicOracle(D), D


def n2_cpu_sample(d, P, seconds):
    """The oracle's exchange (the reference's loop structure, OpenMP) on a
    bounded sample of output blocks, scaled to a full build by the work model;
    J not included."""
    import oracle
    F, D = n2_oracle(d)
    Pd = np.asfortranarray(D.expand(0.5 * P))
    nang = d.nang
    mv = np.asarray(d.mval)
    active = [j + k * nang for k in range(nang) for j in range(nang) if mv[j] == mv[k] and abs(mv[j]) <= 3]
    # a spread sample of active output blocks, grown until it takes `seconds`
    rng = np.random.default_rng(7)
    order = list(rng.permutation(active))
    n, spent, done = 4, 0.0, []
    while order and spent < seconds:
        batch, order = order[:n], order[n:]
        t0 = time.perf_counter()
        F.exchange_dummy_blocks(Pd, batch)
        spent += time.perf_counter() - t0
        done += batch
        n *= 2
    act = np.zeros(nang * nang, np.uint8)
    for i in range(nang):
        for l in range(nang):
            act[i + l * nang] = mv[i] == mv[l] and abs(mv[i]) <= 1
    mask = np.zeros(nang * nang, np.uint8)
    mask[done] = 1
    w_s = d.work(act, mask)
    w_t = d.work(act)
    tot = lambda w: w["k_offdiag_flops"] + w["k_diag_flops"] + w["k_recouple_flops"]
    k_sec = spent * tot(w_t) / max(tot(w_s), 1.0)
    return k_sec, len(done), len(active), spent, oracle.dlib().ora_num_threads_d()


def run_n2_reference(args):
    import helfem_gb300 as hg
    rank, ws, local, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    d, P, _ = n2_setup(hg, host_only=True)
    per = []
    for i in range(args.warmup + args.steps):
        k_sec, ns, na, spent, thr = n2_cpu_sample(d, P, max(args.cpu_seconds, 1.0) / 4)
        if i >= args.warmup:
            per.append(k_sec)
    mean = sum(per) / len(per)
    out = {"impl": "reference", "metric": METRIC, "value": 1.0 / mean, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": N2_WORKLOAD, "inputs_vs_l2": "host run (no GPU)"},
           "cpu_baseline": {"value": 1.0 / mean, "unit": UNIT, "cores": thr, "kind": "port",
                            "sample": "per step: oracle exchange on a sample of active output blocks, scaled "
                                      "by the work model to one K build"},
           "e2e": {"value": 1.0 / mean, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_n2(args):
    import torch
    import helfem_gb300 as hg

    rank, ws, local, dist = dist_setup(args.gpus)
    if dist is not None:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    d, P, act = n2_setup(hg, nelem=args.n2_elements, lmax=args.n2_lmax)
    nbf = d.nbf
    Pd = torch.from_numpy(P.ravel(order="F")).cuda()
    Pa = 0.5 * Pd
    Jd, Kd = torch.empty_like(Pd), torch.empty_like(Pd)
    stream = torch.cuda.current_stream()
    evs = []
    split = not args.plain

    def step(timed=False, split_k=split):
        if timed:
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            e[0].record(stream)
        d.coulomb(Pd, Jd, stream=stream)
        if timed:
            e[1].record(stream)
        d.exchange(Pa, Kd, symmetric=True, stream=stream, split=split_k)
        if timed:
            e[2].record(stream)
            evs.append(e)

    # plain FP64 beside the split form: its K time and the split error
    plain = None
    if split:
        step(split_k=False)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        d.exchange(Pa, Kd, symmetric=True, stream=stream)
        p1.record(stream)
        torch.cuda.synchronize()
        K64 = Kd.clone()
        d.exchange(Pa, Kd, symmetric=True, stream=stream, split=True)
        torch.cuda.synchronize()
        dK = Kd - K64
        plain = {"exchange_ms": p0.elapsed_time(p1),
                 "split_error_vs_fp64": {"k_max_rel": float(dK.abs().max() / K64.abs().max()),
                                         "exchange_energy_abs_eh": abs(float((Pa * dK).sum())),
                                         "exchange_energy_eh": float((Pa * K64).sum())}}
        del K64, dK

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step(True)
        e1.record(stream)
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
    ms = e0.elapsed_time(e1)
    if dist is not None:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    j_ms = statistics.mean(e[0].elapsed_time(e[1]) for e in evs)
    k_ms = statistics.mean(e[1].elapsed_time(e[2]) for e in evs)
    value = ws * args.steps / (ms * 1e-3)
    # DFT form of the same Fock build: J plus the PBE potential on the pure-m
    # grid (the XC path of the reference's diatomic driver at symmetry >= 1)
    xid, cid = hg.parse_xc("gga_x_pbe-gga_c_pbe")
    Hx = torch.empty_like(Pd)
    en = torch.zeros(2, dtype=torch.float64, device="cuda")
    d.xc(xid, cid, Pd, Hx, energies=en, stream=stream)  # first call builds the grid
    torch.cuda.synchronize()
    x0, x1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nx = 5
    x0.record(stream)
    for _ in range(nx):
        d.xc(xid, cid, Pd, Hx, energies=en, stream=stream)
    x1.record(stream)
    torch.cuda.synchronize()
    xc_ms = x0.elapsed_time(x1) / nx
    dft = {"functional": "gga_x_pbe-gga_c_pbe (restricted)", "xc_ms": xc_ms, "coulomb_ms": j_ms,
           "fock_builds_per_s": 1e3 / (j_ms + xc_ms), "exc_eh": float(en[0]), "nel_on_grid": float(en[1]),
           "grid": "5 nnodes Chebyshev mu points per element x (4 lmax + 12) Chebyshev cos(nu) points, "
                   "phi analytic", "path": "hfg_diatomic_coulomb + hfg_diatomic_xc (device pointers)"}
    del Hx
    Ecoul = 0.5 * float((Pd * Jd).sum())
    Exx = 0.5 * float((Pa * Kd).sum()) * 2.0
    # end to end through the host-pointer drop-ins (pinned host buffers)
    def pinned():
        return torch.empty((nbf, nbf), dtype=torch.float64, pin_memory=True).numpy().T
    Ph, Pah, Jh, Kh = pinned(), pinned(), pinned(), pinned()
    Ph[...] = P
    Pah[...] = 0.5 * P
    ne = max(1, min(args.e2e_steps, 2))
    t0 = time.perf_counter()
    for _ in range(ne):
        d.coulomb_host(Ph, out=Jh)
        d.exchange_host(Pah, out=Kh, symmetric=True, split=split)
    te = time.perf_counter() - t0
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    w = d.work(act)
    kflops = w["k_offdiag_sym_flops"] + w["k_diag_sym_flops"] + w["k_recouple_sym_flops"]
    peak = fp64_peak_tflops(torch)
    achieved = kflops / (k_ms * 1e-3) / 1e12
    cpu = None
    if args.cpu_seconds > 0:
        k_sec, ns, na, spent, thr = n2_cpu_sample(d, P, args.cpu_seconds)
        cpu = {"value": 1.0 / k_sec, "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"oracle exchange on {ns} of {na} active output blocks in {spent:.1f} s, "
                         f"scaled by the work model to one K build ({k_sec:.1f} s); J not included"}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": N2_WORKLOAD if (args.n2_elements, args.n2_lmax) == (30, 12) else
                   f"reduced N2 case: {args.n2_elements} mu-elements, l<={args.n2_lmax} (profiling)", "nbf": nbf, "ndummy": d.ndummy, "parallelism": f"replicas x{ws}",
                   "inputs_vs_l2": "P is 8.8 GB > 129 MB L2: no flush needed"},
        "form": ("split precision (FP32-pair contraction, FP64 recombination)" if split else "plain FP64")
                + ", symmetric exchange mode",
        "kernel_ms": {"coulomb": j_ms, "exchange": k_ms},
        "plain_fp64": plain,
        "dft": dft,
        "energies_eh": {"coulomb": Ecoul, "exchange": Exx},
        "roofline": ({"bound": "fp32", "kernel": "dk_tiles_split (whole exchange call)",
                      "achieved": achieved * 12.0, "peak": fp32_peak_tflops(torch), "unit": "TFLOP/s",
                      "frac": achieved * 12.0 / fp32_peak_tflops(torch),
                      "achieved_fp64_equivalent_tflops": achieved, "fp64_peak_tflops": peak,
                      "achieved_note": "FP32 rate = FP64-equivalent algorithmic FLOP rate x 12 FP32 instructions "
                                       "per emulated multiply-add",
                      "flops_per_launch": kflops, "ms_per_launch": k_ms,
                      "peak_source": "measured in this run: cuBLAS SGEMM 8192^3 with TF32 off", "traffic": None}
                     if split else
                     {"bound": "fp64", "kernel": "dk_tiles (whole exchange call)", "achieved": achieved,
                      "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                      "flops_per_launch": kflops, "ms_per_launch": k_ms,
                      "peak_source": "measured in this run: cuBLAS DGEMM 4096^3", "traffic": None}),
        "cpu_baseline": cpu,
        "e2e": {"value": ws * ne / te, "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * nbf * nbf,
                "d2h_bytes_per_step": 2 * 8 * nbf * nbf, "steps": ne,
                "path": "hfg_diatomic_coulomb_host + hfg_diatomic_exchange_host (pinned host P, J, K)"},
        "clocks": clk.summary(),
        "gpu_launches": args.steps * 11,  # J: contract, tiles, scatter; K: expand, norms, act,
                                           # entry_act, compact, tiles, fixup, gather
    }
    print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="seconds of oracle builds for cpu_baseline (0 skips it)")
    ap.add_argument("--e2e-steps", type=int, default=10, help="host-pointer drop-in steps (0 skips)")
    ap.add_argument("--plain", action="store_true", help="time the plain FP64 form only")
    ap.add_argument("--no-n2", dest="n2", action="store_false",
                    help="skip the N2 diatomic Fock-build object of the default line")
    ap.add_argument("--workload", default="fock", choices=["fock", "fock-batch", "scf-batch", "serve", "n2"])
    ap.add_argument("--atoms", type=int, default=32)
    ap.add_argument("--nel-max", type=int, default=30)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--no-plain-serve", dest="plain_serve", action="store_false",
                    help="serve workload: skip the plain-path replay of the stream (long runs)")
    ap.add_argument("--n2-elements", type=int, default=30, help="N2 workload: mu-elements (30 = the benchmark)")
    ap.add_argument("--n2-lmax", type=int, default=12, help="N2 workload: l_max for m = 0..3 (12 = the benchmark)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference" and args.workload == "n2":
        run_n2_reference(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "fock-batch":
        run_fock_batch(args)
    elif args.workload == "scf-batch":
        run_scf_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "n2":
        run_n2(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
