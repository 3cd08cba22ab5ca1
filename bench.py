"""Benchmark of the DBSR_MAT3 Hamiltonian-block assembly on GB300.

One step = one assembled channel-pair matrix: hch zeroed, the R^k/S^k
tables rebuilt, and every coefficient list of the workload passed through
Gen_matrix (R^k direct/exchange for k=0..10, S^k structures 6 and 8 for
both PQ types).  Default workload: 400 B-splines (ks=9, P order 8, Q order
9), r_max=40, Z=26, 20 bound orbitals, 120 channels (7260 blocks of
800x800 FP64 = 37.2 GB), about 1.8e6 unique angular coefficients over 5%
of the (channel pair, k) slots -- seeded synthetic data, no public dataset
(see dbsr_gb300/synth.py).

Output: one JSON line (rank 0).  value = algorithmic GFLOP/s of the
reference's own loop counts (2 x multiply-adds of convol + density) per
assembled matrix, with the lists and orbitals resident in device memory;
e2e = the same with the lists copied from pinned host memory inside the
timed region and the assembled matrix copied back to pinned host memory.
``--impl reference`` times the CPU restatement of the reference
(oracle/, the reference itself needs a Fortran compiler and an external
library that this image lacks) on a bounded sample of the same workload
with all host cores.
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

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

METRIC = "H-block assembly s and GFLOP/s: mixed-prec vs FP64 on GPU at ≤1e-10 rel err"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="split", choices=["plain", "split", "factor"])
    p.add_argument("--no-compare", action="store_true",
                   help="skip the FP64 comparison runs (plain and factored FP64 assemblies)")
    p.add_argument("--block-errors", default=None,
                   help="write the per-block max/RMS relative errors to this CSV file")
    p.add_argument("--scale", type=float, default=1.0, help="fraction of the 2e6 entries")
    p.add_argument("--nch", type=int, default=120)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-graph", action="store_true", help="skip the captured-graph replays")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU sample")
    p.add_argument("--workload", default="config1",
                   choices=["config1", "batch", "basis", "hf", "backward"],
                   help="config1: one 120-channel matrix; batch: independent J-blocks with "
                        "their own grids through dbsrg_gen_batch")
    p.add_argument("--nblocks", type=int, default=64)
    p.add_argument("--nch-max", type=int, default=300)
    p.add_argument("--batch-group", type=int, default=8, help="J-blocks run concurrently")
    p.add_argument("--window-gb", type=float, default=2.0, help="device window per J-block")
    p.add_argument("--tune", default=None,
                   help="batch: autotune the exchange chunk size first, recording into this table")
    p.add_argument("--rows-entries", type=float, default=1e4)
    return p.parse_args()


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# DRAM traffic of k_xfused per algorithmic byte: ncu (dram__bytes_read.sum +
# dram__bytes_write.sum, --clock-control none, k_xfused launches only) on the
# 40-channel case, divided by the algorithmic bytes the same launches state;
# the traffic scales with the hch tiles a launch touches, so the ratio is
# carried to the 120-channel launches.  At 40 channels the 129 MB L2 holds a
# larger share of a launch's tiles than at 120, so the carried figure is a
# lower estimate of the full-size traffic.  None: no traffic reported.
XFUSED_TRAFFIC_PER_ALGORITHMIC_BYTE = 0.882
XFUSED_TRAFFIC_SOURCE = ("ncu over the 35 k_xfused launches of one 40-channel step "
                         "(ns=400, 4.2 GB matrix): 5.087 GB read + 1.938 GB written "
                         "against 7.967 GB stated algorithmic bytes; ratio carried "
                         "to the 120-channel launches (a lower estimate)")


def d2h_gbs(torch, dev, nbytes=4 << 30, dst=None) -> float:
    """Device-to-host copy rate of this machine into pinned memory (best of 3):
    into a new buffer, or into the first nbytes of `dst` (a pinned tensor)."""
    src = torch.empty(nbytes // 8, dtype=torch.float64, device=dev)
    dst = (torch.empty(nbytes // 8, dtype=torch.float64).pin_memory() if dst is None
           else dst[: nbytes // 8])
    best = 1e9
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - t0)
    del src, dst
    return nbytes / best / 1e9


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def fp64_peak_tflops(torch, dev) -> float:
    """Measured FP64 dense-matmul throughput (cuBLAS DGEMM 8192^3), the
    denominator of the FP64 contraction kernels."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    torch.cuda.empty_cache()
    return 2 * n ** 3 / best / 1e12


# ---------------------------------------------------------------------------
# Lists of the CPU sample: R^k direct and exchange at k = 0, 5, 10 and the S^k
# structures 6 and 8 of both PQ types at v = 5 and 11, so that every
# contraction kind, the smallest and largest multipoles and the Breit
# tables of the highest order are in it.
SAMPLE_SEGS = {}
for _k in (0, 5, 10):
    SAMPLE_SEGS[(2, 3, _k)] = 2
    SAMPLE_SEGS[(2, 4, _k)] = 1
for _v in (5, 11):
    for _it in (6, 8, 16, 18):
        SAMPLE_SEGS[(3, _it, _v)] = 1


def convol_flops(w, L, nseg, nent):
    """Reference loop FLOPs (2 x multiply-adds) of nseg segments holding nent
    entries of list L: one convol per segment and PQ type plus the density
    accumulations."""
    ns, ks = w.ns, w.ks
    Ts = ks * ns - ks * (ks - 1) // 2
    Tn = (2 * ks - 1) * ns - ks * (ks - 1)
    if L.icase == 2:
        return (4 * nseg * 2 * (Ts * Ts if L.itype == 3 else Tn * Tn) +
                4 * nent * 2 * ns * (ks if L.itype == 3 else ns))
    return nseg * 2 * Tn * Tn + nent * 2 * ns * ((2 * ks - 1) if L.itype % 10 <= 7 else ns)


def list_kind(L) -> str:
    """Contraction kind of a list: R^k direct / exchange, S^k direct /
    exchange.  The reference's loops run at very different rates per kind
    (the direct 's' convol walks its table with a stride of ns), so CPU
    times are extrapolated kind by kind."""
    if L.icase == 2:
        return "R direct" if L.itype == 3 else "R exchange"
    return "S direct" if L.itype % 10 <= 7 else "S exchange"


def full_flops_by_kind(w) -> dict:
    out = {}
    for L in w.lists:
        if L.icase not in (2, 3) or L.n == 0:
            continue
        nseg = int(np.count_nonzero(np.r_[True, L.k1[1:] != L.k1[:-1]]))
        k = list_kind(L)
        out[k] = out.get(k, 0.0) + convol_flops(w, L, nseg, L.n)
    return out


def cpu_sample(w, budget_s: float, threads: int = 1):
    """Time the CPU restatement on a bounded sample of the workload: the
    first segments of the SAMPLE_SEGS lists (with the tables they need), and
    extrapolate per algorithmic FLOP.  Each list's first entry runs once
    untimed before its sample so that its tables are built outside the
    contraction timing.  Returns (GFLOP/s, seconds per full matrix,
    description, oracle matrix, the sublists in the order they were added)."""
    from dbsr_gb300 import synth
    from oracle import oracle as O

    g = O.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = O.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    t0 = time.perf_counter()
    flops, t_seg, t_tab, n_tab, desc, added = 0.0, 0.0, 0.0, 0, [], []
    kf, kt = {}, {}  # sampled FLOPs and seconds per kind
    for L in w.lists:
        key = (L.icase, L.itype, L.kpol)
        if key not in SAMPLE_SEGS or L.n == 0:
            continue
        segs = np.flatnonzero(np.r_[True, L.k1[1:] != L.k1[:-1]])
        nseg = min(SAMPLE_SEGS[key], segs.size)
        end = segs[nseg] if nseg < segs.size else L.n
        warm = synth.CList(L.icase, L.itype, L.kpol, L.k1[:1], L.k2[:1], L.k3[:1], L.k4[:1],
                           L.c[:1])
        sub = synth.CList(L.icase, L.itype, L.kpol, L.k1[:end], L.k2[:end], L.k3[:end],
                          L.k4[:end], L.c[:end])
        tw = time.perf_counter()
        m.gen_matrix(warm.icase, warm.itype, warm.kpol, warm.k1, warm.k2, warm.k3, warm.k4,
                     warm.c)
        t_tab += time.perf_counter() - tw  # the table builds (4 R or 1 S) + one entry
        n_tab += 4 if L.icase == 2 else 1
        ts = time.perf_counter()
        m.gen_matrix(sub.icase, sub.itype, sub.kpol, sub.k1, sub.k2, sub.k3, sub.k4, sub.c)
        dts = time.perf_counter() - ts
        t_seg += dts
        added += [warm, sub]
        f = convol_flops(w, L, nseg, end)
        flops += f
        kf[list_kind(L)] = kf.get(list_kind(L), 0.0) + f
        kt[list_kind(L)] = kt.get(list_kind(L), 0.0) + dts
        desc.append(f"{key}:{nseg}seg")
        if time.perf_counter() - t0 > budget_s:
            break
    fl = synth.algorithmic_flops(w)
    n_tables = 4 * (w.mk + 1) + 2 * (w.mk + 2)
    full = full_flops_by_kind(w)
    full_s = sum(F * kt[k] / kf[k] for k, F in full.items()) + t_tab / max(n_tab, 1) * n_tables
    rates = ", ".join(f"{k} {kf[k] / kt[k] / 1e9:.2f}" for k in sorted(kf))
    return fl["total"] / full_s / 1e9, full_s, (
        f"oracle (CPU restatement, -O2, 1 thread) on {', '.join(desc)} ({t_seg:.1f} s; GFLOP/s "
        f"by kind: {rates}) plus {n_tab} table builds ({t_tab:.1f} s); extrapolated kind by kind "
        f"to the full matrix ({fl['total'] / 1e12:.2f} TFLOP) and its {n_tables} tables: "
        f"{full_s:.0f} s per matrix"), m, added


def oracle_sample_errors(a, m, added, forms):
    """Per-block max and RMS relative errors, against the oracle's matrix m,
    of the same sublists assembled on the device in each of `forms`
    ({name: precision}); the blocks are those the sublists touch."""
    blocks = [b for b in range(m.iicc) if np.abs(m.hch[:, :, b]).max() > 0]
    out = {}
    for name, prec in forms.items():
        a.set_async(False)
        a.set_precision(prec)
        a.zero_matrix()
        for L in added:
            a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
        emax, erms = [], []
        for b in blocks:
            ich, jch = np.argwhere(np.asarray(a.icc) == b + 1)[0] + 1
            h = a.get_block(int(ich), int(jch))
            r = m.hch[:, :, b]
            d = h - r
            emax.append(float(np.abs(d).max() / np.abs(r).max()))
            erms.append(float(np.sqrt((d * d).sum() / (r * r).sum())))
        out[name] = {"max_rel_err": max(emax), "rms_rel_err": max(erms),
                     "blocks_within_1e-10": int(sum(e <= 1e-10 for e in emax))}
    out["blocks"] = len(blocks)
    out["lists"] = sorted({f"{L.icase}/{L.itype}/k{L.kpol}" for L in added})
    out["reference"] = ("CPU oracle (the C restatement of the reference loops) on the first "
                        "segments of the sampled lists, all blocks they touch; max = "
                        "max|d|/max|ref|, rms = ||d||_2/||ref||_2 per block, worst block")
    return out


def _ref_worker(w, items, conn):
    """Reference-arm worker: builds the tables of its own work items once
    (timed), as a serial reference run builds each table once (irka cache,
    dbsr_lib_dbs.f90:2919-2925), then contracts its items at every "go"."""
    from oracle import oracle as O

    g = O.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = O.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    lists = {(L.icase, L.itype, L.kpol): L for L in w.lists}
    t0 = time.perf_counter()
    ntab = 0
    for key in sorted({it[0] for it in items}):
        L = lists[key]
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1[:1], L.k2[:1], L.k3[:1], L.k4[:1],
                     L.c[:1] * 0.0)
        ntab += 4 if L.icase == 2 else 1
    conn.send((time.perf_counter() - t0, ntab))
    while conn.recv() == "go":
        kt = {}
        for key, lo, hi in items:
            L = lists[key]
            s = slice(lo, hi)
            t1 = time.perf_counter()
            m.gen_matrix(L.icase, L.itype, L.kpol, L.k1[s], L.k2[s], L.k3[s], L.k4[s], L.c[s])
            kt[list_kind(L)] = kt.get(list_kind(L), 0.0) + time.perf_counter() - t1
        conn.send(kt)


def reference_arm(args, w):
    """The reference's CPU path (its C restatement: the Fortran reference
    cannot be built here) on all host cores.  One worker process per core
    holds a fixed share of a bounded sample of segments of every kind (R^k
    direct and exchange, S^k structures 6 and 8 of both PQ types) and builds
    the tables of its share once; every step runs all shares concurrently.
    The value is the whole matrix's algorithmic FLOPs over its extrapolated
    time on these cores: the contraction at the sampled rate (median step)
    plus the matrix's tables at the measured time per table, shared by the
    cores."""
    import multiprocessing as mp

    from dbsr_gb300 import synth

    cores = os.cpu_count() or 1
    # segments per sampled list, in list order
    per_list = {2: max(2, cores), 3: max(2, cores // 2)}
    items, kf = [], {}
    for L in w.lists:
        key = (L.icase, L.itype, L.kpol)
        if key not in SAMPLE_SEGS or L.n == 0:
            continue
        segs = list(np.flatnonzero(np.r_[True, L.k1[1:] != L.k1[:-1]])) + [L.n]
        take = min(max(1, per_list[L.icase] // (2 if L.itype == 4 else 1)), len(segs) - 1)
        for i in range(take):
            lo, hi = int(segs[i]), int(segs[i + 1])
            items.append((key, lo, hi, convol_flops(w, L, 1, hi - lo)))
            kf[list_kind(L)] = kf.get(list_kind(L), 0.0) + items[-1][3]
    flops = sum(it[3] for it in items)
    # contiguous shares of about equal FLOPs (few tables per worker)
    nproc = min(cores, len(items))
    shares, cur, acc = [], [], 0.0
    for it in items:
        cur.append(it[:3])
        acc += it[3]
        if acc >= flops * (len(shares) + 1) / nproc and len(shares) < nproc - 1:
            shares.append(cur)
            cur = []
    shares.append(cur)
    shares = [sh for sh in shares if sh]
    ctx = mp.get_context("spawn")
    procs, conns = [], []
    for sh in shares:
        a, b = ctx.Pipe()
        p = ctx.Process(target=_ref_worker, args=(w, sh, b), daemon=True)
        p.start()
        procs.append(p)
        conns.append(a)
    tabs = [c.recv() for c in conns]
    times, kt = [], {}
    for s in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        for c in conns:
            c.send("go")
        got = [c.recv() for c in conns]
        if s >= args.warmup:
            times.append(time.perf_counter() - t0)
            for g in got:
                for k, v in g.items():
                    kt[k] = kt.get(k, 0.0) + v / args.steps
    for c in conns:
        c.send("stop")
    for p in procs:
        p.join(timeout=30)
    dt = statistics.median(times)
    nw = len(shares)
    t_table = sum(t for t, _ in tabs) / max(1, sum(n for _, n in tabs))
    fl = synth.algorithmic_flops(w)["total"]
    n_tables = 4 * (w.mk + 1) + 2 * (w.mk + 2)
    # per kind: core-seconds per sampled FLOP (all workers running together,
    # so memory contention is in it), the whole matrix's FLOPs of that kind
    # spread over the workers; plus its tables, spread likewise
    full = full_flops_by_kind(w)
    full_s = sum(F * kt[k] / kf[k] for k, F in full.items()) / nw + n_tables * t_table / nw
    v = fl / full_s / 1e9
    rates = ", ".join(f"{k} {kf[k] / kt[k] / 1e9:.2f}" for k in sorted(kf))
    sample = (f"oracle restatement in {nw} worker processes ({cores} cores): per step "
              f"{len(items)} segments of R^k direct/exchange at k=0,5,10 and S^k 6/8 (both PQ "
              f"types) at v=5,11, {flops / 1e9:.1f} GFLOP algorithmic, median step "
              f"{dt:.2f} s (GFLOP/s per core by kind: {rates}); plus {n_tables} table builds at "
              f"{t_table:.2f} s each shared by the workers; extrapolated kind by kind to the "
              f"whole matrix ({fl / 1e12:.2f} TFLOP): {full_s:.0f} s per matrix")
    return {
        "metric": METRIC, "value": v, "unit": "GFLOP/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "impl": "reference",
        "config": {"workload": w.name, "sample": "R^k direct+exchange k=0,5,10; S^k 6/8 v=5,11",
                   "s_per_matrix_extrapolated": full_s},
        "cpu_baseline": {"value": v, "unit": "GFLOP/s", "cores": nw, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def block_errors(torch, hs, hp, nblk, ms, chunk=64):
    """Per-block max and RMS relative errors of hs against hp, both
    (ms, ms, nblk) column-major on the device: max|hs-hp| / max|hp| and
    ||hs-hp||_2 / ||hp||_2 over each ms x ms block."""
    emax, erms = [], []
    hs3 = hs.view(nblk, ms * ms)
    hp3 = hp.view(nblk, ms * ms)
    for b0 in range(0, nblk, chunk):
        s, p = hs3[b0:b0 + chunk], hp3[b0:b0 + chunk]
        d = s - p
        dm = d.abs().amax(dim=1)
        pm = p.abs().amax(dim=1)
        dr = d.square().sum(dim=1).sqrt()
        pr = p.square().sum(dim=1).sqrt()
        emax.append(torch.where(pm > 0, dm / pm.clamp_min(1e-300), dm))
        erms.append(torch.where(pr > 0, dr / pr.clamp_min(1e-300), dr))
    return torch.cat(emax).cpu().numpy(), torch.cat(erms).cpu().numpy()


def fp64_compare(args, a, w, step, dl, timed, torch, dev, world):
    from dbsr_gb300 import FACTOR_FP64, PLAIN_FP64, SPLIT_BF16, synth

    ms, nblk = a.ms, w.iicc
    fl = synth.algorithmic_flops(w)["total"]
    hs = torch.empty(nblk * ms * ms, dtype=torch.float64, device=dev)
    step(dl)  # the headline form again: the e2e leg reused the device matrix as window slots
    a.get_matrix(out=hs)
    out = {}
    if args.precision == "split":
        a.set_precision(FACTOR_FP64)
        step(dl)
        t = timed(lambda: step(dl), 1)
        out["factor_fp64_s_per_matrix"] = t
    a.set_precision(PLAIN_FP64)
    step(dl)
    t = timed(lambda: step(dl), 1)
    out["plain_fp64_s_per_matrix"] = t
    out["plain_fp64_gflops"] = world * fl / t / 1e9
    hp = torch.empty_like(hs)
    a.get_matrix(out=hp)
    a.set_precision({"split": SPLIT_BF16, "factor": FACTOR_FP64}[args.precision])
    emax, erms = block_errors(torch, hs, hp, nblk, ms)
    del hs, hp
    torch.cuda.empty_cache()
    if args.block_errors:
        with open(args.block_errors, "w") as f:
            f.write("block,max_rel,rms_rel\n")
            for b in range(nblk):
                f.write(f"{b + 1},{emax[b]:.3e},{erms[b]:.3e}\n")
    out["reference"] = ("plain FP64 GPU assembly of the same inputs (held to the CPU oracle at "
                        "1e-12 per block by the parity tests)")
    out["blocks"] = int(nblk)
    out["max_rel_err"] = {"max": float(emax.max()), "p99": float(np.percentile(emax, 99)),
                          "median": float(np.median(emax))}
    out["rms_rel_err"] = {"max": float(erms.max()), "p99": float(np.percentile(erms, 99)),
                          "median": float(np.median(erms))}
    out["blocks_within_1e-10"] = int((emax <= 1e-10).sum())
    return out


# ---------------------------------------------------------------------------
def batch_main(args, rank, world, local):
    """The batched form: independent J-parity blocks, each with its own grid,
    orbitals and matrix, through dbsrg_gen_batch_streamed in groups of
    --batch-group blocks run concurrently (one host thread and one stream
    each).  The full batch (about 1.15 TB in the reference layout) exceeds the
    device, so every block holds a window of at most --window-gb of its
    matrix and each assembled window is copied to pinned host memory (the
    streamed output).  Step: per group, the assemblers built (grid, orbitals,
    window), every list run window by window with each window read out, the
    assemblers closed -- tables and pair potentials are built inside the
    step."""
    # eight contexts of four or five streams each: the default of eight
    # hardware work queues would make unrelated streams wait behind one
    # another (set before the process's first CUDA call)
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    import torch

    from dbsr_gb300 import FACTOR_FP64, PLAIN_FP64, SPLIT_BF16, Assembler, synth
    from dbsr_gb300.api import gen_batch_streamed

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    ws = synth.config3(nblocks=args.nblocks, nch_max=args.nch_max, rows_entries=args.rows_entries,
                       seed=1237 + 1000 * rank)
    prec = {"plain": PLAIN_FP64, "split": SPLIT_BF16, "factor": FACTOR_FP64}[args.precision]
    lists = []
    for w in ws:  # device-resident lists
        dl = []
        for L in w.lists:
            t = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (L.k1, L.k2, L.k3, L.k4)]
            dl.append((L.icase, L.itype, L.kpol, *t,
                       torch.from_numpy(np.ascontiguousarray(L.c)).to(dev)))
        lists.append(dl)
    G = max(1, args.batch_group)
    wbytes = int(args.window_gb * 1e9)
    # per context a page-locked host window in huge pages (dbsrg_host_alloc):
    # measured on one box, 10.5-10.6 s per batch against 11.8-12.6 s with
    # torch's pinned windows and 6.3-6.4 s with device windows (the host
    # copies are what the batch waits on)
    from dbsr_gb300.api import HostMatrix

    hostm = [HostMatrix(wbytes // 8) for _ in range(G)]
    host = [h.array for h in hostm]
    torch.cuda.synchronize()
    stats = {"d2h": 0, "windows": 0}
    from dbsr_gb300 import autotune

    tuning = autotune.lookup(0, local, mode="batch") or None  # the batch's own entry

    def step():
        for g0 in range(0, len(ws), G):
            gw, gl = ws[g0:g0 + G], lists[g0:g0 + G]
            asm = []
            for w in gw:
                a = Assembler(w.t, w.ks, w.ksp, w.ksq, device=local, tuning=tuning)
                a.set_orbitals(w.pq, w.ipbs)
                blk = (2 * w.ns) ** 2 * 8
                a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk,
                               window=max(1, min(w.iicc, wbytes // blk)))
                a.set_precision(prec)
                asm.append(a)

            def consume(i, blo, nb, ptr):
                ms = 2 * gw[i].ns
                asm[i].get_matrix(out=host[i][: nb * ms * ms])
                stats["d2h"] += nb * ms * ms * 8
                stats["windows"] += 1

            gen_batch_streamed(asm, gl, consume)
            for a in asm:
                a.close()

    if args.tune:  # autotune the batch's exchange chunk size, record it, use it
        def run_batch(t):
            nonlocal tuning
            tuning = t
            step()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            step()
            torch.cuda.synchronize()
            return time.perf_counter() - t0

        choice = autotune.tune_batch(run_batch, log=lambda m: print(m, file=sys.stderr))
        autotune.record(choice, 0, local, note=f"config3 batch nch<={args.nch_max}",
                        path=args.tune)
        tuning = {"xchunk": choice["xchunk"]}
    for _ in range(args.warmup):
        step()
    clk = Clocks(local)
    clk.start()
    if pg is not None:
        pg.barrier()
    torch.cuda.synchronize()
    stats["d2h"] = stats["windows"] = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    if pg is not None:
        pg.barrier()
    dt = (time.perf_counter() - t0) / args.steps
    clocks = clk.stop()
    if pg is not None:
        tt = torch.tensor([dt], device=dev)
        pg.all_reduce(tt, op=pg.ReduceOp.MAX)
        dt = float(tt.item())
    flops = sum(synth.algorithmic_flops(w)["total"] for w in ws)
    value = world * flops / dt / 1e9
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "plain" else "bf16-split/f32-acc/f64",
            "data": "synthetic",
            "config": {"workload": f"config3 batch: {len(ws)} J-blocks, ns 150..450, "
                                   f"nch 10..{args.nch_max} log-uniform, k=0..8, "
                                   f"{args.rows_entries:g} entries per channel row",
                       "precision": args.precision,
                       "blocks": int(sum(w.iicc for w in ws)),
                       "entries": int(sum(L.n for w in ws for L in w.lists)),
                       "matrix_gb": sum(w.iicc * (2 * w.ns) ** 2 * 8 for w in ws) / 1e9,
                       "algorithmic_tflop": flops / 1e12,
                       "group": G, "window_gb": args.window_gb, "tuning": tuning,
                       "output": "every window copied to huge-page pinned host memory inside the step",
                       "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                       "timing": "host wall clock around the synchronised steps",
                       "parallelism": f"replicas x{world}"},
            "s_per_batch": dt, "d2h_bytes_per_step": stats["d2h"] // max(1, args.steps),
            "windows_per_step": stats["windows"] // max(1, args.steps), "clocks": clocks,
        }
        print(json.dumps(out), flush=True)
    if pg is not None:
        pg.destroy_process_group()


def basis_main(args, rank, world, local):
    """The channel basis of the write-out on the
    120-channel matrix: the split-form assembly, dbsrg_orth_channels (DBS_ORTH:
    every channel orthogonal to the bound orbitals of its
    kappa), then dbsrg_diag_channels
    (one generalized eigenproblem per channel, cuSOLVER sygvd; B = the
    B-spline overlap fppqq, the first and last B-spline of P and Q removed,
    every eigenvalue kept) and dbsrg_channel_basis (D_i^T H D_j for the 7140
    off-diagonal blocks: split-BF16 tcgen05 products, then again with cuBLAS
    DGEMM on the same matrix for comparison).  Timed once each after a
    warm-up, host wall clock around synchronised calls."""
    import torch

    from dbsr_gb300 import PLAIN_FP64, SPLIT_BF16, Assembler, synth

    torch.cuda.set_device(local)
    w = synth.config1(scale=args.scale, nch=args.nch, breit=True)
    a = Assembler(w.t, w.ks, w.ksp, w.ksq, device=local)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(SPLIT_BF16)
    ms, ns, nch = a.ms, a.ns, w.nch
    B = a.grid_array("fppqq").reshape(ms, ms, order="F")
    bdiag = torch.from_numpy(np.asfortranarray(np.repeat(B[:, :, None], nch, axis=2))
                             .ravel(order="F")).cuda()
    iprm = np.ones((ms, nch), dtype=np.int32, order="F")
    for comp in range(2):
        iprm[comp * ns, :] = 0
        iprm[comp * ns + ns - 1, :] = 0
    sol = torch.empty(ms * ms * nch, dtype=torch.float64, device="cuda")

    def assemble():
        a.zero_matrix()
        for L in w.lists:
            a.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
        a.sync()

    # DBS_ORTH (called before Diag_channels, sub1.f90:142-146): every channel
    # orthogonal to the bound orbitals of its kappa
    iort = np.zeros((w.nbf, nch), dtype=np.int32, order="F")
    for ich, kc in enumerate(w.kappa_ch):
        for j in range(w.nbound):
            if w.ipbs[j] == 0 and w.kappa_bound[j] == kc:
                iort[j, ich] = 1
    out = {}
    for rep in range(2):  # warm-up, then timed
        assemble()
        torch.cuda.synchronize()
        to0 = time.perf_counter()
        a.orth_channels(iort)
        torch.cuda.synchronize()
        to1 = time.perf_counter()
        t0 = time.perf_counter()
        _, ev, nsol = a.diag_channels(bdiag, iprm)  # solutions to `sol` below
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        # the solutions stay on the device: rerun into the device buffer
        check_nsol = nsol.copy()
        L = a._L
        rc = L.dbsrg_diag_channels(a._h, bdiag.data_ptr(), iprm.ctypes.data, -1e30, 1e30, 0.0,
                                   sol.data_ptr(), ev.ctypes.data, nsol.ctypes.data)
        assert rc == 0 and np.array_equal(nsol, check_nsol)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        a.channel_basis(sol, nsol)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        out = {"orth_channels_s": to1 - to0, "diag_channels_s": t1 - t0,
               "diag_channels_device_out_s": t2 - t1, "channel_basis_s": t3 - t2}
    # the same transformation by cuBLAS DGEMM (the FP64 forms' path) on the
    # same assembled matrix and solutions, and the split products' error
    # against it on a sample of blocks (max over each block's elements,
    # relative to the block's largest element)
    rng = np.random.default_rng(5)
    pairs = [(i, j) for i in range(2, nch + 1) for j in range(1, i) if w.icc[i - 1, j - 1] > 0]
    sample = [pairs[q] for q in rng.choice(len(pairs), min(48, len(pairs)), replace=False)]
    split_blocks = [a.get_block(i, j) for i, j in sample]
    assemble()
    a.orth_channels(iort)
    a.set_precision(PLAIN_FP64)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    a.channel_basis(sol, nsol)
    torch.cuda.synchronize()
    out["channel_basis_dgemm_s"] = time.perf_counter() - t0
    a.set_precision(SPLIT_BF16)
    worst = 0.0
    for (i, j), sb in zip(sample, split_blocks):
        db = a.get_block(i, j)
        worst = max(worst, float(np.abs(sb - db).max() / max(np.abs(db).max(), 1e-300)))
    out["split_vs_dgemm_max_rel"] = worst
    out["split_vs_dgemm_blocks"] = len(sample)
    # DBS_ORTH work: per block with na (row) and nb (column) orbitals, one
    # read-modify-write of the block (16 B per element) and 4 (na + nb) ms^2
    # FP64 operations (T1, T2 and the update)
    nort = iort[:w.nbound].sum(axis=0)
    ob = ofl = 0.0
    for ich in range(nch):
        for jch in range(ich + 1):
            if w.icc[ich, jch] > 0 and (nort[ich] or nort[jch]):
                ob += 16.0 * ms * ms
                ofl += 4.0 * (nort[ich] + nort[jch]) * ms * ms
    out.update({"orth_blocks_gb": ob / 1e9, "orth_gbs": ob / out["orth_channels_s"] / 1e9,
                "orth_fp64_gflops": ofl / out["orth_channels_s"] / 1e9,
                "orth_orbitals_per_channel": float(nort.mean())})
    fl = 0.0
    for ich in range(1, nch + 1):
        for jch in range(1, ich):
            if w.icc[ich - 1, jch - 1] > 0:
                ni, nj = int(nsol[ich - 1]), int(nsol[jch - 1])
                fl += 2.0 * ni * ms * ms + 2.0 * ni * nj * ms
    out.update({"metric": "channel basis (Diag_channels + Record_matrix transform) s",
                "unit": "s", "value": out["diag_channels_device_out_s"] + out["channel_basis_s"],
                "higher_is_better": False, "dtype": "f64",
                "config": {"workload": f"config1 matrix: ns={ns} nch={nch}", "blocks": w.iicc,
                           "solutions_per_channel": int(np.median(nsol))},
                "basis_fp64_tflop": fl / 1e12,
                "basis_split_tflops": fl / out["channel_basis_s"] / 1e12,
                "basis_dgemm_tflops": fl / out["channel_basis_dgemm_s"] / 1e12})
    print(json.dumps(out), flush=True)
    a.close()


def backward_main(args, rank, world, local):
    """The differentiation workload: E = sum over 5e4 entries of c R^k(a,b;c,d)
    over 30 bound orbitals (ns=300, Z=18, k=0..8) and dE/dpq (30 x 2 x 300)
    through dbsrg_backward, with every table-derived quantity released before
    each step, so the cell moments and diagonal cells are recomputed inside
    the timed region.  One warm-up step, then `--steps` timed steps (host
    wall clock around synchronised calls)."""
    import torch

    from dbsr_gb300 import Assembler, synth

    torch.cuda.set_device(local)
    w = synth.config4()
    a = Assembler(w.t, w.ks, w.ksp, w.ksq, device=local)
    a.set_orbitals(w.pq, w.ipbs)

    def step():
        a.release_tables()
        return a.backward(w.k, w.i1, w.i2, w.i3, w.i4, w.coef)

    E, G = step()
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        E, G = step()
    dt = (time.perf_counter() - t0) / steps
    out = {"metric": "energy functional and gradient (dbsrg_backward) s per evaluation",
           "unit": "s", "value": dt, "higher_is_better": False, "dtype": "f64",
           "config": {"workload": "config4: ns=300 Z=18 30 orbitals k=0..8 5e4 entries",
                      "entries": int(len(w.coef)), "gradient": list(G.shape)},
           "energy": E, "gradient_norm": float(np.linalg.norm(G)),
           "moments_recomputed": True}
    print(json.dumps(out), flush=True)
    a.close()


def hf_main(args, rank, world, local):
    """The SCF potential matrices of DBSR_HF: hf_matrix
    (hf_matrix.f90:2-70, Coulomb part) of all 30 orbitals of the config-4
    basis (ns=300, Z=18, k=0..8), i.e. one SCF iteration's potentials,
    through dbsrg_hf_matrix in the split and plain FP64 forms.  Coefficients
    coef(i,j,k) uniform in [-1,1] where the energy expression's a(i,j,k) and
    b(i,j,k) allow them (hf_MOD_energy.f90:20-57: k even and
    k <= (j_i + j_j) for a; i != j, k + l_i + l_j even and
    |j_i - j_j| <= k <= j_i + j_j for b).  Every iteration sets the orbitals
    again, so what depends on them is rebuilt.  One warm-up iteration, then
    `--steps` timed iterations (host wall clock around synchronised calls)."""
    import torch

    from dbsr_gb300 import PLAIN_FP64, SPLIT_BF16, Assembler, synth

    torch.cuda.set_device(local)
    w = synth.config4(n_entries=8)
    norb, kmax = w.pq.shape[2], 8
    kap = [k for _, k in synth.TARGET_ORBITALS[:norb]]
    ls = [synth.l_kappa(k) for k in kap]
    j2 = [synth.j2_kappa(k) for k in kap]
    rng = np.random.Generator(np.random.Philox(4242))
    coef = rng.uniform(-1.0, 1.0, (norb, norb, kmax + 1))
    A = np.zeros((norb, norb, kmax + 1))
    B = np.zeros((norb, norb, kmax + 1))
    for i in range(norb):
        for j in range(norb):
            for k in range(kmax + 1):
                if k % 2 == 0 and k <= (j2[i] + j2[j]) // 2:
                    A[i, j, k] = coef[max(i, j), min(i, j), k]
                if i != j and (k + ls[i] + ls[j]) % 2 == 0 and \
                        abs(j2[i] - j2[j]) // 2 <= k <= (j2[i] + j2[j]) // 2:
                    B[i, j, k] = coef[min(i, j), max(i, j), k]
    ns, ks = w.ns, w.ks
    Ts = ks * ns - ks * (ks - 1) // 2
    # reference loop work per orbital: per table type and k, convol case 1
    # ('s','s': Ts^2 multiply-adds) when a direct coefficient is nonzero and
    # case 4 (four updates per table element: 4 Ts^2) when an exchange one is
    fl = 0.0
    for i in range(norb):
        for k in range(kmax + 1):
            fl += 4 * 2.0 * Ts * Ts * (A[i, :, k] != 0).any()
            fl += 4 * 2.0 * 4 * Ts * Ts * (B[i, :, k] != 0).any()
    out = {}
    dev_out = torch.empty(4 * ns * ns, dtype=torch.float64, device="cuda")
    for name, prec in (("split", SPLIT_BF16), ("plain", PLAIN_FP64)):
        a = Assembler(w.t, w.ks, w.ksp, w.ksq, device=local)
        a.set_orbitals(w.pq, np.zeros(norb, np.int32))
        a.alloc_matrix(1, np.ones((1, 1), np.int32, order="F"), 1, kmax)
        a.set_precision(prec)

        def iteration():
            # new orbitals every SCF iteration: everything derived from them
            # (pair potentials, far fields) is rebuilt; the tables depend on
            # the grid only and stay cached, as the reference's do
            a.set_orbitals(w.pq, np.zeros(norb, np.int32))
            for i in range(norb):
                a.hf_matrix(i + 1, A[i], B[i], 1.0, out=dev_out)
            torch.cuda.synchronize()

        iteration()
        steps = max(1, args.steps)
        t0 = time.perf_counter()
        for _ in range(steps):
            iteration()
        dt = (time.perf_counter() - t0) / steps
        out[name] = {"s_per_iteration": dt, "ms_per_orbital": dt / norb * 1e3,
                     "gflops": fl / dt / 1e9}
        a.close()
    out.update({"metric": "SCF potential matrices (hf_matrix, all orbitals) s per iteration",
                "unit": "s", "value": out["split"]["s_per_iteration"], "higher_is_better": False,
                "dtype": "bf16-split/f32-acc/f64",
                "config": {"workload": f"config4 basis: ns={ns} Z=18 {norb} orbitals k=0..{kmax}",
                           "direct_terms": int((A != 0).sum()), "exchange_terms": int((B != 0).sum())},
                "reference_loop_gflop_per_iteration": fl / 1e9,
                "split_vs_plain": out["plain"]["s_per_iteration"] / out["split"]["s_per_iteration"]})
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    from dbsr_gb300 import synth

    if args.workload == "batch" and args.impl == "ours":
        return batch_main(args, rank, world, local)
    if args.workload == "basis" and args.impl == "ours":
        return basis_main(args, rank, world, local)
    if args.workload == "hf" and args.impl == "ours":
        return hf_main(args, rank, world, local)
    if args.workload == "backward" and args.impl == "ours":
        return backward_main(args, rank, world, local)
    w = synth.config1(scale=args.scale, nch=args.nch)

    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(reference_arm(args, w)), flush=True)
        return

    import torch

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
        pg = dist

    from dbsr_gb300 import FACTOR_FP64, PLAIN_FP64, SPLIT_BF16, Assembler

    a = Assembler(w.t, w.ks, w.ksp, w.ksq, device=local)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision({"plain": PLAIN_FP64, "split": SPLIT_BF16, "factor": FACTOR_FP64}[args.precision])
    # device-resident lists
    dl = []
    for L in w.lists:
        t = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (L.k1, L.k2, L.k3, L.k4)]
        c = torch.from_numpy(np.ascontiguousarray(L.c)).to(dev)
        dl.append((L.icase, L.itype, L.kpol, *t, c))
    torch.cuda.synchronize()

    # asynchronous mode: the host-side set-up of each list overlaps the
    # kernels of the previous one; sync() ends every step, so the step's
    # time covers all of its kernels
    a.set_async(True)

    # every step rebuilds the tables, cell data, far fields and pair
    # potentials (invalidated, rebuilt in the memory they occupied)
    def step(lists):
        a.zero_matrix()
        a.invalidate_tables()
        for (ic, it, kp, k1, k2, k3, k4, c) in lists:
            a.gen_matrix(ic, it, kp, k1, k2, k3, k4, c)
        a.sync()

    def barrier():
        torch.cuda.synchronize()
        if pg is not None:
            pg.barrier()

    def timed(fn, n):
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        barrier()
        dt = e0.elapsed_time(e1) / 1e3 / n
        if pg is not None:
            t = torch.tensor([dt], device=dev)
            pg.all_reduce(t, op=pg.ReduceOp.MAX)
            dt = float(t.item())
        return dt

    for _ in range(args.warmup):
        step(dl)
    l0 = a.launches
    clk = Clocks(local)
    clk.start()
    dt = timed(lambda: step(dl), args.steps)
    clocks = clk.stop()
    launches = (a.launches - l0) // max(1, args.steps)

    fl = synth.algorithmic_flops(w)
    value = world * fl["total"] / dt / 1e9

    # per-kernel device time of one instrumented step (outside the timed region)
    a.timing(True)
    step(dl)
    rep = a.timing_report()
    a.timing(False)
    top = max(rep.items(), key=lambda kv: kv[1][1])
    tot_ms = sum(v[1] for v in rep.values())

    peaks, peak_kind = measured_peaks()
    # executed work of the kernels that state it (bytes and FLOPs, FP64 or
    # float-float counted as FP64-equivalent multiply-adds x 2) over their
    # measured time: what the factored step actually executes, beside the
    # reference-loop count of the metric
    kernel_work = {}
    for name, (n_l, ms_l, by_l, fl_l) in sorted(rep.items(), key=lambda kv: -kv[1][1]):
        if by_l <= 0 and fl_l <= 0:
            continue
        sec_l = ms_l / 1e3
        kernel_work[name] = {"ms": round(ms_l, 3), "launches": n_l, "gflop": fl_l / 1e9,
                             "gb": by_l / 1e9, "gflops": fl_l / sec_l / 1e9 if sec_l else None,
                             "gbs": by_l / sec_l / 1e9 if sec_l else None}
    executed = {"tflop_stated": sum(v["gflop"] for v in kernel_work.values()) / 1e3,
                "gb_stated": sum(v["gb"] for v in kernel_work.values()),
                "kernels_stated": sorted(kernel_work),
                "note": ("the kernels above state their executed work (the rest, table "
                         "construction and list bookkeeping, do not); k_xfused counts its "
                         "tensor-core MMA FLOPs, the others FP64-equivalent multiply-adds")}
    if args.precision == "plain":
        p64 = fp64_peak_tflops(torch, dev)
        # algorithmic FLOPs of the contraction kernels (convol) over their time
        conv_ms = sum(rep.get(k, (0, 0.0))[1] for k in ("k_exchange", "k_band_contract"))
        n_top = top[1][0]
        if top[0] in ("k_exchange", "k_band_contract"):
            share = rep[top[0]][1] / max(conv_ms, 1e-9)
            per_launch = fl["convol"] * share / max(n_top, 1)
            achieved = per_launch / (top[1][1] / n_top / 1e3) / 1e12
        else:
            achieved = float("nan")
        roofline = {"bound": "fp64", "kernel": top[0], "achieved": achieved, "peak": p64,
                    "unit": "TFLOP/s", "frac": achieved / p64,
                    "peak_source": "measured cuBLAS DGEMM 8192^3 on this GPU",
                    "traffic": None, "launches": n_top, "avg_launch_ms": top[1][1] / n_top,
                    "share_of_step": top[1][1] / tot_ms}
    else:
        # the dominant kernel with the algorithmic work its launches state:
        # bytes (hch read-modify-write of the tiles it touches) against the
        # measured HBM copy bandwidth, and its tensor-core FLOPs against the
        # sustained bf16 GEMM rate (it runs inside a seconds-long step)
        name, (n_top, ms_top, by_top, fl_top) = top
        sec = ms_top / 1e3
        roofline = {"bound": "hbm", "kernel": name, "achieved": None, "peak": peaks["hbm_gbs"],
                    "unit": "GB/s", "frac": None, "traffic": None, "launches": n_top,
                    "avg_launch_ms": ms_top / max(n_top, 1), "share_of_step": ms_top / tot_ms,
                    "algorithmic_bytes_per_launch": by_top / max(n_top, 1),
                    "peak_source": f"{peak_kind} hbm_gbs (copy)"}
        if by_top > 0:
            roofline["achieved"] = by_top / sec / 1e9
            roofline["frac"] = roofline["achieved"] / peaks["hbm_gbs"]
        # DRAM traffic per launch, like achieved: the algorithmic bytes times
        # the traffic ratio of a small-case capture of the same kernel
        if name == "k_xfused" and XFUSED_TRAFFIC_PER_ALGORITHMIC_BYTE is not None:
            roofline["traffic"] = XFUSED_TRAFFIC_PER_ALGORITHMIC_BYTE * by_top / max(n_top, 1)
            roofline["traffic_over_algorithmic"] = XFUSED_TRAFFIC_PER_ALGORITHMIC_BYTE
            roofline["traffic_source"] = XFUSED_TRAFFIC_SOURCE
        if fl_top > 0:
            tpk = peaks.get("bf16_tflops_sustained", peaks["bf16_tflops"])
            roofline["tensor"] = {"achieved": fl_top / sec / 1e12, "peak": tpk,
                                  "unit": "TFLOP/s", "frac": fl_top / sec / 1e12 / tpk,
                                  "peak_source": f"{peak_kind} bf16_tflops_sustained"}

    # e2e: lists from pinned host memory, matrix back to pinned host memory
    e2e = None
    if not args.no_e2e:
        hl = []
        h2d = 0
        for L in w.lists:
            t = [torch.from_numpy(np.ascontiguousarray(x)).pin_memory() for x in
                 (L.k1, L.k2, L.k3, L.k4)]
            c = torch.from_numpy(np.ascontiguousarray(L.c)).pin_memory()
            h2d += sum(x.numel() * 4 for x in t[:3]) + c.numel() * 8
            hl.append((L.icase, L.itype, L.kpol, *[x.numpy() for x in t], c.numpy()))
        # the output in page-locked huge pages (dbsrg_host_alloc)
        from dbsr_gb300.api import HostMatrix

        hbuf = HostMatrix(w.iicc * a.ms * a.ms)
        hout = torch.from_numpy(hbuf.array)
        hacf = torch.empty(w.iicc * (w.mk + 1), dtype=torch.float64).pin_memory()
        nwin = (w.iicc + a.get_tuning("windows") - 1) // a.get_tuning("windows")

        def e2e_step():
            # dbsrg_assemble_to_host: lists from pinned host memory, the matrix
            # window by window into pinned host memory, each window's copy
            # overlapped with the next window's assembly
            a.invalidate_tables()
            a.assemble_to_host(hl, out=hout, acf=hacf)  # windows: the tuned count

        for _ in range(max(3, args.warmup)):
            e2e_step()
        # the median of single timed steps: on a host whose memory system is
        # shared, some steps copy slower (every sample is reported)
        e2e_samples = [timed(e2e_step, 1) for _ in range(5)]
        dte = float(np.median(e2e_samples))
        # the library's partition: windows of nwin blocks, the first and the
        # last max(1, nwin // 8) blocks (when there are more than two)
        edge = max(1, nwin // 8)
        if w.iicc > 2 * nwin:
            npass, rest = 2, w.iicc - 2 * edge
            npass += -(-rest // nwin)
        else:
            npass = -(-w.iicc // nwin)
        d2h = int((hout.numel() + hacf.numel()) * 8)
        # the copy rate into the output buffer itself, its first and last
        # 4 GB (a buffer partly in far host memory copies slower)
        q = hout.numel() - (4 << 30) // 8
        into = [d2h_gbs(torch, dev, dst=hout), d2h_gbs(torch, dev, dst=hout[q:])]
        del hout
        hbuf.close()
        torch.cuda.empty_cache()
        link = d2h_gbs(torch, dev)
        e2e = {"value": world * fl["total"] / dte / 1e9, "unit": "GFLOP/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": d2h,
               "s_per_matrix": dte, "s_per_matrix_samples": e2e_samples,
               "statistic": "median of 5 single-step samples",
               "host_output": "dbsrg_host_alloc: page-locked, transparent huge pages",
               "api": "dbsrg_assemble_to_host",
               "windows": npass, "window_blocks": nwin, "d2h_gbs_measured": link,
               "d2h_gbs_into_output_first_last": into,
               "d2h_copy_floor_s": d2h / link / 1e9}

    # the same assembly captured as one CUDA graph (dbsrg_graph_capture) and
    # replayed: every table and orbital product rebuilt, the matrix zeroed
    # and assembled; the lists' planning happens once, in the capture
    graph = None
    if not args.no_graph and args.precision != "plain":
        a.set_async(False)
        t0 = time.perf_counter()
        a.graph_capture(dl)
        cap_s = time.perf_counter() - t0
        a.graph_launch()
        g0 = a.launches
        dtg = timed(a.graph_launch, max(3, args.steps))
        graph = {"s_per_matrix": dtg, "value": world * fl["total"] / dtg / 1e9,
                 "unit": "GFLOP/s", "capture_and_first_run_s": cap_s,
                 "launches_per_replay": (a.launches - g0) // max(3, args.steps),
                 "api": "dbsrg_graph_capture + dbsrg_graph_launch"}
        a.graph_release()
        a.set_async(True)

    # FP64 comparison: the same matrix by the factored FP64 and the plain FP64
    # assemblies (the plain one is held to the CPU oracle at 1e-12 by the
    # parity tests), per-block errors of the headline form against plain FP64
    compare = None
    if args.precision != "plain" and not args.no_compare:
        compare = fp64_compare(args, a, w, step, dl, timed, torch, dev, world)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:  # the CPU leg at N = 1 only
        gf, full_s, desc, m_or, added = cpu_sample(w, args.cpu_budget)
        cpu = {"value": gf, "unit": "GFLOP/s", "cores": 1, "kind": "port", "sample": desc,
               "s_per_matrix_extrapolated": full_s}
        # the oracle of that sample is also the checker of the device forms
        # on the same sublists (untimed)
        forms = {"plain_fp64": PLAIN_FP64, "factor_fp64": FACTOR_FP64, "split_bf16": SPLIT_BF16}
        against = oracle_sample_errors(a, m_or, added, forms)
        del m_or
        if compare is None:
            compare = {}
        compare["against_oracle"] = against

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "plain" else "bf16-split/f32-acc/f64",
            "data": "synthetic",
            "config": {"workload": w.name, "precision": args.precision, "ns": w.ns,
                       "nch": w.nch, "blocks": w.iicc, "lists": len(w.lists),
                       "entries": int(sum(L.n for L in w.lists)),
                       "matrix_gb": w.iicc * a.ms * a.ms * 8 / 1e9,
                       "algorithmic_tflop": fl["total"] / 1e12,
                       "l2": "inputs and output larger than L2 (hch 37 GB)",
                       "parallelism": f"replicas x{world}"},
            "s_per_matrix": dt,
            "fp64_comparison": compare,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "graph_replay": graph,
            "clocks": clocks,
            "gpu_launches": int(launches),
            "kernel_ms": {k: round(v[1], 3) for k, v in sorted(rep.items(), key=lambda kv: -kv[1][1])},
            "kernel_work": kernel_work,
            "executed": executed,
            "peaks": {"source": peak_kind, "bf16_tflops": peaks.get("bf16_tflops"),
                      "hbm_gbs": peaks.get("hbm_gbs")},
        }
        print(json.dumps(out), flush=True)
    a.close()
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
