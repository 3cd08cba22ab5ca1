"""Autotuner for the runtime parameters of the assembly (dbsrg_set_tuning).

The parameters do not change results (every block sums the same terms in the
same order); they trade launch granularity against scratch size and
parallelism:

* ``xchunk``  -- segments per pass of the factored exchange: the batch of the
  Z-digit kernel and the number of tile rows of one tensor-core launch;
* ``dchunk``  -- segments per pass of the factored direct contraction;
* ``windows`` -- windows of dbsrg_assemble_to_host (assembly of one window
  overlapped with the copy of the previous one).

``tune()`` times the split form on a workload on the current GPU by
coordinate descent (CUDA-event timed steps after a warm-up) and ``record()``
stores the choice in ``tuning.json`` next to this file, keyed by the device
name and the number of B-splines; ``lookup()`` (used by Assembler) returns
the entry of the nearest recorded grid size for the device, or {}.
``tune_batch()`` times the whole streamed batch (many symmetry blocks at
once, small windows) for each exchange chunk size, a regime of its own; its
entry (``"mode": "batch"``) is read by ``lookup(mode="batch")``.

    python -m dbsr_gb300.autotune            # the 120-channel workload
"""
from __future__ import annotations

import json
import os
import time

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning.json")
NAMES = ("xchunk", "dchunk", "windows")
CANDIDATES = {"xchunk": (64, 128, 256, 512, 1024),
              "dchunk": (512, 1024, 2048, 4096, 8192, 16384),
              "windows": (4, 6, 8, 12, 16, 24)}


def _device_name(device: int) -> str | None:
    try:
        import torch

        if torch.cuda.is_available():
            return torch.cuda.get_device_name(device)
    except Exception:  # noqa: BLE001 -- no torch or no GPU: no recorded tuning
        pass
    return None


def lookup(ns: int, device: int = 0, mode: str = "single") -> dict:
    """Recorded parameters for this GPU and the nearest grid size, or {}."""
    name = _device_name(device)
    if name is None or not os.path.exists(TABLE):
        return {}
    with open(TABLE) as f:
        entries = [e for e in json.load(f).get(name, []) if e.get("mode", "single") == mode]
    if not entries:
        return {}
    best = min(entries, key=lambda e: abs(e["ns"] - ns))
    return {k: best[k] for k in NAMES if k in best}


def tune(w, reps: int = 3, device: int = 0, log=print) -> dict:
    """Coordinate descent over CANDIDATES for workload w (synth.Workload):
    xchunk and dchunk on the device-resident assembly step, windows on
    dbsrg_assemble_to_host into pinned host memory."""
    import numpy as np
    import torch

    from . import SPLIT_BF16
    from .api import Assembler

    dev = torch.device("cuda", device)
    a = Assembler(w.t, w.ks, w.ksp, w.ksq, device=device, tuning=None)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk)
    a.set_precision(SPLIT_BF16)
    dl = [(L.icase, L.itype, L.kpol,
           *[torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (L.k1, L.k2, L.k3, L.k4)],
           torch.from_numpy(np.ascontiguousarray(L.c)).to(dev)) for L in w.lists]
    hl = [(L.icase, L.itype, L.kpol,
           *[torch.from_numpy(np.ascontiguousarray(x)).pin_memory().numpy()
             for x in (L.k1, L.k2, L.k3, L.k4)],
           torch.from_numpy(np.ascontiguousarray(L.c)).pin_memory().numpy()) for L in w.lists]
    hout = torch.empty(w.iicc * a.ms * a.ms, dtype=torch.float64).pin_memory()
    a.set_async(True)

    def step():
        a.zero_matrix()
        a.invalidate_tables()
        for item in dl:
            a.gen_matrix(*item)
        a.sync()

    def e2e():
        a.invalidate_tables()
        a.assemble_to_host(hl, out=hout)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best

    choice = {k: a.get_tuning(k) for k in NAMES}
    for name, fn in (("xchunk", step), ("dchunk", step), ("windows", e2e)):
        times = {}
        for v in CANDIDATES[name]:
            a.set_tuning(name, v)
            times[v] = timed(fn)
            log(f"{name}={v}: {1e3 * times[v]:.1f} ms")
        choice[name] = min(times, key=times.get)
        a.set_tuning(name, choice[name])
        choice[f"{name}_ms"] = round(1e3 * times[choice[name]], 2)
    a.close()
    del hout
    return choice


def tune_batch(run_batch, log=print) -> dict:
    """Exchange chunk size of the streamed batch: run_batch(tuning) times one
    whole batch with those parameters (seconds)."""
    times = {}
    for v in CANDIDATES["xchunk"][1:]:
        times[v] = run_batch({"xchunk": v})
        log(f"batch xchunk={v}: {times[v]:.2f} s")
    best = min(times, key=times.get)
    return {"mode": "batch", "xchunk": best, "batch_s": round(times[best], 3)}


def record(choice: dict, ns: int, device: int = 0, note: str = "", path: str = TABLE) -> None:
    name = _device_name(device)
    table = {}
    if os.path.exists(path):
        with open(path) as f:
            table = json.load(f)
    mode = choice.get("mode", "single")
    entries = [e for e in table.get(name, [])
               if not (e["ns"] == ns and e.get("mode", "single") == mode)]
    entries.append({"ns": ns, **choice, **({"workload": note} if note else {})})
    table[name] = sorted(entries, key=lambda e: e["ns"])
    with open(path, "w") as f:
        json.dump(table, f, indent=1)
        f.write("\n")


def main():
    import argparse

    from . import synth

    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("--nch", type=int, default=120)
    p.add_argument("--batch-block", type=int, default=None,
                   help="tune on block N of the batched workload (synth.config3_block) instead")
    p.add_argument("--scale", type=float, default=1.0)
    p.add_argument("--reps", type=int, default=3)
    p.add_argument("--dry", action="store_true", help="print, do not record")
    p.add_argument("--table", default=TABLE, help="tuning table to record into")
    args = p.parse_args()
    if args.batch_block is not None:
        w = synth.config3_block(args.batch_block)
        note = f"config3 block {args.batch_block} (nch={w.nch})"
    else:
        w = synth.config1(scale=args.scale, nch=args.nch)
        note = f"config1 nch={args.nch} scale={args.scale}"
    choice = tune(w, reps=args.reps)
    print(json.dumps(choice))
    if not args.dry:
        record(choice, int(w.t.size - w.ks), note=note, path=args.table)


if __name__ == "__main__":
    main()
