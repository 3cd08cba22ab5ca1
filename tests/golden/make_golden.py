"""Extract golden vectors from the reference's own example files.

Run as ``python make_golden.py <reference root>`` (or with the root in the
DBSR_REFERENCE environment variable); there is no default location.
Writes ``reference_golden.json`` next to this script:

* knot sequences printed to 16 digits in ``knot.dat`` / ``<name>.knot``
  files, with the grid parameters that generated them (mkgrid_01);
* the "memory=" lines of the DBSR_HF logs (size of the R^k table set,
  dbsr_lib_dbs.f90:1619-1620) and the "memory of DBS_integrals" line of a
  DBSR_MAT log;
* the Dirac-Fock "Coulomb energy" lines of the DBSR_HF logs, together with
  the B-spline orbitals of the matching ``.bsw`` file (gfortran sequential
  unformatted records, layout written by hf_read_pqbs.f90:110-121);
* the "Configuration energies" blocks of the DBSR_HF logs (the average
  energy of every jj configuration with the final orbitals) with the
  orbitals of the run, for B and the four Fe runs.

Only numbers are stored; no reference source code is copied.
"""
from __future__ import annotations

import json
import os
import re
import struct
import sys

import numpy as np

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DBSR_REFERENCE", "")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.json")


def fnum(s: str) -> float:
    return float(s.replace("D", "E").replace("d", "e"))


def parse_knot(path: str) -> dict:
    txt = open(path).read()
    out = {"file": os.path.relpath(path, REF)}
    for key in ("grid_type", "ks", "ns", "nv", "ml", "ksp", "ksq"):
        m = re.search(rf"^\s*{key}\s*=\s*(-?\d+)", txt, re.M)
        out[key] = int(m.group(1))
    for key in ("hi", "he", "hmax", "rmax", "tmax", "atomic_number", "atomic_weight", "rrms",
                "c_fermi", "a_fermi"):
        m = re.search(rf"^\s*{key}\s*=\s*([-+0-9.DdEe]+)", txt, re.M)
        if m:
            out[key] = fnum(m.group(1))
    m = re.search(r"^\s*nuclear\s*=\s*(\S+)", txt, re.M)
    out["nuclear"] = m.group(1)
    pts = txt.split("grid points:")[1].split("***")[0]
    t = []
    for line in pts.strip().splitlines():
        f = line.split()
        if len(f) == 2:
            t.append(fnum(f[1]))
    out["t"] = t
    return out


def read_records(path: str):
    """gfortran sequential unformatted: 4-byte length markers."""
    data = open(path, "rb").read()
    pos, recs = 0, []
    while pos < len(data):
        (n,) = struct.unpack_from("<i", data, pos)
        recs.append(data[pos + 4: pos + 4 + n])
        pos += 8 + n
    return recs


def parse_bsw(path: str) -> dict:
    recs = read_records(path)
    h = recs[0]
    grid_type, ns, ks = struct.unpack_from("<3i", h, 0)
    t = np.frombuffer(h, "<f8", ns + ks, 12)
    off = 12 + 8 * (ns + ks)
    ksp, ksq = struct.unpack_from("<2i", h, off)
    z = awt = None
    if len(h) >= off + 24:
        z, awt = struct.unpack_from("<2d", h, off + 8)
    orbs = []
    for i in range(1, len(recs), 3):
        r = recs[i]
        label = r[:5].decode()
        (mbs,) = struct.unpack_from("<i", r, 5)
        (e,) = struct.unpack_from("<d", r, 9)
        p = np.frombuffer(recs[i + 1], "<f8").tolist()
        q = np.frombuffer(recs[i + 2], "<f8").tolist()
        orbs.append({"label": label, "mbs": mbs, "e": e, "p": p, "q": q})
    return {"ns": ns, "ks": ks, "ksp": ksp, "ksq": ksq, "z": z, "awt": awt, "t": t.tolist(),
            "orbitals": orbs}


def config_energies(path: str) -> list:
    """[(subshell occupations {label: q}, energy in au)] of the log's
    "Configuration energies" block."""
    lines = open(path).read().split("Configuration energies:")[1].splitlines()
    out = []
    for line in lines[1:]:
        if " au " not in line:
            if out:
                break
            continue
        head, tail = line.split(" au ")[0].rsplit(None, 1)
        occ = {m.group(1).strip(): int(m.group(2))
               for m in re.finditer(r"(\d+[a-z]-?)\s*\(\s*(\d+)\)", head)}
        out.append((occ, float(tail)))
    return out


def log_value(path: str, pat: str):
    for line in open(path):
        if pat in line:
            return line
    return None


def main():
    if not REF or not os.path.isdir(REF):
        sys.exit("usage: make_golden.py <reference root> (or set DBSR_REFERENCE)")
    g = {"knots": [], "hf": [], "mat_memory": None}
    g["knots"].append(parse_knot(os.path.join(REF, "Rb_bound_example/dbsr_cc27/knot.dat")))
    ex = os.path.join(REF, "DBSR_HF/examples")
    for name in ("Li_092m1", "Rb", "B", "Be", "N"):
        g["knots"].append(parse_knot(os.path.join(ex, f"{name}.knot")))
    g["knots"].append(parse_knot(os.path.join(ex, "Fe/Fe.knot")))
    for name in ("Li_092m1", "Rb", "Be", "B"):
        logp = os.path.join(ex, f"{name}.log")
        mem = log_value(logp, "memory=")
        coul = log_value(logp, "Coulomb energy:")
        kmax = log_value(logp, "kmax =")
        rec = {
            "name": name,
            "memory_mb": float(mem.split("=")[1].split()[0]),
            "kmax": int(kmax.split("=")[1].split()[0]),
            "coulomb_energy": float(coul.split(":")[1].split()[0]),
            "conf": open(os.path.join(ex, f"{name}.conf")).read(),
            "bsw": parse_bsw(os.path.join(ex, f"{name}.bsw")),
        }
        g["hf"].append(rec)
    g["configs"] = []
    for log, bsw in (("B.log", "B.bsw"), ("Fe/Fe.log", "Fe/Fe.bsw"), ("Fe/2.log", "Fe/2.bsw"),
                     ("Fe/3.log", "Fe/3.bsw"), ("Fe/4.log", "Fe/4.bsw")):
        b = parse_bsw(os.path.join(ex, bsw))
        keep = {"2p-", "2p", "3d-", "3d"}
        b["orbitals"] = [o for o in b["orbitals"] if o["label"].strip() in keep]
        g["configs"].append({"log": log, "bsw": bsw, "energies": config_energies(
            os.path.join(ex, log)), "orbitals": b})
    mline = log_value(os.path.join(REF, "Rb_bound_example/dbsr_cc27/mat_log.005"),
                      "memory of DBS_integrals")
    g["mat_memory"] = {"line": mline.strip() if mline else None, "ns": 109, "ks": 9, "kmax": 7,
                       "ntype": 4}
    json.dump(g, open(OUT, "w"), indent=None, separators=(",", ":"))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
