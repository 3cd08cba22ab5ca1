"""Restatement of DBSR_MAT3's dbsr_mat.nnn write-out (test infrastructure
only: the checker of the library's dbsrg_record_* entry points).

* header(): SUB1's records after Diag_channels (sub1.f90:164-168);
* record_matrix(): Record_matrix (record_matrix.f90:2-60) from host arrays,
  the block transformation by the oracle's loops (orc_record_block);
* acf(): the closing records (sub1.f90:286-287).

Records are Fortran sequential unformatted records as gfortran writes
them: a 4-byte length, the bytes, the same length (machine byte order).
read_records() splits a file into its record payloads.  Parity unpinned:
the reference ships no dbsr_mat.nnn.
"""
from __future__ import annotations

import struct

import numpy as np

from . import oracle as O


def _rec(payload: bytes) -> bytes:
    n = struct.pack("=i", len(payload))
    return n + payload + n


def _ints(*v) -> bytes:
    return _rec(np.asarray(v, dtype=np.int32).tobytes())


def _dbl(a) -> bytes:
    return _rec(np.asarray(a, dtype=np.float64).ravel(order="F").tobytes())


def header(ns, nch, npert, nsp, nsq, sol, ev, nsol) -> bytes:
    """(ns,nch,npert,nsp,nsq), (nsol), (jpsol(0:nch)), (eval), (diag
    solutions), as SUB1 writes them after rewind(nui)."""
    nsol = np.asarray(nsol, dtype=np.int64)
    jpsol = np.concatenate([[0], np.cumsum(nsol)]).astype(np.int32)
    evals = [ev[js, ich] for ich in range(nch) for js in range(nsol[ich])]
    cols = [sol[:, js, ich] for ich in range(nch) for js in range(nsol[ich])]
    out = _ints(ns, nch, npert, nsp, nsq) + _ints(int(jpsol[-1]))
    out += _rec(jpsol.tobytes()) + _dbl(evals)
    out += _rec(np.concatenate(cols).tobytes() if cols else b"")
    return out


def record_matrix(hch, icc, sol, nsol, icase=2, npert=0, icb=None, hcp=None, ibb=None,
                  hp=None):
    """Record_matrix's records (bytes) and, for icase 0, the overlaps array
    ((nch+npert)^2) it fills."""
    nch = icc.shape[0]
    out = b""
    ov = np.zeros((nch + npert, nch + npert), order="F")
    for ich in range(2, nch + 1):  # non-diagonal channel blocks
        ni = int(nsol[ich - 1])
        for jch in range(1, ich):
            nj = int(nsol[jch - 1])
            k = int(icc[ich - 1, jch - 1])
            if k == 0:
                continue
            if np.abs(hch[:, :, k - 1]).max() < 1e-20:
                continue
            c = O.record_block(hch[:, :, k - 1], sol[:, :ni, ich - 1], sol[:, :nj, jch - 1])
            out += _ints(ich, jch) + _dbl(c)
            if icase == 0:
                ov[ich - 1, jch - 1] = np.abs(c).max() if c.size else 0.0
    if npert > 0:
        for ich in range(1, nch + 1):  # channel-perturber rows
            ni = int(nsol[ich - 1])
            for ip in range(1, npert + 1):
                k = int(icb[ich - 1, ip - 1])
                if k == 0:
                    continue
                if np.abs(hcp[:, k - 1]).max() < 1e-20:
                    continue
                w = np.zeros(ni)
                for i in range(ni):  # SUM(diag(:,i,ich)*hcp(:,k)), in order
                    s = 0.0
                    for m in range(hcp.shape[0]):
                        s = s + sol[m, i, ich - 1] * hcp[m, k - 1]
                    w[i] = s
                if icase == 0:
                    ov[nch + ip - 1, ich - 1] = np.abs(w).max() if ni else 0.0
                out += _ints(nch + ip, ich) + _dbl(w)
        for ip in range(1, npert + 1):  # perturber-perturber elements
            for jp in range(1, ip + 1):
                k = int(ibb[ip - 1, jp - 1])
                if k == 0 or hp[k - 1] == 0.0:
                    continue
                out += _ints(ip + nch, jp + nch) + _dbl([hp[k - 1]])
                if icase == 0:
                    ov[nch + ip - 1, nch + jp - 1] = abs(hp[k - 1])
    out += _ints(0, 0)
    return out, ov


def acf(mk, bcf) -> bytes:
    return _ints(mk) + _dbl(bcf)


def read_records(data: bytes) -> list:
    """Payloads of the sequential unformatted records of `data`."""
    recs, p = [], 0
    while p < len(data):
        (n,) = struct.unpack_from("=i", data, p)
        payload = data[p + 4:p + 4 + n]
        (m,) = struct.unpack_from("=i", data, p + 4 + n)
        if m != n:
            raise ValueError(f"record markers disagree at byte {p}: {n} != {m}")
        recs.append(payload)
        p += 8 + n
    return recs
