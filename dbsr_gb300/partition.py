"""Partition of the assembly over ranks (one process per GPU).

Channel-pair blocks are independent given the replicated grid, tables and
orbitals: the reference's MPI build hands blocks to ranks round robin
(``icc``, DBSR_MAT3/updates.f90:20-37) and each rank keeps only its own
entries (state_res.f90:135-147).  Here a rank owns a set of whole blocks --
both channel orders of a pair, so UPDATE_HS sees the owner and the partner
segment of a block on the same rank -- chosen greedily by entry count so
the ranks get equal work.  Every rank filters the coefficient lists to its
blocks and assembles them; the blocks are gathered to the writer afterwards
(the reference's Send/Recv, record_matrix_mpi.f90:22-26).  No reduction is
needed: each block is summed on exactly one rank.
"""
from __future__ import annotations

import numpy as np

IBO = 2 ** 15  # K1 = ich*IBO + jch (mod_dbsr_mat.f90:61)


def block_of_list(icase: int, k1: np.ndarray, k2: np.ndarray, icc: np.ndarray,
                  ipbs: np.ndarray) -> np.ndarray:
    """0-based block of every entry of a list: K1 packs the channel pair for
    the R/S lists; for O lists (icase 0) the channels come from the orbitals
    packed in K1 and K2 (O_data.f90:50-61)."""
    if icase == 0:
        ich = ipbs[k1 // IBO - 1]
        jch = ipbs[k2 // IBO - 1]
    else:
        ich, jch = k1 // IBO, k1 % IBO
    return icc[ich - 1, jch - 1] - 1


def assign_blocks(lists, icc: np.ndarray, ipbs: np.ndarray, world: int) -> np.ndarray:
    """Rank of every block: longest-processing-time greedy over the entry
    count of each block (all lists together), ties broken by block index, so
    the assignment is the same on every rank."""
    nblk = int(icc.max())
    work = np.zeros(nblk, dtype=np.int64)
    for L in lists:
        if L.n:
            np.add.at(work, block_of_list(L.icase, L.k1, L.k2, icc, ipbs), 1)
    order = np.lexsort((np.arange(nblk), -work))
    load = np.zeros(world, dtype=np.int64)
    owner = np.zeros(nblk, dtype=np.int32)
    for b in order:
        r = int(np.argmin(load))
        owner[b] = r
        load[r] += work[b]
    return owner


def rank_lists(lists, owner: np.ndarray, icc: np.ndarray, ipbs: np.ndarray, rank: int):
    """The coefficient lists restricted to the blocks of one rank, in the
    original (sorted) order."""
    out = []
    for L in lists:
        if not L.n:
            continue
        keep = owner[block_of_list(L.icase, L.k1, L.k2, icc, ipbs)] == rank
        if keep.any():
            out.append(type(L)(L.icase, L.itype, L.kpol, L.k1[keep], L.k2[keep], L.k3[keep],
                               L.k4[keep], L.c[keep]))
    return out
