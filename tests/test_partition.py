"""Multi-rank partition of the assembly (CPU, gloo, two ranks): every rank
assembles only its own blocks (the oracle stands in for the GPU library, the
partition logic is what is under test), the writer gathers the blocks from
their owners, and the result equals the single-process assembly bit for bit."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _assemble(w, lists):
    from oracle import oracle as O

    g = O.Grid(w.t, w.ks, w.ksp, w.ksq)
    m = O.Matrix(g, w.pq, w.ipbs, w.nch, w.icc, w.mk)
    for L in lists:
        m.gen_matrix(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c)
    return m.hch.copy(), m.acf.copy()


def _rank_main(rank, world, port, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from dbsr_gb300 import partition, synth

    w = synth.small(ns=40, nch=4, mk=2, n_entries=200, breit=True, seed=17)
    owner = partition.assign_blocks(w.lists, w.icc, w.ipbs, world)
    mine = partition.rank_lists(w.lists, owner, w.icc, w.ipbs, rank)
    hch, acf = _assemble(w, mine)
    # writer gathers every rank's blocks and keeps each block from its owner
    hs = [torch.zeros_like(torch.from_numpy(np.ascontiguousarray(hch))) for _ in range(world)]
    ac = [torch.zeros_like(torch.from_numpy(np.ascontiguousarray(acf))) for _ in range(world)]
    dist.all_gather(hs, torch.from_numpy(np.ascontiguousarray(hch)))
    dist.all_gather(ac, torch.from_numpy(np.ascontiguousarray(acf)))
    if rank == 0:
        H = np.zeros_like(np.ascontiguousarray(hch))
        A = np.zeros_like(np.ascontiguousarray(acf))
        for b in range(w.iicc):
            H[:, :, b] = hs[owner[b]].numpy()[:, :, b]
            A[b, :] = ac[owner[b]].numpy()[b, :]
        np.savez(out_path, H=H, A=A, owner=owner)
    dist.barrier()
    dist.destroy_process_group()


def test_partitioned_assembly_equals_single_process(tmp_path):
    from dbsr_gb300 import partition, synth

    w = synth.small(ns=40, nch=4, mk=2, n_entries=200, breit=True, seed=17)
    owner = partition.assign_blocks(w.lists, w.icc, w.ipbs, 2)
    # every list entry lands on exactly one rank; both ranks get work
    for L in w.lists:
        parts = [partition.rank_lists([L], owner, w.icc, w.ipbs, r) for r in range(2)]
        assert sum(p[0].n for p in parts if p) == L.n
    assert set(owner.tolist()) == {0, 1}
    out = str(tmp_path / "gathered.npz")
    mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, start_method="spawn")
    got = np.load(out)
    H, A = _assemble(w, w.lists)
    assert np.array_equal(got["H"], np.ascontiguousarray(H))
    assert np.array_equal(got["A"], np.ascontiguousarray(A))
