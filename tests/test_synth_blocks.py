"""config3_block(i) builds block i of the batched workload alone: the same
grid, orbitals and coefficient lists as config3(...)[i]."""
import numpy as np

from dbsr_gb300 import synth


def test_config3_block_replays_the_batch_draws():
    batch = synth.config3(nblocks=4, nch_max=20, rows_entries=50)
    one = synth.config3_block(3, nch_max=20, rows_entries=50)
    ref = batch[3]
    assert (one.ns, one.nch, one.iicc) == (ref.ns, ref.nch, ref.iicc)
    assert np.array_equal(one.t, ref.t) and np.array_equal(one.pq, ref.pq)
    assert len(one.lists) == len(ref.lists)
    for a, b in zip(one.lists, ref.lists):
        assert (a.icase, a.itype, a.kpol) == (b.icase, b.itype, b.kpol)
        for x, y in zip((a.k1, a.k2, a.k3, a.k4, a.c), (b.k1, b.k2, b.k3, b.k4, b.c)):
            assert np.array_equal(x, y)
