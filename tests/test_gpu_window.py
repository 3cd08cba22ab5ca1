"""Streamed output: a matrix held as a window of consecutive blocks
(dbsrg_alloc_matrix_window / dbsrg_set_window) and assembled window by
window must equal, bit for bit, the matrix assembled whole (every block sums
the same terms in the same order whatever the window), for every precision
form, with the overlaps, UPDATE_HX and acf.  At the full size of the largest
symmetry block of the batched workload (ns=368, 262 channels: 34 453 blocks,
149 GB in the reference layout) the property is checked through per-block
checksums taken on the device for two window sizes."""
import numpy as np
import pytest

from dbsr_gb300 import FACTOR_FP64, PLAIN_FP64, SPLIT_BF16, Assembler, synth
from dbsr_gb300.api import gen_batch_streamed
from dbsr_gb300._lib import DbsrgError

pytestmark = pytest.mark.gpu


def items(w):
    return [(L.icase, L.itype, L.kpol, L.k1, L.k2, L.k3, L.k4, L.c) for L in w.lists]


def make(w, precision, window=None):
    a = Assembler(w.t, w.ks, w.ksp, w.ksq)
    a.set_orbitals(w.pq, w.ipbs)
    a.alloc_matrix(w.nch, w.icc, w.iicc, w.mk, window=window)
    a.set_precision(precision)
    return a


def full(w, precision):
    a = make(w, precision)
    for it in items(w):
        a.gen_matrix(*it)
    h, acf = a.get_matrix(), a.get_acf()
    a.close()
    return h, acf


@pytest.mark.parametrize("precision", [PLAIN_FP64, FACTOR_FP64, SPLIT_BF16])
@pytest.mark.parametrize("window", [1, 4, 7])
def test_windows_equal_whole_matrix(precision, window):
    w = synth.small(ns=60, nch=5, mk=3, n_entries=2000, seed=51)
    h0, acf0 = full(w, precision)
    a = make(w, precision, window)
    parts = []
    for blo, nb in a.stream(items(w)):
        assert nb == min(window, w.iicc - blo + 1)
        parts.append(a.get_matrix())
    acf = a.get_acf()
    a.close()
    assert np.array_equal(np.concatenate(parts, axis=2), h0)
    assert np.array_equal(acf, acf0)


def test_window_block_access_and_update_hx():
    w = synth.small(ns=50, nch=4, mk=2, n_entries=500, seed=52)
    a = make(w, SPLIT_BF16, 3)
    a.set_window(4)  # blocks 4..6
    ich, jch = np.argwhere(w.icc == 1)[0] + 1  # block 1: outside the window
    with pytest.raises(DbsrgError, match="ESTATE"):
        a.get_block(ich, jch)
    d = np.ones((a.ms, a.ms), order="F")
    a.update_hx(int(ich), int(jch), d, 2.0)  # another window's block: no-op
    assert not a.get_matrix().any()
    ich, jch = np.argwhere(w.icc == 5)[0] + 1
    a.update_hx(int(ich), int(jch), d, 2.0)
    blk = a.get_block(int(ich), int(jch))
    assert np.array_equal(blk, 2.0 * (d if ich >= jch else d.T))
    a.close()


def test_streamed_batch_equals_blocks_one_by_one():
    ws = [synth.small(ns=50 + 10 * i, nch=3 + i, mk=3, n_entries=800, seed=60 + i)
          for i in range(3)]
    ref = [full(w, SPLIT_BF16) for w in ws]
    asm = [make(w, SPLIT_BF16, window=2 + i) for i, w in enumerate(ws)]
    got = [[] for _ in ws]

    def consume(i, blo, nb, ptr):
        got[i].append((blo, asm[i].get_matrix()))

    gen_batch_streamed(asm, [items(w) for w in ws], consume)
    for i, w in enumerate(ws):
        blos = [b for b, _ in got[i]]
        assert blos == list(range(1, w.iicc + 1, 2 + i))
        assert np.array_equal(np.concatenate([m for _, m in got[i]], axis=2), ref[i][0])
        assert np.array_equal(asm[i].get_acf(), ref[i][1])
        asm[i].close()


def test_largest_batch_block_full_size_window_independent():
    torch = pytest.importorskip("torch")
    w = synth.config3_block(44)
    assert (w.ns, w.nch) == (368, 262)
    ms = 2 * w.ns

    def checksums(window):
        a = make(w, SPLIT_BF16, window)
        a.set_async(True)
        buf = torch.empty((window, ms, ms), dtype=torch.float64, device="cuda")
        sums, asums = [], []
        for blo, nb in a.stream(items(w)):
            a.get_matrix(out=buf[:nb])
            sums.append(buf[:nb].sum(dim=(1, 2)).cpu())
            asums.append(buf[:nb].abs().sum(dim=(1, 2)).cpu())
        acf = a.get_acf()
        a.close()
        del buf
        torch.cuda.empty_cache()
        return torch.cat(sums).numpy(), torch.cat(asums).numpy(), acf

    s1, t1, acf1 = checksums(1500)
    s2, t2, acf2 = checksums(2311)
    assert s1.shape == (w.iicc,)
    assert np.isfinite(t1).all() and (t1 > 0).sum() > 0.04 * w.iicc
    assert np.array_equal(s1, s2) and np.array_equal(t1, t2)
    assert np.array_equal(acf1, acf2)


@pytest.mark.parametrize("nwin", [1, 2, 5, 0, 10 ** 6])
def test_assemble_to_host_equals_whole_assembly(nwin):
    torch = pytest.importorskip("torch")
    w = synth.small(ns=60, nch=5, mk=3, n_entries=2000, seed=53)
    h0, acf0 = full(w, SPLIT_BF16)
    a = make(w, SPLIT_BF16)
    a.gen_matrix(*items(w)[0])  # leftovers in the device matrix must not matter
    out, acf = a.assemble_to_host(items(w), nwin=nwin)
    assert np.array_equal(out, h0) and np.array_equal(acf, acf0)
    # pinned host and device destinations
    hp = torch.zeros(h0.size, dtype=torch.float64).pin_memory()
    a.assemble_to_host(items(w), out=hp, nwin=nwin)
    assert np.array_equal(hp.numpy().reshape(h0.shape, order="F"), h0)
    hd = torch.zeros(h0.size, dtype=torch.float64, device="cuda")
    a.assemble_to_host(items(w), out=hd, nwin=nwin)
    assert np.array_equal(hd.cpu().numpy().reshape(h0.shape, order="F"), h0)
    a.close()


def test_assemble_to_host_needs_two_windows():
    w = synth.small(ns=50, nch=4, mk=2, n_entries=300, seed=54)
    a = make(w, SPLIT_BF16, window=4)  # 4 of 10 blocks allocated
    with pytest.raises(DbsrgError, match="EINVAL"):
        a.assemble_to_host(items(w), nwin=3)
    out, _ = a.assemble_to_host(items(w), nwin=2)
    a.close()
    assert np.array_equal(out, full(w, SPLIT_BF16)[0])


@pytest.mark.parametrize("nwin", [1, 3, 6, 0, 10 ** 6])
@pytest.mark.parametrize("where", ["pinned", "pageable", "device"])
def test_assemble_streamed_equals_whole_assembly(nwin, where):
    """dbsrg_assemble_streamed_host: the windows handed to the consumer, in
    block order and each at most nwin blocks, put together equal the whole
    assembly bit for bit (acf too), from a staging area of two windows."""
    torch = pytest.importorskip("torch")
    w = synth.small(ns=60, nch=5, mk=3, n_entries=2000, seed=55)
    h0, acf0 = full(w, SPLIT_BF16)
    a = make(w, SPLIT_BF16)
    ms = a.ms
    eff = nwin if nwin > 0 else -(-w.iicc // a.get_tuning("windows"))
    eff = min(eff, w.iicc)
    nstage = (2 if eff < w.iicc else 1) * eff * ms * ms
    if where == "device":
        stage = torch.zeros(nstage, dtype=torch.float64, device="cuda")
    elif where == "pinned":
        stage = torch.zeros(nstage, dtype=torch.float64).pin_memory()
    else:
        stage = np.zeros(nstage)
    a.gen_matrix(*items(w)[0])  # leftovers in the device matrix must not matter
    got, nxt = [], [1]

    def consume(blo, nb, view):
        assert blo == nxt[0] and 1 <= nb <= eff
        nxt[0] = blo + nb
        v = view.cpu().numpy() if hasattr(view, "cpu") else view
        assert v.shape == (ms, ms, nb)
        got.append(np.array(v))

    acf = a.assemble_streamed(items(w), stage, consume, nwin=nwin)
    assert nxt[0] == w.iicc + 1
    assert np.array_equal(np.concatenate(got, axis=2), h0)
    assert np.array_equal(acf, acf0)
    a.close()


def test_assemble_streamed_consumer_error_and_reuse():
    """An exception in the consumer is raised when the call returns; the
    context stays usable and a second call delivers the matrix again."""
    w = synth.small(ns=50, nch=4, mk=2, n_entries=600, seed=56)
    h0, _ = full(w, SPLIT_BF16)
    a = make(w, SPLIT_BF16)
    stage = np.zeros(2 * 3 * a.ms * a.ms)

    def bad(blo, nb, view):
        raise RuntimeError("consumer failed")

    with pytest.raises(RuntimeError, match="consumer failed"):
        a.assemble_streamed(items(w), stage, bad, nwin=3)
    parts = []
    a.assemble_streamed(items(w), stage, lambda blo, nb, v: parts.append(np.array(v)), nwin=3)
    assert np.array_equal(np.concatenate(parts, axis=2), h0)
    a.close()


def test_assemble_streamed_needs_two_windows():
    w = synth.small(ns=50, nch=4, mk=2, n_entries=300, seed=57)
    a = make(w, SPLIT_BF16, window=4)  # 4 of 10 blocks allocated
    stage = np.zeros(2 * 3 * a.ms * a.ms)
    with pytest.raises(DbsrgError, match="EINVAL"):
        a.assemble_streamed(items(w), stage, lambda *x: None, nwin=3)
    parts = []
    a.assemble_streamed(items(w), stage, lambda blo, nb, v: parts.append(np.array(v)), nwin=2)
    a.close()
    assert np.array_equal(np.concatenate(parts, axis=2), full(w, SPLIT_BF16)[0])


def test_host_matrix_destination():
    """dbsrg_host_alloc memory (page-locked, huge pages, zeroed) as the
    destination of dbsrg_assemble_to_host; dbsrg_host_free of an address it
    did not allocate is refused."""
    import ctypes as C

    from dbsr_gb300._lib import load
    from dbsr_gb300.api import HostMatrix

    w = synth.small(ns=60, nch=5, mk=3, n_entries=2000, seed=58)
    h0, acf0 = full(w, SPLIT_BF16)
    a = make(w, SPLIT_BF16)
    hm = HostMatrix(h0.size)
    assert hm.array.shape == (h0.size,) and not hm.array.any()
    out, acf = a.assemble_to_host(items(w), out=hm.array, nwin=3)
    assert np.array_equal(hm.array.reshape(h0.shape, order="F"), h0)
    assert np.array_equal(acf, acf0)
    a.close()
    hm.close()
    hm.close()
    x = np.zeros(16)
    assert load().dbsrg_host_free(C.c_void_p(x.ctypes.data)) == -1
