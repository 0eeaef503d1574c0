"""fa2cu_morton_order_noalloc, the entry point that allocates nothing.

Some callers cannot call cudaMalloc: their GPU memory belongs to another
allocator (a framework's pool that accounts for every byte), or they cannot
afford an allocation's device synchronisation or its failure once started.
For them, the Morton codes and the Morton order of positions already on the
device (the first steps of the tree build) come with all scratch memory in a
static device array of the library. This test calls it through the C
interface on caller-owned device buffers and checks it against the same
step of a resident layout (fa2cu_layout_tree): keys and order bit-exact, on
calls in a row that reuse the shared scratch, each followed by a clean
fa2cu_noalloc_status (no bounded wait of the sort gave up). It sits in a
file of its own, collected last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(n, seed):
    from forceatlas2_rc_gb300 import graphs as G
    pos = G.uniform_positions(n, -1e3, 1e3, seed=seed).astype(np.float32)
    pos[: n // 50] = pos[0]  # coincident nodes: equal codes, ties by index
    return pos


def _expected(pos):
    from forceatlas2_rc_gb300.layout import Graph, Layout
    n = len(pos)
    e = np.zeros(0, np.int32)
    g = Graph(n, e, e, np.zeros(0))
    with Layout(g, pos.astype(np.float64), precision="single") as L:
        t = L.tree(pos.astype(np.float64))
    return t["key"], t["order"]


def test_noalloc_matches_layout_tree(cuda_lib, gpu):
    import torch
    lib = cuda_lib
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    cases = [_case(50_000, 1), _case(70_001, 2), _case(50_000, 1)]
    for pos in cases:  # three calls in a row, the last repeating the first
        n = len(pos)
        dpos = torch.from_numpy(pos.reshape(-1).copy()).to(dev)  # x, y interleaved
        key = torch.empty(n, dtype=torch.int32, device=dev)
        order = torch.empty(n, dtype=torch.int32, device=dev)
        rc = lib.fa2cu_morton_order_noalloc(n, dpos.data_ptr(), key.data_ptr(),
                                            order.data_ptr(), stream)
        assert rc == 0, lib.fa2_gpu_error()
        assert lib.fa2cu_noalloc_status(stream) == 0, lib.fa2_gpu_error()
        torch.cuda.synchronize(dev)
        want_key, want_order = _expected(pos)
        np.testing.assert_array_equal(key.cpu().numpy().view(np.uint32), want_key)
        np.testing.assert_array_equal(order.cpu().numpy().view(np.uint32), want_order)


def test_noalloc_rejects_oversized(cuda_lib, gpu):
    lib = cuda_lib
    rc = lib.fa2cu_morton_order_noalloc((1 << 20) + 1, 16, 16, 16, None)
    assert rc != 0
    assert b"1048576" in lib.fa2_gpu_error()


def test_noalloc_rejects_misaligned(cuda_lib, gpu):
    """Buffers the kernels could not address (pos not 8-byte aligned, key
    or order not 4-byte aligned) are refused on the host; nothing runs."""
    lib = cuda_lib
    for pos, key, order in ((20, 16, 16), (16, 18, 16), (16, 16, 17)):
        assert lib.fa2cu_morton_order_noalloc(100, pos, key, order, None) != 0
        assert b"aligned" in lib.fa2_gpu_error()
