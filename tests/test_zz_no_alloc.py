"""The allocation-free NMS entry point (geye_nms_noalloc).

It exists for callers that cannot call cudaMalloc: their device memory is owned
by another allocator (a framework pool or a fixed budget) or they run a
real-time loop that cannot take cudaMalloc's latency and synchronisation.  It
keeps its working memory in a fixed __device__ array shared by every call.

This test calls it through the C ABI on caller-owned device buffers and checks,
on calls in a row (each later call runs over the earlier calls' leftover
scratch), its kept records against the allocating entry point geye_nms and
against the CPU oracle's kept set (the reference's nms.cpp:94-217), bit for
bit, the tolerance every NMS test here uses; the device kept count it writes
on success; an empty input; and the capacity limit.  The file sorts last so a
run that stops at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _boxes(seed: int, n: int, GL: int = 39) -> np.ndarray:
    rng = np.random.default_rng(seed)
    b = np.zeros((n, GL), np.float32)
    xy = rng.uniform(0, 600, size=(n, 2))
    wh = rng.uniform(10, 150, size=(n, 2))
    b[:, 0], b[:, 1] = xy[:, 1], xy[:, 0]
    b[:, 2], b[:, 3] = xy[:, 1] + wh[:, 1], xy[:, 0] + wh[:, 0]
    b[:, GL - 2] = np.round(rng.normal(size=n) * 3) / 4      # many tied scores
    b[:, GL - 1] = np.arange(n)
    return b


def test_nms_noalloc_matches_geye_nms_on_two_calls():
    torch = pytest.importorskip("torch")
    import geye_gb300 as g
    from oracle import oracle as O

    L = g.lib()
    ctx = g.Context(0)
    stream = torch.cuda.current_stream().cuda_stream
    for seed, n in ((11, 4000), (12, 900), (13, 0), (14, 1), (15, 2500)):
        boxes = _boxes(seed, n)
        ref = ctx.nms(boxes, 0.5, 8)
        keep, _, k = O.nms_keep(boxes, 0.5)
        assert k == ref.shape[0] and np.array_equal(boxes[keep].view(np.int32), ref.view(np.int32))
        d_boxes = torch.from_numpy(boxes).cuda() if n else torch.zeros((1, 39), device="cuda")
        d_out = torch.full_like(d_boxes, float("nan"))
        d_kept = torch.full((1,), -7, dtype=torch.int32, device="cuda")
        st = L.geye_nms_noalloc(C.c_void_p(d_boxes.data_ptr()), n, 8, 0.5, C.c_void_p(d_out.data_ptr()),
                                C.c_void_p(d_kept.data_ptr()), C.c_void_p(stream))
        assert st == 0, L.geye_last_error()
        torch.cuda.synchronize()
        K = int(d_kept.item())
        assert K == k, (seed, n, K, k)   # the count, not the -1 of an internal error
        if n > 2:
            assert K > 0
        got = d_out[:K].cpu().numpy()
        assert np.array_equal(got.view(np.int32), ref.view(np.int32))
    # beyond the fixed capacity: rejected before anything is launched
    too_many = 65536 + 1
    st = L.geye_nms_noalloc(C.c_void_p(d_boxes.data_ptr()), too_many, 8, 0.5, C.c_void_p(d_out.data_ptr()),
                            C.c_void_p(d_kept.data_ptr()), C.c_void_p(stream))
    assert st == 1 and b"capacity" in L.geye_last_error()
    ctx.close()
