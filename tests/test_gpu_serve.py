"""GPU tests of the serving loop: a request's result is the same alone and in
the mix (bit for bit, since its arithmetic does not depend on its batch) and
within the parity tolerance of the FP64 oracle; admission respects the HBM
budget; a request larger than the budget is refused."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

LAYERS = [(64, 96, 14, 14), (128, 128, 28, 28), (32, 48, 9, 11)]  # c, k, h, w


def _setup(wg, srv, seed):
    rng = np.random.default_rng(seed)
    keep, host = [], []
    for c, k, h, w in LAYERS:
        wt = (rng.standard_normal((k, c, 3, 3)) / np.sqrt(9 * c)).astype(np.float16)
        wtt = torch.from_numpy(wt).cuda()
        srv.add_layer(c, k, h, w, wtt.data_ptr())
        keep.append(wtt)
        host.append(wt)
    return rng, keep, host


def _requests(rng, count):
    reqs = []
    for i in range(count):
        li = int(rng.integers(0, len(LAYERS)))
        c, k, h, w = LAYERS[li]
        n = int(rng.integers(1, 6))
        x = rng.uniform(-1, 1, (n, c, h, w)).astype(np.float16)
        reqs.append((li, n, x))
    return reqs


def _run(wg, srv, reqs, together):
    outs, keep = [], []
    ids = []
    for li, n, x in reqs:
        c, k, h, w = LAYERS[li]
        xt = torch.from_numpy(x).cuda()
        y = torch.full((n, k, h, w), float("nan"), dtype=torch.float16, device="cuda")
        torch.cuda.synchronize()
        ids.append(srv.submit(li, n, xt.data_ptr(), y.data_ptr()))
        keep.append((xt, y))
        if not together:
            srv.wait_all()
    srv.wait_all()
    for rid in ids:
        assert srv.poll(rid)[0] == 1
    return [y.cpu().numpy() for _, y in keep]


def test_same_result_alone_and_in_the_mix(wg):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    alone_srv = wg.Server(slots=1, max_batch=1, hbm_budget_bytes=1 << 30)
    rng, k1, host = _setup(wg, alone_srv, 3)
    reqs = _requests(rng, 14)
    alone = _run(wg, alone_srv, reqs, together=False)
    alone_srv.destroy()
    mix_srv = wg.Server(slots=3, max_batch=5, hbm_budget_bytes=1 << 30)
    _setup(wg, mix_srv, 3)
    mixed = _run(wg, mix_srv, reqs, together=True)
    st = mix_srv.stats()
    mix_srv.destroy()
    assert st["completed"] == len(reqs)
    for (li, n, x), a, b in zip(reqs, alone, mixed):
        assert np.array_equal(a.view(np.uint16), b.view(np.uint16))
        _, r64 = O.conv2d_direct(x, host[li], nthreads=8)
        c = LAYERS[li][0]
        tol = 2e-2 if (min(LAYERS[li][0], LAYERS[li][1]) >= 128 and LAYERS[li][2] >= 14) else 1e-2
        assert O.rel_errors(b, r64)[0] <= tol


def test_admission_respects_the_budget(wg):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    # budget that fits about one request of the 128-channel layer at a time
    srv = wg.Server(slots=3, max_batch=8, hbm_budget_bytes=6 << 20)
    rng, keep, host = _setup(wg, srv, 4)
    reqs = [(1, 4, rng.uniform(-1, 1, (4, 128, 28, 28)).astype(np.float16)) for _ in range(6)]
    outs = _run(wg, srv, reqs, together=True)
    st = srv.stats()
    assert st["completed"] == 6 and st["arena_used_bytes"] == 0
    assert st["mean_batch"] <= 2.0
    for (li, n, x), y in zip(reqs, outs):
        _, r64 = O.conv2d_direct(x, host[li], nthreads=8)
        assert O.rel_errors(y, r64)[0] <= 2e-2
    srv.destroy()


def test_oversized_request_is_refused(wg):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    srv = wg.Server(slots=1, max_batch=1, hbm_budget_bytes=2 << 20)
    w = torch.zeros((128, 128, 3, 3), dtype=torch.float16, device="cuda")
    li = srv.add_layer(128, 128, 56, 56, w.data_ptr())
    x = torch.zeros((8, 128, 56, 56), dtype=torch.float16, device="cuda")
    y = torch.zeros((8, 128, 56, 56), dtype=torch.float16, device="cuda")
    with pytest.raises(wg.Conv2dError) as ei:
        srv.submit(li, 8, x.data_ptr(), y.data_ptr())
    assert ei.value.status == wg.ERR_BUSY
    srv.destroy()


def test_plain_per_request_path_gives_the_served_bits(wg):
    """The plain per-call path (each request's own kernels queued on one stream
    at submission) and the batching server compute every request the same
    way, bit for bit."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    plain = wg.Server(per_request=1, hbm_budget_bytes=1 << 30)
    rng, k1, host = _setup(wg, plain, 8)
    reqs = _requests(rng, 12)
    a = _run(wg, plain, reqs, together=True)
    st = plain.stats()
    plain.destroy()
    assert st["completed"] == len(reqs) and st["mean_batch"] == 1.0
    served = wg.Server(slots=3, max_batch=4, hbm_budget_bytes=1 << 30)
    _setup(wg, served, 8)
    b = _run(wg, served, reqs, together=True)
    served.destroy()
    for (li, n, x), ya, yb in zip(reqs, a, b):
        assert np.array_equal(ya.view(np.uint16), yb.view(np.uint16))


def test_batches_overlap_on_the_device(wg):
    """Under a burst of requests the server keeps several batches in flight
    at once, and their device intervals (start and end events on the slots'
    streams) overlap."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    srv = wg.Server(slots=3, max_batch=4, hbm_budget_bytes=4 << 30)
    rng, keep, host = _setup(wg, srv, 9)
    bufs = []
    for li, (c, k, h, w) in enumerate(LAYERS):
        x = (torch.rand((8, c, h, w), device="cuda") * 2 - 1).half()
        y = torch.empty((8, k, h, w), dtype=torch.float16, device="cuda")
        bufs.append((x, y))
    torch.cuda.synchronize()
    for i in range(200):
        li = i % len(LAYERS)
        srv.submit(li, 8, bufs[li][0].data_ptr(), bufs[li][1].data_ptr())
    srv.wait_all()
    st = srv.stats()
    srv.destroy()
    assert st["completed"] == 200
    assert st["max_inflight_batches"] > 1
    assert st["overlap_us"] > 0.0 and st["busy_us"] > 0.0
