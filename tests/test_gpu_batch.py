"""GPU tests of batches of uneven problems: the grouped run (grouped launches
replayed from a CUDA graph) must give exactly the per-call results, and each
problem must be within the parity tolerance of the FP64 oracle."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = {0: 2e-2, 1: 1e-2, 2: 1e-2, 4: 2e-2}

SHAPES = [  # n, c, h, w, k, pad
    (2, 64, 14, 14, 64, 1), (1, 128, 28, 28, 256, 1), (3, 32, 7, 7, 48, 1), (2, 256, 12, 12, 128, 1),
    (1, 16, 56, 56, 32, 1), (4, 48, 9, 13, 40, 0), (1, 80, 20, 20, 300, 2),
]


def _make(wg, shapes, seed):
    rng = np.random.default_rng(seed)
    probs, keep, host = [], [], []
    for n, c, h, w, k, p in shapes:
        x = rng.uniform(-1, 1, (n, c, h, w)).astype(np.float16)
        wt = (rng.standard_normal((k, c, 3, 3)) / np.sqrt(9 * c)).astype(np.float16)
        oh, ow = h + 2 * p - 2, w + 2 * p - 2
        xt, wtt = torch.from_numpy(x).cuda(), torch.from_numpy(wt).cuda()
        y = torch.zeros((n, k, oh, ow), dtype=torch.float16, device="cuda")
        probs.append(wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, w, k, p, p))
        keep.append((xt, wtt, y))
        host.append((x, wt, p))
    return probs, keep, host


@pytest.mark.parametrize("algo", [-1, 3, 0, 1, 4])
def test_batch_grouped_equals_percall_and_oracle(wg, algo):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    probs, keep, host = _make(wg, SHAPES, 5 + algo)
    b = wg.Batch(probs, wg.default_options(algo=algo))
    s = torch.cuda.current_stream().cuda_stream
    b.run_percall(s)
    torch.cuda.synchronize()
    percall = [y.clone() for _, _, y in keep]
    for _, _, y in keep:
        y.zero_()
    b.run(s)          # first run: direct launches, then the graph is recorded
    torch.cuda.synchronize()
    first = [y.clone() for _, _, y in keep]
    for _, _, y in keep:
        y.zero_()
    b.run(s)          # graph replay
    torch.cuda.synchronize()
    st, site = b.check_device()
    assert st == wg.OK, site
    assert b.launches(True) <= b.launches(False)
    for i, ((x, wt, p), (_, _, y)) in enumerate(zip(host, keep)):
        assert torch.equal(y, percall[i]), i
        assert torch.equal(first[i], percall[i]), i
        a, _ = b.info(i)
        _, r64 = O.conv2d_direct(x, wt, p=p, q=p, nthreads=8)
        tol = 3e-2 if (a == 0 and x.shape[1] < 16) else TOL[a]
        assert O.rel_errors(y.cpu().numpy(), r64)[0] <= tol, (i, a)
    b.destroy()


@pytest.mark.parametrize("split", ["0", "1"])
def test_batch_stream_orders_give_the_same_bits(wg, monkeypatch, split):
    """The batch graph's units run as parallel branches on forked streams by
    default; one chain after another on one stream (WG_CONV2D_BATCH_BRANCH=0)
    and one chain per (transform, GEMM tile) (WG_CONV2D_BATCH_SPLIT_BN=1) are
    the same kernels on the same data: every order gives the same bits."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    probs, keep, _ = _make(wg, SHAPES, 23)
    s = torch.cuda.current_stream().cuda_stream
    outs = []
    for branch in ("1", "0"):
        monkeypatch.setenv("WG_CONV2D_BATCH_BRANCH", branch)
        monkeypatch.setenv("WG_CONV2D_BATCH_SPLIT_BN", split)
        for _, _, y in keep:
            y.zero_()
        b = wg.Batch(probs, wg.default_options(algo=3))
        b.run(s)
        b.run(s)
        torch.cuda.synchronize()
        assert b.check_device()[0] == wg.OK
        outs.append([y.clone() for _, _, y in keep])
        b.destroy()
    for i, (a, c) in enumerate(zip(*outs)):
        assert torch.equal(a, c), i
