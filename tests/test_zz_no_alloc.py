"""GPU test of conv2d_fp16_noalloc, the entry point for callers that must not
allocate device memory while they run (a host that gives all device memory
to its own pool at start-up, or a latency-bound loop that cannot afford the
device synchronisation of cudaMalloc/cudaFree).  Its workspace is a fixed
array inside the library, shared by every call on a device; two calls in a
row must each give the same result as the regular entry point, which
allocates its workspace in getkernelInfo.  This file is collected last so
that a failure here stops a run only after every other test has run."""
import ctypes

import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(1, 64, 56, 56, 64), (2, 20, 13, 11, 36)])
def test_noalloc_matches_regular_entry_point_twice(wg, shape):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    n, c, h, w, k = shape
    x, wt = O.uniform_inputs(77, n, c, h, w, k)
    xt, wtt = torch.from_numpy(x).cuda(), torch.from_numpy(wt).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    # regular entry point, same algorithm (F(2x3) non-fused)
    ref, op = wg.conv2d_torch(xt, wtt, 1, 1, wg.default_options(algo=wg.ALGO_2X3), stream=stream)
    torch.cuda.synchronize()
    _, r64 = O.conv2d_direct(x, wt, nthreads=8)
    for _ in range(2):
        y = torch.full((n, k, h, w), float("nan"), dtype=torch.float16, device="cuda")
        prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, w, k)
        wg.conv2d_noalloc(prob, stream)
        torch.cuda.synchronize()
        yh = y.cpu().numpy()
        # same tolerance as the parity tests for F(2x3), against the regular
        # entry point's output and against the FP64 oracle
        assert O.rel_errors(yh, ref.cpu().numpy())[0] <= 1e-2
        assert O.rel_errors(yh, r64)[0] <= 1e-2


@pytest.mark.gpu
def test_noalloc_rejects_problems_beyond_its_scratch(wg):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    # 64 x 256 x 56 x 56 -> 256 needs ~0.8 GB of Winograd-domain workspace
    prob = wg.make_problem(256, 256, 256, 64, 256, 56, 56, 256)
    st = wg.lib().conv2d_fp16_noalloc(ctypes.byref(prob), None)
    assert st == wg.ERR_UNSUPPORTED
    assert b"32 MiB" in wg.lib().conv2d_last_error_message()
