"""GPU tests of conv2d_fp16_noalloc, the entry point for callers that must not
allocate device memory while they run (a host that gives all device memory
to its own pool at start-up, or a latency-bound loop that cannot afford the
device synchronisation of cudaMalloc/cudaFree).  Its workspace is a fixed
array inside the library, shared by every call on a device.  It runs the same
F(2x3) kernels as the regular entry point (which allocates its workspace in
getkernelInfo), so two calls in a row must each give the regular entry
point's output bit for bit, and so within the F(2x3) parity tolerance of the
FP64 oracle.  Its kernels report bounded-wait timeouts through an error word
in the same array, read by conv2d_noalloc_check_device.  This file is
collected last so that a failure here stops a run only after every other
test has run."""
import ctypes

import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")

F2X3_TOL = 1e-2   # max |y - ref| / max(|ref|, rms(ref)) for F(2x3) against FP64


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(1, 64, 56, 56, 64), (2, 20, 13, 11, 36)])
def test_noalloc_matches_regular_entry_point_twice(wg, shape):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    n, c, h, w, k = shape
    x, wt = O.uniform_inputs(77, n, c, h, w, k)
    xt, wtt = torch.from_numpy(x).cuda(), torch.from_numpy(wt).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    # regular entry point, same algorithm (F(2x3) non-fused, default GEMM tile)
    ref, op = wg.conv2d_torch(xt, wtt, 1, 1, wg.default_options(algo=wg.ALGO_2X3), stream=stream)
    torch.cuda.synchronize()
    assert op.check_device()[0] == wg.OK
    ref_h = ref.cpu().numpy()
    _, r64 = O.conv2d_direct(x, wt, nthreads=8)
    for _ in range(2):
        y = torch.full((n, k, h, w), float("nan"), dtype=torch.float16, device="cuda")
        prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, w, k)
        wg.conv2d_noalloc(prob, stream)
        st, site = wg.noalloc_check_device()
        assert st == wg.OK, f"no-allocation kernel gave up a wait at site {site}"
        yh = y.cpu().numpy()
        # the same kernels on the same operands: the regular output bit for bit
        assert np.array_equal(yh.view(np.uint16), ref_h.view(np.uint16))
        assert O.rel_errors(yh, r64)[0] <= F2X3_TOL
    op.destroy()


@pytest.mark.gpu
def test_noalloc_reports_a_wait_that_ran_out(wg):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    stream = torch.cuda.current_stream().cuda_stream
    assert wg.lib().conv2d_noalloc_selftest_expire(ctypes.c_void_p(stream)) == wg.OK
    st, site = wg.noalloc_check_device()
    assert st == wg.ERR_TIMEOUT and site != 0
    # reading the word clears it, and the device is still usable
    assert wg.noalloc_check_device() == (wg.OK, 0)
    n, c, h, w, k = 1, 16, 10, 10, 24
    x, wt = O.uniform_inputs(5, n, c, h, w, k)
    xt, wtt = torch.from_numpy(x).cuda(), torch.from_numpy(wt).cuda()
    y = torch.empty((n, k, h, w), dtype=torch.float16, device="cuda")
    wg.conv2d_noalloc(wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, w, k), stream)
    assert wg.noalloc_check_device()[0] == wg.OK
    _, r64 = O.conv2d_direct(x, wt)
    assert O.rel_errors(y.cpu().numpy(), r64)[0] <= F2X3_TOL


@pytest.mark.gpu
def test_noalloc_rejects_problems_beyond_its_scratch(wg):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    # 64 x 256 x 56 x 56 -> 256 needs ~0.8 GB of Winograd-domain workspace
    prob = wg.make_problem(256, 256, 256, 64, 256, 56, 56, 256)
    st = wg.lib().conv2d_fp16_noalloc(ctypes.byref(prob), None)
    assert st == wg.ERR_UNSUPPORTED
    assert b"32 MiB" in wg.lib().conv2d_last_error_message()


@pytest.mark.gpu
def test_noalloc_rejects_rows_too_wide_before_queueing(wg):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    # 4000 columns fit the scratch (about 2 MB of workspace) but not the
    # input transform's staged rows; refused like getkernelInfo refuses them,
    # with no CUDA error left behind
    prob = wg.make_problem(256, 256, 256, 1, 8, 3, 4000, 8)
    assert wg.lib().conv2d_fp16_noalloc(ctypes.byref(prob), None) == wg.ERR_UNSUPPORTED
    assert b"too wide" in wg.lib().conv2d_last_error_message()
    torch.cuda.synchronize()
    assert wg.noalloc_check_device()[0] == wg.OK
