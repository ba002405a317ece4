"""GPU tests of the row-Winograd F(4x3) kernel (algorithm 4): 1-D F(4,3)
along the width with the three filter rows summed directly, one fused kernel.

Tolerance: max |y - ref| / max(|ref|, rms(ref)) <= 2e-2 against the fp64
direct convolution, the F(4x3) bound; the 1-D transform's operands grow far
less than the 2-D ones, so the measured errors sit near 1e-3."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = 2e-2


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _run(wg, x, wt, p, q, **opts):
    xt = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    wtt = torch.from_numpy(np.ascontiguousarray(wt)).cuda()
    y, op = wg.conv2d_torch(xt, wtt, p, q, wg.default_options(**opts))
    torch.cuda.synchronize()
    st, site = op.check_device()
    assert st == wg.OK, f"device wait gave up at site {site}"
    return y.cpu().numpy(), op


@pytest.mark.parametrize("shape,pad", [
    ((40, 48, 28, 28, 200), (1, 1)),   # 320 items: persistent CTAs walk several each
    ((3, 35, 17, 61, 70), (1, 1)),     # channel tails in both dimensions, 16 tiles per row
    ((2, 24, 30, 246, 40), (1, 1)),    # 62 tiles per row (the widest): two output rows per item
    ((1, 64, 9, 9, 64), (0, 2)),       # asymmetric padding
])
def test_row4x3_against_fp64(wg, shape, pad):
    n, c, h, w, k = shape
    x, wt = O.uniform_inputs(sum(shape) + pad[0], n, c, h, w, k, filt="normal")
    y, op = _run(wg, x, wt, pad[0], pad[1], algo=4)
    assert op.algo == 4
    _, r64 = O.conv2d_direct(x, wt, p=pad[0], q=pad[1], nthreads=8)
    mx, mean, _ = O.rel_errors(y, r64)
    assert mx <= TOL, (shape, pad, mx, mean)


@pytest.mark.parametrize("opts", [dict(operand_bf16=1), dict(f4_points=1), dict(tile_scaling=1)])
def test_row4x3_options_it_does_not_take_run_non_fused(wg, opts):
    x, wt = O.uniform_inputs(3, 1, 16, 12, 12, 16)
    _, op = _run(wg, x, wt, 1, 1, algo=4, **opts)
    assert op.algo == 0


def test_row4x3_wide_rows_run_non_fused(wg):
    # 300 output columns = 75 tiles per row: fewer than two rows per 128-row MMA
    x, wt = O.uniform_inputs(4, 1, 8, 4, 300, 8)
    y, op = _run(wg, x, wt, 1, 1, algo=4)
    assert op.algo == 0
    _, r64 = O.conv2d_direct(x, wt)
    assert O.rel_errors(y, r64)[0] <= 3e-2


@pytest.mark.parametrize("shape,pad", [
    ((2, 32, 14, 14, 64), 1), ((3, 48, 17, 23, 40), 1), ((1, 16, 30, 120, 72), 0), ((2, 64, 9, 9, 136), 2),
])
def test_row4x3_nhwc_matches_nchw_bit_for_bit(wg, shape, pad):
    """NHWC tensors go straight to the kernel; NCHW ones through the NHWC copy
    the plan makes, so the two results are the same numbers."""
    n, c, h, w, k = shape
    x, wt = O.uniform_inputs(61 + c, n, c, h, w, k, filt="normal")
    y_nchw, op1 = _run(wg, x, wt, pad, pad, algo=4)
    assert op1.algo == 4
    xt = torch.from_numpy(np.ascontiguousarray(x.transpose(0, 2, 3, 1))).cuda()
    wtt = torch.from_numpy(wt).cuda()
    oh, ow = h + 2 * pad - 2, w + 2 * pad - 2
    y = torch.full((n, oh, ow, k), float("nan"), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, w, k, pad, pad)
    op = wg.Conv2d(prob, wg.default_options(algo=4, layout_nhwc=1))
    assert op.algo == 4
    assert op.kernel_names() == ["row4x3"]
    op(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert op.check_device()[0] == wg.OK
    got = y.cpu().numpy().transpose(0, 3, 1, 2)
    assert np.array_equal(got.view(np.uint16), y_nchw.view(np.uint16))
    _, r64 = O.conv2d_direct(x, wt, pad, pad, nthreads=8)
    assert O.rel_errors(got, r64)[0] <= TOL
    op.destroy()


def test_row4x3_nhwc_channels_not_a_multiple_of_16_run_non_fused(wg):
    n, c, h, w, k = 1, 24, 10, 10, 16
    x, wt = O.uniform_inputs(8, n, c, h, w, k)
    xt = torch.from_numpy(np.ascontiguousarray(x.transpose(0, 2, 3, 1))).cuda()
    wtt = torch.from_numpy(wt).cuda()
    y = torch.empty((n, h, w, k), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, w, k)
    op = wg.Conv2d(prob, wg.default_options(algo=4, layout_nhwc=1))
    assert op.algo == 0
    op.destroy()


def test_row4x3_reports_its_launch_shape(wg):
    """getkernelInfo describes the kernel that runs: the NCHW kernel has 608
    threads per CTA (16 producer warps + MMA, staging and filter warps), the
    NHWC kernel 352, and at most one CTA per SM."""
    x, wt = O.uniform_inputs(3, 2, 32, 14, 30, 48)
    y, op = _run(wg, x, wt, 1, 1, algo=4)
    assert op.algo == 4 and op.info.threadx == 608
    assert 1 <= op.info.blockx <= torch.cuda.get_device_properties(0).multi_processor_count
    _, r64 = O.conv2d_direct(x, wt)
    assert O.rel_errors(y, r64)[0] <= TOL
    xt = torch.from_numpy(np.ascontiguousarray(x.transpose(0, 2, 3, 1))).cuda()
    wtt = torch.from_numpy(wt).cuda()
    yn = torch.empty((2, 14, 30, 48), dtype=torch.float16, device="cuda")
    opn = wg.Conv2d(wg.make_problem(xt.data_ptr(), wtt.data_ptr(), yn.data_ptr(), 2, 32, 14, 30, 48),
                    wg.default_options(algo=4, layout_nhwc=1))
    assert opn.algo == 4 and opn.info.threadx == 352
    opn.destroy()
