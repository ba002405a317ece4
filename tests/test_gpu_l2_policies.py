"""The L2 priorities and discards between the kernels change no result.

Where V fits in L2 it is written evict_last and read from there; where one
GEMM block covers all output channels its lines are discarded once read; M
larger than L2 is discarded by the output transform as soon as it is staged.
Each case runs a problem large enough to take those paths and compares it bit
for bit with the same call under WG_CONV2D_KEEP_WORKSPACE=1 (no discards),
and spot-checks a few output channels of the first and last images against
the fp64 direct convolution."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _call(wg, x, w, pad, algo, nhwc, keep):
    import os
    if keep:
        os.environ["WG_CONV2D_KEEP_WORKSPACE"] = "1"
    try:
        n, c, h, ww = x.shape
        k = w.shape[0]
        oh, ow = h + 2 * pad - 2, ww + 2 * pad - 2
        xin = x.permute(0, 2, 3, 1).contiguous() if nhwc else x
        y = torch.full((n, oh, ow, k) if nhwc else (n, k, oh, ow), float("nan"), dtype=torch.float16, device="cuda")
        prob = wg.make_problem(xin.data_ptr(), w.data_ptr(), y.data_ptr(), n, c, h, ww, k, pad, pad)
        op = wg.Conv2d(prob, wg.default_options(algo=algo, layout_nhwc=1 if nhwc else 0))
        op(torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert op.check_device()[0] == wg.OK
        got_algo = op.algo
        op.destroy()
        return (y.permute(0, 3, 1, 2) if nhwc else y).contiguous(), got_algo
    finally:
        os.environ.pop("WG_CONV2D_KEEP_WORKSPACE", None)


@pytest.mark.parametrize("shape,pad,algo,nhwc", [
    ((32, 256, 56, 56, 256), 1, 0, False),   # V 116 MB kept and discarded, M 231 MB discarded
    ((32, 256, 56, 56, 256), 1, 1, False),   # F(2x3): V 205 MB (not kept) discarded, M fp16 205 MB discarded
    ((32, 256, 56, 56, 256), 1, 0, True),    # NHWC: row-major M rows discarded
    ((33, 64, 57, 57, 520), 1, 0, False),    # P = 7425 (line-straddling M runs), three GEMM blocks (V kept)
])
def test_discards_change_no_result(wg, shape, pad, algo, nhwc):
    n, c, h, w, k = shape
    g = torch.Generator(device="cuda").manual_seed(sum(shape))
    x = (torch.rand((n, c, h, w), generator=g, device="cuda") * 2 - 1).half()
    wt = (torch.randn((k, c, 3, 3), generator=g, device="cuda") / (3 * c ** 0.5)).half()
    y, a = _call(wg, x, wt, pad, algo, nhwc, keep=False)
    y_keep, a_keep = _call(wg, x, wt, pad, algo, nhwc, keep=True)
    assert a == a_keep == algo
    assert torch.equal(y.view(torch.int16), y_keep.view(torch.int16))
    # fp64 spot check: first and last image, 8 output channels each
    xs, ws = x.cpu().numpy(), wt.cpu().numpy()
    for img in (0, n - 1):
        ks = np.linspace(0, k - 1, 8).astype(int)
        _, r64 = O.conv2d_direct(xs[img:img + 1], ws[ks], p=pad, q=pad, nthreads=8)
        got = y[img:img + 1, ks].cpu().numpy()
        assert O.rel_errors(got, r64)[0] <= (2e-2 if algo == 0 else 1e-2)
