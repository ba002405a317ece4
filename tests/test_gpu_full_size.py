"""Full-size checks of the headline workloads, too large for the CPU oracle to
check whole: every output value against a float64 convolution on the GPU, and
a scaling property.

Scaling by two: with inputs on a 2^-8 grid in [-1, 1] every Winograd-domain
value of the input side is a normal fp16 number or zero, and every rounding on
the path (fp32 transforms, the fp16 operand cast, the tensor-core fp32
accumulation, fp32 M, the final fp16 cast) commutes with a power-of-two scale
of the input.  So y(2x) = 2 y(x) bit for bit wherever |y| lies above the
smallest normal fp16 value; below it the final rounding has a fixed spacing of
2^-24 and the two may differ by one step.  Paths with fp32 M or TMEM-resident
accumulators: F(4x3) non-fused, row F(4x3), fused F(2x3).  (F(2x3) non-fused
stores M in fp16, whose subnormal values break the exact scaling.)"""
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

CFG2 = (32, 256, 56, 56, 256)
CFG3 = (32, 512, 28, 28, 512)


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _conv(wg, x, wt, algo):
    n, c, h, w = x.shape
    k = wt.shape[0]
    y = torch.full((n, k, h, w), float("nan"), dtype=torch.float16, device="cuda")
    op = wg.Conv2d(wg.make_problem(x.data_ptr(), wt.data_ptr(), y.data_ptr(), n, c, h, w, k),
                   wg.default_options(algo=algo))
    op(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert op.check_device()[0] == wg.OK
    assert op.algo == algo
    op.destroy()
    return y


@pytest.mark.parametrize("shape,algo", [(CFG2, 0), (CFG2, 2), (CFG2, 4), (CFG3, 0), (CFG3, 4)])
def test_doubling_the_input_doubles_the_output(wg, shape, algo):
    n, c, h, w, k = shape
    g = torch.Generator(device="cuda").manual_seed(sum(shape) + algo)
    x = (torch.randint(-256, 257, (n, c, h, w), generator=g, device="cuda").float() / 256).half()
    wt = (torch.randn((k, c, 3, 3), generator=g, device="cuda") / (3 * c ** 0.5)).half()
    y1 = _conv(wg, x, wt, algo)
    y2 = _conv(wg, (2 * x.float()).half(), wt, algo)
    assert torch.isfinite(y1).all() and torch.isfinite(y2).all()
    twice = (2 * y1.float())
    normal = y1.float().abs() > 2.0 ** -14
    assert torch.equal(y2.float()[normal], twice[normal])
    if (~normal).any():
        assert float((y2.float()[~normal] - twice[~normal]).abs().max()) <= 2.0 ** -23


def _rel_err_fp64(y, x, wt):
    """max and mean of |y - ref| / max(|ref|, rms(ref)) over every output
    value; ref is torch's float64 convolution (pad 1) of the same fp16 values
    on the GPU, code that is not this library's."""
    ref = torch.nn.functional.conv2d(x.double(), wt.double(), padding=1)
    rms = ref.pow(2).mean().sqrt()
    rel = (y.double() - ref).abs() / torch.maximum(ref.abs(), rms)
    return float(rel.max()), float(rel.mean())


@pytest.mark.parametrize("shape,algo", [(CFG2, 0), (CFG2, 1), (CFG2, 2), (CFG2, 4), (CFG3, 0), (CFG3, 1), (CFG3, 4)])
def test_every_output_against_fp64(wg, shape, algo):
    """The whole output tensor of each headline workload against an FP64
    direct convolution of the same inputs (U[-1,1] input, N(0, 1/sqrt(9C))
    filter), at the bounds the operator is held to: 1e-2 for F(2x3) (non-fused
    and fused), 2e-2 for F(4x3) (non-fused and row)."""
    n, c, h, w, k = shape
    g = torch.Generator(device="cuda").manual_seed(7 + sum(shape) + algo)
    x = (torch.rand((n, c, h, w), generator=g, device="cuda") * 2 - 1).half()
    wt = (torch.randn((k, c, 3, 3), generator=g, device="cuda") / (3 * c ** 0.5)).half()
    y = _conv(wg, x, wt, algo)
    mx, mean = _rel_err_fp64(y, x, wt)
    bound = 1e-2 if algo in (1, 2) else 2e-2
    assert mx <= bound, (mx, mean)
    assert mean <= bound / 5, (mx, mean)
