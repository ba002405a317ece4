"""CPU tests of the oracle itself: it must reproduce the reference verifier
bit for bit before anything is checked against it."""
import ctypes
import hashlib

import numpy as np
import pytest

import oracle as O

GOLDEN = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "conv_golden.npz"))
CASES = sorted({k.split("__")[0] for k in GOLDEN.files})


def _case(name):
    seed, n, c, h, w, k, p, q = (int(v) for v in GOLDEN[name + "__meta"])
    kind = str(GOLDEN[name + "__kind"])
    return kind, seed, n, c, h, w, k, p, q


def _inputs(kind, seed, n, c, h, w, k):
    if kind == "refstyle":
        return O.reference_style_inputs(n, c, h, w, k)
    return O.uniform_inputs(seed, n, c, h, w, k)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_golden_bit_exact(name):
    kind, seed, n, c, h, w, k, p, q = _case(name)
    x, wt = _inputs(kind, seed, n, c, h, w, k)
    dig = hashlib.sha256(x.view(np.uint16).tobytes() + wt.view(np.uint16).tobytes()).hexdigest()
    assert dig == str(GOLDEN[name + "__digest"]), "input generator drifted"
    y16, y64 = O.conv2d_direct(x, wt, p=p, q=q, nthreads=4)
    assert np.array_equal(y16.view(np.uint16), GOLDEN[name + "__out"])
    # the fp16 result is the FP64 result rounded once
    assert np.array_equal(O.double_to_half(y64).view(np.uint16), GOLDEN[name + "__out"])


def test_glibc_rand_restatement_matches_libc():
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    expect = [libc.rand() for _ in range(5000)]
    assert list(O.glibc_rand(5000)) == expect


def test_double_to_half_matches_numpy():
    rng = np.random.default_rng(0)
    xs = rng.standard_normal(100000) * np.exp(rng.uniform(-25, 11, 100000))
    xs = np.concatenate([xs, [0.0, -0.0, 65504.0, 65520.0, 65519.99, 2.0 ** -24, 2.0 ** -25,
                              3 * 2.0 ** -26, np.inf, -np.inf]])
    with np.errstate(over="ignore"):
        expect = xs.astype(np.float16).view(np.uint16)
    assert np.array_equal(O.double_to_half(xs).view(np.uint16), expect)


def test_multithreaded_oracle_is_identical():
    x, wt = O.uniform_inputs(7, 3, 6, 11, 10, 7)
    a16, a64 = O.conv2d_direct(x, wt, nthreads=1)
    b16, b64 = O.conv2d_direct(x, wt, nthreads=5)
    assert np.array_equal(a16.view(np.uint16), b16.view(np.uint16))
    assert np.array_equal(a64, b64)


@pytest.mark.parametrize("variant", ["F2", "F4", "F4Ref"])
@pytest.mark.parametrize("pad", [(1, 1), (0, 0), (2, 2), (1, 0)])
def test_winograd_restatement_equals_direct_fp64(variant, pad):
    x, wt = O.uniform_inputs(5, 2, 5, 9, 11, 6)
    m = O.XFORMS[variant][0]
    y = O.winograd_conv(x.astype(np.float64), wt.astype(np.float64), m, *pad, variant=variant)
    _, r64 = O.conv2d_direct(x, wt, p=pad[0], q=pad[1])
    assert np.abs(y - r64).max() < 1e-10


# Expected selections follow src/conv2d.cpp:83-114 at the contest shapes
# (pre.sh / final.sh) and the three single-shape workloads.
SELECTIONS = [
    ((1, 64, 56, 56, 64), O.SELECT_4X3_NON_FUSED),
    ((32, 256, 56, 56, 256), O.SELECT_2X3_FUSED),
    ((32, 512, 28, 28, 512), O.SELECT_4X3_NON_FUSED),
    ((16, 128, 64, 64, 27), O.SELECT_2X3_FUSED),
    ((16, 256, 32, 32, 256), O.SELECT_4X3_NON_FUSED),
    ((16, 64, 128, 128, 64), O.SELECT_2X3_FUSED),
    ((2, 1920, 32, 32, 640), O.SELECT_2X3_NON_FUSED),
    ((2, 640, 64, 64, 640), O.SELECT_4X3_NON_FUSED),
    ((2, 320, 64, 64, 4), O.SELECT_2X3_FUSED),
]


@pytest.mark.parametrize("shape,expect", SELECTIONS)
def test_selection_restatement(shape, expect):
    assert O.select_reference(*shape) == expect


def test_reference_build_agrees_when_present():
    if O.ref_lib() is None:
        pytest.skip("reference verifier build not present on this machine")
    x, wt = O.uniform_inputs(9, 2, 7, 10, 13, 5)
    for p in (0, 1, 2):
        a, _ = O.conv2d_direct(x, wt, p=p, q=p)
        b = O.ref_conv2dcpu(x, wt, p=p, q=p)
        assert np.array_equal(a.view(np.uint16), b.view(np.uint16))


@pytest.mark.parametrize("variant", ["F4", "F4Ref"])
@pytest.mark.parametrize("shape,pad", [((2, 5, 9, 11, 6), (1, 1)), ((1, 3, 7, 7, 4), (0, 0)),
                                       ((2, 4, 6, 13, 3), (2, 2)), ((1, 6, 10, 5, 5), (1, 0))])
def test_row_winograd_restatement_equals_direct_fp64(variant, shape, pad):
    """The row-Winograd F(4x3) arithmetic (1-D F(4,3) along the width, direct
    sum over the filter rows) is an exact convolution in float64."""
    x, wt = O.uniform_inputs(8, *shape)
    y = O.row_winograd_conv(x.astype(np.float64), wt.astype(np.float64), *pad, variant=variant)
    _, r64 = O.conv2d_direct(x, wt, p=pad[0], q=pad[1])
    assert y.shape == r64.shape
    assert np.abs(y - r64).max() < 1e-10
