"""GPU parity tests: the CUDA operator, called through its C ABI, against the
oracle (the reference verifier restated, pinned to the reference build) and
the golden vectors made by the reference's own verifier.

Tolerances (max over elements of |y - ref| / max(|ref|, rms(ref))):
F(2x3) 1e-2, F(4x3) 2e-2 for fp16 operands; bf16 operands are a precision
study with looser bounds written at each test.
"""
import os

import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "conv_golden.npz"))
GOLDEN_CASES = sorted({k.split("__")[0] for k in GOLDEN.files})
TOL = {2: 1e-2, 4: 2e-2}
# F(4x3) with fp16 operands and fewer than 16 input channels: the rounding of
# the Winograd-domain operands has a longer tail (about 8% of random cases with
# C < 16 reach 2e-2..2.7e-2 in a float64 simulation of the same arithmetic; no
# case with C >= 16 exceeded 1.7e-2)
TOL4_SMALL_C = 3e-2


def tol_for(m, c):
    return TOL4_SMALL_C if (m == 4 and c < 16) else TOL[m]
ALGOS = [-1, 0, 1, 2, 4]  # reference selection, F(4x3), F(2x3), F(2x3) fused, row F(4x3) fused


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def algo_m(algo):
    return 4 if algo in (0, 4) else 2


def run(wg, x16, w16, p=1, q=1, opts=None, stream=None):
    x = torch.from_numpy(np.ascontiguousarray(x16)).cuda()
    w = torch.from_numpy(np.ascontiguousarray(w16)).cuda()
    y, op = wg.conv2d_torch(x, w, p, q, opts, stream=stream)
    torch.cuda.synchronize()
    st, site = op.check_device()
    assert st == wg.OK, f"device wait gave up at site {site}"
    return y.cpu().numpy(), op


def opts_for(wg, algo, **kw):
    return wg.default_options(algo=algo, **kw)


def golden_case(name):
    seed, n, c, h, w, k, p, q = (int(v) for v in GOLDEN[name + "__meta"])
    kind = str(GOLDEN[name + "__kind"])
    if kind == "refstyle":
        x, wt = O.reference_style_inputs(n, c, h, w, k)
    else:
        x, wt = O.uniform_inputs(seed, n, c, h, w, k)
    return kind, x, wt, p, q, GOLDEN[name + "__out"].view(np.float16)


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_golden_vectors(wg, name, algo):
    kind, x, wt, p, q, ref = golden_case(name)
    y, op = run(wg, x, wt, p, q, opts_for(wg, algo))
    m = algo_m(op.algo)
    mx, mean, _ = O.rel_errors(y, ref)
    assert mx <= tol_for(m, x.shape[1]), (name, op.algo, mx, mean)
    if kind == "refstyle" and p == 1 and q == 1:
        # the reference benchmark's own acceptance check (src/main.cpp:123-132),
        # which it only ever applies with pad 1: relative to each output value,
        # it is not meaningful for the near-zero corner outputs of pad 2
        assert O.reference_criterion_failures(y, ref) == 0


@pytest.mark.parametrize("algo", [0, 1, 2, 4])
@pytest.mark.parametrize("shape", [
    (1, 3, 7, 7, 5), (2, 5, 14, 14, 27), (1, 16, 28, 28, 4), (3, 8, 13, 9, 12), (1, 70, 10, 10, 33),
    (1, 130, 9, 9, 130), (2, 64, 20, 20, 64), (1, 200, 8, 8, 300), (1, 24, 112, 112, 16), (4, 40, 7, 7, 260),
])
@pytest.mark.parametrize("pad", [(1, 1), (0, 0), (2, 1)])
def test_ragged_against_fp64(wg, algo, shape, pad):
    n, c, h, w, k = shape
    if h + 2 * pad[0] < 3 or w + 2 * pad[1] < 3:
        pytest.skip("no output")
    x, wt = O.uniform_inputs(hash((shape, pad)) % 1000, n, c, h, w, k, filt="normal")
    y, op = run(wg, x, wt, pad[0], pad[1], opts_for(wg, algo))
    _, r64 = O.conv2d_direct(x, wt, p=pad[0], q=pad[1], nthreads=8)
    mx, mean, _ = O.rel_errors(y, r64)
    assert op.algo == algo
    assert mx <= tol_for(algo_m(algo), c), (shape, pad, algo, mx, mean)


def _dev_array(wg, ptr, count, dtype):
    out = np.empty(count, dtype=dtype)
    wg.copy_to_host(out.ctypes.data, ptr, out.nbytes)
    return out


def read_m(wg, ptr, E, P, kp, mtype):
    """M read back from the workspace as float64 [E][P][Kp]: fp16
    M[E][Kp/8][P][8], fp32 M[E][Kp/4][P][4], or 24-bit M in blocks of 64
    tiles (upper 16 bits of each rounded fp32 value in
    H[NB][Kp/8][E][64][8], the next 8 bits in L[NB][Kp/8][E][64][8] right
    after H, NB = ceil(P / 64))."""
    if mtype == "fp16":
        Mw = _dev_array(wg, ptr, E * P * kp, np.float16).reshape(E, kp // 8, P, 8)
    elif mtype == "fp32":
        Mw = _dev_array(wg, ptr, E * P * kp, np.float32).reshape(E, kp // 4, P, 4)
    else:
        nb = (P + 63) // 64
        raw = _dev_array(wg, ptr, 3 * E * nb * 64 * kp, np.uint8)

        def plane(a):
            a = a.reshape(nb, kp // 8, E, 64, 8).transpose(2, 1, 0, 3, 4)
            return a.reshape(E, kp // 8, nb * 64, 8)[:, :, :P].astype(np.uint32)

        hi = plane(raw[:2 * E * nb * 64 * kp].view(np.uint16))
        lo = plane(raw[2 * E * nb * 64 * kp:])
        Mw = ((hi << 16) | (lo << 8)).view(np.float32)
    return Mw.transpose(0, 2, 1, 3).reshape(E, P, kp).astype(np.float64)


@pytest.mark.parametrize("h,w", [(11, 13), (9, 16), (24, 24)])
@pytest.mark.parametrize("algo,variant,mfp32", [(1, "F2", 0), (0, "F4", 0), (0, "F4", 1), (0, "F4Ref", 0)])
def test_transform_kernels_elementwise(wg, monkeypatch, algo, variant, mfp32, h, w):
    """U, V and M read back from the workspace, each against its restatement
    (the GEMM otherwise drops V from L2 once it is read, leaving its memory
    undefined).  F(4x3) stores M in 24 bits by default, in fp32 on request.
    W = 16 and 24 take the input transform's aligned-word reads, W = 13 its
    16-bit reads; 24 x 24 gives F(4x3) 72 tiles, two 64-tile blocks of 24-bit
    M with a partial last one."""
    monkeypatch.setenv("WG_CONV2D_KEEP_WORKSPACE", "1")
    n, c, k = 2, 20, 24
    x, wt = O.uniform_inputs(31, n, c, h, w, k)
    opts = opts_for(wg, algo, f4_points=1 if variant == "F4Ref" else 0, m_fp32=mfp32)
    y, op = run(wg, x, wt, 1, 1, opts)
    m = O.XFORMS[variant][0]
    E = (m + 2) ** 2
    cp, kp = (c + 7) // 8 * 8, (k + 7) // 8 * 8
    oh, ow = O.out_hw(h, w)
    P = n * (-(-oh // m)) * (-(-ow // m))
    Up, Vp, Mp = op.blob_pointers()
    # granule layouts: U[E][Cp/8][Kp][8], V[E][Cp/8][Pp][8], M[E][Kp/g][P][g]
    Pp = (P + 7) // 8 * 8
    U = _dev_array(wg, Up, E * kp * cp, np.float16).reshape(E, cp // 8, kp, 8).transpose(0, 2, 1, 3)
    assert np.all(U[:, k:] == 0)
    U = U[:, :k].reshape(E, k, cp).astype(np.float64)
    V = _dev_array(wg, Vp, E * Pp * cp, np.float16).reshape(E, cp // 8, Pp, 8).transpose(0, 2, 1, 3)
    V = V[:, :P].reshape(E, P, cp).astype(np.float64)
    mtype = "fp16" if m == 2 else ("fp32" if mfp32 else "24-bit")
    Mw = read_m(wg, Mp, E, P, kp, mtype)

    U_ref = O.filter_transform(wt.astype(np.float64), m, variant)
    V_ref = O.input_transform(x.astype(np.float64), m, 1, 1, variant)
    _, B, Gm, _ = O.XFORMS[variant]
    d = O.input_tiles(x.astype(np.float64), m, 1, 1)
    V_abs = np.einsum("ir,pcrs,js->ijpc", np.abs(B), np.abs(d), np.abs(B)).reshape(E, P, c)
    U_abs = np.einsum("ir,kcrs,js->ijkc", np.abs(Gm), np.abs(wt.astype(np.float64)), np.abs(Gm)).reshape(E, k, c)
    assert np.all(U[:, :, c:] == 0) and np.all(V[:, :, c:] == 0)
    # one fp16 rounding of an fp32 result (fp32 error bounded by the sum of |terms|)
    assert np.all(np.abs(U[:, :, :c] - U_ref) <= np.abs(U_ref) * 2.0 ** -10 + U_abs * 2.0 ** -20)
    assert np.all(np.abs(V[:, :, :c] - V_ref) <= np.abs(V_ref) * 2.0 ** -10 + V_abs * 2.0 ** -20)
    # GEMM of exactly the stored operands, fp32 accumulation
    M_ref = np.einsum("epc,ekc->epk", V, U)
    scale = np.einsum("epc,ekc->epk", np.abs(V), np.abs(U)) + 1e-30
    # fp32 accumulation, then the storage rounding: fp16 2^-11, 24 bits 2^-17
    tol = {"fp16": 2.0 ** -10, "fp32": 1e-5, "24-bit": 2.0 ** -16}[mtype]
    assert np.all(np.abs(Mw[:, :, :k] - M_ref) <= scale * tol)
    # output transform of exactly the stored M
    y_ref = O.output_transform(Mw[:, :, :k], m, n, k, oh, ow, variant)
    yscale = np.abs(y_ref).max()
    assert np.abs(y.astype(np.float64) - y_ref).max() <= yscale * 2.0 ** -10


@pytest.mark.parametrize("algo", [0, 1, 2, 4])
def test_repeat_calls_bit_identical(wg, algo):
    x, wt = O.uniform_inputs(3, 2, 48, 30, 30, 40)
    xt = torch.from_numpy(x).cuda()
    wtt = torch.from_numpy(wt).cuda()
    y, op = wg.conv2d_torch(xt, wtt, 1, 1, opts_for(wg, algo))
    first = y.clone()
    for _ in range(3):
        op(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert torch.equal(first, y)


@pytest.mark.parametrize("selection", ["reference", "default"])
def test_reference_harness_replay_cfg1(wg, selection):
    """1x64x56x56 -> 64, reference-style inputs, with the reference's own
    selection (F(4x3)) and with the default (autotuned) selection, checked as
    the reference benchmark checks it."""
    _, x, wt, p, q, ref = golden_case("refstyle_cfg1")
    y, op = run(wg, x, wt, p, q, opts_for(wg, wg.ALGO_REFERENCE) if selection == "reference" else None)
    if selection == "reference":
        assert op.algo == 0
    assert O.reference_criterion_failures(y, ref) == 0
    assert O.rel_errors(y, ref)[0] <= TOL[algo_m(op.algo)]


# The reference benchmark's contest shapes (N, C, H = W, K), its pre.sh and
# final.sh runs; 3x3, stride 1, pad 1.
CONTEST_SHAPES = [
    (64, 256, 14, 256), (256, 192, 14, 192), (16, 256, 26, 512), (32, 256, 14, 256),
    (2, 1280, 16, 1280), (2, 960, 64, 32), (16, 128, 64, 27), (16, 256, 32, 256),
    (16, 64, 128, 64), (2, 1920, 32, 640), (2, 640, 64, 640), (2, 320, 64, 4),
]


@pytest.mark.parametrize("selection", ["reference", "default"])
@pytest.mark.parametrize("n,c,hw,k", CONTEST_SHAPES)
def test_contest_shapes_as_the_reference_checks_them(wg, n, c, hw, k, selection):
    """Each contest shape through the drop-in API, with the reference's
    selection rule and with the default (autotuned) selection, on the
    reference's input fill (glibc rand, src/main.cpp:36-44), checked with the
    reference benchmark's criterion and against FP64 on image 0 and up to 8
    output channels spread over K (the share of the output the CPU oracle
    computes in about a second)."""
    x, wt = O.reference_style_inputs(n, c, hw, hw, k)
    y, op = run(wg, x, wt, 1, 1, opts_for(wg, wg.ALGO_REFERENCE) if selection == "reference" else None)
    if selection == "reference":
        assert op.algo == O.select_reference(n, c, hw, hw, k)
    ks = np.unique(np.linspace(0, k - 1, min(k, 8)).round().astype(int))
    ref16, r64 = O.conv2d_direct(x[:1], wt[ks], nthreads=8)
    got = y[:1, ks]
    assert O.reference_criterion_failures(got, ref16) == 0
    mx, mean, _ = O.rel_errors(got, r64)
    assert mx <= tol_for(algo_m(op.algo), c), (n, c, hw, k, op.algo, mx, mean)


def test_legacy_void_entry_point(wg):
    import ctypes
    x, wt = O.uniform_inputs(8, 1, 16, 12, 12, 16)
    xt, wtt = torch.from_numpy(x).cuda(), torch.from_numpy(wt).cuda()
    y = torch.empty((1, 16, 12, 12), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), 1, 16, 12, 12, 16)
    op = wg.Conv2d(prob)
    torch.cuda.synchronize()
    wg.lib().conv2d_fp16(op.ptr)  # legacy default stream, like the reference harness
    torch.cuda.synchronize()
    _, r64 = O.conv2d_direct(x, wt)
    assert O.rel_errors(y.cpu().numpy(), r64)[0] <= tol_for(algo_m(op.algo), 16)


def test_side_stream(wg):
    x, wt = O.uniform_inputs(9, 2, 32, 24, 24, 32)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        y, op = run(wg, x, wt, 1, 1, opts_for(wg, 1), stream=s.cuda_stream)
    _, r64 = O.conv2d_direct(x, wt)
    assert O.rel_errors(y, r64)[0] <= TOL[2]


def test_tile_scaling_is_exact(wg):
    """Power-of-two per-tile scaling changes no rounding for normal-range data.
    Heavy-tailed input (1% of entries x64) at C=256: in a float64 simulation of
    the same fp16 arithmetic its F(4x3) error is about 1.2-1.5e-2 (at C=64 it
    reaches 2.4e-2, which is why this case uses the wider channel count)."""
    x, wt = O.normal_inputs(4, 1, 256, 16, 16, 32, heavy=True)
    a, _ = run(wg, x, wt, 1, 1, opts_for(wg, 0, tile_scaling=0))
    b, _ = run(wg, x, wt, 1, 1, opts_for(wg, 0, tile_scaling=1))
    _, r64 = O.conv2d_direct(x, wt, nthreads=8)
    assert O.rel_errors(b, r64)[0] <= TOL[4]
    # only the fp32 sums in the GEMM and the output transform see scaled
    # values; the fp16 operand roundings are identical
    assert O.rel_errors(a, b)[0] <= 1e-3


@pytest.mark.parametrize("algo", [0, 1])
def test_l2_chunking_is_bit_identical(wg, algo):
    x, wt = O.uniform_inputs(5, 7, 32, 16, 16, 40)
    a, _ = run(wg, x, wt, 1, 1, opts_for(wg, algo))
    b, opb = run(wg, x, wt, 1, 1, opts_for(wg, algo, l2_chunk_bytes=1))  # one image per chunk
    assert opb.launches_per_call == 7 * 3
    assert np.array_equal(a.view(np.uint16), b.view(np.uint16))


@pytest.mark.parametrize("algo", [0, 1, 2])
def test_bf16_operands(wg, algo):
    x, wt = O.uniform_inputs(6, 2, 64, 18, 18, 64, filt="normal")
    y, _ = run(wg, x, wt, 1, 1, opts_for(wg, algo, operand_bf16=1))
    _, r64 = O.conv2d_direct(x, wt, nthreads=8)
    mx = O.rel_errors(y, r64)[0]
    assert mx <= (0.3 if algo == 0 else 6e-2), mx


def test_refresh_filter_after_in_place_change(wg):
    x, wt = O.uniform_inputs(12, 1, 16, 10, 10, 8)
    xt, wtt = torch.from_numpy(x).cuda(), torch.from_numpy(wt).cuda()
    y, op = wg.conv2d_torch(xt, wtt, 1, 1, opts_for(wg, 1))
    wt2 = (wt * np.float16(-0.5)).astype(np.float16)
    wtt.copy_(torch.from_numpy(wt2))
    s = torch.cuda.current_stream().cuda_stream
    op.refresh_filter(s)
    op(s)
    torch.cuda.synchronize()
    _, r64 = O.conv2d_direct(x, wt2)
    assert O.rel_errors(y.cpu().numpy(), r64)[0] <= TOL[2]


HOST_CASES = [(a, n, 24, 16, 24) for a in (0, 1, 2, 4) for n in (1, 2, 7)] + \
    [(a, 11, 64, 100, 64) for a in (0, 1, 2, 4)]  # 28.2 MB of copies: 4 chunks of 3, 3, 3, 2 images


@pytest.mark.parametrize("algo,n,c,h,k", HOST_CASES)
def test_host_buffer_entry_point(wg, algo, n, c, h, k):
    """Host in -> device -> host out, with the batch cut into overlapped
    chunks of at least 6 MB of copies (one chunk for the small cases, four
    for the large); equal to the device-buffer call bit for bit."""
    x, wt = O.uniform_inputs(13 + n, n, c, h, h, k)
    xt = torch.empty((n, c, h, h), dtype=torch.float16, device="cuda")
    wtt = torch.from_numpy(wt).cuda()
    y = torch.empty((n, k, h, h), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, h, k)
    op = wg.Conv2d(prob, opts_for(wg, algo))
    hin = torch.from_numpy(x).pin_memory()
    hout = torch.empty((n, k, h, h), dtype=torch.float16).pin_memory()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream().cuda_stream
    op.host(hin.data_ptr(), hout.data_ptr(), s)
    op.host(hin.data_ptr(), hout.data_ptr(), s)  # second call reuses the pipeline
    dev, _ = run(wg, x, wt, 1, 1, opts_for(wg, algo))
    assert np.array_equal(hout.numpy().view(np.uint16), dev.view(np.uint16))
    _, r64 = O.conv2d_direct(x, wt)
    assert O.rel_errors(hout.numpy(), r64)[0] <= TOL[algo_m(algo)]


def test_autotune_choice_is_cached_and_correct(wg):
    x, wt = O.uniform_inputs(21, 2, 64, 24, 24, 96)
    xt, wtt = torch.from_numpy(x).cuda(), torch.from_numpy(wt).cuda()
    y = torch.empty((2, 96, 24, 24), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), 2, 64, 24, 24, 96)
    wg.lib().conv2d_autotune_clear()
    a1 = wg.autotune(prob)
    a2 = wg.autotune(prob)
    assert a1 == a2 and a1[0] in (0, 1, 2, 4)
    op = wg.Conv2d(prob, opts_for(wg, wg.ALGO_AUTO))
    assert op.algo == a1[0]
    op(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    _, r64 = O.conv2d_direct(x, wt, nthreads=8)
    assert O.rel_errors(y.cpu().numpy(), r64)[0] <= TOL[algo_m(op.algo)]


def _to_bf16_bits(a):
    """float32 -> bf16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def _bf16_to_f64(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def _direct64(x, w, p=1):
    n, c, h, ww = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (p, p), (p, p)))
    out = np.zeros((n, w.shape[0], h + 2 * p - 2, ww + 2 * p - 2))
    for r in range(3):
        for s_ in range(3):
            out += np.einsum("nchw,kc->nkhw", xp[:, :, r:r + out.shape[2], s_:s_ + out.shape[3]], w[:, :, r, s_])
    return out


# bf16 tensors: F(2x3) and fused run bf16 operands (max error 2.0e-2 at C=512 in
# the precision study), F(4x3) fp16 operands with per-tile scaling; the bf16
# output rounding adds up to 2^-9 relative
BF16_TOL = {0: 2.5e-2, 1: 4e-2, 2: 4e-2}


@pytest.mark.parametrize("algo", [0, 1, 2])
@pytest.mark.parametrize("shape", [(2, 24, 16, 16, 32), (1, 40, 13, 11, 20), (3, 96, 28, 28, 64)])
def test_bf16_end_to_end(wg, algo, shape):
    """bf16 input, filter and output tensors against the FP64 direct
    convolution of the same bf16 values."""
    n, c, h, w, k = shape
    rng = np.random.default_rng(101 + algo)
    xb = _to_bf16_bits(rng.uniform(-1, 1, (n, c, h, w)))
    wb = _to_bf16_bits(rng.standard_normal((k, c, 3, 3)) / np.sqrt(9 * c))
    x = torch.from_numpy(xb.view(np.int16)).cuda().view(torch.bfloat16)
    wt = torch.from_numpy(wb.view(np.int16)).cuda().view(torch.bfloat16)
    y, op = wg.conv2d_torch(x, wt, 1, 1, opts_for(wg, algo))
    torch.cuda.synchronize()
    assert y.dtype == torch.bfloat16 and op.algo == algo
    got = _bf16_to_f64(y.view(torch.int16).cpu().numpy().view(np.uint16))
    ref = _direct64(_bf16_to_f64(xb), _bf16_to_f64(wb))
    assert O.rel_errors(got, ref)[0] <= BF16_TOL[algo]
    op.destroy()


NHWC_SHAPES = [(2, 24, 16, 16, 32, 1), (1, 16, 13, 11, 27, 1), (3, 40, 9, 30, 36, 2), (2, 64, 28, 28, 64, 0)]


@pytest.mark.parametrize("algo,mfp32", [(0, 0), (0, 1), (1, 0), (2, 0)])
@pytest.mark.parametrize("shape", NHWC_SHAPES)
def test_nhwc_matches_nchw_bit_for_bit(wg, algo, mfp32, shape):
    """Channels-last input and output (filter KCRS): the same V, M and output
    arithmetic as the NCHW path, so the result is the NCHW result transposed,
    bit for bit (the fused selection runs F(2x3) non-fused for NHWC).  F(4x3)
    with 24-bit M (granule layout, as NCHW) and with fp32 M (row-major, the
    NHWC output transform's own layout)."""
    n, c, h, w, k, pad = shape
    x, wt = O.uniform_inputs(41 + algo, n, c, h, w, k)
    y_nchw, op1 = run(wg, x, wt, pad, pad, opts_for(wg, 1 if algo == 2 else algo, m_fp32=mfp32))
    xt = torch.from_numpy(np.ascontiguousarray(x.transpose(0, 2, 3, 1))).cuda()
    wtt = torch.from_numpy(wt).cuda()
    oh, ow = h + 2 * pad - 2, w + 2 * pad - 2
    y = torch.full((n, oh, ow, k), float("nan"), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, w, k, pad, pad)
    op = wg.Conv2d(prob, opts_for(wg, algo, layout_nhwc=1, m_fp32=mfp32))
    op(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert op.check_device()[0] == wg.OK
    got = y.cpu().numpy().transpose(0, 3, 1, 2)
    assert np.array_equal(got.view(np.uint16), y_nchw.view(np.uint16))
    _, r64 = O.conv2d_direct(x, wt, pad, pad)
    assert O.rel_errors(got, r64)[0] <= TOL[algo_m(algo)]
    op.destroy()


@pytest.mark.parametrize("algo", [1, 0])
def test_nhwc_host_buffers_in_chunks(wg, algo):
    """NHWC through the host-buffer entry point, cut into 3 image chunks
    (F(2x3) with row-major fp16 M, F(4x3) with 24-bit granule-layout M)."""
    n, c, h, w, k = 11, 64, 100, 100, 64
    x, wt = O.uniform_inputs(77, n, c, h, w, k)
    xh = np.ascontiguousarray(x.transpose(0, 2, 3, 1))
    xt = torch.empty((n, h, w, c), dtype=torch.float16, device="cuda")
    wtt = torch.from_numpy(wt).cuda()
    y = torch.empty((n, h, w, k), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, w, k)
    op = wg.Conv2d(prob, opts_for(wg, algo, layout_nhwc=1))
    hin = torch.from_numpy(xh).pin_memory()
    hout = torch.empty((n, h, w, k), dtype=torch.float16).pin_memory()
    op.host(hin.data_ptr(), hout.data_ptr(), torch.cuda.current_stream().cuda_stream)
    dev, _ = run(wg, x, wt, 1, 1, opts_for(wg, algo))
    assert np.array_equal(hout.numpy().transpose(0, 3, 1, 2).view(np.uint16), dev.view(np.uint16))
    op.destroy()


def test_nhwc_refuses_channels_not_a_multiple_of_8(wg):
    x = torch.zeros((1, 12, 12, 20), dtype=torch.float16, device="cuda")
    w = torch.zeros((8, 20, 3, 3), dtype=torch.float16, device="cuda")
    y = torch.zeros((1, 12, 12, 8), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(x.data_ptr(), w.data_ptr(), y.data_ptr(), 1, 20, 12, 12, 8)
    with pytest.raises(wg.Conv2dError) as ei:
        wg.Conv2d(prob, opts_for(wg, 1, layout_nhwc=1))
    assert ei.value.status == wg.ERR_UNSUPPORTED


@pytest.mark.parametrize("sizes", ["6", "2,2,2", "1,1,1,1,1,1"])
@pytest.mark.parametrize("algo", [0, 1, 4])
def test_host_steps_match_single_host_calls(wg, monkeypatch, algo, sizes):
    """Consecutive host batches through one pipelined call (chunk i of batch
    b ordered only against chunk i of batch b-1) give each batch the output of
    its own conv2d_fp16_host call, bit for bit, with 1, 3 and 6 image chunks."""
    monkeypatch.setenv("WG_CONV2D_HOST_SIZES", sizes)
    n, c, h, k = 6, 40, 60, 48
    wt = O.uniform_inputs(5, n, c, h, h, k)[1]
    xs = [O.uniform_inputs(100 + i, n, c, h, h, k)[0] for i in range(3)]
    xt = torch.empty((n, c, h, h), dtype=torch.float16, device="cuda")
    wtt = torch.from_numpy(wt).cuda()
    y = torch.empty((n, k, h, h), dtype=torch.float16, device="cuda")
    op = wg.Conv2d(wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, h, k), opts_for(wg, algo))
    s = torch.cuda.current_stream().cuda_stream
    hins = [torch.from_numpy(x).pin_memory() for x in xs]
    single = []
    for hin in hins:
        hout = torch.empty((n, k, h, h), dtype=torch.float16).pin_memory()
        op.host(hin.data_ptr(), hout.data_ptr(), s)
        single.append(hout.numpy().copy())
    houts = [torch.full((n, k, h, h), float("nan"), dtype=torch.float16).pin_memory() for _ in xs]
    op.host_steps([hi.data_ptr() for hi in hins], [ho.data_ptr() for ho in houts], s)
    assert op.check_device()[0] == wg.OK
    for a, b in zip(single, houts):
        assert np.array_equal(a.view(np.uint16), b.numpy().view(np.uint16))
    _, r64 = O.conv2d_direct(xs[2], wt, nthreads=8)
    assert O.rel_errors(houts[2].numpy(), r64)[0] <= TOL[algo_m(algo)]
    op.destroy()


@pytest.mark.parametrize("algo", [0, 1, 2, 4])
def test_host_chunks_of_unaligned_images(wg, algo):
    """Images of 1,202,850 bytes: every host chunk after the first starts off
    a 16-byte boundary (chunks of 3, 3 and 2 images, 19 MB of copies)."""
    n, c, h, k = 8, 33, 135, 33
    x, wt = O.uniform_inputs(77, n, c, h, h, k)
    xt = torch.empty((n, c, h, h), dtype=torch.float16, device="cuda")
    wtt = torch.from_numpy(wt).cuda()
    y = torch.empty((n, k, h, h), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, h, k)
    op = wg.Conv2d(prob, opts_for(wg, algo))
    assert op.algo == algo
    hin = torch.from_numpy(x).pin_memory()
    hout = torch.empty((n, k, h, h), dtype=torch.float16).pin_memory()
    torch.cuda.synchronize()
    op.host(hin.data_ptr(), hout.data_ptr(), torch.cuda.current_stream().cuda_stream)
    st, site = op.check_device()
    assert st == wg.OK, site
    _, r64 = O.conv2d_direct(x, wt, nthreads=8)
    assert O.rel_errors(hout.numpy(), r64)[0] <= TOL[algo_m(algo)]


@pytest.mark.parametrize("algo", [0, 1])
def test_host_chunks_over_a_smaller_image_chunk_workspace(wg, algo):
    """With image chunking the non-fused workspace holds one image; every host
    chunk then runs as ranges of one image, and the result equals the
    device-buffer call bit for bit."""
    n, c, h, k = 11, 64, 100, 64
    x, wt = O.uniform_inputs(5, n, c, h, h, k)
    xt = torch.empty((n, c, h, h), dtype=torch.float16, device="cuda")
    wtt = torch.from_numpy(wt).cuda()
    y = torch.empty((n, k, h, h), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, h, k)
    op = wg.Conv2d(prob, opts_for(wg, algo, l2_chunk_bytes=1))
    hin = torch.from_numpy(x).pin_memory()
    hout = torch.empty((n, k, h, h), dtype=torch.float16).pin_memory()
    torch.cuda.synchronize()
    op.host(hin.data_ptr(), hout.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert op.check_device()[0] == wg.OK
    dev, _ = run(wg, x, wt, 1, 1, opts_for(wg, algo))
    assert np.array_equal(hout.numpy().view(np.uint16), dev.view(np.uint16))


@pytest.mark.parametrize("algo", [0, 2])
def test_host_chunk_sizes_from_the_environment(wg, monkeypatch, algo):
    """WG_CONV2D_HOST_SIZES lists the image count of every host chunk; valid
    lists (ragged, one chunk, one image per chunk, a trailing comma) and
    invalid ones (wrong sum, a zero, junk: these fall back to the default
    schedule) all equal the device-buffer call bit for bit."""
    n, c, h, k = 11, 64, 100, 64
    x, wt = O.uniform_inputs(21 + algo, n, c, h, h, k)
    xt = torch.empty((n, c, h, h), dtype=torch.float16, device="cuda")
    wtt = torch.from_numpy(wt).cuda()
    y = torch.empty((n, k, h, h), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, h, k)
    op = wg.Conv2d(prob, opts_for(wg, algo))
    dev, _ = run(wg, x, wt, 1, 1, opts_for(wg, algo))
    s = torch.cuda.current_stream().cuda_stream
    hin = torch.from_numpy(x).pin_memory()
    for sizes in ["1,3,5,2", "11", ",".join(["1"] * 11), "1,2,3", "4,0,7", "4,x,7", "5,6,", "1,2,3,4,1"]:
        monkeypatch.setenv("WG_CONV2D_HOST_SIZES", sizes)
        hout = torch.zeros((n, k, h, h), dtype=torch.float16).pin_memory()
        op.host(hin.data_ptr(), hout.data_ptr(), s)
        assert np.array_equal(hout.numpy().view(np.uint16), dev.view(np.uint16)), sizes
    assert op.check_device()[0] == wg.OK


@pytest.mark.parametrize("algo", [0, 4])
def test_host_pipeline_graph_replay(wg, monkeypatch, algo):
    """WG_CONV2D_HOST_GRAPH=1: the first host call captures the pipeline into
    a CUDA graph, later calls replay it; both equal the device-buffer call bit
    for bit, and a call with other host buffers captures a new graph."""
    monkeypatch.setenv("WG_CONV2D_HOST_GRAPH", "1")
    n, c, h, k = 11, 64, 100, 64
    x, wt = O.uniform_inputs(9 + algo, n, c, h, h, k)
    xt = torch.empty((n, c, h, h), dtype=torch.float16, device="cuda")
    wtt = torch.from_numpy(wt).cuda()
    y = torch.empty((n, k, h, h), dtype=torch.float16, device="cuda")
    prob = wg.make_problem(xt.data_ptr(), wtt.data_ptr(), y.data_ptr(), n, c, h, h, k)
    op = wg.Conv2d(prob, opts_for(wg, algo))
    dev, _ = run(wg, x, wt, 1, 1, opts_for(wg, algo))
    s = torch.cuda.current_stream().cuda_stream
    hin = torch.from_numpy(x).pin_memory()
    for _ in range(2):
        hout = torch.zeros((n, k, h, h), dtype=torch.float16).pin_memory()
        op.host(hin.data_ptr(), hout.data_ptr(), s)   # capture, then replay
        op.host(hin.data_ptr(), hout.data_ptr(), s)
        assert np.array_equal(hout.numpy().view(np.uint16), dev.view(np.uint16))
    assert op.check_device()[0] == wg.OK
