"""CPU oracle for the Winograd 3x3 conv2d operator -- TEST INFRASTRUCTURE ONLY.

Only the tests, the smoke check and the benchmark's CPU-baseline leg import
this module, and only as the checker.  The operator library never calls it.

Contents
  * ctypes bindings of ``conv_oracle.c``: the reference verifier ``conv2dcpu``
    (reference ``include/verfiy.h:5-44``) restated in C, returning both the
    fp16-rounded result and the FP64 sum; the benchmark's glibc-``rand()``
    input fill (``src/main.cpp:36-44``); the algorithm selection of
    ``getkernelInfo`` (``src/conv2d.cpp:24-116``).
  * ctypes binding of the reference's own ``conv2dcpu`` compiled from the
    reference sources (``oracle/_ref``), when that build exists.
  * numpy float64 restatements of the Winograd transforms, with the matrices
    read off the reference kernels:
      F(2x3): B^T ``src/winograd_2x3_non_fused.cpp:321-375``,
              G ``:260-300``, A^T ``:184-227``;
      F(4x3): B^T ``src/winograd_4x3_non_fused.cpp:41-146``,
              G ``:342-404``, A^T ``:427-525``.
    Tile order p = b*tilesPerImg + th*tilesW + tw (``include/common.h:113-120``)
    and element order e = row*alpha + col (``V[h*TILE_IN_W + w]``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_verify.so")

SELECT_4X3_NON_FUSED = 0
SELECT_2X3_NON_FUSED = 1
SELECT_2X3_FUSED = 2

_lib = None
_ref = None


def build(ref_dir: str | None = None) -> None:
    """Compile the oracle (and the reference verifier when its tree exists)."""
    cmd = ["make", "-s", "-C", HERE]
    if ref_dir:
        cmd.append(f"REF={ref_dir}")
    subprocess.run(cmd, check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        u16p = ctypes.POINTER(ctypes.c_uint16)
        f64p = ctypes.POINTER(ctypes.c_double)
        L.orc_conv2d_direct.argtypes = [u16p, u16p, u16p, f64p] + [ctypes.c_int] * 12
        L.orc_conv2d_direct.restype = ctypes.c_int
        L.orc_fill_reference_style.argtypes = [u16p, ctypes.c_size_t, u16p, ctypes.c_size_t]
        L.orc_glibc_rand.argtypes = [ctypes.c_uint32, ctypes.POINTER(ctypes.c_int32), ctypes.c_size_t]
        L.orc_double_to_half_array.argtypes = [f64p, u16p, ctypes.c_size_t]
        L.orc_select_reference.argtypes = [ctypes.c_uint] * 11
        L.orc_select_reference.restype = ctypes.c_int
        _lib = L
    return _lib


def ref_lib():
    """The reference's own conv2dcpu, or None when oracle/_ref was not built."""
    global _ref
    if _ref is None and os.path.exists(REF_LIB_PATH):
        try:
            R = ctypes.CDLL(REF_LIB_PATH)
        except OSError:  # e.g. a build for another machine architecture
            return None
        u16p = ctypes.POINTER(ctypes.c_uint16)
        R.ref_conv2dcpu.argtypes = [u16p, u16p, u16p] + [ctypes.c_int] * 11
        R.ref_fill_reference_style.argtypes = [u16p, ctypes.c_long, u16p, ctypes.c_long]
        _ref = R
    return _ref


def _u16(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))


def _f64(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def out_hw(h, w, r=3, s=3, u=1, v=1, p=1, q=1):
    return (h + 2 * p - r) // u + 1, (w + 2 * q - s) // v + 1


def conv2d_direct(x16, w16, p=1, q=1, u=1, v=1, nthreads=1, want64=True):
    """Restated conv2dcpu.  x16 [N,C,H,W] and w16 [K,C,R,S] as float16 arrays.

    Returns (out16 float16 [N,K,OH,OW], out64 float64 or None)."""
    x16 = np.ascontiguousarray(x16, dtype=np.float16)
    w16 = np.ascontiguousarray(w16, dtype=np.float16)
    n, c, h, w = x16.shape
    k, c2, r, s = w16.shape
    assert c == c2
    oh, ow = out_hw(h, w, r, s, u, v, p, q)
    out16 = np.zeros((n, k, oh, ow), dtype=np.uint16)
    out64 = np.zeros((n, k, oh, ow), dtype=np.float64) if want64 else None
    rc = lib().orc_conv2d_direct(
        _u16(x16.view(np.uint16)), _u16(w16.view(np.uint16)), _u16(out16),
        _f64(out64) if want64 else ctypes.POINTER(ctypes.c_double)(),
        n, c, h, w, k, r, s, u, v, p, q, int(nthreads))
    if rc != 0:
        raise ValueError("shape has no output")
    return out16.view(np.float16), out64


def ref_conv2dcpu(x16, w16, p=1, q=1, u=1, v=1):
    """The reference's own conv2dcpu (compiled from its sources); fp16 result."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference verifier build not available")
    x16 = np.ascontiguousarray(x16, dtype=np.float16)
    w16 = np.ascontiguousarray(w16, dtype=np.float16)
    n, c, h, w = x16.shape
    k, _, r, s = w16.shape
    oh, ow = out_hw(h, w, r, s, u, v, p, q)
    out = np.zeros((n, k, oh, ow), dtype=np.uint16)
    R.ref_conv2dcpu(_u16(x16.view(np.uint16)), _u16(w16.view(np.uint16)), _u16(out),
                    n, c, h, w, k, r, s, u, v, p, q)
    return out.view(np.float16)


def reference_style_inputs(n, c, h, w, k, r=3, s=3):
    """Inputs exactly as the reference benchmark makes them (glibc rand)."""
    x = np.zeros(n * c * h * w, dtype=np.uint16)
    wt = np.zeros(k * c * r * s, dtype=np.uint16)
    lib().orc_fill_reference_style(_u16(x), x.size, _u16(wt), wt.size)
    return x.view(np.float16).reshape(n, c, h, w), wt.view(np.float16).reshape(k, c, r, s)


def ref_reference_style_inputs(n, c, h, w, k, r=3, s=3):
    """Same fill through the host compiler's own rand() (reference build)."""
    R = ref_lib()
    x = np.zeros(n * c * h * w, dtype=np.uint16)
    wt = np.zeros(k * c * r * s, dtype=np.uint16)
    R.ref_fill_reference_style(_u16(x), x.size, _u16(wt), wt.size)
    return x.view(np.float16).reshape(n, c, h, w), wt.view(np.float16).reshape(k, c, r, s)


def glibc_rand(count, seed=1):
    out = np.zeros(count, dtype=np.int32)
    lib().orc_glibc_rand(seed, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), count)
    return out


def double_to_half(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros(x.shape, dtype=np.uint16)
    lib().orc_double_to_half_array(_f64(x), _u16(out), x.size)
    return out.view(np.float16)


def select_reference(n, c, h, w, k, r=3, s=3, u=1, v=1, p=1, q=1):
    return lib().orc_select_reference(n, c, h, w, k, r, s, u, v, p, q)


# ---- seeded synthetic inputs ------------------------------------------------

def uniform_inputs(seed, n, c, h, w, k, lo=-1.0, hi=1.0, filt="uniform"):
    """fp16 input ~U[lo,hi]; filter ~U[lo,hi] or N(0, std=1/sqrt(9C))."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(lo, hi, size=(n, c, h, w)).astype(np.float16)
    if filt == "uniform":
        wt = rng.uniform(lo, hi, size=(k, c, 3, 3)).astype(np.float16)
    else:
        wt = (rng.standard_normal((k, c, 3, 3)) / np.sqrt(9.0 * c)).astype(np.float16)
    return x, wt


def normal_inputs(seed, n, c, h, w, k, heavy=False):
    """fp16 input ~N(0,1) (optionally 1% of entries x64); filter N(0, 1/sqrt(9C))."""
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, c, h, w))
    if heavy:
        mask = rng.random((n, c, h, w)) < 0.01
        x = np.where(mask, x * 64.0, x)
    wt = rng.standard_normal((k, c, 3, 3)) / np.sqrt(9.0 * c)
    return x.astype(np.float16), wt.astype(np.float16)


# ---- error metrics -----------------------------------------------------------

def rel_errors(y, ref):
    """rel_i = |y_i - ref_i| / max(|ref_i|, rms(ref)); returns (max, mean, l2)."""
    y = np.asarray(y, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    rms = float(np.sqrt(np.mean(ref * ref))) if ref.size else 0.0
    denom = np.maximum(np.abs(ref), rms if rms > 0 else 1.0)
    rel = np.abs(y - ref) / denom
    l2 = float(np.linalg.norm(y - ref) / max(np.linalg.norm(ref), 1e-300))
    if not np.all(np.isfinite(y)):
        return float("inf"), float("inf"), float("inf")
    return float(rel.max(initial=0.0)), float(rel.mean()) if rel.size else 0.0, l2


def reference_criterion_failures(gpu, cpu):
    """The reference benchmark's check (src/main.cpp:123-132):
    |gpu - cpu| / gpu > 0.01, or NaN/Inf -> error.  Returns the failing count
    (the reference stops at the first one)."""
    g = np.asarray(gpu, dtype=np.float32)
    c = np.asarray(cpu, dtype=np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = np.abs(g - c) / g
    bad = (ratio > 0.01) | np.isnan(g) | np.isinf(g)
    return int(bad.sum())


# ---- Winograd transforms (float64 restatements) ------------------------------

def _mat(rows):
    return np.array([[float(Fraction(x)) for x in r] for r in rows], dtype=np.float64)


BT = {
    2: _mat([[1, 0, -1, 0], [0, 1, 1, 0], [0, -1, 1, 0], [0, 1, 0, -1]]),
    4: _mat([[4, 0, -5, 0, 1, 0], [0, -4, -4, 1, 1, 0], [0, 4, -4, -1, 1, 0],
             [0, -2, -1, 2, 1, 0], [0, 2, -1, -2, 1, 0], [0, 4, 0, -5, 0, 1]]),
}
G = {
    2: _mat([[1, 0, 0], ["1/2", "1/2", "1/2"], ["1/2", "-1/2", "1/2"], [0, 0, 1]]),
    4: _mat([["1/4", 0, 0], ["-1/6", "-1/6", "-1/6"], ["-1/6", "1/6", "-1/6"],
             ["1/24", "1/12", "1/6"], ["1/24", "-1/12", "1/6"], [0, 0, 1]]),
}
AT = {
    2: _mat([[1, 1, 1, 0], [0, 1, -1, -1]]),
    4: _mat([[1, 1, 1, 1, 1, 0], [0, 1, -1, 2, -2, 0], [0, 1, 1, 4, 4, 0], [0, 1, -1, 8, -8, 1]]),
}

# F(4x3) with interpolation points 0, +-1, 1/2, -2 (the operator's default
# F(4x3) transform; the reference's points are 0, +-1, +-2 above).  Same
# Cook-Toom construction: A^T columns are the points' powers, G rows are the
# Lagrange weights, B^T solves A^T((G g) . (B^T d)) = correlation(d, g).
BT_F4S = _mat([[1, "-3/2", -2, "3/2", 1, 0], [0, -1, "1/2", "5/2", 1, 0], [0, 1, "-5/2", "1/2", 1, 0],
               [0, -2, -1, 2, 1, 0], [0, "1/2", -1, "-1/2", 1, 0], [0, 1, "-3/2", -2, "3/2", 1]])
G_F4S = _mat([[1, 0, 0], ["1/3", "1/3", "1/3"], ["-1/3", "1/3", "-1/3"], ["-16/15", "-8/15", "-4/15"],
              ["1/15", "-2/15", "4/15"], [0, 0, 1]])
AT_F4S = _mat([[1, 1, 1, 1, 1, 0], [0, 1, -1, "1/2", -2, 0], [0, 1, 1, "1/4", 4, 0], [0, 1, -1, "1/8", -8, 1]])

# transform sets by name: "F2", "F4" (points 0,+-1,1/2,-2), "F4Ref" (0,+-1,+-2)
XFORMS = {
    "F2": (2, BT[2], G[2], AT[2]),
    "F4": (4, BT_F4S, G_F4S, AT_F4S),
    "F4Ref": (4, BT[4], G[4], AT[4]),
}


def tile_grid(n, h, w, m, p=1, q=1):
    oh, ow = out_hw(h, w, 3, 3, 1, 1, p, q)
    th, tw = -(-oh // m), -(-ow // m)
    return oh, ow, th, tw, n * th * tw


def input_tiles(x, m, p=1, q=1):
    """Input patches d[P][C][alpha][alpha] (zero outside the image)."""
    x = np.asarray(x, dtype=np.float64)
    n, c, h, w = x.shape
    a = m + 2
    oh, ow, th, tw, P = tile_grid(n, h, w, m, p, q)
    Hp, Wp = th * m + 2, tw * m + 2
    xp = np.zeros((n, c, Hp, Wp))
    hh = min(h, Hp - p)
    ww = min(w, Wp - q)
    xp[:, :, p:p + hh, q:q + ww] = x[:, :, :hh, :ww]
    d = np.zeros((n, th, tw, c, a, a))
    for i in range(th):
        for j in range(tw):
            d[:, i, j] = xp[:, :, i * m:i * m + a, j * m:j * m + a]
    return d.reshape(P, c, a, a)


def _xf(m, variant):
    if variant is None:
        return m, BT[m], G[m], AT[m]
    return XFORMS[variant]


def input_transform(x, m, p=1, q=1, variant=None):
    """V[e][P][C] = (B^T d B)[e // alpha][e % alpha]."""
    m, B, _, _ = _xf(m, variant)
    d = input_tiles(x, m, p, q)
    v = np.einsum("ir,pcrs,js->ijpc", B, d, B)
    a = m + 2
    return v.reshape(a * a, d.shape[0], d.shape[1])


def filter_transform(wt, m, variant=None):
    """U[e][K][C] = (G g G^T)[e // alpha][e % alpha]."""
    m, _, Gm, _ = _xf(m, variant)
    g = np.asarray(wt, dtype=np.float64)
    u = np.einsum("ir,kcrs,js->ijkc", Gm, g, Gm)
    a = m + 2
    return u.reshape(a * a, g.shape[0], g.shape[1])


def output_transform(Mw, m, n, k, oh, ow, variant=None):
    """Mw[e][P][K] -> out [N][K][OH][OW] via A^T M A, clipped to the image."""
    m, _, _, A = _xf(m, variant)
    a = m + 2
    P = Mw.shape[1]
    th, tw = -(-oh // m), -(-ow // m)
    Mm = Mw.reshape(a, a, P, k)
    y = np.einsum("ir,rspk,js->pkij", A, Mm, A)  # [P][K][m][m]
    y = y.reshape(n, th, tw, k, m, m).transpose(0, 3, 1, 4, 2, 5).reshape(n, k, th * m, tw * m)
    return y[:, :, :oh, :ow]


def winograd_conv(x, wt, m, p=1, q=1, variant=None):
    """Whole Winograd convolution in float64 (equals the direct conv up to
    float64 rounding)."""
    n, c, h, w = x.shape
    k = wt.shape[0]
    oh, ow = out_hw(h, w, 3, 3, 1, 1, p, q)
    V = input_transform(x, m, p, q, variant)
    U = filter_transform(wt, m, variant)
    Mw = np.einsum("epc,ekc->epk", V, U)
    return output_transform(Mw, m, n, k, oh, ow, variant)


def row_winograd_conv(x, wt, p=1, q=1, variant="F4"):
    """Row-Winograd F(4x3) in float64: the 1-D transform F(4,3) along the
    width and the three filter rows summed directly along the height, the
    arithmetic of the operator's fused row kernel (it has no counterpart in
    the reference).  For output row i and 4-wide tile t:
        y[i][4t:4t+4] = A^T sum_r sum_c (G g[k][c][r]) . (B^T x[c][i+r-p][4t-q:4t-q+6]).
    Equals the direct convolution up to float64 rounding."""
    m, B, Gm, A = XFORMS[variant]
    x = np.asarray(x, dtype=np.float64)
    g = np.asarray(wt, dtype=np.float64)
    n, c, h, w = x.shape
    k = g.shape[0]
    oh, ow = out_hw(h, w, 3, 3, 1, 1, p, q)
    a = m + 2
    tw = -(-ow // m)
    wp = tw * m + 2
    xp = np.zeros((n, c, oh + 2, wp))
    hh = min(h, oh + 2 - p)
    ww = min(w, wp - q)
    xp[:, :, p:p + hh, q:q + ww] = x[:, :, :hh, :ww]
    d = np.stack([xp[:, :, :, t * m:t * m + a] for t in range(tw)], axis=3)   # [N][C][OH+2][TW][alpha]
    v = np.einsum("ej,nchtj->nchte", B, d)
    u = np.einsum("es,kcrs->kcre", Gm, g)                                    # [K][C][3][alpha]
    mm = sum(np.einsum("kce,ncite->nkite", u[:, :, r, :], v[:, :, r:r + oh]) for r in range(3))
    y = np.einsum("oe,nkite->nkito", A, mm).reshape(n, k, oh, tw * m)
    return y[:, :, :, :ow]


def direct_flops(n, c, h, w, k, p=1, q=1):
    oh, ow = out_hw(h, w, 3, 3, 1, 1, p, q)
    return 2.0 * n * k * oh * ow * c * 9
