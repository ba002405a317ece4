// Winograd filter, input and output transform kernels (HBM-bound).
//
// Layouts in HBM (one convolution, E = alpha^2 Winograd elements):
//   input   x[N][C][H][W]            fp16 (caller's NCHW)
//   filter  w[K][C][3][3]            fp16 (caller's KCRS)
//   U       U[E][Cp/8][Kp][8]        operand type (fp16 or bf16)
//   V       V[E][Cp/8][Pp][8]        operand type, P = tiles in the batch,
//                                    Pp = P rounded up to 8
//   M       M[E][Kp/8][P][8]  fp16   (F(2x3)),  M[E][Kp/4][P][4]  fp32  (F(4x3) on
//           request), 24-bit planes H[NB][Kp/8][E][64][8] and L[NB][Kp/8][E][64][8]
//           (F(4x3) default; NB = ceil(P/64) blocks of 64 tiles)
//   output  y[N][K][OH][OW]          fp16
// Cp, Kp are C, K rounded up to 8.  The contraction index is split into
// 16-byte granules of 8 channels; within an element e, granule g holds one
// 16-byte row per tile (V), output channel (U) or tile (M).  So:
//   * a thread that owns one tile and one granule writes (or reads) 16
//     contiguous bytes and a warp of consecutive tiles a contiguous 512 bytes;
//   * a TMA box of 8 granules x 128 rows lands in shared memory exactly in the
//     tcgen05 canonical K-major layout (8-row x 16-byte core matrices).
// The reference keeps the tile index innermost instead (V[e][C][P],
// U[e][K][C], M[e][K][P]; src/winograd_2x3_non_fused.cpp:296-299,371-374,
// include/hep_sgemm.h:32-34).
//
// The input transform stages the rows its block of tiles needs with
// cp.async.bulk (one contiguous copy per channel), then computes from shared
// memory with lanes over consecutive tiles.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdlib>

#include "wg_kernels.h"
#include "wg_launch.h"
#include "wg_ptx.cuh"
#include "wg_transforms.cuh"

namespace wg {

Geom make_geom(int n, int c, int h, int w, int k, int pad_h, int pad_w, int m) {
    Geom g;
    g.n = n; g.c = c; g.h = h; g.w = w; g.k = k;
    g.pad_h = pad_h; g.pad_w = pad_w;
    g.oh = h + 2 * pad_h - 2;
    g.ow = w + 2 * pad_w - 2;
    g.m = m;
    g.alpha = m + 2;
    g.tiles_h = (g.oh + m - 1) / m;
    g.tiles_w = (g.ow + m - 1) / m;
    g.P = static_cast<long long>(n) * g.tiles_h * g.tiles_w;
    g.cp = (c + 7) / 8 * 8;
    g.kp = (k + 7) / 8 * 8;
    return g;
}

namespace {

template <class T> __device__ __forceinline__ uint32_t pack2(float a, float b);
template <> __device__ __forceinline__ uint32_t pack2<__half>(float a, float b) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}
template <> __device__ __forceinline__ uint32_t pack2<__nv_bfloat16>(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}
template <class T> __device__ __forceinline__ T from_f32(float v);
template <> __device__ __forceinline__ __half from_f32<__half>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

// Element type of the caller's tensors (input, filter, output): fp16, or
// bf16 for the end-to-end bf16 option.
template <bool BF> struct IO;
template <> struct IO<false> {
    using T = __half;
    __device__ static float to_f(T v) { return __half2float(v); }
    // two 16-bit values packed in one word (low = first) to fp32
    __device__ static float2 pair(uint32_t h) { return __half22float2(*reinterpret_cast<const __half2*>(&h)); }
};
template <> struct IO<true> {
    using T = __nv_bfloat16;
    __device__ static float to_f(T v) { return __bfloat162float(v); }
    __device__ static float2 pair(uint32_t h) { return make_float2(__uint_as_float(h << 16), __uint_as_float(h & 0xffff0000u)); }
};

// ---- filter transform --------------------------------------------------------
// One thread per (k, c); U[e][c/8][k][c%8].

template <class TF, class OutT, bool WB>
__global__ void __launch_bounds__(256) filter_transform_kernel(const typename IO<WB>::T* __restrict__ w,
                                                               OutT* __restrict__ U, int K, int C, int Cp, int Kp) {
    constexpr int A = TF::ALPHA;
    const long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<long long>(Kp) * Cp) return;
    const int k = static_cast<int>(idx / Cp), c = static_cast<int>(idx % Cp);
    float g[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) g[i] = 0.f;
    if (c < C && k < K) {
        const typename IO<WB>::T* src = w + (static_cast<long long>(k) * C + c) * 9;
#pragma unroll
        for (int i = 0; i < 9; ++i) g[i] = IO<WB>::to_f(src[i]);
    }
    float u[A * A];
    filter_tile_transform<TF>(g, u);
    const int CG = Cp / 8;
#pragma unroll
    for (int e = 0; e < A * A; ++e)
        U[((static_cast<long long>(e) * CG + c / 8) * Kp + k) * 8 + (c & 7)] = from_f32<OutT>(u[e]);
}

// ---- per-tile scale ------------------------------------------------------------
// scale[p] = 2^(8 - floor(log2 amax)): the scaled patch maximum lies in
// [256, 512), far from the fp16 subnormal range; V then stays below 65504
// for both F(4x3) point sets (|V| <= 100 max|d|).  A power of two changes
// no rounding of normal-range values.

template <int M, bool XB>
__global__ void __launch_bounds__(256) tile_scale_kernel(const typename IO<XB>::T* __restrict__ x, float* __restrict__ scale,
                                                         int C, int H, int W, int pad_h, int pad_w, int tiles_h,
                                                         int tiles_w, long long P) {
    constexpr int A = M + 2;
    pdl_wait();
    pdl_trigger();
    const long long p = static_cast<long long>(blockIdx.x) * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= P) return;
    const int tw = static_cast<int>(p % tiles_w);
    const int th = static_cast<int>((p / tiles_w) % tiles_h);
    const long long n = p / (static_cast<long long>(tiles_w) * tiles_h);
    const int y0 = th * M - pad_h, x0 = tw * M - pad_w;
    float amax = 0.f;
    for (int c = lane; c < C; c += 32) {
        const typename IO<XB>::T* plane = x + (n * C + c) * static_cast<long long>(H) * W;
        for (int i = 0; i < A; ++i) {
            const int y = y0 + i;
            if (y < 0 || y >= H) continue;
            for (int j = 0; j < A; ++j) {
                const int xx = x0 + j;
                if (xx < 0 || xx >= W) continue;
                amax = fmaxf(amax, fabsf(IO<XB>::to_f(plane[static_cast<long long>(y) * W + xx])));
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if (lane == 0) {
        float s = 1.f;
        if (amax > 0.f && isfinite(amax)) {
            int ex;
            frexpf(amax, &ex);                   // amax = f * 2^ex, f in [0.5, 1)
            const int fl = ex - 1;               // floor(log2(amax))
            s = ldexpf(1.f, max(-100, min(100, 8 - fl)));
        }
        scale[p] = s;
    }
}

// ---- input transform -------------------------------------------------------------
// Persistent CTAs walk a list of work items (image, block of tile rows, block
// of up to 32 channels).  Each item's input rows are staged in shared memory
// with one cp.async.bulk per channel, issued by the producer warp one or two
// items ahead into a ring of two or three buffers, so the copies of the next
// items overlap the arithmetic of this one.  A thread transforms one channel pair of one tile in
// packed fp32x2 arithmetic; four lanes complete one 16-byte granule row and a
// warp of eight consecutive tiles stores 128 contiguous bytes per element.

constexpr int kInComputeWarps = 7;
constexpr int kInThreads = 32 * (kInComputeWarps + 1);  // + one producer warp
constexpr int kInMaxBufs = 3;   // staging buffers: 3 where two CTAs of them fit an SM, else 2
constexpr int kInHeader = 96;   // 2 x kInMaxBufs mbarriers, an abort flag, 32 zero bytes at 64
constexpr int kInSlack = 256;   // bytes before and after the two buffers: reads
                                // of columns in the padding (masked to zero)
                                // stay inside the CTA's shared memory

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
// a*b + c and friends in packed fp32x2 (one instruction for two channels)
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); }

// B^T d on an ALPHA-vector of channel pairs (same matrices as TF::bt).
template <class TF> struct Bt2;
template <> struct Bt2<F2> {
    __device__ __forceinline__ static void run(const float2 (&d)[4], float2 (&o)[4]) {
        o[0] = sub2(d[0], d[2]);
        o[1] = add2(d[1], d[2]);
        o[2] = sub2(d[2], d[1]);
        o[3] = sub2(d[1], d[3]);
    }
};
template <> struct Bt2<F4> {  // points 0, +-1, 1/2, -2
    __device__ __forceinline__ static void run(const float2 (&d)[6], float2 (&o)[6]) {
        const float2 t = sub2(d[3], d[1]), u = sub2(d[4], d[2]);
        o[0] = add2(fma2(d[2], f2(-2.f), fma2(t, f2(1.5f), d[0])), d[4]);
        o[1] = sub2(fma2(d[3], f2(2.5f), fma2(d[2], f2(0.5f), d[4])), d[1]);
        o[2] = add2(fma2(d[2], f2(-2.5f), fma2(d[3], f2(0.5f), d[4])), d[1]);
        o[3] = fma2(t, f2(2.f), u);
        o[4] = fma2(t, f2(-0.5f), u);
        o[5] = add2(fma2(d[3], f2(-2.f), fma2(u, f2(1.5f), d[1])), d[5]);
    }
};
template <> struct Bt2<F4Ref> {  // points 0, +-1, +-2
    __device__ __forceinline__ static void run(const float2 (&d)[6], float2 (&o)[6]) {
        const float2 t = sub2(d[3], d[1]), u = sub2(d[4], d[2]);
        o[0] = fma2(d[2], f2(-5.f), fma2(d[0], f2(4.f), d[4]));
        o[1] = fma2(add2(d[1], d[2]), f2(-4.f), add2(d[3], d[4]));
        o[2] = fma2(sub2(d[1], d[2]), f2(4.f), sub2(d[4], d[3]));
        o[3] = fma2(t, f2(2.f), u);
        o[4] = fma2(t, f2(-2.f), u);
        o[5] = fma2(d[3], f2(-5.f), fma2(d[1], f2(4.f), d[5]));
    }
};

template <class T> __device__ __forceinline__ uint32_t pack2v(float2 v) { return pack2<T>(v.x, v.y); }

// Item geometry.  Work item `local` = bx * gy + by: the channel blocks of one
// (image, tile-row block) are adjacent, so the CTAs in flight stage rows of a
// few images at a time.
struct InItem {
    long long n;
    int c0, th0, ntb, ylo, yhi, rows, nch;
};

// Work item `local` of a problem: (image, tile-row block) = local / gy and
// channel block = local % gy, by multiply-shift division (a problem has
// fewer than 2^31 items: N x tile-row blocks x channel blocks).
__device__ __forceinline__ InItem in_item(const InDesc& d, long long local, int M, int A) {
    InItem it;
    const uint32_t lu = static_cast<uint32_t>(local);
    const uint32_t bx = fast_div(d.fd_gy, lu);
    const int by = static_cast<int>(lu - bx * static_cast<uint32_t>(d.gy));
    const uint32_t n = fast_div(d.fd_nbh, bx);
    const int bh = static_cast<int>(bx - n * static_cast<uint32_t>(d.nbh));
    it.n = n;
    it.c0 = by * d.cb;
    it.th0 = bh * d.tb;
    it.ntb = min(d.tb, d.tiles_h - it.th0);
    it.ylo = max(0, it.th0 * M - d.pad_h);
    it.yhi = min(d.H, (it.th0 + it.ntb - 1) * M - d.pad_h + A);
    it.rows = max(0, it.yhi - it.ylo);
    it.nch = min(d.cb, d.C - it.c0);
    return it;
}

// Problem of a work item (descriptors sorted by blk_begin).
__device__ __forceinline__ const InDesc& in_desc_of(const InDesc* descs, int ndesc, long long item) {
    int lo = 0, hi = ndesc - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (descs[mid].blk_begin <= item) lo = mid; else hi = mid - 1;
    }
    return descs[lo];
}

// The producer warp: lane c stages channel c of the item (rows [ylo, yhi), whole width)
// at byte c*stride + (src & 15) of buf and arrives on bar with its byte count.
// Bulk copies stop at the last 16-byte boundary of the input tensor; the few
// elements after it are copied with plain loads before the arrival (whose
// release orders them before the consumers' reads).
template <int M, int A>
__device__ __forceinline__ void in_issue(const InDesc& d, long long local, unsigned char* buf, uint64_t* bar) {
    const int lane = threadIdx.x & 31;
    const InItem it = in_item(d, local, M, A);
    uint32_t bytes = 0;
    uintptr_t a16 = 0;
    unsigned char* dst = buf + static_cast<size_t>(lane) * d.stride_bytes;
    if (lane < it.nch && it.rows > 0) {
        const long long plane = static_cast<long long>(d.H) * d.W;
        const uintptr_t a =
            reinterpret_cast<uintptr_t>(d.x + (it.n * d.C + it.c0 + lane) * plane + static_cast<long long>(it.ylo) * d.W);
        const uintptr_t b = a + static_cast<uintptr_t>(it.rows) * d.W * 2;
        const uintptr_t lim = reinterpret_cast<uintptr_t>(d.x_end) & ~uintptr_t(15);
        a16 = a & ~uintptr_t(15);
        const uintptr_t b16 = min_uptr((b + 15) & ~uintptr_t(15), lim);
        if (b16 > a16) bytes = static_cast<uint32_t>(b16 - a16);
        for (uintptr_t q = (b16 > a16 ? b16 : a16); q < b; q += 2)
            *reinterpret_cast<uint16_t*>(dst + (q - a16)) = *reinterpret_cast<const uint16_t*>(q);
    }
    if (bytes) fence_proxy_async_smem();  // earlier generic reads of this buffer before the async writes
    mbar_arrive_expect_tx(bar, bytes);
    if (bytes) bulk_g2s(dst, reinterpret_cast<const void*>(a16), bytes, bar);
}

// Compute warp cw (of kInComputeWarps) transforms its share of the item:
// lanes are (tile offset q, channel pair sub) with four pairs per granule
// row; tiles q, q + Q, q + 2Q, ... of the item for every granule.
//
// WORDS (problems with pad 1, W a multiple of M and an 8-byte aligned input;
// InDesc::words): a tile's row of ALPHA elements starts 2 bytes before a
// word boundary, so it is read as ALPHA/2 + 1 aligned words (F(4x3): one
// 32-bit, one 64-bit and one 32-bit load; F(2x3): three 32-bit loads)
// instead of ALPHA 16-bit loads, and a byte permute takes each element's
// half of the two channels' words.  Only the first column of the first tile
// and the last column of the last tile of a row can fall outside the image
// there; they are set to zero after the permute.
template <class TF, class OutT, bool SCALED, bool XB, bool KEEP, bool WORDS>
__device__ __forceinline__ void in_compute(const InDesc& d, long long local, const unsigned char* buf,
                                           const unsigned char* zero, int cw) {
    constexpr int M = TF::M, A = TF::ALPHA;
    constexpr int Q = kInComputeWarps * 8;  // tiles in flight per granule
    const int lane = threadIdx.x & 31;
    const InItem it = in_item(d, local, M, A);
    const int W = d.W, tiles_w = d.tiles_w, rows = it.rows;
    const long long Pp = d.Pp;
    const long long plane2 = static_cast<long long>(d.H) * d.W * 2;
    // byte offset of the first staged element of channel (c0 + c): low 4 bits
    // of its global address (the buffer holds whole 16-byte blocks)
    const uintptr_t first =
        reinterpret_cast<uintptr_t>(d.x + (it.n * d.C + it.c0) * (plane2 / 2) + static_cast<long long>(it.ylo) * W);
    const int ntiles = it.ntb * tiles_w;
    const int G = (min(d.cb, d.CG * 8 - it.c0) + 7) / 8;
    const long long estride = static_cast<long long>(d.CG) * Pp * 8;
    const long long p0 = (it.n * d.tiles_h + it.th0) * tiles_w;  // first tile of the item
    const int sub = lane & 3;
    const int q = cw * 8 + (lane >> 2);
    const int dtr = Q / tiles_w, dtw = Q - dtr * tiles_w;
    OutT* __restrict__ V = static_cast<OutT*>(d.V);
    const uint64_t keep = KEEP ? l2_evict_last() : 0;
    for (int g = 0; g < G; ++g) {
        const int c = g * 8 + sub * 2;  // channel pair (c, c+1) of the block
        const bool ok0 = c < it.nch, ok1 = c + 1 < it.nch;
        const unsigned char* cb0 =
            buf + static_cast<size_t>(c) * d.stride_bytes + ((first + static_cast<uintptr_t>(c) * plane2) & 15);
        const unsigned char* cb1 = buf + static_cast<size_t>(c + 1) * d.stride_bytes +
                                   ((first + static_cast<uintptr_t>(c + 1) * plane2) & 15);
        OutT* vg = V + (static_cast<long long>(it.c0 / 8 + g) * Pp + p0) * 8 + sub * 2;
        int tr = q / tiles_w, tw = q - tr * tiles_w;
        for (int t = q; t < ntiles; t += Q) {
            const int y0 = (it.th0 + tr) * M - d.pad_h - it.ylo, x0 = tw * M - d.pad_w;
            // zero padding without per-element masks: a row outside the
            // staged rows (or a channel past C) reads the zero block, and a
            // column outside the image takes the zero upper half of the
            // zero-extended 16-bit loads through the byte-permute selector
            uint32_t sel[A];
            bool lpad = false, rpad = false;
            if constexpr (WORDS) {
                lpad = tw == 0;
                rpad = tw == tiles_w - 1;
            } else {
#pragma unroll
                for (int j = 0; j < A; ++j) sel[j] = (x0 + j >= 0 && x0 + j < W) ? 0x5410u : 0x3232u;
            }
            float2 s2 = f2(1.f);
            if constexpr (SCALED) s2 = f2(d.scale ? d.scale[p0 + t] : 1.f);  // unscaled problems of a group
            // rows first: r[i][.] = d[i][.] B, then columns: V[.][j] = B^T r[.][j]
            float2 r[A][A];
#pragma unroll
            for (int i = 0; i < A; ++i) {
                const int yr = y0 + i;
                const bool rok = yr >= 0 && yr < rows;
                float2 dv[A];
                if constexpr (WORDS) {
                    // word k of a channel's row covers bytes [4k - 4, 4k) from the
                    // tile's second element; element j is half (j + 1) & 1 of word (j + 1) / 2
                    constexpr int NW = A / 2 + 1;
                    const int ofs = yr * W * 2 + 2 * M * tw;
                    const unsigned char* q0 = rok && ok0 ? cb0 + ofs : zero + 8;
                    const unsigned char* q1 = rok && ok1 ? cb1 + ofs : zero + 8;
                    uint32_t w0[NW], w1[NW];
                    w0[0] = *reinterpret_cast<const uint32_t*>(q0 - 4);
                    w1[0] = *reinterpret_cast<const uint32_t*>(q1 - 4);
                    if constexpr (A == 6) {
                        const uint2 a = *reinterpret_cast<const uint2*>(q0);
                        const uint2 b = *reinterpret_cast<const uint2*>(q1);
                        w0[1] = a.x; w0[2] = a.y;
                        w1[1] = b.x; w1[2] = b.y;
                    } else {
                        w0[1] = *reinterpret_cast<const uint32_t*>(q0);
                        w1[1] = *reinterpret_cast<const uint32_t*>(q1);
                    }
                    w0[NW - 1] = *reinterpret_cast<const uint32_t*>(q0 + 4 * (NW - 2));
                    w1[NW - 1] = *reinterpret_cast<const uint32_t*>(q1 + 4 * (NW - 2));
#pragma unroll
                    for (int j = 0; j < A; ++j) {
                        uint32_t h = __byte_perm(w0[(j + 1) / 2], w1[(j + 1) / 2], ((j + 1) & 1) ? 0x7632u : 0x5410u);
                        if (j == 0 && lpad) h = 0u;
                        if (j == A - 1 && rpad) h = 0u;
                        float2 v = IO<XB>::pair(h);
                        if constexpr (SCALED) v = __fmul2_rn(v, s2);
                        dv[j] = v;
                    }
                } else {
                    const int ofs = yr * W * 2 + 2 * x0;
                    const uint16_t* r0 = reinterpret_cast<const uint16_t*>(rok && ok0 ? cb0 + ofs : zero);
                    const uint16_t* r1 = reinterpret_cast<const uint16_t*>(rok && ok1 ? cb1 + ofs : zero);
#pragma unroll
                    for (int j = 0; j < A; ++j) {
                        const uint32_t h = __byte_perm(r0[j], r1[j], sel[j]);
                        float2 v = IO<XB>::pair(h);
                        if constexpr (SCALED) v = __fmul2_rn(v, s2);
                        dv[j] = v;
                    }
                }
                Bt2<TF>::run(dv, r[i]);
            }
            uint32_t pk[A * A];
#pragma unroll
            for (int j = 0; j < A; ++j) {
                float2 col[A], v[A];
#pragma unroll
                for (int i = 0; i < A; ++i) col[i] = r[i][j];
                Bt2<TF>::run(col, v);
#pragma unroll
                for (int i = 0; i < A; ++i) pk[i * A + j] = pack2v<OutT>(v[i]);
            }
            // element e at dst + e * estride, stored in order with one running pointer
            // V is read once by the GEMM that follows: kept in L2 when it fits
            // (KEEP; plain stores otherwise)
            OutT* dst = vg + static_cast<long long>(t) * 8;
#pragma unroll
            for (int e = 0; e < A * A; ++e) {
                if constexpr (KEEP)
                    st_hint_b32(dst, pk[e], keep);
                else
                    *reinterpret_cast<uint32_t*>(dst) = pk[e];
                dst += estride;
            }
            tw += dtw;
            tr += dtr;
            if (tw >= tiles_w) {
                tw -= tiles_w;
                ++tr;
            }
        }
    }
}

// descs: one problem (kernel parameter) or many (device array sorted by
// blk_begin); items [0, total) are split round robin over the grid.
// Warp kInComputeWarps is the producer: it stages item k into buffer
// k % nbufs once the compute warps have released that buffer (empty barrier,
// one arrival per compute warp) and signals the full barrier; the compute
// warps never wait for one another.
template <class TF, class OutT, bool SCALED, bool XB, bool KEEP>
__device__ __forceinline__ void input_body(const InDesc* descs, int ndesc, long long total, int buf_bytes, int nbufs,
                                           unsigned char* smem_raw, DevErr* err) {
    constexpr int M = TF::M, A = TF::ALPHA;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* empty = full + kInMaxBufs;
    volatile int* abort_flag = reinterpret_cast<volatile int*>(full + 2 * kInMaxBufs);
    unsigned char* zero = smem_raw + 64;  // 32 zero bytes: the ALPHA elements of a padding row
                                          // (16-bit loads from zero, word loads around zero + 8)
    unsigned char* bufs = smem_raw + kInHeader + kInSlack;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int i = 0; i < kInMaxBufs; ++i) {
            mbar_init(&full[i], 32);                // every producer lane arrives
            mbar_init(&empty[i], kInComputeWarps);  // one arrival per compute warp
        }
        *abort_flag = 0;
        *reinterpret_cast<uint4*>(zero) = make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4*>(zero + 16) = make_uint4(0u, 0u, 0u, 0u);
        fence_barrier_init();
    }
    pdl_wait();     // input written, earlier readers of V done
    pdl_trigger();
    __syncthreads();
    if (warp == kInComputeWarps) {
        int k = 0;
        for (long long item = blockIdx.x; item < total; item += gridDim.x, ++k) {
            const int b = k % nbufs;
            if (!mbar_wait(&empty[b], ((k / nbufs) & 1) ^ 1u, abort_flag, err, ERR_SITE_EMPTY)) break;
            const InDesc& d = in_desc_of(descs, ndesc, item);
            in_issue<M, A>(d, item - d.blk_begin, bufs + b * buf_bytes, &full[b]);
        }
    } else {
        int k = 0;
        for (long long item = blockIdx.x; item < total; item += gridDim.x, ++k) {
            const int b = k % nbufs;
            if (!mbar_wait(&full[b], (k / nbufs) & 1, abort_flag, err, ERR_SITE_FULL)) break;
            const InDesc& d = in_desc_of(descs, ndesc, item);
            if (d.words)
                in_compute<TF, OutT, SCALED, XB, KEEP, true>(d, item - d.blk_begin, bufs + b * buf_bytes, zero, warp);
            else
                in_compute<TF, OutT, SCALED, XB, KEEP, false>(d, item - d.blk_begin, bufs + b * buf_bytes, zero, warp);
            __syncwarp();
            if ((threadIdx.x & 31) == 0) mbar_arrive(&empty[b]);
        }
    }
    if (*abort_flag) {
        // let the copies still in flight land before the CTA retires
        const unsigned long long t0 = globaltimer_ns();
        while (globaltimer_ns() - t0 < 2000000ull) {
        }
    }
}

template <class TF, class OutT, bool SCALED, bool XB, bool KEEP>
__global__ void __launch_bounds__(kInThreads, 2)
    input_transform_kernel(const __grid_constant__ InDesc d, long long total, int buf_bytes, int nbufs, DevErr* err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    input_body<TF, OutT, SCALED, XB, KEEP>(&d, 1, total, buf_bytes, nbufs, smem_raw, err);
}

template <class TF, class OutT, bool SCALED>
__global__ void __launch_bounds__(kInThreads, 2) input_transform_grouped(const InDesc* __restrict__ descs, int ndesc,
                                                                       long long total, int buf_bytes, DevErr* err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    input_body<TF, OutT, SCALED, false, false>(descs, ndesc, total, buf_bytes, 2, smem_raw, err);
}

// ---- output transform ----------------------------------------------------------

template <class MT> struct MG;  // 8-byte half granule: 4 fp16 or 2 fp32 channels
template <> struct MG<__half> {
    static constexpr int kPerGranule = 8, kPerHalf = 4;
    __device__ static void load(const __half* p, float* out) {
        const uint2 u = *reinterpret_cast<const uint2*>(p);
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
        out[0] = a.x; out[1] = a.y; out[2] = b.x; out[3] = b.y;
    }
};
template <> struct MG<float> {
    static constexpr int kPerGranule = 4, kPerHalf = 2;
    __device__ static void load(const float* p, float* out) {
        const float2 u = *reinterpret_cast<const float2*>(p);
        out[0] = u.x; out[1] = u.y;
    }
};

// One output row of a tile (M values, `valid` of them inside the image) in
// the caller's element type YT (fp16 or bf16).
template <int M, class YT>
__device__ __forceinline__ void store_row(YT* dst, const float* y, int valid) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst);
    if (M == 2 && valid == 2 && (a & 3) == 0) {
        *reinterpret_cast<uint32_t*>(dst) = pack2<YT>(y[0], y[1]);
    } else if (M == 4 && valid == 4 && (a & 7) == 0) {
        *reinterpret_cast<uint2*>(dst) = make_uint2(pack2<YT>(y[0], y[1]), pack2<YT>(y[2], y[3]));
    } else {
#pragma unroll
        for (int j = 0; j < M; ++j)
            if (j < valid) dst[j] = from_f32<YT>(y[j]);
    }
}

// Persistent CTAs; a work item is (64 tiles, one granule); warp 4 stages the
// item's E granule rows (E runs of up to 1 KB, contiguous in M[e][g][P][.])
// with cp.async.bulk into one half of a double buffer while warps 0-3
// transform the previous item from shared memory: thread = (tile, half
// granule), so two lanes read the two halves of one 16-byte row and a warp
// reads 256 contiguous bytes of shared memory per element, and the NCHW row
// writes of a warp are contiguous across tiles.
constexpr int kOsTiles = 64;
static_assert(kOsTiles == kM24Tiles, "a 24-bit M block is one output-transform work item");
constexpr int kOsThreads = 32 * 5;

template <class TF> constexpr int os_smem_bytes() { return 128 + 2 * TF::ALPHA * TF::ALPHA * kOsTiles * 16; }

// Problem of a work item (descriptors sorted by blk_begin).
__device__ __forceinline__ const OutDesc& out_desc_of(const OutDesc* descs, int ndesc, long long item) {
    int lo = 0, hi = ndesc - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (descs[mid].blk_begin <= item) lo = mid; else hi = mid - 1;
    }
    return descs[lo];
}

// Work item -> (first tile p0, granule g), and tile -> (image, tile row,
// tile column), by multiply-shift division.  The tile count P of a problem is
// below 2^31 (the GEMM descriptor refuses more), and so is its item count
// ceil(P/64) * KG for any M that fits in device memory (2^31 items would be
// P * K >= 2^40, 10^14 bytes of M).
struct OutItem {
    uint32_t p0;
    int g;
};
__device__ __forceinline__ OutItem out_item(const OutDesc& d, long long item) {
    const uint32_t iu = static_cast<uint32_t>(item);
    const uint32_t blk = fast_div(d.fd_kg, iu);
    return OutItem{blk * static_cast<uint32_t>(kOsTiles), static_cast<int>(iu - blk * static_cast<uint32_t>(d.KG))};
}
struct OutTile {
    uint32_t n;
    int th, tw;
};
__device__ __forceinline__ OutTile out_tile(const OutDesc& d, uint32_t p) {
    const uint32_t r = fast_div(d.fd_tw, p);
    const uint32_t n = fast_div(d.fd_th, r);
    return OutTile{n, static_cast<int>(r - n * static_cast<uint32_t>(d.tiles_h)),
                   static_cast<int>(p - r * static_cast<uint32_t>(d.tiles_w))};
}

// descs: one problem (kernel parameter) or many (device array sorted by
// blk_begin, items = ceil(P/64) * KG per problem, granule fastest).
template <class TF, class MT, bool YB>
__device__ __forceinline__ void output_staged_body(const OutDesc* descs, int ndesc, long long total, DevErr* err) {
    using YT = typename IO<YB>::T;
    constexpr int M = TF::M, A = TF::ALPHA, E = A * A;
    constexpr int PG = MG<MT>::kPerGranule, PH = MG<MT>::kPerHalf;
    constexpr int kItemBytes = E * kOsTiles * 16;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* empty = full + 2;
    volatile int* abort_flag = reinterpret_cast<volatile int*>(full + 4);
    unsigned char* bufs = smem_raw + 128;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&full[i], 32);
            mbar_init(&empty[i], 4);
        }
        *abort_flag = 0;
        fence_barrier_init();
    }
    pdl_wait();     // M written, earlier readers of the output done
    pdl_trigger();
    __syncthreads();
    if (warp == 4) {
        int k = 0;
        for (long long gitem = blockIdx.x; gitem < total; gitem += gridDim.x, ++k) {
            const int b = k & 1;
            if (!mbar_wait(&empty[b], ((k >> 1) & 1) ^ 1u, abort_flag, err, ERR_SITE_EMPTY)) break;
            const OutDesc& d = out_desc_of(descs, ndesc, gitem);
            const long long item = gitem - d.blk_begin;
            const long long P = d.P;
            const int KG = d.KG;
            const unsigned char* Mb = static_cast<const unsigned char*>(d.Mw);
            const OutItem oi = out_item(d, item);
            const long long p0 = oi.p0;
            const int g = oi.g;
            const uint32_t bytes = static_cast<uint32_t>(min(static_cast<long long>(kOsTiles), P - p0)) * 16u;
            uint32_t mine = 0;
            for (int e = lane; e < E; e += 32) mine += bytes;
            if (mine) fence_proxy_async_smem();  // earlier reads of this buffer before the async writes
            mbar_arrive_expect_tx(&full[b], mine);
            const uint64_t drop = l2_evict_first();   // M is read once
            for (int e = lane; e < E; e += 32)
                bulk_g2s_hint(bufs + b * kItemBytes + e * (kOsTiles * 16),
                              Mb + ((static_cast<long long>(e) * KG + g) * P + p0) * 16, bytes, &full[b], drop);
        }
    } else {
        const int t = threadIdx.x >> 1, hh = threadIdx.x & 1;
        int k = 0;
        for (long long gitem = blockIdx.x; gitem < total; gitem += gridDim.x, ++k) {
            const int b = k & 1;
            if (!mbar_wait(&full[b], (k >> 1) & 1, abort_flag, err, ERR_SITE_FULL)) break;
            const OutDesc& d = out_desc_of(descs, ndesc, gitem);
            const long long item = gitem - d.blk_begin;
            const long long P = d.P;
            const int KG = d.KG;
            const int K = d.K, OH = d.OH, OW = d.OW, tiles_h = d.tiles_h, tiles_w = d.tiles_w;
            YT* __restrict__ out = reinterpret_cast<YT*>(d.out);
            const OutItem oi = out_item(d, item);
            const long long p = static_cast<long long>(oi.p0) + t;
            const int g = oi.g;
            if (p < P) {
                const OutTile ot = out_tile(d, static_cast<uint32_t>(p));
                const int tw = ot.tw, th = ot.th;
                const long long n = ot.n;
                const int oh0 = th * M, ow0 = tw * M;
                const int vr = min(M, OH - oh0), vc = min(M, OW - ow0);
                const unsigned char* src = bufs + b * kItemBytes + t * 16 + hh * 8;
                float m[E][PH];
#pragma unroll
                for (int e = 0; e < E; ++e) MG<MT>::load(reinterpret_cast<const MT*>(src + e * (kOsTiles * 16)), m[e]);
#pragma unroll
                for (int ch = 0; ch < PH; ++ch) {
                    const int kc = g * PG + hh * PH + ch;
                    if (kc >= K) break;
                    float mm[E], y[M * M];
#pragma unroll
                    for (int e = 0; e < E; ++e) mm[e] = m[e][ch];
                    output_tile_transform<TF>(mm, y);
                    if (d.scale) {
                        const float inv = 1.f / d.scale[p];  // exact: scale is a power of two
#pragma unroll
                        for (int i = 0; i < M * M; ++i) y[i] *= inv;
                    }
                    YT* o = out + ((n * K + kc) * OH + oh0) * static_cast<long long>(OW) + ow0;
#pragma unroll
                    for (int i = 0; i < M; ++i)
                        if (i < vr) store_row<M>(o + static_cast<long long>(i) * OW, &y[i * M], vc);
                }
            }
            if (d.discard_m) {
                // the item's M runs are in shared memory and nothing reads
                // them again: drop the 128-byte lines that lie wholly inside
                // them (a line shared with the next granule's rows stays)
                const long long p0 = oi.p0;
                const long long nbytes = min(static_cast<long long>(kOsTiles), P - p0) * 16;
                const unsigned char* Mb = static_cast<const unsigned char*>(d.Mw);
                for (int i = threadIdx.x; i < E * 8; i += 128) {
                    const int e = i >> 3, l = i & 7;
                    const long long s0 = ((static_cast<long long>(e) * KG + g) * P + p0) * 16;
                    const long long first = (s0 + 127) & ~127LL, end = (s0 + nbytes) & ~127LL;
                    if (first + (l + 1) * 128LL <= end) discard_l2_line(Mb + first + l * 128LL);
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[b]);
        }
    }
    if (*abort_flag) {
        const unsigned long long t0 = globaltimer_ns();
        while (globaltimer_ns() - t0 < 2000000ull) {
        }
    }
}

template <class TF, class MT, bool YB>
__global__ void __launch_bounds__(kOsThreads, 3)
    output_transform_staged(const __grid_constant__ OutDesc d, long long total, DevErr* err) {
    output_staged_body<TF, MT, YB>(&d, 1, total, err);
}

// A^T m A on a channel pair in packed fp32x2 (one instruction for both
// channels): the F(4x3) output transforms of both point sets, same matrices
// as TF::at.
template <class TF> struct At2;
template <> struct At2<F4> {   // points 0, +-1, 1/2, -2
    __device__ __forceinline__ static void run(const float2* m, int sm, float2* o, int so) {
        const float2 m0 = m[0], m1 = m[sm], m2 = m[2 * sm], m3 = m[3 * sm], m4 = m[4 * sm], m5 = m[5 * sm];
        const float2 a = __fadd2_rn(m1, m2), b = sub2(m1, m2);
        o[0] = __fadd2_rn(__fadd2_rn(m0, a), __fadd2_rn(m3, m4));
        o[so] = fma2(m4, f2(-2.f), fma2(m3, f2(0.5f), b));
        o[2 * so] = fma2(m4, f2(4.f), fma2(m3, f2(0.25f), a));
        o[3 * so] = __fadd2_rn(fma2(m4, f2(-8.f), fma2(m3, f2(0.125f), b)), m5);
    }
};
template <> struct At2<F4Ref> {   // points 0, +-1, +-2
    __device__ __forceinline__ static void run(const float2* m, int sm, float2* o, int so) {
        const float2 m0 = m[0], m1 = m[sm], m2 = m[2 * sm], m3 = m[3 * sm], m4 = m[4 * sm], m5 = m[5 * sm];
        const float2 a = __fadd2_rn(m1, m2), b = sub2(m1, m2), c = __fadd2_rn(m3, m4), d = sub2(m3, m4);
        o[0] = __fadd2_rn(__fadd2_rn(m0, a), c);
        o[so] = fma2(d, f2(2.f), b);
        o[2 * so] = fma2(c, f2(4.f), a);
        o[3 * so] = __fadd2_rn(fma2(d, f2(8.f), b), m5);
    }
};

template <class TF>
__device__ __forceinline__ void output_tile_transform2(const float2 (&m)[TF::ALPHA * TF::ALPHA],
                                                       float2 (&y)[TF::M * TF::M]) {
    constexpr int A = TF::ALPHA, M = TF::M;
    float2 t[M * A];
#pragma unroll
    for (int j = 0; j < A; ++j) At2<TF>::run(&m[j], A, &t[j], A);      // A^T m
#pragma unroll
    for (int i = 0; i < M; ++i) At2<TF>::run(&t[i * A], 1, &y[i * M], 1);  // (A^T m) A
}

// 24-bit M (high plane H[NB][KG][E][64][8] of 16-bit words, low plane
// L[NB][KG][E][64][8] of bytes, NB blocks of 64 tiles): a work item is one
// block of 64 tiles x one granule of 8 channels, whose E high runs (1 KB
// each) and E low runs (512 B each) are contiguous: warp 8 stages them with
// two bulk copies into one half of a double buffer while warps 0-7 transform
// the previous item (2E copies of the single runs took 36.9 against 28.7 us
// on N32 C256 56x56 K256): thread = (tile, channel pair), so a warp reads 128
// contiguous bytes of the high run and 64 of the low run per element and
// rebuilds each value as high << 16 | low << 8.
constexpr int kOs24Threads = 32 * 9;
template <class TF> __host__ __device__ constexpr int os24_item_bytes() { return TF::ALPHA * TF::ALPHA * kOsTiles * (16 + 8); }
template <class TF> __host__ __device__ constexpr int os24_smem_bytes() { return 128 + 2 * os24_item_bytes<TF>(); }

// YNHWC: the output is channels-last, y[N][OH][OW][K] (fp16, unscaled): a
// thread writes its channel pair at each of the tile's pixels.
template <class TF, bool YB, bool YNHWC = false>
__device__ __forceinline__ void output_staged_body_m24(const OutDesc* descs, int ndesc, long long total, DevErr* err) {
    using YT = typename IO<YB>::T;
    constexpr int M = TF::M, A = TF::ALPHA, E = A * A;
    constexpr int kItemBytes = os24_item_bytes<TF>();
    constexpr int kLoBase = E * kOsTiles * 16;   // low runs after the E high runs
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* empty = full + 2;
    volatile int* abort_flag = reinterpret_cast<volatile int*>(full + 4);
    unsigned char* bufs = smem_raw + 128;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&full[i], 32);
            mbar_init(&empty[i], 8);
        }
        *abort_flag = 0;
        fence_barrier_init();
    }
    pdl_wait();     // M written, earlier readers of the output done
    __syncthreads();
    if (warp == 8) {
        int k = 0;
        for (long long gitem = blockIdx.x; gitem < total; gitem += gridDim.x, ++k) {
            const int b = k & 1;
            const uint32_t ph = (k >> 1) & 1;
            if (!mbar_wait(&empty[b], ph ^ 1u, abort_flag, err, ERR_SITE_EMPTY)) break;
            const OutDesc& d = out_desc_of(descs, ndesc, gitem);
            const long long item = gitem - d.blk_begin;
            const long long P = d.P;
            const int KG = d.KG;
            const unsigned char* Mb = static_cast<const unsigned char*>(d.Mw);
            const OutItem oi = out_item(d, item);
            const long long p0 = oi.p0;
            const int g = oi.g;
            // the item's E runs are one contiguous range in each plane (the
            // last block's rows past P are padding, copied and not read)
            const long long run = (p0 / kOsTiles * KG + g) * E;
            const uint32_t mine = lane == 0 ? E * kOsTiles * 16u : lane == 1 ? E * kOsTiles * 8u : 0u;
            if (mine) fence_proxy_async_smem();  // earlier reads of this buffer before the async writes
            mbar_arrive_expect_tx(&full[b], mine);
            const uint64_t drop = l2_evict_first();   // M is read once
            if (lane == 0)
                bulk_g2s_hint(bufs + b * kItemBytes, Mb + run * (kOsTiles * 16), mine, &full[b], drop);
            else if (lane == 1)
                bulk_g2s_hint(bufs + b * kItemBytes + kLoBase, Mb + d.m_lo + run * (kOsTiles * 8), mine, &full[b], drop);
        }
    } else {
        const int t = threadIdx.x >> 2, qd = threadIdx.x & 3;
        int k = 0;
        for (long long gitem = blockIdx.x; gitem < total; gitem += gridDim.x, ++k) {
            const int b = k & 1;
            const uint32_t ph = (k >> 1) & 1;
            if (!mbar_wait(&full[b], ph, abort_flag, err, ERR_SITE_FULL)) break;
            const OutDesc& d = out_desc_of(descs, ndesc, gitem);
            const long long item = gitem - d.blk_begin;
            const long long P = d.P;
            const int KG = d.KG;
            const int K = d.K, OH = d.OH, OW = d.OW, tiles_h = d.tiles_h, tiles_w = d.tiles_w;
            YT* __restrict__ out = reinterpret_cast<YT*>(d.out);
            const OutItem oi = out_item(d, item);
            const long long p = static_cast<long long>(oi.p0) + t;
            const int g = oi.g;
            if (p < P) {
                const OutTile ot = out_tile(d, static_cast<uint32_t>(p));
                const int tw = ot.tw, th = ot.th;
                const long long n = ot.n;
                const int oh0 = th * M, ow0 = tw * M;
                const int vr = min(M, OH - oh0), vc = min(M, OW - ow0);
                const unsigned char* hsrc = bufs + b * kItemBytes + t * 16 + qd * 4;
                const unsigned char* lsrc = bufs + b * kItemBytes + kLoBase + t * 8 + qd * 2;
                // value bits = high 16 | low 8 << 8: one byte permute per
                // value, the zero byte taken from the zero-extended 16-bit
                // load of the low pair
                float2 m[E];
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const uint32_t h = *reinterpret_cast<const uint32_t*>(hsrc + e * (kOsTiles * 16));
                    const uint32_t l = *reinterpret_cast<const uint16_t*>(lsrc + e * (kOsTiles * 8));
                    m[e] = make_float2(__uint_as_float(__byte_perm(l, h, 0x5403)),
                                       __uint_as_float(__byte_perm(l, h, 0x7613)));
                }
                float2 y2[M * M];
                output_tile_transform2<TF>(m, y2);
                if constexpr (YNHWC) {
                    // channels kc, kc + 1 of each pixel: one 4-byte store where
                    // both exist and the pair is 4-byte aligned (K even)
                    const int kc = g * 8 + qd * 2;
                    if (kc < K) {
                        YT* o = out + ((n * OH + oh0) * static_cast<long long>(OW) + ow0) * K + kc;
                        const bool pair = kc + 1 < K, even = (K & 1) == 0;
#pragma unroll
                        for (int i = 0; i < M; ++i) {
                            if (i >= vr) break;
#pragma unroll
                            for (int j = 0; j < M; ++j) {
                                if (j >= vc) break;
                                YT* q = o + (static_cast<long long>(i) * OW + j) * K;
                                const float2 v = y2[i * M + j];
                                if (pair && even) {
                                    *reinterpret_cast<uint32_t*>(q) = pack2<YT>(v.x, v.y);
                                } else {
                                    q[0] = from_f32<YT>(v.x);
                                    if (pair) q[1] = from_f32<YT>(v.y);
                                }
                            }
                        }
                    }
                } else {
                    if (d.scale) {
                        const float inv = 1.f / d.scale[p];  // exact: scale is a power of two
#pragma unroll
                        for (int i = 0; i < M * M; ++i) y2[i] = __fmul2_rn(y2[i], f2(inv));
                    }
                    // a whole tile of a whole granule with 8-byte aligned rows
                    // (OW a multiple of 4, y 8-byte aligned): M row stores per
                    // channel without per-row checks
                    const bool whole = M == 4 && vr == M && vc == M && g * 8 + 8 <= K && (OW & 3) == 0 &&
                                       (reinterpret_cast<uintptr_t>(out) & 7) == 0;
                    if (whole) {
#pragma unroll
                        for (int ch = 0; ch < 2; ++ch) {
                            YT* o = out + ((n * K + g * 8 + qd * 2 + ch) * OH + oh0) * static_cast<long long>(OW) + ow0;
#pragma unroll
                            for (int i = 0; i < M; ++i) {
                                const float2* r = &y2[i * M];
                                *reinterpret_cast<uint2*>(o + static_cast<long long>(i) * OW) =
                                    ch == 0 ? make_uint2(pack2<YT>(r[0].x, r[1].x), pack2<YT>(r[2].x, r[3].x))
                                            : make_uint2(pack2<YT>(r[0].y, r[1].y), pack2<YT>(r[2].y, r[3].y));
                            }
                        }
                    } else {
#pragma unroll
                        for (int ch = 0; ch < 2; ++ch) {
                            const int kc = g * 8 + qd * 2 + ch;
                            if (kc >= K) break;
                            float y[M * M];
#pragma unroll
                            for (int i = 0; i < M * M; ++i) y[i] = ch == 0 ? y2[i].x : y2[i].y;
                            YT* o = out + ((n * K + kc) * OH + oh0) * static_cast<long long>(OW) + ow0;
#pragma unroll
                            for (int i = 0; i < M; ++i)
                                if (i < vr) store_row<M>(o + static_cast<long long>(i) * OW, &y[i * M], vc);
                        }
                    }
                }
            }
            if (d.discard_m) {
                // the item's ranges (E KB of the high plane, E/2 KB of the low
                // one, 128-byte aligned) are in shared memory and nothing reads
                // them again: drop their L2 lines
                const long long run = (static_cast<long long>(oi.p0) / kOsTiles * KG + g) * E;
                const unsigned char* hb = static_cast<const unsigned char*>(d.Mw) + run * (kOsTiles * 16);
                const unsigned char* lb = static_cast<const unsigned char*>(d.Mw) + d.m_lo + run * (kOsTiles * 8);
                for (int i = threadIdx.x; i < E * 12; i += 256)
                    discard_l2_line(i < E * 8 ? hb + i * 128 : lb + (i - E * 8) * 128);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[b]);
        }
    }
    // the next kernel is released when this CTA's items are done: released at
    // the start instead, back-to-back channels-last calls measured 1.6 us
    // slower per call and NCHW calls no faster
    pdl_trigger();
    if (*abort_flag) {
        const unsigned long long t0 = globaltimer_ns();
        while (globaltimer_ns() - t0 < 2000000ull) {
        }
    }
}

template <class TF, bool YB, bool YNHWC = false>
__global__ void __launch_bounds__(kOs24Threads, 2)
    output_transform_staged_m24(const __grid_constant__ OutDesc d, long long total, DevErr* err) {
    output_staged_body_m24<TF, YB, YNHWC>(&d, 1, total, err);
}

template <class TF>
__global__ void __launch_bounds__(kOs24Threads, 2)
    output_transform_staged_m24_grouped(const OutDesc* __restrict__ descs, int ndesc, long long total, DevErr* err) {
    output_staged_body_m24<TF, false>(descs, ndesc, total, err);
}

template <class TF, class MT>
__global__ void __launch_bounds__(kOsThreads, 3)
    output_transform_staged_grouped(const OutDesc* __restrict__ descs, int ndesc, long long total, DevErr* err) {
    output_staged_body<TF, MT, false>(descs, ndesc, total, err);
}


struct InBlocking {
    int tb, nbh, cb, stride, buf;
};

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
    if (!cached[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
        cached[dev] = n;
    }
    return cached[dev];
}

constexpr int kInBufBudget = 56 * 1024;   // per buffer: two CTAs of two buffers per SM
constexpr int kSmemPerSm = 233472;        // shared memory of one SM (228 KB)

int in_smem_total(int buf) { return kInHeader + 2 * kInSlack + 2 * buf; }   // two buffers
int in_ctas_per_sm(int smem) { return std::max(1, std::min(2, kSmemPerSm / (smem + 1024))); }

// Tile-row block tb and channel block cb: the items (image, tile-row block,
// channel block) are spread over the persistent grid; the choice minimises
// rounds of items per CTA x rounds of tiles per compute lane x staged rows
// per output row (halo re-reads).
InBlocking choose_in_blocking(const Geom& g) {
    const int M = g.m, A = g.alpha;
    // a channel's staged rows take whole 16-byte blocks, padded so that
    // channels two apart start 8 or 24 banks apart: the four channel pairs
    // that a warp reads at once then fall in different banks
    auto stride_for = [&](int tb) {
        const int rows = std::min(g.h, tb * M + A - M);
        int st = (rows * g.w * 2 + 16 + 15) / 16 * 16;
        while ((st / 4) % 16 != 4 && (st / 4) % 16 != 12) st += 16;
        return st;
    };
    InBlocking best{1, g.tiles_h, 8, stride_for(1), 8 * stride_for(1)};
    double best_cost = 1e300;
    const long long slots = static_cast<long long>(sm_count()) * 2;
    for (int cb = 32; cb >= 8; cb /= 2) {
        if (cb > 8 && cb * stride_for(1) > kInBufBudget) continue;
        if (cb > 8 && cb >= 2 * ((g.c + 7) / 8 * 8)) continue;  // no block twice the channel count
        for (int tb = 1; tb <= g.tiles_h; ++tb) {
            const int st = stride_for(tb);
            if ((tb > 1 && cb * st > kInBufBudget) || tb * g.tiles_w > 1024) break;
            const int nbh = (g.tiles_h + tb - 1) / tb;
            const long long items = static_cast<long long>(g.n) * nbh * ((g.c + cb - 1) / cb);
            // per compute lane: granules x rounds of kInComputeWarps*8 tiles
            const long long lane_rounds = static_cast<long long>(cb / 8) *
                                          ((static_cast<long long>(tb) * g.tiles_w + kInComputeWarps * 8 - 1) /
                                           (kInComputeWarps * 8));
            const double rounds = static_cast<double>((items + slots - 1) / slots);
            const double cost = rounds * static_cast<double>(lane_rounds) * (static_cast<double>(tb * M + A - M) / (tb * M));
            if (cost < best_cost * 0.999) {
                best_cost = cost;
                best = InBlocking{tb, nbh, cb, st, (cb * st + 15) / 16 * 16};
            }
        }
    }
    return best;
}

template <class TF, class OutT, bool SCALED, bool XB = false, bool KEEP = false>
cudaError_t input_launch(const InDesc& d, int smem, DevErr* err, cudaStream_t s) {
    auto kern = input_transform_kernel<TF, OutT, SCALED, XB, KEEP>;
    // a third staging buffer where two CTAs of three still fit an SM: the
    // next item's copies then start two items ahead of the arithmetic
    const int buf = (smem - kInHeader - 2 * kInSlack) / 2;
    const int smem3 = kInHeader + 2 * kInSlack + 3 * buf;
    const int nbufs = in_ctas_per_sm(smem3) >= 2 ? 3 : 2;
    if (nbufs == 3) smem = smem3;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const long long total = d.gx * d.gy;
    const long long grid = std::min<long long>(total, static_cast<long long>(sm_count()) * in_ctas_per_sm(smem));
    return launch_pdl(kern, dim3(static_cast<unsigned>(grid)), dim3(kInThreads), smem, s, d, total, buf, nbufs, err);
}

template <class TF, class OutT, bool SCALED>
cudaError_t input_grouped_launch(const InDesc* descs, int ndesc, long long total, int smem, DevErr* err,
                                 cudaStream_t s) {
    auto kern = input_transform_grouped<TF, OutT, SCALED>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const long long grid = std::min<long long>(total, static_cast<long long>(sm_count()) * in_ctas_per_sm(smem));
    return launch_pdl(kern, dim3(static_cast<unsigned>(grid)), dim3(kInThreads), smem, s, descs, ndesc, total,
                      (smem - kInHeader - 2 * kInSlack) / 2, err);
}

template <class TF, class MT, bool YB = false>
cudaError_t output_launch(const OutDesc& d, DevErr* err, cudaStream_t s) {
    const long long total = (d.P + kOsTiles - 1) / kOsTiles * d.KG;
    if (total <= 0) return cudaSuccess;
    auto kern = output_transform_staged<TF, MT, YB>;
    constexpr int smem = os_smem_bytes<TF>();
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const int per_sm = std::max(1, std::min(4, 233472 / (smem + 1024)));
    const long long grid = std::min<long long>(total, static_cast<long long>(sm_count()) * per_sm);
    return launch_pdl(kern, dim3(static_cast<unsigned>(grid)), dim3(kOsThreads), smem, s, d, total, err);
}

template <class TF, bool YB = false, bool YNHWC = false>
cudaError_t output_launch_m24(const OutDesc& d, DevErr* err, cudaStream_t s) {
    const long long total = (d.P + kOsTiles - 1) / kOsTiles * d.KG;
    if (total <= 0) return cudaSuccess;
    auto kern = output_transform_staged_m24<TF, YB, YNHWC>;
    constexpr int smem = os24_smem_bytes<TF>();
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const int per_sm = std::max(1, std::min(2, 233472 / (smem + 1024)));
    const long long grid = std::min<long long>(total, static_cast<long long>(sm_count()) * per_sm);
    return launch_pdl(kern, dim3(static_cast<unsigned>(grid)), dim3(kOs24Threads), smem, s, d, total, err);
}

template <class TF>
cudaError_t output_grouped_launch_m24(const OutDesc* descs, int ndesc, long long blocks, DevErr* err, cudaStream_t s) {
    if (blocks <= 0) return cudaSuccess;
    auto kern = output_transform_staged_m24_grouped<TF>;
    constexpr int smem = os24_smem_bytes<TF>();
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const int per_sm = std::max(1, std::min(2, 233472 / (smem + 1024)));
    const long long grid = std::min<long long>(blocks, static_cast<long long>(sm_count()) * per_sm);
    return launch_pdl(kern, dim3(static_cast<unsigned>(grid)), dim3(kOs24Threads), smem, s, descs, ndesc, blocks, err);
}

template <class TF, class MT>
cudaError_t output_grouped_launch(const OutDesc* descs, int ndesc, long long blocks, DevErr* err, cudaStream_t s) {
    if (blocks <= 0) return cudaSuccess;
    auto kern = output_transform_staged_grouped<TF, MT>;
    constexpr int smem = os_smem_bytes<TF>();
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const int per_sm = std::max(1, std::min(4, 233472 / (smem + 1024)));
    const long long grid = std::min<long long>(blocks, static_cast<long long>(sm_count()) * per_sm);
    return launch_pdl(kern, dim3(static_cast<unsigned>(grid)), dim3(kOsThreads), smem, s, descs, ndesc, blocks, err);
}

template <class TF, class OutT>
cudaError_t filter_launch(const void* w, void* U, int K, int C, int Cp, cudaStream_t s, bool wb) {
    const int Kp = (K + 7) / 8 * 8;
    const long long total = static_cast<long long>(Kp) * Cp;
    const unsigned blocks = static_cast<unsigned>((total + 255) / 256);
    if (wb)
        filter_transform_kernel<TF, OutT, true><<<blocks, 256, 0, s>>>(static_cast<const __nv_bfloat16*>(w),
                                                                      static_cast<OutT*>(U), K, C, Cp, Kp);
    else
        filter_transform_kernel<TF, OutT, false><<<blocks, 256, 0, s>>>(static_cast<const __half*>(w),
                                                                       static_cast<OutT*>(U), K, C, Cp, Kp);
    return cudaGetLastError();
}

}  // namespace

long long l2_cache_bytes() {
    static long long cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    if (!cached[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrL2CacheSize, dev);
        cached[dev] = v > 0 ? v : 1;
    }
    return cached[dev];
}

cudaError_t launch_filter_transform(Xform xf, OpType op, const void* weight, void* U, int K, int C, int Cp,
                                    cudaStream_t stream, bool w_bf16) {
    const bool bf = op == OpType::BF16;
    switch (xf) {
        case Xform::F2:
            return bf ? filter_launch<F2, __nv_bfloat16>(weight, U, K, C, Cp, stream, w_bf16)
                      : filter_launch<F2, __half>(weight, U, K, C, Cp, stream, w_bf16);
        case Xform::F4:
            return bf ? filter_launch<F4, __nv_bfloat16>(weight, U, K, C, Cp, stream, w_bf16)
                      : filter_launch<F4, __half>(weight, U, K, C, Cp, stream, w_bf16);
        case Xform::F4Ref:
            return bf ? filter_launch<F4Ref, __nv_bfloat16>(weight, U, K, C, Cp, stream, w_bf16)
                      : filter_launch<F4Ref, __half>(weight, U, K, C, Cp, stream, w_bf16);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_tile_scale(const Geom& g, const void* x, float* scale, cudaStream_t stream, bool x_bf16) {
    const unsigned blocks = static_cast<unsigned>((g.P + 7) / 8);
    if (x_bf16) {
        const __nv_bfloat16* xb = static_cast<const __nv_bfloat16*>(x);
        if (g.m == 2)
            return launch_pdl(tile_scale_kernel<2, true>, dim3(blocks), dim3(256), 0, stream, xb, scale, g.c, g.h, g.w,
                              g.pad_h, g.pad_w, g.tiles_h, g.tiles_w, g.P);
        return launch_pdl(tile_scale_kernel<4, true>, dim3(blocks), dim3(256), 0, stream, xb, scale, g.c, g.h, g.w,
                          g.pad_h, g.pad_w, g.tiles_h, g.tiles_w, g.P);
    }
    const __half* xh = static_cast<const __half*>(x);
    if (g.m == 2)
        return launch_pdl(tile_scale_kernel<2, false>, dim3(blocks), dim3(256), 0, stream, xh, scale, g.c, g.h, g.w,
                          g.pad_h, g.pad_w, g.tiles_h, g.tiles_w, g.P);
    return launch_pdl(tile_scale_kernel<4, false>, dim3(blocks), dim3(256), 0, stream, xh, scale, g.c, g.h, g.w,
                      g.pad_h, g.pad_w, g.tiles_h, g.tiles_w, g.P);
}

InDesc make_in_desc(const Geom& g, const void* x, const void* x_end, void* V, const float* scale, int* smem) {
    const InBlocking b = choose_in_blocking(g);
    InDesc d{};
    d.x = static_cast<const __half*>(x);
    d.x_end = static_cast<const __half*>(x_end);
    d.V = V;
    d.scale = scale;
    d.C = g.c; d.H = g.h; d.W = g.w; d.pad_h = g.pad_h; d.pad_w = g.pad_w;
    d.tiles_h = g.tiles_h; d.tiles_w = g.tiles_w;
    d.Pp = round_rows(g.P);
    d.CG = g.cp / 8;
    d.tb = b.tb; d.nbh = b.nbh; d.cb = b.cb; d.stride_bytes = b.stride;
    d.gx = static_cast<long long>(g.n) * b.nbh;
    d.gy = (g.c + b.cb - 1) / b.cb;
    d.fd_gy = make_fastdiv(static_cast<uint32_t>(d.gy));
    d.fd_nbh = make_fastdiv(static_cast<uint32_t>(b.nbh));
    d.blk_begin = 0;
    d.words = (g.m == 2 || g.m == 4) && g.pad_w == 1 && g.w % g.m == 0 && (reinterpret_cast<uintptr_t>(x) & 7) == 0;
    *smem = in_smem_total(b.buf);
    return d;
}

OutDesc make_out_desc(const Geom& g, MType mt, const void* Mw, void* out, const float* scale) {
    OutDesc d{};
    d.Mw = Mw;
    d.out = static_cast<__half*>(out);
    d.scale = scale;
    d.K = g.k; d.OH = g.oh; d.OW = g.ow; d.tiles_h = g.tiles_h; d.tiles_w = g.tiles_w;
    d.P = g.P;
    d.KG = mt == MType::F32 ? g.kp / 4 : g.kp / 8;
    d.m_lo = m24_lo_offset(static_cast<long long>(g.alpha) * g.alpha, g.P, g.kp);
    d.gx = (g.P + kOsTiles - 1) / kOsTiles;
    d.gy = d.KG;
    d.blk_begin = 0;
    d.fd_kg = make_fastdiv(static_cast<uint32_t>(d.KG));
    d.fd_tw = make_fastdiv(static_cast<uint32_t>(g.tiles_w));
    d.fd_th = make_fastdiv(static_cast<uint32_t>(g.tiles_h));
    // M larger than L2 streams through it: its lines are dropped as soon as
    // they are read (32 x 256 x 56^2 -> 256 F(4x3), 231 MB of fp32 M: output
    // transform 48.4 -> 42.1 us on one box); M that fits stays in L2 for this
    // kernel, where discarding only costs time (32 x 512 x 28^2 -> 512, 116 MB:
    // 22.5 -> 23.8 us).  WG_CONV2D_KEEP_WORKSPACE=1 keeps M readable after the
    // call.
    const char* keep_ws = std::getenv("WG_CONV2D_KEEP_WORKSPACE");
    d.discard_m = !(keep_ws && std::atoi(keep_ws) != 0) && (reinterpret_cast<uintptr_t>(Mw) & 127) == 0 &&
                  m_bytes(mt, static_cast<long long>(g.alpha) * g.alpha, g.P, g.kp) > l2_cache_bytes();
    return d;
}

cudaError_t launch_input_transform(Xform xf, OpType op, const Geom& g, const void* x, const void* x_end, void* V,
                                   const float* scale, DevErr* err, cudaStream_t stream, bool x_bf16) {
    int smem = 0;
    const InDesc d = make_in_desc(g, x, x_end, V, scale, &smem);
    // V of this launch within the L2 size: written with the evict_last
    // priority, the GEMM that follows reads most of it from L2 (32 x 256 x
    // 56^2 -> 256 F(4x3), 116 MB of V: 146 -> 140 us per call, same box); a
    // larger V (F(2x3) on the same layer: 205 MB) would only push itself out.
    // fp16 unscaled paths only.
    const long long v_bytes = static_cast<long long>(g.alpha) * g.alpha * d.CG * 8 * d.Pp * 2;
    const bool keep = v_bytes <= l2_cache_bytes();
    const bool bf = op == OpType::BF16, sc = scale != nullptr;
    if (x_bf16) {
        // bf16 tensors: F(2x3) with bf16 operands, F(4x3) with fp16 operands
        // and per-tile scaling (the plan arranges these pairings)
        if (xf == Xform::F2 && bf && !sc) return input_launch<F2, __nv_bfloat16, false, true>(d, smem, err, stream);
        if (xf == Xform::F4 && !bf && sc) return input_launch<F4, __half, true, true>(d, smem, err, stream);
        if (xf == Xform::F4Ref && !bf && sc) return input_launch<F4Ref, __half, true, true>(d, smem, err, stream);
        return cudaErrorNotSupported;
    }
    switch (xf) {
        case Xform::F2:  // never scaled
            if (bf) return input_launch<F2, __nv_bfloat16, false>(d, smem, err, stream);
            return keep ? input_launch<F2, __half, false, false, true>(d, smem, err, stream)
                        : input_launch<F2, __half, false>(d, smem, err, stream);
        case Xform::F4:
            if (sc)
                return bf ? input_launch<F4, __nv_bfloat16, true>(d, smem, err, stream)
                          : input_launch<F4, __half, true>(d, smem, err, stream);
            if (bf) return input_launch<F4, __nv_bfloat16, false>(d, smem, err, stream);
            return keep ? input_launch<F4, __half, false, false, true>(d, smem, err, stream)
                        : input_launch<F4, __half, false>(d, smem, err, stream);
        case Xform::F4Ref:
            if (sc)
                return bf ? input_launch<F4Ref, __nv_bfloat16, true>(d, smem, err, stream)
                          : input_launch<F4Ref, __half, true>(d, smem, err, stream);
            return bf ? input_launch<F4Ref, __nv_bfloat16, false>(d, smem, err, stream)
                      : input_launch<F4Ref, __half, false>(d, smem, err, stream);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_input_transform_grouped(Xform xf, OpType op, const InDesc* descs, int ndesc, long long blocks,
                                           int smem, bool scaled, DevErr* err, cudaStream_t stream) {
    const bool bf = op == OpType::BF16;
    switch (xf) {
        case Xform::F2:
            return bf ? input_grouped_launch<F2, __nv_bfloat16, false>(descs, ndesc, blocks, smem, err, stream)
                      : input_grouped_launch<F2, __half, false>(descs, ndesc, blocks, smem, err, stream);
        case Xform::F4:
            if (scaled)
                return bf ? input_grouped_launch<F4, __nv_bfloat16, true>(descs, ndesc, blocks, smem, err, stream)
                          : input_grouped_launch<F4, __half, true>(descs, ndesc, blocks, smem, err, stream);
            return bf ? input_grouped_launch<F4, __nv_bfloat16, false>(descs, ndesc, blocks, smem, err, stream)
                      : input_grouped_launch<F4, __half, false>(descs, ndesc, blocks, smem, err, stream);
        case Xform::F4Ref:
            if (scaled)
                return bf ? input_grouped_launch<F4Ref, __nv_bfloat16, true>(descs, ndesc, blocks, smem, err, stream)
                          : input_grouped_launch<F4Ref, __half, true>(descs, ndesc, blocks, smem, err, stream);
            return bf ? input_grouped_launch<F4Ref, __nv_bfloat16, false>(descs, ndesc, blocks, smem, err, stream)
                      : input_grouped_launch<F4Ref, __half, false>(descs, ndesc, blocks, smem, err, stream);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_output_transform(Xform xf, MType mt, const Geom& g, const void* Mw, void* out,
                                    const float* scale, DevErr* err, cudaStream_t stream, bool y_bf16) {
    const OutDesc d = make_out_desc(g, mt, Mw, out, scale);
    if (mt == MType::F24) {  // F(4x3) only
        switch (xf) {
            case Xform::F2: return cudaErrorNotSupported;
            case Xform::F4: return y_bf16 ? output_launch_m24<F4, true>(d, err, stream) : output_launch_m24<F4>(d, err, stream);
            case Xform::F4Ref:
                return y_bf16 ? output_launch_m24<F4Ref, true>(d, err, stream) : output_launch_m24<F4Ref>(d, err, stream);
        }
        return cudaErrorInvalidValue;
    }
    const bool m_fp32 = mt == MType::F32;
    if (y_bf16) {  // bf16 tensors: fp32 or 24-bit M
        if (!m_fp32) return cudaErrorNotSupported;
        switch (xf) {
            case Xform::F2: return output_launch<F2, float, true>(d, err, stream);
            case Xform::F4: return output_launch<F4, float, true>(d, err, stream);
            case Xform::F4Ref: return output_launch<F4Ref, float, true>(d, err, stream);
        }
        return cudaErrorInvalidValue;
    }
    switch (xf) {
        case Xform::F2:
            return m_fp32 ? output_launch<F2, float>(d, err, stream) : output_launch<F2, __half>(d, err, stream);
        case Xform::F4:
            return m_fp32 ? output_launch<F4, float>(d, err, stream) : output_launch<F4, __half>(d, err, stream);
        case Xform::F4Ref:
            return m_fp32 ? output_launch<F4Ref, float>(d, err, stream) : output_launch<F4Ref, __half>(d, err, stream);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_output_transform_nhwc24(Xform xf, const Geom& g, const void* Mw, void* out, DevErr* err,
                                          cudaStream_t stream) {
    const OutDesc d = make_out_desc(g, MType::F24, Mw, out, nullptr);
    switch (xf) {
        case Xform::F2: return cudaErrorNotSupported;
        case Xform::F4: return output_launch_m24<F4, false, true>(d, err, stream);
        case Xform::F4Ref: return output_launch_m24<F4Ref, false, true>(d, err, stream);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_output_transform_grouped(Xform xf, MType mt, const OutDesc* descs, int ndesc, long long blocks,
                                            DevErr* err, cudaStream_t stream) {
    if (mt == MType::F24) {
        switch (xf) {
            case Xform::F2: return cudaErrorNotSupported;
            case Xform::F4: return output_grouped_launch_m24<F4>(descs, ndesc, blocks, err, stream);
            case Xform::F4Ref: return output_grouped_launch_m24<F4Ref>(descs, ndesc, blocks, err, stream);
        }
        return cudaErrorInvalidValue;
    }
    const bool m_fp32 = mt == MType::F32;
    switch (xf) {
        case Xform::F2:
            return m_fp32 ? output_grouped_launch<F2, float>(descs, ndesc, blocks, err, stream)
                          : output_grouped_launch<F2, __half>(descs, ndesc, blocks, err, stream);
        case Xform::F4:
            return m_fp32 ? output_grouped_launch<F4, float>(descs, ndesc, blocks, err, stream)
                          : output_grouped_launch<F4, __half>(descs, ndesc, blocks, err, stream);
        case Xform::F4Ref:
            return m_fp32 ? output_grouped_launch<F4Ref, float>(descs, ndesc, blocks, err, stream)
                          : output_grouped_launch<F4Ref, __half>(descs, ndesc, blocks, err, stream);
    }
    return cudaErrorInvalidValue;
}

}  // namespace wg
