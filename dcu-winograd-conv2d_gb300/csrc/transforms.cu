// Winograd filter, input and output transform kernels (HBM-bound).
//
// Layouts in HBM (one convolution, E = alpha^2 Winograd elements):
//   input   x[N][C][H][W]          fp16 (caller's NCHW)
//   filter  w[K][C][3][3]          fp16 (caller's KCRS)
//   U       U[E][K][Cp]            operand type, Cp = C rounded up to 8
//   V       V[E][P][Cp]            operand type, P = tiles in the batch
//   M       M[E][P][Kp]            fp16 (F(2x3)) or fp32 (F(4x3))
//   output  y[N][K][OH][OW]        fp16
// U and V keep the contraction index (C) innermost so both GEMM operands are
// K-major 128-byte rows for TMA and tcgen05.  The reference keeps the tile
// index innermost instead (V[e][C][P], U[e][K][C], M[e][K][P];
// src/winograd_2x3_non_fused.cpp:296-299,371-374, include/hep_sgemm.h:32-34).
//
// The input and output transforms work on a block of tile rows x tile
// columns x 64 channels per CTA: the input patch (with halo) is staged in
// shared memory once with coalesced loads, and one lane owns a channel pair,
// so every HBM write of V or read of M is a contiguous 128-byte row.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "wg_kernels.h"
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

template <class T> __device__ __forceinline__ T from_f32(float v);
template <> __device__ __forceinline__ __half from_f32<__half>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

template <class T> struct Pair;
template <> struct Pair<__half> {
    using type = __half2;
    __device__ static type make(float a, float b) { return __floats2half2_rn(a, b); }
};
template <> struct Pair<__nv_bfloat16> {
    using type = __nv_bfloat162;
    __device__ static type make(float a, float b) { return __floats2bfloat162_rn(a, b); }
};

// ---- filter transform --------------------------------------------------------

template <class TF, class OutT>
__global__ void __launch_bounds__(256) filter_transform_kernel(const __half* __restrict__ w, OutT* __restrict__ U,
                                                               int K, int C, int Cp) {
    constexpr int A = TF::ALPHA;
    const long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<long long>(K) * Cp) return;
    const int k = static_cast<int>(idx / Cp), c = static_cast<int>(idx % Cp);
    float g[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) g[i] = 0.f;
    if (c < C) {
        const __half* src = w + (static_cast<long long>(k) * C + c) * 9;
#pragma unroll
        for (int i = 0; i < 9; ++i) g[i] = __half2float(src[i]);
    }
    float u[A * A];
    filter_tile_transform<TF>(g, u);
#pragma unroll
    for (int e = 0; e < A * A; ++e) U[(static_cast<long long>(e) * K + k) * Cp + c] = from_f32<OutT>(u[e]);
}

// ---- per-tile scale ------------------------------------------------------------

template <int M>
__global__ void __launch_bounds__(256) tile_scale_kernel(const __half* __restrict__ x, float* __restrict__ scale,
                                                         int C, int H, int W, int pad_h, int pad_w, int tiles_h,
                                                         int tiles_w, long long P) {
    constexpr int A = M + 2;
    const long long p = static_cast<long long>(blockIdx.x) * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= P) return;
    const int tw = static_cast<int>(p % tiles_w);
    const int th = static_cast<int>((p / tiles_w) % tiles_h);
    const long long n = p / (static_cast<long long>(tiles_w) * tiles_h);
    const int y0 = th * M - pad_h, x0 = tw * M - pad_w;
    float amax = 0.f;
    for (int c = lane; c < C; c += 32) {
        const __half* plane = x + (n * C + c) * static_cast<long long>(H) * W;
        for (int i = 0; i < A; ++i) {
            const int y = y0 + i;
            if (y < 0 || y >= H) continue;
            for (int j = 0; j < A; ++j) {
                const int xx = x0 + j;
                if (xx < 0 || xx >= W) continue;
                amax = fmaxf(amax, fabsf(__half2float(plane[static_cast<long long>(y) * W + xx])));
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if (lane == 0) {
        float s = 1.f;
        if (amax > 0.f && isfinite(amax)) {
            int ex;
            frexpf(amax, &ex);                 // amax = f * 2^ex, f in [0.5, 1)
            ex = max(-20, min(20, ex - 1));    // floor(log2(amax))
            s = ldexpf(1.f, -ex);              // scaled patch max in [1, 2)
        }
        scale[p] = s;
    }
}

// ---- input transform -------------------------------------------------------------

constexpr int kCB = 64;        // channels per CTA (one channel pair per lane)
constexpr int kCS = kCB + 2;   // staged channel stride in halves: odd word stride

template <class TF, class OutT>
__global__ void __launch_bounds__(256) input_transform_kernel(const __half* __restrict__ x, OutT* __restrict__ V,
                                                              const float* __restrict__ scale, int C, int H, int W,
                                                              int pad_h, int pad_w, int tiles_h, int tiles_w,
                                                              long long P, int Cp, int tb, int twb, int nbh,
                                                              int nbw) {
    constexpr int M = TF::M, A = TF::ALPHA;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __half* sm = reinterpret_cast<__half*>(smem_raw);
    const int rows = tb * M + 2, cols = twb * M + 2;
    int bid = blockIdx.x;
    const int bw = bid % nbw;
    bid /= nbw;
    const int bh = bid % nbh;
    const long long n = bid / nbh;
    const int c0 = blockIdx.y * kCB;
    const int th0 = bh * tb, tw0 = bw * twb;
    const int y0 = th0 * M - pad_h, x0 = tw0 * M - pad_w;
    const __half* xn = x + n * C * static_cast<long long>(H) * W;
    const __half zero = __float2half_rn(0.f);

    const int total = kCB * rows * cols;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        const int col = i % cols;
        const int t = i / cols;
        const int r = t % rows;
        const int c = t / rows;
        const int gy = y0 + r, gx = x0 + col, gc = c0 + c;
        __half v = zero;
        if (gc < C && gy >= 0 && gy < H && gx >= 0 && gx < W)
            v = xn[(static_cast<long long>(gc) * H + gy) * W + gx];
        sm[(r * cols + col) * kCS + c] = v;
    }
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int ch = c0 + 2 * lane;
    const bool active = ch < Cp;
    const int ntb = min(tb, tiles_h - th0), ntw = min(twb, tiles_w - tw0);
    using P2 = Pair<OutT>;
    for (int t = warp; t < ntb * ntw; t += nwarps) {
        const int tr = t / ntw, tc = t % ntw;
        const long long p = (n * tiles_h + th0 + tr) * tiles_w + tw0 + tc;
        float d0[A * A], d1[A * A];
        const __half* base = sm + ((tr * M) * cols + tc * M) * kCS + 2 * lane;
#pragma unroll
        for (int i = 0; i < A; ++i) {
#pragma unroll
            for (int j = 0; j < A; ++j) {
                const float2 f = __half22float2(*reinterpret_cast<const __half2*>(base + (i * cols + j) * kCS));
                d0[i * A + j] = f.x;
                d1[i * A + j] = f.y;
            }
        }
        if (scale) {
            const float s = scale[p];
#pragma unroll
            for (int i = 0; i < A * A; ++i) {
                d0[i] *= s;
                d1[i] *= s;
            }
        }
        float v0[A * A], v1[A * A];
        input_tile_transform<TF>(d0, v0);
        input_tile_transform<TF>(d1, v1);
        if (active) {
            OutT* dst = V + p * Cp + ch;
#pragma unroll
            for (int e = 0; e < A * A; ++e)
                *reinterpret_cast<typename P2::type*>(dst + static_cast<long long>(e) * P * Cp) =
                    P2::make(v0[e], v1[e]);
        }
    }
}

// ---- output transform ----------------------------------------------------------

template <class MT> struct MLoad;
template <> struct MLoad<__half> {
    __device__ static float2 load(const __half* p) { return __half22float2(*reinterpret_cast<const __half2*>(p)); }
};
template <> struct MLoad<float> {
    __device__ static float2 load(const float* p) { return *reinterpret_cast<const float2*>(p); }
};

template <class TF, class MT>
__global__ void __launch_bounds__(256) output_transform_kernel(const MT* __restrict__ Mw, __half* __restrict__ out,
                                                               const float* __restrict__ scale, int K, int OH, int OW,
                                                               int tiles_h, int tiles_w, long long P, int Kp, int tb,
                                                               int twb, int nbh, int nbw) {
    constexpr int M = TF::M, A = TF::ALPHA;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __half* so = reinterpret_cast<__half*>(smem_raw);
    const int orows = tb * M, ocols = twb * M;
    const int ps = (orows * ocols) | 1;  // odd plane stride: lanes hit distinct banks
    int bid = blockIdx.x;
    const int bw = bid % nbw;
    bid /= nbw;
    const int bh = bid % nbh;
    const long long n = bid / nbh;
    const int k0 = blockIdx.y * kCB;
    const int th0 = bh * tb, tw0 = bw * twb;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int ntb = min(tb, tiles_h - th0), ntw = min(twb, tiles_w - tw0);
    const int kk = k0 + 2 * lane;
    const bool active = kk < Kp;
    for (int t = warp; t < ntb * ntw; t += nwarps) {
        const int tr = t / ntw, tc = t % ntw;
        const long long p = (n * tiles_h + th0 + tr) * tiles_w + tw0 + tc;
        float m0[A * A], m1[A * A];
        if (active) {
            const MT* src = Mw + p * Kp + kk;
#pragma unroll
            for (int e = 0; e < A * A; ++e) {
                const float2 f = MLoad<MT>::load(src + static_cast<long long>(e) * P * Kp);
                m0[e] = f.x;
                m1[e] = f.y;
            }
        } else {
#pragma unroll
            for (int e = 0; e < A * A; ++e) m0[e] = m1[e] = 0.f;
        }
        float y0[M * M], y1[M * M];
        output_tile_transform<TF>(m0, y0);
        output_tile_transform<TF>(m1, y1);
        const float inv = scale ? 1.f / scale[p] : 1.f;  // exact: scale is a power of two
        __half* d0 = so + (2 * lane) * ps + (tr * M) * ocols + tc * M;
        __half* d1 = d0 + ps;
#pragma unroll
        for (int i = 0; i < M; ++i) {
#pragma unroll
            for (int j = 0; j < M; ++j) {
                d0[i * ocols + j] = __float2half_rn(y0[i * M + j] * inv);
                d1[i * ocols + j] = __float2half_rn(y1[i * M + j] * inv);
            }
        }
    }
    __syncthreads();
    const int total = kCB * orows * ocols;
    const int vrows = ntb * M, vcols = ntw * M;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        const int ocol = i % ocols;
        const int t = i / ocols;
        const int orow = t % orows;
        const int c = t / orows;
        const int k = k0 + c, oh = th0 * M + orow, ow = tw0 * M + ocol;
        if (k < K && orow < vrows && ocol < vcols && oh < OH && ow < OW)
            out[((n * K + k) * OH + oh) * static_cast<long long>(OW) + ow] = so[c * ps + orow * ocols + ocol];
    }
}

struct Blocking {
    int tb, twb, nbh, nbw, smem_in, smem_out;
};

Blocking choose_blocking(const Geom& g) {
    Blocking b;
    const int M = g.m;
    b.twb = std::min(g.tiles_w, M == 2 ? 16 : 8);
    const int cols = b.twb * M + 2;
    b.tb = 1;
    for (int tb = 1; tb <= g.tiles_h; ++tb) {
        const int rows = tb * M + 2;
        if (rows * cols * kCS * 2 > 48 * 1024 || tb * b.twb > 64) break;
        b.tb = tb;
    }
    b.nbh = (g.tiles_h + b.tb - 1) / b.tb;
    b.nbw = (g.tiles_w + b.twb - 1) / b.twb;
    b.smem_in = (b.tb * M + 2) * cols * kCS * 2;
    b.smem_out = kCB * ((b.tb * M * b.twb * M) | 1) * 2;
    return b;
}

template <class TF, class OutT>
cudaError_t input_launch(const Geom& g, const void* x, void* V, const float* scale, cudaStream_t s) {
    const Blocking b = choose_blocking(g);
    auto kern = input_transform_kernel<TF, OutT>;
    if (b.smem_in > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, b.smem_in);
        if (e != cudaSuccess) return e;
    }
    dim3 grid(static_cast<unsigned>(static_cast<long long>(g.n) * b.nbh * b.nbw), (g.cp + kCB - 1) / kCB);
    kern<<<grid, 256, b.smem_in, s>>>(static_cast<const __half*>(x), static_cast<OutT*>(V), scale, g.c, g.h, g.w,
                                      g.pad_h, g.pad_w, g.tiles_h, g.tiles_w, g.P, g.cp, b.tb, b.twb, b.nbh, b.nbw);
    return cudaGetLastError();
}

template <class TF, class MT>
cudaError_t output_launch(const Geom& g, const void* Mw, void* out, const float* scale, cudaStream_t s) {
    const Blocking b = choose_blocking(g);
    auto kern = output_transform_kernel<TF, MT>;
    if (b.smem_out > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, b.smem_out);
        if (e != cudaSuccess) return e;
    }
    dim3 grid(static_cast<unsigned>(static_cast<long long>(g.n) * b.nbh * b.nbw), (g.kp + kCB - 1) / kCB);
    kern<<<grid, 256, b.smem_out, s>>>(static_cast<const MT*>(Mw), static_cast<__half*>(out), scale, g.k, g.oh, g.ow,
                                       g.tiles_h, g.tiles_w, g.P, g.kp, b.tb, b.twb, b.nbh, b.nbw);
    return cudaGetLastError();
}

template <class TF, class OutT>
cudaError_t filter_launch(const void* w, void* U, int K, int C, int Cp, cudaStream_t s) {
    const long long total = static_cast<long long>(K) * Cp;
    const unsigned blocks = static_cast<unsigned>((total + 255) / 256);
    filter_transform_kernel<TF, OutT><<<blocks, 256, 0, s>>>(static_cast<const __half*>(w), static_cast<OutT*>(U), K, C,
                                                            Cp);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_filter_transform(Xform xf, OpType op, const void* weight, void* U, int K, int C, int Cp,
                                    cudaStream_t stream) {
    const bool bf = op == OpType::BF16;
    switch (xf) {
        case Xform::F2:
            return bf ? filter_launch<F2, __nv_bfloat16>(weight, U, K, C, Cp, stream)
                      : filter_launch<F2, __half>(weight, U, K, C, Cp, stream);
        case Xform::F4:
            return bf ? filter_launch<F4, __nv_bfloat16>(weight, U, K, C, Cp, stream)
                      : filter_launch<F4, __half>(weight, U, K, C, Cp, stream);
        case Xform::F4Ref:
            return bf ? filter_launch<F4Ref, __nv_bfloat16>(weight, U, K, C, Cp, stream)
                      : filter_launch<F4Ref, __half>(weight, U, K, C, Cp, stream);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_tile_scale(const Geom& g, const void* x, float* scale, cudaStream_t stream) {
    const unsigned blocks = static_cast<unsigned>((g.P + 7) / 8);
    if (g.m == 2)
        tile_scale_kernel<2><<<blocks, 256, 0, stream>>>(static_cast<const __half*>(x), scale, g.c, g.h, g.w, g.pad_h,
                                                         g.pad_w, g.tiles_h, g.tiles_w, g.P);
    else
        tile_scale_kernel<4><<<blocks, 256, 0, stream>>>(static_cast<const __half*>(x), scale, g.c, g.h, g.w, g.pad_h,
                                                         g.pad_w, g.tiles_h, g.tiles_w, g.P);
    return cudaGetLastError();
}

cudaError_t launch_input_transform(Xform xf, OpType op, const Geom& g, const void* x, void* V, const float* scale,
                                   cudaStream_t stream) {
    const bool bf = op == OpType::BF16;
    switch (xf) {
        case Xform::F2:
            return bf ? input_launch<F2, __nv_bfloat16>(g, x, V, scale, stream)
                      : input_launch<F2, __half>(g, x, V, scale, stream);
        case Xform::F4:
            return bf ? input_launch<F4, __nv_bfloat16>(g, x, V, scale, stream)
                      : input_launch<F4, __half>(g, x, V, scale, stream);
        case Xform::F4Ref:
            return bf ? input_launch<F4Ref, __nv_bfloat16>(g, x, V, scale, stream)
                      : input_launch<F4Ref, __half>(g, x, V, scale, stream);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_output_transform(Xform xf, bool m_fp32, const Geom& g, const void* Mw, void* out,
                                    const float* scale, cudaStream_t stream) {
    switch (xf) {
        case Xform::F2:
            return m_fp32 ? output_launch<F2, float>(g, Mw, out, scale, stream)
                          : output_launch<F2, __half>(g, Mw, out, scale, stream);
        case Xform::F4:
            return m_fp32 ? output_launch<F4, float>(g, Mw, out, scale, stream)
                          : output_launch<F4, __half>(g, Mw, out, scale, stream);
        case Xform::F4Ref:
            return m_fp32 ? output_launch<F4Ref, float>(g, Mw, out, scale, stream)
                          : output_launch<F4Ref, __half>(g, Mw, out, scale, stream);
    }
    return cudaErrorInvalidValue;
}

}  // namespace wg
