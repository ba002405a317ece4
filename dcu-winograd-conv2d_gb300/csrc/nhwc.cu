// NHWC input and output transforms (channels-last tensors).
//
// Input: x[N][H][W][C] fp16.  A work item (image, block of tile rows, block
// of cb channels) is one 4-D TMA box {cb channels, the padded row width,
// the item's padded rows, 1 image} starting at (c0, -pad_w, y0 - pad_h, n):
// the tensor-map zero fill supplies every padding pixel and every channel
// past C, so the arithmetic needs no masks.  In shared memory a pixel's cb
// channels are contiguous, so a thread's channel pair is one 4-byte load and
// a warp's loads of one element cover 64-128 contiguous bytes.  The V it
// writes is the same V[E][Cp/8][Pp][8] as the NCHW kernel's, so the GEMM is
// shared.  Persistent CTAs; warp 7 issues the next item's TMA into the other
// half of a double buffer while warps 0-6 transform the current one.
//
// Output: y[N][OH][OW][K] fp16 from a row-major M[E][P][Kp] (the GEMM's
// row-major epilogue): thread = (tile, output-channel pair), so both the
// M loads and the NHWC stores of a warp are contiguous.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdlib>

#include "wg_kernels.h"
#include "wg_launch.h"
#include "wg_ptx.cuh"
#include "wg_transforms.cuh"

namespace wg {

namespace {

constexpr int kNhComputeWarps = 7;
constexpr int kNhThreads = 32 * (kNhComputeWarps + 1);

__device__ __forceinline__ float2 f2c(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 nfma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 nadd2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 nsub2(float2 a, float2 b) { return __ffma2_rn(b, f2c(-1.f), a); }

// B^T d on an ALPHA-vector of channel pairs (the matrices of TF::bt).
template <class TF> struct NBt;
template <> struct NBt<F2> {
    __device__ __forceinline__ static void run(const float2 (&d)[4], float2 (&o)[4]) {
        o[0] = nsub2(d[0], d[2]);
        o[1] = nadd2(d[1], d[2]);
        o[2] = nsub2(d[2], d[1]);
        o[3] = nsub2(d[1], d[3]);
    }
};
template <> struct NBt<F4> {
    __device__ __forceinline__ static void run(const float2 (&d)[6], float2 (&o)[6]) {
        const float2 t = nsub2(d[3], d[1]), u = nsub2(d[4], d[2]);
        o[0] = nadd2(nfma2(d[2], f2c(-2.f), nfma2(t, f2c(1.5f), d[0])), d[4]);
        o[1] = nsub2(nfma2(d[3], f2c(2.5f), nfma2(d[2], f2c(0.5f), d[4])), d[1]);
        o[2] = nadd2(nfma2(d[2], f2c(-2.5f), nfma2(d[3], f2c(0.5f), d[4])), d[1]);
        o[3] = nfma2(t, f2c(2.f), u);
        o[4] = nfma2(t, f2c(-0.5f), u);
        o[5] = nadd2(nfma2(d[3], f2c(-2.f), nfma2(u, f2c(1.5f), d[1])), d[5]);
    }
};
template <> struct NBt<F4Ref> {
    __device__ __forceinline__ static void run(const float2 (&d)[6], float2 (&o)[6]) {
        const float2 t = nsub2(d[3], d[1]), u = nsub2(d[4], d[2]);
        o[0] = nfma2(d[2], f2c(-5.f), nfma2(d[0], f2c(4.f), d[4]));
        o[1] = nfma2(nadd2(d[1], d[2]), f2c(-4.f), nadd2(d[3], d[4]));
        o[2] = nfma2(nsub2(d[1], d[2]), f2c(4.f), nsub2(d[4], d[3]));
        o[3] = nfma2(t, f2c(2.f), u);
        o[4] = nfma2(t, f2c(-2.f), u);
        o[5] = nfma2(d[3], f2c(-5.f), nfma2(d[1], f2c(4.f), d[5]));
    }
};

template <class T> __device__ __forceinline__ uint32_t npack(float2 v);
template <> __device__ __forceinline__ uint32_t npack<__half>(float2 v) {
    __half2 h = __floats2half2_rn(v.x, v.y);
    return *reinterpret_cast<uint32_t*>(&h);
}
template <> __device__ __forceinline__ uint32_t npack<__nv_bfloat16>(float2 v) {
    __nv_bfloat162 h = __floats2bfloat162_rn(v.x, v.y);
    return *reinterpret_cast<uint32_t*>(&h);
}

template <class TF, class OutT, bool KEEP>
__device__ __forceinline__ void nh_compute(const NhwcInDesc& d, long long local, int n_base, const unsigned char* buf,
                                           int cw) {
    constexpr int M = TF::M, A = TF::ALPHA;
    const int bx = static_cast<int>(local / d.gy), by = static_cast<int>(local % d.gy);
    const int bh = bx % d.nbh;
    const long long n = n_base + bx / d.nbh;
    const int c0 = by * d.cb;
    const int th0 = bh * d.tb;
    const int ntb = min(d.tb, d.tiles_h - th0);
    const int tiles_w = d.tiles_w, bw = d.bw, cb = d.cb;
    const int ntiles = ntb * tiles_w;
    const int G = min(cb, d.CG * 8 - c0) / 8;  // granules of this block inside Cp
    const long long Pp = d.Pp;
    const long long estride = static_cast<long long>(d.CG) * Pp * 8;
    const long long p0 = ((n - n_base) * d.tiles_h + th0) * tiles_w;  // tiles of this launch's images
    OutT* __restrict__ V = static_cast<OutT*>(d.V);
    const int tasks = ntiles * G * 4;
    // G is 1-4 and rest below 2^14: rest / 3 by multiply-shift (exact below 2^17)
    const uint32_t g_shift = static_cast<uint32_t>(G >> 1);
    for (int task = cw * 32 + (threadIdx.x & 31); task < tasks; task += kNhComputeWarps * 32) {
        const int sub = task & 3;
        const uint32_t rest = static_cast<uint32_t>(task >> 2);
        const int t = static_cast<int>(G == 3 ? (rest * 43691u) >> 17 : rest >> g_shift);
        const int g = static_cast<int>(rest) - t * G;
        const int tr = static_cast<int>(fast_div(d.fd_tw, static_cast<uint32_t>(t))), tw = t - tr * tiles_w;
        // pixel (tr*M + i, tw*M + j) of the box, channels g*8 + sub*2 + {0,1}
        const unsigned char* src = buf + (static_cast<size_t>(tr * M) * bw + tw * M) * cb * 2 + (g * 8 + sub * 2) * 2;
        float2 r[A][A];
#pragma unroll
        for (int i = 0; i < A; ++i) {
            float2 dv[A];
#pragma unroll
            for (int j = 0; j < A; ++j)
                dv[j] = __half22float2(*reinterpret_cast<const __half2*>(src + (static_cast<size_t>(i) * bw + j) * cb * 2));
            NBt<TF>::run(dv, r[i]);
        }
        uint32_t pk[A * A];
#pragma unroll
        for (int j = 0; j < A; ++j) {
            float2 col[A], v[A];
#pragma unroll
            for (int i = 0; i < A; ++i) col[i] = r[i][j];
            NBt<TF>::run(col, v);
#pragma unroll
            for (int i = 0; i < A; ++i) pk[i * A + j] = npack<OutT>(v[i]);
        }
        // V kept in L2 for the GEMM where it fits (KEEP), plain stores otherwise
        OutT* dst = V + ((static_cast<long long>(c0 / 8 + g)) * Pp + p0 + t) * 8 + sub * 2;
        const uint64_t keep = KEEP ? l2_evict_last() : 0;
#pragma unroll
        for (int e = 0; e < A * A; ++e) {
            if constexpr (KEEP)
                st_hint_b32(dst, pk[e], keep);
            else
                *reinterpret_cast<uint32_t*>(dst) = pk[e];
            dst += estride;
        }
    }
}

template <class TF, class OutT, bool KEEP>
__global__ void __launch_bounds__(kNhThreads, 2)
    nhwc_input_transform(const __grid_constant__ NhwcInDesc d, int n_base, long long total, int buf_bytes,
                         DevErr* err) {
    constexpr int M = TF::M;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* empty = full + 2;
    volatile int* abort_flag = reinterpret_cast<volatile int*>(full + 4);
    unsigned char* bufs = smem_raw + 128;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], kNhComputeWarps);
        }
        *abort_flag = 0;
        fence_barrier_init();
    }
    pdl_wait();     // input written, earlier readers of V done
    pdl_trigger();
    __syncthreads();
    if (warp == kNhComputeWarps) {
        if ((threadIdx.x & 31) == 0) {
            tma_prefetch_desc(&d.tmX);
            int k = 0;
            for (long long item = blockIdx.x; item < total; item += gridDim.x, ++k) {
                const int b = k & 1;
                if (!mbar_wait(&empty[b], ((k >> 1) & 1) ^ 1u, abort_flag, err, ERR_SITE_EMPTY)) break;
                const int bx = static_cast<int>(item / d.gy), by = static_cast<int>(item % d.gy);
                const int bh = bx % d.nbh;
                const int n = n_base + bx / d.nbh;
                mbar_arrive_expect_tx(&full[b], static_cast<uint32_t>(buf_bytes));
                tma_load_4d(bufs + b * buf_bytes, &d.tmX, &full[b], by * d.cb, -d.pad_w, bh * d.tb * M - d.pad_h, n);
            }
        }
    } else {
        int k = 0;
        for (long long item = blockIdx.x; item < total; item += gridDim.x, ++k) {
            const int b = k & 1;
            if (!mbar_wait(&full[b], (k >> 1) & 1, abort_flag, err, ERR_SITE_FULL)) break;
            nh_compute<TF, OutT, KEEP>(d, item, n_base, bufs + b * buf_bytes, warp);
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

// ---- output: row-major M -> NHWC ------------------------------------------------

template <class MT> struct MP;  // a channel pair of M
template <> struct MP<float> {
    __device__ static float2 load(const float* p) { return *reinterpret_cast<const float2*>(p); }
};
template <> struct MP<__half> {
    __device__ static float2 load(const __half* p) { return __half22float2(*reinterpret_cast<const __half2*>(p)); }
};

template <class TF, class MT>
__device__ __forceinline__ void nh_out_tile(const NhwcOutDesc& d, long long p);

template <class TF, class MT>
__global__ void __launch_bounds__(256) nhwc_output_transform(const __grid_constant__ NhwcOutDesc d) {
    constexpr int A = TF::ALPHA, E = A * A;
    pdl_wait();     // M written, earlier readers of the output done
    pdl_trigger();
    const long long p = static_cast<long long>(blockIdx.x) * d.tpc + fast_div(d.fd_tpt, threadIdx.x);
    if (p < d.P && threadIdx.x < d.tpt * d.tpc) nh_out_tile<TF, MT>(d, p);
    if (d.discard_m) {
        // every M row of the CTA's tiles has been read (rows are whole 128-byte
        // lines, each read by this CTA only): drop them without write-back
        __syncthreads();
        const long long p_first = static_cast<long long>(blockIdx.x) * d.tpc;
        const int tiles = static_cast<int>(min(static_cast<long long>(d.tpc), d.P - p_first));
        const int lpr = d.Kp * static_cast<int>(sizeof(MT)) / 128;   // lines per row
        const unsigned char* Mb = static_cast<const unsigned char*>(d.Mw);
        // i = (e * tpc + tt) * lpr + l over whole CTAs' worth of tiles; the
        // last CTA skips its missing ones
        for (int i = threadIdx.x; i < E * d.tpc * lpr; i += blockDim.x) {
            const uint32_t rest = fast_div(d.fd_lpr, i), e = fast_div(d.fd_tpc, rest);
            const int l = static_cast<int>(i - rest * lpr), tt = static_cast<int>(rest - e * d.tpc);
            if (tt < tiles)
                discard_l2_line(Mb + ((static_cast<long long>(e) * d.P + p_first + tt) * d.Kp) * sizeof(MT) + l * 128);
        }
    }
}

template <class TF, class MT>
__device__ __forceinline__ void nh_out_tile(const NhwcOutDesc& d, long long p) {
    constexpr int M = TF::M, A = TF::ALPHA, E = A * A;
    // p < P < 2^31 (the GEMM descriptor refuses more tiles)
    const uint32_t pu = static_cast<uint32_t>(p);
    const uint32_t r = fast_div(d.fd_tw, pu), nn = fast_div(d.fd_th, r);
    const int tw = static_cast<int>(pu - r * static_cast<uint32_t>(d.tiles_w));
    const int th = static_cast<int>(r - nn * static_cast<uint32_t>(d.tiles_h));
    const long long n = nn;
    const int oh0 = th * M, ow0 = tw * M;
    const int vr = min(M, d.OH - oh0), vc = min(M, d.OW - ow0);
    const MT* Mw = static_cast<const MT*>(d.Mw);
    const long long estride = d.P * d.Kp;
    const int kk0 = static_cast<int>(threadIdx.x - fast_div(d.fd_tpt, threadIdx.x) * static_cast<uint32_t>(d.tpt));
    for (int kk = kk0; 2 * kk < d.K; kk += d.tpt) {
        const MT* src = Mw + p * d.Kp + 2 * kk;
        float2 m[E];
#pragma unroll
        for (int e = 0; e < E; ++e) m[e] = MP<MT>::load(src + e * estride);
        float y[2][M * M];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            float mm[E];
#pragma unroll
            for (int e = 0; e < E; ++e) mm[e] = h ? m[e].y : m[e].x;
            float yy[M * M];
            output_tile_transform<TF>(mm, yy);
#pragma unroll
            for (int q = 0; q < M * M; ++q) y[h][q] = yy[q];
        }
        const bool pair = 2 * kk + 1 < d.K;
#pragma unroll
        for (int i = 0; i < M; ++i) {
            if (i >= vr) continue;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                if (j >= vc) continue;
                __half* o = d.out + ((n * d.OH + oh0 + i) * d.OW + ow0 + j) * static_cast<long long>(d.K) + 2 * kk;
                if (pair && (d.K & 1) == 0)
                    *reinterpret_cast<__half2*>(o) = __floats2half2_rn(y[0][i * M + j], y[1][i * M + j]);
                else {
                    o[0] = __float2half_rn(y[0][i * M + j]);
                    if (pair) o[1] = __float2half_rn(y[1][i * M + j]);
                }
            }
        }
    }
}

}  // namespace

cudaError_t make_nhwc_in_desc(NhwcInDesc& d, const Geom& g, const void* x, void* V, int* smem) {
    const int M = g.m, A = g.alpha;
    d = NhwcInDesc{};
    d.V = V;
    d.C = g.c; d.H = g.h; d.W = g.w; d.pad_h = g.pad_h; d.pad_w = g.pad_w;
    d.tiles_h = g.tiles_h; d.tiles_w = g.tiles_w;
    d.fd_tw = make_fastdiv(static_cast<uint32_t>(g.tiles_w));
    d.Pp = round_rows(g.P);
    d.CG = g.cp / 8;
    d.bw = g.tiles_w * M + A - M;
    // a TMA tensor's strides are multiples of 16 bytes: C a multiple of 8
    if (d.bw > 256 || g.c % 8 != 0) return cudaErrorNotSupported;
    // channel block: 32 (or C rounded up to 8 when smaller); tile-row block:
    // the most rows whose box stays within 48 KB, at most 256 rows
    d.cb = std::min(32, g.cp);
    int tb = 1;
    while (tb < g.tiles_h && ((tb + 1) * M + A - M) <= 256 &&
           static_cast<long long>(d.cb) * d.bw * ((tb + 1) * M + A - M) * 2 <= 48 * 1024)
        ++tb;
    d.tb = tb;
    d.rows = tb * M + A - M;
    d.nbh = (g.tiles_h + tb - 1) / tb;
    d.gy = (g.c + d.cb - 1) / d.cb;
    d.gx = static_cast<long long>(g.n) * d.nbh;
    const int box_bytes = d.cb * d.bw * d.rows * 2;
    *smem = 128 + 2 * box_bytes;
    if (*smem > 227 * 1024) return cudaErrorNotSupported;
    // x[N][H][W][C]: dims innermost first
    cuuint64_t dims[4] = {static_cast<cuuint64_t>(g.c), static_cast<cuuint64_t>(g.w), static_cast<cuuint64_t>(g.h),
                          static_cast<cuuint64_t>(g.n)};
    cuuint64_t strides[3] = {static_cast<cuuint64_t>(g.c) * 2, static_cast<cuuint64_t>(g.w) * g.c * 2,
                             static_cast<cuuint64_t>(g.h) * g.w * g.c * 2};
    cuuint32_t box[4] = {static_cast<cuuint32_t>(d.cb), static_cast<cuuint32_t>(d.bw), static_cast<cuuint32_t>(d.rows), 1};
    if (encode_tiled(&d.tmX, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 4, const_cast<void*>(x), dims, strides, box,
                     CU_TENSOR_MAP_SWIZZLE_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    return cudaSuccess;
}

cudaError_t launch_nhwc_input_transform(Xform xf, OpType op, const NhwcInDesc& d, int smem, int n_base, int n_images,
                                        DevErr* err, cudaStream_t s) {
    const long long total = static_cast<long long>(n_images) * d.nbh * d.gy;
    if (total <= 0) return cudaSuccess;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0)
        sms = 148;
    const int per_sm = std::max(1, std::min(2, 233472 / (smem + 1024)));
    const unsigned grid = static_cast<unsigned>(std::min<long long>(total, static_cast<long long>(sms) * per_sm));
    const int buf = (smem - 128) / 2;
    const bool bf = op == OpType::BF16;
    auto go = [&](auto kern) -> cudaError_t {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        return launch_pdl(kern, dim3(grid), dim3(kNhThreads), smem, s, d, n_base, total, buf, err);
    };
    // V of this launch within the L2 size: kept there for the GEMM (fp16)
    const int A = xf == Xform::F2 ? 4 : 6;
    const bool keep = !bf && static_cast<long long>(A) * A * d.CG * 8 * d.Pp * 2 <= l2_cache_bytes();
    switch (xf) {
        case Xform::F2:
            if (bf) return go(nhwc_input_transform<F2, __nv_bfloat16, false>);
            return keep ? go(nhwc_input_transform<F2, __half, true>) : go(nhwc_input_transform<F2, __half, false>);
        case Xform::F4:
            if (bf) return go(nhwc_input_transform<F4, __nv_bfloat16, false>);
            return keep ? go(nhwc_input_transform<F4, __half, true>) : go(nhwc_input_transform<F4, __half, false>);
        case Xform::F4Ref:
            return bf ? go(nhwc_input_transform<F4Ref, __nv_bfloat16, false>)
                      : go(nhwc_input_transform<F4Ref, __half, false>);
    }
    return cudaErrorInvalidValue;
}

NhwcOutDesc make_nhwc_out_desc(const Geom& g, const void* Mw, void* out) {
    NhwcOutDesc d{};
    d.Mw = Mw;
    d.out = static_cast<__half*>(out);
    d.K = g.k; d.Kp = g.kp; d.OH = g.oh; d.OW = g.ow; d.tiles_h = g.tiles_h; d.tiles_w = g.tiles_w;
    d.P = g.P;
    d.tpt = std::min(256, (g.kp / 2 + 31) / 32 * 32);
    d.tpc = 256 / d.tpt;
    d.fd_tpt = make_fastdiv(static_cast<uint32_t>(d.tpt));
    d.fd_tw = make_fastdiv(static_cast<uint32_t>(g.tiles_w));
    d.fd_th = make_fastdiv(static_cast<uint32_t>(g.tiles_h));
    d.fd_tpc = make_fastdiv(static_cast<uint32_t>(d.tpc));
    return d;
}

cudaError_t launch_nhwc_output_transform(Xform xf, MType mt, const NhwcOutDesc& dd, cudaStream_t s) {
    if (mt == MType::F24) return cudaErrorNotSupported;   // row-major M is fp16 or fp32
    const bool m_fp32 = mt == MType::F32;
    const long long blocks = (dd.P + dd.tpc - 1) / dd.tpc;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    const dim3 grid(static_cast<unsigned>(blocks));
    // M larger than L2 is dropped from it as soon as it is read, where its rows
    // are whole 128-byte lines; WG_CONV2D_KEEP_WORKSPACE=1 keeps it
    NhwcOutDesc d = dd;
    const int esize = m_fp32 ? 4 : 2, A = xf == Xform::F2 ? 4 : 6;
    const char* keep_ws = std::getenv("WG_CONV2D_KEEP_WORKSPACE");
    d.discard_m = !(keep_ws && std::atoi(keep_ws) != 0) && (d.Kp * esize) % 128 == 0 &&
                  static_cast<long long>(A) * A * d.P * d.Kp * esize > l2_cache_bytes();
    d.fd_lpr = make_fastdiv(static_cast<uint32_t>(std::max(1, d.Kp * esize / 128)));
    switch (xf) {
        case Xform::F2:
            return m_fp32 ? launch_pdl(nhwc_output_transform<F2, float>, grid, dim3(256), 0, s, d)
                          : launch_pdl(nhwc_output_transform<F2, __half>, grid, dim3(256), 0, s, d);
        case Xform::F4: return launch_pdl(nhwc_output_transform<F4, float>, grid, dim3(256), 0, s, d);
        case Xform::F4Ref: return launch_pdl(nhwc_output_transform<F4Ref, float>, grid, dim3(256), 0, s, d);
    }
    return cudaErrorInvalidValue;
}

}  // namespace wg
