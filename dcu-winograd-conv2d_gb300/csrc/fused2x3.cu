// Fully fused F(2x2,3x3): input transform, Winograd-domain GEMM and output
// transform in one kernel; transformed tiles never leave the SM.
//
// This is the reference's winograd_2x3_kernel (src/winograd_2x3_fused.cpp:10-369,
// launcher :372-392) re-designed for tcgen05:
//   * CTA = 128 output tiles x 32 output channels, looping over the input
//     channels in chunks of 16 (the reference: 32 tiles x 32 channels,
//     chunks of 16, 16 wave64 MMAC GEMMs);
//   * warps 0-7 load the 4x4 input patches (zero halo), run B^T d B in fp32
//     and write the 16 Winograd-domain tiles straight into shared memory in
//     the tcgen05 canonical K-major layout (no swizzle);
//   * the transformed filter U (made once per weight set) arrives by TMA;
//   * warp 8 issues the 16 tcgen05.mma (M=128, N=32, K=16) per chunk from
//     one thread, accumulating all 16 elements in the 512 TMEM columns;
//   * after the last chunk warps 0-7 read TMEM, apply A^T m A and write
//     the 2x2 outputs to NCHW.
// Two pipeline stages; every wait is bounded (wg_ptx.cuh).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "wg_kernels.h"
#include "wg_ptx.cuh"
#include "wg_transforms.cuh"

namespace wg {

namespace {

constexpr int kTilesPerCta = 128;
constexpr int kOcPerCta = 32;
constexpr int kChunk = 16;                               // input channels per stage
constexpr int kElems = 16;                               // 4x4 Winograd elements
constexpr int kAHalf = kElems * kTilesPerCta * 16;       // 8 channels of every element: 32 KB
constexpr int kABytes = 2 * kAHalf;                      // 64 KB
constexpr int kBHalf = kElems * kOcPerCta * 16;          // 8 KB
constexpr int kBBytes = 2 * kBHalf;                      // 16 KB
constexpr int kStageBytes = kABytes + kBBytes;           // 80 KB
constexpr int kStages = 2;
constexpr int kSmem = kStages * kStageBytes + 1024 + 256;
constexpr int kProducers = 256;
constexpr int kThreads = kProducers + 32;

template <bool BF16> struct OpT;
template <> struct OpT<false> {
    __device__ static uint32_t pack(float a, float b) {
        __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<uint32_t*>(&h);
    }
};
template <> struct OpT<true> {
    __device__ static uint32_t pack(float a, float b) {
        __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<uint32_t*>(&h);
    }
};

template <bool BF16>
__global__ void __launch_bounds__(kThreads, 1)
    fused2x3_kernel(const __half* __restrict__ x, const __grid_constant__ CUtensorMap tmU, __half* __restrict__ out,
                    int C, int H, int W, int K, int pad_h, int pad_w, int OH, int OW, int tiles_h, int tiles_w,
                    int P, int c_chunks, int n_blocks, DevErr* err) {
    constexpr uint32_t kIdesc = make_idesc_f16(128, kOcPerCta, BF16);
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes);
    uint64_t* full = bars;             // [2] producers (256) + TMA expect_tx (1)
    uint64_t* empty = bars + 2;        // [2] MMA commit
    uint64_t* tfull = bars + 4;        // accumulators ready
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 5);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n_blk = blockIdx.x % n_blocks;
    const int m_blk = blockIdx.x / n_blocks;

    if (tid == 0) {
        for (int i = 0; i < kStages; ++i) {
            mbar_init(&full[i], kProducers + 1);
            mbar_init(&empty[i], 1);
        }
        mbar_init(tfull, 1);
        *abort_flag = 0;
        fence_barrier_init();
    }
    if (warp == 8) tmem_alloc(tmem_slot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 8) {
        if (lane == 0) {
            tma_prefetch_desc(&tmU);
            auto issue_tma = [&](int chunk) {
                const int s = chunk & 1;
                unsigned char* b = smem + s * kStageBytes + kABytes;
                mbar_arrive_expect_tx(&full[s], kBBytes);
                tma_load_3d(b, &tmU, &full[s], chunk * kChunk, n_blk * kOcPerCta, 0);
                tma_load_3d(b + kBHalf, &tmU, &full[s], chunk * kChunk + 8, n_blk * kOcPerCta, 0);
            };
            issue_tma(0);
            if (c_chunks > 1) issue_tma(1);
            for (int c = 0; c < c_chunks; ++c) {
                const int s = c & 1;
                if (!mbar_wait(&full[s], (c >> 1) & 1, abort_flag, err, ERR_SITE_FULL)) break;
                tc_fence_after();
                const uint32_t a_base = smem_u32(smem + s * kStageBytes);
                const uint32_t b_base = a_base + kABytes;
#pragma unroll
                for (int e = 0; e < kElems; ++e) {
                    const uint64_t ad = make_smem_desc(a_base + e * (kTilesPerCta * 16), kAHalf, 128, Swz::None);
                    const uint64_t bd = make_smem_desc(b_base + e * (kOcPerCta * 16), kBHalf, 128, Swz::None);
                    tc_mma_f16(tmem_base + e * kOcPerCta, ad, bd, kIdesc, c > 0 ? 1u : 0u);
                }
                tc_commit(&empty[s]);
                if (c >= 1 && c + 1 < c_chunks) {
                    // stage of chunk c+1 is free once the MMAs of chunk c-1 are done
                    const int u = (c + 1) >> 1;
                    if (!mbar_wait(&empty[(c + 1) & 1], (u - 1) & 1, abort_flag, err, ERR_SITE_EMPTY)) break;
                    issue_tma(c + 1);
                }
            }
            if (!*abort_flag) tc_commit(tfull);
        }
    } else {
        // ---- producers: one tile row and 8 channels of every chunk per thread
        const int r = tid & 127;
        const int hsel = tid >> 7;
        const int p = m_blk * kTilesPerCta + r;
        const bool pvalid = p < P;
        int n = 0, th = 0, tw = 0;
        if (pvalid) {
            const int tpi = tiles_h * tiles_w;
            n = p / tpi;
            const int rem = p - n * tpi;
            th = rem / tiles_w;
            tw = rem - th * tiles_w;
        }
        const int y0 = th * 2 - pad_h, x0 = tw * 2 - pad_w;
        bool rv[4], cv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            rv[i] = pvalid && (y0 + i >= 0) && (y0 + i < H);
            cv[i] = (x0 + i >= 0) && (x0 + i < W);
        }
        const long long plane = static_cast<long long>(H) * W;
        const __half* img = x + static_cast<long long>(n) * C * plane + static_cast<long long>(y0) * W + x0;

        bool ok = true;
        for (int c = 0; c < c_chunks && ok; ++c) {
            const int s = c & 1;
            if (!mbar_wait(&empty[s], ((c >> 1) & 1) ^ 1, abort_flag, err, ERR_SITE_EMPTY)) {
                ok = false;
                break;
            }
            uint32_t pk[kElems][4];
#pragma unroll
            for (int j2 = 0; j2 < 4; ++j2) {
                float v[2][16];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int ch = c * kChunk + hsel * 8 + j2 * 2 + h;
                    float d[16];
                    const bool chv = ch < C;
                    const __half* src = img + static_cast<long long>(ch) * plane;
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            d[i * 4 + j] = (chv && rv[i] && cv[j]) ? __half2float(src[i * W + j]) : 0.f;
                    input_tile_transform<F2>(d, v[h]);
                }
#pragma unroll
                for (int e = 0; e < kElems; ++e) pk[e][j2] = OpT<BF16>::pack(v[0][e], v[1][e]);
            }
            unsigned char* a = smem + s * kStageBytes + hsel * kAHalf + r * 16;
#pragma unroll
            for (int e = 0; e < kElems; ++e)
                *reinterpret_cast<uint4*>(a + e * (kTilesPerCta * 16)) = make_uint4(pk[e][0], pk[e][1], pk[e][2], pk[e][3]);
            fence_proxy_async_smem();
            mbar_arrive(&full[s]);
        }

        // ---- epilogue: A^T m A from TMEM
        if (ok && mbar_wait(tfull, 0, abort_flag, err, ERR_SITE_TMEM_FULL)) {
            tc_fence_after();
            const int quarter = warp & 3;
            const int chalf = warp >> 2;
            const int row = quarter * 32 + lane;
            const int pe = m_blk * kTilesPerCta + row;
            int en = 0, eth = 0, etw = 0;
            const bool pev = pe < P;
            if (pev) {
                const int tpi = tiles_h * tiles_w;
                en = pe / tpi;
                const int rem = pe - en * tpi;
                eth = rem / tiles_w;
                etw = rem - eth * tiles_w;
            }
            const uint32_t lane_base = tmem_base + (static_cast<uint32_t>(quarter * 32) << 16);
#pragma unroll 1
            for (int g = 0; g < 2; ++g) {
                const int kl0 = chalf * 16 + g * 8;
                float y[8][4];
#pragma unroll
                for (int q = 0; q < 8; ++q) y[q][0] = y[q][1] = y[q][2] = y[q][3] = 0.f;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    uint32_t m[4][8];
#pragma unroll
                    for (int j = 0; j < 4; ++j) tmem_ld_x8(lane_base + (4 * i + j) * kOcPerCta + kl0, m[j]);
                    tc_wait_ld();
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const float m0 = __uint_as_float(m[0][q]), m1 = __uint_as_float(m[1][q]);
                        const float m2 = __uint_as_float(m[2][q]), m3 = __uint_as_float(m[3][q]);
                        const float s0 = m0 + m1 + m2, s1 = m1 - m2 - m3;
                        if (i == 0) { y[q][0] += s0; y[q][1] += s1; }
                        if (i == 1) { y[q][0] += s0; y[q][1] += s1; y[q][2] += s0; y[q][3] += s1; }
                        if (i == 2) { y[q][0] += s0; y[q][1] += s1; y[q][2] -= s0; y[q][3] -= s1; }
                        if (i == 3) { y[q][2] -= s0; y[q][3] -= s1; }
                    }
                }
                if (pev) {
                    const int oh0 = eth * 2, ow0 = etw * 2;
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int k = n_blk * kOcPerCta + kl0 + q;
                        if (k >= K) continue;
                        __half* o = out + (static_cast<long long>(en) * K + k) * OH * static_cast<long long>(OW);
#pragma unroll
                        for (int a = 0; a < 2; ++a) {
                            if (oh0 + a >= OH) continue;
#pragma unroll
                            for (int b = 0; b < 2; ++b)
                                if (ow0 + b < OW)
                                    o[static_cast<long long>(oh0 + a) * OW + ow0 + b] = __float2half_rn(y[q][a * 2 + b]);
                        }
                    }
                }
            }
            tc_fence_before();
        }
    }

    __syncthreads();
    if (*abort_flag) {
        const unsigned long long t0 = globaltimer_ns();
        while (globaltimer_ns() - t0 < 2000000ull) {
        }
    }
    if (warp == 8) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 512);
    }
}

}  // namespace

cudaError_t plan_fused2x3(FusedPlan& fp, OpType op, const Geom& g, const void* U) {
    if (g.m != 2) return cudaErrorInvalidValue;
    fp.op = op;
    fp.m_blocks = static_cast<int>((g.P + kTilesPerCta - 1) / kTilesPerCta);
    fp.n_blocks = (g.k + kOcPerCta - 1) / kOcPerCta;
    fp.c_chunks = (g.c + kChunk - 1) / kChunk;
    fp.smem_bytes = kSmem;
    const CUtensorMapDataType dt = op == OpType::BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    cuuint64_t dims[3] = {static_cast<cuuint64_t>(g.cp), static_cast<cuuint64_t>(g.k), 16};
    cuuint64_t strides[2] = {static_cast<cuuint64_t>(g.cp) * 2, static_cast<cuuint64_t>(g.k) * g.cp * 2};
    cuuint32_t box[3] = {8, kOcPerCta, 16};
    if (encode_tiled(&fp.tmU, dt, 3, const_cast<void*>(U), dims, strides, box, CU_TENSOR_MAP_SWIZZLE_NONE) !=
        CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    return cudaSuccess;
}

cudaError_t launch_fused2x3(const FusedPlan& fp, const Geom& g, const void* x, void* out, DevErr* err,
                            cudaStream_t stream) {
    if (g.P > 0x7fffffffLL) return cudaErrorInvalidValue;
    const long long blocks = static_cast<long long>(fp.m_blocks) * fp.n_blocks;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    auto kern = fp.op == OpType::BF16 ? fused2x3_kernel<true> : fused2x3_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    if (e != cudaSuccess) return e;
    kern<<<static_cast<unsigned>(blocks), kThreads, kSmem, stream>>>(
        static_cast<const __half*>(x), fp.tmU, static_cast<__half*>(out), g.c, g.h, g.w, g.k, g.pad_h, g.pad_w, g.oh,
        g.ow, g.tiles_h, g.tiles_w, static_cast<int>(g.P), fp.c_chunks, fp.n_blocks, err);
    return cudaGetLastError();
}

}  // namespace wg
