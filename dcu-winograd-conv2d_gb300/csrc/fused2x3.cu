// Fully fused F(2x2,3x3): input transform, Winograd-domain GEMM and output
// transform in one kernel; transformed tiles never leave the SM.
//
// This is the reference's winograd_2x3_kernel (src/winograd_2x3_fused.cpp:10-369,
// launcher :372-392) re-designed for tcgen05:
//   * CTA = 128 consecutive output tiles x 32 output channels, looping over the
//     input channels in chunks of 16 (the reference: 32 tiles x 32 channels,
//     chunks of 16, 16 wave64 MMAC GEMMs);
//   * the input rows a chunk needs are staged with cp.async.bulk (one
//     contiguous copy per channel and image), double-buffered one chunk ahead;
//   * warps 0-7 (lanes over consecutive tiles) run B^T d B from shared memory
//     (packed fp16 on channel pairs for fp16 operands, fp32 for bf16) and
//     write the 16 Winograd-domain tiles into shared memory in the tcgen05
//     canonical K-major layout;
//   * the transformed filter U (made once per weight set) arrives by one 4-D
//     TMA per chunk;
//   * warp 8 issues the 16 tcgen05.mma (M=128, N=32, K=16) per chunk from one
//     thread, accumulating all 16 elements in the 512 TMEM columns;
//   * warp 9 issues the staging copies (so no producer warp diverges to
//     wait for the others);
//   * after the last chunk warps 0-7 read TMEM, apply A^T m A and write the
//     2x2 outputs to NCHW.
// Every wait is bounded (wg_ptx.cuh).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "wg_kernels.h"
#include "wg_launch.h"
#include "wg_ptx.cuh"
#include "wg_transforms.cuh"

namespace wg {

namespace {

constexpr int kTilesPerCta = 128;
constexpr int kOcPerCta = 32;
constexpr int kChunk = 16;                               // input channels per stage
constexpr int kElems = 16;                               // 4x4 Winograd elements
constexpr int kAHalf = kElems * kTilesPerCta * 16;       // one granule of every element: 32 KB
constexpr int kABytes = 2 * kAHalf;                      // 64 KB
constexpr int kBBytes = kElems * 2 * kOcPerCta * 16;     // 16 KB: [e][granule][k][8]
constexpr int kStageBytes = kABytes + kBBytes;           // 80 KB
constexpr int kStages = 2;
constexpr int kMaxSeg = 16;                              // images one CTA's tiles may span
constexpr int kProducers = 256;
constexpr int kThreads = kProducers + 64;  // + MMA warp + staging-loader warp
// + 256 bytes after the staging buffers: loads of padding columns (pad <= 64)
// past the last staged row stay inside the CTA's shared memory
constexpr int kSmemFixed = kStages * kStageBytes + 1024 /*align*/ + 512 /*barriers, segment table, zero block*/ + 256;

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

// The caller's element type (fp16, or bf16 for the end-to-end bf16 option).
template <bool IOB> __device__ __forceinline__ float io_load(const __half* p) {
    if constexpr (IOB) return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(p));
    return __half2float(*p);
}
template <bool IOB> __device__ __forceinline__ void io_store1(__half* p, float v) {
    if constexpr (IOB) *reinterpret_cast<__nv_bfloat16*>(p) = __float2bfloat16_rn(v);
    else *p = __float2half_rn(v);
}

struct SegTable {
    int nseg;
    int n_first;
    int ylo[kMaxSeg], yhi[kMaxSeg], off[kMaxSeg];
};

template <bool BF16, bool IOB>
__global__ void __launch_bounds__(kThreads, 1)
    fused2x3_kernel(const __half* __restrict__ x, const __half* __restrict__ x_end,
                    const __grid_constant__ CUtensorMap tmU, __half* __restrict__ out, int C, int H, int W, int K,
                    int pad_h, int pad_w, int OH, int OW, int tiles_h, int tiles_w, int P, int c_chunks, int n_blocks,
                    int stg_ch_bytes, int nbuf, DevErr* err) {
    constexpr uint32_t kIdesc = make_idesc_f16(128, kOcPerCta, BF16);
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned base by pointer arithmetic (an integer round trip would
    // hide that this is shared memory and turn every access generic)
    unsigned char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes);
    uint64_t* full = bars;             // [2] producers (256) + TMA expect_tx (1)
    uint64_t* empty = bars + 2;        // [2] MMA commit
    uint64_t* tfull = bars + 4;        // accumulators of the current item ready
    uint64_t* sfull = bars + 5;        // [2] staging copies landed
    uint64_t* sempty = bars + 7;       // [2] staging buffer read by all producers
    uint64_t* tempty = bars + 9;       // accumulators drained by the epilogue (256 arrivals)
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 10);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    SegTable* segs = reinterpret_cast<SegTable*>(bars + 11);  // [2], by item parity
    static_assert(11 * 8 + 2 * sizeof(SegTable) <= 496, "barrier area");
    unsigned char* stg = smem + kStages * kStageBytes + 512;  // nbuf x 16 channels x stg_ch_bytes
    unsigned char* zero = smem + kStages * kStageBytes + 496;  // 16 zero bytes: a padding row

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tpi = tiles_h * tiles_w;
    const long long plane = static_cast<long long>(H) * W;
    const uintptr_t lim = reinterpret_cast<uintptr_t>(x_end) & ~uintptr_t(15);
    // persistent CTA: work items (tile block, 32-channel block) blockIdx.x,
    // blockIdx.x + gridDim.x, ...; the output-channel block runs fastest so
    // CTAs working at the same time read the same input rows (L2)
    const int m_blocks = (P + kTilesPerCta - 1) / kTilesPerCta;
    const int total_items = m_blocks * n_blocks;
    const int my_items = blockIdx.x < total_items ? (total_items - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int total_chunks = my_items * c_chunks;

    if (tid == 0) {
        for (int i = 0; i < kStages; ++i) {
            mbar_init(&full[i], kProducers + 1);
            mbar_init(&empty[i], 1);
            mbar_init(&sfull[i], kChunk);  // one arrival per staged channel (loader lanes)
            mbar_init(&sempty[i], kProducers);
        }
        mbar_init(tfull, 1);
        mbar_init(tempty, kProducers);
        *abort_flag = 0;
        *reinterpret_cast<uint4*>(zero) = make_uint4(0u, 0u, 0u, 0u);
        fence_barrier_init();
    }
    pdl_wait();     // input written, earlier readers of the output done
    pdl_trigger();
    if (warp == 8) tmem_alloc(tmem_slot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    // images covered by an item's 128 tiles and the input rows each needs
    auto make_seg = [&](int item, SegTable* sg) {
        const int p_first = (item / n_blocks) * kTilesPerCta;
        const int p_last = min(P, p_first + kTilesPerCta) - 1;
        const int na = p_first / tpi, nb = p_last / tpi;
        int nseg = nb - na + 1;
        if (nseg > kMaxSeg) {  // host sizing guarantees this never happens
            record_error(err, ERR_SITE_CONFIG);
            *abort_flag = 1;
            nseg = kMaxSeg;
        }
        sg->nseg = nseg;
        sg->n_first = na;
        int off = 0;
        for (int q = 0; q < nseg; ++q) {
            const int n = na + q;
            const int pa = max(p_first, n * tpi) - n * tpi, pb = min(p_last, n * tpi + tpi - 1) - n * tpi;
            const int tha = pa / tiles_w, thb = pb / tiles_w;
            const int ylo = max(0, tha * 2 - pad_h), yhi = min(H, thb * 2 - pad_h + 4);
            sg->ylo[q] = ylo;
            sg->yhi[q] = max(ylo, yhi);
            sg->off[q] = off;
            off += (max(0, yhi - ylo) * W * 2 + 16 + 15) / 16 * 16;
        }
    };

    // staging of chunk gc (the CTA's running chunk count: item gc / c_chunks,
    // 16 channels from (gc % c_chunks) * 16) into buffer gc % nbuf: loader
    // lane j copies channel j's rows of every image segment and accounts its
    // own bytes on the barrier (16 arrivals complete the phase).  Lane 0
    // writes the item's segment table before its first chunk.
    auto issue_stage = [&](int gc, int j) {
        const int k = gc / c_chunks, c = gc - k * c_chunks;
        SegTable* sg = &segs[k & 1];
        if (c == 0) {
            if (j == 0) make_seg(blockIdx.x + k * gridDim.x, sg);
            __syncwarp(0xffffu);
        }
        const int bsel = gc % nbuf;
        unsigned char* buf = stg + bsel * (kChunk * stg_ch_bytes) + j * stg_ch_bytes;
        const int ch = c * kChunk + j;
        uint32_t total = 0;
        uintptr_t a16s[kMaxSeg];
        uint32_t lens[kMaxSeg];
        const int nseg = sg->nseg;
        for (int q = 0; q < nseg; ++q) {
            lens[q] = 0;
            const int rows = sg->yhi[q] - sg->ylo[q];
            if (ch >= C || rows <= 0) continue;
            const uintptr_t a = reinterpret_cast<uintptr_t>(
                x + (static_cast<long long>(sg->n_first + q) * C + ch) * plane + static_cast<long long>(sg->ylo[q]) * W);
            const uintptr_t a16 = a & ~uintptr_t(15);
            const uintptr_t b16 = min_uptr((a + static_cast<uintptr_t>(rows) * W * 2 + 15) & ~uintptr_t(15), lim);
            if (b16 <= a16) continue;
            a16s[q] = a16;
            lens[q] = static_cast<uint32_t>(b16 - a16);
            total += lens[q];
        }
        mbar_arrive_expect_tx(&sfull[bsel], total);
        for (int q = 0; q < nseg; ++q)
            if (lens[q]) bulk_g2s(buf + sg->off[q], reinterpret_cast<const void*>(a16s[q]), lens[q], &sfull[bsel]);
    };

    if (warp == 9) {
        if (lane < kChunk) {
            for (int gc = 0; gc < nbuf && gc < total_chunks; ++gc) issue_stage(gc, lane);
            for (int gc = 0; gc + nbuf < total_chunks; ++gc) {
                // buffer gc % nbuf is free once every producer has read chunk gc
                if (!mbar_wait(&sempty[gc % nbuf], (gc / nbuf) & 1, abort_flag, err, ERR_SITE_EMPTY)) break;
                issue_stage(gc + nbuf, lane);
            }
        }
    } else if (warp == 8) {
        if (lane == 0) {
            tma_prefetch_desc(&tmU);
            auto issue_tma = [&](int gc) {
                const int k = gc / c_chunks, c = gc - k * c_chunks;
                const int n_blk = (blockIdx.x + k * gridDim.x) % n_blocks;
                const int s = gc & 1;
                mbar_arrive_expect_tx(&full[s], kBBytes);
                tma_load_4d(smem + s * kStageBytes + kABytes, &tmU, &full[s], 0, n_blk * (kOcPerCta / 8), c * 2, 0);
            };
            if (total_chunks > 0) issue_tma(0);
            if (total_chunks > 1) issue_tma(1);
            bool ok = true;
            for (int k = 0; k < my_items && ok; ++k) {
                // the previous item's accumulators must be drained first
                if (!mbar_wait(tempty, (k & 1) ^ 1, abort_flag, err, ERR_SITE_TMEM_EMPTY)) break;
                tc_fence_after();
                for (int c = 0; c < c_chunks; ++c) {
                    const int gc = k * c_chunks + c;
                    const int s = gc & 1;
                    if (!mbar_wait(&full[s], (gc >> 1) & 1, abort_flag, err, ERR_SITE_FULL)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a_base = smem_u32(smem + s * kStageBytes);
                    const uint32_t b_base = a_base + kABytes;
#pragma unroll
                    for (int e = 0; e < kElems; ++e) {
                        const uint64_t ad = make_smem_desc(a_base + e * (kTilesPerCta * 16), kAHalf, 128, Swz::None);
                        const uint64_t bd =
                            make_smem_desc(b_base + e * (2 * kOcPerCta * 16), kOcPerCta * 16, 128, Swz::None);
                        tc_mma_f16(tmem_base + e * kOcPerCta, ad, bd, kIdesc, c > 0 ? 1u : 0u);
                    }
                    tc_commit(&empty[s]);
                    if (gc + 2 < total_chunks) {
                        // the filter tile of chunk gc+2 reuses this stage: issue it
                        // as soon as these MMAs retire, a whole chunk ahead of its use
                        if (!mbar_wait(&empty[s], (gc >> 1) & 1, abort_flag, err, ERR_SITE_EMPTY)) {
                            ok = false;
                            break;
                        }
                        issue_tma(gc + 2);
                    }
                }
                if (ok && !*abort_flag) tc_commit(tfull);
            }
        }
    } else {
        // ---- producers: one tile and 8 channels of every chunk per thread,
        //      lanes over consecutive tiles; then the item's epilogue
        const int r = tid & 127;
        const int hsel = tid >> 7;
        bool ok = true;
        for (int k = 0; k < my_items && ok; ++k) {
            const int item = blockIdx.x + k * gridDim.x;
            const int n_blk = item % n_blocks;
            const int p_first = (item / n_blocks) * kTilesPerCta;
            const int p = p_first + r;
            const bool pvalid = p < P;
            int n = 0, th = 0, tw = 0;
            if (pvalid) {
                n = p / tpi;
                const int rem = p - n * tpi;
                th = rem / tiles_w;
                tw = rem - th * tiles_w;
            }
            int ylo = 0, yhi = 0, soff = 0;
            const int y0 = th * 2 - pad_h, x0 = tw * 2 - pad_w;
            bool rv[4], cv[4];
            uint32_t sel[4];
            long long row0 = 0;
            for (int c = 0; c < c_chunks; ++c) {
                const int gc = k * c_chunks + c;
                const int s = gc & 1;
                const int bsel = gc % nbuf;
                const uint32_t bpar = (gc / nbuf) & 1;
                if (!mbar_wait(&sfull[bsel], bpar, abort_flag, err, ERR_SITE_FULL)) {
                    ok = false;
                    break;
                }
                if (c == 0) {
                    // the item's segment table arrived with its first chunk
                    const SegTable* sg = &segs[k & 1];
                    const int s_idx = pvalid ? n - sg->n_first : 0;
                    ylo = sg->ylo[s_idx];
                    yhi = sg->yhi[s_idx];
                    soff = sg->off[s_idx];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        rv[i] = pvalid && (y0 + i >= ylo) && (y0 + i < yhi);
                        cv[i] = (x0 + i >= 0) && (x0 + i < W);
                        sel[i] = cv[i] ? 0x5410u : 0x3232u;
                    }
                    row0 = static_cast<long long>(y0 - ylo) * W + x0;  // patch origin within the staged rows
                }
                const unsigned char* buf = stg + bsel * (kChunk * stg_ch_bytes);
                uint32_t pk[kElems][4];
#pragma unroll
                for (int j2 = 0; j2 < 4; ++j2) {
                    if constexpr (!BF16) {
                        // fp16 operands: the channel pair (jl, jl+1) is transformed
                        // in packed fp16 (the F(2x3) B^T has only +-1 entries, so
                        // this is two roundings of sums instead of one; the
                        // reference's transforms are fp16 as well).  Padding rows
                        // and channels past C read a zero block; padding columns
                        // take the zero upper half of the 16-bit loads through the
                        // byte-permute selector.
                        const int jl = hsel * 8 + j2 * 2;
                        const int ch = c * kChunk + jl;
                        const bool v0 = ch < C, v1 = ch + 1 < C;
                        const uintptr_t a0 = reinterpret_cast<uintptr_t>(
                            x + (static_cast<long long>(n) * C + ch) * plane + static_cast<long long>(ylo) * W);
                        const uintptr_t a1 = a0 + static_cast<uintptr_t>(plane) * 2;
                        const uintptr_t rb = static_cast<uintptr_t>(yhi - ylo) * W * 2;
                        if ((!v0 || a0 + rb <= lim) && (!v1 || a1 + rb <= lim)) {
                            const __half* b0 =
                                reinterpret_cast<const __half*>(buf + jl * stg_ch_bytes + soff + (a0 & 15)) + row0;
                            const __half* b1 =
                                reinterpret_cast<const __half*>(buf + (jl + 1) * stg_ch_bytes + soff + (a1 & 15)) + row0;
                            __half2 t[4][4];
#pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const uint16_t* r0 =
                                    reinterpret_cast<const uint16_t*>(rv[i] && v0 ? b0 + i * W : reinterpret_cast<const __half*>(zero));
                                const uint16_t* r1 =
                                    reinterpret_cast<const uint16_t*>(rv[i] && v1 ? b1 + i * W : reinterpret_cast<const __half*>(zero));
#pragma unroll
                                for (int j = 0; j < 4; ++j) {
                                    const uint32_t h = __byte_perm(r0[j], r1[j], sel[j]);
                                    t[i][j] = *reinterpret_cast<const __half2*>(&h);
                                }
                            }
                            // columns: B^T d
#pragma unroll
                            for (int j = 0; j < 4; ++j) {
                                const __half2 d0 = t[0][j], d1 = t[1][j], d2 = t[2][j], d3 = t[3][j];
                                t[0][j] = __hsub2(d0, d2);
                                t[1][j] = __hadd2(d1, d2);
                                t[2][j] = __hsub2(d2, d1);
                                t[3][j] = __hsub2(d1, d3);
                            }
                            // rows: (B^T d) B
#pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const __half2 q0 = t[i][0], q1 = t[i][1], q2 = t[i][2], q3 = t[i][3];
                                const __half2 o[4] = {__hsub2(q0, q2), __hadd2(q1, q2), __hsub2(q2, q1), __hsub2(q1, q3)};
#pragma unroll
                                for (int j = 0; j < 4; ++j) pk[i * 4 + j][j2] = *reinterpret_cast<const uint32_t*>(&o[j]);
                            }
                            continue;
                        }
                    }
                    float v[2][16];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int jl = hsel * 8 + j2 * 2 + h;
                        const int ch = c * kChunk + jl;
                        const bool chv = ch < C;
                        const __half* gsrc = x + (static_cast<long long>(n) * C + ch) * plane;
                        const uintptr_t a = reinterpret_cast<uintptr_t>(gsrc + static_cast<long long>(ylo) * W);
                        // rows staged whole unless they run into the input's last
                        // partial 16-byte block (then read from global memory)
                        const bool staged = a + static_cast<uintptr_t>(yhi - ylo) * W * 2 <= lim;
                        float d[16];
                        // staged rows through shared-memory loads; the rare rows
                        // that run into the input's last partial 16-byte block
                        // through global loads (separate code, not one pointer)
                        if (staged) {
                            const __half* src =
                                reinterpret_cast<const __half*>(buf + jl * stg_ch_bytes + soff + (a & 15)) + row0;
#pragma unroll
                            for (int i = 0; i < 4; ++i)
#pragma unroll
                                for (int j = 0; j < 4; ++j)
                                    d[i * 4 + j] = (chv && rv[i] && cv[j]) ? io_load<IOB>(src + i * W + j) : 0.f;
                        } else {
                            const __half* src = gsrc + static_cast<long long>(ylo) * W + row0;
#pragma unroll
                            for (int i = 0; i < 4; ++i)
#pragma unroll
                                for (int j = 0; j < 4; ++j)
                                    d[i * 4 + j] = (chv && rv[i] && cv[j]) ? io_load<IOB>(src + i * W + j) : 0.f;
                        }
                        input_tile_transform<F2>(d, v[h]);
                    }
#pragma unroll
                    for (int e = 0; e < kElems; ++e) pk[e][j2] = OpT<BF16>::pack(v[0][e], v[1][e]);
                }
                mbar_arrive(&sempty[bsel]);  // this thread is done reading the staged rows
                if (!mbar_wait(&empty[s], ((gc >> 1) & 1) ^ 1, abort_flag, err, ERR_SITE_EMPTY)) {
                    ok = false;
                    break;
                }
                unsigned char* a = smem + s * kStageBytes + hsel * kAHalf + r * 16;
#pragma unroll
                for (int e = 0; e < kElems; ++e)
                    *reinterpret_cast<uint4*>(a + e * (kTilesPerCta * 16)) =
                        make_uint4(pk[e][0], pk[e][1], pk[e][2], pk[e][3]);
                fence_proxy_async_smem();
                mbar_arrive(&full[s]);
            }
            if (!ok) break;

            // ---- epilogue: A^T m A from TMEM
            if (!mbar_wait(tfull, k & 1, abort_flag, err, ERR_SITE_TMEM_FULL)) break;
            tc_fence_after();
            const int quarter = warp & 3;
            const int chalf = warp >> 2;
            const int row = quarter * 32 + lane;
            const int pe = p_first + row;
            int en = 0, eth = 0, etw = 0;
            const bool pev = pe < P;
            if (pev) {
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
                            __half* dst = o + static_cast<long long>(oh0 + a) * OW + ow0;
                            if (ow0 + 1 < OW && (reinterpret_cast<uintptr_t>(dst) & 3) == 0) {
                                *reinterpret_cast<uint32_t*>(dst) = OpT<IOB>::pack(y[q][a * 2], y[q][a * 2 + 1]);
                            } else {
                                io_store1<IOB>(dst, y[q][a * 2]);
                                if (ow0 + 1 < OW) io_store1<IOB>(dst + 1, y[q][a * 2 + 1]);
                            }
                        }
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(tempty);
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

// Bytes of staged input per channel: the largest over all CTAs of the sum,
// over the images its 128 tiles touch, of the rows those tiles need.
int staging_bytes_per_channel(const Geom& g, int* max_segments) {
    const int tpi = g.tiles_h * g.tiles_w;
    const long long blocks = (g.P + kTilesPerCta - 1) / kTilesPerCta;
    long long best = 0;
    int segs = 0;
    // the pattern repeats every tpi tiles; one period of block starts suffices
    const long long lim = std::min<long long>(blocks, static_cast<long long>(tpi) + 1);
    for (long long b = 0; b < lim; ++b) {
        const long long pf = b * kTilesPerCta, pl = std::min<long long>(g.P, pf + kTilesPerCta) - 1;
        const long long na = pf / tpi, nb = pl / tpi;
        long long bytes = 0;
        for (long long n = na; n <= nb; ++n) {
            const long long pa = std::max(pf, n * tpi) - n * tpi, pb = std::min(pl, n * tpi + tpi - 1) - n * tpi;
            const int tha = static_cast<int>(pa / g.tiles_w), thb = static_cast<int>(pb / g.tiles_w);
            const int ylo = std::max(0, tha * 2 - g.pad_h), yhi = std::min(g.h, thb * 2 - g.pad_h + 4);
            bytes += (std::max(0, yhi - ylo) * 2LL * g.w + 16 + 15) / 16 * 16;
        }
        best = std::max(best, bytes);
        segs = std::max(segs, static_cast<int>(nb - na + 1));
    }
    *max_segments = segs;
    return static_cast<int>(std::min<long long>(best, 1 << 30));
}

}  // namespace

cudaError_t plan_fused2x3(FusedPlan& fp, OpType op, const Geom& g, const void* U) {
    if (g.m != 2) return cudaErrorInvalidValue;
    fp.io_bf16 = false;
    int segs = 0;
    fp.stg_ch_bytes = staging_bytes_per_channel(g, &segs);
    // two staging buffers when they fit (copies run a chunk ahead), else one
    fp.nbuf = 2;
    fp.smem_bytes = kSmemFixed + fp.nbuf * kChunk * fp.stg_ch_bytes;
    if (fp.smem_bytes > 227 * 1024) {
        fp.nbuf = 1;
        fp.smem_bytes = kSmemFixed + kChunk * fp.stg_ch_bytes;
    }
    if (segs > kMaxSeg || fp.smem_bytes > 227 * 1024) return cudaErrorNotSupported;
    fp.op = op;
    fp.m_blocks = static_cast<int>((g.P + kTilesPerCta - 1) / kTilesPerCta);
    fp.n_blocks = (g.k + kOcPerCta - 1) / kOcPerCta;
    fp.c_chunks = (g.c + kChunk - 1) / kChunk;
    const CUtensorMapDataType dt = op == OpType::BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    // U[16][CG][Kp][8] viewed as 128-byte rows of 8 output channels: a box of
    // 4 rows (32 output channels) x 2 granules x 16 elements per chunk
    const cuuint64_t CG = static_cast<cuuint64_t>(g.cp / 8);
    const cuuint64_t Kr = static_cast<cuuint64_t>(g.kp / 8);
    cuuint64_t dims[4] = {64, Kr, CG, 16};
    cuuint64_t strides[3] = {128, Kr * 128, CG * Kr * 128};
    cuuint32_t box[4] = {64, kOcPerCta / 8, 2, 16};
    if (encode_tiled(&fp.tmU, dt, 4, const_cast<void*>(U), dims, strides, box, CU_TENSOR_MAP_SWIZZLE_NONE) !=
        CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    return cudaSuccess;
}

cudaError_t launch_fused2x3(const FusedPlan& fp, const Geom& g, const void* x, const void* x_end, void* out,
                            DevErr* err, cudaStream_t stream) {
    if (g.P > 0x7fffffffLL) return cudaErrorInvalidValue;
    // work items of this launch (a launch may cover a subset of the images),
    // one persistent CTA per SM
    const long long items = (g.P + kTilesPerCta - 1) / kTilesPerCta * fp.n_blocks;
    if (items > 0x7fffffffLL) return cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0)
        sms = 148;
    const long long blocks = std::min<long long>(items, sms);
    // bf16 tensors run with bf16 operands
    if (fp.io_bf16 && fp.op != OpType::BF16) return cudaErrorNotSupported;
    auto kern = fp.io_bf16 ? fused2x3_kernel<true, true>
                           : (fp.op == OpType::BF16 ? fused2x3_kernel<true, false> : fused2x3_kernel<false, false>);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, fp.smem_bytes);
    if (e != cudaSuccess) return e;
    return launch_pdl(kern, dim3(static_cast<unsigned>(blocks)), dim3(kThreads), fp.smem_bytes, stream,
                      static_cast<const __half*>(x), static_cast<const __half*>(x_end), fp.tmU, static_cast<__half*>(out),
                      g.c, g.h, g.w, g.k, g.pad_h, g.pad_w, g.oh, g.ow, g.tiles_h, g.tiles_w, static_cast<int>(g.P),
                      fp.c_chunks, fp.n_blocks, fp.stg_ch_bytes, fp.nbuf, err);
}

}  // namespace wg
