// Row-Winograd F(4x3), fully fused: the 1-D Winograd transform F(4,3) along
// the image width (points 0, +-1, 1/2, -2, as in the F(4x3) path) and the
// direct 3-tap sum along the height, in one kernel.
//
// A "tile" is 4 consecutive outputs of one output row.  For output row i and
// tile tw the result is
//     y[i][4tw + j] = sum_e AT[j][e] sum_r sum_c U[e][r][k][c] * V[e][row i + r][tw][c]
// where V[e][rho][tw][c] = (B^T d)[e] of the 6 input values of input row rho,
// columns 4tw - pad .. 4tw - pad + 5, and U[e][r] = G w[k][c][r][.].  So each
// of the 6 elements is a GEMM over K = 3C (filter row x channel): the three
// filter rows use the SAME transformed input rows shifted by one row of tiles,
// which in the tcgen05 canonical layout is only a different start address of
// the A operand.  Nothing is recomputed per filter row, and the 1-D output
// transform runs on the accumulators in the epilogue, so neither V nor M
// touches HBM.
//
// CTA work item = (image, block of R output rows, 64 output channels), with
// R * tiles_w <= 128 (the MMA M dimension).  Per 16-channel chunk:
//   * warp 17 stages the R+2 input rows of the chunk's channels (cp.async.bulk,
//     one copy per channel, double-buffered a chunk ahead);
//   * warps 0-15 compute V for the (R+2) x tiles_w tiles x 16 channels (channel
//     pairs in packed fp16, the precision V is stored in) into the canonical
//     K-major layout;
//   * warp 16 loads the chunk's filter tile (one 4-D TMA: 6 elements x 3 rows
//     x 64 channels x 16 input channels) and issues 18 tcgen05.mma (M=128,
//     N=64, K=16), accumulating element e in TMEM columns [64e, 64e + 64);
//   * after the last chunk warps 0-15 read the 6 accumulators, apply A^T and
//     store 4-wide output rows.
// Shared-memory bandwidth bounds this kernel: every MMA reads its 4 KB A tile
// and 2 KB B tile (N = 64, as 6 accumulators of 64 columns fill TMEM).
// Persistent CTAs walk the items; every wait is bounded (wg_ptx.cuh).
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "wg_kernels.h"
#include "wg_launch.h"
#include "wg_ptx.cuh"
#include "wg_transforms.cuh"

namespace wg {

namespace {

constexpr int kE = 6, kTaps = 3;
constexpr int kBN = 64;                                  // output channels per item
constexpr int kChunk = 16;                               // input channels per stage
constexpr int kBBytes = kE * kTaps * 2 * kBN * 16;       // 36 KB: [e*3+r][granule][k][8]
constexpr int kAStages = 2;                              // transformed input (A) ring
constexpr int kMaxBStages = 4, kMaxBufs = 4;             // filter-tile ring, staging ring
constexpr int kProducers = 512;                          // 16 warps: transform, then epilogue
constexpr int kThreads = kProducers + 96;                // + MMA, staging-loader and filter-TMA warps
constexpr int kMmaWarp = kProducers / 32, kLoaderWarp = kMmaWarp + 1, kBWarp = kMmaWarp + 2;
constexpr int kTasksPerThread = 4;                       // (128 + 2 * 64) rows x 8 pairs / 512
constexpr int kHdr = 512;                                // barriers
constexpr int kSlack = 256;                              // padding-column loads past the staged rows

__device__ __forceinline__ __half2 h2c(float a) { return __float2half2_rn(a); }

// B^T d of F(4,3), points 0, +-1, 1/2, -2 (the rows of F4::bt), two channels
// per value
__device__ __forceinline__ void bt6(const __half2 (&d)[6], __half2 (&o)[6]) {
    const __half2 t = __hsub2(d[3], d[1]), u = __hsub2(d[4], d[2]);
    o[0] = __hadd2(__hfma2(d[2], h2c(-2.f), __hfma2(t, h2c(1.5f), d[0])), d[4]);
    o[1] = __hsub2(__hfma2(d[3], h2c(2.5f), __hfma2(d[2], h2c(0.5f), d[4])), d[1]);
    o[2] = __hadd2(__hfma2(d[2], h2c(-2.5f), __hfma2(d[3], h2c(0.5f), d[4])), d[1]);
    o[3] = __hfma2(t, h2c(2.f), u);
    o[4] = __hfma2(t, h2c(-0.5f), u);
    o[5] = __hadd2(__hfma2(d[3], h2c(-2.f), __hfma2(u, h2c(1.5f), d[1])), d[5]);
}

struct RowGeo {     // shared by host and device
    int C, H, W, K, pad_h, pad_w, OH, OW, tiles_w;
    int R, row_blocks, n_blocks, c_chunks;
    int stg_ch;     // staged bytes per channel
    int nbuf;       // staging buffers
    int nbs;        // filter-tile stages
    // rows of one A granule: 128 MMA rows plus two rows of tiles of shift,
    // 4 mod 8 so the two granules of a warp's stores sit 64 bytes apart in
    // the bank space and do not conflict
    int arows;
};

__global__ void __launch_bounds__(kThreads, 1)
    row4x3_kernel(const __half* __restrict__ x, const __half* __restrict__ x_end, const __grid_constant__ CUtensorMap tmU,
                  __half* __restrict__ out, const __grid_constant__ RowGeo gg, int n_images, DevErr* err) {
    constexpr uint32_t kIdesc = make_idesc_f16(128, kBN, false);
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int a_gran = gg.arows * 16;              // bytes of one granule of one element
    const int a_bytes = kE * 2 * a_gran;           // one A stage
    const int nbs = gg.nbs;
    // smem: B stages (1024-aligned) | A stages | barriers | staging buffers
    unsigned char* bstage = smem;
    unsigned char* astage = smem + nbs * kBBytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(astage + kAStages * a_bytes);
    uint64_t* afull = bars;                        // [2] producers
    uint64_t* aempty = bars + 2;                   // [2] MMA commit
    uint64_t* bfull = bars + 4;                    // [4] filter TMA (expect_tx)
    uint64_t* bempty = bars + 8;                   // [4] MMA commit
    uint64_t* sfull = bars + 12;                   // [4] staging copies landed
    uint64_t* sempty = bars + 16;                  // [4] staging buffer read by all producers
    uint64_t* tfull = bars + 20;                   // accumulators of the current item ready
    uint64_t* tempty = bars + 21;                  // accumulators drained
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 22);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    unsigned char* stg = reinterpret_cast<unsigned char*>(bars) + kHdr;   // nbuf x 16 channels x stg_ch

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int C = gg.C, H = gg.H, W = gg.W, K = gg.K, R = gg.R, tiles_w = gg.tiles_w;
    const int c_chunks = gg.c_chunks, nbuf = gg.nbuf, stg_ch = gg.stg_ch;
    const long long plane = static_cast<long long>(H) * W;
    const uintptr_t lim = reinterpret_cast<uintptr_t>(x_end) & ~uintptr_t(15);
    const int total_items = n_images * gg.row_blocks * gg.n_blocks;
    const int my_items = blockIdx.x < total_items ? (total_items - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int total_chunks = my_items * c_chunks;

    if (tid == 0) {
        for (int i = 0; i < kAStages; ++i) {
            mbar_init(&afull[i], kProducers);
            mbar_init(&aempty[i], 1);
        }
        for (int i = 0; i < kMaxBStages; ++i) {
            mbar_init(&bfull[i], 1);
            mbar_init(&bempty[i], 1);
        }
        for (int i = 0; i < kMaxBufs; ++i) {
            mbar_init(&sfull[i], kChunk);
            mbar_init(&sempty[i], kProducers);
        }
        mbar_init(tfull, 1);
        mbar_init(tempty, kProducers);
        *abort_flag = 0;
        fence_barrier_init();
    }
    pdl_wait();     // input written, earlier readers of the output done
    pdl_trigger();
    if (warp == kMmaWarp) tmem_alloc(tmem_slot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    // item -> (image, first output row, output-channel block); the channel
    // block runs fastest so CTAs working together read the same input rows
    auto item_of = [&](int k, int& n, int& oh0, int& nb) {
        const int item = blockIdx.x + k * gridDim.x;
        nb = item % gg.n_blocks;
        const int rest = item / gg.n_blocks;
        oh0 = (rest % gg.row_blocks) * R;
        n = rest / gg.row_blocks;
    };
    // staged input rows of an item: [ylo, yhi) of the image, all columns
    auto rows_of = [&](int oh0, int& ylo, int& yhi) {
        ylo = max(0, oh0 - gg.pad_h);
        yhi = min(H, oh0 - gg.pad_h + R + kTaps - 1);
        yhi = max(ylo, yhi);
    };

    if (warp == kLoaderWarp) {
        // staging: lane j copies channel j of the chunk; the bytes after the
        // input's last 16-byte boundary are copied with plain loads, and the
        // buffer of a channel past C is zero-filled, before the arrival (whose
        // release orders them before the producers' reads)
        if (lane < kChunk) {
            auto issue = [&](int gc) {
                const int k = gc / c_chunks, c = gc - k * c_chunks;
                int n, oh0, nb;
                item_of(k, n, oh0, nb);
                int ylo, yhi;
                rows_of(oh0, ylo, yhi);
                const int bsel = gc % nbuf;
                unsigned char* dst = stg + bsel * (kChunk * stg_ch) + lane * stg_ch;
                const int ch = c * kChunk + lane;
                uint32_t bytes = 0;
                uintptr_t a16 = 0;
                if (ch >= C) {
                    for (int o = 0; o < stg_ch; o += 16) *reinterpret_cast<uint4*>(dst + o) = make_uint4(0u, 0u, 0u, 0u);
                } else if (yhi > ylo) {
                    const uintptr_t a = reinterpret_cast<uintptr_t>(x + (static_cast<long long>(n) * C + ch) * plane +
                                                                    static_cast<long long>(ylo) * W);
                    const uintptr_t b = a + static_cast<uintptr_t>(yhi - ylo) * W * 2;
                    a16 = a & ~uintptr_t(15);
                    const uintptr_t b16 = min_uptr((b + 15) & ~uintptr_t(15), lim);
                    if (b16 > a16) bytes = static_cast<uint32_t>(b16 - a16);
                    for (uintptr_t q = (b16 > a16 ? b16 : a16); q < b; q += 2)
                        *reinterpret_cast<uint16_t*>(dst + (q - a16)) = *reinterpret_cast<const uint16_t*>(q);
                }
                if (bytes) fence_proxy_async_smem();
                mbar_arrive_expect_tx(&sfull[bsel], bytes);
                if (bytes) bulk_g2s(dst, reinterpret_cast<const void*>(a16), bytes, &sfull[bsel]);
            };
            for (int gc = 0; gc < nbuf && gc < total_chunks; ++gc) issue(gc);
            for (int gc = 0; gc + nbuf < total_chunks; ++gc) {
                if (!mbar_wait(&sempty[gc % nbuf], (gc / nbuf) & 1, abort_flag, err, ERR_SITE_EMPTY)) break;
                issue(gc + nbuf);
            }
        }
    } else if (warp == kBWarp) {
        // filter tiles: one 4-D TMA per chunk, nbs chunks ahead of the MMAs
        if (lane == 0) {
            tma_prefetch_desc(&tmU);
            for (int gc = 0; gc < total_chunks; ++gc) {
                const int sb = gc % nbs;
                if (gc >= nbs && !mbar_wait(&bempty[sb], ((gc / nbs) & 1) ^ 1, abort_flag, err, ERR_SITE_EMPTY)) break;
                const int k = gc / c_chunks, c = gc - k * c_chunks;
                int n, oh0, nb;
                item_of(k, n, oh0, nb);
                mbar_arrive_expect_tx(&bfull[sb], kBBytes);
                tma_load_4d(bstage + sb * kBBytes, &tmU, &bfull[sb], 0, nb * (kBN / 8), c * 2, 0);
            }
        }
    } else if (warp == kMmaWarp) {
        // one thread issues the MMAs and never waits on their completion
        if (lane == 0) {
            bool ok = true;
            for (int k = 0; k < my_items && ok; ++k) {
                if (!mbar_wait(tempty, (k & 1) ^ 1, abort_flag, err, ERR_SITE_TMEM_EMPTY)) break;
                tc_fence_after();
                for (int c = 0; c < c_chunks; ++c) {
                    const int gc = k * c_chunks + c;
                    const int sa = gc & 1, sb = gc % nbs;
                    if (!mbar_wait(&afull[sa], (gc >> 1) & 1, abort_flag, err, ERR_SITE_FULL) ||
                        !mbar_wait(&bfull[sb], (gc / nbs) & 1, abort_flag, err, ERR_SITE_FULL)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a_base = smem_u32(astage + sa * a_bytes);
                    const uint32_t b_base = smem_u32(bstage + sb * kBBytes);
#pragma unroll
                    for (int e = 0; e < kE; ++e) {
#pragma unroll
                        for (int r = 0; r < kTaps; ++r) {
                            // filter row r reads the transformed rows shifted by r rows of tiles
                            const uint64_t ad =
                                make_smem_desc(a_base + e * (2 * a_gran) + r * tiles_w * 16, a_gran, 128, Swz::None);
                            const uint64_t bd = make_smem_desc(b_base + (e * kTaps + r) * (2 * kBN * 16), kBN * 16, 128,
                                                               Swz::None);
                            tc_mma_f16(tmem_base + e * kBN, ad, bd, kIdesc, (c > 0 || r > 0) ? 1u : 0u);
                        }
                    }
                    tc_commit(&aempty[sa]);
                    tc_commit(&bempty[sb]);
                }
                if (ok && !*abort_flag) tc_commit(tfull);
            }
        }
    } else {
        // ---- producers: V of (R+2) x tiles_w tiles x 16 channels per chunk.
        //      Task = (row of tiles, channel pair), pairs fastest; a thread's
        //      pair is fixed (tid & 7) and its rows are tid/8 + 64 i.
        const int pr = tid & 7;
        const int nrt = (R + kTaps - 1) * tiles_w;   // transformed rows of tiles
        // element phase of x inside its 16-byte granule (x is 2-byte aligned)
        const uint32_t xph = static_cast<uint32_t>((reinterpret_cast<uintptr_t>(x) >> 1) & 7u);
        bool ok = true;
        for (int k = 0; k < my_items && ok; ++k) {
            int n, oh0, nb;
            item_of(k, n, oh0, nb);
            int ylo, yhi;
            rows_of(oh0, ylo, yhi);
            // per task: element offset of its first input in the channel's
            // staged rows, the valid inputs (bit j: column x0 + j inside the
            // image, 0 for padding rows), the byte offset of its V row
            int soff[kTasksPerThread];
            uint32_t vmask[kTasksPerThread], doff[kTasksPerThread];
#pragma unroll
            for (int i = 0; i < kTasksPerThread; ++i) {
                const int row = (tid >> 3) + i * (kProducers / 8);
                const int rho = row / tiles_w, tw = row - rho * tiles_w;
                const int y = oh0 - gg.pad_h + rho, x0 = tw * 4 - gg.pad_w;
                const bool rok = row < nrt && y >= ylo && y < yhi;
                uint32_t m = 0;
#pragma unroll
                for (int j = 0; j < 6; ++j) m |= (x0 + j >= 0 && x0 + j < W) ? (1u << j) : 0u;
                vmask[i] = rok ? m : 0u;
                soff[i] = rok ? (y - ylo) * W + x0 : 0;
                doff[i] = row < nrt ? static_cast<uint32_t>(row * 16 + (pr >> 2) * a_gran + (pr & 3) * 4) : 0xffffffffu;
            }
            // phase of a channel's first staged element inside its buffer (the
            // copy starts at the 16-byte boundary below it); x is 16-byte aligned
            const uint32_t row0 = static_cast<uint32_t>(ylo) * static_cast<uint32_t>(W);
            for (int c = 0; c < c_chunks; ++c) {
                const int gc = k * c_chunks + c;
                const int s = gc & 1;
                const int bsel = gc % nbuf;
                if (!mbar_wait(&sfull[bsel], (gc / nbuf) & 1, abort_flag, err, ERR_SITE_FULL)) {
                    ok = false;
                    break;
                }
                // the stage's A may be rewritten once the MMAs of chunk gc-2 are done
                if (!mbar_wait(&aempty[s], ((gc >> 1) & 1) ^ 1, abort_flag, err, ERR_SITE_EMPTY)) {
                    ok = false;
                    break;
                }
                const int ch = c * kChunk + 2 * pr;
                const uint32_t pl0 = (static_cast<uint32_t>(n) * C + ch) * static_cast<uint32_t>(plane) + row0 + xph;
                const uint32_t pl1 = pl0 + static_cast<uint32_t>(plane);
                const unsigned char* cb = stg + bsel * (kChunk * stg_ch) + 2 * pr * stg_ch;
                const uint16_t* base0 = reinterpret_cast<const uint16_t*>(cb) + (ch < C ? (pl0 & 7u) : 0u);
                const uint16_t* base1 = reinterpret_cast<const uint16_t*>(cb + stg_ch) + (ch + 1 < C ? (pl1 & 7u) : 0u);
                unsigned char* A = astage + s * a_bytes;
                // two tasks at a time, loads first, so their load latencies overlap
#pragma unroll
                for (int i0 = 0; i0 < kTasksPerThread; i0 += 2) {
                    __half2 d[2][6];
#pragma unroll
                    for (int t = 0; t < 2; ++t) {
                        const int i = i0 + t;
                        if (doff[i] == 0xffffffffu) continue;
                        const uint16_t* p0 = base0 + soff[i];
                        const uint16_t* p1 = base1 + soff[i];
#pragma unroll
                        for (int j = 0; j < 6; ++j) {
                            const uint32_t h =
                                __byte_perm(static_cast<uint32_t>(p0[j]), static_cast<uint32_t>(p1[j]), 0x5410);
                            d[t][j] = *reinterpret_cast<const __half2*>(&h);
                        }
                    }
#pragma unroll
                    for (int t = 0; t < 2; ++t) {
                        const int i = i0 + t;
                        if (doff[i] == 0xffffffffu) continue;
                        if (vmask[i] != 0x3fu) {
#pragma unroll
                            for (int j = 0; j < 6; ++j)
                                if (!((vmask[i] >> j) & 1u)) d[t][j] = __half2(__ushort_as_half(0), __ushort_as_half(0));
                        }
                        __half2 v[6];
                        bt6(d[t], v);
                        unsigned char* dst = A + doff[i];
#pragma unroll
                        for (int e = 0; e < 6; ++e) *reinterpret_cast<__half2*>(dst + e * (2 * a_gran)) = v[e];
                    }
                }
                mbar_arrive(&sempty[bsel]);   // staged rows read
                fence_proxy_async_smem();     // A visible to the tensor core
                mbar_arrive(&afull[s]);
            }
            if (!ok) break;

            // ---- epilogue: the 6 accumulators of each (tile, channel) -> 4 outputs
            if (!mbar_wait(tfull, k & 1, abort_flag, err, ERR_SITE_TMEM_FULL)) break;
            tc_fence_after();
            const int quarter = warp & 3;
            const int part = warp >> 2;                 // 16 output channels each
            const int m = quarter * 32 + lane;          // MMA row = output row i, tile tw
            const int i = m / tiles_w, tw = m - (m / tiles_w) * tiles_w;
            const int oh = oh0 + i;
            const bool mv = i < R && oh < gg.OH;
            const int ow0 = tw * 4;
            const int vc = min(4, gg.OW - ow0);
            const uint32_t lane_base = tmem_base + (static_cast<uint32_t>(quarter * 32) << 16);
#pragma unroll 1
            for (int g8 = 0; g8 < 2; ++g8) {
                const int kl0 = part * 16 + g8 * 8;
                uint32_t acc[6][8];
#pragma unroll
                for (int e = 0; e < 6; ++e) tmem_ld_x8(lane_base + e * kBN + kl0, acc[e]);
                tc_wait_ld();
#pragma unroll
                for (int e = 0; e < 6; ++e) tc_hold(acc[e]);
                if (!mv) continue;
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int kk = nb * kBN + kl0 + q;
                    if (kk >= K) continue;
                    const float m0 = __uint_as_float(acc[0][q]), m1 = __uint_as_float(acc[1][q]);
                    const float m2 = __uint_as_float(acc[2][q]), m3 = __uint_as_float(acc[3][q]);
                    const float m4 = __uint_as_float(acc[4][q]), m5 = __uint_as_float(acc[5][q]);
                    const float a = m1 + m2, b = m1 - m2;   // A^T of F4 (wg_transforms.cuh)
                    float yv[4];
                    yv[0] = m0 + a + m3 + m4;
                    yv[1] = b + 0.5f * m3 - 2.f * m4;
                    yv[2] = a + 0.25f * m3 + 4.f * m4;
                    yv[3] = b + 0.125f * m3 - 8.f * m4 + m5;
                    __half* o = out + ((static_cast<long long>(n) * K + kk) * gg.OH + oh) * static_cast<long long>(gg.OW) + ow0;
                    if (vc == 4 && (reinterpret_cast<uintptr_t>(o) & 7) == 0) {
                        __half2 lo = __floats2half2_rn(yv[0], yv[1]), hi = __floats2half2_rn(yv[2], yv[3]);
                        *reinterpret_cast<uint2*>(o) =
                            make_uint2(*reinterpret_cast<uint32_t*>(&lo), *reinterpret_cast<uint32_t*>(&hi));
                    } else {
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            if (j < vc) o[j] = __float2half_rn(yv[j]);
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
    if (warp == kMmaWarp) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 512);
    }
}

// ---- channel-interleaved variant ---------------------------------------------
// The input is the caller's NHWC tensor x[n][y][x][C], C a multiple of 16.
// One 4-D TMA box {16 channels, WB columns, R+2 rows, 1 image} per chunk
// stages [row][column][16 channels]; its out-of-range parts (padding rows and
// columns, channels past Cs) arrive as zeros, so the producers need no masks,
// and each of their loads moves 16 bytes (8 channels of one input value).
// WB = 4 * tiles_w + 5 (>= the 4 * tiles_w + 2 columns read, 1 mod 4): the
// staged rows then start 32 bytes apart modulo 128, and a quarter-warp of 4
// rows x 2 channel granules reads 8 distinct 16-byte bank groups.
constexpr int kMaxAStages = 4;
constexpr int kProducersI = 256;                         // 8 warps: transform, then epilogue
constexpr int kThreadsI = kProducersI + 96;              // + MMA, staging-TMA and filter-TMA warps
constexpr int kMmaWarpI = kProducersI / 32, kLoaderWarpI = kMmaWarpI + 1, kBWarpI = kMmaWarpI + 2;

struct RowGeoI {    // shared by host and device
    int C, K, pad_h, pad_w, OH, OW, tiles_w;
    int R, row_blocks, n_blocks, c_chunks;
    int wb;         // staged columns
    int stg_bytes;  // one staging buffer (box bytes rounded to 1024)
    int box_bytes;  // bytes one staging TMA delivers
    int nbuf, nbs;  // staging buffers, filter-tile stages
    int nas;        // transformed-input (A) stages
    int arows;      // rows of one A granule (>= 128 + 2 * tiles_w)
    int tb4;        // blocks of 4 tiles per row of tiles
    int tasks;      // producer task slots per chunk (4 rows x 4 tiles x 2 granules blocks)
};

__device__ __forceinline__ void bt6x8(const uint4 (&q)[6], uint4 (&o)[6]) {
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        __half2 d[6], v[6];
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            const uint32_t w = l == 0 ? q[j].x : l == 1 ? q[j].y : l == 2 ? q[j].z : q[j].w;
            d[j] = *reinterpret_cast<const __half2*>(&w);
        }
        bt6(d, v);
#pragma unroll
        for (int e = 0; e < 6; ++e) {
            const uint32_t w = *reinterpret_cast<const uint32_t*>(&v[e]);
            if (l == 0) o[e].x = w;
            else if (l == 1) o[e].y = w;
            else if (l == 2) o[e].z = w;
            else o[e].w = w;
        }
    }
}

template <bool OUT_NHWC>
__global__ void __launch_bounds__(kThreadsI, 1)
    row4x3i_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmU,
                   __half* __restrict__ out, const __grid_constant__ RowGeoI gg, int n_base, int n_images, DevErr* err) {
    constexpr uint32_t kIdesc = make_idesc_f16(128, kBN, false);
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int a_gran = gg.arows * 16;
    const int a_bytes = kE * 2 * a_gran;
    const int nbs = gg.nbs, nbuf = gg.nbuf, nas = gg.nas;
    // smem: B stages | staging buffers | A stages | barriers (1024-aligned parts first)
    unsigned char* bstage = smem;
    unsigned char* stg = smem + nbs * kBBytes;
    unsigned char* astage = stg + nbuf * gg.stg_bytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(astage + nas * a_bytes);
    uint64_t* afull = bars;                        // [4] producers
    uint64_t* aempty = bars + 4;                   // [4] MMA commit
    uint64_t* bfull = bars + 8;                    // [4] filter TMA (expect_tx)
    uint64_t* bempty = bars + 12;                  // [4] MMA commit
    uint64_t* sfull = bars + 16;                   // [4] staging TMA (expect_tx)
    uint64_t* sempty = bars + 20;                  // [4] staging buffer read by all producers
    uint64_t* tfull = bars + 24;                   // accumulators of the current item ready
    uint64_t* tempty = bars + 25;                  // accumulators drained
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 26);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int K = gg.K, R = gg.R, tiles_w = gg.tiles_w, c_chunks = gg.c_chunks;
    const int total_items = n_images * gg.row_blocks * gg.n_blocks;
    const int my_items = blockIdx.x < total_items ? (total_items - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int total_chunks = my_items * c_chunks;

    if (tid == 0) {
        for (int i = 0; i < kMaxAStages; ++i) {
            mbar_init(&afull[i], kProducersI);
            mbar_init(&aempty[i], 1);
        }
        for (int i = 0; i < kMaxBStages; ++i) {
            mbar_init(&bfull[i], 1);
            mbar_init(&bempty[i], 1);
        }
        for (int i = 0; i < kMaxBufs; ++i) {
            mbar_init(&sfull[i], 1);
            mbar_init(&sempty[i], kProducersI);
        }
        mbar_init(tfull, 1);
        mbar_init(tempty, kProducersI);
        *abort_flag = 0;
        fence_barrier_init();
    }
    pdl_wait();     // input written, earlier readers of the output done
    pdl_trigger();
    if (warp == kMmaWarpI) tmem_alloc(tmem_slot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    auto item_of = [&](int k, int& n, int& oh0, int& nb) {
        const int item = blockIdx.x + k * gridDim.x;
        nb = item % gg.n_blocks;
        const int rest = item / gg.n_blocks;
        oh0 = (rest % gg.row_blocks) * R;
        n = rest / gg.row_blocks;
    };

    if (warp == kLoaderWarpI) {
        // staged input rows: one TMA box per chunk, nbuf chunks ahead
        if (lane == 0) {
            tma_prefetch_desc(&tmX);
            for (int gc = 0; gc < total_chunks; ++gc) {
                const int sb = gc % nbuf;
                if (gc >= nbuf && !mbar_wait(&sempty[sb], ((gc / nbuf) & 1) ^ 1, abort_flag, err, ERR_SITE_EMPTY)) break;
                const int k = gc / c_chunks, c = gc - k * c_chunks;
                int n, oh0, nb;
                item_of(k, n, oh0, nb);
                mbar_arrive_expect_tx(&sfull[sb], static_cast<uint32_t>(gg.box_bytes));
                tma_load_4d(stg + sb * gg.stg_bytes, &tmX, &sfull[sb], c * kChunk, -gg.pad_w, oh0 - gg.pad_h,
                            n_base + n);
            }
        }
    } else if (warp == kBWarpI) {
        if (lane == 0) {
            tma_prefetch_desc(&tmU);
            for (int gc = 0; gc < total_chunks; ++gc) {
                const int sb = gc % nbs;
                if (gc >= nbs && !mbar_wait(&bempty[sb], ((gc / nbs) & 1) ^ 1, abort_flag, err, ERR_SITE_EMPTY)) break;
                const int k = gc / c_chunks, c = gc - k * c_chunks;
                int n, oh0, nb;
                item_of(k, n, oh0, nb);
                mbar_arrive_expect_tx(&bfull[sb], kBBytes);
                tma_load_4d(bstage + sb * kBBytes, &tmU, &bfull[sb], 0, nb * (kBN / 8), c * 2, 0);
            }
        }
    } else if (warp == kMmaWarpI) {
        if (lane == 0) {
            bool ok = true;
            for (int k = 0; k < my_items && ok; ++k) {
                if (!mbar_wait(tempty, (k & 1) ^ 1, abort_flag, err, ERR_SITE_TMEM_EMPTY)) break;
                tc_fence_after();
                for (int c = 0; c < c_chunks; ++c) {
                    const int gc = k * c_chunks + c;
                    const int sa = gc % nas, sb = gc % nbs;
                    if (!mbar_wait(&afull[sa], (gc / nas) & 1, abort_flag, err, ERR_SITE_FULL) ||
                        !mbar_wait(&bfull[sb], (gc / nbs) & 1, abort_flag, err, ERR_SITE_FULL)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a_base = smem_u32(astage + sa * a_bytes);
                    const uint32_t b_base = smem_u32(bstage + sb * kBBytes);
#pragma unroll
                    for (int e = 0; e < kE; ++e) {
#pragma unroll
                        for (int r = 0; r < kTaps; ++r) {
                            const uint64_t ad =
                                make_smem_desc(a_base + e * (2 * a_gran) + r * tiles_w * 16, a_gran, 128, Swz::None);
                            const uint64_t bd = make_smem_desc(b_base + (e * kTaps + r) * (2 * kBN * 16), kBN * 16, 128,
                                                               Swz::None);
                            tc_mma_f16(tmem_base + e * kBN, ad, bd, kIdesc, (c > 0 || r > 0) ? 1u : 0u);
                        }
                    }
                    tc_commit(&aempty[sa]);
                    tc_commit(&bempty[sb]);
                }
                if (ok && !*abort_flag) tc_commit(tfull);
            }
        }
    } else {
        // ---- producers: task = (row of tiles rho, tile tw, granule g) in
        //      blocks of 4 rows x 4 tiles x 2 granules (a warp = one block)
        const int nrow = R + kTaps - 1;
        bool ok = true;
        for (int k = 0; k < my_items && ok; ++k) {
            int n, oh0, nb;
            item_of(k, n, oh0, nb);
            for (int c = 0; c < c_chunks; ++c) {
                const int gc = k * c_chunks + c;
                const int s = gc % nas;
                const int sb = gc % nbuf;
                // the A stage may be rewritten once the MMAs of chunk gc - nas are done
                if (!mbar_wait(&sfull[sb], (gc / nbuf) & 1, abort_flag, err, ERR_SITE_FULL) ||
                    !mbar_wait(&aempty[s], ((gc / nas) & 1) ^ 1, abort_flag, err, ERR_SITE_EMPTY)) {
                    ok = false;
                    break;
                }
                const unsigned char* buf = stg + sb * gg.stg_bytes;
                unsigned char* A = astage + s * a_bytes;
                for (int t = tid; t < gg.tasks; t += kProducersI) {
                    const int g = t & 1, rq = (t >> 1) & 3, tq = (t >> 3) & 3, blk = t >> 5;
                    const int rb = blk / gg.tb4, tb = blk - rb * gg.tb4;
                    const int rho = rb * 4 + rq, tw = tb * 4 + tq;
                    if (rho >= nrow || tw >= tiles_w) continue;
                    const unsigned char* src = buf + ((rho * gg.wb + tw * 4) * 2 + g) * 16;
                    uint4 q[6], o[6];
#pragma unroll
                    for (int j = 0; j < 6; ++j) q[j] = *reinterpret_cast<const uint4*>(src + j * 32);
                    bt6x8(q, o);
                    unsigned char* dst = A + g * a_gran + (rho * tiles_w + tw) * 16;
#pragma unroll
                    for (int e = 0; e < 6; ++e) *reinterpret_cast<uint4*>(dst + e * (2 * a_gran)) = o[e];
                }
                mbar_arrive(&sempty[sb]);     // staged rows read
                fence_proxy_async_smem();     // A visible to the tensor core
                mbar_arrive(&afull[s]);
            }
            if (!ok) break;

            // ---- epilogue: the 6 accumulators of each (tile, channel) -> 4 outputs
            if (!mbar_wait(tfull, k & 1, abort_flag, err, ERR_SITE_TMEM_FULL)) break;
            tc_fence_after();
            const int quarter = warp & 3;
            const int chalf = warp >> 2;                // 32 output channels each
            const int m = quarter * 32 + lane;          // MMA row = output row i, tile tw
            const int i = m / tiles_w, tw = m - (m / tiles_w) * tiles_w;
            const int oh = oh0 + i;
            const bool mv = i < R && oh < gg.OH;
            const int ow0 = tw * 4;
            const int vc = min(4, gg.OW - ow0);
            const uint32_t lane_base = tmem_base + (static_cast<uint32_t>(quarter * 32) << 16);
#pragma unroll 1
            for (int g8 = 0; g8 < 4; ++g8) {
                const int kl0 = chalf * 32 + g8 * 8;
                uint32_t acc[6][8];
#pragma unroll
                for (int e = 0; e < 6; ++e) tmem_ld_x8(lane_base + e * kBN + kl0, acc[e]);
                tc_wait_ld();
#pragma unroll
                for (int e = 0; e < 6; ++e) tc_hold(acc[e]);
                const int kk0 = nb * kBN + kl0;
                if (!mv || kk0 >= K) continue;
                float yv[8][4];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float m0 = __uint_as_float(acc[0][q]), m1 = __uint_as_float(acc[1][q]);
                    const float m2 = __uint_as_float(acc[2][q]), m3 = __uint_as_float(acc[3][q]);
                    const float m4 = __uint_as_float(acc[4][q]), m5 = __uint_as_float(acc[5][q]);
                    const float a = m1 + m2, b = m1 - m2;   // A^T of F4 (wg_transforms.cuh)
                    yv[q][0] = m0 + a + m3 + m4;
                    yv[q][1] = b + 0.5f * m3 - 2.f * m4;
                    yv[q][2] = a + 0.25f * m3 + 4.f * m4;
                    yv[q][3] = b + 0.125f * m3 - 8.f * m4 + m5;
                }
                if (OUT_NHWC) {
                    // y[n][oh][ow][K]: 8 consecutive channels of each output column
                    __half* o = out + ((static_cast<long long>(n) * gg.OH + oh) * gg.OW + ow0) * K + kk0;
                    const bool vec = kk0 + 8 <= K && (K & 7) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        if (j >= vc) break;
                        if (vec) {
                            uint4 w;
                            __half2 h0 = __floats2half2_rn(yv[0][j], yv[1][j]), h1 = __floats2half2_rn(yv[2][j], yv[3][j]);
                            __half2 h2 = __floats2half2_rn(yv[4][j], yv[5][j]), h3 = __floats2half2_rn(yv[6][j], yv[7][j]);
                            w.x = *reinterpret_cast<uint32_t*>(&h0);
                            w.y = *reinterpret_cast<uint32_t*>(&h1);
                            w.z = *reinterpret_cast<uint32_t*>(&h2);
                            w.w = *reinterpret_cast<uint32_t*>(&h3);
                            *reinterpret_cast<uint4*>(o + static_cast<long long>(j) * K) = w;
                        } else {
#pragma unroll
                            for (int q = 0; q < 8; ++q)
                                if (kk0 + q < K) o[static_cast<long long>(j) * K + q] = __float2half_rn(yv[q][j]);
                        }
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int kk = kk0 + q;
                        if (kk >= K) break;
                        __half* o = out + ((static_cast<long long>(n) * K + kk) * gg.OH + oh) * static_cast<long long>(gg.OW) + ow0;
                        if (vc == 4 && (reinterpret_cast<uintptr_t>(o) & 7) == 0) {
                            __half2 lo = __floats2half2_rn(yv[q][0], yv[q][1]), hi = __floats2half2_rn(yv[q][2], yv[q][3]);
                            *reinterpret_cast<uint2*>(o) =
                                make_uint2(*reinterpret_cast<uint32_t*>(&lo), *reinterpret_cast<uint32_t*>(&hi));
                        } else {
#pragma unroll
                            for (int j = 0; j < 4; ++j)
                                if (j < vc) o[j] = __float2half_rn(yv[q][j]);
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
    if (warp == kMmaWarpI) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 512);
    }
}

// U1[e*3 + r][Cp16/8][Kp64][8] = G w[k][c][r][.] (1-D F(4,3) filter transform,
// the G of F4), zero for c >= C or k >= K.
__global__ void __launch_bounds__(256) row4x3_filter_kernel(const __half* __restrict__ w, __half* __restrict__ U, int K,
                                                           int C, int Cp, int Kp) {
    const long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= static_cast<long long>(Kp) * Cp) return;
    const int k = static_cast<int>(idx / Cp), c = static_cast<int>(idx % Cp);
    const int CG = Cp / 8;
#pragma unroll
    for (int r = 0; r < kTaps; ++r) {
        float g[3] = {0.f, 0.f, 0.f};
        if (c < C && k < K) {
            const __half* src = w + ((static_cast<long long>(k) * C + c) * 3 + r) * 3;
            for (int s = 0; s < 3; ++s) g[s] = __half2float(src[s]);
        }
        float u[6];
        F4::g(g, 1, u, 1);
#pragma unroll
        for (int e = 0; e < kE; ++e)
            U[((static_cast<long long>(e * kTaps + r) * CG + c / 8) * Kp + k) * 8 + (c & 7)] = __float2half_rn(u[e]);
    }
}

}  // namespace

namespace {

// U1 viewed as 128-byte rows of 8 output channels: a box of 8 rows (64
// channels) x 2 granules x 18 (element, filter row) per chunk
cudaError_t encode_u1(RowPlan& rp, const Geom& g, const void* U) {
    rp.c = g.c;
    rp.k = g.k;
    rp.cp16 = (g.c + 15) / 16 * 16;
    rp.kp64 = (g.k + kBN - 1) / kBN * kBN;
    if (!U) return cudaSuccess;
    const cuuint64_t CG = static_cast<cuuint64_t>(rp.cp16 / 8);
    const cuuint64_t Kr = static_cast<cuuint64_t>(rp.kp64 / 8);
    cuuint64_t dims[4] = {64, Kr, CG, kE * kTaps};
    cuuint64_t strides[3] = {128, Kr * 128, CG * Kr * 128};
    cuuint32_t box[4] = {64, kBN / 8, 2, kE * kTaps};
    if (encode_tiled(&rp.tmU, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 4, const_cast<void*>(U), dims, strides, box,
                     CU_TENSOR_MAP_SWIZZLE_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    return cudaSuccess;
}

}  // namespace

cudaError_t plan_row4x3(RowPlan& rp, const Geom& g, const void* U) {
    RowGeo& gg = *reinterpret_cast<RowGeo*>(rp.geo);
    static_assert(sizeof(RowGeo) <= sizeof(rp.geo), "RowPlan geometry storage");
    if (g.pad_h > 64 || g.pad_w > 64) return cudaErrorNotSupported;
    gg.C = g.c; gg.H = g.h; gg.W = g.w; gg.K = g.k; gg.pad_h = g.pad_h; gg.pad_w = g.pad_w;
    gg.OH = g.oh; gg.OW = g.ow;
    gg.tiles_w = (g.ow + 3) / 4;
    if (gg.tiles_w > 64) return cudaErrorNotSupported;   // at least two output rows per item
    const int rmax = 128 / gg.tiles_w;
    gg.row_blocks = (g.oh + rmax - 1) / rmax;
    gg.R = (g.oh + gg.row_blocks - 1) / gg.row_blocks;    // balanced blocks of at most rmax rows
    gg.n_blocks = (g.k + kBN - 1) / kBN;
    gg.c_chunks = (g.c + kChunk - 1) / kChunk;
    const int rows = std::min(g.h, gg.R + kTaps - 1);
    gg.stg_ch = (rows * g.w * 2 + 16 + 15) / 16 * 16;
    gg.arows = (128 + 2 * gg.tiles_w + 7) / 8 * 8 + 4;
    const int a_bytes = kE * 2 * gg.arows * 16;
    // deepest filter-tile ring first (its loads come from L2 and cover a whole
    // chunk of MMAs), then as many staging buffers as fit
    rp.smem_bytes = 0;
    for (int nbs = kMaxBStages; nbs >= 2 && !rp.smem_bytes; --nbs) {
        for (int nbuf = kMaxBufs; nbuf >= 1; --nbuf) {
            const int bytes = nbs * kBBytes + kAStages * a_bytes + kHdr + nbuf * kChunk * gg.stg_ch + kSlack + 1024;
            if (bytes <= 227 * 1024 && (nbuf >= 2 || nbs == 2)) {
                gg.nbs = nbs;
                gg.nbuf = nbuf;
                rp.smem_bytes = bytes;
                break;
            }
        }
    }
    if (!rp.smem_bytes) return cudaErrorNotSupported;
    rp.interleaved = 0;
    return encode_u1(rp, g, U);
}

// channel-interleaved variant: geometry, shared-memory split and the filter map
cudaError_t plan_row4x3i(RowPlan& rp, const Geom& g, const void* U, bool out_nhwc) {
    RowGeoI& gg = *reinterpret_cast<RowGeoI*>(rp.geo);
    static_assert(sizeof(RowGeoI) <= sizeof(rp.geo), "RowPlan geometry storage");
    gg.C = g.c; gg.K = g.k; gg.pad_h = g.pad_h; gg.pad_w = g.pad_w;
    gg.OH = g.oh; gg.OW = g.ow;
    gg.tiles_w = (g.ow + 3) / 4;
    if (gg.tiles_w > 62) return cudaErrorNotSupported;   // the staged columns are one TMA box (<= 256)
    const int rmax = 128 / gg.tiles_w;
    gg.row_blocks = (g.oh + rmax - 1) / rmax;
    gg.R = (g.oh + gg.row_blocks - 1) / gg.row_blocks;
    gg.n_blocks = (g.k + kBN - 1) / kBN;
    gg.c_chunks = (g.c + kChunk - 1) / kChunk;
    gg.wb = 4 * gg.tiles_w + 5;
    gg.box_bytes = 2 * kChunk * gg.wb * (gg.R + kTaps - 1);
    gg.stg_bytes = (gg.box_bytes + 127) / 128 * 128;
    gg.tb4 = (gg.tiles_w + 3) / 4;
    gg.tasks = (gg.R + kTaps - 1 + 3) / 4 * gg.tb4 * 32;
    // A granule rows: 128 + 2 * tiles_w at least; the rows mod 8 set where the
    // second granule falls in the bank space relative to the first, chosen so
    // a quarter-warp's stores (4 rows of tiles x 2 granules) hit distinct
    // 16-byte bank groups where the tile row count allows it
    const int base = (128 + 2 * gg.tiles_w + 7) / 8 * 8;
    int best = 0, best_distinct = -1;
    for (int k = 0; k < 8; ++k) {
        unsigned used = 0;
        int distinct = 0;
        for (int r = 0; r < 4; ++r)
            for (int gr = 0; gr < 2; ++gr) {
                const int slot = ((r * gg.tiles_w) + gr * k) & 7;
                if (!(used & (1u << slot))) ++distinct;
                used |= 1u << slot;
            }
        if (distinct > best_distinct) {
            best_distinct = distinct;
            best = k;
        }
    }
    gg.arows = base + best;
    const int a_bytes = kE * 2 * gg.arows * 16;
    // (A stages, filter-tile stages, staging buffers), deepest first;
    // WG_CONV2D_ROW_STAGES="a,b,s" asks for one split (if it fits)
    static const int kPrefs[][3] = {{2, 4, 4}, {2, 4, 3}, {2, 3, 4}, {2, 3, 3}, {2, 4, 2},
                                    {2, 3, 2}, {2, 2, 3}, {2, 2, 2}, {2, 2, 1}};
    rp.smem_bytes = 0;
    int want[3] = {0, 0, 0};
    if (const char* e = std::getenv("WG_CONV2D_ROW_STAGES"))
        if (std::sscanf(e, "%d,%d,%d", &want[0], &want[1], &want[2]) != 3 || want[0] < 2 || want[0] > kMaxAStages ||
            want[1] < 2 || want[1] > kMaxBStages || want[2] < 1 || want[2] > kMaxBufs)
            want[0] = 0;
    auto fits = [&](int a, int b, int sb) {
        const int bytes = b * kBBytes + sb * gg.stg_bytes + a * a_bytes + kHdr + 128;
        if (bytes > 227 * 1024) return false;
        gg.nas = a;
        gg.nbs = b;
        gg.nbuf = sb;
        rp.smem_bytes = bytes;
        return true;
    };
    if (!(want[0] && fits(want[0], want[1], want[2])))
        for (const auto& pf : kPrefs)
            if (fits(pf[0], pf[1], pf[2])) break;
    if (!rp.smem_bytes) return cudaErrorNotSupported;
    rp.interleaved = 1;
    rp.out_nhwc = out_nhwc ? 1 : 0;
    rp.cs = (g.c + 15) / 16 * 16;
    return encode_u1(rp, g, U);
}

cudaError_t bind_row4x3i_input(RowPlan& rp, const void* x_nhwc, int cs, int h, int w, int n_total) {
    const RowGeoI& gg = *reinterpret_cast<const RowGeoI*>(rp.geo);
    cuuint64_t dims[4] = {static_cast<cuuint64_t>(cs), static_cast<cuuint64_t>(w), static_cast<cuuint64_t>(h),
                          static_cast<cuuint64_t>(n_total)};
    cuuint64_t strides[3] = {static_cast<cuuint64_t>(cs) * 2, static_cast<cuuint64_t>(w) * cs * 2,
                             static_cast<cuuint64_t>(h) * w * cs * 2};
    cuuint32_t box[4] = {kChunk, static_cast<cuuint32_t>(gg.wb), static_cast<cuuint32_t>(gg.R + kTaps - 1), 1};
    if (encode_tiled(&rp.tmX, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 4, const_cast<void*>(x_nhwc), dims, strides, box,
                     CU_TENSOR_MAP_SWIZZLE_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    return cudaSuccess;
}

cudaError_t launch_row4x3i(const RowPlan& rp, void* out, int n_base, int n_images, DevErr* err, cudaStream_t s) {
    const RowGeoI& gg = *reinterpret_cast<const RowGeoI*>(rp.geo);
    const long long items = row4x3_items(rp, n_images);
    if (items <= 0) return cudaSuccess;
    if (items > 0x7fffffffLL) return cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0)
        sms = 148;
    const dim3 grid(static_cast<unsigned>(std::min<long long>(items, sms)));
    if (rp.out_nhwc) {
        cudaError_t e = cudaFuncSetAttribute(row4x3i_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, rp.smem_bytes);
        if (e != cudaSuccess) return e;
        return launch_pdl(row4x3i_kernel<true>, grid, dim3(kThreadsI), rp.smem_bytes, s, rp.tmX, rp.tmU,
                          static_cast<__half*>(out), gg, n_base, n_images, err);
    }
    cudaError_t e = cudaFuncSetAttribute(row4x3i_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, rp.smem_bytes);
    if (e != cudaSuccess) return e;
    return launch_pdl(row4x3i_kernel<false>, grid, dim3(kThreadsI), rp.smem_bytes, s, rp.tmX, rp.tmU,
                      static_cast<__half*>(out), gg, n_base, n_images, err);
}

int row4x3_threads(const RowPlan& rp) { return rp.interleaved ? kThreadsI : kThreads; }

long long row4x3_filter_bytes(const RowPlan& rp) { return static_cast<long long>(kE * kTaps) * rp.kp64 * rp.cp16 * 2; }

long long row4x3_items(const RowPlan& rp, int n_images) {
    if (rp.interleaved) {
        const RowGeoI& gi = *reinterpret_cast<const RowGeoI*>(rp.geo);
        return static_cast<long long>(n_images) * gi.row_blocks * gi.n_blocks;
    }
    const RowGeo& gg = *reinterpret_cast<const RowGeo*>(rp.geo);
    return static_cast<long long>(n_images) * gg.row_blocks * gg.n_blocks;
}

cudaError_t launch_row4x3_filter(const RowPlan& rp, const void* weight, void* U, cudaStream_t s) {
    const long long total = static_cast<long long>(rp.kp64) * rp.cp16;
    row4x3_filter_kernel<<<static_cast<unsigned>((total + 255) / 256), 256, 0, s>>>(
        static_cast<const __half*>(weight), static_cast<__half*>(U), rp.k, rp.c, rp.cp16, rp.kp64);
    return cudaGetLastError();
}

cudaError_t launch_row4x3(const RowPlan& rp, const void* x, const void* x_end, void* out, int n_images, DevErr* err,
                          cudaStream_t s) {
    const RowGeo& gg = *reinterpret_cast<const RowGeo*>(rp.geo);
    const long long items = row4x3_items(rp, n_images);
    if (items <= 0) return cudaSuccess;
    if (items > 0x7fffffffLL) return cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        sms <= 0)
        sms = 148;
    cudaError_t e = cudaFuncSetAttribute(row4x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, rp.smem_bytes);
    if (e != cudaSuccess) return e;
    return launch_pdl(row4x3_kernel, dim3(static_cast<unsigned>(std::min<long long>(items, sms))), dim3(kThreads),
                      rp.smem_bytes, s, static_cast<const __half*>(x), static_cast<const __half*>(x_end), rp.tmU,
                      static_cast<__half*>(out), gg, n_images, err);
}

}  // namespace wg
