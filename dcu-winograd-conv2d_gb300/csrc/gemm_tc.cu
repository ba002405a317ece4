// Winograd-domain batched GEMM on the 5th-generation tensor cores.
//
// For every Winograd element e (16 for F(2x3), 36 for F(4x3)):
//     M_e[P][K] = V_e[P][Cp] * U_e[K][Cp]^T      (fp32 accumulation)
// which is the reference's hep_sgemm call (src/winograd_2x3_non_fused.cpp:403-413,
// src/winograd_4x3_non_fused.cpp:587-597; kernels in include/hep_sgemm.h) with
// the operands stored K-major.
//
// Design (one persistent CTA per SM, 320 threads):
//   warp 0      TMA producer: 128 tiles x 64 channels of V plus BN x 64 of U
//               per stage, as 4-D boxes of 8 granules that land in the
//               canonical no-swizzle K-major layout; S-stage mbarrier ring;
//   warp 1      allocates TMEM and issues tcgen05.mma (M=128, N=BN, K=16)
//               from one thread; accumulators double-buffered in TMEM so the
//               epilogue of one output tile overlaps the main loop of the next;
//   warps 2-9   epilogue (two warps per TMEM lane quarter, each half of the
//               columns when BN >= 64): tcgen05.ld 32 lanes x 32 columns (the
//               next chunk's load in flight while this one is stored), convert,
//               16-byte granule stores of M (a warp writes 512 contiguous bytes).
// Work items are (problem, e, 128-tile block, BN-channel block), handed out
// round robin over one global index; a grouped launch covers many problems
// (each with its own tensor maps, sizes and output) in one persistent grid.
// Within a problem, channel blocks of one (e, tile block) are adjacent so the
// V tile is reused from L2.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "wg_kernels.h"
#include "wg_launch.h"
#include "wg_ptx.cuh"

namespace wg {

namespace {

constexpr int kBM = 128;
constexpr int kBK = 64;                 // 8 granules of 8 channels per stage
constexpr int kTileABytes = kBM * kBK * 2;

// RESB: the U block of a work item (BN rows x all Cp channels) stays in
// shared memory across consecutive work items that use it, and only V goes
// through the stage ring (single-problem launches whose U block fits).
constexpr int kResBBytes = 128 * 1024;

template <int BN, bool RESB = false>
struct GemmCfg {
    static constexpr int kTileB = BN * kBK * 2;
    static constexpr int kStageBytes = kTileABytes + (RESB ? 0 : kTileB);
    static constexpr int kBRegion = RESB ? kResBBytes : 0;   // + the ring's B tiles, below
    static constexpr int kStages = std::min(8, (200 * 1024 - kBRegion) / kStageBytes);
    static constexpr int kTmemCols = (2 * BN < 32) ? 32 : 2 * BN;  // two accumulators
    static constexpr int kSmem = kStages * kStageBytes + kBRegion + 1024 /*align*/ + 256 /*barriers*/;
    // + the row-major epilogue's transpose blocks (32x32 fp32 per epilogue
    // warp), only in launches that write row-major M
    static constexpr int kSmemRow = kSmem + 8 * 32 * 32 * 4;
};

// Epilogue stores of 32 accumulator columns (output channels k0..k0+31) of
// one tile row p into the granule layout.
template <class MT>
__device__ __forceinline__ void store32(MT* Mw, const uint32_t (&r)[32], long long P, long long p, int k0, int kg_count,
                                        int e, uint64_t pol);

// fp16 M[e][Kp/8][P][8]: four granules
template <>
__device__ __forceinline__ void store32<__half>(__half* Mw, const uint32_t (&r)[32], long long P, long long p, int k0,
                                                int kg_count, int e, uint64_t pol) {
    uint32_t h[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        __half2 v = __floats2half2_rn(__uint_as_float(r[2 * i]), __uint_as_float(r[2 * i + 1]));
        h[i] = *reinterpret_cast<uint32_t*>(&v);
    }
    const int g0 = k0 / 8;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (g0 + j < kg_count)
            st_hint_v4(Mw + ((static_cast<long long>(e) * kg_count + g0 + j) * P + p) * 8,
                       make_uint4(h[4 * j], h[4 * j + 1], h[4 * j + 2], h[4 * j + 3]), pol);
}

// fp32 M[e][Kp/4][P][4]: eight granules
template <>
__device__ __forceinline__ void store32<float>(float* Mw, const uint32_t (&r)[32], long long P, long long p, int k0,
                                               int kg_count, int e, uint64_t pol) {
    const int g0 = k0 / 4;
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (g0 + j < kg_count)
            st_hint_v4(Mw + ((static_cast<long long>(e) * kg_count + g0 + j) * P + p) * 4,
                       make_uint4(r[4 * j], r[4 * j + 1], r[4 * j + 2], r[4 * j + 3]), pol);
}

// 24-bit M: tag type of the split-plane storage (upper 16 bits of each
// rounded fp32 value in H[NB][Kp/8][E][64][8], next 8 bits in
// L[NB][Kp/8][E][64][8]: blocks of 64 tiles, NB = ceil(P/64)).
struct M24 {};

// 24-bit M: 32 accumulator columns (four granules of 8 channels) of tile row
// p.  Each fp32 value is rounded to nearest at bit 8 (ties away from zero;
// a carry into the exponent is the correct rounding, and the largest finite
// values round to infinity as at any precision); bytes 2-3 go to the high
// plane (one 16-byte store per granule), byte 1 to the low plane (one 8-byte
// store per granule); a warp's 32 rows lie in one 64-tile block, so its
// stores cover 512 and 256 contiguous bytes.
__device__ __forceinline__ void store32_m24(unsigned char* Mb, const uint32_t (&r)[32], long long p, int k0,
                                            int kg_count, int e, int E, long long m_lo, uint64_t pol) {
    const int g0 = k0 / 8;
    const long long row0 = (((p >> 6) * kg_count + g0) * E + e) * 64 + (p & 63);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (g0 + j >= kg_count) break;
        uint32_t v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) v[i] = r[8 * j + i] + 0x80u;
        const uint4 hi = make_uint4(__byte_perm(v[0], v[1], 0x7632), __byte_perm(v[2], v[3], 0x7632),
                                    __byte_perm(v[4], v[5], 0x7632), __byte_perm(v[6], v[7], 0x7632));
        const uint32_t l01 = __byte_perm(v[0], v[1], 0x5151), l23 = __byte_perm(v[2], v[3], 0x5151);
        const uint32_t l45 = __byte_perm(v[4], v[5], 0x5151), l67 = __byte_perm(v[6], v[7], 0x5151);
        const uint2 lo = make_uint2(__byte_perm(l01, l23, 0x5410), __byte_perm(l45, l67, 0x5410));
        const long long row = row0 + j * E * 64;
        st_hint_v4(Mb + row * 16, hi, pol);
        st_hint_v2(Mb + m_lo + row * 8, lo, pol);
    }
}

// Row-major M[e][P][Kp] (the NHWC output path): 4 consecutive columns of
// row p (one 16-byte store for fp32, 8 bytes for fp16); Kp is a multiple of 8.
template <class MT>
__device__ __forceinline__ void store4_row(MT* Mw, const uint32_t (&v)[4], long long P, long long p, int k0, int kp,
                                           int e, uint64_t pol) {
    MT* dst = Mw + (static_cast<long long>(e) * P + p) * kp + k0;
    if constexpr (sizeof(MT) == 4) {
        st_hint_v4(dst, make_uint4(v[0], v[1], v[2], v[3]), pol);
    } else {
        __half2 a = __floats2half2_rn(__uint_as_float(v[0]), __uint_as_float(v[1]));
        __half2 b = __floats2half2_rn(__uint_as_float(v[2]), __uint_as_float(v[3]));
        *reinterpret_cast<uint2*>(dst) = make_uint2(*reinterpret_cast<uint32_t*>(&a), *reinterpret_cast<uint32_t*>(&b));
    }
}

// Work item t -> problem index (advanced monotonically) and (e, mb, nb):
// channel block fastest (the V tile is reused from L2), then tile block, then
// element, so concurrent CTAs write M in long runs of a few element planes.
// The divisions are multiply-shifts (a problem has fewer than 2^31 items).
struct Item {
    int e, mb, nb;
};

__device__ __forceinline__ Item locate(const GemmDesc* __restrict__ descs, int ndesc, long long t, int& pi) {
    while (pi + 1 < ndesc && t >= descs[pi + 1].tile_begin) ++pi;
    const GemmDesc& d = descs[pi];
    const uint32_t local = static_cast<uint32_t>(t - d.tile_begin);
    Item it;
    const uint32_t rest = fast_div(d.fd_nb, local);
    it.nb = static_cast<int>(local - rest * static_cast<uint32_t>(d.n_blocks));
    const uint32_t e = fast_div(d.fd_mb, rest);
    it.mb = static_cast<int>(rest - e * static_cast<uint32_t>(d.m_blocks));
    it.e = static_cast<int>(e);
    return it;
}

// Resident-U order (one problem): tile block fastest, then channel block,
// then element, so the items of one (element, channel block) -- one U block --
// are consecutive; each CTA takes a contiguous range of them.
__device__ __forceinline__ Item locate_resb(const GemmDesc& d, long long t) {
    Item it;
    const uint32_t tu = static_cast<uint32_t>(t);
    const uint32_t rest = fast_div(d.fd_mb, tu);
    it.mb = static_cast<int>(tu - rest * static_cast<uint32_t>(d.m_blocks));
    const uint32_t e = fast_div(d.fd_nb, rest);
    it.nb = static_cast<int>(rest - e * static_cast<uint32_t>(d.n_blocks));
    it.e = static_cast<int>(e);
    return it;
}

template <bool RESB>
__device__ __forceinline__ Item locate_item(const GemmDesc* __restrict__ descs, int ndesc, long long t, int& pi) {
    if constexpr (RESB)
        return locate_resb(descs[0], t);
    else
        return locate(descs, ndesc, t, pi);
}

constexpr int kGemmThreads = 320;  // TMA warp, MMA warp, 8 epilogue warps

template <int BN, bool BF16, class MT, bool RESB>
__device__ __forceinline__ void gemm_body(const GemmDesc* __restrict__ descs, int ndesc, long long total_tiles,
                                          DevErr* err) {
    using Cfg = GemmCfg<BN, RESB>;
    constexpr int S = Cfg::kStages;
    constexpr int kEpiHalves = BN >= 64 ? 2 : 1;  // epilogue warps per TMEM lane quarter
    constexpr uint32_t kIdesc = make_idesc_f16(kBM, BN, BF16);

    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned base by pointer arithmetic (an integer round trip would
    // hide that this is shared memory and turn every access generic)
    unsigned char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    unsigned char* sA = smem;
    unsigned char* sB = smem + S * kTileABytes;   // B ring stages, or the resident U block
    unsigned char* after = smem + S * Cfg::kStageBytes + Cfg::kBRegion;
    uint64_t* bars = reinterpret_cast<uint64_t*>(after);
    uint64_t* full = bars;
    uint64_t* empty = bars + S;
    uint64_t* tfull = bars + 2 * S;
    uint64_t* tempty = bars + 2 * S + 2;
    uint64_t* bfull = bars + 2 * S + 4;    // resident U loaded
    uint64_t* bempty = bars + 2 * S + 5;   // the MMAs reading the resident U are done
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * S + 6);
    uint32_t* xpose = reinterpret_cast<uint32_t*>(after + 256);  // [8 warps][32][32]
    // items: round robin over the grid, or a contiguous range per CTA (RESB)
    const long long t_lo = RESB ? static_cast<long long>(blockIdx.x) * total_tiles / gridDim.x : blockIdx.x;
    const long long t_hi = RESB ? static_cast<long long>(blockIdx.x + 1) * total_tiles / gridDim.x : total_tiles;
    const long long t_step = RESB ? 1 : gridDim.x;
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&tfull[i], 1);
            mbar_init(&tempty[i], 128 * kEpiHalves);
        }
        mbar_init(bfull, 1);
        mbar_init(bempty, 1);
        *abort_flag = 0;
        fence_barrier_init();
    }
    // The first resident U block is read before the wait: U comes from the
    // filter transform, which completed before the kernel ahead of this one
    // (the input transform) passed its own wait and released this grid, so
    // only V depends on the kernel ahead; the copy overlaps that kernel's tail.
    int first_key = -1;
    if constexpr (RESB) {
        if (threadIdx.x == 0 && t_lo < t_hi) {   // the producer thread (warp 0, lane 0)
            int pi0 = 0;
            const Item it0 = locate_item<RESB>(descs, ndesc, t_lo, pi0);
            const GemmDesc& d0 = descs[pi0];
            tma_prefetch_desc(&d0.tmB);
            mbar_arrive_expect_tx(bfull, static_cast<uint32_t>(d0.k_blocks) * Cfg::kTileB);
            for (int kb = 0; kb < d0.k_blocks; ++kb)
                tma_load_4d(sB + kb * Cfg::kTileB, &d0.tmB, bfull, 0, it0.nb * (BN / 8), kb * 8, it0.e);
            first_key = it0.e * d0.n_blocks + it0.nb;
        }
    }
    pdl_wait();     // V written, earlier readers of M done
    pdl_trigger();
    if (warp == 1) tmem_alloc(tmem_slot, Cfg::kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            const uint64_t drop = l2_evict_first(), keep_as_is = l2_evict_unchanged();
            int stage = 0;
            uint32_t phase = 0;
            int pi = 0, prefetched = -1;
            int bkey = first_key;   // (element, channel block) of the resident U
            uint32_t bphase = 0;
            for (long long t = t_lo; t < t_hi; t += t_step) {
                const Item it = locate_item<RESB>(descs, ndesc, t, pi);
                const GemmDesc& d = descs[pi];
                if (prefetched != pi) {
                    tma_prefetch_desc(&d.tmA);
                    tma_prefetch_desc(&d.tmB);
                    prefetched = pi;
                }
                bool ok = true;
                if constexpr (RESB) {
                    const int key = it.e * d.n_blocks + it.nb;
                    if (key != bkey) {
                        // replace the resident U once the MMAs reading it are done
                        if (bkey >= 0) {
                            if (!mbar_wait(bempty, bphase, abort_flag, err, ERR_SITE_EMPTY)) break;
                            bphase ^= 1u;
                        }
                        mbar_arrive_expect_tx(bfull, static_cast<uint32_t>(d.k_blocks) * Cfg::kTileB);
                        for (int kb = 0; kb < d.k_blocks; ++kb)
                            tma_load_4d(sB + kb * Cfg::kTileB, &d.tmB, bfull, 0, it.nb * (BN / 8), kb * 8, it.e);
                        bkey = key;
                    }
                }
                for (int kb = 0; kb < d.k_blocks; ++kb) {
                    if (!mbar_wait(&empty[stage], phase ^ 1u, abort_flag, err, ERR_SITE_EMPTY)) {
                        ok = false;
                        break;
                    }
                    mbar_arrive_expect_tx(&full[stage], Cfg::kStageBytes);
                    // V: dropped from L2 by its last reader (the last N block)
                    tma_load_4d_hint(sA + stage * kTileABytes, &d.tmA, &full[stage], 0, it.mb * (kBM / 8), kb * 8, it.e,
                                     it.nb == d.n_blocks - 1 ? drop : keep_as_is);
                    if constexpr (!RESB)
                        tma_load_4d(sB + stage * Cfg::kTileB, &d.tmB, &full[stage], 0, it.nb * (BN / 8), kb * 8, it.e);
                    if (++stage == S) {
                        stage = 0;
                        phase ^= 1u;
                    }
                }
                if (!ok) break;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            int acc = 0;
            uint32_t acc_phase = 0;
            int pi = 0;
            int bkey = -1;
            uint32_t bphase = 0;
            for (long long t = t_lo; t < t_hi; t += t_step) {
                const Item it = locate_item<RESB>(descs, ndesc, t, pi);
                const int k_blocks = descs[pi].k_blocks;
                if (!mbar_wait(&tempty[acc], acc_phase ^ 1u, abort_flag, err, ERR_SITE_TMEM_EMPTY)) break;
                if constexpr (RESB) {
                    const int key = it.e * descs[0].n_blocks + it.nb;
                    if (key != bkey) {
                        if (!mbar_wait(bfull, bphase, abort_flag, err, ERR_SITE_FULL)) break;
                        bphase ^= 1u;
                        bkey = key;
                    }
                }
                tc_fence_after();
                const uint32_t d_tmem = tmem_base + static_cast<uint32_t>(acc * BN);
                bool ok = true;
                for (int kb = 0; kb < k_blocks; ++kb) {
                    if (!mbar_wait(&full[stage], phase, abort_flag, err, ERR_SITE_FULL)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a_base = smem_u32(sA + stage * kTileABytes);
                    const uint32_t b_base = smem_u32(sB + (RESB ? kb : stage) * Cfg::kTileB);
                    // K = 16 per MMA = 2 granules: core matrices at +0 and +LBO
#pragma unroll
                    for (int k = 0; k < kBK / 16; ++k) {
                        const uint64_t ad = make_smem_desc(a_base + k * (2 * kBM * 16), kBM * 16, 128, Swz::None);
                        const uint64_t bd = make_smem_desc(b_base + k * (2 * BN * 16), BN * 16, 128, Swz::None);
                        tc_mma_f16(d_tmem, ad, bd, kIdesc, (kb | k) != 0 ? 1u : 0u);
                    }
                    tc_commit(&empty[stage]);
                    if (++stage == S) {
                        stage = 0;
                        phase ^= 1u;
                    }
                }
                if (!ok) break;
                tc_commit(&tfull[acc]);
                if constexpr (RESB) {
                    // the next item reads another U block: free this one when
                    // the MMAs issued so far are done
                    if (t + 1 < t_hi) {
                        const Item nx = locate_resb(descs[0], t + 1);
                        if (nx.e * descs[0].n_blocks + nx.nb != bkey) tc_commit(bempty);
                    }
                }
                if (++acc == 2) {
                    acc = 0;
                    acc_phase ^= 1u;
                }
            }
        }
    } else if (warp - 2 < 4 * kEpiHalves) {
        // epilogue warps 2..9: TMEM lane quarter = warp % 4; warps 2-5 store
        // the first half of the accumulator columns, 6-9 the second (BN >= 64)
        const int quarter = warp & 3;
        // M that fits in L2 stays for the output transform; larger M must not
        // push V out
        const uint64_t m_pol = descs[0].keep_m ? l2_evict_last() : l2_evict_first();
        const int half = (warp - 2) >> 2;
        const int row = quarter * 32 + lane;
        int acc = 0;
        uint32_t acc_phase = 0;
        int pi = 0;
        for (long long t = t_lo; t < t_hi; t += t_step) {
            const Item it = locate_item<RESB>(descs, ndesc, t, pi);
            const GemmDesc& d = descs[pi];
            MT* Mw = static_cast<MT*>(d.Mw);
            const long long P = d.P;
            const int kg_count = d.kg_count;
            const int m_row = d.m_row, kp = d.kp;
            const long long m_lo = d.m_lo;
            if (!mbar_wait(&tfull[acc], acc_phase, abort_flag, err, ERR_SITE_TMEM_FULL)) break;
            tc_fence_after();
            const long long p = static_cast<long long>(it.mb) * kBM + row;
            const int col0 = half * (BN / kEpiHalves);
            const uint32_t taddr = tmem_base + (static_cast<uint32_t>(quarter * 32) << 16) +
                                   static_cast<uint32_t>(acc * BN + col0);
            // 32 columns per load; the load of chunk i+1 is in flight while
            // chunk i is stored
            constexpr int kChunks = BN / 32 / kEpiHalves;
            uint32_t r[2][32];
            tmem_ld_x32(taddr, r[0]);
            tc_wait_ld(r[0]);
#pragma unroll
            for (int ch = 0; ch < kChunks; ++ch) {
                if (ch + 1 < kChunks) tmem_ld_x32(taddr + (ch + 1) * 32, r[(ch + 1) & 1]);
                if (!std::is_same<MT, M24>::value && m_row) {
                    // row-major M: transpose the warp's 32 rows x 32 columns
                    // through shared memory (XOR-swizzled, conflict-free) so
                    // that 8 lanes write one row's 128 contiguous bytes
                    uint32_t* xp = xpose + (warp - 2) * 1024;
#pragma unroll
                    for (int c = 0; c < 32; ++c) xp[lane * 32 + (c ^ lane)] = r[ch & 1][c];
                    __syncwarp();
                    const int k0 = it.nb * BN + col0 + ch * 32 + (lane & 7) * 4;
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int row_w = 4 * i + (lane >> 3);  // row within the warp's 32
                        const int c0 = (lane & 7) * 4;
                        uint32_t v[4];
#pragma unroll
                        for (int j = 0; j < 4; ++j) v[j] = xp[row_w * 32 + ((c0 + j) ^ row_w)];
                        const long long pr = static_cast<long long>(it.mb) * kBM + quarter * 32 + row_w;
                        if constexpr (!std::is_same<MT, M24>::value)
                            if (pr < P && k0 < kp) store4_row<MT>(Mw, v, P, pr, k0, kp, it.e, m_pol);
                    }
                    __syncwarp();
                } else if (p < P) {
                    if constexpr (std::is_same<MT, M24>::value)
                        store32_m24(static_cast<unsigned char*>(d.Mw), r[ch & 1], p, it.nb * BN + col0 + ch * 32,
                                    kg_count, it.e, d.E, m_lo, m_pol);
                    else
                        store32<MT>(Mw, r[ch & 1], P, p, it.nb * BN + col0 + ch * 32, kg_count, it.e, m_pol);
                }
                if (ch + 1 < kChunks) tc_wait_ld(r[(ch + 1) & 1]);
            }
            tc_fence_before();
            mbar_arrive(&tempty[acc]);
            if (d.discard_v) {
                // this tile consumed every granule of its 128 rows of V, and
                // no other tile reads them: drop the lines without write-back
                const int et = (warp - 2) * 32 + lane, n_et = 128 * kEpiHalves;
                const int rows = min(kBM, d.v_pp - it.mb * kBM);   // a multiple of 8: whole lines
                const int lpg = rows / 8;
                const unsigned char* vb = static_cast<const unsigned char*>(d.V) +
                                          ((static_cast<long long>(it.e) * d.v_cg) * d.v_pp + static_cast<long long>(it.mb) * kBM) * 16;
                for (int i = et; i < d.v_cg * lpg; i += n_et) {
                    const int g = i / lpg, l = i - g * lpg;
                    discard_l2_line(vb + static_cast<long long>(g) * d.v_pp * 16 + l * 128);
                }
            }
            if (++acc == 2) {
                acc = 0;
                acc_phase ^= 1u;
            }
        }
    }

    __syncthreads();
    if (*abort_flag) {
        // let any copy or MMA still in flight land before the CTA retires
        const unsigned long long t0 = globaltimer_ns();
        while (globaltimer_ns() - t0 < 2000000ull) {
        }
    }
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem_base, Cfg::kTmemCols);
    }
}

template <int BN, bool BF16, class MT, bool RESB>
__global__ void __launch_bounds__(kGemmThreads, 1) wino_gemm_kernel(const __grid_constant__ GemmDesc d, DevErr* err) {
    gemm_body<BN, BF16, MT, RESB>(&d, 1, d.tiles, err);
}

template <int BN, bool BF16, class MT>
__global__ void __launch_bounds__(kGemmThreads, 1)
    wino_gemm_grouped(const GemmDesc* __restrict__ descs, int ndesc, long long total_tiles, DevErr* err) {
    gemm_body<BN, BF16, MT, false>(descs, ndesc, total_tiles, err);
}

template <int BN, bool BF16, class MT, bool RESB>
cudaError_t gemm_launch_r(const GemmDesc& d, int grid, DevErr* err, cudaStream_t s) {
    using Cfg = GemmCfg<BN, RESB>;
    auto kern = wino_gemm_kernel<BN, BF16, MT, RESB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg::kSmemRow);
    if (e != cudaSuccess) return e;
    return launch_pdl(kern, dim3(grid), dim3(kGemmThreads), d.m_row ? Cfg::kSmemRow : Cfg::kSmem, s, d, err);
}

template <int BN, bool BF16, class MT>
cudaError_t gemm_launch(const GemmDesc& d, int grid, DevErr* err, cudaStream_t s) {
    return d.resb ? gemm_launch_r<BN, BF16, MT, true>(d, grid, err, s) : gemm_launch_r<BN, BF16, MT, false>(d, grid, err, s);
}

template <int BN, bool BF16, class MT>
cudaError_t gemm_grouped_launch(const GemmDesc* descs, int ndesc, long long total, int grid, DevErr* err,
                                cudaStream_t s) {
    auto kern = wino_gemm_grouped<BN, BF16, MT>;
    // grouped problems write granule-layout M
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, GemmCfg<BN>::kSmemRow);
    if (e != cudaSuccess) return e;
    return launch_pdl(kern, dim3(grid), dim3(kGemmThreads), GemmCfg<BN>::kSmem, s, descs, ndesc, total, err);
}

// One template instance per (BN, operand type, M type); `single` selects the
// one-problem kernel (descriptor by value) or the grouped one (device array).
// 24-bit M is written by fp16-operand GEMMs only (F(4x3) with fp16 tensors).
template <int BN, class MT>
cudaError_t dispatch_single_or_grouped(bool bf, bool single, const GemmDesc* d, int ndesc, long long total, int grid,
                                       DevErr* err, cudaStream_t s) {
    if (single) return bf ? gemm_launch<BN, true, MT>(*d, grid, err, s) : gemm_launch<BN, false, MT>(*d, grid, err, s);
    return bf ? gemm_grouped_launch<BN, true, MT>(d, ndesc, total, grid, err, s)
              : gemm_grouped_launch<BN, false, MT>(d, ndesc, total, grid, err, s);
}

template <int BN>
cudaError_t dispatch_types(bool bf, MType mt, bool single, const GemmDesc* d, int ndesc, long long total, int grid,
                           DevErr* err, cudaStream_t s) {
    switch (mt) {
        case MType::F32: return dispatch_single_or_grouped<BN, float>(bf, single, d, ndesc, total, grid, err, s);
        case MType::F16: return dispatch_single_or_grouped<BN, __half>(bf, single, d, ndesc, total, grid, err, s);
        case MType::F24:
            if (bf) return cudaErrorNotSupported;
            return single ? gemm_launch<BN, false, M24>(*d, grid, err, s)
                          : gemm_grouped_launch<BN, false, M24>(d, ndesc, total, grid, err, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t dispatch(int bn, bool bf, MType mt, bool single, const GemmDesc* d, int ndesc, long long total, int grid,
                     DevErr* err, cudaStream_t s) {
    switch (bn) {
        case 32: return dispatch_types<32>(bf, mt, single, d, ndesc, total, grid, err, s);
        case 64: return dispatch_types<64>(bf, mt, single, d, ndesc, total, grid, err, s);
        case 128: return dispatch_types<128>(bf, mt, single, d, ndesc, total, grid, err, s);
        case 256: return dispatch_types<256>(bf, mt, single, d, ndesc, total, grid, err, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace

CUresult encode_tiled(CUtensorMap* map, CUtensorMapDataType dt, cuuint32_t rank, void* addr, const cuuint64_t* dims,
                      const cuuint64_t* strides_bytes, const cuuint32_t* box, CUtensorMapSwizzle swz) {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p)
            return CUDA_ERROR_NOT_FOUND;
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    cuuint32_t elem_strides[5] = {1, 1, 1, 1, 1};
    return fn(map, dt, rank, addr, dims, strides_bytes, box, elem_strides, CU_TENSOR_MAP_INTERLEAVE_NONE, swz,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
}

int gemm_smem_bytes(int bn) {
    switch (bn) {
        case 32: return GemmCfg<32>::kSmem;
        case 64: return GemmCfg<64>::kSmem;
        case 128: return GemmCfg<128>::kSmem;
        default: return GemmCfg<256>::kSmem;
    }
}

cudaError_t make_gemm_desc(GemmDesc& d, OpType op, int E, long long P, int K, int Kp, int Cp, const void* V,
                           const void* U, void* Mw, MType mt, int bn, bool m_row) {
    if (bn != 32 && bn != 64 && bn != 128 && bn != 256) return cudaErrorInvalidValue;
    if (P <= 0 || P > 0x7fffffffLL || Cp % 8 != 0 || Kp % 8 != 0) return cudaErrorInvalidValue;
    if (mt == MType::F24 && (m_row || op != OpType::F16)) return cudaErrorNotSupported;
    d.Mw = Mw;
    d.P = static_cast<int>(P);
    d.kg_count = mt == MType::F32 ? Kp / 4 : Kp / 8;
    d.m_lo = m24_lo_offset(E, P, Kp);
    d.m_row = m_row ? 1 : 0;
    d.kp = Kp;
    d.keep_m = 0;   // plan_gemm decides for single launches; grouped ones stream M
    d.V = V;
    d.v_cg = Cp / 8;
    d.v_pp = static_cast<int>(round_rows(P));
    d.discard_v = 0;
    d.resb = 0;      // plan_gemm decides for single launches; grouped ones hand out items round robin
    d.m_blocks = static_cast<int>((P + kBM - 1) / kBM);
    d.n_blocks = (K + bn - 1) / bn;
    d.k_blocks = (Cp + kBK - 1) / kBK;
    d.E = E;
    d.tile_begin = 0;
    d.tiles = static_cast<long long>(E) * d.m_blocks * d.n_blocks;
    if (d.tiles >= (1LL << 31)) return cudaErrorInvalidValue;
    d.fd_mb = make_fastdiv(static_cast<uint32_t>(d.m_blocks));
    d.fd_nb = make_fastdiv(static_cast<uint32_t>(d.n_blocks));
    const CUtensorMapDataType dt = op == OpType::BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    // V[E][CG][Pp][8] and U[E][CG][Kp][8] viewed as rows of 64 elements (8
    // tiles or output channels x one granule = 128 contiguous bytes): a box of
    // 8 granules x 16 rows (V) or BN/8 rows (U) fills shared memory in the
    // same [granule][row][8] order as 16-byte rows would, with full-line reads
    const cuuint64_t CG = static_cast<cuuint64_t>(Cp / 8);
    const cuuint64_t Pr = static_cast<cuuint64_t>(round_rows(P)) / 8;
    const cuuint64_t Kr = static_cast<cuuint64_t>(Kp) / 8;
    {
        cuuint64_t dims[4] = {64, Pr, CG, static_cast<cuuint64_t>(E)};
        cuuint64_t strides[3] = {128, Pr * 128, CG * Pr * 128};
        cuuint32_t box[4] = {64, kBM / 8, 8, 1};
        if (encode_tiled(&d.tmA, dt, 4, const_cast<void*>(V), dims, strides, box, CU_TENSOR_MAP_SWIZZLE_NONE) !=
            CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    {
        cuuint64_t dims[4] = {64, Kr, CG, static_cast<cuuint64_t>(E)};
        cuuint64_t strides[3] = {128, Kr * 128, CG * Kr * 128};
        cuuint32_t box[4] = {64, static_cast<cuuint32_t>(bn / 8), 8, 1};
        if (encode_tiled(&d.tmB, dt, 4, const_cast<void*>(U), dims, strides, box, CU_TENSOR_MAP_SWIZZLE_NONE) !=
            CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    return cudaSuccess;
}

cudaError_t plan_gemm(GemmPlan& gp, OpType op, int E, long long P, int K, int Kp, int Cp, const void* V,
                      const void* U, void* Mw, MType mt, int bn, int num_sms, bool m_row) {
    cudaError_t e = make_gemm_desc(gp.desc, op, E, P, K, Kp, Cp, V, U, Mw, mt, bn, m_row);
    if (e != cudaSuccess) return e;
    // M of this launch within the L2 size: kept there for the output transform
    // that reads it next (32 x 512 x 28^2 -> 512 F(4x3): 87 MB in 24 bits); larger M is streamed out
    gp.desc.keep_m = m_bytes(mt, E, P, Kp) <= l2_cache_bytes();
    // V has one reader per tile when one block covers all output channels;
    // WG_CONV2D_KEEP_WORKSPACE=1 keeps it (to read the workspace back)
    const char* keep_ws = std::getenv("WG_CONV2D_KEEP_WORKSPACE");
    gp.desc.discard_v = gp.desc.n_blocks == 1 && !(keep_ws && std::atoi(keep_ws) != 0);
    // U block of one (element, channel block) within the resident budget: it
    // stays in shared memory over consecutive tile blocks instead of being
    // reloaded from L2 for every work item (32 x 256 x 56^2 -> 256: 226 of
    // the 339 MB of operand loads); WG_CONV2D_GEMM_RESIDENT_U=0 turns it off
    const char* res = std::getenv("WG_CONV2D_GEMM_RESIDENT_U");
    gp.desc.resb = !(res && res[0] == '0') &&
                   static_cast<long long>(gp.desc.k_blocks) * bn * kBK * 2 <= kResBBytes &&
                   gp.desc.tiles >= num_sms;
    gp.op = op;
    gp.bn = bn;
    gp.mt = mt;
    gp.grid = static_cast<int>(std::min<long long>(gp.desc.tiles, num_sms));
    gp.smem_bytes = gemm_smem_bytes(bn);
    return cudaSuccess;
}

cudaError_t launch_gemm(const GemmPlan& gp, DevErr* err, cudaStream_t stream) {
    return dispatch(gp.bn, gp.op == OpType::BF16, gp.mt, true, &gp.desc, 1, gp.desc.tiles, gp.grid, err, stream);
}

cudaError_t launch_gemm_grouped(const GemmDesc* descs, int ndesc, long long total_tiles, OpType op, MType mt, int bn,
                                int grid, DevErr* err, cudaStream_t stream) {
    return dispatch(bn, op == OpType::BF16, mt, false, descs, ndesc, total_tiles, grid, err, stream);
}

}  // namespace wg
