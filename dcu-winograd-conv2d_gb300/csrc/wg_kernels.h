// Host-side launchers of the operator's CUDA kernels.  All pointers are
// device pointers; every launcher enqueues work on `stream` and returns the
// cudaError_t of the launch.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace wg {

// Device error word written by kernels whose bounded waits give up.
struct DevErr {
    unsigned int code;   // first failing wait site (0 = none)
    unsigned int count;  // number of failures
};

// Transform family: which interpolation points F(4x3) uses.
enum class Xform : int { F2 = 0, F4 = 1, F4Ref = 2 };

inline int xform_m(Xform x) { return x == Xform::F2 ? 2 : 4; }
inline int xform_alpha(Xform x) { return xform_m(x) + 2; }

enum class OpType : int { F16 = 0, BF16 = 1 };

// Storage of the GEMM result M (fp32 accumulators):
//   F16  M[e][Kp/8][P][8] fp16 (F(2x3));
//   F32  M[e][Kp/4][P][4] fp32 (granule layout), or M[e][P][Kp] row-major for
//        the channels-last output path;
//   F24  each fp32 value rounded to nearest at 24 bits and split in two
//        planes: its upper 16 bits in H[NB][Kp/8][E][64][8] (16-byte granules
//        of 8 channels, blocks of 64 tiles, NB = ceil(P/64)) and its next 8
//        bits in L[NB][Kp/8][E][64][8] (8-byte granules), L right after H.
//        Relative rounding 2^-17 (fp16 M: 2^-12) for 3/4 of the fp32 bytes;
//        the F(4x3) default.
enum class MType : int { F16 = 0, F32 = 1, F24 = 2 };

inline const char* mtype_name(MType t) { return t == MType::F16 ? "fp16" : t == MType::F32 ? "fp32" : "24-bit"; }

// Geometry of one convolution as the Winograd path sees it.
struct Geom {
    int n, c, h, w, k;   // NCHW input, K output channels
    int pad_h, pad_w;    // 3x3 filter, stride 1
    int oh, ow;          // output size
    int m, alpha;        // output tile size and input tile size
    int tiles_h, tiles_w;
    long long P;         // tiles in the batch = n * tiles_h * tiles_w
    int cp;              // C padded to a multiple of 8 (U and V row length)
    int kp;              // K padded to a multiple of 8 (M row length)
};

Geom make_geom(int n, int c, int h, int w, int k, int pad_h, int pad_w, int m);

// Rows of V per element and granule: P rounded up to 8 (TMA reads V in
// 128-byte rows of 8 tiles).
inline long long round_rows(long long P) { return (P + 7) / 8 * 8; }

// 24-bit M is stored in blocks of kM24Tiles tiles (the output transform's
// work item): H[NB][Kp/8][E][kM24Tiles][8] of 16-bit words, then
// L[NB][Kp/8][E][kM24Tiles][8] of bytes, NB = ceil(P / kM24Tiles), so the E
// runs of one (tile block, granule) are one contiguous range in each plane
// and the granules of one tile block lie together.
constexpr int kM24Tiles = 64;
inline long long m24_blocks(long long P) { return (P + kM24Tiles - 1) / kM24Tiles; }

// Bytes of M for E elements, P tiles and Kp (a multiple of 8) channels.
inline long long m_bytes(MType t, long long E, long long P, long long Kp) {
    if (t == MType::F16) return E * P * Kp * 2;
    if (t == MType::F32) return E * P * Kp * 4;
    return E * m24_blocks(P) * kM24Tiles * Kp * 3;
}
// Byte offset of the low plane of 24-bit M.
inline long long m24_lo_offset(long long E, long long P, long long Kp) { return E * m24_blocks(P) * kM24Tiles * Kp * 2; }

// U[e][Cp/8][Kp][8] = G g G^T, from KCRS fp16 weights; fp32 arithmetic, result
// in the operand type; zero for c >= C or k >= K.
cudaError_t launch_filter_transform(Xform xf, OpType op, const void* weight, void* U, int K, int C, int Cp,
                                    cudaStream_t stream, bool w_bf16 = false);

// Per-tile power-of-two scale (F(4x3) scaling option): scale[p] = 2^-floor(log2 max|d|)
// over the tile's input patch in every channel; 1 for an all-zero patch.
cudaError_t launch_tile_scale(const Geom& g, const void* x, float* scale, cudaStream_t stream, bool x_bf16 = false);

// V[e][Cp/8][round_rows(P)][8] = B^T d B for the g.n images starting at x (x may point
// into a larger tensor that ends at x_end; the full tensor must start on a
// 16-byte boundary).  scale may be null.
cudaError_t launch_input_transform(Xform xf, OpType op, const Geom& g, const void* x, const void* x_end, void* V,
                                   const float* scale, DevErr* err, cudaStream_t stream, bool x_bf16 = false);

// Per-problem descriptors of the transform kernels (device-resident arrays of
// them drive the grouped launches that run many problems at once).
// Division by a runtime-invariant divisor d (1 <= d < 2^31) as a multiply
// and a shift, for dividends below 2^31 (Granlund and Montgomery's method):
// with l = ceil(log2 d), mul = ceil(2^(31+l) / d) < 2^32 and
// n / d = (n * mul) >> (31 + l) exactly for every n < 2^31.
struct FastDiv {
    uint32_t d = 1, mul = 0, shift = 0;
};
inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    if (d > 1) {
        uint32_t l = 0;
        while ((1u << l) < d) ++l;
        const uint32_t p = 31 + l;
        f.mul = static_cast<uint32_t>(((1ull << p) + d - 1) / d);
        f.shift = p - 32;
    }
    return f;
}
__host__ __device__ inline uint32_t fast_div(const FastDiv& f, uint32_t n) {
#ifdef __CUDA_ARCH__
    return f.d == 1 ? n : (__umulhi(n, f.mul) >> f.shift);
#else
    return f.d == 1 ? n : static_cast<uint32_t>((static_cast<uint64_t>(n) * f.mul) >> 32) >> f.shift;
#endif
}

struct InDesc {
    const __half* x;
    const __half* x_end;
    void* V;
    const float* scale;
    int C, H, W, pad_h, pad_w, tiles_h, tiles_w;
    long long Pp;
    int CG, tb, nbh, cb, stride_bytes;
    long long gx;         // work items along (image, tile-row block)
    int gy;               // work items along channel blocks (cb <= 32)
    long long blk_begin;  // first work item of this problem in a grouped launch
    FastDiv fd_gy, fd_nbh;   // item -> (image x tile-row block, channel block), -> (image, tile-row block)
    int words;               // rows read as aligned words (pad 1, W % M == 0, x 8-byte aligned)
};

struct OutDesc {
    const void* Mw;
    __half* out;
    const float* scale;
    int K, OH, OW, tiles_h, tiles_w;
    long long P;
    int KG;
    long long gx;         // work items along blocks of 64 tiles
    int gy;               // work items along granules
    long long blk_begin;
    int discard_m;        // M is read once here: drop its L2 lines without write-back
    long long m_lo;       // 24-bit M: byte offset of the low plane from Mw
    FastDiv fd_kg, fd_tw, fd_th;   // item -> (tile block, granule), tile -> (image, row, column)
};

// Descriptor of one problem's input transform and the dynamic shared memory
// of its (persistent, double-buffered) launch.
InDesc make_in_desc(const Geom& g, const void* x, const void* x_end, void* V, const float* scale, int* smem);
OutDesc make_out_desc(const Geom& g, MType mt, const void* Mw, void* out, const float* scale);
// Grouped launches: `blocks` = sum of gx*gy work items; descs device-resident,
// sorted by blk_begin; smem = the largest of the problems' *smem; `scaled` when
// any problem has a per-tile scale.
cudaError_t launch_input_transform_grouped(Xform xf, OpType op, const InDesc* descs, int ndesc, long long blocks,
                                           int smem, bool scaled, DevErr* err, cudaStream_t stream);
cudaError_t launch_output_transform_grouped(Xform xf, MType mt, const OutDesc* descs, int ndesc, long long blocks,
                                            DevErr* err, cudaStream_t stream);
// out[N][OH][OW][K] (channels-last, fp16) from the 24-bit granule-layout M
// of F(4x3): the arithmetic of launch_output_transform, other store order.
cudaError_t launch_output_transform_nhwc24(Xform xf, const Geom& g, const void* Mw, void* out, DevErr* err,
                                          cudaStream_t stream);

// out[N][K][OH][OW] = A^T M A from M stored as `mt` (granule layouts above);
// divides by scale[p] when scale is not null.
cudaError_t launch_output_transform(Xform xf, MType mt, const Geom& g, const void* Mw, void* out,
                                    const float* scale, DevErr* err, cudaStream_t stream, bool y_bf16 = false);

// ---- tcgen05 batched GEMM: M_e[P][K] = V_e[P][Cp] * U_e[K][Cp]^T -----------
// (operands and result in the 16-byte granule layouts above)
// One problem's GEMM: tensor maps of V and U, output, sizes, and its range of
// the global work index when several problems share one launch.
struct alignas(64) GemmDesc {
    CUtensorMap tmA;     // V
    CUtensorMap tmB;     // U
    void* Mw;
    int P, kg_count, m_blocks, n_blocks, k_blocks, E;
    int m_row;           // 1: M[e][P][Kp] (rows of output channels, NHWC output path)
    int kp;
    long long m_lo;      // 24-bit M: byte offset of the low plane from Mw
    int keep_m;          // M fits in L2: store it with the evict_last priority
    // V[E][v_cg][v_pp][8] is read by this GEMM only (one block of output
    // channels): its lines are discarded from L2 once a tile is done, so the
    // dirty lines are never written back to HBM
    const void* V;
    int v_cg, v_pp, discard_v;
    int resb;            // single launches: U block resident in shared memory, contiguous item ranges per CTA
    long long tile_begin;
    long long tiles;     // E * m_blocks * n_blocks (below 2^31)
    FastDiv fd_mb, fd_nb;   // division by m_blocks, n_blocks
};

struct GemmPlan {
    GemmDesc desc;
    int bn;              // 32, 64, 128 or 256
    int grid;
    int smem_bytes;
    MType mt;
    OpType op;
};

// Builds the tensor maps; V, U, M must stay at these addresses.
cudaError_t make_gemm_desc(GemmDesc& d, OpType op, int E, long long P, int K, int Kp, int Cp, const void* V,
                           const void* U, void* Mw, MType mt, int bn, bool m_row = false);
cudaError_t plan_gemm(GemmPlan& gp, OpType op, int E, long long P, int K, int Kp, int Cp, const void* V,
                      const void* U, void* Mw, MType mt, int bn, int num_sms, bool m_row = false);
cudaError_t launch_gemm(const GemmPlan& gp, DevErr* err, cudaStream_t stream);
// Many problems (same BN, operand and M types) in one persistent launch; descs
// device-resident (64-byte aligned), sorted by tile_begin.
cudaError_t launch_gemm_grouped(const GemmDesc* descs, int ndesc, long long total_tiles, OpType op, MType mt, int bn,
                                int grid, DevErr* err, cudaStream_t stream);
int gemm_smem_bytes(int bn);

// ---- NHWC (channels-last) input and output transforms ---------------------
// Input x[N][H][W][C] fp16 through one TMA box per work item (zero fill for
// the padding); writes the same V as launch_input_transform.
struct alignas(64) NhwcInDesc {
    CUtensorMap tmX;
    void* V;
    int C, H, W, pad_h, pad_w, tiles_h, tiles_w;
    long long Pp;
    int CG, tb, nbh, cb, bw, rows;
    long long gx;         // work items along (image, tile-row block)
    int gy;               // work items along channel blocks
    FastDiv fd_tw;        // tile of an item -> (tile row, tile column)
};
// cudaErrorNotSupported when C is not a multiple of 8 (TMA strides), the
// padded row width exceeds one TMA box (256) or two boxes do not fit in
// shared memory.
cudaError_t make_nhwc_in_desc(NhwcInDesc& d, const Geom& g, const void* x, void* V, int* smem);
// images [n_base, n_base + n_images) of the tensor; V holds their tiles from 0
cudaError_t launch_nhwc_input_transform(Xform xf, OpType op, const NhwcInDesc& d, int smem, int n_base, int n_images,
                                        DevErr* err, cudaStream_t stream);
// Output y[N][OH][OW][K] fp16 from row-major M[E][P][Kp] (fp32 for F(4x3)).
struct NhwcOutDesc {
    const void* Mw;
    __half* out;
    int K, Kp, OH, OW, tiles_h, tiles_w;
    long long P;
    int tpt, tpc;         // threads per tile, tiles per CTA
    int discard_m;        // drop M's lines from L2 once read (set by the launcher)
    FastDiv fd_tpt, fd_tw, fd_th, fd_tpc, fd_lpr;   // divisions by tpt, tiles_w, tiles_h, tpc, M lines per row
};
NhwcOutDesc make_nhwc_out_desc(const Geom& g, const void* Mw, void* out);
cudaError_t launch_nhwc_output_transform(Xform xf, MType mt, const NhwcOutDesc& d, cudaStream_t stream);

// ---- fused F(2x3): input transform + tcgen05 GEMM + output transform ------
struct FusedPlan {
    CUtensorMap tmU;
    int m_blocks, n_blocks, c_chunks;
    int stg_ch_bytes;    // staged input bytes per channel of one chunk
    int nbuf;            // staging buffers (2 = copies one chunk ahead)
    int smem_bytes;
    OpType op;
    bool io_bf16;        // input and output tensors bf16 (operands then bf16 too)
};

// cudaErrorNotSupported when the staged rows of one CTA do not fit in shared
// memory (very wide images); the caller then uses the non-fused path.
cudaError_t plan_fused2x3(FusedPlan& fp, OpType op, const Geom& g, const void* U);
cudaError_t launch_fused2x3(const FusedPlan& fp, const Geom& g, const void* x, const void* x_end, void* out,
                            DevErr* err, cudaStream_t stream);

// ---- row-Winograd F(4x3), fully fused (1-D F(4,3) along the width) --------
struct RowPlan {
    CUtensorMap tmU;                   // U1 filter tiles
    CUtensorMap tmX;                   // interleaved kernel: the NHWC input rows
    alignas(8) unsigned char geo[96];  // kernel geometry (row4x3.cu)
    int c, k;
    int cp16, kp64;
    int smem_bytes;
    int interleaved;                   // 1: channel-interleaved kernel (NHWC rows)
    int out_nhwc;                      // interleaved kernel: y is NHWC
    int cs;                            // interleaved kernel: channels of the input pixels (C, a multiple of 16)
};
// Channel-planar kernel over NCHW input.  cudaErrorNotSupported for padding
// above 64, more than 256 output columns or when the stages do not fit in
// shared memory.  U may be null (a size probe).
cudaError_t plan_row4x3(RowPlan& rp, const Geom& g, const void* U);
// Channel-interleaved kernel over x[n][h][w][cs]; cudaErrorNotSupported for
// more than 248 output columns.  U may be null (a size probe).
cudaError_t plan_row4x3i(RowPlan& rp, const Geom& g, const void* U, bool out_nhwc);
// tensor map of the interleaved kernel's input x[n_total][h][w][cs]
cudaError_t bind_row4x3i_input(RowPlan& rp, const void* x_nhwc, int cs, int h, int w, int n_total);
long long row4x3_filter_bytes(const RowPlan& rp);
int row4x3_threads(const RowPlan& rp);                      // threads per CTA of the planned kernel
long long row4x3_items(const RowPlan& rp, int n_images);   // CTA work items of n images
// U1[e*3 + r][Cp16/8][Kp64][8] fp16 from KCRS fp16 weights
cudaError_t launch_row4x3_filter(const RowPlan& rp, const void* weight, void* U, cudaStream_t stream);
// planar kernel: images [0, n_images) of the tensor starting at x (which ends at x_end)
cudaError_t launch_row4x3(const RowPlan& rp, const void* x, const void* x_end, void* out, int n_images, DevErr* err,
                          cudaStream_t stream);
// interleaved kernel: images [n_base, n_base + n_images) of the bound input into
// out (which holds those images)
cudaError_t launch_row4x3i(const RowPlan& rp, void* out, int n_base, int n_images, DevErr* err, cudaStream_t stream);

// L2 size of the current device in bytes.
long long l2_cache_bytes();

// Tensor-map encoder from the driver (resolved once through the runtime).
CUresult encode_tiled(CUtensorMap* map, CUtensorMapDataType dt, cuuint32_t rank, void* addr, const cuuint64_t* dims,
                      const cuuint64_t* strides_bytes, const cuuint32_t* box, CUtensorMapSwizzle swz);

}  // namespace wg
