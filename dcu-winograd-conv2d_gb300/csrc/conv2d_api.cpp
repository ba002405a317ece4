// C ABI of the operator: descriptor -> plan -> launches.
//
// Mirrors the reference's operator API (include/conv2d.h:8-42,
// src/conv2d.cpp:1-133): getParamsize returns the size of the opaque param
// blob, getkernelInfo fills it (selection + device workspace, as
// src/conv2d.cpp:24-116 does), conv2d_fp16 runs the selected algorithm
// (src/conv2d.cpp:118-133).  Differences, each deliberate:
//   * sizes are computed in 64-bit arithmetic (the reference's unsigned 32-bit
//     products overflow for large batches);
//   * no file-static state is mutated (the reference rewrites its tile
//     constants on the F(2x3)-non-fused branch, src/conv2d.cpp:89-92);
//   * unsupported descriptors return a status code;
//   * the filter transform runs once per weight set (first call) instead of
//     on every call, and the workspace can be released (conv2d_destroy).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/conv2d.h"
#include "wg_kernels.h"
#include "wg_plan.h"

namespace wg {

namespace {

thread_local int t_last_status = CONV2D_OK;
thread_local std::string t_last_msg;

int fail(int status, const std::string& msg) {
    t_last_status = status;
    t_last_msg = msg;
    return status;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(CONV2D_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int env_int(const char* name, int dflt) {
    const char* v = std::getenv(name);
    if (!v || !*v) return dflt;
    return std::atoi(v);
}

int env_algo(int dflt) {
    const char* v = std::getenv("WG_CONV2D_ALGO");
    if (!v || !*v) return dflt;
    std::string s(v);
    if (s == "ref" || s == "reference") return CONV2D_ALGO_REFERENCE;
    if (s == "4x3") return CONV2D_ALGO_4X3_NON_FUSED;
    if (s == "2x3") return CONV2D_ALGO_2X3_NON_FUSED;
    if (s == "fused" || s == "2x3_fused") return CONV2D_ALGO_2X3_FUSED;
    if (s == "auto") return CONV2D_ALGO_AUTO;
    if (s == "row" || s == "4x3_row") return CONV2D_ALGO_4X3_ROW;
    return dflt;
}

}  // namespace

int select_reference64(unsigned long long n, unsigned long long c, unsigned long long h, unsigned long long w,
                       unsigned long long k, unsigned long long r, unsigned long long s, unsigned long long oh,
                       unsigned long long ow) {
    // src/conv2d.cpp:76-114 with the tile constants of a first call:
    // fused F(2x3) when the image is at least 10x the filter, F(2x3)
    // non-fused when the F(4x3) filter workspace exceeds 4x the input one,
    // else F(4x3).
    const unsigned long long image = n * c * h * w;
    const unsigned long long filter = k * c * r * s;
    const unsigned long long tiles4 = n * ((oh + 3) / 4) * ((ow + 3) / 4);
    const unsigned long long U = 36ull * k * c;
    const unsigned long long V = 36ull * tiles4 * c;
    if (image >= 10ull * filter) return CONV2D_ALGO_2X3_FUSED;
    if (U > 4ull * V) return CONV2D_ALGO_2X3_NON_FUSED;
    return CONV2D_ALGO_4X3_NON_FUSED;
}

int validate_problem(const problem_t* pr) {
    if (!pr) return fail(CONV2D_ERR_INVALID, "null problem");
    if (!pr->in || !pr->weight || !pr->out) return fail(CONV2D_ERR_INVALID, "null tensor pointer");
    if (!pr->n || !pr->c || !pr->h || !pr->w || !pr->k) return fail(CONV2D_ERR_INVALID, "zero dimension");
    if (pr->r != 3 || pr->s != 3) return fail(CONV2D_ERR_UNSUPPORTED, "only 3x3 filters are supported");
    if (pr->u != 1 || pr->v != 1) return fail(CONV2D_ERR_UNSUPPORTED, "only stride 1 is supported");
    if (pr->p > 64 || pr->q > 64) return fail(CONV2D_ERR_UNSUPPORTED, "padding above 64");
    const long long oh = static_cast<long long>(pr->h) + 2LL * pr->p - 2;
    const long long ow = static_cast<long long>(pr->w) + 2LL * pr->q - 2;
    if (oh <= 0 || ow <= 0) return fail(CONV2D_ERR_INVALID, "empty output");
    if (pr->c > 65535 || pr->k > 65535 || pr->h > 65535 || pr->w > 65535)
        return fail(CONV2D_ERR_UNSUPPORTED, "dimension above 65535");
    const long long tiles = static_cast<long long>(pr->n) * ((oh + 1) / 2) * ((ow + 1) / 2);
    if (tiles > 0x7fffffffLL) return fail(CONV2D_ERR_UNSUPPORTED, "more than 2^31 tiles");
    return CONV2D_OK;
}

int options_default(conv2d_options_t* o) {
    std::memset(o, 0, sizeof(*o));
    // the per-shape autotuner by default: among the reference's three
    // algorithms (and the row F(4x3) kernel) the fastest measured for the
    // shape, the reference rule's pick unless another is >3% faster;
    // WG_CONV2D_ALGO=ref keeps the reference rule itself
    o->algo = env_algo(CONV2D_ALGO_AUTO);
    o->operand_bf16 = env_int("WG_CONV2D_BF16", 0) ? 1 : 0;
    o->tile_scaling = env_int("WG_CONV2D_TILE_SCALING", 0) ? 1 : 0;
    o->f4_points = env_int("WG_CONV2D_F4_REFERENCE_POINTS", 0) ? 1 : 0;
    o->filter_policy = env_int("WG_CONV2D_FILTER_EVERY_CALL", 0) ? 1 : 0;
    o->gemm_bn = env_int("WG_CONV2D_GEMM_BN", 0);
    const char* l2 = std::getenv("WG_CONV2D_L2_CHUNK_BYTES");
    o->l2_chunk_bytes = (l2 && *l2) ? std::atoll(l2) : 0;
    o->io_bf16 = env_int("WG_CONV2D_IO_BF16", 0) ? 1 : 0;
    o->layout_nhwc = env_int("WG_CONV2D_NHWC", 0) ? 1 : 0;
    o->m_fp32 = env_int("WG_CONV2D_M_FP32", 0) ? 1 : 0;
    return CONV2D_OK;
}

int default_bn(int K) {
    if (K <= 32) return 32;
    if (K <= 64) return 64;
    if (K <= 128) return 128;
    // prefer the tile with the least padding waste; ties go to the wider tile
    const int w256 = ((K + 255) / 256) * 256 - K;
    const int w128 = ((K + 127) / 128) * 128 - K;
    return w256 <= w128 ? 256 : 128;
}

Plan::~Plan() { release(); }

void Plan::release() {
    if (host_graph) cudaGraphExecDestroy(host_graph);
    host_graph = nullptr;
    if (host_in_stream) cudaStreamDestroy(host_in_stream);
    if (host_out_stream) cudaStreamDestroy(host_out_stream);
    if (host_cap_stream) cudaStreamDestroy(host_cap_stream);
    host_cap_stream = nullptr;
    for (cudaEvent_t& e : host_ev)
        if (e) cudaEventDestroy(e);
    host_in_stream = host_out_stream = nullptr;
    if (ws) cudaFree(ws);
    ws = nullptr;
    U = V = Mw = nullptr;
    scale = nullptr;
    err = nullptr;
}

int Plan::build(const problem_t* pr, const conv2d_options_t* opt_in) {
    int st = validate_problem(pr);
    if (st) return st;
    prob = *pr;
    if (opt_in)
        opt = *opt_in;
    else
        options_default(&opt);
    if (reinterpret_cast<uintptr_t>(pr->in) % 16 != 0)
        return fail(CONV2D_ERR_UNSUPPORTED, "input pointer must be 16-byte aligned");
    if (cudaGetDevice(&device) != cudaSuccess) return fail(CONV2D_ERR_CUDA, "no CUDA device");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    num_sms = sms > 0 ? sms : 1;

    const unsigned oh = pr->h + 2 * pr->p - 2, ow = pr->w + 2 * pr->q - 2;
    algo = opt.algo;
    if (algo == CONV2D_ALGO_REFERENCE || algo == CONV2D_ALGO_AUTO)
        algo = select_reference64(pr->n, pr->c, pr->h, pr->w, pr->k, pr->r, pr->s, oh, ow);
    if (opt.algo == CONV2D_ALGO_AUTO) {
        int a = algo, bn = 0;
        autotune_choose(*pr, opt, algo, &a, &bn);
        algo = a;
        if (bn) opt.gemm_bn = bn;
    }
    if (algo < 0 || (algo > 2 && algo != CONV2D_ALGO_4X3_ROW)) return fail(CONV2D_ERR_INVALID, "bad algorithm");

    op = opt.operand_bf16 ? OpType::BF16 : OpType::F16;
    nhwc = opt.layout_nhwc != 0;
    if (nhwc) {
        if (opt.io_bf16 || opt.tile_scaling)
            return fail(CONV2D_ERR_UNSUPPORTED, "NHWC tensors are fp16 without per-tile scaling");
        if (algo == CONV2D_ALGO_2X3_FUSED) algo = CONV2D_ALGO_2X3_NON_FUSED;  // the fused kernel reads NCHW
    }
    if (algo == CONV2D_ALGO_2X3_FUSED) {
        // the fused kernel stages the input rows of 128 tiles in shared memory;
        // for very wide images they do not fit and F(2x3) runs non-fused
        FusedPlan probe{};
        const Geom g2 = make_geom(pr->n, pr->c, pr->h, pr->w, pr->k, pr->p, pr->q, 2);
        if (plan_fused2x3(probe, op, g2, nullptr) == cudaErrorNotSupported) algo = CONV2D_ALGO_2X3_NON_FUSED;
        cudaGetLastError();
    }
    if (algo == CONV2D_ALGO_4X3_ROW) {
        // fp16 tensors and operands with the {0, +-1, 1/2, -2} points only; NCHW
        // tensors run the channel-planar kernel (the staged rows of one block
        // of output rows must fit in shared memory), NHWC ones the
        // channel-interleaved kernel (at most 248 output columns, C a multiple
        // of 16); otherwise F(4x3) runs non-fused
        const Geom g4 = make_geom(pr->n, pr->c, pr->h, pr->w, pr->k, pr->p, pr->q, 4);
        const cudaError_t pe = nhwc ? (pr->c % 16 == 0 ? plan_row4x3i(row, g4, nullptr, true) : cudaErrorNotSupported)
                                    : plan_row4x3(row, g4, nullptr);
        if (opt.io_bf16 || opt.operand_bf16 || opt.tile_scaling || opt.f4_points || pe != cudaSuccess)
            algo = CONV2D_ALGO_4X3_NON_FUSED;
        cudaGetLastError();
    }
    const int m = (algo == CONV2D_ALGO_4X3_NON_FUSED || algo == CONV2D_ALGO_4X3_ROW) ? 4 : 2;
    xf = m == 2 ? Xform::F2 : (opt.f4_points ? Xform::F4Ref : Xform::F4);
    // bf16 tensors: bf16 operands for F(2x3) (sums of +-1 multiples stay in
    // range), fp16 operands with per-tile scaling for F(4x3) (bf16 operands
    // lose ~10x accuracy there); M in fp32 either way
    if (opt.io_bf16) op = m == 2 ? OpType::BF16 : OpType::F16;
    // M: 24-bit for F(4x3) with fp16 operands (fp16 M would add ~1e-2
    // through A^T m A; channels-last outputs too, from the same granule
    // layout), fp32 where asked, for bf16 operands and for F(2x3) with bf16
    // tensors, fp16 for F(2x3) otherwise.  Channels-last F(2x3) and fp32 M
    // take the row-major M of the NHWC output transform.
    if (algo == CONV2D_ALGO_4X3_ROW)
        mt = MType::F16;   // no M
    else if (m == 4)
        mt = (opt.m_fp32 || op == OpType::BF16) ? MType::F32 : MType::F24;
    else
        mt = opt.io_bf16 ? MType::F32 : MType::F16;
    scaling = (m == 4) && (opt.tile_scaling || opt.io_bf16) && algo != CONV2D_ALGO_4X3_ROW;
    g = make_geom(pr->n, pr->c, pr->h, pr->w, pr->k, pr->p, pr->q, m);
    const int E = g.alpha * g.alpha;
    const long long op_bytes = 2;
    if (!single_kernel() && !nhwc) {
        // the input transform stages whole input rows of 8 channels, twice
        int in_smem = 0;
        make_in_desc(g, pr->in, pr->in, nullptr, nullptr, &in_smem);
        if (in_smem > 232448) return fail(CONV2D_ERR_UNSUPPORTED, "input rows too wide for the staged input transform");
    }

    // image chunking keeps V and M of one chunk L2-resident between kernels
    chunk_n = static_cast<int>(pr->n);
    if (!single_kernel() && opt.l2_chunk_bytes > 0) {
        const long long tiles_img = static_cast<long long>(g.tiles_h) * g.tiles_w;
        const long long per_img = static_cast<long long>(E) * tiles_img * g.cp * op_bytes + m_bytes(mt, E, tiles_img, g.kp);
        chunk_n = static_cast<int>(std::max(1LL, std::min<long long>(pr->n, opt.l2_chunk_bytes / std::max(1LL, per_img))));
    }
    const long long Pc = static_cast<long long>(chunk_n) * g.tiles_h * g.tiles_w;

    // one workspace: U | V | M | scale | device error word (256-byte aligned parts)
    auto al = [](long long b) { return (b + 255) / 256 * 256; };
    u_bytes = algo == CONV2D_ALGO_4X3_ROW ? row4x3_filter_bytes(row) : static_cast<long long>(E) * g.kp * g.cp * op_bytes;
    const long long bU = al(u_bytes);
    long long bV = 0, bM = 0, bS = 0;
    if (!single_kernel()) {
        bV = al(static_cast<long long>(E) * round_rows(Pc) * g.cp * op_bytes);
        bM = al(m_bytes(mt, E, Pc, g.kp));
        if (scaling) bS = al(Pc * 4);
    }
    const long long bE = 256;
    ws_bytes = bU + bV + bM + bS + bE;
    cudaError_t ce = cudaMalloc(&ws, static_cast<size_t>(ws_bytes));
    if (ce != cudaSuccess) {
        ws = nullptr;
        cudaGetLastError();
        return fail(CONV2D_ERR_NOMEM, "workspace cudaMalloc failed");
    }
    char* b = static_cast<char*>(ws);
    U = b;
    V = bV ? b + bU : nullptr;
    Mw = bM ? b + bU + bV : nullptr;
    scale = bS ? reinterpret_cast<float*>(b + bU + bV + bM) : nullptr;
    err = reinterpret_cast<DevErr*>(b + bU + bV + bM + bS);
    ce = cudaMemset(err, 0, sizeof(DevErr));
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemset");

    if (algo == CONV2D_ALGO_2X3_FUSED) {
        ce = plan_fused2x3(fused, op, g, U);
        fused.io_bf16 = opt.io_bf16 != 0;
        if (ce != cudaSuccess) return cuda_fail(ce, "fused plan");
        launches = 1;
        info_grid = static_cast<unsigned>(fused.m_blocks * fused.n_blocks);
        info_threads = 320;
        info_smem = fused.smem_bytes;
    } else if (algo == CONV2D_ALGO_4X3_ROW) {
        if (nhwc) {
            ce = plan_row4x3i(row, g, U, true);
            if (ce == cudaSuccess)
                ce = bind_row4x3i_input(row, pr->in, static_cast<int>(pr->c), static_cast<int>(pr->h),
                                        static_cast<int>(pr->w), static_cast<int>(pr->n));
        } else {
            ce = plan_row4x3(row, g, U);
        }
        if (ce != cudaSuccess) return cuda_fail(ce, "row F(4x3) plan");
        launches = 1;
        info_grid = static_cast<unsigned>(std::min<long long>(row4x3_items(row, static_cast<int>(pr->n)), num_sms));
        info_threads = static_cast<unsigned>(row4x3_threads(row));
        info_smem = row.smem_bytes;
    } else {
        if (nhwc) {
            ce = make_nhwc_in_desc(nh_in, g, pr->in, V, &nh_smem);
            if (ce == cudaErrorNotSupported)
                return fail(CONV2D_ERR_UNSUPPORTED,
                            "NHWC needs C a multiple of 8 and rows within one TMA box (about 250 columns)");
            if (ce != cudaSuccess) return cuda_fail(ce, "NHWC tensor map");
        }
        const int bn = opt.gemm_bn ? opt.gemm_bn : default_bn(g.k);
        ce = plan_gemm(gemm_full, op, E, Pc, g.k, g.kp, g.cp, V, U, Mw, mt, bn, num_sms, m_row());
        if (ce != cudaSuccess) return cuda_fail(ce, "GEMM plan (tensor maps)");
        n_chunks = (static_cast<int>(pr->n) + chunk_n - 1) / chunk_n;
        const int tail_n = static_cast<int>(pr->n) - (n_chunks - 1) * chunk_n;
        has_tail = tail_n != chunk_n;
        if (has_tail) {
            const long long Pt = static_cast<long long>(tail_n) * g.tiles_h * g.tiles_w;
            ce = plan_gemm(gemm_tail, op, E, Pt, g.k, g.kp, g.cp, V, U, Mw, mt, bn, num_sms, m_row());
            if (ce != cudaSuccess) return cuda_fail(ce, "GEMM plan (tail)");
        }
        launches = n_chunks * (3 + (scaling ? 1 : 0));
        info_grid = static_cast<unsigned>(gemm_full.grid);
        info_threads = 320;
        info_smem = gemm_full.smem_bytes;
    }
    filter_ready = false;
    return CONV2D_OK;
}

int Plan::filter(cudaStream_t s) {
    cudaError_t ce = algo == CONV2D_ALGO_4X3_ROW
                         ? launch_row4x3_filter(row, prob.weight, U, s)
                         : launch_filter_transform(xf, op, prob.weight, U, g.k, g.c, g.cp, s, opt.io_bf16 != 0);
    if (ce != cudaSuccess) return cuda_fail(ce, "filter transform launch");
    filter_ready = true;
    return CONV2D_OK;
}

void Plan::mark(cudaStream_t s) {
    if (marks && n_marks < max_marks) cudaEventRecord(marks[n_marks++], s);
}

int Plan::run_range(int n0, int nc, const GemmPlan* gp, cudaStream_t s) {
    cudaError_t ce;
    const void* x_end = static_cast<const uint16_t*>(prob.in) + static_cast<long long>(prob.n) * g.c * g.h * g.w;
    const long long in_img = static_cast<long long>(g.c) * g.h * g.w;
    const long long out_img = static_cast<long long>(g.k) * g.oh * g.ow;
    const Geom gc = make_geom(nc, g.c, g.h, g.w, g.k, g.pad_h, g.pad_w, g.m);
    const uint16_t* xin = static_cast<const uint16_t*>(prob.in) + n0 * in_img;
    uint16_t* yout = static_cast<uint16_t*>(prob.out) + n0 * out_img;
    if (algo == CONV2D_ALGO_2X3_FUSED) {
        ce = launch_fused2x3(fused, gc, xin, x_end, yout, err, s);
        if (ce != cudaSuccess) return cuda_fail(ce, "fused F(2x3) launch");
        mark(s);
        return CONV2D_OK;
    }
    if (algo == CONV2D_ALGO_4X3_ROW) {
        ce = nhwc ? launch_row4x3i(row, yout, n0, nc, err, s) : launch_row4x3(row, xin, x_end, yout, nc, err, s);
        if (ce != cudaSuccess) return cuda_fail(ce, "row F(4x3) launch");
        mark(s);
        return CONV2D_OK;
    }
    if (nhwc) {
        NhwcInDesc d = nh_in;        // V of this launch holds its nc images' tiles
        d.Pp = round_rows(gc.P);
        ce = launch_nhwc_input_transform(xf, op, d, nh_smem, n0, nc, err, s);
        if (ce != cudaSuccess) return cuda_fail(ce, "NHWC input transform launch");
        mark(s);
        ce = launch_gemm(*gp, err, s);
        if (ce != cudaSuccess) return cuda_fail(ce, "GEMM launch");
        mark(s);
        ce = mt == MType::F24 ? launch_output_transform_nhwc24(xf, gc, Mw, yout, err, s)
                              : launch_nhwc_output_transform(xf, mt, make_nhwc_out_desc(gc, Mw, yout), s);
        if (ce != cudaSuccess) return cuda_fail(ce, "NHWC output transform launch");
        mark(s);
        return CONV2D_OK;
    }
    if (scaling) {
        ce = launch_tile_scale(gc, xin, scale, s, opt.io_bf16 != 0);
        if (ce != cudaSuccess) return cuda_fail(ce, "tile scale launch");
        mark(s);
    }
    ce = launch_input_transform(xf, op, gc, xin, x_end, V, scale, err, s, opt.io_bf16 != 0);
    if (ce != cudaSuccess) return cuda_fail(ce, "input transform launch");
    mark(s);
    ce = launch_gemm(*gp, err, s);
    if (ce != cudaSuccess) return cuda_fail(ce, "GEMM launch");
    mark(s);
    ce = launch_output_transform(xf, mt, gc, Mw, yout, scale, err, s, opt.io_bf16 != 0);
    if (ce != cudaSuccess) return cuda_fail(ce, "output transform launch");
    mark(s);
    return CONV2D_OK;
}

int Plan::run(cudaStream_t s) {
    DeviceGuard dg(device);
    if (!filter_ready || opt.filter_policy == 1) {
        int st = filter(s);
        if (st) return st;
    }
    if (single_kernel()) return run_range(0, static_cast<int>(prob.n), nullptr, s);
    for (int ci = 0; ci < n_chunks; ++ci) {
        const int n0 = ci * chunk_n;
        const int nc = std::min<int>(chunk_n, static_cast<int>(prob.n) - n0);
        const GemmPlan& gp = (has_tail && ci == n_chunks - 1) ? gemm_tail : gemm_full;
        const int st = run_range(n0, nc, &gp, s);
        if (st) return st;
    }
    return CONV2D_OK;
}

// Host input -> device -> host output.  The batch is cut into equal image
// chunks; chunk i's input copy (copy-in stream), compute (caller stream) and
// output copy (copy-out stream) are ordered by events, so the copies of one
// chunk overlap the compute of its neighbours and the two copy directions
// overlap each other.  The host link bounds this call for large inputs (on
// the GB300 measured: 206 GB/s in, 190 GB/s out, 312 GB/s for both at once,
// whether copy engines or SM loads and stores move the bytes).  Chunks hold at
// least 6 MB of copies and there are at most 8 of them: on the 32 x 256 x 56^2
// layer (103 MB of copies) 8 chunks took 402-411 us per call, 6 took 420,
// 4 took 439, 12 and 16 took 450; chunks ramping from 1 image up to 4 and
// back measured 418-428 us against 415 for 8 x 4.  WG_CONV2D_HOST_CHUNKS sets
// another maximum (1-16), WG_CONV2D_HOST_SIZES every chunk's image count.
// Each chunk's copies and kernels are queued together, the input copies
// three chunks ahead.
namespace {

// WG_CONV2D_HOST_SIZES="a,b,..." (positive image counts summing to n, at most
// kMaxHostChunks of them, at most kMaxHostPlans distinct ones) -> their count,
// else 0.
int host_sizes_env(int n, int* sizes) {
    const char* p = std::getenv("WG_CONV2D_HOST_SIZES");
    if (!p || !*p) return 0;
    int cnt = 0;
    long long sum = 0;
    while (*p) {
        char* q = nullptr;
        const long v = std::strtol(p, &q, 10);
        if (q == p || v <= 0 || v > n || cnt == Plan::kMaxHostChunks || (*q && *q != ',')) return 0;
        sizes[cnt++] = static_cast<int>(v);
        sum += v;
        p = *q ? q + 1 : q;
    }
    int distinct = 0;
    for (int i = 0; i < cnt; ++i) {
        bool seen = false;
        for (int j = 0; j < i; ++j) seen = seen || sizes[j] == sizes[i];
        distinct += seen ? 0 : 1;
    }
    return (sum == n && distinct <= Plan::kMaxHostPlans) ? cnt : 0;
}

int host_schedule(int n, long long img_copy_bytes, int* sizes) {
    if (const int cnt = host_sizes_env(n, sizes)) return cnt;
    const long long total = static_cast<long long>(n) * img_copy_bytes;
    long long max_chunks = 8;
    if (const char* e = std::getenv("WG_CONV2D_HOST_CHUNKS")) max_chunks = std::max(1, std::min(std::atoi(e), Plan::kMaxHostChunks));
    const int chunks = static_cast<int>(
        std::max(1LL, std::min<long long>({static_cast<long long>(n), max_chunks, total / (6LL << 20)})));
    const int per = (n + chunks - 1) / chunks;
    int cnt = 0;
    for (int done = 0; done < n; done += per) sizes[cnt++] = std::min(per, n - done);
    return cnt;
}

}  // namespace

const GemmPlan* Plan::host_gemm_for(int nc) {
    for (int i = 0; i < n_host_plans; ++i)
        if (host_plan_n[i] == nc) return &host_gemm[i];
    if (n_host_plans == kMaxHostPlans) return nullptr;
    const int E = g.alpha * g.alpha;
    GemmPlan& gp = host_gemm[n_host_plans];
    if (plan_gemm(gp, op, E, static_cast<long long>(nc) * g.tiles_h * g.tiles_w, g.k, g.kp, g.cp, V, U, Mw, mt,
                  gemm_full.bn, num_sms, m_row()) != cudaSuccess)
        return nullptr;
    host_plan_n[n_host_plans++] = nc;
    return &gp;
}

// The pipeline queues about ten operations per chunk.  With
// WG_CONV2D_HOST_GRAPH=1 the pipeline for a pair of host buffers is captured
// once into a CUDA graph (on a stream of the plan, as the caller's stream may
// be the legacy default stream, which cannot be captured) and replayed on the
// caller's stream by later calls with the same buffers.  By default the
// operations are queued directly: at 8 chunks the host queues them faster than
// the copies run and the first copies start at once, while a graph launch
// front-loads its set-up (on the 32 x 256 x 56^2 layer: 413-418 us per call
// queued directly, 434-437 us replayed).
int Plan::host_setup() {
    if (!host_in_stream) {
        if (cudaStreamCreateWithFlags(&host_in_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&host_out_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&host_cap_stream, cudaStreamNonBlocking) != cudaSuccess)
            return fail(CONV2D_ERR_CUDA, "copy stream creation failed");
        for (cudaEvent_t& e : host_ev)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                return fail(CONV2D_ERR_CUDA, "event creation failed");
    }
    return CONV2D_OK;
}

int Plan::run_host(const void* host_in, void* host_out, cudaStream_t s) {
    DeviceGuard dg(device);
    if (!filter_ready || opt.filter_policy == 1) {
        int st = filter(s);
        if (st) return st;
    }
    if (const int st = host_setup()) return st;
    if (host_graph && (graph_in != host_in || graph_out != host_out)) {
        cudaGraphExecDestroy(host_graph);
        host_graph = nullptr;
    }
    const bool use_graph = env_int("WG_CONV2D_HOST_GRAPH", 0) != 0;
    if (use_graph && !host_graph &&
        cudaStreamBeginCapture(host_cap_stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const int st = enqueue_host(&host_in, &host_out, 1, host_cap_stream);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(host_cap_stream, &graph);
        if (st == CONV2D_OK && ce == cudaSuccess && graph &&
            cudaGraphInstantiate(&host_graph, graph, 0) == cudaSuccess) {
            graph_in = host_in;
            graph_out = host_out;
        } else {
            host_graph = nullptr;
        }
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();   // a failed capture leaves its error; the direct path follows
    }
    if (host_graph) {
        const cudaError_t ce = cudaGraphLaunch(host_graph, s);
        if (ce != cudaSuccess) return cuda_fail(ce, "host pipeline graph launch");
    } else {
        const int st = enqueue_host(&host_in, &host_out, 1, s);
        if (st) return st;
    }
    const cudaError_t ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return cuda_fail(ce, "stream sync");
    return CONV2D_OK;
}

int Plan::run_host_steps(const void* const* host_in, void* const* host_out, int steps, cudaStream_t s) {
    DeviceGuard dg(device);
    if (!filter_ready || opt.filter_policy == 1) {
        int st = filter(s);
        if (st) return st;
    }
    if (const int st = host_setup()) return st;
    if (const int st = enqueue_host(host_in, host_out, steps, s)) return st;
    const cudaError_t ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) return cuda_fail(ce, "stream sync");
    return CONV2D_OK;
}

// Steps run one after another through the same device buffers; chunk i of a
// step is ordered only against chunk i of the step before: its input copy
// after that step's compute of chunk i (which read the same input rows), its
// compute after that step's output copy of chunk i (which read the same output
// rows).  So the output copies of one step overlap the input copies of the
// next, and the link carries both directions at once across step boundaries.
int Plan::enqueue_host(const void* const* host_in, void* const* host_out, int steps, cudaStream_t s) {
    const int n = static_cast<int>(prob.n);
    const long long in_img_b = static_cast<long long>(g.c) * g.h * g.w * 2;
    const long long out_img_b = static_cast<long long>(g.k) * g.oh * g.ow * 2;
    int sizes[kMaxHostChunks];
    const int nch = host_schedule(n, in_img_b + out_img_b, sizes);
    // the non-fused workspace holds chunk_n images: a host chunk runs as
    // ranges of at most that many
    const int cap = single_kernel() ? n : chunk_n;
    cudaEvent_t* ev_in = host_ev;                         // [kMaxHostChunks]
    cudaEvent_t* ev_done = host_ev + kMaxHostChunks;      // [kMaxHostChunks]
    cudaEvent_t* ev_out = host_ev + 2 * kMaxHostChunks;   // [kMaxHostChunks]
    cudaEvent_t ev_start = host_ev[3 * kMaxHostChunks], ev_end = host_ev[3 * kMaxHostChunks + 1];
    // the copies must not overwrite the input before earlier work on s is done
    cudaEventRecord(ev_start, s);
    cudaStreamWaitEvent(host_in_stream, ev_start, 0);
    cudaStreamWaitEvent(host_out_stream, ev_start, 0);
    int first[kMaxHostChunks + 1];
    first[0] = 0;
    for (int i = 0; i < nch; ++i) first[i + 1] = first[i] + sizes[i];
    // queue positions q = step * nch + chunk
    auto copy_in = [&](int q) {
        const int st = q / nch, i = q % nch;
        if (st > 0) cudaStreamWaitEvent(host_in_stream, ev_done[i], 0);   // step st-1 read these rows
        const cudaError_t ce = cudaMemcpyAsync(static_cast<char*>(prob.in) + first[i] * in_img_b,
                                               static_cast<const char*>(host_in[st]) + first[i] * in_img_b,
                                               sizes[i] * in_img_b, cudaMemcpyHostToDevice, host_in_stream);
        cudaEventRecord(ev_in[i], host_in_stream);
        return ce;
    };
    // input copies are queued up to three chunks ahead, never a whole step
    // (each chunk's events are reused by the next step)
    const int ahead = std::min(3, nch - 1), total = steps * nch;
    for (int q = 0; q < std::min(ahead, total); ++q)
        if (cudaError_t ce = copy_in(q); ce != cudaSuccess) return cuda_fail(ce, "input copy");
    for (int q = 0; q < total; ++q) {
        const int st = q / nch, i = q % nch, n0 = first[i];
        cudaError_t ce = q + ahead < total && ahead > 0 ? copy_in(q + ahead) : cudaSuccess;
        if (ahead == 0) ce = copy_in(q);
        if (ce != cudaSuccess) return cuda_fail(ce, "input copy");
        cudaStreamWaitEvent(s, ev_in[i], 0);
        if (st > 0) cudaStreamWaitEvent(s, ev_out[i], 0);   // step st-1's output copy read these rows
        for (int r0 = n0; r0 < n0 + sizes[i]; r0 += cap) {
            const int nc = std::min(cap, n0 + sizes[i] - r0);
            const GemmPlan* gp = nullptr;
            if (!single_kernel() && !(gp = host_gemm_for(nc))) return fail(CONV2D_ERR_CUDA, "GEMM plan (host chunks) failed");
            const int rs = run_range(r0, nc, gp, s);
            if (rs) return rs;
        }
        cudaEventRecord(ev_done[i], s);
        cudaStreamWaitEvent(host_out_stream, ev_done[i], 0);
        ce = cudaMemcpyAsync(static_cast<char*>(host_out[st]) + n0 * out_img_b,
                             static_cast<const char*>(prob.out) + n0 * out_img_b, sizes[i] * out_img_b,
                             cudaMemcpyDeviceToHost, host_out_stream);
        if (ce != cudaSuccess) return cuda_fail(ce, "output copy");
        cudaEventRecord(ev_out[i], host_out_stream);
    }
    cudaEventRecord(ev_end, host_out_stream);
    cudaStreamWaitEvent(s, ev_end, 0);
    return CONV2D_OK;
}

int set_last_error(int status, const char* msg) { return fail(status, msg); }

Plan* plan_of(const void* param) {
    if (!param) return nullptr;
    const ParamBlob* pb = static_cast<const ParamBlob*>(param);
    if (pb->magic != kParamMagic || !pb->plan) return nullptr;
    return static_cast<Plan*>(pb->plan);
}

void fill_blob(ParamBlob* pb, Plan* pl) {
    const problem_t& pr = pl->prob;
    pb->pin = pr.in;
    pb->pweight = pr.weight;
    pb->pout = pr.out;
    pb->U_d = pl->U;
    pb->V_d = pl->V;
    pb->M_d = pl->Mw;
    pb->Y_d = nullptr;
    pb->n = pr.n; pb->c = pr.c; pb->h = pr.h; pb->w = pr.w; pb->k = pr.k;
    pb->r = pr.r; pb->s = pr.s; pb->u = pr.u; pb->v = pr.v; pb->p = pr.p; pb->q = pr.q;
    pb->Oh = static_cast<unsigned>(pl->g.oh);
    pb->Ow = static_cast<unsigned>(pl->g.ow);
    pb->kernel = pl->algo;
    pb->magic = kParamMagic;
    pb->plan = pl;
}

}  // namespace wg

using namespace wg;

extern "C" {

int wg_getParamsize(problem_t* problem, int* paramSize) {
    (void)problem;
    if (!paramSize) return fail(CONV2D_ERR_INVALID, "null paramSize");
    *paramSize = static_cast<int>(sizeof(ParamBlob));
    return CONV2D_OK;
}

int getParamsize(problem_t* problem, int* paramSize) { return wg_getParamsize(problem, paramSize); }

int conv2d_options_default(conv2d_options_t* opt) {
    if (!opt) return fail(CONV2D_ERR_INVALID, "null options");
    return options_default(opt);
}

int getkernelInfo_ex(problem_t* problem, kernelInfo_t* kernelInfo, void* param, const conv2d_options_t* opt) {
    if (!param) return fail(CONV2D_ERR_INVALID, "null param");
    ParamBlob* pb = static_cast<ParamBlob*>(param);
    std::memset(pb, 0, sizeof(*pb));
    Plan* pl = new Plan();
    int st = pl->build(problem, opt);
    if (st) {
        delete pl;
        return st;
    }
    fill_blob(pb, pl);
    if (kernelInfo) {
        kernelInfo->blockx = pl->info_grid;
        kernelInfo->blocky = 1;
        kernelInfo->blockz = 1;
        kernelInfo->threadx = pl->info_threads;
        kernelInfo->thready = 1;
        kernelInfo->threadz = 1;
        kernelInfo->dynmicLdsSize = static_cast<unsigned>(pl->info_smem);
        kernelInfo->kernelPtr = nullptr;
    }
    return CONV2D_OK;
}

int wg_getkernelInfo(problem_t* problem, kernelInfo_t* kernelInfo, void* param) {
    return getkernelInfo_ex(problem, kernelInfo, param, nullptr);
}

int getkernelInfo(problem_t* problem, kernelInfo_t* kernelInfo, void* param) {
    return wg_getkernelInfo(problem, kernelInfo, param);
}

int conv2d_fp16_ex(const void* param_ptr, void* stream) {
    Plan* pl = plan_of(param_ptr);
    if (!pl) return fail(CONV2D_ERR_INVALID, "param blob not set up by getkernelInfo");
    return pl->run(static_cast<cudaStream_t>(stream));
}

// Same behaviour as the reference on a failed launch (include/error.h:18-27):
// message on stderr and process exit.
void conv2d_fp16(const void* param_ptr) {
    const int st = conv2d_fp16_ex(param_ptr, nullptr);
    if (st == CONV2D_ERR_INVALID) {
        std::fprintf(stderr, "conv2d_fp16: %s\n", t_last_msg.c_str());
        return;
    }
    if (st != CONV2D_OK) {
        std::fprintf(stderr, "Kernel panic!!!: %s\n", t_last_msg.c_str());
        std::exit(-1);
    }
}

int conv2d_fp16_host(const void* param_ptr, const void* host_in, void* host_out, void* stream) {
    Plan* pl = plan_of(param_ptr);
    if (!pl) return fail(CONV2D_ERR_INVALID, "param blob not set up by getkernelInfo");
    if (!host_in || !host_out) return fail(CONV2D_ERR_INVALID, "null host buffer");
    return pl->run_host(host_in, host_out, static_cast<cudaStream_t>(stream));
}

int conv2d_fp16_host_steps(const void* param_ptr, int steps, const void* const* host_in, void* const* host_out,
                           void* stream) {
    Plan* pl = plan_of(param_ptr);
    if (!pl) return fail(CONV2D_ERR_INVALID, "param blob not set up by getkernelInfo");
    if (steps <= 0 || !host_in || !host_out) return fail(CONV2D_ERR_INVALID, "bad step count or null buffer list");
    for (int i = 0; i < steps; ++i)
        if (!host_in[i] || !host_out[i]) return fail(CONV2D_ERR_INVALID, "null host buffer");
    return pl->run_host_steps(host_in, host_out, steps, static_cast<cudaStream_t>(stream));
}

int conv2d_refresh_filter(const void* param_ptr, void* stream) {
    Plan* pl = plan_of(param_ptr);
    if (!pl) return fail(CONV2D_ERR_INVALID, "param blob not set up by getkernelInfo");
    DeviceGuard dg(pl->device);
    return pl->filter(static_cast<cudaStream_t>(stream));
}

int conv2d_destroy(void* param_ptr) {
    Plan* pl = plan_of(param_ptr);
    if (!pl) return fail(CONV2D_ERR_INVALID, "param blob not set up by getkernelInfo");
    {
        DeviceGuard dg(pl->device);
        cudaDeviceSynchronize();
        delete pl;
    }
    std::memset(param_ptr, 0, sizeof(ParamBlob));
    return CONV2D_OK;
}

int conv2d_get_algo(const void* param_ptr) {
    Plan* pl = plan_of(param_ptr);
    return pl ? pl->algo : -1;
}

long long conv2d_workspace_bytes(const void* param_ptr) {
    Plan* pl = plan_of(param_ptr);
    return pl ? pl->ws_bytes : -1;
}

int conv2d_launches_per_call(const void* param_ptr) {
    Plan* pl = plan_of(param_ptr);
    return pl ? pl->launches : -1;
}

int conv2d_check_device(const void* param_ptr, int* site) {
    Plan* pl = plan_of(param_ptr);
    if (!pl) return fail(CONV2D_ERR_INVALID, "param blob not set up by getkernelInfo");
    DeviceGuard dg(pl->device);
    cudaError_t ce = cudaDeviceSynchronize();
    if (ce != cudaSuccess) return cuda_fail(ce, "device synchronize");
    DevErr h{};
    ce = cudaMemcpy(&h, pl->err, sizeof(h), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return cuda_fail(ce, "error word copy");
    if (site) *site = static_cast<int>(h.code);
    if (h.code) {
        cudaMemset(pl->err, 0, sizeof(DevErr));
        return fail(CONV2D_ERR_TIMEOUT, "a kernel gave up a bounded wait");
    }
    return CONV2D_OK;
}

int conv2d_last_error(void) { return t_last_status; }

const char* conv2d_last_error_message(void) { return t_last_msg.c_str(); }

const char* conv2d_status_string(int status) {
    switch (status) {
        case CONV2D_OK: return "ok";
        case CONV2D_ERR_INVALID: return "invalid argument";
        case CONV2D_ERR_UNSUPPORTED: return "unsupported descriptor";
        case CONV2D_ERR_NOMEM: return "out of device memory";
        case CONV2D_ERR_CUDA: return "CUDA error";
        case CONV2D_ERR_TIMEOUT: return "device wait timed out";
        case CONV2D_ERR_BUSY: return "busy";
    }
    return "unknown status";
}

int conv2d_select_reference(const problem_t* pr) {
    if (!pr) return -1;
    const unsigned long long oh = pr->h + 2ull * pr->p - pr->r + 1;
    const unsigned long long ow = pr->w + 2ull * pr->q - pr->s + 1;
    return select_reference64(pr->n, pr->c, pr->h, pr->w, pr->k, pr->r, pr->s, oh, ow);
}

int conv2d_fp16_timed(const void* param_ptr, void* stream, float* kernel_ms, int max_kernels) {
    Plan* pl = plan_of(param_ptr);
    if (!pl) return fail(CONV2D_ERR_INVALID, "param blob not set up by getkernelInfo");
    if (!kernel_ms || max_kernels <= 0) return fail(CONV2D_ERR_INVALID, "null output array");
    DeviceGuard dg(pl->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!pl->filter_ready) {
        int st = pl->filter(s);
        if (st) return -st;
    }
    const int n = std::min(max_kernels, pl->launches) + 1;
    cudaEvent_t ev[64];
    const int ne = std::min(n, 64);
    for (int i = 0; i < ne; ++i) cudaEventCreate(&ev[i]);
    cudaEventRecord(ev[0], s);
    pl->marks = ev + 1;
    pl->n_marks = 0;
    pl->max_marks = ne - 1;
    int st = pl->run(s);
    const int got = pl->n_marks;
    pl->marks = nullptr;
    pl->n_marks = pl->max_marks = 0;
    cudaError_t ce = cudaStreamSynchronize(s);
    for (int i = 0; i < got; ++i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
        kernel_ms[i] = ms;
    }
    for (int i = 0; i < ne; ++i) cudaEventDestroy(ev[i]);
    if (st) return -st;
    if (ce != cudaSuccess) return -cuda_fail(ce, "stream sync");
    return got;
}

int conv2d_autotune(const problem_t* problem, const conv2d_options_t* opt, int* algo, int* gemm_bn) {
    int st = validate_problem(problem);
    if (st) return st;
    if (!algo || !gemm_bn) return fail(CONV2D_ERR_INVALID, "null output");
    conv2d_options_t o;
    if (opt)
        o = *opt;
    else
        options_default(&o);
    const unsigned oh = problem->h + 2 * problem->p - 2, ow = problem->w + 2 * problem->q - 2;
    const int ref = select_reference64(problem->n, problem->c, problem->h, problem->w, problem->k, 3, 3, oh, ow);
    return autotune_choose(*problem, o, ref, algo, gemm_bn);
}

void conv2d_autotune_clear(void) { autotune_clear(); }

int conv2d_copy_to_host(void* host_dst, const void* device_src, size_t bytes) {
    if (!host_dst || !device_src) return fail(CONV2D_ERR_INVALID, "null pointer");
    cudaError_t ce = cudaMemcpy(host_dst, device_src, bytes, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaMemcpy");
    return CONV2D_OK;
}

}  // extern "C"
