// Many convolutions of uneven shape in one graph launch.
//
// A batch holds one Plan per problem (algorithm and GEMM tile chosen per
// shape, by default by the autotuner; workspace and transformed filter of
// each problem resident) and runs them either
//   * grouped: the input transforms of all problems in one launch per
//     transform family, the GEMMs of all problems in one persistent launch
//     per (channel tile, M type) whose work queue holds every (problem,
//     element, tile block, channel block) item, the output transforms in one
//     launch per family -- captured once into a CUDA graph and replayed; or
//   * per call: each problem's own launches, one problem after another
//     (the comparison the grouped run is measured against).
// Both use the same workspaces, so their results are bit-identical.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "../../include/conv2d.h"
#include "wg_kernels.h"
#include "wg_plan.h"

namespace wg {

struct Batch {
    std::vector<std::unique_ptr<Plan>> plans;
    void* dev = nullptr;         // descriptor arrays + error word
    DevErr* err = nullptr;
    struct InGroup {
        Xform xf;
        OpType op;
        int bn;    // GEMM tile of the chain this group starts
        const InDesc* descs;
        int n;
        long long blocks;
        int smem;
        bool scaled;
    };
    struct GemmGroup {
        int bn;
        MType mt;
        OpType op;
        Xform xf;
        const GemmDesc* descs;
        int n;
        long long tiles;
        int grid;
    };
    struct OutGroup {
        Xform xf;
        MType mt;
        int bn;
        const OutDesc* descs;
        int n;
        long long blocks;
    };
    std::vector<InGroup> in_groups;
    std::vector<GemmGroup> gemm_groups;
    std::vector<OutGroup> out_groups;
    std::vector<int> fused;      // problems run by their own fused kernel
    std::vector<int> scaled;     // problems whose tile scale is computed per problem
    cudaGraphExec_t graph = nullptr;
    int grouped_launches = 0;

    ~Batch() {
        if (graph) cudaGraphExecDestroy(graph);
        if (dev) cudaFree(dev);
        for (int i = 0; i < kSides; ++i) {
            if (side[i]) cudaStreamDestroy(side[i]);
            if (join[i]) cudaEventDestroy(join[i]);
        }
        if (fork) cudaEventDestroy(fork);
    }

    // Independent branches of the graph: each chain of grouped launches (one
    // per transform, or per transform and GEMM tile: its tile scales, input
    // transforms, GEMMs and output transforms; bn 0 = every tile) and each
    // problem run by its own kernel (row
    // F(4x3), fused F(2x3)) is a unit; units go to kSides + 1 streams forked
    // from the caller's, largest first to the least loaded, so that one
    // branch's CTAs fill the others' tails.  Without side streams
    // (WG_CONV2D_BATCH_BRANCH=0) the units run one after another on one stream.
    static constexpr int kSides = 5;
    cudaStream_t side[kSides] = {};
    cudaEvent_t fork = nullptr, join[kSides] = {};
    struct Unit {
        Xform xf;      // chain: transform and GEMM tile
        int bn;
        int single;    // or the problem run by its own kernel (>= 0)
        double flops;  // direct-convolution work
        int stream;    // 0: the caller's stream, k: side[k - 1]
    };
    std::vector<Unit> units;

    cudaError_t launch_chain(Xform xf, int bn, cudaStream_t s) {
        cudaError_t e = cudaSuccess;
        for (int i : scaled) {
            Plan& p = *plans[i];
            if (p.xf == xf && (bn == 0 || p.gemm_full.bn == bn) &&
                (e = launch_tile_scale(p.g, p.prob.in, p.scale, s)) != cudaSuccess)
                return e;
        }
        for (const InGroup& g : in_groups)
            if (g.xf == xf && g.bn == bn &&
                (e = launch_input_transform_grouped(g.xf, g.op, g.descs, g.n, g.blocks, g.smem, g.scaled, err, s)) !=
                    cudaSuccess)
                return e;
        for (const GemmGroup& g : gemm_groups)
            if (g.xf == xf && (bn == 0 || g.bn == bn) &&
                (e = launch_gemm_grouped(g.descs, g.n, g.tiles, g.op, g.mt, g.bn, g.grid, err, s)) != cudaSuccess)
                return e;
        for (const OutGroup& g : out_groups)
            if (g.xf == xf && g.bn == bn &&
                (e = launch_output_transform_grouped(g.xf, g.mt, g.descs, g.n, g.blocks, err, s)) != cudaSuccess)
                return e;
        return cudaSuccess;
    }

    cudaError_t launch_unit(const Unit& u, cudaStream_t s) {
        return u.single >= 0 ? launch_single(u.single, s) : launch_chain(u.xf, u.bn, s);
    }

    cudaError_t launch_grouped(cudaStream_t s) {
        cudaError_t e = cudaSuccess;
        if (!side[0]) {
            for (const Unit& u : units)
                if ((e = launch_unit(u, s)) != cudaSuccess) return e;
            return cudaSuccess;
        }
        if ((e = cudaEventRecord(fork, s)) != cudaSuccess) return e;
        for (int i = 0; i < kSides; ++i)
            if ((e = cudaStreamWaitEvent(side[i], fork, 0)) != cudaSuccess) return e;
        for (const Unit& u : units)
            if ((e = launch_unit(u, u.stream ? side[u.stream - 1] : s)) != cudaSuccess) return e;
        for (int i = 0; i < kSides; ++i)
            if ((e = cudaEventRecord(join[i], side[i])) != cudaSuccess || (e = cudaStreamWaitEvent(s, join[i], 0)) != cudaSuccess)
                return e;
        return cudaSuccess;
    }

    // a problem run by its own kernel
    cudaError_t launch_single(int i, cudaStream_t s) {
        Plan& p = *plans[i];
        const void* x_end =
            static_cast<const uint16_t*>(p.prob.in) + static_cast<long long>(p.prob.n) * p.g.c * p.g.h * p.g.w;
        if (p.algo == CONV2D_ALGO_4X3_ROW)
            return launch_row4x3(p.row, p.prob.in, x_end, p.prob.out, static_cast<int>(p.prob.n), err, s);
        return launch_fused2x3(p.fused, p.g, p.prob.in, x_end, p.prob.out, err, s);
    }
};

namespace {

int batch_fail(int st, const char* msg) { return set_last_error(st, msg); }

}  // namespace

int batch_create(const problem_t* problems, int count, const conv2d_options_t* opt_in, Batch** out) {
    if (!problems || count <= 0 || !out) return batch_fail(CONV2D_ERR_INVALID, "empty batch");
    conv2d_options_t opt;
    if (opt_in)
        opt = *opt_in;
    else
        options_default(&opt);
    opt.l2_chunk_bytes = 0;
    if (opt.io_bf16 || opt.layout_nhwc)
        return batch_fail(CONV2D_ERR_UNSUPPORTED, "grouped batches take fp16 NCHW tensors");
    std::unique_ptr<Batch> b(new Batch());
    for (int i = 0; i < count; ++i) {
        std::unique_ptr<Plan> p(new Plan());
        int st = p->build(&problems[i], &opt);
        if (st) return st;
        st = p->filter(nullptr);  // transformed filters stay resident
        if (st) return st;
        b->plans.push_back(std::move(p));
    }
    // group the problems and lay out their descriptors
    // one chain of grouped launches per transform: input transform, GEMM
    // and output transform groups of the same problems
    std::map<std::tuple<int, int, int>, std::vector<int>> in_keys, out_keys;  // (xform, op | M type, bn) -> problems
    const char* sb = std::getenv("WG_CONV2D_BATCH_SPLIT_BN");
    const bool split_bn = sb && sb[0] == '1';
    std::map<std::tuple<int, int, int, int>, std::vector<int>> gemm_keys;     // (bn, M type, op, xform) -> problems
    for (int i = 0; i < count; ++i) {
        Plan& p = *b->plans[i];
        if (p.single_kernel()) {
            b->fused.push_back(i);
            continue;
        }
        if (p.scaling) b->scaled.push_back(i);
        // WG_CONV2D_BATCH_SPLIT_BN=1: one chain per (transform, GEMM tile)
        // instead of one per transform
        const int cbn = split_bn ? p.gemm_full.bn : 0;
        in_keys[{static_cast<int>(p.xf), static_cast<int>(p.op), cbn}].push_back(i);
        out_keys[{static_cast<int>(p.xf), static_cast<int>(p.mt), cbn}].push_back(i);
        gemm_keys[{p.gemm_full.bn, static_cast<int>(p.mt), static_cast<int>(p.op), static_cast<int>(p.xf)}].push_back(i);
    }
    std::vector<InDesc> in_descs;
    std::vector<OutDesc> out_descs;
    std::vector<GemmDesc> gemm_descs;
    struct Range {
        size_t first, n;
        long long total;
        int extra;
        bool scaled;
    };
    std::vector<std::pair<std::tuple<int, int, int>, Range>> in_r, out_r;
    std::vector<std::pair<std::tuple<int, int, int, int>, Range>> gemm_r;
    for (auto& kv : in_keys) {
        Range r{in_descs.size(), kv.second.size(), 0, 0, false};
        for (int i : kv.second) {
            Plan& p = *b->plans[i];
            r.scaled = r.scaled || p.scale != nullptr;
            const void* x_end =
                static_cast<const uint16_t*>(p.prob.in) + static_cast<long long>(p.prob.n) * p.g.c * p.g.h * p.g.w;
            int smem = 0;
            InDesc d = make_in_desc(p.g, p.prob.in, x_end, p.V, p.scale, &smem);
            d.blk_begin = r.total;
            r.total += d.gx * d.gy;
            r.extra = std::max(r.extra, smem);
            in_descs.push_back(d);
        }
        in_r.push_back({kv.first, r});
    }
    for (auto& kv : out_keys) {
        Range r{out_descs.size(), kv.second.size(), 0, 0, false};
        for (int i : kv.second) {
            Plan& p = *b->plans[i];
            OutDesc d = make_out_desc(p.g, p.mt, p.Mw, p.prob.out, p.scale);
            d.blk_begin = r.total;
            r.total += d.gx * d.gy;
            out_descs.push_back(d);
        }
        out_r.push_back({kv.first, r});
    }
    for (auto& kv : gemm_keys) {
        Range r{gemm_descs.size(), kv.second.size(), 0, 0, false};
        for (int i : kv.second) {
            GemmDesc d = b->plans[i]->gemm_full.desc;
            d.tile_begin = r.total;
            r.total += d.tiles;
            gemm_descs.push_back(d);
        }
        gemm_r.push_back({kv.first, r});
    }
    // one device block: error word | GemmDesc[] (64-byte aligned) | InDesc[] | OutDesc[]
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t oE = 0, oG = 256, oI = oG + al(gemm_descs.size() * sizeof(GemmDesc)),
                 oO = oI + al(in_descs.size() * sizeof(InDesc)), total = oO + al(out_descs.size() * sizeof(OutDesc));
    if (cudaMalloc(&b->dev, total) != cudaSuccess) {
        cudaGetLastError();
        return batch_fail(CONV2D_ERR_NOMEM, "batch descriptor allocation failed");
    }
    char* base = static_cast<char*>(b->dev);
    b->err = reinterpret_cast<DevErr*>(base + oE);
    cudaMemset(b->err, 0, sizeof(DevErr));
    if (!gemm_descs.empty()) cudaMemcpy(base + oG, gemm_descs.data(), gemm_descs.size() * sizeof(GemmDesc), cudaMemcpyHostToDevice);
    if (!in_descs.empty()) cudaMemcpy(base + oI, in_descs.data(), in_descs.size() * sizeof(InDesc), cudaMemcpyHostToDevice);
    if (!out_descs.empty()) cudaMemcpy(base + oO, out_descs.data(), out_descs.size() * sizeof(OutDesc), cudaMemcpyHostToDevice);
    int sms = b->plans[0]->num_sms;
    for (auto& kr : in_r)
        b->in_groups.push_back({static_cast<Xform>(std::get<0>(kr.first)), static_cast<OpType>(std::get<1>(kr.first)),
                                std::get<2>(kr.first), reinterpret_cast<const InDesc*>(base + oI) + kr.second.first,
                                static_cast<int>(kr.second.n), kr.second.total, kr.second.extra, kr.second.scaled});
    for (auto& kr : gemm_r)
        b->gemm_groups.push_back({std::get<0>(kr.first), static_cast<MType>(std::get<1>(kr.first)),
                                  static_cast<OpType>(std::get<2>(kr.first)), static_cast<Xform>(std::get<3>(kr.first)),
                                  reinterpret_cast<const GemmDesc*>(base + oG) + kr.second.first,
                                  static_cast<int>(kr.second.n), kr.second.total,
                                  static_cast<int>(std::min<long long>(kr.second.total, sms))});
    for (auto& kr : out_r)
        b->out_groups.push_back({static_cast<Xform>(std::get<0>(kr.first)), static_cast<MType>(std::get<1>(kr.first)),
                                 std::get<2>(kr.first), reinterpret_cast<const OutDesc*>(base + oO) + kr.second.first,
                                 static_cast<int>(kr.second.n), kr.second.total});
    int single = 0;   // launches of the problems run by their own kernels
    for (int i : b->fused) single += b->plans[i]->launches;
    b->grouped_launches = static_cast<int>(b->scaled.size() + b->in_groups.size() + b->gemm_groups.size() +
                                           b->out_groups.size()) + single;
    if (cudaDeviceSynchronize() != cudaSuccess) return batch_fail(CONV2D_ERR_CUDA, "batch setup failed");
    // work units (chains and single-kernel problems), largest first, each to
    // the stream with the least direct-convolution work so far
    auto flops = [&](int i) {
        const Plan& p = *b->plans[i];
        return 18.0 * p.prob.n * p.prob.k * p.g.oh * p.g.ow * p.prob.c;
    };
    for (const Batch::InGroup& g : b->in_groups) {
        bool seen = false;   // one unit per chain, whatever its operand types
        for (const Batch::Unit& v : b->units) seen = seen || (v.single < 0 && v.xf == g.xf && v.bn == g.bn);
        if (seen) continue;
        Batch::Unit u{g.xf, g.bn, -1, 0.0, 0};
        for (int i = 0; i < count; ++i) {
            const Plan& p = *b->plans[i];
            if (!p.single_kernel() && p.xf == g.xf && (g.bn == 0 || p.gemm_full.bn == g.bn)) u.flops += flops(i);
        }
        b->units.push_back(u);
    }
    for (int i : b->fused) b->units.push_back({Xform::F2, 0, i, flops(i), 0});
    std::stable_sort(b->units.begin(), b->units.end(),
                     [](const Batch::Unit& x, const Batch::Unit& y) { return x.flops > y.flops; });
    {
        double load[Batch::kSides + 1] = {};
        for (Batch::Unit& u : b->units) {
            int best = 0;
            for (int k = 1; k <= Batch::kSides; ++k)
                if (load[k] < load[best]) best = k;
            u.stream = best;
            load[best] += u.flops;
        }
    }
    const char* br = std::getenv("WG_CONV2D_BATCH_BRANCH");
    if (!(br && br[0] == '0')) {
        bool ok = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) == cudaSuccess;
        for (int i = 0; i < Batch::kSides && ok; ++i)
            ok = cudaStreamCreateWithFlags(&b->side[i], cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming) == cudaSuccess;
        if (!ok) return batch_fail(CONV2D_ERR_CUDA, "side streams of the batch graph");
    }
    *out = b.release();
    return CONV2D_OK;
}

int batch_run(Batch* b, cudaStream_t s) {
    if (!b->graph) {
        // first run: set every kernel up outside capture, then record the
        // grouped launches once into a graph
        cudaError_t e = b->launch_grouped(s);
        if (e != cudaSuccess) return batch_fail(CONV2D_ERR_CUDA, cudaGetErrorString(e));
        cudaStream_t cs;
        cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        cudaGraph_t g = nullptr;
        if (cudaStreamSynchronize(s) != cudaSuccess ||
            cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaStreamDestroy(cs);
            return batch_fail(CONV2D_ERR_CUDA, "graph capture could not start");
        }
        e = b->launch_grouped(cs);
        cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        cudaStreamDestroy(cs);
        if (e != cudaSuccess || e2 != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return batch_fail(CONV2D_ERR_CUDA, "graph capture failed");
        }
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->graph = nullptr;
            return batch_fail(CONV2D_ERR_CUDA, "graph instantiation failed");
        }
        return CONV2D_OK;
    }
    cudaError_t e = cudaGraphLaunch(b->graph, s);
    if (e != cudaSuccess) return batch_fail(CONV2D_ERR_CUDA, cudaGetErrorString(e));
    return CONV2D_OK;
}

int batch_run_percall(Batch* b, cudaStream_t s) {
    for (auto& p : b->plans) {
        int st = p->run(s);
        if (st) return st;
    }
    return CONV2D_OK;
}

}  // namespace wg

using namespace wg;

extern "C" {

int conv2d_batch_create(const problem_t* problems, int count, const conv2d_options_t* opt, conv2d_batch_t** out) {
    Batch* b = nullptr;
    const int st = batch_create(problems, count, opt, &b);
    if (st == CONV2D_OK) *out = reinterpret_cast<conv2d_batch_t*>(b);
    return st;
}

int conv2d_batch_run(conv2d_batch_t* batch, void* stream) {
    if (!batch) return set_last_error(CONV2D_ERR_INVALID, "null batch");
    return batch_run(reinterpret_cast<Batch*>(batch), static_cast<cudaStream_t>(stream));
}

int conv2d_batch_run_percall(conv2d_batch_t* batch, void* stream) {
    if (!batch) return set_last_error(CONV2D_ERR_INVALID, "null batch");
    return batch_run_percall(reinterpret_cast<Batch*>(batch), static_cast<cudaStream_t>(stream));
}

int conv2d_batch_info(const conv2d_batch_t* batch, int index, int* algo, int* gemm_bn) {
    const Batch* b = reinterpret_cast<const Batch*>(batch);
    if (!b || index < 0 || index >= static_cast<int>(b->plans.size())) return set_last_error(CONV2D_ERR_INVALID, "bad index");
    const Plan& p = *b->plans[index];
    if (algo) *algo = p.algo;
    if (gemm_bn) *gemm_bn = p.algo == CONV2D_ALGO_2X3_FUSED ? 32 : p.algo == CONV2D_ALGO_4X3_ROW ? 64 : p.gemm_full.bn;
    return CONV2D_OK;
}

int conv2d_batch_launches(const conv2d_batch_t* batch, int grouped) {
    const Batch* b = reinterpret_cast<const Batch*>(batch);
    if (!b) return -1;
    if (grouped) return b->grouped_launches;
    int n = 0;
    for (const auto& p : b->plans) n += p->launches;
    return n;
}

int conv2d_batch_check_device(conv2d_batch_t* batch, int* site) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    if (!b) return set_last_error(CONV2D_ERR_INVALID, "null batch");
    if (cudaDeviceSynchronize() != cudaSuccess) return set_last_error(CONV2D_ERR_CUDA, "device synchronize failed");
    unsigned code = 0;
    DevErr h{};
    cudaMemcpy(&h, b->err, sizeof(h), cudaMemcpyDeviceToHost);
    code = h.code;
    for (auto& p : b->plans) {
        cudaMemcpy(&h, p->err, sizeof(h), cudaMemcpyDeviceToHost);
        if (!code) code = h.code;
    }
    if (site) *site = static_cast<int>(code);
    return code ? set_last_error(CONV2D_ERR_TIMEOUT, "a kernel gave up a bounded wait") : CONV2D_OK;
}

int conv2d_batch_destroy(conv2d_batch_t* batch) {
    Batch* b = reinterpret_cast<Batch*>(batch);
    if (!b) return set_last_error(CONV2D_ERR_INVALID, "null batch");
    cudaDeviceSynchronize();
    delete b;
    return CONV2D_OK;
}

}  // extern "C"
