// Serving loop: continuous batching of conv2d requests over resident layers.
//
// A server owns
//   * layers: the filter of each is transformed once, for F(2x3) and F(4x3),
//     and stays on the device;
//   * a workspace arena of the configured HBM budget, from which every
//     admitted request takes its Winograd-domain buffers (V and M) and to
//     which it returns them when it completes;
//   * `slots` in-flight batches, each on its own stream.
// A scheduler thread admits queued requests in arrival order while their
// workspace fits in the arena, packs what it admitted into a batch (at most
// `max_batch` requests), and launches the batch as grouped kernels on a free
// slot: one input-transform launch per transform family, one persistent GEMM
// launch per (channel tile, M type) over every request's tiles, one
// output-transform launch per family.  Requests that arrive while other
// batches are on the GPU are admitted as soon as a slot and workspace free
// up, and their batch runs concurrently with the ones still in flight.
// A request's arithmetic does not depend on what else is in its batch, so its
// result is bit-identical alone and in the mix.
//
// With `per_request` set the server is instead the plain per-call path the
// batching is measured against: every request's own kernels (the single-
// problem launches conv2d_fp16_ex makes: input transform, GEMM, output
// transform) are queued on one stream as the request is submitted, in
// arrival order, with no batching and no wait for earlier requests; since
// they run in stream order they share one workspace region.  Completion is
// observed the same way in both modes (an event per request or batch, polled
// by the scheduler thread).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/conv2d.h"
#include "wg_kernels.h"
#include "wg_plan.h"

namespace wg {

namespace {

double now_us() {
    using namespace std::chrono;
    return duration<double, std::micro>(steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over one device arena (offsets, 256-byte granules).
class Arena {
   public:
    void init(size_t bytes) {
        free_.clear();
        free_[0] = bytes;
        cap_ = bytes;
    }
    bool alloc(size_t bytes, size_t* off) {
        bytes = (bytes + 255) / 256 * 256;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes;
                const size_t start = it->first + bytes;
                free_.erase(it);
                if (rest) free_[start] = rest;
                used_ += bytes;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = (bytes + 255) / 256 * 256;
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t used() const { return used_; }
    size_t capacity() const { return cap_; }

   private:
    std::map<size_t, size_t> free_;
    size_t cap_ = 0, used_ = 0;
};

struct Layer {
    unsigned c, k, h, w, p, q;
    void* U2 = nullptr;  // F(2x3) transformed filter
    void* U4 = nullptr;  // F(4x3)
};

struct Request {
    long long id;
    int layer;
    unsigned n;
    const void* in;
    void* out;
    double t_arrive, t_start = 0, t_done = 0;
    int m;              // 2 or 4
    size_t ws_off = 0, ws_bytes = 0;
    bool done = false;
};

struct Slot {
    cudaStream_t stream = nullptr;
    // a batch's F(2x3) chain runs on stream2, beside its F(4x3) chain
    cudaStream_t stream2 = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaEvent_t start = nullptr;   // timing events: the batch's device interval
    cudaEvent_t done = nullptr;
    void* desc_dev = nullptr;
    void* desc_host = nullptr;   // pinned staging
    size_t desc_bytes = 0;
    std::vector<long long> reqs;
    bool busy = false;
};

constexpr size_t kDescBytesPerRequest = sizeof(GemmDesc) + sizeof(InDesc) + sizeof(OutDesc) + 256;

}  // namespace

struct Server {
    conv2d_server_config_t cfg{};
    int device = 0, num_sms = 1;
    std::vector<Layer> layers;
    void* arena_base = nullptr;
    void* ufilt = nullptr;       // resident transformed filters of all layers (grown per layer)
    std::vector<void*> u_blocks;
    DevErr* err = nullptr;
    Arena arena;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<long long> pending;
    std::unordered_map<long long, Request> reqs;
    long long next_id = 1;
    std::atomic<bool> stop{false};
    std::thread sched;
    long long completed = 0;
    double flops_done = 0;
    int batches = 0, batch_requests = 0, max_inflight = 0;
    // device intervals [start, done] of completed batches (ms from t0_ev)
    cudaEvent_t t0_ev = nullptr;
    std::vector<std::pair<float, float>> intervals;
    // plain per-request mode: one stream, requests in flight in stream order
    cudaStream_t plain_stream = nullptr;
    struct Inflight {
        long long id;
        cudaEvent_t ev;
    };
    std::deque<Inflight> plain_inflight;
    std::vector<cudaEvent_t> event_pool;

    ~Server() {
        stop = true;
        cv.notify_all();
        if (sched.joinable()) sched.join();
        if (plain_stream) {
            cudaStreamSynchronize(plain_stream);
            cudaStreamDestroy(plain_stream);
        }
        for (Inflight& f : plain_inflight) cudaEventDestroy(f.ev);
        for (cudaEvent_t e : event_pool) cudaEventDestroy(e);
        if (t0_ev) cudaEventDestroy(t0_ev);
        for (Slot& s : slots) {
            if (s.stream) cudaStreamSynchronize(s.stream);
            if (s.stream) cudaStreamDestroy(s.stream);
            if (s.stream2) cudaStreamSynchronize(s.stream2);
            if (s.stream2) cudaStreamDestroy(s.stream2);
            if (s.fork) cudaEventDestroy(s.fork);
            if (s.join) cudaEventDestroy(s.join);
            if (s.start) cudaEventDestroy(s.start);
            if (s.done) cudaEventDestroy(s.done);
            if (s.desc_dev) cudaFree(s.desc_dev);
            if (s.desc_host) cudaFreeHost(s.desc_host);
        }
        for (void* p : u_blocks) cudaFree(p);
        if (arena_base) cudaFree(arena_base);
        if (err) cudaFree(err);
    }

    // M storage: 24-bit for F(4x3), fp16 for F(2x3) (as a plan of the shape has it)
    static MType mtype_for(int m) { return m == 4 ? MType::F24 : MType::F16; }

    static size_t ws_bytes_for(const Geom& g) {
        const long long E = g.alpha * g.alpha;
        const size_t v = static_cast<size_t>(E * round_rows(g.P) * g.cp * 2);
        const size_t m = static_cast<size_t>(m_bytes(mtype_for(g.m), E, g.P, g.kp));
        return (v + 255) / 256 * 256 + (m + 255) / 256 * 256;
    }

    int choose_m(const Layer& L) const {
        if (cfg.algo == CONV2D_ALGO_4X3_NON_FUSED) return 4;
        if (cfg.algo == CONV2D_ALGO_2X3_NON_FUSED) return 2;
        // F(4x3) does 44% of F(2x3)'s GEMM work but moves more bytes per tile;
        // it wins once both channel counts are wide and the image is not tiny
        return (std::min(L.c, L.k) >= 128 && L.h >= 14 && L.w >= 14) ? 4 : 2;
    }

    // launch one batch (requests already admitted: workspace assigned)
    int launch(Slot& slot) {
        std::vector<InDesc> in2, in4;
        std::vector<OutDesc> out2, out4;
        std::map<std::pair<int, int>, std::vector<GemmDesc>> gemm;  // (bn, m) -> descs
        long long blk_in2 = 0, blk_in4 = 0, blk_out2 = 0, blk_out4 = 0;
        int smem2 = 0, smem4 = 0;
        char* arena = static_cast<char*>(arena_base);
        for (long long id : slot.reqs) {
            Request& r = reqs[id];
            const Layer& L = layers[r.layer];
            const Geom g = make_geom(r.n, L.c, L.h, L.w, L.k, L.p, L.q, r.m);
            const int E = g.alpha * g.alpha;
            char* V = arena + r.ws_off;
            char* Mw = V + (static_cast<size_t>(E) * round_rows(g.P) * g.cp * 2 + 255) / 256 * 256;
            const void* x_end = static_cast<const uint16_t*>(r.in) + static_cast<long long>(r.n) * L.c * L.h * L.w;
            int smem = 0;
            InDesc di = make_in_desc(g, r.in, x_end, V, nullptr, &smem);
            OutDesc dout = make_out_desc(g, mtype_for(r.m), Mw, r.out, nullptr);
            GemmDesc dg;
            const int bn = default_bn(static_cast<int>(L.k));
            if (make_gemm_desc(dg, OpType::F16, E, g.P, L.k, g.kp, g.cp, V, r.m == 4 ? L.U4 : L.U2, Mw, mtype_for(r.m), bn) !=
                cudaSuccess)
                return set_last_error(CONV2D_ERR_CUDA, "tensor map encoding failed");
            if (r.m == 2) {
                di.blk_begin = blk_in2;
                blk_in2 += di.gx * di.gy;
                smem2 = std::max(smem2, smem);
                in2.push_back(di);
                dout.blk_begin = blk_out2;
                blk_out2 += dout.gx * dout.gy;
                out2.push_back(dout);
            } else {
                di.blk_begin = blk_in4;
                blk_in4 += di.gx * di.gy;
                smem4 = std::max(smem4, smem);
                in4.push_back(di);
                dout.blk_begin = blk_out4;
                blk_out4 += dout.gx * dout.gy;
                out4.push_back(dout);
            }
            gemm[{bn, r.m}].push_back(dg);
        }
        // descriptors: GemmDesc[] | InDesc[] | OutDesc[] in the slot's staging area
        char* h = static_cast<char*>(slot.desc_host);
        size_t off = 0;
        struct GG {
            int bn, m;
            size_t off;
            int n;
            long long tiles;
        };
        std::vector<GG> gg;
        for (auto& kv : gemm) {
            long long t = 0;
            for (GemmDesc& d : kv.second) {
                d.tile_begin = t;
                t += d.tiles;
            }
            std::memcpy(h + off, kv.second.data(), kv.second.size() * sizeof(GemmDesc));
            gg.push_back({kv.first.first, kv.first.second, off, static_cast<int>(kv.second.size()), t});
            off += kv.second.size() * sizeof(GemmDesc);
        }
        const size_t o_in2 = off;
        std::memcpy(h + off, in2.data(), in2.size() * sizeof(InDesc));
        off += in2.size() * sizeof(InDesc);
        const size_t o_in4 = off;
        std::memcpy(h + off, in4.data(), in4.size() * sizeof(InDesc));
        off += in4.size() * sizeof(InDesc);
        const size_t o_out2 = off;
        std::memcpy(h + off, out2.data(), out2.size() * sizeof(OutDesc));
        off += out2.size() * sizeof(OutDesc);
        const size_t o_out4 = off;
        std::memcpy(h + off, out4.data(), out4.size() * sizeof(OutDesc));
        off += out4.size() * sizeof(OutDesc);
        cudaStream_t s = slot.stream;
        char* d = static_cast<char*>(slot.desc_dev);
        cudaEventRecord(slot.start, s);
        if (cudaMemcpyAsync(d, h, off, cudaMemcpyHostToDevice, s) != cudaSuccess)
            return set_last_error(CONV2D_ERR_CUDA, "descriptor copy failed");
        cudaError_t e = cudaSuccess;
        // with requests of both transforms, the F(2x3) chain goes to stream2
        // (forked after the descriptor copy, joined before `done`) and runs
        // beside the F(4x3) chain
        const bool both = !in2.empty() && !in4.empty();
        cudaStream_t s2 = both ? slot.stream2 : s;
        if (both) {
            if ((e = cudaEventRecord(slot.fork, s)) == cudaSuccess) e = cudaStreamWaitEvent(s2, slot.fork, 0);
        }
        if (!in2.empty() && e == cudaSuccess)
            e = launch_input_transform_grouped(Xform::F2, OpType::F16, reinterpret_cast<const InDesc*>(d + o_in2),
                                               static_cast<int>(in2.size()), blk_in2, smem2, false, err, s2);
        for (const GG& g : gg)
            if (g.m == 2 && e == cudaSuccess)
                e = launch_gemm_grouped(reinterpret_cast<const GemmDesc*>(d + g.off), g.n, g.tiles, OpType::F16, mtype_for(g.m),
                                        g.bn, static_cast<int>(std::min<long long>(g.tiles, num_sms)), err, s2);
        if (!out2.empty() && e == cudaSuccess)
            e = launch_output_transform_grouped(Xform::F2, MType::F16, reinterpret_cast<const OutDesc*>(d + o_out2),
                                                static_cast<int>(out2.size()), blk_out2, err, s2);
        if (!in4.empty() && e == cudaSuccess)
            e = launch_input_transform_grouped(Xform::F4, OpType::F16, reinterpret_cast<const InDesc*>(d + o_in4),
                                               static_cast<int>(in4.size()), blk_in4, smem4, false, err, s);
        for (const GG& g : gg)
            if (g.m == 4 && e == cudaSuccess)
                e = launch_gemm_grouped(reinterpret_cast<const GemmDesc*>(d + g.off), g.n, g.tiles, OpType::F16, mtype_for(g.m),
                                        g.bn, static_cast<int>(std::min<long long>(g.tiles, num_sms)), err, s);
        if (!out4.empty() && e == cudaSuccess)
            e = launch_output_transform_grouped(Xform::F4, MType::F24, reinterpret_cast<const OutDesc*>(d + o_out4),
                                                static_cast<int>(out4.size()), blk_out4, err, s);
        if (both && e == cudaSuccess) {
            if ((e = cudaEventRecord(slot.join, s2)) == cudaSuccess) e = cudaStreamWaitEvent(s, slot.join, 0);
        }
        if (e == cudaSuccess) e = cudaEventRecord(slot.done, s);
        if (e != cudaSuccess) return set_last_error(CONV2D_ERR_CUDA, cudaGetErrorString(e));
        return CONV2D_OK;
    }

    // Plain per-request mode: the request's own single-problem launches on the
    // plain stream (the same launches conv2d_fp16_ex makes for this shape),
    // then an event that marks its completion.  Caller holds `mu`.
    int launch_plain(Request& r) {
        const Layer& L = layers[r.layer];
        const Geom g = make_geom(r.n, L.c, L.h, L.w, L.k, L.p, L.q, r.m);
        const int E = g.alpha * g.alpha;
        // requests run in stream order: all of them use the arena's start
        char* V = static_cast<char*>(arena_base);
        char* Mw = V + (static_cast<size_t>(E) * round_rows(g.P) * g.cp * 2 + 255) / 256 * 256;
        const Xform xf = r.m == 4 ? Xform::F4 : Xform::F2;
        GemmPlan gp;
        if (plan_gemm(gp, OpType::F16, E, g.P, L.k, g.kp, g.cp, V, r.m == 4 ? L.U4 : L.U2, Mw, mtype_for(r.m),
                      default_bn(static_cast<int>(L.k)), num_sms) != cudaSuccess)
            return set_last_error(CONV2D_ERR_CUDA, "tensor map encoding failed");
        const void* x_end = static_cast<const uint16_t*>(r.in) + static_cast<long long>(r.n) * L.c * L.h * L.w;
        cudaError_t e = launch_input_transform(xf, OpType::F16, g, r.in, x_end, V, nullptr, err, plain_stream);
        if (e == cudaSuccess) e = launch_gemm(gp, err, plain_stream);
        if (e == cudaSuccess) e = launch_output_transform(xf, mtype_for(r.m), g, Mw, r.out, nullptr, err, plain_stream);
        cudaEvent_t ev = nullptr;
        if (e == cudaSuccess) {
            if (event_pool.empty()) {
                e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            } else {
                ev = event_pool.back();
                event_pool.pop_back();
            }
        }
        if (e == cudaSuccess) e = cudaEventRecord(ev, plain_stream);
        if (e != cudaSuccess) {
            if (ev) event_pool.push_back(ev);
            return set_last_error(CONV2D_ERR_CUDA, cudaGetErrorString(e));
        }
        plain_inflight.push_back({r.id, ev});
        ++batches;
        ++batch_requests;
        max_inflight = std::max(max_inflight, static_cast<int>(plain_inflight.size()));
        return CONV2D_OK;
    }

    void complete(Request& r, double t) {
        r.t_done = t;
        r.done = true;
        const Layer& L = layers[r.layer];
        flops_done += 2.0 * r.n * L.k * (L.h + 2.0 * L.p - 2) * (L.w + 2.0 * L.q - 2) * L.c * 9;
        ++completed;
    }

    bool per_request() const { return cfg.per_request != 0; }

    void loop() {
        cudaSetDevice(device);
        while (true) {
            std::unique_lock<std::mutex> lk(mu);
            // completions
            int inflight = 0;
            while (!plain_inflight.empty() && cudaEventQuery(plain_inflight.front().ev) == cudaSuccess) {
                complete(reqs[plain_inflight.front().id], now_us());
                event_pool.push_back(plain_inflight.front().ev);
                plain_inflight.pop_front();
                cv.notify_all();
            }
            inflight += static_cast<int>(plain_inflight.size());
            for (Slot& s : slots) {
                if (!s.busy) continue;
                if (cudaEventQuery(s.done) == cudaSuccess) {
                    const double t = now_us();
                    for (long long id : s.reqs) {
                        Request& r = reqs[id];
                        arena.release(r.ws_off, r.ws_bytes);
                        complete(r, t);
                    }
                    float a = 0.f, b = 0.f;
                    if (cudaEventElapsedTime(&a, t0_ev, s.start) == cudaSuccess &&
                        cudaEventElapsedTime(&b, t0_ev, s.done) == cudaSuccess)
                        intervals.emplace_back(a, b);
                    s.reqs.clear();
                    s.busy = false;
                    cv.notify_all();
                } else {
                    ++inflight;
                }
            }
            // admission: arrival order, while a slot and workspace are free
            Slot* free_slot = nullptr;
            for (Slot& s : slots)
                if (!s.busy) {
                    free_slot = &s;
                    break;
                }
            if (free_slot && !pending.empty()) {
                std::vector<long long> batch;
                while (!pending.empty() && static_cast<int>(batch.size()) < cfg.max_batch) {
                    Request& r = reqs[pending.front()];
                    const Layer& L = layers[r.layer];
                    const Geom g = make_geom(r.n, L.c, L.h, L.w, L.k, L.p, L.q, r.m);
                    r.ws_bytes = ws_bytes_for(g);
                    size_t off = 0;
                    if (!arena.alloc(r.ws_bytes, &off)) break;  // wait for workspace
                    r.ws_off = off;
                    r.t_start = now_us();
                    batch.push_back(pending.front());
                    pending.pop_front();
                }
                if (!batch.empty()) {
                    free_slot->reqs = batch;
                    free_slot->busy = true;
                    ++batches;
                    batch_requests += static_cast<int>(batch.size());
                    if (launch(*free_slot) != CONV2D_OK) {
                        // a launch that fails completes its requests at once
                        for (long long id : batch) {
                            reqs[id].done = true;
                            reqs[id].t_done = now_us();
                            arena.release(reqs[id].ws_off, reqs[id].ws_bytes);
                        }
                        free_slot->reqs.clear();
                        free_slot->busy = false;
                    }
                    max_inflight = std::max(max_inflight, inflight + 1);
                    continue;
                }
            }
            if (stop && pending.empty() && inflight == 0) break;
            if (inflight == 0 && pending.empty())
                cv.wait_for(lk, std::chrono::microseconds(200));
            else {
                lk.unlock();
                std::this_thread::sleep_for(std::chrono::microseconds(5));
            }
        }
    }
};

}  // namespace wg

using namespace wg;

extern "C" {

int conv2d_server_config_default(conv2d_server_config_t* cfg) {
    if (!cfg) return set_last_error(CONV2D_ERR_INVALID, "null config");
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->hbm_budget_bytes = 40ll << 30;
    // measured on the 2,000-request trace of 16 layers (all arriving at once):
    // 3 slots x 64 requests 864 TFLOP/s, 6 x 16 895, 8 x 16 897; smaller
    // batches in more slots overlap better
    cfg->max_batch = 16;
    cfg->slots = 6;
    cfg->algo = CONV2D_ALGO_AUTO;
    return CONV2D_OK;
}

int conv2d_server_create(const conv2d_server_config_t* cfg, conv2d_server_t** out) {
    if (!cfg || !out) return set_last_error(CONV2D_ERR_INVALID, "null argument");
    if (cfg->slots < 1 || cfg->max_batch < 1 || cfg->hbm_budget_bytes < (1 << 20))
        return set_last_error(CONV2D_ERR_INVALID, "bad server config");
    std::unique_ptr<Server> sv(new Server());
    sv->cfg = *cfg;
    cudaGetDevice(&sv->device);
    cudaDeviceGetAttribute(&sv->num_sms, cudaDevAttrMultiProcessorCount, sv->device);
    if (cudaMalloc(&sv->arena_base, static_cast<size_t>(cfg->hbm_budget_bytes)) != cudaSuccess) {
        cudaGetLastError();
        return set_last_error(CONV2D_ERR_NOMEM, "workspace arena allocation failed");
    }
    sv->arena.init(static_cast<size_t>(cfg->hbm_budget_bytes));
    if (cudaMalloc(&sv->err, 256) != cudaSuccess) return set_last_error(CONV2D_ERR_NOMEM, "allocation failed");
    cudaMemset(sv->err, 0, 256);
    if (cudaEventCreate(&sv->t0_ev) != cudaSuccess || cudaEventRecord(sv->t0_ev, nullptr) != cudaSuccess)
        return set_last_error(CONV2D_ERR_CUDA, "event setup failed");
    if (cfg->per_request && cudaStreamCreateWithFlags(&sv->plain_stream, cudaStreamNonBlocking) != cudaSuccess)
        return set_last_error(CONV2D_ERR_CUDA, "stream setup failed");
    sv->slots.resize(cfg->per_request ? 0 : cfg->slots);
    for (Slot& s : sv->slots) {
        s.desc_bytes = static_cast<size_t>(cfg->max_batch) * kDescBytesPerRequest + 4096;
        if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&s.stream2, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&s.fork, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&s.join, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreate(&s.start) != cudaSuccess || cudaEventCreate(&s.done) != cudaSuccess ||
            cudaMalloc(&s.desc_dev, s.desc_bytes) != cudaSuccess ||
            cudaMallocHost(&s.desc_host, s.desc_bytes) != cudaSuccess)
            return set_last_error(CONV2D_ERR_NOMEM, "slot setup failed");
    }
    Server* raw = sv.get();
    sv->sched = std::thread([raw] { raw->loop(); });
    *out = reinterpret_cast<conv2d_server_t*>(sv.release());
    return CONV2D_OK;
}

int conv2d_server_add_layer(conv2d_server_t* server, unsigned c, unsigned k, unsigned h, unsigned w, unsigned p,
                            unsigned q, const void* weight, int* layer) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv || !weight || !layer) return set_last_error(CONV2D_ERR_INVALID, "null argument");
    problem_t pr{reinterpret_cast<void*>(16), const_cast<void*>(weight), reinterpret_cast<void*>(16), 1, c, h, w, k, 3, 3,
                 1, 1, p, q};
    int st = validate_problem(&pr);
    if (st) return st;
    Layer L{c, k, h, w, p, q};
    const int cp = (c + 7) / 8 * 8, kp = (k + 7) / 8 * 8;
    const size_t b2 = static_cast<size_t>(16) * kp * cp * 2, b4 = static_cast<size_t>(36) * kp * cp * 2;
    void* blk = nullptr;
    if (cudaMalloc(&blk, b2 + b4) != cudaSuccess) return set_last_error(CONV2D_ERR_NOMEM, "filter allocation failed");
    sv->u_blocks.push_back(blk);
    L.U2 = blk;
    L.U4 = static_cast<char*>(blk) + b2;
    if (launch_filter_transform(Xform::F2, OpType::F16, weight, L.U2, k, c, cp, nullptr) != cudaSuccess ||
        launch_filter_transform(Xform::F4, OpType::F16, weight, L.U4, k, c, cp, nullptr) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess)
        return set_last_error(CONV2D_ERR_CUDA, "filter transform failed");
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->layers.push_back(L);
    *layer = static_cast<int>(sv->layers.size()) - 1;
    return CONV2D_OK;
}

int conv2d_server_submit(conv2d_server_t* server, int layer, unsigned n, const void* in, void* out,
                         long long* request) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv || !in || !out || n == 0) return set_last_error(CONV2D_ERR_INVALID, "bad request");
    std::lock_guard<std::mutex> lk(sv->mu);
    if (layer < 0 || layer >= static_cast<int>(sv->layers.size())) return set_last_error(CONV2D_ERR_INVALID, "bad layer");
    const Layer& L = sv->layers[layer];
    Request r;
    r.id = sv->next_id++;
    r.layer = layer;
    r.n = n;
    r.in = in;
    r.out = out;
    r.t_arrive = now_us();
    r.m = sv->choose_m(L);
    const Geom g = make_geom(n, L.c, L.h, L.w, L.k, L.p, L.q, r.m);
    if (Server::ws_bytes_for(g) > sv->arena.capacity())
        return set_last_error(CONV2D_ERR_BUSY, "request workspace exceeds the server's HBM budget");
    sv->reqs[r.id] = r;
    if (request) *request = r.id;
    if (sv->per_request()) {
        // plain path: the request's kernels are queued now, behind the
        // requests submitted before it
        DeviceGuard dg(sv->device);
        Request& q = sv->reqs[r.id];
        q.t_start = q.t_arrive;
        const int st = sv->launch_plain(q);
        if (st) {
            sv->reqs.erase(r.id);
            return st;
        }
        sv->cv.notify_all();
        return CONV2D_OK;
    }
    sv->pending.push_back(r.id);
    sv->cv.notify_all();
    return CONV2D_OK;
}

int conv2d_server_poll(conv2d_server_t* server, long long request, double* latency_us) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv) return -1;
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(request);
    if (it == sv->reqs.end()) return -1;
    if (!it->second.done) return 0;
    if (latency_us) *latency_us = it->second.t_done - it->second.t_arrive;
    return 1;
}

int conv2d_server_wait_all(conv2d_server_t* server) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv) return set_last_error(CONV2D_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(sv->mu);
    sv->cv.wait(lk, [sv] {
        if (!sv->pending.empty() || !sv->plain_inflight.empty()) return false;
        for (const Slot& s : sv->slots)
            if (s.busy) return false;
        return true;
    });
    return CONV2D_OK;
}

int conv2d_server_replay(conv2d_server_t* server, int count, const int* layer, const unsigned* n,
                         const double* arrival_us, const void* const* in, void* const* out, double* latency_us,
                         double* wall_us) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv || count <= 0 || !layer || !n || !arrival_us || !in || !out || !latency_us)
        return set_last_error(CONV2D_ERR_INVALID, "bad replay arguments");
    std::vector<long long> ids(count);
    const double t0 = now_us();
    for (int i = 0; i < count; ++i) {
        while (now_us() - t0 < arrival_us[i]) {
        }
        const int st = conv2d_server_submit(server, layer[i], n[i], in[i], out[i], &ids[i]);
        if (st) return st;
    }
    conv2d_server_wait_all(server);
    if (wall_us) *wall_us = now_us() - t0;
    std::lock_guard<std::mutex> lk(sv->mu);
    for (int i = 0; i < count; ++i) {
        const Request& r = sv->reqs[ids[i]];
        latency_us[i] = r.t_done - r.t_arrive;
    }
    for (int i = 0; i < count; ++i) sv->reqs.erase(ids[i]);
    return CONV2D_OK;
}

int conv2d_server_stats(conv2d_server_t* server, conv2d_server_stats_t* st) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv || !st) return set_last_error(CONV2D_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    st->completed = sv->completed;
    st->batches = sv->batches;
    st->mean_batch = sv->batches ? static_cast<double>(sv->batch_requests) / sv->batches : 0.0;
    st->max_inflight_batches = sv->max_inflight;
    st->arena_used_bytes = static_cast<long long>(sv->arena.used());
    st->flops = sv->flops_done;
    // sweep the completed batches' device intervals: time covered by at
    // least one batch, and by two or more at once
    std::vector<std::pair<float, int>> edges;
    edges.reserve(2 * sv->intervals.size());
    for (const auto& iv : sv->intervals) {
        edges.emplace_back(iv.first, 1);
        edges.emplace_back(iv.second, -1);
    }
    std::sort(edges.begin(), edges.end());
    double busy = 0, overlap = 0;
    int depth = 0;
    for (size_t i = 0; i < edges.size(); ++i) {
        if (i > 0) {
            const double dt = edges[i].first - edges[i - 1].first;
            if (depth >= 1) busy += dt;
            if (depth >= 2) overlap += dt;
        }
        depth += edges[i].second;
    }
    st->busy_us = busy * 1e3;
    st->overlap_us = overlap * 1e3;
    return CONV2D_OK;
}

// ---- resident layers to and from a file (warm restart) ----------------------
// magic "WGCSRVL1", version, layer count; per layer its geometry, the byte
// counts of its F(2x3) and F(4x3) filters and an FNV-1a checksum of both;
// then the filters as they lie in device memory (U[E][Cp/8][Kp][8], fp16).

namespace {

constexpr char kServerMagic[8] = {'W', 'G', 'C', 'S', 'R', 'V', 'L', '1'};

struct LayerRecord {
    uint32_t c, k, h, w, p, q;
    uint64_t b2, b4, checksum;
};

uint64_t fnv1a64(const unsigned char* p, size_t n, uint64_t h = 1469598103934665603ull) {
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

}  // namespace

int conv2d_server_save_layers(conv2d_server_t* server, const char* path) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv || !path) return set_last_error(CONV2D_ERR_INVALID, "null argument");
    std::vector<Layer> layers;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        layers = sv->layers;
    }
    std::vector<LayerRecord> recs;
    std::vector<std::vector<unsigned char>> data;
    for (const Layer& L : layers) {
        const uint64_t cp = (L.c + 7) / 8 * 8, kp = (L.k + 7) / 8 * 8;
        LayerRecord r{L.c, L.k, L.h, L.w, L.p, L.q, 16 * kp * cp * 2, 36 * kp * cp * 2, 0};
        std::vector<unsigned char> buf(r.b2 + r.b4);
        if (cudaMemcpy(buf.data(), L.U2, r.b2, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(buf.data() + r.b2, L.U4, r.b4, cudaMemcpyDeviceToHost) != cudaSuccess)
            return set_last_error(CONV2D_ERR_CUDA, "copy of a resident filter failed");
        r.checksum = fnv1a64(buf.data(), buf.size());
        recs.push_back(r);
        data.push_back(std::move(buf));
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return set_last_error(CONV2D_ERR_INVALID, "cannot open the layer file for writing");
    const uint32_t version = 1, count = static_cast<uint32_t>(recs.size());
    bool ok = std::fwrite(kServerMagic, 8, 1, f) == 1 && std::fwrite(&version, 4, 1, f) == 1 &&
              std::fwrite(&count, 4, 1, f) == 1 &&
              (recs.empty() || std::fwrite(recs.data(), sizeof(LayerRecord), recs.size(), f) == recs.size());
    for (const auto& d : data) ok = ok && std::fwrite(d.data(), 1, d.size(), f) == d.size();
    if (std::fclose(f) != 0 || !ok) return set_last_error(CONV2D_ERR_INVALID, "layer file write failed");
    return CONV2D_OK;
}

int conv2d_server_load_layers(conv2d_server_t* server, const char* path, int* first_layer, int* count) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv || !path) return set_last_error(CONV2D_ERR_INVALID, "null argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return set_last_error(CONV2D_ERR_INVALID, "cannot open the layer file");
    char magic[8];
    uint32_t version = 0, n = 0;
    bool ok = std::fread(magic, 8, 1, f) == 1 && std::fread(&version, 4, 1, f) == 1 && std::fread(&n, 4, 1, f) == 1 &&
              std::memcmp(magic, kServerMagic, 8) == 0 && version == 1 && n < (1u << 20);
    std::vector<LayerRecord> recs(ok ? n : 0);
    if (ok && n) ok = std::fread(recs.data(), sizeof(LayerRecord), n, f) == n;
    std::vector<std::vector<unsigned char>> data;
    for (uint32_t i = 0; ok && i < n; ++i) {
        const LayerRecord& r = recs[i];
        const uint64_t cp = (r.c + 7) / 8 * 8, kp = (r.k + 7) / 8 * 8;
        problem_t pr{reinterpret_cast<void*>(16), reinterpret_cast<void*>(16), reinterpret_cast<void*>(16), 1, r.c, r.h,
                     r.w, r.k, 3, 3, 1, 1, r.p, r.q};
        if (validate_problem(&pr) != CONV2D_OK || r.b2 != 16 * kp * cp * 2 || r.b4 != 36 * kp * cp * 2) {
            ok = false;
            break;
        }
        std::vector<unsigned char> buf(r.b2 + r.b4);
        ok = std::fread(buf.data(), 1, buf.size(), f) == buf.size() && fnv1a64(buf.data(), buf.size()) == r.checksum;
        data.push_back(std::move(buf));
    }
    std::fclose(f);
    if (!ok) return set_last_error(CONV2D_ERR_INVALID, "not a valid layer file (magic, version, sizes or checksum)");
    int first = -1;
    for (uint32_t i = 0; i < n; ++i) {
        const LayerRecord& r = recs[i];
        void* blk = nullptr;
        if (cudaMalloc(&blk, r.b2 + r.b4) != cudaSuccess) return set_last_error(CONV2D_ERR_NOMEM, "filter allocation failed");
        if (cudaMemcpy(blk, data[i].data(), r.b2 + r.b4, cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaFree(blk);
            return set_last_error(CONV2D_ERR_CUDA, "copy of a resident filter failed");
        }
        Layer L{r.c, r.k, r.h, r.w, r.p, r.q};
        L.U2 = blk;
        L.U4 = static_cast<char*>(blk) + r.b2;
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->u_blocks.push_back(blk);
        sv->layers.push_back(L);
        if (first < 0) first = static_cast<int>(sv->layers.size()) - 1;
    }
    if (first_layer) *first_layer = first;
    if (count) *count = static_cast<int>(n);
    return CONV2D_OK;
}

int conv2d_server_destroy(conv2d_server_t* server) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv) return set_last_error(CONV2D_ERR_INVALID, "null server");
    conv2d_server_wait_all(server);
    delete sv;
    return CONV2D_OK;
}

}  // extern "C"
