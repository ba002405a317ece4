// Per-shape algorithm and tile choice (CONV2D_ALGO_AUTO).
//
// The reference picks F(2x3) fused / F(2x3) / F(4x3) with fixed size rules
// (src/conv2d.cpp:83-114).  Here every candidate (algorithm x GEMM channel
// tile, plus the row-Winograd F(4x3) kernel this operator adds) is planned on scratch output memory and timed on the device the
// first time a shape is seen; the winner is cached per shape and, when
// WG_CONV2D_TUNE_FILE names a file, persisted there so later processes make
// the same choice without measuring.  The reference selection wins unless
// another candidate is more than 3% faster, so noise between nearly equal
// candidates cannot flip the choice from run to run.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "wg_plan.h"

namespace wg {

namespace {

using Key = std::tuple<unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, int, int, int>;

struct Choice {
    int algo;
    int bn;
    float ms;
};

std::mutex g_mu;
std::map<Key, Choice> g_cache;
bool g_loaded = false;

Key key_of(const problem_t& pr, const conv2d_options_t& opt) {
    return Key(pr.n, pr.c, pr.h, pr.w, pr.k, pr.p, pr.q,
               opt.operand_bf16 + 2 * opt.io_bf16 + 4 * opt.layout_nhwc + 8 * opt.m_fp32,
               opt.f4_points, opt.tile_scaling);
}

const char* tune_file() {
    const char* f = std::getenv("WG_CONV2D_TUNE_FILE");
    return (f && *f) ? f : nullptr;
}

void load_file_locked() {
    if (g_loaded) return;
    g_loaded = true;
    const char* path = tune_file();
    if (!path) return;
    FILE* fp = std::fopen(path, "r");
    if (!fp) return;
    unsigned n, c, h, w, k, p, q;
    int bf, f4, sc, algo, bn;
    float ms;
    while (std::fscanf(fp, "%u %u %u %u %u %u %u %d %d %d %d %d %f", &n, &c, &h, &w, &k, &p, &q, &bf, &f4, &sc, &algo,
                       &bn, &ms) == 13)
        g_cache[Key(n, c, h, w, k, p, q, bf, f4, sc)] = Choice{algo, bn, ms};
    std::fclose(fp);
}

void append_file_locked(const Key& kk, const Choice& ch) {
    const char* path = tune_file();
    if (!path) return;
    FILE* fp = std::fopen(path, "a");
    if (!fp) return;
    std::fprintf(fp, "%u %u %u %u %u %u %u %d %d %d %d %d %.5f\n", std::get<0>(kk), std::get<1>(kk), std::get<2>(kk),
                 std::get<3>(kk), std::get<4>(kk), std::get<5>(kk), std::get<6>(kk), std::get<7>(kk), std::get<8>(kk),
                 std::get<9>(kk), ch.algo, ch.bn, ch.ms);
    std::fclose(fp);
}

// Device time of one call of a candidate plan (best of 3 after a warm-up), or
// a negative value when the candidate cannot be planned.
float time_candidate(const problem_t& pr, conv2d_options_t opt, int algo, int bn, void* scratch_out,
                     cudaStream_t s) {
    problem_t p = pr;
    p.out = scratch_out;
    opt.algo = algo;
    opt.gemm_bn = bn;
    Plan pl;
    if (pl.build(&p, &opt) != CONV2D_OK || pl.algo != algo) return -1.f;
    if (pl.run(s) != CONV2D_OK) return -1.f;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = -1.f;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(a, s);
        if (pl.run(s) != CONV2D_OK) break;
        cudaEventRecord(b, s);
        if (cudaEventSynchronize(b) != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (best < 0.f || ms < best) best = ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamSynchronize(s);
    return best;
}

}  // namespace

int autotune_choose(const problem_t& pr, const conv2d_options_t& opt, int fallback, int* algo_out, int* bn_out) {
    const Key kk = key_of(pr, opt);
    {
        std::lock_guard<std::mutex> lk(g_mu);
        load_file_locked();
        auto it = g_cache.find(kk);
        if (it != g_cache.end()) {
            *algo_out = it->second.algo;
            *bn_out = it->second.bn;
            return CONV2D_OK;
        }
    }
    const size_t out_bytes = static_cast<size_t>(pr.n) * pr.k * (pr.h + 2 * pr.p - 2) * (pr.w + 2 * pr.q - 2) * 2;
    void* scratch = nullptr;
    if (cudaMalloc(&scratch, out_bytes) != cudaSuccess) {
        cudaGetLastError();
        *algo_out = fallback;
        *bn_out = 0;
        return CONV2D_ERR_NOMEM;
    }
    cudaStream_t s;
    cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    struct Cand {
        int algo, bn;
    };
    std::vector<Cand> cands;
    cands.push_back({CONV2D_ALGO_2X3_FUSED, 0});
    cands.push_back({CONV2D_ALGO_4X3_ROW, 0});
    const int bn0 = default_bn(static_cast<int>(pr.k));
    for (int a : {CONV2D_ALGO_2X3_NON_FUSED, CONV2D_ALGO_4X3_NON_FUSED}) {
        cands.push_back({a, bn0});
        if (pr.k > 128) cands.push_back({a, bn0 == 256 ? 128 : 256});
    }
    Choice best{fallback, 0, -1.f};
    float ref_ms = -1.f;
    int ref_bn = 0;
    for (const Cand& cd : cands) {
        const float ms = time_candidate(pr, opt, cd.algo, cd.bn, scratch, s);
        if (ms < 0.f) continue;
        if (cd.algo == fallback && (ref_ms < 0.f || ms < ref_ms)) {
            ref_ms = ms;
            ref_bn = cd.bn;
        }
        if (best.ms < 0.f || ms < best.ms) best = Choice{cd.algo, cd.bn, ms};
    }
    cudaStreamDestroy(s);
    cudaFree(scratch);
    if (ref_ms > 0.f && best.ms > 0.f && best.ms > ref_ms / 1.03f) best = Choice{fallback, ref_bn, ref_ms};
    if (best.ms < 0.f) best = Choice{fallback, 0, 0.f};
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_cache.find(kk) == g_cache.end()) {
            g_cache[kk] = best;
            append_file_locked(kk, best);
        }
    }
    *algo_out = best.algo;
    *bn_out = best.bn;
    return CONV2D_OK;
}

void autotune_clear() {
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache.clear();
    g_loaded = false;
}

}  // namespace wg
