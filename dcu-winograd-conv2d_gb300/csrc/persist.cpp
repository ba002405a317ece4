// Plan persistence: the Winograd-domain filter U of a plan written to a file
// together with what it was made for, and read back into a plan of the same
// layer, so a restarted process skips the filter transform (and, with the
// autotuner's WG_CONV2D_TUNE_FILE, the tuning runs).  The reference has no
// counterpart (it transforms the filter on every call).
//
// File: a fixed header (magic, version, the layer's C, K, padding, the
// transform, operand type and padded sizes, the byte count and an FNV-1a
// checksum of the payload) followed by U exactly as it lies in device memory:
// U[E][Cp/8][Kp][8] in the operand type, or for the row F(4x3) kernel
// U1[18][Cp16/8][Kp64][8] fp16 (its own transform code in the header).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/conv2d.h"
#include "wg_plan.h"

namespace wg {

namespace {

constexpr char kPlanMagic[8] = {'W', 'G', 'C', 'P', 'L', 'A', 'N', '1'};

struct PlanFileHeader {
    char magic[8];
    uint32_t version;
    uint32_t c, k, p, q;
    int32_t xform, op;
    uint32_t e, cp, kp;
    uint64_t u_bytes;
    uint64_t checksum;
};

uint64_t fnv1a(const unsigned char* p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

PlanFileHeader header_of(const Plan& pl) {
    PlanFileHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kPlanMagic, 8);
    h.version = 1;
    h.c = pl.prob.c;
    h.k = pl.prob.k;
    h.p = pl.prob.p;
    h.q = pl.prob.q;
    h.xform = static_cast<int32_t>(pl.xf) + (pl.algo == CONV2D_ALGO_4X3_ROW ? 16 : 0);   // row F(4x3): own layout
    h.op = static_cast<int32_t>(pl.op);
    h.e = static_cast<uint32_t>(pl.g.alpha * pl.g.alpha);
    h.cp = static_cast<uint32_t>(pl.g.cp);
    h.kp = static_cast<uint32_t>(pl.g.kp);
    h.u_bytes = static_cast<uint64_t>(pl.u_bytes);
    return h;
}

}  // namespace

}  // namespace wg

using namespace wg;

extern "C" {

int conv2d_plan_save(const void* param, const char* path) {
    Plan* pl = plan_of(param);
    if (!pl || !path) return set_last_error(CONV2D_ERR_INVALID, "param blob not set up, or null path");
    DeviceGuard dg(pl->device);
    if (!pl->filter_ready || pl->opt.filter_policy == 1) {
        const int st = pl->filter(nullptr);
        if (st) return st;
    }
    PlanFileHeader h = header_of(*pl);
    std::vector<unsigned char> u(h.u_bytes);
    if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(u.data(), pl->U, h.u_bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
        return set_last_error(CONV2D_ERR_CUDA, "copy of the transformed filter failed");
    h.checksum = fnv1a(u.data(), u.size());
    FILE* f = std::fopen(path, "wb");
    if (!f) return set_last_error(CONV2D_ERR_INVALID, "cannot open the plan file for writing");
    const bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(u.data(), 1, u.size(), f) == u.size();
    if (std::fclose(f) != 0 || !ok) return set_last_error(CONV2D_ERR_INVALID, "plan file write failed");
    return CONV2D_OK;
}

int conv2d_plan_load(const void* param, const char* path) {
    Plan* pl = plan_of(param);
    if (!pl || !path) return set_last_error(CONV2D_ERR_INVALID, "param blob not set up, or null path");
    FILE* f = std::fopen(path, "rb");
    if (!f) return set_last_error(CONV2D_ERR_INVALID, "cannot open the plan file");
    PlanFileHeader h;
    std::vector<unsigned char> u;
    bool ok = std::fread(&h, sizeof(h), 1, f) == 1;
    const PlanFileHeader want = header_of(*pl);
    if (ok && (std::memcmp(h.magic, kPlanMagic, 8) != 0 || h.version != 1)) {
        std::fclose(f);
        return set_last_error(CONV2D_ERR_INVALID, "not a plan file");
    }
    if (ok && (h.c != want.c || h.k != want.k || h.xform != want.xform || h.op != want.op || h.e != want.e ||
               h.cp != want.cp || h.kp != want.kp || h.u_bytes != want.u_bytes)) {
        std::fclose(f);
        return set_last_error(CONV2D_ERR_INVALID,
                              "plan file was made for another layer, transform or operand type");
    }
    if (ok) {
        u.resize(h.u_bytes);
        ok = std::fread(u.data(), 1, u.size(), f) == u.size();
    }
    std::fclose(f);
    if (!ok) return set_last_error(CONV2D_ERR_INVALID, "plan file truncated");
    if (fnv1a(u.data(), u.size()) != h.checksum) return set_last_error(CONV2D_ERR_INVALID, "plan file checksum mismatch");
    DeviceGuard dg(pl->device);
    // U may still be read by work queued earlier on any stream
    if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(pl->U, u.data(), u.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return set_last_error(CONV2D_ERR_CUDA, "copy of the transformed filter failed");
    pl->filter_ready = true;
    return CONV2D_OK;
}

}  // extern "C"
