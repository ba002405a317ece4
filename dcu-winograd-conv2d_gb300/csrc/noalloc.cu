// conv2d_fp16_noalloc: the F(2x3) non-fused convolution with its Winograd-
// domain workspace (transformed filter U, transformed input V, GEMM result M
// and the device error word) in a fixed device array that lives in this
// library, instead of memory from cudaMalloc.
//
// Who needs this: callers that must not allocate device memory while they
// run -- for example a host that gives all of its device memory to its own
// pool at start-up and has none left for a library, or a latency-bound loop
// that cannot afford cudaMalloc/cudaFree, which synchronise the device.  The
// price is a fixed array of kNoAllocScratchBytes on every GPU that loads this
// library, held until the process exits, and a size limit per call.
//
// Setup: the first call on a device, with that device current, looks up the
// array's device address (cudaGetSymbolAddress) and caches it for the device;
// make that first call before any stream capture.  Every call on a device
// uses the same array: calls whose work overlaps on the GPU (two streams, or
// two host threads) race on it and must be ordered by the caller.
//
// Errors: the kernels' bounded waits report into an error word at the start
// of the array, which every call clears first; conv2d_noalloc_check_device
// waits for the device and reports (and clears) it, as conv2d_check_device
// does for a param blob.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/conv2d.h"
#include "wg_kernels.h"
#include "wg_plan.h"
#include "wg_ptx.cuh"

namespace wg {

// 32 MiB: enough for the F(2x3) workspace of, e.g., N=1, C=K=64, 56x56
// (U 0.13 MB, V 1.6 MB, M 1.6 MB) or N=8, C=K=128, 56x56 (26 MB).
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_dev_ptr[kMaxDevices] = {};

// Device address of the array for the current device (looked up once).
cudaError_t scratch_for(int device, void** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_dev_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_dev_ptr[device] = p;
    }
    *out = g_dev_ptr[device];
    return cudaSuccess;
}

int noalloc_fail(int status, const char* msg) { return set_last_error(status, msg); }

// Test hook of the error path: one thread waits on a barrier that nothing
// completes; the bounded wait gives up after its time limit and records the
// timeout in `err`, as a kernel of the no-allocation path would.
__global__ void noalloc_expire_kernel(DevErr* err) {
    __shared__ uint64_t bar;
    mbar_init(&bar, 1);
    fence_barrier_init();
    mbar_wait(&bar, 0, nullptr, err, ERR_SITE_FULL);
}

}  // namespace

}  // namespace wg

using namespace wg;

extern "C" int conv2d_fp16_noalloc(const problem_t* problem, void* stream) {
    const int st = validate_problem(problem);
    if (st) return st;
    if (reinterpret_cast<uintptr_t>(problem->in) % 16 != 0)
        return noalloc_fail(CONV2D_ERR_UNSUPPORTED, "input pointer must be 16-byte aligned");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const Geom g = make_geom(problem->n, problem->c, problem->h, problem->w, problem->k, problem->p, problem->q, 2);
    const long long E = 16;
    auto al = [](long long b) { return (b + 255) / 256 * 256; };
    const long long bErr = 256;
    const long long bU = al(E * g.kp * g.cp * 2);
    const long long bV = al(E * round_rows(g.P) * g.cp * 2);
    const long long bM = al(E * g.P * g.kp * 2);
    if (bErr + bU + bV + bM > static_cast<long long>(kNoAllocScratchBytes))
        return noalloc_fail(CONV2D_ERR_UNSUPPORTED,
                            "problem needs more workspace than the 32 MiB no-allocation scratch holds");
    {
        // the input transform stages whole input rows in shared memory: rows
        // too wide for it are refused before anything is queued
        int in_smem = 0;
        make_in_desc(g, problem->in, problem->in, nullptr, nullptr, &in_smem);
        if (in_smem > 232448)
            return noalloc_fail(CONV2D_ERR_UNSUPPORTED, "input rows too wide for the staged input transform");
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return noalloc_fail(CONV2D_ERR_CUDA, "no CUDA device");
    void* base = nullptr;
    if (scratch_for(device, &base) != cudaSuccess)
        return noalloc_fail(CONV2D_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
    char* b = static_cast<char*>(base);
    DevErr* err = reinterpret_cast<DevErr*>(b);
    void* U = b + bErr;
    void* V = b + bErr + bU;
    void* Mw = b + bErr + bU + bV;

    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    GemmPlan gp;
    if (plan_gemm(gp, OpType::F16, 16, g.P, g.k, g.kp, g.cp, V, U, Mw, MType::F16, default_bn(g.k), sms > 0 ? sms : 1) !=
        cudaSuccess)
        return noalloc_fail(CONV2D_ERR_CUDA, "tensor map encoding failed");
    // the error word starts every call at zero; U, V and M are rewritten in
    // full (padding included) by the kernels below
    if (cudaMemsetAsync(err, 0, sizeof(DevErr), s) != cudaSuccess)
        return noalloc_fail(CONV2D_ERR_CUDA, "cudaMemsetAsync failed");
    const void* x_end = static_cast<const uint16_t*>(problem->in) + static_cast<long long>(g.n) * g.c * g.h * g.w;
    if (launch_filter_transform(Xform::F2, OpType::F16, problem->weight, U, g.k, g.c, g.cp, s) != cudaSuccess ||
        launch_input_transform(Xform::F2, OpType::F16, g, problem->in, x_end, V, nullptr, err, s) != cudaSuccess ||
        launch_gemm(gp, err, s) != cudaSuccess ||
        launch_output_transform(Xform::F2, MType::F16, g, Mw, problem->out, nullptr, err, s) != cudaSuccess)
        return noalloc_fail(CONV2D_ERR_CUDA, "kernel launch failed");
    return CONV2D_OK;
}

extern "C" int conv2d_noalloc_check_device(int* site) {
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return noalloc_fail(CONV2D_ERR_CUDA, "no CUDA device");
    if (site) *site = 0;
    if (device < 0 || device >= kMaxDevices) return noalloc_fail(CONV2D_ERR_CUDA, "device index out of range");
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        base = g_dev_ptr[device];
    }
    if (!base) return CONV2D_OK;   // no call has run on this device
    if (cudaDeviceSynchronize() != cudaSuccess) return noalloc_fail(CONV2D_ERR_CUDA, "device synchronize failed");
    DevErr h{};
    if (cudaMemcpy(&h, base, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
        return noalloc_fail(CONV2D_ERR_CUDA, "error word copy failed");
    if (site) *site = static_cast<int>(h.code);
    if (h.code) {
        if (cudaMemset(base, 0, sizeof(DevErr)) != cudaSuccess)
            return noalloc_fail(CONV2D_ERR_CUDA, "error word reset failed");
        return noalloc_fail(CONV2D_ERR_TIMEOUT, "a kernel of the no-allocation path gave up a bounded wait");
    }
    return CONV2D_OK;
}

extern "C" int conv2d_noalloc_selftest_expire(void* stream) {
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return noalloc_fail(CONV2D_ERR_CUDA, "no CUDA device");
    void* base = nullptr;
    if (scratch_for(device, &base) != cudaSuccess)
        return noalloc_fail(CONV2D_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed");
    noalloc_expire_kernel<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<DevErr*>(base));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CONV2D_OK : noalloc_fail(CONV2D_ERR_CUDA, cudaGetErrorString(e));
}
