// Plan object behind the opaque param blob of the C ABI.
#pragma once
#include <cstdint>

#include "../../include/conv2d.h"
#include "wg_kernels.h"

namespace wg {

constexpr uint32_t kParamMagic = 0x57474233u;  // "WGB3"

// The param blob the caller allocates with getParamsize's size.  Its leading
// fields mirror the reference's mykernelParamType (include/common.h:146-175)
// so a debugger shows the familiar values; `plan` holds everything else.
struct ParamBlob {
    void* pin;
    void* pweight;
    void* pout;
    void* U_d;
    void* V_d;
    void* M_d;
    void* Y_d;
    unsigned int n, c, h, w, k, r, s, u, v, p, q, Oh, Ow;
    int kernel;  // selected algorithm (enum winograd_select order)
    uint32_t magic;
    void* plan;
};

struct Plan {
    problem_t prob{};
    conv2d_options_t opt{};
    int device = 0;
    int num_sms = 1;
    int algo = 0;
    Xform xf = Xform::F2;
    OpType op = OpType::F16;
    MType mt = MType::F16;  // storage of the GEMM result M
    bool scaling = false;
    Geom g{};
    int chunk_n = 1, n_chunks = 1;
    bool has_tail = false;
    void* ws = nullptr;
    long long ws_bytes = 0;
    void* U = nullptr;
    void* V = nullptr;
    void* Mw = nullptr;
    float* scale = nullptr;
    DevErr* err = nullptr;
    GemmPlan gemm_full{}, gemm_tail{};
    FusedPlan fused{};
    RowPlan row{};
    long long u_bytes = 0;   // bytes of the transformed filter U
    bool nhwc = false;   // channels-last input and output
    NhwcInDesc nh_in{};
    int nh_smem = 0;
    bool filter_ready = false;
    int launches = 0;
    unsigned info_grid = 0, info_threads = 0;
    int info_smem = 0;

    // when set, run() records an event on the stream after every launch
    cudaEvent_t* marks = nullptr;
    int n_marks = 0, max_marks = 0;
    // host-buffer pipeline: image chunks, a GEMM plan per chunk size, copy
    // streams, events
    static constexpr int kMaxHostPlans = 8;
    int host_plan_n[kMaxHostPlans] = {};
    GemmPlan host_gemm[kMaxHostPlans]{};
    int n_host_plans = 0;
    cudaStream_t host_in_stream = nullptr, host_out_stream = nullptr;
    cudaStream_t host_cap_stream = nullptr;   // compute stream of the captured pipeline
    cudaGraphExec_t host_graph = nullptr;     // the pipeline for (graph_in, graph_out)
    const void* graph_in = nullptr;
    void* graph_out = nullptr;
    static constexpr int kMaxHostChunks = 16;
    // per chunk: input copied, computed, output copied; start and end
    cudaEvent_t host_ev[3 * kMaxHostChunks + 2] = {};

    // one kernel per call, no Winograd-domain workspace
    bool single_kernel() const { return algo == CONV2D_ALGO_2X3_FUSED || algo == CONV2D_ALGO_4X3_ROW; }
    // GEMM result row-major (M[E][P][Kp]) for the NHWC output transform of
    // fp16 / fp32 M; 24-bit M keeps the granule layout in both layouts
    bool m_row() const { return nhwc && mt != MType::F24; }

    ~Plan();
    int build(const problem_t* pr, const conv2d_options_t* opt);
    int filter(cudaStream_t s);
    int run(cudaStream_t s);
    // images [n0, n0 + nc) with the given GEMM plan (sized for nc images)
    int run_range(int n0, int nc, const GemmPlan* gp, cudaStream_t s);
    // host input -> device -> host output, copies overlapped with compute
    int run_host(const void* host_in, void* host_out, cudaStream_t s);
    // `steps` host batches one after another, copies of consecutive batches
    // overlapping; waits for the stream at the end
    int run_host_steps(const void* const* host_in, void* const* host_out, int steps, cudaStream_t s);
    // queue the host-buffer pipeline of `steps` batches with cs as the compute stream
    int enqueue_host(const void* const* host_in, void* const* host_out, int steps, cudaStream_t cs);
    int host_setup();
    // GEMM plan for a host chunk of nc images (made once per size), or null
    const GemmPlan* host_gemm_for(int nc);
    void mark(cudaStream_t s);
    void release();
};

// Makes `device` current for the guard's lifetime and then restores the
// device that was current before: an entry point working on a plan of another
// device must not change the calling thread's current device.
class DeviceGuard {
   public:
    explicit DeviceGuard(int device) {
        int cur = -1;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != device && cudaSetDevice(device) == cudaSuccess) prev_ = cur;
    }
    ~DeviceGuard() {
        if (prev_ >= 0) cudaSetDevice(prev_);
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;

   private:
    int prev_ = -1;
};

int validate_problem(const problem_t* pr);
int options_default(conv2d_options_t* o);
int default_bn(int K);
int select_reference64(unsigned long long n, unsigned long long c, unsigned long long h, unsigned long long w,
                       unsigned long long k, unsigned long long r, unsigned long long s, unsigned long long oh,
                       unsigned long long ow);
Plan* plan_of(const void* param);

// Records the status and message conv2d_last_error / _message report.
int set_last_error(int status, const char* msg);

// Per-shape algorithm and GEMM tile choice for CONV2D_ALGO_AUTO
// (autotune.cpp): measured once per shape, cached, optionally persisted.
int autotune_choose(const problem_t& pr, const conv2d_options_t& opt, int fallback, int* algo, int* bn);
void autotune_clear();

}  // namespace wg
