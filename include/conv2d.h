/*
 * GB300 (sm_103a) Winograd 3x3 conv2d operator -- C ABI.
 *
 * Drop-in for the reference operator interface (reference include/conv2d.h:8-42):
 * the same descriptor structs with the same field order and meaning, and the
 * same three entry points called in the same order (src/main.cpp:58-105):
 *
 *     problem_t prob = {in, weight, out, n, c, h, w, k, r, s, u, v, p, q};
 *     int size;  getParamsize(&prob, &size);
 *     void* param = malloc(size);
 *     kernelInfo_t info;  getkernelInfo(&prob, &info, param);
 *     conv2d_fp16(param);            // as often as wanted
 *     conv2d_destroy(param); free(param);   // extension: frees the workspace
 *
 * All tensor pointers are DEVICE pointers to IEEE binary16 data (the
 * reference's _Float16*, ABI-identical to void*).  Input NCHW, weights KCRS,
 * output N K Oh Ow (options: bf16 tensors, channels-last input/output).
 * Supported: r = s = 3, u = v = 1, padding p, q up to 64 with a positive
 * output size, dimensions up to 65535, image rows that fit the staged input
 * transform (about 1,200 columns for F(4x3)).  Unsupported descriptors are
 * rejected with a status code (the reference computes garbage for them).
 *
 * WEIGHTS ARE READ ONCE.  Unlike the reference, which re-reads `weight` on
 * every call, the filter is transformed into the Winograd domain on the first
 * conv2d_fp16 call after getkernelInfo and the transformed copy is reused by
 * every later call.  A caller that changes the weights in place must call
 * conv2d_refresh_filter (or set filter_policy = 1 / WG_CONV2D_FILTER_EVERY_CALL=1
 * to transform on every call, as the reference does); otherwise later calls
 * use the old weights.
 *
 * The reference exports getParamsize/getkernelInfo with C++ linkage; this
 * library exports them both with C linkage (declared here) and with the
 * reference's C++-mangled names, so code compiled against either header links.
 */
#ifndef GB300_WINOGRAD_CONV2D_H
#define GB300_WINOGRAD_CONV2D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* reference include/conv2d.h:8-24 */
typedef struct
{
    void*        in;       /* input  [n][c][h][w]  fp16, device */
    void*        weight;   /* filter [k][c][r][s]  fp16, device */
    void*        out;      /* output [n][k][Oh][Ow] fp16, device */
    unsigned int n;        /* batch */
    unsigned int c;        /* input channels */
    unsigned int h;        /* input height */
    unsigned int w;        /* input width */
    unsigned int k;        /* output channels */
    unsigned int r;        /* filter height (must be 3) */
    unsigned int s;        /* filter width  (must be 3) */
    unsigned int u;        /* stride, height (must be 1) */
    unsigned int v;        /* stride, width  (must be 1) */
    unsigned int p;        /* padding, height */
    unsigned int q;        /* padding, width */
} problem_t;

/* reference include/conv2d.h:26-36.  Filled with the launch shape of the
 * main kernel of the selected algorithm (the reference leaves it unset). */
typedef struct
{
    unsigned int blockx;
    unsigned int blocky;
    unsigned int blockz;
    unsigned int threadx;
    unsigned int thready;
    unsigned int threadz;
    unsigned int dynmicLdsSize;
    void*        kernelPtr;
} kernelInfo_t;

/* Status codes (the reference always returns 0). */
enum {
    CONV2D_OK = 0,
    CONV2D_ERR_INVALID = 1,      /* null pointer, zero size, or param blob not set up */
    CONV2D_ERR_UNSUPPORTED = 2,  /* r,s != 3, u,v != 1, sizes beyond 32-bit tile counts */
    CONV2D_ERR_NOMEM = 3,        /* device workspace allocation failed */
    CONV2D_ERR_CUDA = 4,         /* a CUDA call or kernel launch failed */
    CONV2D_ERR_TIMEOUT = 5,      /* a kernel gave up a bounded wait (device error word set) */
    CONV2D_ERR_BUSY = 6          /* resource limit reached (server admission, queue full) */
};

/* Algorithms; values 0..2 are the reference's enum winograd_select
 * (include/common.h:140-144). */
enum {
    CONV2D_ALGO_REFERENCE = -1,  /* the reference's selection rule (src/conv2d.cpp:83-114) */
    CONV2D_ALGO_4X3_NON_FUSED = 0,
    CONV2D_ALGO_2X3_NON_FUSED = 1,
    CONV2D_ALGO_2X3_FUSED = 2,
    CONV2D_ALGO_AUTO = 3,        /* per-shape autotuner (measures candidates once per shape) */
    CONV2D_ALGO_4X3_ROW = 4      /* row-Winograd F(4x3), one fused kernel: 1-D F(4,3) along the
                                    width, the 3 filter rows summed directly; fp16 NCHW tensors */
};

/* Options for getkernelInfo_ex.  conv2d_options_default() gives the values
 * getkernelInfo uses, after applying the WG_CONV2D_* environment overrides.
 *
 * ALGORITHM CHOICE.  getkernelInfo picks the algorithm with the per-shape
 * autotuner (algo = CONV2D_ALGO_AUTO): the first time a shape is seen it
 * times the candidates (the reference's three algorithms and the row F(4x3)
 * kernel) on the device, reading the problem's input and weights and writing
 * a scratch output, and keeps the reference rule's pick unless another is
 * more than 3% faster; the choice is cached per shape (and in
 * WG_CONV2D_TUNE_FILE).  On GB300 the reference rule's fused F(2x3) pick is
 * several times slower than the alternatives for wide K (e.g. 392 against
 * 115 us on 32x256x56^2 -> 256).  algo = CONV2D_ALGO_REFERENCE, or
 * WG_CONV2D_ALGO=ref, applies the reference rule (src/conv2d.cpp:83-114)
 * exactly; conv2d_get_algo reports what was chosen. */
typedef struct
{
    int algo;            /* CONV2D_ALGO_* */
    int operand_bf16;    /* 0: fp16 Winograd-domain operands, 1: bf16 */
    int tile_scaling;    /* F(4x3): per-tile power-of-two scaling of the input transform */
    int f4_points;       /* F(4x3) interpolation points: 0 = {0,+-1,1/2,-2}, 1 = reference {0,+-1,+-2} */
    int filter_policy;   /* 0: transform the filter on the first call, then reuse; 1: every call */
    int gemm_bn;         /* GEMM output-channel tile: 0 = automatic, else 32/64/128/256 */
    long long l2_chunk_bytes; /* non-fused: process images in chunks whose V+M fit this many bytes (0 = one pass) */
    int io_bf16;         /* 1: input, filter and output tensors are bf16 (end to end); F(2x3) then uses bf16
                            operands, F(4x3) fp16 operands with per-tile scaling, both an fp32 M */
    int layout_nhwc;     /* 1: input and output tensors are NHWC (channels last; filter stays KCRS);
                            non-fused F(2x3)/F(4x3), fp16 tensors, images up to ~250 columns */
    int m_fp32;          /* F(4x3) non-fused: 1 stores the GEMM result M in fp32; 0 (default) in 24 bits
                            (each fp32 accumulator rounded to its upper 24 bits: relative rounding
                            2^-17, 3/4 of the fp32 bytes), for NCHW and NHWC tensors alike */
    int reserved[1];
} conv2d_options_t;

/* reference include/conv2d.h:39-42 */
int getParamsize(problem_t* problem, int* paramSize);
int getkernelInfo(problem_t* problem, kernelInfo_t* kernelInfo, void* param);
void conv2d_fp16(const void* param_ptr);

/* ---- extensions (no counterpart in the reference unless noted) ---------- */

/* Same entry points under distinct names (used by the C++-linkage shims). */
int wg_getParamsize(problem_t* problem, int* paramSize);
int wg_getkernelInfo(problem_t* problem, kernelInfo_t* kernelInfo, void* param);

int conv2d_options_default(conv2d_options_t* opt);

/* getkernelInfo with explicit options (opt may be NULL = defaults). */
int getkernelInfo_ex(problem_t* problem, kernelInfo_t* kernelInfo, void* param, const conv2d_options_t* opt);

/* conv2d_fp16 on a caller stream (cudaStream_t passed as void*; NULL = legacy
 * default stream), returning a status instead of exiting the process. */
int conv2d_fp16_ex(const void* param_ptr, void* stream);

/* End-to-end call with HOST buffers: copies host_in (n*c*h*w fp16) to the
 * problem's device input, runs, copies the output to host_out and waits for
 * the stream.  The batch is cut into up to 8 image chunks (at least 6 MB of
 * copies each; WG_CONV2D_HOST_CHUNKS / WG_CONV2D_HOST_SIZES override) whose
 * input copies, compute and output copies overlap (two internal copy
 * streams); with pinned host memory the copies run at full link speed. */
int conv2d_fp16_host(const void* param_ptr, const void* host_in, void* host_out, void* stream);

/* `steps` end-to-end calls of the same layer on consecutive host batches
 * (host_in[i] -> host_out[i], the same pointers may repeat), queued as one
 * pipeline: chunk j of batch i waits only for chunk j of batch i-1, so the
 * output copies of one batch overlap the input copies of the next and the
 * host link carries both directions at once.  Waits for the stream at the
 * end.  Every batch is copied in and out in full; results are those of
 * `steps` conv2d_fp16_host calls. */
int conv2d_fp16_host_steps(const void* param_ptr, int steps, const void* const* host_in, void* const* host_out,
                           void* stream);

/* Re-run the filter transform (after the caller changed the weights in place). */
int conv2d_refresh_filter(const void* param_ptr, void* stream);

/* Frees the device workspace that getkernelInfo allocated (the reference has no
 * release path: include/common.h:174 never runs).  The blob is unusable after. */
int conv2d_destroy(void* param_ptr);

/* Selected algorithm (CONV2D_ALGO_4X3_NON_FUSED .. CONV2D_ALGO_2X3_FUSED, or
 * CONV2D_ALGO_4X3_ROW), or -1. */
int conv2d_get_algo(const void* param_ptr);

/* Device workspace bytes held by the blob. */
long long conv2d_workspace_bytes(const void* param_ptr);

/* Kernel launches one conv2d_fp16 call makes (with the filter already transformed). */
int conv2d_launches_per_call(const void* param_ptr);

/* Waits for the device, then reports (and clears) the device error word of the
 * blob's kernels: CONV2D_OK or CONV2D_ERR_TIMEOUT; `site` receives the first
 * failing wait site (may be NULL). */
int conv2d_check_device(const void* param_ptr, int* site);

/* Status and message of the last failing call on this thread. */
int conv2d_last_error(void);
const char* conv2d_last_error_message(void);
const char* conv2d_status_string(int status);

/* The reference selection rule evaluated in 64-bit arithmetic (0..2). */
int conv2d_select_reference(const problem_t* problem);

/* Per-shape choice of algorithm and GEMM output-channel tile, as
 * CONV2D_ALGO_AUTO makes it: measured on the device the first time a shape is
 * seen (candidates run on scratch output memory, reading the problem's input
 * and weights), then cached; WG_CONV2D_TUNE_FILE persists the cache.  The
 * reference selection is kept unless another candidate is >3% faster. */
int conv2d_autotune(const problem_t* problem, const conv2d_options_t* opt, int* algo, int* gemm_bn);
void conv2d_autotune_clear(void);

/* ---- batches of uneven problems (no counterpart in the reference) -------- */

/* Many convolutions of different shapes run together: one grouped launch per
 * kernel family covers every problem (the GEMM as one persistent work queue of
 * (problem, element, tile block, channel block) items), captured once into a
 * CUDA graph and replayed.  Each problem's algorithm and GEMM tile follow
 * `opt->algo` (CONV2D_ALGO_AUTO: per-shape autotuner).  Workspaces and
 * transformed filters stay resident until conv2d_batch_destroy. */
typedef struct conv2d_batch conv2d_batch_t;
int conv2d_batch_create(const problem_t* problems, int count, const conv2d_options_t* opt, conv2d_batch_t** batch);
/* Grouped run (the first call also records the graph). */
int conv2d_batch_run(conv2d_batch_t* batch, void* stream);
/* The same problems, one conv2d call after another (for comparison). */
int conv2d_batch_run_percall(conv2d_batch_t* batch, void* stream);
int conv2d_batch_info(const conv2d_batch_t* batch, int index, int* algo, int* gemm_bn);
/* Kernel launches of one grouped (grouped != 0) or per-call run. */
int conv2d_batch_launches(const conv2d_batch_t* batch, int grouped);
int conv2d_batch_check_device(conv2d_batch_t* batch, int* site);
int conv2d_batch_destroy(conv2d_batch_t* batch);

/* ---- serving (no counterpart in the reference) ---------------------------- */

/* A request loop over resident layers: filters transformed once (F(2x3) and
 * F(4x3)) and kept on the device; requests admitted in arrival order while
 * their Winograd-domain workspace fits in an arena of `hbm_budget_bytes`;
 * admitted requests packed into batches of at most `max_batch` and launched
 * as grouped kernels on one of `slots` streams, so batches overlap on the
 * device (continuous batching).  A request's result does not depend on what
 * else is in its batch.  per_request = 1 gives the plain per-call path: each
 * request's own kernels queued at submission on one stream. */
typedef struct conv2d_server conv2d_server_t;
typedef struct
{
    long long hbm_budget_bytes;  /* workspace arena (default 40 GiB) */
    int max_batch;               /* requests per batch (default 16) */
    int slots;                   /* batches in flight (default 6) */
    int algo;                    /* CONV2D_ALGO_AUTO (shape rule), _2X3_NON_FUSED or _4X3_NON_FUSED */
    int per_request;             /* 1: the plain per-call path instead of batching: each request's own
                                    kernels queued on one stream when it is submitted, in arrival
                                    order, no wait for earlier requests (slots and max_batch unused) */
    int reserved[3];
} conv2d_server_config_t;
typedef struct
{
    long long completed;
    int batches;
    double mean_batch;
    int max_inflight_batches;
    long long arena_used_bytes;
    double flops;                /* direct-convolution FLOPs of completed requests */
    double busy_us;              /* device time with at least one batch between its start and end events */
    double overlap_us;           /* device time with two or more batches in flight at once */
} conv2d_server_stats_t;
int conv2d_server_config_default(conv2d_server_config_t* cfg);
int conv2d_server_create(const conv2d_server_config_t* cfg, conv2d_server_t** server);
/* Registers a layer (3x3, stride 1, padding p,q, input h x w, c -> k channels)
 * whose fp16 KCRS weights are on the device; returns its index. */
int conv2d_server_add_layer(conv2d_server_t* server, unsigned c, unsigned k, unsigned h, unsigned w, unsigned p,
                            unsigned q, const void* weight, int* layer);
/* Queues a request of n images (device input/output); returns its id.
 * CONV2D_ERR_BUSY when its workspace alone exceeds the budget. */
int conv2d_server_submit(conv2d_server_t* server, int layer, unsigned n, const void* in, void* out,
                         long long* request);
/* 1 when done (latency in microseconds, arrival to completion), 0 pending, -1 unknown. */
int conv2d_server_poll(conv2d_server_t* server, long long request, double* latency_us);
int conv2d_server_wait_all(conv2d_server_t* server);
/* Submits `count` requests at their arrival times (microseconds from the call),
 * waits for all, returns each latency and the wall time. */
int conv2d_server_replay(conv2d_server_t* server, int count, const int* layer, const unsigned* n,
                         const double* arrival_us, const void* const* in, void* const* out, double* latency_us,
                         double* wall_us);
int conv2d_server_stats(conv2d_server_t* server, conv2d_server_stats_t* stats);
int conv2d_server_destroy(conv2d_server_t* server);

/* ---- Persistence (no counterpart in the reference, which transforms the
 * filter on every call) ----------------------------------------------------
 * A plan's Winograd-domain filter U, with the layer (C, K, padding),
 * transform and operand type it was made for and a checksum, written to a
 * file; loading it into a plan of the same layer skips the filter transform
 * (a restarted process pairs this with WG_CONV2D_TUNE_FILE for the autotuner's
 * choices).  Load fails with CONV2D_ERR_INVALID when the file was made for
 * another layer, transform or operand type, or is damaged. */
int conv2d_plan_save(const void* param, const char* path);
int conv2d_plan_load(const void* param, const char* path);
/* A server's resident layers (both transformed filters of each) to a file,
 * and back into a server: the loaded layers get indices first_layer ..
 * first_layer + count - 1, in the saved order. */
int conv2d_server_save_layers(conv2d_server_t* server, const char* path);
int conv2d_server_load_layers(conv2d_server_t* server, const char* path, int* first_layer, int* count);

/* One call with a CUDA event recorded on the stream after every kernel
 * launch; waits, writes each launch's duration (ms, launch order) to
 * kernel_ms and returns the number of launches (negative status on error). */
int conv2d_fp16_timed(const void* param_ptr, void* stream, float* kernel_ms, int max_kernels);

/* No counterpart in the reference.  The F(2x3) non-fused convolution of
 * `problem` on `stream`, for callers that must not allocate device memory
 * while they run (a host that hands all device memory to its own pool at
 * start-up, or a latency-bound loop that cannot afford the device-wide
 * synchronisation of cudaMalloc/cudaFree).  It needs no param blob and calls
 * no allocator: its Winograd-domain workspace lives in a 32 MiB array inside
 * this library that every GPU loading the library holds until the process
 * exits.  Problems whose workspace (16*Kp*Cp + 16*P8*Cp + 16*P*Kp halves, P
 * tiles rounded up to 8 for P8) exceeds it return CONV2D_ERR_UNSUPPORTED.
 * The first call on a device looks the array up (make it before any stream
 * capture); all calls on a device share the array, so calls that overlap on
 * the GPU race and the caller must order them.  Input rows too wide for the
 * staged input transform also return CONV2D_ERR_UNSUPPORTED, before anything
 * is queued.  A kernel that gives up a bounded wait leaves a garbage output
 * and records the failure in an error word inside the array (each call
 * clears it first): read it with conv2d_noalloc_check_device. */
int conv2d_fp16_noalloc(const problem_t* problem, void* stream);

/* No counterpart in the reference.  Waits for the current device, then
 * reports (and clears) the error word of conv2d_fp16_noalloc on that device:
 * CONV2D_OK, or CONV2D_ERR_TIMEOUT when one of its kernels gave up a bounded
 * wait since the last call; `site` (may be NULL) receives the first failing
 * wait site.  Allocates nothing. */
int conv2d_noalloc_check_device(int* site);

/* No counterpart in the reference; a test hook of the error path above.
 * Queues on `stream` one thread that waits on a barrier nothing completes:
 * after the wait limit (0.5 s) it gives up and records a timeout in the
 * no-allocation error word, as a kernel of conv2d_fp16_noalloc would.  The
 * device stays usable. */
int conv2d_noalloc_selftest_expire(void* stream);

/* Copies `bytes` from device memory to host memory and waits (used by tests
 * to read the Winograd-domain workspaces U_d/V_d/M_d of the param blob). */
int conv2d_copy_to_host(void* host_dst, const void* device_src, size_t bytes);

#ifdef __cplusplus
}
#endif

#endif /* GB300_WINOGRAD_CONV2D_H */
