"""Python mirror of the operator's C ABI (include/conv2d.h), over ctypes.

The operator itself is C++/CUDA in ``csrc/`` built into ``_build/libwgconv.so``;
this module only binds that library so tests and the benchmark can call it the
way the reference's harness does (reference ``src/main.cpp:58-105``:
``getParamsize`` -> ``getkernelInfo`` -> ``conv2d_fp16``).  There is no
compute here and no fallback: if the library is missing, loading fails.

Device memory in the helpers comes from PyTorch tensors (plumbing only).
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwgconv.so")

# status codes and algorithms (include/conv2d.h)
OK, ERR_INVALID, ERR_UNSUPPORTED, ERR_NOMEM, ERR_CUDA, ERR_TIMEOUT, ERR_BUSY = range(7)
ALGO_REFERENCE, ALGO_4X3, ALGO_2X3, ALGO_2X3_FUSED, ALGO_AUTO, ALGO_4X3_ROW = -1, 0, 1, 2, 3, 4
ALGO_NAMES = {ALGO_4X3: "F(4x3) non-fused", ALGO_2X3: "F(2x3) non-fused", ALGO_2X3_FUSED: "F(2x3) fused",
              ALGO_4X3_ROW: "row F(4x3) fused"}


class Problem(ctypes.Structure):
    """problem_t (reference include/conv2d.h:8-24)."""
    _fields_ = [("in_", ctypes.c_void_p), ("weight", ctypes.c_void_p), ("out", ctypes.c_void_p)] + [
        (f, ctypes.c_uint) for f in ("n", "c", "h", "w", "k", "r", "s", "u", "v", "p", "q")]


class KernelInfo(ctypes.Structure):
    """kernelInfo_t (reference include/conv2d.h:26-36)."""
    _fields_ = [(f, ctypes.c_uint) for f in ("blockx", "blocky", "blockz", "threadx", "thready", "threadz",
                                              "dynmicLdsSize")] + [("kernelPtr", ctypes.c_void_p)]


class Options(ctypes.Structure):
    """conv2d_options_t."""
    _fields_ = [("algo", ctypes.c_int), ("operand_bf16", ctypes.c_int), ("tile_scaling", ctypes.c_int),
                ("f4_points", ctypes.c_int), ("filter_policy", ctypes.c_int), ("gemm_bn", ctypes.c_int),
                ("l2_chunk_bytes", ctypes.c_longlong), ("io_bf16", ctypes.c_int), ("layout_nhwc", ctypes.c_int),
                ("m_fp32", ctypes.c_int), ("reserved", ctypes.c_int * 1)]


# every symbol include/conv2d.h declares
EXPORTS = [
    "getParamsize", "getkernelInfo", "conv2d_fp16", "wg_getParamsize", "wg_getkernelInfo",
    "conv2d_options_default", "getkernelInfo_ex", "conv2d_fp16_ex", "conv2d_fp16_host", "conv2d_fp16_host_steps",
    "conv2d_refresh_filter", "conv2d_destroy", "conv2d_get_algo", "conv2d_workspace_bytes",
    "conv2d_launches_per_call", "conv2d_check_device", "conv2d_last_error", "conv2d_last_error_message",
    "conv2d_status_string", "conv2d_select_reference", "conv2d_copy_to_host", "conv2d_fp16_timed",
    "conv2d_autotune", "conv2d_autotune_clear", "conv2d_fp16_noalloc", "conv2d_noalloc_check_device",
    "conv2d_noalloc_selftest_expire",
    "conv2d_batch_create", "conv2d_batch_run", "conv2d_batch_run_percall", "conv2d_batch_info",
    "conv2d_batch_launches", "conv2d_batch_check_device", "conv2d_batch_destroy",
    "conv2d_server_config_default", "conv2d_server_create", "conv2d_server_add_layer", "conv2d_server_submit",
    "conv2d_server_poll", "conv2d_server_wait_all", "conv2d_server_replay", "conv2d_server_stats",
    "conv2d_server_destroy",
    "conv2d_plan_save",
    "conv2d_plan_load",
    "conv2d_server_save_layers",
    "conv2d_server_load_layers",
]

_lib = None


class Conv2dError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"status {status}: {msg}")
        self.status = status


def build(verbose: bool = False) -> str:
    import importlib.util
    spec = importlib.util.spec_from_file_location("_wg_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(verbose=verbose)


def lib():
    """The operator library.  Raises if it was not built: there is no fallback."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"operator library not built: {LIB_PATH} (run build.py)")
        L = ctypes.CDLL(LIB_PATH)
        vp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)
        L.getParamsize.argtypes = [ctypes.POINTER(Problem), ip]
        L.getkernelInfo.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(KernelInfo), vp]
        L.getkernelInfo_ex.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(KernelInfo), vp,
                                       ctypes.POINTER(Options)]
        L.conv2d_fp16.argtypes = [vp]
        L.conv2d_fp16.restype = None
        L.conv2d_fp16_ex.argtypes = [vp, vp]
        L.conv2d_fp16_host.argtypes = [vp, vp, vp, vp]
        L.conv2d_fp16_host_steps.argtypes = [vp, ctypes.c_int, ctypes.POINTER(vp), ctypes.POINTER(vp), vp]
        L.conv2d_refresh_filter.argtypes = [vp, vp]
        L.conv2d_destroy.argtypes = [vp]
        L.conv2d_get_algo.argtypes = [vp]
        L.conv2d_workspace_bytes.argtypes = [vp]
        L.conv2d_workspace_bytes.restype = ctypes.c_longlong
        L.conv2d_launches_per_call.argtypes = [vp]
        L.conv2d_check_device.argtypes = [vp, ip]
        L.conv2d_last_error_message.restype = ctypes.c_char_p
        L.conv2d_status_string.restype = ctypes.c_char_p
        L.conv2d_options_default.argtypes = [ctypes.POINTER(Options)]
        L.conv2d_select_reference.argtypes = [ctypes.POINTER(Problem)]
        L.conv2d_copy_to_host.argtypes = [vp, vp, ctypes.c_size_t]
        L.conv2d_fp16_timed.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_float), ctypes.c_int]
        L.conv2d_autotune.argtypes = [ctypes.POINTER(Problem), ctypes.POINTER(Options), ip, ip]
        L.conv2d_autotune_clear.restype = None
        L.conv2d_fp16_noalloc.argtypes = [ctypes.POINTER(Problem), vp]
        L.conv2d_noalloc_check_device.argtypes = [ip]
        L.conv2d_noalloc_selftest_expire.argtypes = [vp]
        L.conv2d_batch_create.argtypes = [ctypes.POINTER(Problem), ctypes.c_int, ctypes.POINTER(Options),
                                          ctypes.POINTER(vp)]
        L.conv2d_batch_run.argtypes = [vp, vp]
        L.conv2d_batch_run_percall.argtypes = [vp, vp]
        L.conv2d_batch_info.argtypes = [vp, ctypes.c_int, ip, ip]
        L.conv2d_batch_launches.argtypes = [vp, ctypes.c_int]
        L.conv2d_batch_check_device.argtypes = [vp, ip]
        L.conv2d_batch_destroy.argtypes = [vp]
        L.conv2d_server_config_default.argtypes = [vp]
        L.conv2d_server_create.argtypes = [vp, ctypes.POINTER(vp)]
        L.conv2d_server_add_layer.argtypes = [vp] + [ctypes.c_uint] * 6 + [vp, ip]
        L.conv2d_server_submit.argtypes = [vp, ctypes.c_int, ctypes.c_uint, vp, vp, ctypes.POINTER(ctypes.c_longlong)]
        L.conv2d_server_poll.argtypes = [vp, ctypes.c_longlong, ctypes.POINTER(ctypes.c_double)]
        L.conv2d_server_wait_all.argtypes = [vp]
        L.conv2d_server_replay.argtypes = [vp, ctypes.c_int, ip, ctypes.POINTER(ctypes.c_uint),
                                           ctypes.POINTER(ctypes.c_double), ctypes.POINTER(vp), ctypes.POINTER(vp),
                                           ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.conv2d_server_stats.argtypes = [vp, vp]
        L.conv2d_server_destroy.argtypes = [vp]
        L.conv2d_plan_save.argtypes = [vp, ctypes.c_char_p]
        L.conv2d_plan_load.argtypes = [vp, ctypes.c_char_p]
        L.conv2d_server_save_layers.argtypes = [vp, ctypes.c_char_p]
        L.conv2d_server_load_layers.argtypes = [vp, ctypes.c_char_p, ip, ip]
        _lib = L
    return _lib


def _check(status):
    if status != OK:
        raise Conv2dError(status, lib().conv2d_last_error_message().decode())
    return status


def default_options(**kw) -> Options:
    o = Options()
    _check(lib().conv2d_options_default(ctypes.byref(o)))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def make_problem(x_ptr, w_ptr, y_ptr, n, c, h, w, k, p=1, q=1, r=3, s=3, u=1, v=1) -> Problem:
    return Problem(x_ptr, w_ptr, y_ptr, n, c, h, w, k, r, s, u, v, p, q)


class Conv2d:
    """One configured convolution: the param blob of getkernelInfo plus its calls."""

    def __init__(self, problem: Problem, options: Options | None = None):
        L = lib()
        self.problem = problem
        size = ctypes.c_int(0)
        _check(L.getParamsize(ctypes.byref(problem), ctypes.byref(size)))
        self.param = (ctypes.c_ubyte * size.value)()
        self.info = KernelInfo()
        if options is None:
            _check(L.getkernelInfo(ctypes.byref(problem), ctypes.byref(self.info), self.param))
        else:
            _check(L.getkernelInfo_ex(ctypes.byref(problem), ctypes.byref(self.info), self.param,
                                      ctypes.byref(options)))
        self._alive = True
        opts = options if options is not None else default_options()
        self.scaling = bool(opts.tile_scaling or opts.io_bf16) and self.algo == ALGO_4X3
        self.nhwc = bool(opts.layout_nhwc)

    @property
    def ptr(self):
        return ctypes.cast(self.param, ctypes.c_void_p)

    def __call__(self, stream: int | None = None):
        _check(lib().conv2d_fp16_ex(self.ptr, ctypes.c_void_p(stream or 0)))

    def host(self, host_in: int, host_out: int, stream: int | None = None):
        _check(lib().conv2d_fp16_host(self.ptr, ctypes.c_void_p(host_in), ctypes.c_void_p(host_out),
                                      ctypes.c_void_p(stream or 0)))

    def host_steps(self, host_ins, host_outs, stream: int | None = None):
        """Consecutive host batches through one pipelined call."""
        n = len(host_ins)
        _check(lib().conv2d_fp16_host_steps(self.ptr, n, (ctypes.c_void_p * n)(*host_ins),
                                            (ctypes.c_void_p * n)(*host_outs), ctypes.c_void_p(stream or 0)))

    def timed(self, stream: int | None = None, max_kernels: int = 64):
        """One call; per-kernel durations in ms (CUDA events on the stream)."""
        buf = (ctypes.c_float * max_kernels)()
        n = lib().conv2d_fp16_timed(self.ptr, ctypes.c_void_p(stream or 0), buf, max_kernels)
        if n < 0:
            _check(-n)
        return list(buf[:n])

    def kernel_names(self):
        """Kernels launched by one call, in launch order."""
        if self.algo == ALGO_2X3_FUSED:
            return ["fused2x3"]
        if self.algo == ALGO_4X3_ROW:
            return ["row4x3"]
        per = (["tile_scale"] if self.scaling else []) + ["input_transform", "gemm_tcgen05", "output_transform"]
        return per * (self.launches_per_call // len(per))

    def save(self, path: str):
        """Write the transformed filter (and what it was made for) to a file."""
        _check(lib().conv2d_plan_save(self.ptr, os.fsencode(path)))

    def load(self, path: str):
        """Use a saved transformed filter instead of transforming the weights."""
        _check(lib().conv2d_plan_load(self.ptr, os.fsencode(path)))

    def refresh_filter(self, stream: int | None = None):
        _check(lib().conv2d_refresh_filter(self.ptr, ctypes.c_void_p(stream or 0)))

    def check_device(self):
        site = ctypes.c_int(0)
        st = lib().conv2d_check_device(self.ptr, ctypes.byref(site))
        return st, site.value

    @property
    def algo(self):
        return lib().conv2d_get_algo(self.ptr)

    @property
    def workspace_bytes(self):
        return lib().conv2d_workspace_bytes(self.ptr)

    @property
    def launches_per_call(self):
        return lib().conv2d_launches_per_call(self.ptr)

    def blob_pointers(self):
        """(U_d, V_d, M_d) device pointers recorded in the param blob."""
        vals = (ctypes.c_void_p * 7).from_buffer(self.param)
        return vals[3], vals[4], vals[5]

    def destroy(self):
        if self._alive:
            _check(lib().conv2d_destroy(self.ptr))
            self._alive = False

    def __del__(self):
        try:
            if self._alive and _lib is not None:
                _lib.conv2d_destroy(self.ptr)
        except Exception:
            pass


def autotune(problem: Problem, options: Options | None = None):
    """(algo, gemm_bn) the autotuner picks for this shape (measures once)."""
    a, b = ctypes.c_int(0), ctypes.c_int(0)
    _check(lib().conv2d_autotune(ctypes.byref(problem), ctypes.byref(options) if options is not None else None,
                                 ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def conv2d_noalloc(problem: Problem, stream: int | None = None):
    """F(2x3) convolution through the entry point that allocates no device
    memory (workspace in the library's fixed scratch array)."""
    _check(lib().conv2d_fp16_noalloc(ctypes.byref(problem), ctypes.c_void_p(stream or 0)))


def noalloc_check_device():
    """(status, site) of the no-allocation path's error word on the current
    device (waits for the device; clears the word)."""
    site = ctypes.c_int(0)
    st = lib().conv2d_noalloc_check_device(ctypes.byref(site))
    return st, site.value


class ServerConfig(ctypes.Structure):
    """conv2d_server_config_t."""
    _fields_ = [("hbm_budget_bytes", ctypes.c_longlong), ("max_batch", ctypes.c_int), ("slots", ctypes.c_int),
                ("algo", ctypes.c_int), ("per_request", ctypes.c_int), ("reserved", ctypes.c_int * 3)]


class ServerStats(ctypes.Structure):
    """conv2d_server_stats_t."""
    _fields_ = [("completed", ctypes.c_longlong), ("batches", ctypes.c_int), ("mean_batch", ctypes.c_double),
                ("max_inflight_batches", ctypes.c_int), ("arena_used_bytes", ctypes.c_longlong),
                ("flops", ctypes.c_double), ("busy_us", ctypes.c_double), ("overlap_us", ctypes.c_double)]


class Server:
    """Continuous-batching request loop over resident layers (C++ scheduler)."""

    def __init__(self, **cfg):
        L = lib()
        c = ServerConfig()
        _check(L.conv2d_server_config_default(ctypes.byref(c)))
        for k, v in cfg.items():
            setattr(c, k, v)
        h = ctypes.c_void_p()
        _check(L.conv2d_server_create(ctypes.byref(c), ctypes.byref(h)))
        self.handle = h

    def add_layer(self, c, k, h, w, weight_ptr, p=1, q=1):
        idx = ctypes.c_int()
        _check(lib().conv2d_server_add_layer(self.handle, c, k, h, w, p, q, ctypes.c_void_p(weight_ptr),
                                             ctypes.byref(idx)))
        return idx.value

    def save_layers(self, path: str):
        _check(lib().conv2d_server_save_layers(self.handle, os.fsencode(path)))

    def load_layers(self, path: str):
        """Register the layers of a saved file; returns their indices."""
        first, count = ctypes.c_int(-1), ctypes.c_int(0)
        _check(lib().conv2d_server_load_layers(self.handle, os.fsencode(path), ctypes.byref(first), ctypes.byref(count)))
        return list(range(first.value, first.value + count.value))

    def submit(self, layer, n, in_ptr, out_ptr):
        rid = ctypes.c_longlong()
        _check(lib().conv2d_server_submit(self.handle, layer, n, ctypes.c_void_p(in_ptr), ctypes.c_void_p(out_ptr),
                                          ctypes.byref(rid)))
        return rid.value

    def wait_all(self):
        _check(lib().conv2d_server_wait_all(self.handle))

    def poll(self, rid):
        lat = ctypes.c_double()
        st = lib().conv2d_server_poll(self.handle, rid, ctypes.byref(lat))
        return st, lat.value

    def replay(self, layers, ns, arrivals_us, in_ptrs, out_ptrs):
        """Submit at the given arrival times; returns (latencies_us, wall_us)."""
        cnt = len(layers)
        lat = (ctypes.c_double * cnt)()
        wall = ctypes.c_double()
        _check(lib().conv2d_server_replay(self.handle, cnt, (ctypes.c_int * cnt)(*layers),
                                          (ctypes.c_uint * cnt)(*ns), (ctypes.c_double * cnt)(*arrivals_us),
                                          (ctypes.c_void_p * cnt)(*in_ptrs), (ctypes.c_void_p * cnt)(*out_ptrs),
                                          lat, ctypes.byref(wall)))
        return list(lat), wall.value

    def stats(self):
        st = ServerStats()
        _check(lib().conv2d_server_stats(self.handle, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def destroy(self):
        if self.handle:
            _check(lib().conv2d_server_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            if self.handle and _lib is not None:
                _lib.conv2d_server_destroy(self.handle)
        except Exception:
            pass


class Batch:
    """Many problems of uneven shape: grouped launches replayed from a CUDA
    graph (run) or one conv2d call each (run_percall)."""

    def __init__(self, problems, options: Options | None = None):
        L = lib()
        arr = (Problem * len(problems))(*problems)
        self._problems = arr
        h = ctypes.c_void_p()
        _check(L.conv2d_batch_create(arr, len(problems), ctypes.byref(options) if options is not None else None,
                                     ctypes.byref(h)))
        self.handle = h
        self.count = len(problems)

    def run(self, stream: int | None = None):
        _check(lib().conv2d_batch_run(self.handle, ctypes.c_void_p(stream or 0)))

    def run_percall(self, stream: int | None = None):
        _check(lib().conv2d_batch_run_percall(self.handle, ctypes.c_void_p(stream or 0)))

    def info(self, i):
        a, b = ctypes.c_int(), ctypes.c_int()
        _check(lib().conv2d_batch_info(self.handle, i, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def launches(self, grouped=True):
        return lib().conv2d_batch_launches(self.handle, 1 if grouped else 0)

    def check_device(self):
        site = ctypes.c_int(0)
        return lib().conv2d_batch_check_device(self.handle, ctypes.byref(site)), site.value

    def destroy(self):
        if self.handle:
            _check(lib().conv2d_batch_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            if self.handle and _lib is not None:
                _lib.conv2d_batch_destroy(self.handle)
        except Exception:
            pass


def copy_to_host(host_ptr: int, dev_ptr: int, nbytes: int):
    _check(lib().conv2d_copy_to_host(ctypes.c_void_p(host_ptr), ctypes.c_void_p(dev_ptr), nbytes))


# ---- torch convenience (tests / benchmark) ------------------------------------

def conv2d_torch(x, w, p=1, q=1, options: Options | None = None, stream=None):
    """Run the operator on CUDA tensors x [N,C,H,W], w [K,C,3,3], both fp16 or
    both bf16 (then with the bf16 end-to-end option); returns (output tensor,
    Conv2d handle)."""
    import torch
    assert x.is_cuda and w.is_cuda and x.dtype == w.dtype and x.dtype in (torch.float16, torch.bfloat16)
    x = x.contiguous()
    w = w.contiguous()
    n, c, h, wd = x.shape
    k = w.shape[0]
    oh, ow = h + 2 * p - 2, wd + 2 * q - 2
    if x.dtype == torch.bfloat16:
        options = options if options is not None else default_options()
        options.io_bf16 = 1
    y = torch.empty((n, k, oh, ow), dtype=x.dtype, device=x.device)
    prob = make_problem(x.data_ptr(), w.data_ptr(), y.data_ptr(), n, c, h, wd, k, p, q)
    op = Conv2d(prob, options)
    op._keep = (x, w, y)
    s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    op(s)
    return y, op
