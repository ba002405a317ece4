"""CPU tests of the C ABI: the library loads, exports every declared symbol,
links against code written for the reference header, rejects unsupported
descriptors, and selects algorithms as the reference does.  No GPU needed:
nothing here launches a kernel."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "conv2d.h")
# the reference tree is read only where it is present (its header, to compile
# a caller written for it); WG_REFERENCE_TREE points elsewhere
REF_HEADER_DIR = os.path.join(os.environ.get("WG_REFERENCE_TREE", "/root/reference"), "include")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M)
    return sorted(set(names))


def test_missing_library_fails_loudly(tmp_path):
    """Without the built library the operator refuses to run: there is no
    fallback path to compute on."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "wgconv_unbuilt", os.path.join(ROOT, "dcu-winograd-conv2d_gb300", "__init__.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.LIB_PATH = str(tmp_path / "libwgconv.so")
    with pytest.raises(RuntimeError, match="not built"):
        mod.lib()
    with pytest.raises(RuntimeError, match="not built"):
        mod.Conv2d(mod.make_problem(16, 16, 16, 1, 8, 8, 8, 8))


def test_header_declares_what_the_binding_expects(wg):
    assert set(declared_functions()) == set(wg.EXPORTS)


def test_library_exports_every_declared_symbol(wg):
    out = subprocess.run(["nm", "-D", "--defined-only", wg.LIB_PATH], capture_output=True, text=True).stdout
    syms = {line.split()[-1] for line in out.splitlines() if line.strip()}
    for name in declared_functions():
        assert name in syms, name
    # the reference header's C++-linkage names (include/conv2d.h:39-40)
    assert "_Z12getParamsizeP9problem_tPi" in syms
    assert "_Z13getkernelInfoP9problem_tP12kernelInfo_tPv" in syms


def test_struct_layouts_match_reference(wg):
    # problem_t: three pointers then eleven unsigned ints
    assert ctypes.sizeof(wg.Problem) == 3 * 8 + 11 * 4 + 4  # padded to 8
    assert wg.Problem.n.offset == 24 and wg.Problem.q.offset == 24 + 10 * 4
    assert wg.KernelInfo.kernelPtr.offset == 32


def test_param_size(wg):
    size = ctypes.c_int(0)
    assert wg.lib().getParamsize(None, ctypes.byref(size)) == wg.OK
    assert size.value >= 7 * 8 + 13 * 4


@pytest.mark.parametrize("field,value,status", [
    ("r", 5, 2), ("s", 1, 2), ("u", 2, 2), ("v", 2, 2), ("n", 0, 1), ("k", 0, 1), ("h", 1, 1),
    ("c", 0, 1), ("h", 0, 1), ("w", 0, 1), ("w", 1, 1), ("p", 65, 2), ("q", 65, 2),
    ("c", 65536, 2), ("k", 65536, 2), ("h", 65536, 2), ("w", 65536, 2), ("n", 1 << 28, 2),
])
def test_unsupported_descriptors_rejected(wg, field, value, status):
    prob = wg.make_problem(16, 16, 16, 2, 8, 8, 8, 8)
    setattr(prob, field, value)
    if (field, value) in (("h", 1), ("w", 1)):
        prob.p = prob.q = 0  # a 1-pixel image without padding has no 3x3 output
    with pytest.raises(wg.Conv2dError) as ei:
        wg.Conv2d(prob)
    assert ei.value.status == status


def test_null_pointers_rejected(wg):
    prob = wg.make_problem(0, 16, 16, 1, 8, 8, 8, 8)
    with pytest.raises(wg.Conv2dError) as ei:
        wg.Conv2d(prob)
    assert ei.value.status == wg.ERR_INVALID
    # a blob that getkernelInfo never filled
    blob = (ctypes.c_ubyte * 256)()
    assert wg.lib().conv2d_fp16_ex(ctypes.cast(blob, ctypes.c_void_p), None) == wg.ERR_INVALID


def test_noalloc_refuses_before_any_cuda_call(wg):
    """The no-allocation entry point checks its scratch size and the staged
    input rows on the host, before it touches the device."""
    too_big = wg.make_problem(256, 256, 256, 64, 256, 56, 56, 256)
    assert wg.lib().conv2d_fp16_noalloc(ctypes.byref(too_big), None) == wg.ERR_UNSUPPORTED
    assert b"32 MiB" in wg.lib().conv2d_last_error_message()
    too_wide = wg.make_problem(256, 256, 256, 1, 8, 3, 4000, 8)
    assert wg.lib().conv2d_fp16_noalloc(ctypes.byref(too_wide), None) == wg.ERR_UNSUPPORTED
    assert b"too wide" in wg.lib().conv2d_last_error_message()


SHAPES = [
    (1, 64, 56, 56, 64), (32, 256, 56, 56, 256), (32, 512, 28, 28, 512), (16, 128, 64, 64, 27),
    (16, 256, 32, 32, 256), (16, 64, 128, 128, 64), (2, 1920, 32, 32, 640), (2, 640, 64, 64, 640),
    (2, 320, 64, 64, 4), (64, 256, 14, 14, 256), (256, 192, 14, 14, 192), (16, 256, 26, 26, 512),
    (32, 256, 14, 14, 256), (2, 1280, 16, 16, 1280), (2, 960, 64, 64, 32),
]


def test_selection_matches_reference_rule(wg):
    rng = np.random.default_rng(0)
    shapes = list(SHAPES)
    for _ in range(300):
        shapes.append(tuple(int(v) for v in (rng.integers(1, 9), rng.choice([3, 16, 64, 256, 1024]),
                                              rng.integers(3, 80), rng.integers(3, 80),
                                              rng.choice([4, 27, 64, 256, 2048]))))
    for n, c, h, w, k in shapes:
        prob = wg.make_problem(16, 16, 16, n, c, h, w, k)
        assert wg.lib().conv2d_select_reference(ctypes.byref(prob)) == O.select_reference(n, c, h, w, k), (n, c, h, w, k)


REF_CALLER = r"""
#include <stdio.h>
#include "conv2d.h"
int main() {
    problem_t p; p.in = (_Float16*)16; p.weight = (_Float16*)16; p.out = (_Float16*)16;
    p.n = 1; p.c = 8; p.h = 8; p.w = 8; p.k = 8; p.r = 5; p.s = 5; p.u = 1; p.v = 1; p.p = 1; p.q = 1;
    int size = 0; getParamsize(&p, &size);
    char buf[4096]; kernelInfo_t info;
    int rc = getkernelInfo(&p, &info, buf);   /* 5x5 is rejected before any CUDA call */
    printf("%d %d\n", size > 0, rc);
    if (0) conv2d_fp16(buf);
    return 0;
}
"""


def test_code_written_for_reference_header_links(wg, tmp_path):
    if not os.path.exists(os.path.join(REF_HEADER_DIR, "conv2d.h")):
        pytest.skip("reference header not present on this machine")
    src = tmp_path / "caller.cpp"
    src.write_text(REF_CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(wg.LIB_PATH)
    r = subprocess.run(["g++", "-o", str(exe), str(src), "-I", REF_HEADER_DIR, "-L", libdir, "-lwgconv",
                        f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.split() == ["1", "2"], r.stdout + r.stderr


def test_default_selection_is_the_autotuner_and_ref_is_strict(wg, monkeypatch):
    """getkernelInfo's default options pick the algorithm per shape with the
    autotuner; WG_CONV2D_ALGO=ref gives the reference's own rule."""
    monkeypatch.delenv("WG_CONV2D_ALGO", raising=False)
    assert wg.default_options().algo == wg.ALGO_AUTO
    monkeypatch.setenv("WG_CONV2D_ALGO", "ref")
    assert wg.default_options().algo == wg.ALGO_REFERENCE
    monkeypatch.setenv("WG_CONV2D_ALGO", "4x3")
    assert wg.default_options().algo == wg.ALGO_4X3
    # 24-bit M is the F(4x3) default; WG_CONV2D_M_FP32=1 asks for fp32
    monkeypatch.delenv("WG_CONV2D_M_FP32", raising=False)
    assert wg.default_options().m_fp32 == 0
    monkeypatch.setenv("WG_CONV2D_M_FP32", "1")
    assert wg.default_options().m_fp32 == 1
