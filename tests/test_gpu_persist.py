"""Plan and server persistence: a transformed filter saved from one plan and
loaded into a fresh plan of the same layer gives the same output bit for bit
while the fresh plan's own weight buffer holds garbage (so the filter came
from the file); files made for another layer, transform or operand type, or
damaged ones, are refused."""
import os

import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _plan(wg, x, w_dev, y, algo, bf16=0):
    n, c, h, ww = x.shape
    k = w_dev.shape[0]
    prob = wg.make_problem(x.data_ptr(), w_dev.data_ptr(), y.data_ptr(), n, c, h, ww, k)
    return wg.Conv2d(prob, wg.default_options(algo=algo, operand_bf16=bf16))


@pytest.mark.parametrize("algo", [0, 1, 2, 4])
def test_saved_filter_reproduces_the_output(wg, tmp_path, algo):
    n, c, h, w, k = 2, 40, 18, 18, 56
    xh, wh = O.uniform_inputs(91, n, c, h, w, k)
    x = torch.from_numpy(xh).cuda()
    wt = torch.from_numpy(wh).cuda()
    y1 = torch.empty((n, k, h, w), dtype=torch.float16, device="cuda")
    y2 = torch.full((n, k, h, w), float("nan"), dtype=torch.float16, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    a = _plan(wg, x, wt, y1, algo)
    a(s)
    path = str(tmp_path / "layer.wgplan")
    a.save(path)
    garbage = torch.full_like(wt, 7.0)  # the fresh plan's weights are not the layer's
    b = _plan(wg, x, garbage, y2, algo)
    b.load(path)
    b(s)
    torch.cuda.synchronize()
    assert np.array_equal(y1.cpu().numpy().view(np.uint16), y2.cpu().numpy().view(np.uint16))
    a.destroy()
    b.destroy()


def test_mismatched_or_damaged_files_are_refused(wg, tmp_path):
    n, c, h, w, k = 1, 24, 12, 12, 32
    xh, wh = O.uniform_inputs(5, n, c, h, w, k)
    x = torch.from_numpy(xh).cuda()
    wt = torch.from_numpy(wh).cuda()
    y = torch.empty((n, k, h, w), dtype=torch.float16, device="cuda")
    a = _plan(wg, x, wt, y, 1)
    path = str(tmp_path / "f2.wgplan")
    a.save(path)
    other_t = _plan(wg, x, wt, y, 0)           # F(4x3): another transform
    with pytest.raises(wg.Conv2dError):
        other_t.load(path)
    other_op = _plan(wg, x, wt, y, 1, bf16=1)  # bf16 operands
    with pytest.raises(wg.Conv2dError):
        other_op.load(path)
    w2 = torch.from_numpy(O.uniform_inputs(6, n, c, h, w, k + 8)[1]).cuda()
    y2 = torch.empty((n, k + 8, h, w), dtype=torch.float16, device="cuda")
    other_k = _plan(wg, x, w2, y2, 1)          # another layer
    with pytest.raises(wg.Conv2dError):
        other_k.load(path)
    raw = bytearray(open(path, "rb").read())
    raw[-1] ^= 0x55                            # damaged payload
    bad = str(tmp_path / "bad.wgplan")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(wg.Conv2dError):
        a.load(bad)
    a.load(path)                               # the intact file still loads
    for p in (a, other_t, other_op, other_k):
        p.destroy()


def test_server_layers_survive_a_restart(wg, tmp_path):
    layers = [(64, 96, 14, 14), (32, 48, 9, 11)]
    rng = np.random.default_rng(12)
    srv = wg.Server(slots=2, max_batch=4, hbm_budget_bytes=1 << 30)
    keep = []
    for c, k, h, w in layers:
        wt = torch.from_numpy((rng.standard_normal((k, c, 3, 3)) / np.sqrt(9 * c)).astype(np.float16)).cuda()
        srv.add_layer(c, k, h, w, wt.data_ptr())
        keep.append(wt)
    path = str(tmp_path / "layers.wgsrv")
    srv.save_layers(path)

    def run(server, idx):
        outs = []
        for li, (c, k, h, w) in zip(idx, layers):
            x = torch.from_numpy(rng.uniform(-1, 1, (3, c, h, w)).astype(np.float16)).cuda()
            y = torch.full((3, k, h, w), float("nan"), dtype=torch.float16, device="cuda")
            torch.cuda.synchronize()
            server.submit(li, 3, x.data_ptr(), y.data_ptr())
            outs.append((x, y))
        server.wait_all()
        return [y.cpu().numpy() for _, y in outs]

    state = rng.bit_generator.state
    before = run(srv, [0, 1])
    srv.destroy()
    fresh = wg.Server(slots=2, max_batch=4, hbm_budget_bytes=1 << 30)  # no weights registered
    idx = fresh.load_layers(path)
    assert idx == [0, 1]
    rng.bit_generator.state = state   # the same request inputs
    after = run(fresh, idx)
    fresh.destroy()
    for a, b in zip(before, after):
        assert np.array_equal(a.view(np.uint16), b.view(np.uint16))
