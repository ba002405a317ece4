"""Generate the golden vectors in tests/golden/conv_golden.npz.

Every output in the file is produced by the reference project's own CPU
verifier ``conv2dcpu`` (reference ``include/verfiy.h:5-44``), compiled from
the reference sources by ``oracle/Makefile`` into ``oracle/_ref``.  Inputs are
either the reference benchmark's own fill (glibc ``rand()``, default seed,
``(rand()%255)/255.0``, input then weights: ``src/main.cpp:36-44``), made by
the reference build's own ``rand()``, or seeded numpy ``U[-1,1]`` data.

The inputs are not stored: both generators are deterministic and are
re-created by the oracle at test time; their SHA-256 is stored so a drift in
either generator is caught.  Run from the repository root:

    make -C oracle REF=<reference tree> && python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

# (name, kind, seed, n, c, h, w, k, p, q)
CASES = [
    ("refstyle_tiny", "refstyle", 0, 1, 4, 8, 8, 4, 1, 1),
    ("refstyle_ragged", "refstyle", 0, 2, 3, 7, 9, 5, 1, 1),
    ("refstyle_k27", "refstyle", 0, 1, 16, 14, 14, 27, 1, 1),
    ("refstyle_pad0", "refstyle", 0, 1, 8, 10, 12, 8, 0, 0),
    ("refstyle_pad2", "refstyle", 0, 1, 8, 9, 9, 6, 2, 2),
    ("refstyle_cfg1", "refstyle", 0, 1, 64, 56, 56, 64, 1, 1),
    ("uniform_small", "uniform", 11, 2, 8, 12, 12, 16, 1, 1),
    ("uniform_odd", "uniform", 12, 3, 5, 13, 7, 9, 1, 1),
    ("uniform_w28", "uniform", 13, 2, 32, 28, 28, 32, 1, 1),
    ("uniform_k4", "uniform", 14, 1, 24, 16, 16, 4, 1, 1),
]


def make_inputs(kind, seed, n, c, h, w, k, use_ref=False):
    if kind == "refstyle":
        if use_ref:
            return O.ref_reference_style_inputs(n, c, h, w, k)
        return O.reference_style_inputs(n, c, h, w, k)
    return O.uniform_inputs(seed, n, c, h, w, k)


def digest(x, wt):
    hsh = hashlib.sha256()
    hsh.update(np.ascontiguousarray(x).view(np.uint16).tobytes())
    hsh.update(np.ascontiguousarray(wt).view(np.uint16).tobytes())
    return hsh.hexdigest()


def main():
    if O.ref_lib() is None:
        raise SystemExit("oracle/_ref not built: make -C oracle REF=<reference tree>")
    out = {}
    for name, kind, seed, n, c, h, w, k, p, q in CASES:
        x, wt = make_inputs(kind, seed, n, c, h, w, k, use_ref=True)
        y = O.ref_conv2dcpu(x, wt, p=p, q=q)
        out[name + "__meta"] = np.array([seed, n, c, h, w, k, p, q], dtype=np.int64)
        out[name + "__kind"] = np.array(kind)
        out[name + "__digest"] = np.array(digest(x, wt))
        out[name + "__out"] = y.view(np.uint16)
        print(name, y.shape)
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "conv_golden.npz"), **out)


if __name__ == "__main__":
    main()
