"""Seeded synthetic workloads of the benchmark configurations.

* ``grouped_shapes``: 256 independent SGEMMs, M, N, K log-uniform in
  [32, 1024], transposes drawn from {NN, NT, TN} (the batching form).
* ``conv_layers``: the 12-layer im2col convolution stack -- 4 stages of 3
  3x3 convolutions (pad 1), widths 64, 128, 256, 512, spatial 56, 28, 14, 7,
  batch 32; the first layer of stages 1-3 has stride 2 and takes the
  previous stage's width.  Each layer is the GEMM M = Cout, N = 32*Ho*Wo,
  K = Cin*9 of the reference's ocl_convolution (sgemm_ocl1.h:271-300), with
  the batch folded into N.
"""
from __future__ import annotations

import numpy as np

GROUPED_SEED = 20261206


def grouped_shapes(count: int = 256, seed: int = GROUPED_SEED, lo: int = 32, hi: int = 1024):
    rng = np.random.default_rng(seed)
    dims = np.exp(rng.uniform(np.log(lo), np.log(hi), (count, 3))).round().astype(int)
    trans = ["NN", "NT", "TN"]
    picks = rng.integers(0, 3, count)
    return [(trans[t][0], trans[t][1], int(m), int(n), int(k))
            for (m, n, k), t in zip(dims, picks)]


def conv_layers(batch: int = 32):
    """[(cin, cout, h_in, w_in, stride)] for the 12-layer stack."""
    layers = []
    cin, size = 64, 56
    for s in range(4):
        cout = 64 << s
        for i in range(3):
            stride = 2 if (s > 0 and i == 0) else 1
            layers.append((cin, cout, size, size, stride))
            size = (size + 2 - 3) // stride + 1
            cin = cout
    return layers


def conv_gemm_shapes(batch: int = 32):
    """Forward GEMM (M, N, K) of each conv layer."""
    out = []
    for (cin, cout, h, w, stride) in conv_layers(batch):
        ho = (h + 2 - 3) // stride + 1
        wo = (w + 2 - 3) // stride + 1
        out.append((cout, batch * ho * wo, cin * 9))
    return out
