"""The inference image of the neural shader (sglc_nn.cuh: first-layer columns in the deferred kernel's
two-half order, biases folded into the MMAs as BF16 high and low parts beside ones columns) computes
the same network as the canonical parameters the oracle uses.

The column map `inferColumn` is compiled from the header itself (a host program built by nvcc; no
GPU needed); the network with the permuted, folded weights is then evaluated in numpy exactly as the
kernel does (ones in the bias columns, ReLU and BF16 rounding of the hidden layers) and compared
with oracle/nn_oracle.py's forward pass."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import nn_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "softglrender_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include "sglc_nn.cuh"
int main() {
  for (int f = 0; f < sglc::nn::kFeat; f++) printf("%d\n", sglc::nn::inferColumn(f));
  printf("%d %d %d %d %d\n", sglc::nn::kIW1, sglc::nn::kIW2, sglc::nn::kIW3, sglc::nn::kInferBytes,
         sglc::nn::kInferOffset);
  return 0;
}
"""


@pytest.fixture(scope="module")
def columns(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    d = tmp_path_factory.mktemp("nnlayout")
    src, exe = d / "layout.cu", d / "layout"
    src.write_text(PROGRAM)
    subprocess.run([nvcc, "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    cols = [int(x) for x in out[:O.N_FEAT]]
    sizes = [int(x) for x in out[O.N_FEAT].split()]
    return cols, sizes


def test_columns_are_a_permutation_around_the_bias_columns(columns):
    cols, (iw1, iw2, iw3, total, offset) = columns
    assert len(set(cols)) == O.N_FEAT and min(cols) >= 0 and max(cols) < 160
    assert not set(cols) & {78, 79, 158, 159}          # pads and the bias pair
    # half H holds inputs 6H..6H+5: feature 24k + 2i (+1) and 144 + i map into half i // 6
    for f, c in enumerate(cols):
        i = (f % 24) // 2 if f < 144 else f - 144
        assert c // 80 == i // 6, (f, c)
    assert (iw1, iw2, iw3, total) == (0, 64 * 160 * 2, 64 * 160 * 2 + 64 * 80 * 2, 64 * 160 * 2 + 64 * 80 * 2 + 16 * 80 * 2)
    assert offset % 16 == 0


def test_folded_network_equals_the_canonical_one(columns):
    cols, _ = columns
    rng = np.random.default_rng(7)
    p = O.unflatten(rng.normal(0, 0.3, O.N_PARAMS).astype(np.float32))
    x = rng.uniform(-1, 1, (256, O.N_IN)).astype(np.float32)
    y, _ = O.forward(p, x)
    bf = O.bf16

    def split(b):
        hi = bf(b)
        return hi, bf(b - hi)

    W1 = np.zeros((64, 160), np.float32)
    W1[:, cols] = bf(p["W1"])
    W1[:, 158], W1[:, 159] = split(p["b1"])
    W2 = np.zeros((64, 80), np.float32)
    W2[:, :64] = bf(p["W2"])
    W2[:, 64], W2[:, 65] = split(p["b2"])
    W3 = np.zeros((16, 80), np.float32)
    W3[:3, :64] = bf(p["W3"])
    W3[:3, 64], W3[:3, 65] = split(p["b3"])
    X = np.zeros((256, 160), np.float32)
    X[:, cols] = bf(O.encode(x))
    X[:, 158] = X[:, 159] = 1.0
    mm = lambda a, b: (a.astype(np.float64) @ b.astype(np.float64).T).astype(np.float32)
    H1 = np.zeros((256, 80), np.float32)
    H1[:, :64] = bf(np.maximum(mm(X, W1), 0))
    H1[:, 64:66] = 1.0
    H2 = np.zeros((256, 80), np.float32)
    H2[:, :64] = bf(np.maximum(mm(H1, W2), 0))
    H2[:, 64:66] = 1.0
    yi = mm(H2, W3)[:, :3]
    # the bias pair carries 16 significant bits against FP32: the differences come from hidden
    # activations whose BF16 rounding the bias's last bits move (about 5e-4 of the output range here)
    np.testing.assert_allclose(yi, y, rtol=0, atol=1e-3 * float(np.abs(y).max()))
