"""The tcgen05 engine's weight block (host packing, no GPU): the layout the
kernels' shared-memory descriptors assume, restated in numpy from the
documented contract of kpt_surrogate_pack_tc, bit for bit; and the bias
split into a 16-bit head and remainder reproducing the FP32 bias (BF16:
within 2^-15 of its size; FP16: 2^-20, plus half the subnormal spacing for
small biases)."""
from __future__ import annotations

import numpy as np
import pytest


def _to16(x, fp16):
    x = np.asarray(x, dtype=np.float32)
    if fp16:
        return x.astype(np.float16).view(np.uint16)
    bits = x.view(np.uint32).astype(np.uint64)
    return ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)


def _from16(h, fp16):
    h = np.asarray(h, dtype=np.uint16)
    if fp16:
        return h.view(np.float16).astype(np.float32)
    return (h.astype(np.uint32) << 16).view(np.float32)


def _operand(w, n_rows, k_cols, fp16):
    """Canonical K-major, unswizzled operand of an n_rows x k_cols matrix."""
    out = np.zeros(n_rows * k_cols, dtype=np.uint16)
    n, k = np.meshgrid(np.arange(n_rows), np.arange(k_cols), indexing="ij")
    idx = (n // 8) * (k_cols // 8) * 64 + (k // 8) * 64 + (n % 8) * 8 + k % 8
    out[idx.ravel()] = _to16(w, fp16).ravel()
    return out


def _reference_block(params, h, fp16):
    w1 = params[: 5 * h].reshape(h, 5)
    b1 = params[5 * h: 6 * h]
    w2 = params[6 * h: 6 * h + h * h].reshape(h, h)
    b2 = params[6 * h + h * h: 7 * h + h * h]
    w3 = params[7 * h + h * h: 10 * h + h * h].reshape(3, h)
    b3 = params[10 * h + h * h:]

    def split(b):
        hi = _from16(_to16(b, fp16), fp16)
        return hi, (b.astype(np.float32) - hi).astype(np.float32)

    k2 = h + 16
    a1 = np.zeros((h, 16), np.float32)
    a1[:, :5] = w1
    a1[:, 5], a1[:, 6] = split(b1)
    a2 = np.zeros((h, k2), np.float32)
    a2[:, :h] = w2
    a2[:, h], a2[:, h + 1] = split(b2)
    a3 = np.zeros((16, k2), np.float32)
    a3[:3, :h] = w3
    a3[:3, h], a3[:3, h + 1] = split(b3)
    return np.concatenate([_operand(a1, h, 16, fp16), _operand(a2, h, k2, fp16),
                           _operand(a3, 16, k2, fp16)])


@pytest.mark.parametrize("fp16", [False, True])
@pytest.mark.parametrize("hidden", [64, 32])
def test_tc_block_layout_matches_the_contract(kpt, hidden, fp16):
    rng = np.random.default_rng(hidden + fp16)
    count = 5 * hidden + hidden + hidden * hidden + hidden + 3 * hidden + 3
    params = rng.normal(0.0, 0.5, count).astype(np.float32)
    got = kpt.surrogate_pack_tc(params, hidden, fp16)
    want = _reference_block(params, hidden, fp16)
    assert got.size == want.size == 16 * hidden + hidden * (hidden + 16) + 16 * (hidden + 16)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("fp16", [False, True])
def test_bias_head_and_remainder_reproduce_the_bias(kpt, fp16):
    h = 64
    rng = np.random.default_rng(7)
    count = 5 * h + h + h * h + h + 3 * h + 3
    params = rng.normal(0.0, 0.5, count).astype(np.float32)
    block = kpt.surrogate_pack_tc(params, h, fp16)
    b1 = params[5 * h: 6 * h]
    # layer 1 is an h x 16 operand: (n, 5) head, (n, 6) remainder
    n = np.arange(h)
    base = (n // 8) * 2 * 64 + (n % 8) * 8
    head = _from16(block[base + 5], fp16)
    rest = _from16(block[base + 6], fp16)
    err = np.abs(head.astype(np.float64) + rest - b1)
    if fp16:
        # an FP16 remainder of a small bias can fall among the subnormals
        # (spacing 2^-24)
        assert np.all(err <= 2.0 ** -20 * np.abs(b1) + 2.0 ** -25)
    else:
        assert np.all(err <= 2.0 ** -15 * np.abs(b1))


def test_pack_rejects_other_widths(kpt):
    with pytest.raises(kpt.KptError, match="hidden_width"):
        kpt.surrogate_pack_tc(np.zeros(100, np.float32), 48)
