"""The 8-wide node quantization (csrc/bvh8.cu, quantize_node8) run on the
host through its test hook: every decoded child box o + q * 2^e must contain
the original fp32 box, whatever the coordinates' magnitude, the boxes'
extents or the number of children. The GPU upload runs the same function
(k_quantize8); the traversal's pruning is conservative exactly when this
containment holds, which the GPU parity tests then show as unchanged hits."""
import ctypes

import numpy as np
import pytest


def quantize(rt, boxes, refs=None, fmask=None):
    """Quantizes n child boxes into slots 0..n-1 (or into the slots of
    `fmask`, in increasing order)."""
    boxes = np.ascontiguousarray(boxes, np.float32).reshape(-1, 6)
    n = len(boxes)
    if fmask is None:
        fmask = (1 << n) - 1
    slots = [s for s in range(8) if (fmask >> s) & 1]
    assert len(slots) == n
    b8 = np.zeros((8, 6), np.float32)
    r8 = np.full(8, np.iinfo(np.int32).min, np.int32)
    b8[slots] = boxes
    r8[slots] = np.arange(n) if refs is None else refs
    out = np.zeros(24, np.uint32)
    ok = rt.LIB.rtgbQuantizeNode8(b8.ctypes.data, r8.ctypes.data, fmask, out.ctypes.data)
    return ok, out


def decode(words, slots):
    """The given slots' child boxes as float64 (len(slots), 6), as the
    traversal reads them; also the exponents and the filled mask."""
    origin = words[0:3].view(np.float32).astype(np.float64)
    exps = [int(np.int8(np.uint8((int(words[3]) >> (8 * k)) & 0xFF))) for k in range(3)]
    mask = int(words[3]) >> 24
    q = np.zeros((len(slots), 6), np.int64)
    for i, s in enumerate(slots):
        for k in range(3):
            q[i, k] = (int(words[4 + 2 * k + (s >> 2)]) >> (8 * (s & 3))) & 0xFF
            q[i, 3 + k] = (int(words[10 + 2 * k + (s >> 2)]) >> (8 * (s & 3))) & 0xFF
    scale = np.array([2.0 ** e for e in exps])
    lo = origin + q[:, :3] * scale
    hi = origin + q[:, 3:] * scale
    return np.concatenate([lo, hi], axis=1), exps, mask


def random_boxes(rng, n, center, extent, size):
    c = center + rng.uniform(-extent, extent, size=(n, 3))
    h = rng.uniform(0.0, size, size=(n, 3))
    return np.concatenate([c - h, c + h], axis=1).astype(np.float32)


@pytest.mark.parametrize("center,extent,size", [
    (0.0, 1.0, 0.3), (0.0, 1e-3, 1e-4), (1000.0, 5.0, 0.5), (-3e4, 100.0, 10.0), (1e6, 1.0, 0.01),
    (0.5, 1e-5, 0.0), (0.0, 4.0, 4.0)])
@pytest.mark.parametrize("n", [1, 2, 5, 8])
def test_decoded_boxes_contain_originals(rt, center, extent, size, n):
    rng = np.random.default_rng(n * 7919 + int(abs(center)) % 1000)
    for _ in range(200):
        boxes = random_boxes(rng, n, center, extent, size)
        ok, words = quantize(rt, boxes)
        assert ok == 1
        dec, exps, mask = decode(words, list(range(n)))
        assert mask == (1 << n) - 1
        assert all(-126 <= e <= 127 for e in exps)
        b = boxes.astype(np.float64)
        assert (dec[:, :3] <= b[:, :3]).all() and (dec[:, 3:] >= b[:, 3:]).all()
        # Loose by at most one grid step per side on top of the node's own
        # union box (the grid covers the union with 255 steps).
        step = np.array([2.0 ** e for e in exps])
        assert (b[:, :3] - dec[:, :3] <= step + 1e-300).all() and (dec[:, 3:] - b[:, 3:] <= step + 1e-300).all()
        assert np.array_equal(words[16:16 + n].view(np.int32), np.arange(n))
        if n < 8:
            assert (words[16 + n:].view(np.int32) == -1).all()


def test_identical_and_flat_children(rt):
    """Eight copies of one box, and boxes flat on one axis (zero extent)."""
    box = np.array([0.25, -1.0, 3.0, 0.75, -0.5, 3.0], np.float32)
    ok, words = quantize(rt, np.tile(box, (8, 1)))
    assert ok == 1
    dec, _, _ = decode(words, list(range(8)))
    assert (dec[:, :3] <= box[:3]).all() and (dec[:, 3:] >= box[3:]).all()


def test_padded_reference_leaves(rt):
    """Boxes as Bvh.h pads them (triangle box +- 1e-4) around a mesh patch."""
    tris_lo = np.array([[0.1, 0.2, 0.3], [0.1001, 0.2, 0.31], [0.12, 0.19, 0.3]], np.float32)
    boxes = np.concatenate([tris_lo - np.float32(1e-4), tris_lo + np.float32(0.01) + np.float32(1e-4)], axis=1)
    ok, words = quantize(rt, boxes)
    assert ok == 1
    dec, _, _ = decode(words, [0, 1, 2])
    b = boxes.astype(np.float64)
    assert (dec[:, :3] <= b[:, :3]).all() and (dec[:, 3:] >= b[:, 3:]).all()


def test_sparse_masks_and_empty_slots(rt):
    """Children in any subset of the slots (the fold places them by octant):
    filled slots decode to boxes containing the originals, empty slots hold
    an inverted box (qlo = 255, qhi = 0) and ref ~0 (a leaf of triangle 0,
    harmless to test)."""
    rng = np.random.default_rng(5)
    for _ in range(300):
        fmask = int(rng.integers(1, 256))
        slots = [s for s in range(8) if (fmask >> s) & 1]
        boxes = random_boxes(rng, len(slots), 0.3, 2.0, 0.4)
        ok, words = quantize(rt, boxes, fmask=fmask)
        assert ok == 1
        dec, _, mask = decode(words, slots)
        assert mask == fmask
        b = boxes.astype(np.float64)
        assert (dec[:, :3] <= b[:, :3]).all() and (dec[:, 3:] >= b[:, 3:]).all()
        for s in range(8):
            ref = int(np.uint32(words[16 + s]).view(np.int32))
            if (fmask >> s) & 1:
                assert ref == slots.index(s)
                continue
            assert ref == -1
            for k in range(3):
                assert (int(words[4 + 2 * k + (s >> 2)]) >> (8 * (s & 3))) & 0xFF == 255
                assert (int(words[10 + 2 * k + (s >> 2)]) >> (8 * (s & 3))) & 0xFF == 0


def test_rejects_empty_mask(rt):
    out = np.zeros(24, np.uint32)
    boxes = np.zeros(6 * 8, np.float32)
    refs = np.zeros(8, np.int32)
    assert rt.LIB.rtgbQuantizeNode8(boxes.ctypes.data, refs.ctypes.data, 0, out.ctypes.data) == 0
    assert rt.LIB.rtgbQuantizeNode8(boxes.ctypes.data, refs.ctypes.data, 256, out.ctypes.data) == 0
