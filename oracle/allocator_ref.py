"""Minimum-sample labels of the learned sample allocator, in numpy.  TEST
INFRASTRUCTURE ONLY (the checker of the GPU label search).

The label search renders every entry (pose, ommatidium) `seeds` times with
independent random streams at 4, 8, ..., 1024 samples; an entry's label is
the first count at which the sample standard deviation (n - 1) of its colour
across the renders is below a threshold in every channel, 0 when no count up
to 1024 gets there.  The idea follows the reference's minimum-sample-rate
search, which renders repeated frames per sample count and thresholds their
spread (data/tools/minimumSampleRateFinder.py:25-47; it takes the summed
squared deviation of the colour vector, the label rule here takes each
channel on its own).  The arithmetic is the GPU labelKernel's
(compound-ray_gb300/csrc/render.cu), one correctly rounded float operation at
a time: the mean as a sum in render order divided by the count, then the
squared deviations summed in render order, divided by count - 1, the square
root, and the largest over the channels.
"""
import numpy as np


def label_pass(outs, spp, thr, label):
    """One sample count: outs (k, rows, 3) float32 renders; entries of `label`
    (uint16, rows) still 0 become `spp` where every channel's deviation < thr.
    Updates label in place and returns it."""
    f = np.float32
    outs = np.asarray(outs, np.float32)
    k = outs.shape[0]
    worst = np.zeros(outs.shape[1], np.float32)
    with np.errstate(invalid="ignore", over="ignore"):
        for ch in range(3):
            m = np.zeros(outs.shape[1], np.float32)
            for j in range(k):
                m = m + outs[j, :, ch]
            m = m / f(k)
            v = np.zeros(outs.shape[1], np.float32)
            for j in range(k):
                d = outs[j, :, ch] - m
                v = v + d * d
            worst = np.fmax(worst, np.sqrt(v / f(k - 1)))
    hit = (label == 0) & (worst < f(thr))
    label[hit] = spp
    return label


def min_sample_labels(renders, thr):
    """renders: {spp: (k, rows, 3) float32} for spp = 4, 8, ..., 1024.
    Returns the uint16 labels of the rows."""
    counts = sorted(renders)
    label = np.zeros(np.asarray(renders[counts[0]]).shape[1], np.uint16)
    for c in counts:
        label_pass(renders[c], c, thr, label)
    return label


NO_RENDER = 0xFF  # level of an entry whose feature render suffices (kNoRender)
COST_REF = 16.0


def allocate_levels(pred, cost, feature_spp, halvings, exponent, cost_exponent):
    """Bucket level of every entry as the GPU allocateKernel
    (compound-ray_gb300/csrc/render.cu) decides it: the predicted count is
    2^(10 l), l the mean of the allocator's three outputs (pred: rows x 3);
    the count rendered is 2^k with k = ceil(exponent * min(10 l, 11) -
    halvings - cost_exponent * log2(max(cost, 1) / 16) - 1e-3) clamped to
    [2, 11]; 2^k <= feature_spp -> NO_RENDER, k = 11 -> 0x80 | 8 (fallback
    to a 1024-sample render alone), else k - 2.
    Returns (levels uint8, near) where `near` marks entries whose ceil
    argument lies within 1e-4 of an integer: the GPU's log2 is the fast
    hardware approximation, so the level there may differ by one."""
    f = np.float32
    pred = np.asarray(pred, np.float32).reshape(-1, 3)
    cost = np.asarray(cost, np.float32).reshape(-1)
    l = (pred[:, 0] + pred[:, 1] + pred[:, 2]) * f(1.0 / 3.0)
    l10 = l * f(10.0)
    shift = (f(cost_exponent) * np.log2(np.maximum(cost, f(1.0)) / f(COST_REF)).astype(np.float32)
             if cost_exponent != 0 else np.zeros_like(l10))
    arg = np.minimum(l10, f(11.0)) * f(exponent) - f(halvings) - shift - f(1e-3)
    near = np.abs(arg - np.round(arg)) < 1e-4
    kf = np.ceil(arg)
    kf = np.where(np.isnan(l10), f(2.0), kf)
    kf = np.clip(np.where(kf >= 2.0, kf, 2.0), 2.0, 11.0).astype(np.int64)
    lv = np.where((1 << kf) <= feature_spp, NO_RENDER, np.where(kf == 11, 0x80 | 8, kf - 2)).astype(np.uint8)
    return lv, near
