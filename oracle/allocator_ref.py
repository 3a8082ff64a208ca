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
