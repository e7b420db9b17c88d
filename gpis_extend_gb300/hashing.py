"""Vectorised xxhash32 of one and four words (numpy uint32 arithmetic).

The hash of the sparse-convolution cell and path coordinates
(MathUtil::xxhash32, src/core/math/MathUtil.hpp:179-224), used on the host to
derive flight seeds for whole batches.
"""
import numpy as np

P2 = np.uint32(2246822519)
P3 = np.uint32(3266489917)
P4 = np.uint32(668265263)
P5 = np.uint32(374761393)


def _rotl17(h):
    return (h << np.uint32(17)) | (h >> np.uint32(15))


def _finish(h):
    h = P2 * (h ^ (h >> np.uint32(15)))
    h = P3 * (h ^ (h >> np.uint32(13)))
    return h ^ (h >> np.uint32(16))


def xxhash32_1(p):
    with np.errstate(over="ignore"):
        h = np.asarray(p, np.uint32) + P5
        h = P4 * _rotl17(h)
        return _finish(h)


def xxhash32_2(x, y):
    with np.errstate(over="ignore"):
        h = np.asarray(y, np.uint32) + P5 + np.asarray(x, np.uint32) * P3
        h = P4 * _rotl17(h)
        return _finish(h)


def xxhash32_4(x, y, z, w):
    with np.errstate(over="ignore"):
        h = np.asarray(w, np.uint32) + P5 + np.asarray(x, np.uint32) * P3
        h = P4 * _rotl17(h)
        h = h + np.asarray(y, np.uint32) * P3
        h = P4 * _rotl17(h)
        h = h + np.asarray(z, np.uint32) * P3
        h = P4 * _rotl17(h)
        return _finish(h)
