"""Algorithmic work of one field evaluation, for the roofline of the march kernel.

Counted once from the reference formulation of the 1D noise evaluation
(evaluateNoise1DNormalized + noise1D + cell1D, SparseConvolutionNoise.cpp:379-485)
with FMA = 2 flops and exp = 1 op, independent of how the kernel computes it:

* impulses inside the truncated kernel per evaluation: 3 cells x N impulses x 2/3
  (uniform impulse positions, support of half-width one cell) = 2N;
* per inside impulse: difference, square, scale, exp, weighted accumulate of the
  value and the derivative (2 FMA) = 1 + 1 + 1 + 1 + 4 = 8 flops, rounded up to 9 to
  count the inside test;
* per evaluation: 40 flops of frame transform, coordinate, normalisation,
  conditioning splats and mean.

The integer work of the cell hash and the PCG draws (3 hashes, 6 warm-up draws
and 6N draws per evaluation in the reference) is not counted as flops; it is
counted separately below as 32-bit operations.
"""

FLOPS_PER_INSIDE_IMPULSE = 9
FLOPS_PER_EVAL_OVERHEAD = 40


def flops_per_eval_1d(impulses_per_cell):
    return 2 * impulses_per_cell * FLOPS_PER_INSIDE_IMPULSE + FLOPS_PER_EVAL_OVERHEAD


def flops_per_eval_3d(impulses_per_cell):
    # every impulse of the 27 cells: 3 differences and the squared length (5 flops);
    # the (4 pi / 3) / 27 = 0.155 inside: ~20 flops (scaled differences, quadratic
    # form, exp, weighted accumulate); 60 flops of overhead (evaluateNoise3D).
    impulses = 27 * impulses_per_cell
    return impulses * 5 + impulses * 0.155 * 20 + 60


# Integer and compare work of one 1D evaluation in the reference formulation, reported
# beside the flops (the path's arithmetic is mostly this): 32-bit operations counted
# from MathUtil::xxhash32(Vec2u) (MathUtil.hpp:190-198: a multiply-add and an add, the
# rotate, three multiplies and three xor-shifts = 12) and UniformSampler::nextI
# (UniformSampler.hpp:44-51: the 64-bit multiply-add as three 32-bit multiply-adds and
# a carried add, the 64-bit xor-shift, the extract and the variable rotate = 17), plus
# BitManip::normalizedUint (shift, or, subtract = 3).  Per cell: the hash, set_state
# and the two warm-up draws; per impulse: two draws with their float conversion, the
# Bernoulli select and the inside test (difference and compare) = 6 more.
INT_OPS_HASH2 = 12
INT_OPS_DRAW = 17 + 3
INT_OPS_PER_CELL = INT_OPS_HASH2 + 1 + 2 * INT_OPS_DRAW
INT_OPS_PER_IMPULSE = 2 * INT_OPS_DRAW + 6


def int_ops_per_eval_1d(impulses_per_cell):
    return 3 * INT_OPS_PER_CELL + 3 * impulses_per_cell * INT_OPS_PER_IMPULSE


# 32-bit lanes per SM that execute integer and FP32 operations (Blackwell SM: 4 x 32)
LANES_PER_SM = 128


# Flight record traffic: 4 input streams of 16 B and 2 result records of 16 B.
BYTES_IN_PER_FLIGHT = 64
BYTES_OUT_PER_FLIGHT = 32
