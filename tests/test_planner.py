"""Invariants of the planner's candidate plans, checked on the CPU.

For every shape and length policy, each candidate the planner offers
(gbsp_plan_candidates) must describe a transform the kernels can run: radices
the row kernel is compiled for, a channel length (their product) that divides
the row's FFT length into at most 64 channels, a whole number of warps per
block and a pass-1 shape index in range.  The FFT length is the Bluestein
length of the policy -- next 3-smooth, 7-smooth or power of two >= 2*cols - 1,
as the reference computes it (oracle/ref_port.py, pinned to the reference's
own functions) -- or, when cols itself has the policy's smoothness and fits
one CTA, cols (one direct FFT per row; force_bluestein restores the former).
"""
import numpy as np
import pytest

import cuspfft_gb300 as gb
from cuspfft_gb300 import tuning
from oracle import ref_port

SUPPORTED_RADICES = {2, 3, 4, 5, 7, 8, 9, 12, 15, 16, 20, 21, 24, 25, 28, 32, 35, 40}
MAX_CHANNELS = 64


def bluestein_length(cols: int, policy: int) -> int:
    n = 2 * cols - 1
    if policy == gb.GBSP_LEN_POW2:
        return ref_port.next_power_of_two(n)
    return ref_port.next_smooth(n, seven=policy == gb.GBSP_LEN_7SMOOTH)


def row_fft_length(cols: int, policy: int, force_bluestein: bool = False) -> int:
    # a smooth row runs as one FFT of length cols when its buffer fits in
    # shared memory (227 KB on GB300)
    if not force_bluestein and 2 <= cols and cols * 8 <= 227 * 1024:
        smooth = ref_port.next_power_of_two(cols) if policy == gb.GBSP_LEN_POW2 else \
            ref_port.next_smooth(cols, seven=policy == gb.GBSP_LEN_7SMOOTH)
        if smooth == cols:
            return cols
    return bluestein_length(cols, policy)


SHAPES = [(5, 8), (64, 97), (1000, 999), (3001, 2048), (8219, 8219), (16706, 16706), (40421, 40421),
          (131071, 33), (33, 120001), (5, 200003)]


@pytest.mark.parametrize("policy", [gb.GBSP_LEN_3SMOOTH, gb.GBSP_LEN_7SMOOTH, gb.GBSP_LEN_POW2])
@pytest.mark.parametrize("rows,cols", SHAPES)
def test_candidates_are_runnable(rows, cols, policy):
    assert gb.next_smooth(2 * cols - 1, policy) == bluestein_length(cols, policy)
    L = row_fft_length(cols, policy)
    cands, nr, npp = tuning.candidates(rows, cols, length_policy=policy)
    assert nr >= 1 and npp >= 1 and len(cands) == nr * npp
    for c in cands:
        rad = c.radices()
        assert rad and set(rad) <= SUPPORTED_RADICES, rad
        lp = int(np.prod(rad))
        assert L % lp == 0, (rad, L)
        assert 1 <= L // lp <= MAX_CHANNELS
        assert c.rows_threads % 32 == 0 and 32 <= c.rows_threads <= 1024
        assert 1 <= c.pass1_shape <= gb._capi.GBSP_N_PASS1_SHAPES
        assert c.length_policy == policy


@pytest.mark.parametrize("rows,cols", [(3001, 2048), (8219, 8219)])
def test_single_channel_when_the_row_fits(rows, cols):
    # a row that fits one CTA's shared memory runs as one channel
    for policy in (gb.GBSP_LEN_3SMOOTH, gb.GBSP_LEN_7SMOOTH):
        cands, _, _ = tuning.candidates(rows, cols, length_policy=policy)
        assert all(int(np.prod(c.radices())) == row_fft_length(cols, policy) for c in cands)
        forced, _, _ = tuning.candidates(rows, cols, length_policy=policy, force_bluestein=1)
        assert all(int(np.prod(c.radices())) == bluestein_length(cols, policy) for c in forced)


@pytest.mark.parametrize("cols,policy,length,channels", [
    (12100, gb.GBSP_LEN_7SMOOTH, 24300, 1),    # a Bluestein length above 24000 still fits one CTA
    (13000, gb.GBSP_LEN_7SMOOTH, 26244, 1),
    (25000, gb.GBSP_LEN_7SMOOTH, 25000, 1),    # smooth columns: one direct FFT of length cols
    (16706, gb.GBSP_LEN_7SMOOTH, 33600, 2),    # 33600 points do not fit: two channels
    (40421, gb.GBSP_LEN_7SMOOTH, 81000, 3),
    (40421, gb.GBSP_LEN_3SMOOTH, 82944, 3),
])
def test_smallest_channel_count_that_fits(cols, policy, length, channels):
    # the convolution splits into the fewest channels whose buffer and inner
    # twiddles fit in shared memory (measured fastest in 15 of 18 cases)
    cands, _, _ = tuning.candidates(4001, cols, length_policy=policy)
    lp = {int(np.prod(c.radices())) for c in cands}
    assert lp == {length // channels}, lp


def test_channel_length_cap_still_applies():
    # max_channel_len bounds the channel: 40421 columns at 24000 points run
    # as five channels of 16200
    cands, _, _ = tuning.candidates(4001, 40421, length_policy=gb.GBSP_LEN_7SMOOTH, max_channel_len=24000)
    assert {int(np.prod(c.radices())) for c in cands} == {16200}


@pytest.mark.parametrize("cols,policy", [(40421, gb.GBSP_LEN_3SMOOTH), (3460, gb.GBSP_LEN_3SMOOTH),
                                         (9861, gb.GBSP_LEN_7SMOOTH), (5088, gb.GBSP_LEN_7SMOOTH)])
def test_first_pick_avoids_a_radix_3_fused_stage(cols, policy):
    # a last (fused) stage of radix 2 or 3 costs twice its share in the row
    # model: these lengths used to rank an x, ..., 3 plan first, measured
    # 4-10 % slower on GB300 than the plan ranked first now
    cands, _, npp = tuning.candidates(4001, cols, length_policy=policy)
    assert cands[0].radices()[-1] > 3, cands[0].radices()
