"""The column-chunk plan of the host-buffer mixed LU (gbs_streamed_input_plan),
checked on the CPU against the rules of the look-ahead schedule for every order
it covers.  The model below follows getrf_lookahead's joins: a chunk that joins
at iteration k gets blocks 0..k-1 replayed before iteration k's wide update;
the rolling chunk is gathered after the wide update of its iteration and
replays two block updates after each wide update until it has caught up.  A
chunk whose first block is b must take the wide updates by iteration b - 2,
because iteration b - 1's narrow update works on block b."""
import ctypes as C

import pytest

from eigen_gb300 import _lib

NB = 128                 # outer block of the mixed LU
ROLL_PER_ITERATION = 2   # replays of the rolling chunk after each wide update
MAX_CHUNKS = 16


def plan(n):
    col = (C.c_int * (MAX_CHUNKS + 1))()
    it = (C.c_int * MAX_CHUNKS)()
    rolling = C.c_int(-2)
    m = _lib.lib().gbs_streamed_input_plan(n, MAX_CHUNKS, col, it, C.byref(rolling))
    return m, list(col[:m + 1]), list(it[:m]), rolling.value


def simulate(n, m, col, it, rolling):
    """Runs the schedule's join logic; returns the replayed block updates."""
    at_once = rolling if rolling >= 0 else m
    joined, frontier = 1, col[1]
    rolled_in, replayed, replays = rolling < 0, -1, 0
    k, blk = 0, 0
    while k < n:
        kb = min(NB, n - k)
        nr = n - k - kb
        if nr == 0:
            break
        c1 = k + kb + min(NB, nr)
        assert frontier >= c1, (n, blk, frontier, c1)
        while joined < at_once and it[joined] <= blk:
            replays += blk
            frontier = col[joined + 1]
            joined += 1
        if not rolled_in and replayed == blk:
            rolled_in, frontier, joined = True, col[rolling + 1], m
        if not rolled_in and replayed < 0 and joined == at_once and it[rolling] <= blk:
            replayed = 0
        q = 0
        while not rolled_in and replayed >= 0 and q < ROLL_PER_ITERATION and replayed <= blk:
            replayed += 1
            q += 1
            replays += 1
        k += NB
        blk += 1
    assert joined == m and rolled_in, (n, joined, m, rolled_in)
    return replays


def check(n):
    m, col, it, rolling = plan(n)
    assert 2 <= m <= MAX_CHUNKS, (n, m)
    assert col[0] == 0 and col[m] == n
    assert all(a < b for a, b in zip(col, col[1:])), col
    assert all(c % NB == 0 for c in col[1:m]), col
    assert rolling in (-1, m - 1)
    assert it[0] == 0 and all(a <= b for a, b in zip(it, it[1:])), it
    return simulate(n, m, col, it, rolling)


def test_orders_outside_the_range_copy_whole():
    assert plan(2047)[0] == 0
    assert plan(20481)[0] == 0


def test_headline_order():
    """n = 8192: the first four blocks, one chunk that joins at iteration 0,
    and the rest rolling in from iteration 5 (10 replayed block updates)."""
    m, col, it, rolling = plan(8192)
    assert (m, col, it, rolling) == (3, [0, 512, 1536, 8192], [0, 0, 5], 2)
    assert check(8192) == 10


@pytest.mark.parametrize("lo,hi", [(2048, 8192), (8192, 14336), (14336, 20481)])
def test_every_chunk_joins_before_its_columns_are_needed(lo, hi):
    for n in range(lo, hi):
        check(n)


def test_plan_respects_the_capacity_and_null_pointers():
    """cap bounds what is written (col gets cap + 1 entries, iter cap); NULL
    pointers are allowed; the count is returned either way."""
    m, col_full, it_full, rolling = plan(16384)
    assert m > 3
    col = (C.c_int * 4)(*([-5] * 4))
    it = (C.c_int * 4)(*([-5] * 4))
    lib = _lib.lib()
    assert lib.gbs_streamed_input_plan(16384, 2, col, it, None) == m
    assert list(col) == col_full[:3] + [-5]
    assert list(it) == it_full[:2] + [-5, -5]
    assert lib.gbs_streamed_input_plan(16384, 0, None, None, None) == m
    assert lib.gbs_streamed_input_plan(16384, -1, None, None, None) < 0
