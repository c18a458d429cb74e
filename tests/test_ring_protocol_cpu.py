"""Model check of the band kernels' ring protocol (csrc/dp_band.cuh, csrc/dp_band16.cuh) and of the chain of
warps' hand-over (csrc/myers_chain.cuh), run on the CPU.

Strips of one pair go round a ring of W warps (strip k on member k mod W, each member sweeping its strips in order).
A strip writes its bottom row into ring slot k mod W and publishes how many columns it has written; the strip below
waits, at the start of each staging chunk, until the columns that chunk stages are published, then reads them. This
restates, per kernel variant, the arithmetic the kernels use for those three things:

    variant            lane skew   columns per step   staged per chunk   bottom row's column(s) at step t
    32-bit, 1 column   31          1                  32                 t - 30
    32-bit, 2 columns  31          2                  32                 2(t - 31) + 1, + 2
    16-bit, 1 column   63          1                  64                 t - 62            (high half of lane 31)
    16-bit, 2 columns  63          2                  64                 2(t - 63) + 1, + 2

and plays the warps step by step. It checks that every published count covers only columns already written, that
every staged column was published before it was read, that a slot's columns are read before the strip W places
further down overwrites them, and that the ring never stalls (every wait ends).
"""
import itertools

import pytest

VARIANTS = {  # name: (lane skew, columns per step, columns staged per chunk)
    "band32-one-column": (31, 1, 32),
    "band32-two-columns": (31, 2, 32),
    "band16-one-column": (63, 1, 64),
    "band16-two-columns": (63, 2, 64),
}


class Strip:
    def __init__(self, k, m, skew, columns, chunk, last_skew):
        self.k, self.m, self.skew, self.columns, self.chunk = k, m, skew, columns, chunk
        self.steps = (m + columns - 1) // columns + last_skew
        self.t = 0

    def staged(self, t):
        """Columns lane 0 stages at step t (a chunk boundary): the chunk starting at its current column."""
        first = self.columns * t + 1
        return range(first, min(self.m, first + self.chunk - 1) + 1)

    def need(self, t):
        return min(self.m, self.columns * t + self.chunk)

    def published_before(self, t):
        """The count the bottom-row writer publishes at the start of step t (t a chunk boundary past the skew)."""
        return min(self.m, self.columns * (t - self.skew))

    def written_at(self, t):
        """Bottom-row columns the last lane writes during step t."""
        first = self.columns * (t - self.skew) + 1
        return [j for j in range(first, first + self.columns) if 1 <= j <= self.m]


def play(m, strips, members, variant, last_rows_lanes=None):
    skew, columns, chunk = VARIANTS[variant]
    steps_per_chunk = chunk // columns
    # The last strip may hold fewer lanes (its last lane is then lower): its sweep is shorter.
    last_skew = skew if last_rows_lanes is None else last_rows_lanes
    queue = {w: [k for k in range(strips) if k % members == w] for w in range(members)}
    current = {w: None for w in range(members)}
    published = {}                 # strip -> published count
    written = {}                   # (strip, column) -> tick written
    staged_by = {}                 # (strip, column) -> tick the strip below staged it
    overwritten = {}               # (slot, column) -> list of (tick, strip) writes
    tick = 0
    finished = 0
    while finished < strips:
        tick += 1
        progressed = False
        for w in range(members):
            if current[w] is None:
                if not queue[w]:
                    continue
                k = queue[w].pop(0)
                current[w] = Strip(k, m, skew, columns, chunk, last_skew if k == strips - 1 else skew)
            s = current[w]
            t = s.t
            if t < s.steps:
                if t % steps_per_chunk == 0:
                    if s.k > 0 and columns * t + 1 <= m:
                        if published.get(s.k - 1, 0) < s.need(t):
                            continue  # waits; retried next tick
                        for j in s.staged(t):
                            assert (s.k - 1, j) in written, (variant, m, s.k, t, j)
                            staged_by[(s.k - 1, j)] = tick
                    if s.k + 1 < strips and t > skew:
                        count = s.published_before(t)
                        assert all((s.k, j) in written for j in range(1, count + 1)), (variant, m, s.k, t, count)
                        published[s.k] = max(published.get(s.k, 0), count)
                if s.k + 1 < strips:
                    for j in s.written_at(t):
                        written[(s.k, j)] = tick
                        overwritten.setdefault((s.k % members, j), []).append((tick, s.k))
                s.t += 1
                progressed = True
            if s.t >= s.steps:
                if s.k + 1 < strips:
                    assert all((s.k, j) in written for j in range(1, m + 1))
                    published[s.k] = m
                current[w] = None
                finished += 1
                progressed = True
        assert progressed, f"ring stalled: {variant} m={m} strips={strips} members={members}"
    # A slot's column is staged by strip k + 1 before strip k + W writes the same slot and column.
    for (slot, j), writes in overwritten.items():
        for (tick_a, k_a), (tick_b, k_b) in zip(writes, writes[1:]):
            assert k_b == k_a + members
            if k_a + 1 < strips:
                assert staged_by[(k_a, j)] < tick_b, (variant, m, slot, j, k_a, k_b)
    return tick


@pytest.mark.parametrize("variant", sorted(VARIANTS))
@pytest.mark.parametrize("m", [1, 2, 3, 31, 32, 33, 63, 64, 65, 95, 127, 128, 129, 200, 301])
def test_ring_protocol(variant, m):
    for strips, members in itertools.product([1, 2, 3, 5, 9], [2, 3, 8]):
        play(m, strips, members, variant)
        play(m, strips, members, variant, last_rows_lanes=0)


@pytest.mark.parametrize("variant", sorted(VARIANTS))
def test_two_columns_shorten_the_ring(variant):
    """Steps until a ring of one strip per warp finishes: the two-column sweeps need fewer (the sweep halves and
    the strip below starts 48 / 96 steps behind instead of 64 / 128)."""
    skew, columns, chunk = VARIANTS[variant]
    ticks = play(4000, 24, 24, variant)
    one_column = play(4000, 24, 24, variant.replace("two-columns", "one-column"))
    if columns == 2:
        assert ticks < 0.7 * one_column


def play_chain(m, warps):
    """The chain of warps (0-based columns): warp k's lane 31 writes the byte of column j = t - 31 at step t and
    publishes j + 1 after each 32nd column and after the last; at every 32nd step t < m warp k + 1 waits until
    min(m, t + 32) columns are published, then its lanes read columns t .. t + 31. All warps are resident."""
    steps = m + 31
    t = [0] * warps
    published = [0] * warps
    written = [set() for _ in range(warps)]
    while min(t) < steps:
        progressed = False
        for k in range(warps):
            if t[k] >= steps:
                continue
            step = t[k]
            if step % 32 == 0 and k > 0 and step < m:
                if published[k - 1] < min(m, step + 32):
                    continue
                for column in range(step, min(m, step + 32)):
                    assert column in written[k - 1], (m, warps, k, step, column)
            j = step - 31
            if k + 1 < warps and 0 <= j < m:
                written[k].add(j)
                if j % 32 == 31 or j + 1 == m:
                    assert all(c in written[k] for c in range(j + 1))
                    published[k] = j + 1
            t[k] += 1
            progressed = True
        assert progressed, f"chain stalled: m={m} warps={warps}"


@pytest.mark.parametrize("m", [1, 2, 31, 32, 33, 63, 64, 65, 100, 257])
def test_chain_protocol(m):
    for warps in (1, 2, 3, 7):
        play_chain(m, warps)
