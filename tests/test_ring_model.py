"""A CPU model of the ring kernels' row staging (k_bmaps0 in
inovesa_gb300/csrc/batch_kernels.cuh, tile lists from build_tiles in
inovesa_gb300/csrc/batch.cu), checked for the invariants the kernels rely
on, for mixes of mesh sizes, halos and tile sizes:

* every row a tile reads (its rows and their halos) sits in its ring slot
  when the tile is computed;
* staging the next tile's rows overwrites no slot that the current tile
  still reads (the ring holds twice the rows a tile reads);
* the slot arithmetic's precondition: 0 <= x - xref + pref < 2 rb, so one
  conditional subtraction reduces it;
* the byte count of a tile's bulk copies is never negative (a short last
  tile whose new rows all lie beyond the mesh stages none);
* the fast kernel's row copies, spread over its warps, copy every new row
  of a tile exactly once.

No GPU: the model restates the kernels' index arithmetic in Python."""
import itertools

import pytest

RING_MAX_ROWS = 32   # staged rows per tile (build_tiles)


def tiles_of(bunches, tile_cells):
    """(bunch, x0, rows) of every tile, and the ring's slot count."""
    tiles, ring_rows = [], 0
    for b, (n, hlo, hhi) in enumerate(bunches):
        tx = max(4, tile_cells // n)
        tx = min(tx, max(4, RING_MAX_ROWS - hlo - hhi))
        tx = min(tx, n)
        for x0 in range(0, n, tx):
            tiles.append((b, x0, min(tx, n - x0)))
        ring_rows = max(ring_rows, tx + hlo + hhi)
    return tiles, 2 * ring_rows


EMPTY = []   # (bunch, lo, hi) of continuation tiles staging no mesh row


def window_walk(bunches, b, x0, rows, rb, off, ring, nthreads=128):
    """Stage 2 of k_bmaps0f (inovesa_gb300/csrc/ring_fast.cuh) on one
    tile: every segment of n/8 lanes (512 rows: a pair of warps, one per
    half of the row) walks its run of output rows in steps of 4 with a
    window of 4 staged rows per column group, the window's ring offset
    advanced one slot per row from a start reduced modulo the ring.  For
    every drift shift the mesh can have, the rows a valid output row reads
    must be in the slots the walk loads (and every load must stay inside
    the ring, also for rows past the tile); the halves' row sums of a
    512-row tile fit their buffer of rb/2 rows."""
    n, hlo, hhi = bunches[b]
    seg = n // 8
    assert rows <= rb // 2
    # 1024 rows: 5-row windows (256-thread CTAs, two groups of 4 parts)
    depth = 5 if n >= 1024 else 4
    if n >= 1024:
        nthreads = 256
    rp = nthreads // seg
    per = -(-rows // rp)
    steps = -(-per // 4) * 4
    checked = 0
    for sh in range(-hlo, hhi - (depth - 1) + 1):
        for rl in range(rp):
            ra = rl * per
            xend = x0 + min(rows, ra + per)
            raw = x0 + ra + sh + off
            # slot0's reduction: one conditional step each way suffices
            assert -rb <= raw < 2 * rb, ("slot0 range", raw, rb)
            q = raw + rb if raw < 0 else (raw - rb if raw >= rb else raw)
            win = []
            for j in range(depth - 1):
                win.append(q)
                q = q + 1 if q + 1 < rb else 0
            for X in range(x0 + ra, x0 + ra + steps):
                win.append(q)                      # row X + sh + depth - 1
                q = q + 1 if q + 1 < rb else 0
                assert all(0 <= w < rb for w in win)
                if X < xend:
                    for j in range(depth):
                        assert ring.get(win[j]) == (b, X + sh + j), (
                            "window row", b, X, sh, j)
                        checked += 1
                win.pop(0)
    return checked


def walk(bunches, tiles, rb, c, nctas, windows=False):
    """One CTA's chunk, as the kernel walks it; raises on a violation."""
    ntiles = len(tiles)
    t_begin, t_end = c * ntiles // nctas, (c + 1) * ntiles // nctas
    if t_begin == t_end:
        return 0
    ring = {}

    def slot(x, off):
        s = x + off
        assert 0 <= s < 2 * rb, (x, off, rb)
        return s - rb if s >= rb else s

    def stage(b, lo, hi, off, reads):
        n = bunches[b][0]
        a = max(lo, 0)
        if min(hi, n) < a:
            EMPTY.append((b, lo, hi))
        e = max(min(hi, n), a)
        assert e >= a
        for x in range(lo, hi):
            s = slot(x, off)
            assert s not in reads, ("overwrites a row in use", b, x, s)
            ring[s] = (b, x)

    b, x0, rows = tiles[t_begin]
    n, hlo, hhi = bunches[b]
    lo_c, hi_c = x0 - hlo, x0 + rows + hhi
    off = 0 - lo_c
    front = hi_c - lo_c
    stage(b, lo_c, hi_c, off, set())
    checked = 0
    for tid in range(t_begin, t_end):
        b, x0, rows = tiles[tid]
        n, hlo, hhi = bunches[b]
        reads = {}
        for x in range(x0 - hlo, x0 + rows + hhi):
            s = slot(x, off)
            assert ring.get(s) == (b, x), ("row missing", b, x, s)
            reads[s] = x
            checked += 1
        if windows and n <= 256:
            checked += window_walk(bunches, b, x0, rows, rb, off, ring)
        if tid + 1 < t_end:
            bn, xn, rn = tiles[tid + 1]
            _, hlo_n, hhi_n = bunches[bn]
            cont = bn == b and xn == x0 + rows
            hi_n = xn + rn + hhi_n
            xr = xn - hlo_n
            if cont:
                off_n = slot(xr, off) - xr
                lo_n = hi_c
            else:
                lo_n = xr
                off_n = front - xr
            front = slot(hi_n, off_n)
            stage(bn, lo_n, hi_n, off_n, reads)
            off, lo_c, hi_c = off_n, lo_n, hi_n
    return checked


MIXES = {
    "scan 256": [(256, 2, 3)] * 12,
    "narrow halos": [(64, 0, 3), (128, 1, 3), (256, 2, 4)] * 4,
    "wide halos": [(128, 6, 9), (256, 10, 12), (64, 3, 3)] * 3,
    "512 rows": [(512, 3, 4)] * 3 + [(512, 1, 3)] * 2,
    "1024 rows": [(1024, 2, 5)] * 3 + [(1024, 1, 4)] * 2,
    "short tails": [(512, 1, 3), (256, 3, 4), (128, 2, 6)] * 2,
}


@pytest.mark.parametrize("mix", sorted(MIXES))
@pytest.mark.parametrize("tile_cells", [2048, 3072, 4096, 6144, 8192, 12288])
def test_ring_staging_invariants(mix, tile_cells):
    bunches = MIXES[mix]
    tiles, rb = tiles_of(bunches, tile_cells)
    total = 0
    for nctas in sorted({1, 3, 7, max(1, len(tiles) // 3), len(tiles)}):
        for c in range(nctas):
            total += walk(bunches, tiles, rb, c, nctas)
    assert total > 0


@pytest.mark.parametrize("mix", ["scan 256", "narrow halos", "wide halos",
                                 "512 rows", "1024 rows", "short tails"])
@pytest.mark.parametrize("tile_cells", [2048, 4096, 8192])
def test_fast_ring_windows(mix, tile_cells):
    bunches = MIXES[mix]
    tiles, rb = tiles_of(bunches, tile_cells)
    total = 0
    for nctas in sorted({1, 5, max(1, len(tiles) // 2)}):
        for c in range(nctas):
            total += walk(bunches, tiles, rb, c, nctas, windows=True)
    assert total > 0


def test_short_tail_beyond_the_halo_is_staged_empty():
    """512-row meshes in 6-row tiles with a halo of 3 below: the last tile
    (2 rows) continues one whose halo already reached past the mesh end,
    so it stages no mesh row (the case that once wrapped the byte count)."""
    del EMPTY[:]
    bunches = [(512, 1, 3)]
    tiles, rb = tiles_of(bunches, 3072)
    walk(bunches, tiles, rb, 0, 1)
    assert EMPTY and all(lo >= 512 for _, lo, _ in EMPTY)


def test_model_detects_a_small_ring():
    """The model is not vacuous: a ring one slot short of twice the rows a
    tile reads overwrites rows in use (or fails the slot precondition)."""
    bunches = [(256, 2, 3)] * 2
    tiles, rb = tiles_of(bunches, 4096)
    with pytest.raises(AssertionError):
        for c in range(3):
            walk(bunches, tiles, rb - 1, c, 3)


@pytest.mark.parametrize("nt", [128, 256])
def test_row_copies_spread_over_warps(nt):
    """issue_rows_cta (ring_fast.cuh): thread t issues rows a + i,
    a + i + NT, ... with i = t / 32 + (NT / 32) (t % 32); every new row of
    a tile is copied exactly once, for every count of new rows, and the
    rows of a tile of at most 32 land on a few lanes of each warp."""
    nw = nt // 32
    for m in range(0, 3 * nt + 5):
        seen = []
        lanes_per_warp = [0] * nw
        for t in range(nt):
            i = t // 32 + nw * (t % 32)
            rows = list(range(i, m, nt))
            seen.extend(rows)
            if rows:
                lanes_per_warp[t // 32] += 1
        assert sorted(seen) == list(range(m)), m
        if m <= 32:
            assert max(lanes_per_warp) - min(lanes_per_warp) <= 1, m
