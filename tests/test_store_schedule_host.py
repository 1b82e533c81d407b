"""The flush schedule of K4's tiled AdaptedPathData stores, on the host.

`TiledStoreSink` (csrc/k_store_kern.cuh) parks each lane's rows in a tile of
kT slots: state row r (paths, left, jumps, time; row r = k + 1 after step k,
row 0 from init) in slot r % kT, normals row k in slot k % kT.  A group of
state rows is written when its last slot fills (after step k with
(k + 1) % kT == kT - 1), a group of normals rows likewise ((k % kT) == kT - 1);
after the loop the padding steps kend .. S-1 fill the slots the same way and
the open groups are written.  This model replays that schedule for every tile
length the kernels use and checks that each of the rows 0..S (state) and
0..S-1 (normals) is written exactly once, from the slot the step that owns the
row filled, and that every group starts on a multiple of kT (whole lines when
a path's row is).  The GPU tests compare the kernel's output with per-lane
stores and the oracle on a few step caps; this covers all of them."""
import pytest


def schedule(S, kT, kend):
    """Rows written by the model: {array: {row: (slot, source)}} where source
    is ('step', k) / ('init',) / ('pad', k)."""
    slot_state = [None] * kT
    slot_norm = [None] * kT
    written = {"state": {}, "normals": {}}
    starts = []

    def flush(kind, slots, r0, cnt):
        assert r0 % kT == 0, (kind, r0)
        starts.append((kind, r0))
        for j in range(cnt):
            row = r0 + j
            assert row not in written[kind], (kind, row)
            assert slots[j] is not None, (kind, row)
            written[kind][row] = slots[j]

    slot_state[0] = ("init", 0)                       # init(): row 0
    for k in range(min(kend, S)):                     # step(k), k < S
        sn, ss = k % kT, (k + 1) % kT
        slot_state[ss] = ("step", k + 1)
        slot_norm[sn] = ("step", k)
        if ss == kT - 1:
            flush("state", slot_state, k + 2 - kT, kT)
        if sn == kT - 1:
            flush("normals", slot_norm, k + 1 - kT, kT)
    for k in range(min(kend, S), S):                  # finish(): padding
        sn, ss = k % kT, (k + 1) % kT
        slot_state[ss] = ("pad", k + 1)
        slot_norm[sn] = ("pad", k)
        if ss == kT - 1:
            flush("state", slot_state, k + 2 - kT, kT)
        if sn == kT - 1:
            flush("normals", slot_norm, k + 1 - kT, kT)
    if (S + 1) % kT:
        flush("state", slot_state, S + 1 - (S + 1) % kT, (S + 1) % kT)
    if S % kT:
        flush("normals", slot_norm, S - S % kT, S % kT)
    return written, starts


def tile_rows(d, nw):
    """kT of TiledStoreSink<D, NW> (64-thread CTAs: 192 floats per lane)."""
    kw = 3 * d + 1 + d * nw
    want = max(32 // d, 2)

    def odd(kt):
        return kt * kw + (1 if (kt * kw) % 2 == 0 else 2)
    kt = want if odd(want) <= 192 else max(want // 2, 2)
    assert odd(kt) <= 192
    return kt


@pytest.mark.parametrize("d,nw", [(d, nw) for d in range(1, 9) for nw in (1, 2)])
def test_every_row_written_once_from_its_step(d, nw):
    kT = tile_rows(d, nw)
    for S in sorted({1, 2, kT - 1, kT, kT + 1, 2 * kT - 1, 2 * kT, 3 * kT + 5, 271, 272}):
        if S < 1:
            continue
        for kend in sorted({0, 1, S // 2, S - 1, S, S + 3}):
            written, starts = schedule(S, kT, kend)
            assert sorted(written["state"]) == list(range(S + 1)), (S, kend)
            assert sorted(written["normals"]) == list(range(S)), (S, kend)
            for row, src in written["state"].items():
                if row == 0:
                    assert src == ("init", 0)
                elif row <= min(kend, S):
                    assert src == ("step", row), (S, kend, row, src)
                else:
                    assert src == ("pad", row), (S, kend, row, src)
            for row, src in written["normals"].items():
                assert src == (("step", row) if row < min(kend, S) else ("pad", row)), (S, kend, row, src)
            assert all(r0 % kT == 0 for _, r0 in starts)


def test_tile_lengths_fit_and_segments_are_128_bytes_where_they_can_be():
    for d in range(1, 9):
        kT = tile_rows(d, 1)
        assert kT * d * 4 <= 128
        if d in (1, 2, 4, 8):
            assert kT * d * 4 == 128
