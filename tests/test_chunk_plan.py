"""Host logic of the chunked line walks (CPU).

1. The work plan (`plan_lines` / `line_record` in accrqa_gb300/csrc/rqa_kernels.cuh,
   restated here): for DET (diagonals 1..nc-1, band b has nbands-b blocks) and LAM
   (rows, nbands blocks each), the non-empty (band, chunk) units cover every block of
   every band exactly once, and their boundary records map one to one onto
   [0, nrecords) -- DET's records are packed by chunk.
2. The join: a bit-level model of the kernels' run closing (`close_slot` in
   rqa_device.cuh: a 32-cell mask per block, first cell in bit 31, open run carried)
   started at the chunk sentinel, leads and trails recorded per chunk, and the stitch
   (`line_stitch`) joining them, must give the same run-length histogram as counting
   the runs of the whole line -- for lines that are empty, full, sparse and dense,
   and chunks of one to six blocks.
"""
import random
from collections import Counter

import numpy as np
import pytest

WARPS_PER_CTA = 4
DET_UNITS_PER_WARP = 16
LAM_UNITS_PER_WARP = 16
SENTINEL = 0x80000000
M32 = 0xFFFFFFFF


def band_blocks(det, nbands, b):
    return nbands - b if det else nbands


def line_record(det, nbands, chunk, c, b):
    return c * nbands - chunk * (c * (c - 1) // 2) + b if det else c * nbands + b


def plan_lines(det, nc, sms, allow=True, units=None):
    nbands = (nc - 1 + 31) // 32 if det else (nc + 31) // 32
    blocks = nbands * (nbands + 1) // 2 if det else nbands * nbands
    if units is None:   # the defaults until the autotuner replaces them
        units = DET_UNITS_PER_WARP if det else LAM_UNITS_PER_WARP
    target = units * sms * 8 * WARPS_PER_CTA
    B = -(-blocks // target) if target > 0 else nbands
    B = max(B, 8)
    K = -(-nbands // B) if nbands > 0 else 1
    if not allow or K < 2 or B >= (1 << 25):
        return dict(nbands=nbands, chunk=max(nbands, 1), nchunks=1,
                    nunits=(nbands + 1) // 2 if det else nbands, nrecords=0)
    B = -(-nbands // K)
    K = -(-nbands // B)
    return dict(nbands=nbands, chunk=B, nchunks=K, nunits=K * nbands,
                nrecords=line_record(det, nbands, B, K, 0))


@pytest.mark.parametrize("det", [True, False])
@pytest.mark.parametrize("sms", [1, 8, 152])
@pytest.mark.parametrize("units", [None, 4, 8, 32])   # the autotuner's candidates
def test_plan_covers_blocks_and_records_once(det, sms, units):
    rng = np.random.default_rng(5)
    sizes = [2, 3, 31, 32, 33, 64, 65, 257, 1000, 4097, 20000, 200000, 199944]
    sizes += [int(v) for v in rng.integers(2, 60000, 20)]
    chunked = 0
    for nc in sizes:
        q = plan_lines(det, nc, sms, units=units)
        nb, B = q["nbands"], q["chunk"]
        if q["nrecords"] == 0:
            continue
        chunked += 1
        u = np.arange(q["nunits"], dtype=np.int64)
        c, b = u // nb, u % nb
        blocks = nb - b if det else np.full_like(b, nb)
        live = c * B < blocks
        # blocks of each band, chunk by chunk: [cB, min((c+1)B, blocks)) tile [0, blocks)
        got = np.zeros(nb, dtype=np.int64)
        np.add.at(got, b[live], np.minimum((c[live] + 1) * B, blocks[live]) - c[live] * B)
        np.testing.assert_array_equal(got, nb - np.arange(nb) if det else np.full(nb, nb))
        rec = c[live] * nb - B * (c[live] * (c[live] - 1) // 2) + b[live] if det \
            else c[live] * nb + b[live]
        assert len(np.unique(rec)) == len(rec) == q["nrecords"]
        assert rec.min() == 0 and rec.max() == q["nrecords"] - 1
    if sms == 1:
        assert chunked > 5


def test_whole_lines_when_short():
    assert plan_lines(True, 200, 152)["nrecords"] == 0      # 7 bands: no two chunks of 8 blocks
    assert plan_lines(False, 200, 152)["nrecords"] == 0
    assert plan_lines(True, 200000, 152, allow=False)["nunits"] == (6250 + 1) // 2


def _clz(v):
    return 32 if v == 0 else 32 - v.bit_length()


def _close_slot(m, carry, emit):
    """close_slot of rqa_device.cuh on Python ints (32-bit arithmetic)."""
    full = m == M32
    lead = _clz(~m & M32)
    first = (carry + lead) & M32
    if not full and first:
        emit(first)
    trail = m & (~(m + 1) & M32)
    mid = m & (~trail & M32) & ((M32 >> min(lead, 32)) if lead < 32 else 0)
    carry = (carry + 32) & M32 if full else bin(trail).count("1")
    while mid:
        t = _clz(mid)
        n = _clz(~((mid << t) & M32) & M32)
        emit(n)
        s = t + n
        mid &= (M32 >> s) if s < 32 else 0
    return carry


def _masks(cells):
    out = []
    for k in range(0, len(cells), 32):
        blk = cells[k:k + 32] + [0] * (32 - len(cells[k:k + 32]))
        v = 0
        for bit in blk:
            v = (v << 1) | bit
        out.append(v)
    return out


def _runs(cells):
    h, r = Counter(), 0
    for bit in cells + [0]:
        if bit:
            r += 1
        elif r:
            h[r] += 1
            r = 0
    return h


def _chunked_runs(cells, chunk):
    ms, h, recs = _masks(cells), Counter(), []
    for c0 in range(0, len(ms), chunk):
        lead = [None]

        def emit(n):
            if n >= SENTINEL:
                lead[0] = n - SENTINEL
            else:
                h[n] += 1
        carry = SENTINEL
        for m in ms[c0:c0 + chunk]:
            carry = _close_slot(m, carry, emit)
        recs.append((lead[0], carry))
    pending = 0
    for ld, tr in recs:                       # line_stitch
        if tr >= SENTINEL:
            pending += tr - SENTINEL
            continue
        pending += ld
        if pending:
            h[pending] += 1
        pending = tr
    if pending:
        h[pending] += 1
    return h


def test_stitched_runs_equal_whole_line_runs():
    rnd = random.Random(3)
    for _ in range(1500):
        n = rnd.randint(1, 600)
        p = rnd.choice([0.0, 0.03, 0.5, 0.9, 0.99, 1.0])
        cells = [1 if rnd.random() < p else 0 for _ in range(n)]
        assert _chunked_runs(cells, rnd.randint(1, 6)) == _runs(cells), (n, p)
