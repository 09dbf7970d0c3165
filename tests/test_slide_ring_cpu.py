"""The window the slide_3 replay's ring of pending re-tests relies on
(hc_slide.cu): a move at loop position P (P = y*(imax+2) + x, x the
down_scan row, visited at the clamped row 2..imax-1) queues only positions
in (P, P + 2*(imax+2) + 4], which the ring of R positions covers, R the
power of two >= 2*(imax+2) + 64.  The queued positions are restated here
from push_affected's rule: the cells within one of the visited cell or of a
moved-to neighbour, their down_scan entries, and the clamped entries of
rows 1 and imax."""
import itertools

import numpy as np

DXS = (1, 0, -1, -1, -1, 0, 1, 1)
DYS = (1, 1, 1, 0, -1, -1, -1, 0)


def ring_positions(imax):
    R = 64
    while R < 2 * (imax + 2) + 64:
        R <<= 1
    return R


def queued(imax, jmax, x_row, y, moved):
    """positions push_affected queues after the visit of down_scan entry
    (x_row, y), every mask cell wet"""
    H = imax + 2
    x = min(max(x_row, 2), imax - 1)
    P = y * H + x_row
    changed = [(x, y)] + [(x + DXS[k], y + DYS[k]) for k in range(8) if (moved >> k) & 1]
    out = set()
    for cx, cy in changed:
        for dx, dy in itertools.product((-1, 0, 1), repeat=2):
            xx, yy = cx + dx, cy + dy
            if not (2 <= xx <= imax - 1 and 2 <= yy <= jmax - 1):
                continue
            if abs(xx - x) > 2 or abs(yy - y) > 2:
                continue
            for row in [xx] + ([1] if xx == 2 else []) + ([imax] if xx == imax - 1 else []):
                Q = yy * H + row
                if Q > P:
                    out.add(Q)
    return P, out


def test_ring_covers_every_queued_position():
    rng = np.random.default_rng(1)
    for imax, jmax in ((5, 5), (6, 40), (40, 6), (300, 100), (2000, 2000), (9000, 20)):
        H = imax + 2
        R = ring_positions(imax)
        worst = 0
        rows = sorted({1, 2, 3, imax - 2, imax - 1, imax} | set(rng.integers(1, imax + 1, 20)))
        cols = sorted({2, 3, jmax - 2, jmax - 1} | set(rng.integers(2, jmax, 10)))
        for x_row in rows:
            if not 1 <= x_row <= imax:
                continue
            for y in cols:
                if not 2 <= y <= jmax - 1:
                    continue
                for moved in (0, 0xFF, 0x01, 0x80, 0x0F, 0xF0) + tuple(rng.integers(0, 256, 4)):
                    P, qs = queued(imax, jmax, x_row, y, int(moved))
                    for Q in qs:
                        worst = max(worst, Q - P)
        assert worst <= 2 * H + 4, (imax, jmax, worst)
        assert 2 * H + 4 < R, (imax, R)
        # the words of the ring are a power of two (index = (P >> 5) & (RW - 1))
        assert R & (R - 1) == 0 and R >= 64
