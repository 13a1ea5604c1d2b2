"""The FP32 chronicle's node-span rounding (onekapy_gb300/csrc/track32.cu,
insert32 and disk32), restated on the host in float32.

For a row interval (LO, HI) in node units and the columns [cl, cr) of the
frame, the kernel marks the nodes

    nearest(max(LO - 1/2, cl - 5/4)) + 1  ..  nearest(min(HI + 1/2, cr + 1/4)) - 1

where nearest() is the round-to-nearest-even of adding 1.5 * 2^23.  These
tests pin the two facts the kernel relies on: the clamp values are never
ties, so an interval reaching past the frame gives exactly cl and cr - 1
(the earlier clamp at cl - 1 and cr was a tie and reached one column
outside for an even cl or an odd cr), and inside the clamps the span is
floor(LO) + 1 .. ceil(HI) - 1 except when LO or HI is an integer.
"""
import numpy as np

F = np.float32
MAGIC = F(12582912.0)          # 1.5 * 2^23
MAGIC_BITS = 0x4B400000


def _bits(x):
    return int(np.array(x, dtype=np.float32).view(np.int32))


def span(lo, hi, cl, cr, coff=0):
    """(glo, ghi) as the kernel computes them (float32 throughout)."""
    xlo = F(F(cl) - F(1.25))
    xhi = F(F(cr) + F(0.25))
    lom = F(F(lo) - F(0.5))
    hip = F(F(hi) + F(0.5))
    klo = (MAGIC_BITS - 1) - coff
    khi = (MAGIC_BITS + 1) - coff
    glo = _bits(F(max(lom, xlo) + MAGIC)) - klo
    ghi = _bits(F(min(hip, xhi) + MAGIC)) - khi
    return glo, ghi


def old_span(lo, hi, cl, cr):
    """The earlier clamp at cl - 1 and cr (with the halves added after it)."""
    xlo = F(F(cl) - F(1.0))
    xhi = F(cr)
    jlo = _bits(F(F(max(F(lo), xlo) - F(0.5)) + MAGIC)) - (MAGIC_BITS - 1)
    jhi = _bits(F(F(min(F(hi), xhi) + F(0.5)) + MAGIC)) - (MAGIC_BITS + 1)
    return jlo, jhi


def test_clamps_give_exactly_the_frame_columns():
    for cl in range(0, 70):
        for cr in range(cl + 1, cl + 40):
            glo, ghi = span(-1.0e5, 1.0e5, cl, cr)
            assert (glo, ghi) == (cl, cr - 1), (cl, cr, glo, ghi)


def test_old_clamp_reached_one_column_outside():
    even_cl = [cl for cl in range(0, 20, 2) if old_span(-1.0e5, 1.0e5, cl, cl + 8)[0] == cl - 1]
    odd_cr = [cr for cr in range(1, 21, 2) if old_span(-1.0e5, 1.0e5, 0, cr)[1] == cr]
    assert len(even_cl) == 10 and len(odd_cr) == 10


def test_span_inside_the_clamps_is_floor_and_ceil():
    rng = np.random.default_rng(7)
    lo = rng.uniform(-5.0, 900.0, 20000).astype(np.float32)
    hi = (lo + rng.uniform(0.0, 12.0, lo.size)).astype(np.float32)
    cl, cr = 3, 880
    bad = 0
    for a, b in zip(lo, hi):
        glo, ghi = span(a, b, cl, cr)
        a64, b64 = float(a), float(b)
        if a64 == np.floor(a64) or b64 == np.floor(b64):
            continue                       # integer ends: ties, within the boundary tolerance
        want_lo = max(int(np.floor(a64)) + 1, cl)
        want_hi = min(int(np.ceil(b64)) - 1, cr - 1)
        # the halves folded into the ends add one float32 rounding of LO and HI
        if (glo, ghi) != (want_lo, want_hi):
            near = min(abs(a64 - round(a64)), abs(b64 - round(b64)))
            assert near < 1e-3, (a64, b64, glo, ghi, want_lo, want_hi)
            bad += 1
    assert bad <= 2


def test_empty_intervals_give_empty_spans():
    for cl, cr in [(0, 10), (5, 64), (2, 3)]:
        glo, ghi = span(np.inf, -np.inf, cl, cr)
        assert glo > ghi
        for a in np.linspace(cl - 3.3, cr + 2.7, 41):
            for d in (0.0, 0.25, 3.0):
                glo, ghi = span(a + d, a, cl, cr)      # LO >= HI
                assert glo >= ghi
                if (glo == ghi):
                    # only at an integer end (a tie), never a node away from it
                    assert abs(F(a) - np.round(F(a))) < 1e-6 or abs(F(a + d) - np.round(F(a + d))) < 1e-6


def test_column_offset_is_folded_exactly():
    for coff in (-7, 0, 13, 400):
        for cl, cr in [(0, 9), (4, 33)]:
            glo, ghi = span(1.3, 6.8, cl, cr, coff)
            base = span(1.3, 6.8, cl, cr)
            assert (glo, ghi) == (base[0] + coff, base[1] + coff)
