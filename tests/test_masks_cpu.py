"""The chunk masks of the integrate kernel's A operand (chunk_mask in
libgpw_gb300/csrc/gpw_mixed.cu), emulated on the CPU: bit k of an 8-bit row
mask selects half k of a 16-byte chunk of packed fp16 values.  The kernel moves
bit k to the top of byte k with one 32-bit multiply per 4 bits and spreads each
byte's top bit over its half with prmt.b32, whose selector nibbles with the top
bit set replicate the sign bit of the selected byte (the generic mode of the
PTX instruction).  This checks that construction against the definition for
every mask pattern; the kernel itself is compared with the oracle in the GPU
tests."""
import numpy as np

SPREAD = 0x10204080  # 2^7 + 2^14 + 2^21 + 2^28


def prmt(a: int, b: int, sel: int) -> int:
    """prmt.b32 d, a, b, sel (generic mode): byte n of d is byte sel[n] & 7 of
    {b, a} (a = bytes 0-3), or that byte's sign bit replicated when sel[n] & 8."""
    src = [(a >> (8 * i)) & 0xFF for i in range(4)] + [(b >> (8 * i)) & 0xFF for i in range(4)]
    d = 0
    for n in range(4):
        s = (sel >> (4 * n)) & 0xF
        v = src[s & 7]
        if s & 8:
            v = 0xFF if v & 0x80 else 0x00
        d |= v << (8 * n)
    return d


def chunk_mask(b: int) -> tuple:
    lo = ((b & 0xF) * SPREAD) & 0x80808080
    hi = (((b >> 4) & 0xF) * SPREAD) & 0x80808080
    return prmt(lo, 0, 0x9988), prmt(lo, 0, 0xBBAA), prmt(hi, 0, 0x9988), prmt(hi, 0, 0xBBAA)


def definition(b: int) -> tuple:
    halves = [0xFFFF if (b >> k) & 1 else 0 for k in range(8)]
    return tuple(halves[2 * w] | (halves[2 * w + 1] << 16) for w in range(4))


def test_spread_has_no_carries():
    # the four shifted copies of a 4-bit value lie 7 bits apart and fit in 32 bits
    for v in range(16):
        p = v * SPREAD
        assert p < 2**32
        assert p == sum(v << s for s in (7, 14, 21, 28))
        for k in range(4):
            assert ((p >> (8 * k + 7)) & 1) == ((v >> k) & 1)


def test_chunk_masks_match_definition():
    for b in range(256):
        want = definition(b)
        assert chunk_mask(b) == want
        # the kernel passes the row mask shifted to the chunk: bits above 7 are ignored
        for high in (0x100, 0xFFFFFF00):
            assert chunk_mask(b | high) == want


def test_masks_select_halves():
    rng = np.random.default_rng(3)
    vals = rng.integers(0, 2**16, size=8, dtype=np.uint32)
    words = [int(vals[2 * w]) | (int(vals[2 * w + 1]) << 16) for w in range(4)]
    for b in range(256):
        masked = [w & m for w, m in zip(words, chunk_mask(b))]
        got = [(masked[k // 2] >> (16 * (k % 2))) & 0xFFFF for k in range(8)]
        assert got == [int(vals[k]) if (b >> k) & 1 else 0 for k in range(8)]
