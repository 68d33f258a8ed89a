"""CPU check of the row division the build kernels use instead of an integer division per pixel:
with M = floor((2^64 - 1) / w) + 1 in 64-bit unsigned arithmetic (computed on the host per frame
level, FrameDev::rowdiv), the high 64 bits of i * M equal floor(i / w) for every 32-bit pixel index
i.  Exhaustive over small indices and the widths a level can have (every level is at least 4 pixels
wide: frameset_alloc rejects smaller top levels), random over the full index range."""
import random

import pytest

M64 = (1 << 64) - 1


def magic(w: int) -> int:
    # the host's `0xffffffffffffffffull / w + 1ull`, wrapping like the 64-bit unsigned it is
    return (M64 // w + 1) & M64


def row(i: int, w: int) -> int:
    return (i * magic(w)) >> 64


@pytest.mark.parametrize("w", list(range(4, 700)) + [1280, 1920, 2048, 4096, 8191, 8192, 16384])
def test_row_of_flat_index(w):
    rng = random.Random(w)
    idx = list(range(0, 4 * w + 3)) + [rng.randrange(0, 1 << 31) for _ in range(300)] + [(1 << 31) - 1]
    for i in idx:
        assert row(i, w) == i // w, (w, i)


def test_width_one_wraps():
    # why levels narrower than 4 pixels are refused: at w = 1 the magic number wraps to 0
    assert magic(1) == 0 and row(5, 1) != 5


def test_bound_of_the_rule():
    # M w = 2^64 + e with 0 <= e < w; exact while i e < 2^64, so any i < 2^32 and w < 2^32 works
    for w in (4, 40, 640, 4095, 65537):
        e = magic(w) * w - (1 << 64)
        assert 0 <= e < w
        assert ((1 << 32) - 1) * e < (1 << 64)
