"""The force mix converts 2^32 fixed point to FP64 in integer arithmetic
(fix_to_double in csrc/sdm_kernels.cu): magnitude normalised by its leading
zeros, 52 mantissa bits rounded to nearest with ties to even, the 2^-32 scale
in the exponent field.  The same steps in Python integers against the
correctly rounded conversion (float(v) * 2^-32, exact scaling) on the
rounding edges and on random values of every magnitude."""
import random
import struct


def fix_to_double(u: int) -> float:
    u &= (1 << 64) - 1
    if u == 0:
        return 0.0
    sign = u & (1 << 63)
    m = ((1 << 64) - u) & ((1 << 64) - 1) if sign else u
    lz = 64 - m.bit_length()
    m = (m << lz) & ((1 << 64) - 1)
    mant = (m >> 11) & ((1 << 52) - 1)
    rest = m & 0x7FF
    bits = ((63 - lz + 1023 - 32) << 52) | mant
    if rest > 0x400 or (rest == 0x400 and (mant & 1)):
        bits += 1
    return struct.unpack("<d", struct.pack("<Q", sign | bits))[0]


def reference(u: int) -> float:
    v = u - (1 << 64) if u >= (1 << 63) else u
    return float(v) * 2.0 ** -32


def test_rounding_edges_and_extremes():
    edges = [0, 1, 2, 3, (1 << 63) - 1, 1 << 52, (1 << 53) - 1, 1 << 53, (1 << 53) + 1, (1 << 53) + 2,
             (1 << 53) + 3, (1 << 54) + 2, (1 << 54) + 6, (1 << 62) + 1024, (1 << 62) + 1536,
             (1 << 62) + 512 + 2048]
    for e in edges:
        for u in (e, ((1 << 64) - e) & ((1 << 64) - 1)):
            assert fix_to_double(u) == reference(u), hex(u)
    assert fix_to_double(1 << 63) == -(2.0 ** 31)          # the most negative value


def test_random_values_of_every_magnitude():
    rng = random.Random(7)
    for _ in range(200000):
        v = rng.getrandbits(64) >> rng.randrange(64)
        u = v if rng.random() < 0.5 else ((1 << 64) - v) & ((1 << 64) - 1)
        a, b = fix_to_double(u), reference(u)
        assert struct.pack("<d", a) == struct.pack("<d", b), hex(u)
