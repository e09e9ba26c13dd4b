"""PCG64 (XSL-RR 128/64) restated from the published PCG description.

TEST INFRASTRUCTURE ONLY: the checker for the device generator.

The reference draws every Monte-Carlo random number from
``numpy.random.default_rng(seed)`` (qutip/solver/multitraj.py:382-393), i.e.
numpy's PCG64 bit generator (numpy 2.x, third-party, not vendored in the
reference).  The published algorithm: a 128-bit LCG ``s <- s*M + inc`` with
``M = 0x2360ED051FC65DA44385DF649FCCF645``, advanced before each output, and the
XSL-RR output ``rotr64(hi(s) ^ lo(s), s >> 122)``.  ``Generator.random()`` maps
one output to ``(x >> 11) * 2**-53``.  Parity is pinned draw for draw against
numpy in ``tests/test_oracle.py``.
"""
MULT = 0x2360ED051FC65DA44385DF649FCCF645
MASK128 = (1 << 128) - 1
MASK64 = (1 << 64) - 1


class PCG64:
    def __init__(self, state: int, inc: int):
        self.state = state & MASK128
        self.inc = inc & MASK128

    def next_u64(self) -> int:
        self.state = (self.state * MULT + self.inc) & MASK128
        hi, lo = self.state >> 64, self.state & MASK64
        x = hi ^ lo
        r = self.state >> 122
        return ((x >> r) | (x << ((64 - r) & 63))) & MASK64

    def random(self) -> float:
        return (self.next_u64() >> 11) * (1.0 / 9007199254740992.0)
