"""Seeded synthetic inputs for WHIR workloads.

The reference draws inputs with rand 0.8 ``StdRng`` and ark-ff's ``Standard`` distribution, which are
not reproducible here; workloads instead use SplitMix64 with rejection sampling:

* Goldilocks element: next SplitMix64 output, rejected when >= p = 2^64 - 2^32 + 1.
* Extension element (Fp2 / Fp3): consecutive accepted base draws, lowest degree first.
* Field192 / Field256 element: one SplitMix64 draw per little-endian u64 limb, the top limb masked to
  the modulus bit length, the whole candidate rejected when >= p.

Elements are returned as canonical little-endian u64 limbs (the C ABI layout).
"""

import numpy as np

GOLDILOCKS_P = 0xFFFFFFFF00000001
F192_P = 3801539170989320091464968600173246866371124347557388484609
F256_P = 21888242871839275222246405745257275088548364400416034343698204186575808495617

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, start, count):
    """Outputs start..start+count of the SplitMix64 stream seeded with `seed`."""
    with np.errstate(over="ignore"):
        idx = np.arange(start + 1, start + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


class Rng:
    """Stateful SplitMix64 stream with the rejection samplers above."""

    def __init__(self, seed):
        self.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        self.pos = 0

    def raw(self, count):
        out = splitmix64(self.seed, self.pos, count)
        self.pos += count
        return out

    def goldilocks(self, count):
        out = np.empty(count, dtype=np.uint64)
        filled = 0
        p = np.uint64(GOLDILOCKS_P)
        while filled < count:
            need = count - filled
            draw = self.raw(need + need // 1000000 + 16)
            ok = draw[draw < p]
            take = min(need, ok.size)
            out[filled:filled + take] = ok[:take]
            # rewind the stream to just after the last consumed draw so the sequence stays exact
            if take < ok.size:
                last = np.nonzero(draw < p)[0][take - 1]
                self.pos -= draw.size - (int(last) + 1)
            filled += take
        return out

    def big_prime(self, count, p):
        limbs = (p.bit_length() + 63) // 64
        top_bits = p.bit_length() - 64 * (limbs - 1)
        mask = (1 << top_bits) - 1
        out = np.zeros((count, limbs), dtype=np.uint64)
        i = 0
        while i < count:
            draw = [int(x) for x in self.raw(limbs)]
            draw[-1] &= mask
            v = sum(d << (64 * k) for k, d in enumerate(draw))
            if v < p:
                out[i] = draw
                i += 1
        return out


def field_elements(field, count, seed=0, rng=None):
    """`count` uniform elements of the named field as an (count, limbs) uint64 array
    (shape (count,) for Goldilocks)."""
    r = rng if rng is not None else Rng(seed)
    if field in ("Goldilocks1", "Field64"):
        return r.goldilocks(count)
    if field in ("Goldilocks2", "Field64_2"):
        return r.goldilocks(2 * count).reshape(count, 2)
    if field in ("Goldilocks3", "Field64_3"):
        return r.goldilocks(3 * count).reshape(count, 3)
    if field == "Field192":
        return r.big_prime(count, F192_P)
    if field == "Field256":
        return r.big_prime(count, F256_P)
    raise ValueError("unknown field %r" % (field,))
