"""Seeded splitmix64 stream of the oracle side (test infrastructure).

The same published generator (Steele, Lea and Flood, "Fast splittable
pseudorandom number generators", 2014) as the product's input generator,
written out separately so that the host-core baseline builds its inputs
without loading the product library.  Element i of the stream is
mix(seed + (i+1) * 0x9E3779B97F4A7C15) mod 2^64; uniform01 maps the top 53
bits to [0, 1).
"""
import numpy as np

_STEP = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, n):
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + np.arange(1, n + 1, dtype=np.uint64) * _STEP
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform01(seed, n):
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) / 9007199254740992.0
