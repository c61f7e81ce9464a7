"""Host restatement of the counter-based stream in csrc/philox.h.

Used to predict proposals on the host (tests, replay tooling) and to check the
device stream.  Philox4x32-10, Salmon et al., SC'11.
"""
from __future__ import annotations

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(c0: int, c1: int, c2: int, c3: int, k0: int, k1: int):
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = (p0 >> 32) & MASK, p0 & MASK
        hi1, lo1 = (p1 >> 32) & MASK, p1 & MASK
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    return c0, c1, c2, c3


def u01_53(a: int, b: int) -> float:
    return ((a >> 5) * 67108864.0 + (b >> 6)) * (1.0 / 9007199254740992.0)


def below(w: int, n: int) -> int:
    return (w * n) >> 32


def trial_draw(seed: int, chain: int, trial: int, lane: int):
    return philox4x32_10(trial & MASK, (trial >> 32) & MASK, lane, 0, seed & MASK, ((seed >> 32) & MASK) ^ chain)


def flip_proposal(seed: int, chain: int, trial: int, n_sites: int, old_species_of, n_species: int):
    """(site, new species, uniform) of a semi-grand-canonical trial."""
    w = trial_draw(seed, chain, trial, 0)
    site = below(w[0], n_sites)
    old = old_species_of(site)
    k = below(w[1], n_species - 1)
    return site, k + (k >= old), u01_53(w[2], w[3])


def pt_uniform(seed: int, round_index: int, position: int) -> float:
    """Uniform of the replica exchange at ladder position ``position`` of exchange round ``round_index``."""
    w = philox4x32_10(round_index & MASK, (round_index >> 32) & MASK, position, 0xA5A5, seed & MASK,
                      (seed >> 32) & MASK)
    return u01_53(w[0], w[1])
