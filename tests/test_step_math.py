"""The integer identities the walk kernels rest on, checked in exact Python
arithmetic on random moduli (CPU only; the GPU parity tests check the kernels
themselves against the oracle):

* the reference's shift reduction K <- (K + m p) / 2^s, m = -K p^-1 mod 2^s
  (pps/appcu.cu:591-707), is K 2^-s mod p and below p for K < p;
* the carry-free form used on the device: with p = (phi+1) 2^32 - (2^32 - plo),
  (K + m p) / 2^32 = khi + m (phi+1) - hi32(m (2^32 - plo));
* the same for s < 32 on K 2^(32-s): high word K >> s, m = klo (pinv << (32-s));
* every true candidate K = k 2^i (k <= kmax, i < s) passes the pre-tests: the
  window (hi word 0 or low 32-kb bits zero, s = 32), the window K < 2^s (or low
  s+1-kb bits zero) for s < 32, and the single bound (hi word <= kmax/2) when
  p > kmax 2^43.
"""
from __future__ import annotations

import random

M32 = (1 << 32) - 1


def _pinv(p: int) -> int:
    return (-pow(p, -1, 1 << 32)) & M32


def _random_prime_like(rng: random.Random, bits: int) -> int:
    # the identities need p odd only (primality is not used)
    return rng.getrandbits(bits) | 1 | (1 << (bits - 1))


def test_shift_reduction_is_division_by_power_of_two():
    rng = random.Random(1)
    for _ in range(3000):
        s = rng.randint(1, 32)
        p = _random_prime_like(rng, rng.randint(33, 62))
        K = rng.randrange(p)
        m = (-K * pow(p, -1, 1 << s)) % (1 << s)
        r = (K + m * p) >> s
        assert (K + m * p) % (1 << s) == 0
        assert r < p and r == K * pow(2, -s, p) % p


def test_carry_free_step_32():
    rng = random.Random(2)
    for _ in range(20000):
        p = _random_prime_like(rng, rng.randint(33, 62))
        K = rng.randrange(p)
        klo, khi = K & M32, K >> 32
        m = (klo * _pinv(p)) & M32
        plon, phi1 = (-(p & M32)) & M32, (p >> 32) + 1
        assert (m * plon) & M32 == klo  # so the low word of K + m p is exactly zero
        r = khi + m * phi1 - ((m * plon) >> 32)
        assert r == (K + m * p) >> 32 == K * pow(2, -32, p) % p


def test_carry_free_step_below_32():
    rng = random.Random(3)
    n = 0
    while n < 20000:
        s = rng.randint(1, 31)
        p = _random_prime_like(rng, rng.randint(33, 32 + s))
        if p > 1 << (32 + s):
            continue
        n += 1
        K = rng.randrange(p)
        klo = K & M32
        hi = ((K << (32 - s)) >> 32) & M32
        assert hi == K >> s
        m = (klo * ((_pinv(p) << (32 - s)) & M32)) & M32
        plon, phi1 = (-(p & M32)) & M32, (p >> 32) + 1
        r = hi + m * phi1 - ((m * plon) >> 32)
        assert r == K * pow(2, -s, p) % p


def test_pretests_pass_every_candidate():
    rng = random.Random(4)
    for _ in range(20000):
        kb = rng.randint(2, 20)
        kmax = rng.randrange(1 << (kb - 1), 1 << kb)
        k = rng.randrange(1, kmax + 1, 2) if kmax > 1 else 1
        # s = 32 window with u = 0: hi word zero or the low 32-kb bits zero
        i = rng.randrange(32)
        K = k << i
        assert (K >> 32) == 0 or (K & ((1 << (32 - kb)) - 1)) == 0
        # s < 32 window on the step's high word: K >> s zero or the low s+1-kb bits zero
        s = rng.randint(kb, 31)
        i = rng.randrange(s)
        K = k << i
        mask = (1 << (s + 1 - kb)) - 1
        assert (K >> s) == 0 or (K & mask) == 0
        # single bound: K = k 2^i with i < 32 has hi word <= kmax / 2
        i = rng.randrange(32)
        assert ((k << i) >> 32) <= kmax >> 1


def test_twin_pretest_reads_the_other_side():
    """Twin walks hold K for one side and test p - K for the other: p - K is
    below a bound lim iff K > p - lim, and its low bits (mask) are zero iff K's
    low bits equal p's."""
    rng = random.Random(5)
    for _ in range(20000):
        p = _random_prime_like(rng, rng.randint(33, 62))
        K = rng.randrange(1, p)
        lim = 1 << rng.randint(20, 40)
        mask = (1 << rng.randint(1, 31)) - 1
        v = p - K
        assert (v < lim) == (p > lim and K > p - lim or p <= lim)
        assert ((v & mask) == 0) == ((K & mask) == (p & mask))
