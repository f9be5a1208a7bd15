"""ORACLE (test infrastructure only) - Philox4x32-10 in Python/NumPy, from
Salmon et al., SC'11, to check the device stream: counter (step, traj),
key = seed, two 53-bit uniforms per step as CPython builds random()."""
import numpy as np

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    c0, c1, c2, c3 = ctr
    k0, k1 = key
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> 32, p0 & MASK
        hi1, lo1 = p1 >> 32, p1 & MASK
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & MASK, lo1, (hi0 ^ c3 ^ k1) & MASK, lo0
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    return c0, c1, c2, c3


def u53(a, b):
    return ((a >> 5) * 67108864.0 + (b >> 6)) * (1.0 / 9007199254740992.0)


def step_uniforms(seed, traj, step):
    r = philox4x32_10((step & MASK, step >> 32, traj & MASK, traj >> 32),
                      (seed & MASK, seed >> 32))
    return u53(r[0], r[1]), u53(r[2], r[3])
