"""numpy model of the GPU delay sampler (test infrastructure).

Restates, on the CPU, what ``mc_dagprop_gb300/csrc/mcd_device.cuh`` draws for one
(sample seed, link): Philox4x32-10 (Salmon et al., SC'11) under a fixed key with
the counter (seed low, seed high, block, salt ^ attempt), and the per-kind
transforms.  A link's block and word come from the compiled DAG
(``MonteCarloPropagator.link_streams``): exponential links and empirical tables
of at most 4,096 bins take one 32-bit word of a block shared with up to three
other links; a lone link (block = its index) takes word 0.  The integer parts
(Philox words, alias-table bin choice) must match the GPU bit for bit; the FP32
transforms match to float rounding, so tests compare those with a tolerance.
"""
from __future__ import annotations

import struct

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)
SALT = 0x6D636470
KEY0, KEY1 = 0x243F6A88, 0x85A308D3


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32-10 over uint32 arrays (broadcast); returns 4 uint32 arrays."""
    c0, c1, c2, c3, k0, k1 = (np.asarray(x, dtype=np.uint64) & MASK for x in (c0, c1, c2, c3, k0, k1))
    c0, c1, c2, c3, k0, k1 = np.broadcast_arrays(c0, c1, c2, c3, k0, k1)
    c0, c1, c2, c3, k0, k1 = (x.copy() for x in (c0, c1, c2, c3, k0, k1))
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        n0 = hi1 ^ c1 ^ k0
        n2 = hi0 ^ c3 ^ k1
        c0, c1, c2, c3 = n0, lo1, n2, lo0
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    return tuple(x.astype(np.uint32) for x in (c0, c1, c2, c3))


ONE_WORD_BINS = 4096


def words(seeds, block, attempt=0, sel=0):
    s = np.asarray(seeds, dtype=np.int64).view(np.uint64)
    return philox4x32_10(s & MASK, s >> np.uint64(32), block, SALT ^ ((attempt << 1) | sel), KEY0, KEY1)


def u01_open0(r):
    """(r + 1/2) / 2^32 as the kernel rounds it to float32."""
    f = np.asarray(r, dtype=np.uint32).astype(np.float32)
    return (f.astype(np.float64) * 2.0 ** -32 + 2.0 ** -33).astype(np.float32)


def _from_bits(b: int) -> float:
    return struct.unpack("<d", struct.pack("<q", b))[0]


def scale_by(base: float, m) -> float:
    """The kernel's base * m for a float32 m >= 1: one IEEE double multiply by the
    double equal to m."""
    return float(base) * float(min(np.float32(m), np.float32(3.4028234663852886e38)))


def exponential_durations(seeds, link, base, lam, max_scale, block=None, word=0):
    """Truncated exponential by inverse CDF, the kernel's formula in float32."""
    r0 = words(seeds, link if block is None else block)[word]
    w = u01_open0(r0).astype(np.float64)
    ratio = max_scale / lam
    c = 1.0 if np.isinf(ratio) else -np.expm1(-ratio)
    omc = 0.0 if np.isinf(ratio) else np.exp(-ratio)
    V = (np.float32(c) * w.astype(np.float32) + np.float32(omc)).astype(np.float32)
    # the kernel takes the logarithm with the MUFU approximation (within 2^-21.4
    # absolute on [0.5, 2], 3 ulp elsewhere); this model takes the exact one
    X = np.maximum(np.minimum(-np.float32(lam) * np.log(V), np.float32(max_scale)), np.float32(0.0)).astype(np.float32)
    return np.array([scale_by(base, np.float32(1.0) + x) for x in X])  # base * (1 + X), 1 + X in float


def alias_table(values, weights):
    """Walker/Vose table as the host compiler builds it: (thresh u32, self value, alias value)."""
    w = np.asarray(weights, np.float64)
    v = np.asarray(values, np.float64)
    n = len(w)
    q = list(w / w.sum() * n)
    small = [i for i in range(n) if q[i] < 1.0]
    large = [i for i in range(n) if q[i] >= 1.0]
    prob = [1.0] * n
    alias = list(range(n))
    while small and large:
        s = small.pop()
        l = large.pop()
        prob[s] = q[s]
        alias[s] = l
        q[l] = (q[l] + q[s]) - 1.0
        (small if q[l] < 1.0 else large).append(l)
    th = np.empty(n, np.uint64)
    va = np.empty(n, np.float64)
    for i in range(n):
        p = prob[i]
        if not p < 1.0:
            th[i] = 0xFFFFFFFF
        elif not p > 0.0:
            th[i] = 0
        else:
            t = np.floor(p * 4294967296.0)
            th[i] = 0xFFFFFFFF if t >= 4294967295.0 else int(t)
        va[i] = v[i] if th[i] == 0xFFFFFFFF else v[alias[i]]
    return th, v, va


def empirical_durations(seeds, link, base, values, weights, relative, block=None, word=0):
    """The kernel's duration for each seed (exact): base + value, or
    base + factor * base, in IEEE double arithmetic as the reference forms them."""
    v = empirical_values(seeds, link, values, weights, block, word)
    return base + v * base if relative else base + v


def empirical_values(seeds, link, values, weights, block=None, word=0):
    """The table value the kernel picks for each seed (exact): the bin from the
    high half of r * n, bin-or-alias from its low half (one word), or from a
    second word for tables of more than ONE_WORD_BINS bins."""
    th, vs, va = alias_table(values, weights)
    n = len(vs)
    w = words(seeds, link if block is None else block)
    if n <= ONE_WORD_BINS:
        x = w[word].astype(np.uint64) * np.uint64(n)
        j = (x >> np.uint64(32)).astype(np.int64)
        u = x & MASK
    else:
        j = ((w[0].astype(np.uint64) * np.uint64(n)) >> np.uint64(32)).astype(np.int64)
        u = w[1].astype(np.uint64)
    keep = u < th[j]
    return np.where(keep, vs[j], va[j])
