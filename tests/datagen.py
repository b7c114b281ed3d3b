"""Seeded synthetic inputs shaped like the benchmark configurations."""
import numpy as np


def keys(rng, n, dtype, dist="uniform"):
    dtype = np.dtype(dtype)
    bits = 8 * dtype.itemsize
    udt = np.uint32 if bits == 32 else np.uint64

    def ubits(m):
        return rng.integers(0, 2 ** bits, m, dtype=np.uint64).astype(udt) if bits == 32 else \
            rng.integers(0, 2 ** 63, m, dtype=np.uint64) * 2 + rng.integers(0, 2, m, dtype=np.uint64)

    if dist == "uniform":
        if dtype.kind == "f":
            x = rng.standard_normal(n) * 1000
            return x.astype(dtype)
        return ubits(n).view(dtype)
    if dist == "and2":
        return (ubits(n) & ubits(n)).view(dtype) if dtype.kind != "f" else \
            (rng.standard_normal(n) * rng.standard_normal(n)).astype(dtype)
    if dist == "distinct256":
        table = ubits(256).view(dtype) if dtype.kind != "f" else rng.standard_normal(256).astype(dtype)
        return table[rng.integers(0, 256, n)]
    if dist == "equal":
        return np.full(n, 7, dtype)
    if dist == "two":
        return np.where(rng.integers(0, 2, n) == 1, 5, 3).astype(dtype)
    if dist == "sorted":
        return np.sort(keys(rng, n, dtype, "uniform"))
    if dist == "reverse":
        return np.sort(keys(rng, n, dtype, "uniform"))[::-1].copy()
    if dist == "fbits":
        # Finite float bit patterns plus the special values the bit order ranks.
        if dtype.kind != "f":
            raise ValueError(dist)
        ib = np.int32 if bits == 32 else np.int64
        raw = ubits(n)
        x = raw.view(dtype)
        x = np.where(np.isfinite(x), x, dtype.type(1.5)).astype(dtype)
        specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan, 1e-40, -1e-40],
                            dtype=dtype)
        m = min(n, 64)
        x[:m] = specials[rng.integers(0, specials.size, m)]
        rng.shuffle(x)
        _ = ib
        return x
    raise ValueError(dist)


def wide_keys(rng, n, kind):
    """Keys of the 2^27-key radix configurations: "u64" uniform 64-bit;
    "f32bits" uniform 32-bit patterns with the non-finite ones' exponent
    cleared (finite floats of every magnitude); "f32normal" N(0,1) floats."""
    if kind == "u64":
        return rng.integers(0, 2 ** 63, n, dtype=np.uint64) * 2 + \
            rng.integers(0, 2, n, dtype=np.uint64)
    if kind == "f32bits":
        raw = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
        bad = (raw & 0x7F800000) == 0x7F800000
        raw[bad] &= np.uint32(0x807FFFFF)
        return raw.view(np.float32)
    if kind == "f32normal":
        return rng.standard_normal(n).astype(np.float32)
    raise ValueError(kind)
