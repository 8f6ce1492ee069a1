"""The double-float arithmetic of the subspace GEMM (csrc/dfgemm.cu), step for
step in NumPy float32: the integer hi/lo split of an FP64 value, the exact
product (FMA error plus cross terms), TwoSum accumulation and the
renormalisation after every 16 K steps.  Pins the scheme's error on the host;
the GPU kernel itself is checked against cuBLAS FP64 in test_gpu_kernels.py."""

from __future__ import annotations

import numpy as np
import pytest

F32 = np.float32


def split_d(x: float):
    """hi = x truncated to 24 significand bits, lo = the remainder rounded to 24 bits."""
    u = int(np.float64(x).view(np.uint64))
    sign = (u >> 63) << 31
    e = (u >> 52) & 0x7FF
    fe = e - 1023 + 127
    if fe <= 0:
        return F32(0), F32(0)
    m = u & 0xFFFFFFFFFFFFF
    hi = np.uint32(sign | (fe << 23) | (m >> 29)).view(np.float32)
    se = e - 1075 + 127
    r = F32(m & 0x1FFFFFFF)
    lo = F32(r * np.uint32(se << 23).view(np.float32)) if se > 0 else F32(0)
    return F32(hi), (-lo if sign else lo)


def _fma(a, b, c):
    # a b is exact in FP64 (48 bits); one rounding to FP32 as the hardware FMA
    return F32(np.float64(a) * np.float64(b) + np.float64(c))


def df_mac(s, c, ah, al, bh, bl):
    p = F32(ah * bh)
    e = _fma(al, bh, _fma(ah, bl, _fma(ah, bh, -p)))
    t = F32(s + p)
    z = F32(t - s)
    err = F32(F32(s - F32(t - z)) + F32(p - z))
    return t, F32(c + F32(err + e))


def renorm(s, c):
    t = F32(s + c)
    return t, F32(c - F32(t - s))


def df_dot(a, b):
    """sum_k conj(a_k) b_k the way one output of the kernel accumulates it."""
    acc = [F32(0)] * 4
    for k in range(len(a)):
        arh, arl = split_d(a[k].real)
        aih, ail = split_d(-a[k].imag)          # conjugated operand
        brh, brl = split_d(b[k].real)
        bih, bil = split_d(b[k].imag)
        acc[0], acc[1] = df_mac(acc[0], acc[1], arh, arl, brh, brl)
        acc[0], acc[1] = df_mac(acc[0], acc[1], -aih, -ail, bih, bil)
        acc[2], acc[3] = df_mac(acc[2], acc[3], arh, arl, bih, bil)
        acc[2], acc[3] = df_mac(acc[2], acc[3], aih, ail, brh, brl)
        if k % 16 == 15:
            acc[0], acc[1] = renorm(acc[0], acc[1])
            acc[2], acc[3] = renorm(acc[2], acc[3])
    return complex(float(acc[0]) + float(acc[1]), float(acc[2]) + float(acc[3]))


def test_split_keeps_48_bits():
    rng = np.random.default_rng(3)
    xs = rng.normal(size=500) * np.exp(rng.uniform(-40, 40, 500))
    for x in xs:
        hi, lo = split_d(x)
        assert abs(float(hi) + float(lo) - x) <= 4e-15 * abs(x)
        assert abs(float(hi)) <= abs(x)              # truncation toward zero
    assert split_d(0.0) == (0.0, 0.0)
    assert split_d(1e-40) == (0.0, 0.0)              # below the FP32 normal range


@pytest.mark.parametrize("K", [1, 17, 300, 2000])
def test_double_float_dot_matches_extended_precision(K):
    rng = np.random.default_rng(K)
    a = rng.normal(size=K) * np.exp(rng.uniform(-6, 0, K)) + 1j * rng.normal(size=K)
    b = rng.normal(size=K) + 1e-3j * rng.normal(size=K)
    exact = complex(np.sum(np.conj(a).astype(np.clongdouble) * b.astype(np.clongdouble)))
    scale = float(np.sum(np.abs(a) * np.abs(b)))
    assert abs(df_dot(a, b) - exact) <= 3e-14 * scale
