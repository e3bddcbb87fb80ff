"""The numerical scheme of the n = 64 tensor-core column transform (k_col_tc),
emulated in NumPy on the CPU; the kernel itself is tested on the GPU.

Per column X[a], a < 64, and direction DIR (+1: the unnormalised inverse
transform of the first stage, -1: the forward transform of the last):
radix-2 decimation in frequency, S = X[a'] + X[a' + 32], D = X[a'] - X[a' + 32];
each half is the real GEMM D_g[o] = sum_kappa Z_g[kappa] F_g[o][kappa] with
Z_g = (Re, Im) of S or D (K = 64) and F_g the images the host builds
(F_g[2k'][a'] = C, F_g[2k'][32 + a'] = -S, F_g[2k' + 1][a'] = S,
F_g[2k' + 1][32 + a'] = C, C + i S = W^{(2k' + g) a'}); the column is scaled by
the power of two that brings max_a' (|X[a']|_1 + |X[a' + 32]|_1) into
[1/2, 1), both operands are split into FP16 pairs x = hi + lo (hi = fp16(x),
lo = fp16(x - hi), round to nearest even) and the product is
Z_hi F_hi + Z_lo F_hi + Z_hi F_lo, summed in FP32.
"""
import numpy as np
import pytest

N = 64


def _images(direction):
    """F_even, F_odd as (64 outputs x 64 K) float64 matrices."""
    o = np.arange(N)[:, None]
    kap = np.arange(N)[None, :]
    k, ap = o >> 1, kap & 31
    out = []
    for g in (0, 1):
        ang = 2 * np.pi * (((2 * k + g) * ap) % N) / N
        c, s = np.cos(ang), direction * np.sin(ang)
        v = np.where(o % 2 == 0, np.where(kap < 32, c, -s), np.where(kap < 32, s, c))
        out.append(v)
    return out


def _split(x):
    hi = x.astype(np.float16)
    lo = (x - hi.astype(x.dtype)).astype(np.float16)
    return hi.astype(np.float64), lo.astype(np.float64)


def _column_dft(X, direction, with_lo=True):
    """Emulated tensor-core transform of the columns X (64 x m complex)."""
    X = X.astype(np.complex64)
    l1 = np.abs(X.real) + np.abs(X.imag)
    mx = (l1[:32] + l1[32:]).max(axis=0)
    ex = np.frexp(mx)[1]  # mx = f 2^ex, f in [1/2, 1)
    down = np.ldexp(np.float32(1.0), -ex).astype(np.float32)
    S = (X[:32] + X[32:]) * down
    D = (X[:32] - X[32:]) * down
    Y = np.empty_like(X, dtype=np.complex128)
    for g, Z in ((0, S), (1, D)):
        Zr = np.concatenate([Z.real, Z.imag]).astype(np.float32)  # K = 64 rows per column
        zh, zl = _split(Zr)
        F = _images(direction)[g]
        fh, fl = _split(F)
        acc = fh @ zh + (fh @ zl if with_lo else 0) + (fl @ zh if with_lo else 0)
        acc = acc.astype(np.float32).astype(np.float64)
        Y[g::2] = acc[0::2] + 1j * acc[1::2]
    return Y * np.ldexp(1.0, ex)


def _reference(X, direction):
    return np.fft.fft(X, axis=0) if direction < 0 else N * np.fft.ifft(X, axis=0)


@pytest.mark.parametrize("direction", [+1, -1])
def test_split_fp16_scheme_accuracy(direction):
    rng = np.random.default_rng(64 + direction)
    smooth = rng.uniform(-1, 1, (N, 96)) + 1j * rng.uniform(-1, 1, (N, 96))
    peaked = 1e-3 * (rng.uniform(-1, 1, (N, 32)) + 1j * rng.uniform(-1, 1, (N, 32)))
    peaked[rng.integers(0, N, 32), np.arange(32)] += 5e3 * (1 + 1j)
    tiny = 1e-30 * smooth[:, :16]  # scales far below FP16's range
    X = np.concatenate([smooth, peaked, tiny], axis=1)
    ref = _reference(X.astype(np.complex64).astype(np.complex128), direction)
    Y = _column_dft(X, direction)
    err = np.abs(Y - ref).max(axis=0) / np.abs(ref).max(axis=0)
    assert err.max() < 2e-6, err.max()
    # (measured: 1.8e-7 on the smooth columns, 1.1e-6 on the peaked ones); without
    # the lo halves (plain FP16 operands) the same columns are off by 2e-4 to 4e-4
    Y16 = _column_dft(X, direction, with_lo=False)
    err16 = np.abs(Y16 - ref).max(axis=0) / np.abs(ref).max(axis=0)
    assert err16.max() > 1e-4


def test_zero_column_takes_scale_one():
    """A zero column (bound 0) takes scale 1 and transforms to zero."""
    X = np.zeros((N, 2), np.complex128)
    X[:, 1] = 1.0
    Y = _column_dft(X, -1)
    assert np.all(Y[:, 0] == 0)
    assert abs(Y[0, 1] - N) < 1e-5 and np.abs(Y[1:, 1]).max() < 1e-5
