"""The algebra of the FFT-based (Makhoul) DCT passes, restated in NumPy (CPU).

The CUDA line bodies (csrc/ns_fft_core.cuh: dct_y_body, dct_x_fwd_body,
dct_x_inv_body) transform two real lines a, b of N points at once:
  v_n = z_{s(n)},  s(n) = 2n (n < N/2), 2(N-1-n)+1 (n >= N/2),  z = a + i b,
  V = DFT_N(v),  U_k = V_k exp(-i pi k / (2N)) / 2  (V_N = V_0),
  A_k = Re U_k - Im U_{N-k},  B_k = Im U_k + Re U_{N-k},
which is the DCT-II (sum_s x_s cos(pi k (2s+1) / (2N))) of a and of b.
Pressure code 2 negates the even (0-based) samples first and reverses the
modes (k -> N-1-k).  The inverse forms V_k = exp(i pi k / (2N)) (Z_k - i Z_{N-k}) / N,
Z = A + i B, Z_N = 0, and x_{s(n)} = (sum_k V_k exp(2 pi i k n / N)).
24 and 48 use a 12-point DFT by the prime-factor split 12 = 3 x 4.
These tests check the restatements; the GPU tests check the kernels.
"""
import numpy as np
import pytest


def src(N):
    n = np.arange(N)
    return np.where(n < N // 2, 2 * n, 2 * (N - 1 - n) + 1)


def dct2_half(x):
    N = len(x)
    s = np.arange(N)
    return np.array([np.sum(x * np.cos(np.pi * k * (2 * s + 1) / (2 * N))) for k in range(N)])


def makhoul_fwd(a, b, pb):
    N = len(a)
    z = a + 1j * b
    if pb == 2:
        z = z * np.where(np.arange(N) % 2 == 0, -1.0, 1.0)
    v = z[src(N)]
    V = np.fft.fft(v)
    Vx = np.concatenate((V, V[:1]))
    k = np.arange(N + 1)
    U = Vx * np.exp(-1j * np.pi * k / (2 * N)) / 2
    Um = U[N - np.arange(N + 1)]
    A = (U.real - Um.imag)[:N]
    B = (U.imag + Um.real)[:N]
    if pb == 2:
        A, B = A[::-1], B[::-1]
    return A, B


def makhoul_inv(A, B, pb):
    N = len(A)
    if pb == 2:
        A, B = A[::-1], B[::-1]
    Z = np.concatenate((A + 1j * B, [0.0]))
    k = np.arange(N)
    V = np.exp(1j * np.pi * k / (2 * N)) * (Z[k] - 1j * Z[N - k]) / N
    v = np.fft.ifft(V) * N
    z = np.empty(N, complex)
    z[src(N)] = v
    if pb == 2:
        z = z * np.where(np.arange(N) % 2 == 0, -1.0, 1.0)
    return z.real, z.imag


@pytest.mark.parametrize("N", [24, 32, 48, 64, 256])
@pytest.mark.parametrize("pb", [3, 2])
def test_paired_forward_is_the_dct(N, pb):
    rng = np.random.default_rng(N + pb)
    a, b = rng.standard_normal(N), rng.standard_normal(N)
    A, B = makhoul_fwd(a, b, pb)
    for x, X in ((a, A), (b, B)):
        w = x * (np.where(np.arange(N) % 2 == 0, -1.0, 1.0) if pb == 2 else 1.0)
        ref = dct2_half(w)
        if pb == 2:
            ref = ref[::-1]
        assert np.abs(X - ref).max() < 1e-12 * N


@pytest.mark.parametrize("N", [24, 32, 48, 64, 256])
@pytest.mark.parametrize("pb", [3, 2])
def test_paired_inverse_is_the_exact_inverse(N, pb):
    rng = np.random.default_rng(3 * N + pb)
    a, b = rng.standard_normal(N), rng.standard_normal(N)
    ra, rb = makhoul_inv(*makhoul_fwd(a, b, pb), pb)
    assert np.abs(ra - a).max() < 1e-13 * N and np.abs(rb - b).max() < 1e-13 * N


def test_code_2_is_the_dst_up_to_sign():
    """Negating the even samples, DCT-II and reversing the modes gives
    -DST-II: cos(pi (N-1-k)(2s+1)/(2N)) = (-1)^s sin(pi (k+1)(2s+1)/(2N))."""
    N = 16
    x = np.random.default_rng(1).standard_normal(N)
    A, _ = makhoul_fwd(x, np.zeros(N), 2)
    s = np.arange(N)
    dst = np.array([np.sum(x * np.sin(np.pi * (k + 1) * (2 * s + 1) / (2 * N))) for k in range(N)])
    assert np.abs(A + dst).max() < 1e-12


def test_prime_factor_12():
    """dft12: 3-point DFTs over x[(4 n1 + 3 n2) mod 12], then 4-point DFTs,
    output k2 of row k1 at (4 k1 + 9 k2) mod 12, both directions."""
    x = np.random.default_rng(12).standard_normal(12) + 1j * np.random.default_rng(13).standard_normal(12)
    for sign in (-1, 1):
        y = np.zeros((4, 3), complex)
        for n2 in range(4):
            a = np.array([x[(4 * n1 + 3 * n2) % 12] for n1 in range(3)])
            s_, d = a[1] + a[2], a[1] - a[2]
            t = a[0] - 0.5 * s_
            g = np.sqrt(3) / 2 * (1 if sign < 0 else -1)
            y[n2] = [a[0] + s_, t - 1j * g * d, t + 1j * g * d]
        X = np.zeros(12, complex)
        for k1 in range(3):
            z = np.fft.fft(y[:, k1]) if sign < 0 else np.fft.ifft(y[:, k1]) * 4
            for k2 in range(4):
                X[(4 * k1 + 9 * k2) % 12] = z[k2]
        ref = np.fft.fft(x) if sign < 0 else np.fft.ifft(x) * 12
        assert np.abs(X - ref).max() < 1e-12
