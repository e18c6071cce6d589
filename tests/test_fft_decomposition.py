"""The register-level row transforms' decompositions, restated in numpy on the CPU.

`k_rows_r2c3` (forward) and `c2r3_row` (inverse) in csrc/fft_impl.cuh split a row of
M = L1 L2 L3 complex points (J = L2 L3) into three register levels:
  level 1, item j < J:        z[J a + j] (a < L1), DFT_L1 over a, twiddle W_M^(j k1)
  level 2, item (k1, m < L3): DFT_L2 over b of s[k1 J + L3 b + m], twiddle W_J^(m k2)
  level 3, item (k1, k2):     DFT_L3 over m -> Z[k1 + L1 (k2 + L2 k3)]
with the twiddles read from the row's Nx-entry table exp(-2 pi i e / Nx) at e = 2 j k1
and e = 2 L1 m k2.  These tests run exactly that index arithmetic with numpy DFTs and
compare it, and the split into Nx/2 + 1 spectrum values (and its inverse), with numpy's
FFT for every row length that has a register kernel.  The fused convolution (P0-P3) is
restated the same way: the map's column passes A and B leaving the spectrum in the
digit-transposed row order, P1's profile column sub-pass per kk (the two-term form for
profiles of at most 2 N2 rows and the general loop), and P2, against the oracle's FFT
convolution.  The GPU tests check the kernels themselves.
"""
import numpy as np
import pytest

SIZES = [(8, 25, 25), (16, 16, 16), (8, 10, 25), (10, 10, 10)]  # M = 5000, 4096, 2000, 1000


def _dft(x, inv=False):
    return np.fft.ifft(x, axis=-1) * x.shape[-1] if inv else np.fft.fft(x, axis=-1)


def three_level(z, L1, L2, L3, twx, inv=False):
    """The three register levels over one row z (length M), in the kernels' index order."""
    J, M = L2 * L3, L1 * L2 * L3
    conj = np.conj if inv else (lambda v: v)
    s = np.empty(M, complex)
    for j in range(J):  # level 1
        v = _dft(z[J * np.arange(L1) + j], inv)
        for k1 in range(L1):
            s[k1 * J + j] = v[k1] * conj(twx[2 * j * k1])
    wJ = twx[2 * L1 * np.arange(J)]
    t = np.empty(M, complex)
    for k1 in range(L1):  # level 2
        for m in range(L3):
            u = _dft(s[k1 * J + L3 * np.arange(L2) + m], inv)
            for k2 in range(L2):
                t[k1 * J + k2 * L3 + m] = u[k2] * conj(wJ[m * k2])
    out = np.empty(M, complex)
    for k2 in range(L2):  # level 3
        for k1 in range(L1):
            w = _dft(t[k1 * J + k2 * L3 + np.arange(L3)], inv)
            for k3 in range(L3):
                out[k1 + L1 * (k2 + L2 * k3)] = w[k3]
    return out


def r2c_split(Z, twx):
    """X[k] = (Z[k] + conj Z[M-k]) / 2 - i W^k (Z[k] - conj Z[M-k]) / 2, k <= M."""
    M = Z.shape[0]
    k = np.arange(M + 1)
    zk, zc = Z[k % M], np.conj(Z[(M - k) % M])
    return 0.5 * (zk + zc) - 0.5j * twx[k] * (zk - zc)


@pytest.mark.parametrize("L1,L2,L3", SIZES)
def test_forward_row_decomposition_matches_rfft(L1, L2, L3):
    M = L1 * L2 * L3
    Nx = 2 * M
    twx = np.exp(-2j * np.pi * np.arange(Nx) / Nx)
    x = np.random.default_rng(M).lognormal(0.0, 0.5, Nx)
    Z = three_level(x[0::2] + 1j * x[1::2], L1, L2, L3, twx)
    np.testing.assert_allclose(Z, np.fft.fft(x[0::2] + 1j * x[1::2]), rtol=0, atol=1e-9 * np.abs(x).sum())
    X = r2c_split(Z, twx)
    np.testing.assert_allclose(X, np.fft.rfft(x), rtol=0, atol=1e-9 * np.abs(x).sum())


@pytest.mark.parametrize("L1,L2,L3", SIZES)
def test_inverse_row_decomposition_matches_irfft(L1, L2, L3):
    """c2r3_row: b[k] = (X[k] + conj X[M-k]) + i (X[k] - conj X[M-k]) W^-k, the three levels
    inverted (conjugate twiddles), real row (z.re, z.im) interleaved, unnormalised."""
    M = L1 * L2 * L3
    Nx = 2 * M
    twx = np.exp(-2j * np.pi * np.arange(Nx) / Nx)
    x = np.random.default_rng(M + 1).lognormal(0.0, 0.5, Nx)
    X = np.fft.rfft(x)
    k = np.arange(M)
    xk, xm = X[k], np.conj(X[M - k])
    b = (xk + xm) + 1j * (xk - xm) * np.conj(twx[k])
    z = three_level(b, L1, L2, L3, twx, inv=True)
    row = np.empty(Nx)
    row[0::2], row[1::2] = z.real, z.imag
    np.testing.assert_allclose(row, Nx * x, rtol=0, atol=1e-9 * Nx * np.abs(x).sum())


def radix5_levels(b, twx, inv=True):
    """c2r5_row (float-float rows of M = 5000 = 8 x 5^4; inv=False: the forward mirror in
    k_rows_r2c5): level 1 as in three_level (DFT8 over stride 625, twiddle W_M^(-/+)(j n1),
    formed in the kernels as products of the one loaded power W_M^j, at most three deep),
    then in-place decimation-in-frequency radix-5 levels on blocks of 625, 125, 25 (item
    (block, m): DFT5 over stride J'/5, twiddle W_J'^(-/+)(m r), written back to the slots it
    read) and blocks of 5, whose outputs go to natural order: output r of item
    it = 125 k1 + 25 a + 5 b + c is z[n0 + 1000 r] with n0 = k1 + 8 (a + 5 (b + 5 c))."""
    M, J = 5000, 625
    conj = np.conj if inv else (lambda v: v)
    s = np.empty(M, complex)
    for j in range(J):
        v = _dft(b[J * np.arange(8) + j], inv)
        p1 = twx[2 * j]
        p2 = p1 * p1
        p3 = p2 * p1
        p4 = p2 * p2
        pw = [1.0, p1, p2, p3, p4, p3 * p2, p3 * p3, p4 * p3]
        for n1 in range(8):
            s[n1 * J + j] = v[n1] * conj(pw[n1])
    w = twx[16 * np.arange(J)]  # W_625^e
    for Jp in (625, 125, 25):
        Sp, ws = Jp // 5, 625 // Jp
        for it in range(1000):
            blk, m = divmod(it, Sp)
            idx = blk * Jp + m + Sp * np.arange(5)
            u = _dft(s[idx], inv)
            s[idx] = u * conj(w[m * np.arange(5) * ws])
    z = np.empty(M, complex)
    for it in range(1000):
        u = _dft(s[5 * it + np.arange(5)], inv)
        k1, a5, b5, c5 = it // 125, (it // 25) % 5, (it // 5) % 5, it % 5
        z[k1 + 8 * (a5 + 5 * (b5 + 5 * c5)) + 1000 * np.arange(5)] = u
    return z


def c2r_input_pairs(X, twx):
    """c2r5_row's input: one read of X[k] and X[M-k] (k <= M/2) gives b[k] = e + i o and, for
    the partner, b[M-k] = (e.x + o.y) + i (o.x - e.y), with e = X[k] + conj X[M-k] and
    o = (X[k] - conj X[M-k]) W^-k."""
    M = X.shape[0] - 1
    b = np.empty(M, complex)
    for k in range(M // 2 + 1):
        e = X[k] + np.conj(X[M - k])
        o = (X[k] - np.conj(X[M - k])) * np.conj(twx[k])
        b[k] = complex(e.real - o.imag, e.imag + o.real)
        if 0 < k < M // 2:
            b[M - k] = complex(e.real + o.imag, o.real - e.imag)
    return b


def test_radix5_last_pass_decomposition_matches_irfft():
    M = 5000
    Nx = 2 * M
    twx = np.exp(-2j * np.pi * np.arange(Nx) / Nx)
    x = np.random.default_rng(7).lognormal(0.0, 0.5, Nx)
    X = np.fft.rfft(x)
    z = radix5_levels(c2r_input_pairs(X, twx), twx)
    row = np.empty(Nx)
    row[0::2], row[1::2] = z.real, z.imag
    np.testing.assert_allclose(row, Nx * x, rtol=0, atol=1e-9 * Nx * np.abs(x).sum())


def test_c2r_input_pairs_equal_direct_form():
    M = 5000
    Nx = 2 * M
    twx = np.exp(-2j * np.pi * np.arange(Nx) / Nx)
    X = np.fft.rfft(np.random.default_rng(8).lognormal(0.0, 0.5, Nx))
    k = np.arange(M)
    xk, xm = X[k], np.conj(X[M - k])
    direct = (xk + xm) + 1j * (xk - xm) * np.conj(twx[k])
    np.testing.assert_allclose(c2r_input_pairs(X, twx), direct, rtol=0, atol=1e-9 * np.abs(X).max())


def test_radix5_forward_rows_match_rfft():
    """k_rows_r2c5: the forward five-level transform of the row's pairs, then the split."""
    M = 5000
    Nx = 2 * M
    twx = np.exp(-2j * np.pi * np.arange(Nx) / Nx)
    x = np.random.default_rng(9).lognormal(0.0, 0.5, Nx)
    Z = radix5_levels(x[0::2] + 1j * x[1::2], twx, inv=False)
    X = r2c_split(Z, twx)
    np.testing.assert_allclose(X, np.fft.rfft(x), rtol=0, atol=1e-9 * np.abs(x).sum())


def test_winograd_dft5_matches_fft():
    """Dft<T, 5>: the cosine part as u +/- m, u = x0 - (sa + sb)/4, m = sqrt(5)/4 (sa - sb)."""
    rng = np.random.default_rng(10)
    for inv in (False, True):
        x = rng.normal(size=5) + 1j * rng.normal(size=5)
        s1, s2 = np.sin(2 * np.pi / 5), np.sin(4 * np.pi / 5)
        b = (np.cos(2 * np.pi / 5) - np.cos(4 * np.pi / 5)) / 2
        sa, da, sb, db = x[1] + x[4], x[1] - x[4], x[2] + x[3], x[2] - x[3]
        t1, t2 = sa + sb, sa - sb
        u = x[0] - t1 / 4
        m = b * t2
        p1, p2 = u + m, u - m
        q1, q2 = s1 * da + s2 * db, s2 * da - s1 * db
        iq1, iq2 = (1j * q1, 1j * q2) if inv else (-1j * q1, -1j * q2)
        got = np.array([x[0] + t1, p1 + iq1, p2 + iq2, p2 - iq2, p1 - iq1])
        np.testing.assert_allclose(got, _dft(x, inv), rtol=0, atol=1e-12)


def test_prime_factor_dft10_matches_fft():
    """Dft<T, 10>: DFT2 over x[(5 n1 + 2 n2) mod 10], DFT5 over n2, X[(5 k1 + 6 k2) mod 10]."""
    x = np.random.default_rng(3).normal(size=10) + 1j * np.random.default_rng(4).normal(size=10)
    for inv in (False, True):
        a = np.array([x[(2 * n2) % 10] + x[(5 + 2 * n2) % 10] for n2 in range(5)])
        b = np.array([x[(2 * n2) % 10] - x[(5 + 2 * n2) % 10] for n2 in range(5)])
        A, B = _dft(a, inv), _dft(b, inv)
        X = np.empty(10, complex)
        for k2 in range(5):
            X[(6 * k2) % 10], X[(5 + 6 * k2) % 10] = A[k2], B[k2]
        np.testing.assert_allclose(X, _dft(x, inv), rtol=0, atol=1e-12)


def _profile_rows(prof, Ny, Nx):
    """ProfileRows: the 2h non-zero rows of the wrapped kernel, compacted (rows j < h are
    kernel rows j, rows j >= h kernel rows Ny - 2h + j), columns wrapped the same way."""
    N = prof.shape[0]
    h = N // 2
    rows = np.zeros((2 * h, Nx))
    for j in range(2 * h):
        pr = h + j if j < h else j - h
        rows[j, :h] = prof[pr, h:]
        rows[j, Nx - h:] = prof[pr, :h]
    return rows


def fused_convolution(mp, prof, N1, N2):
    """P0-P3 of the fused convolution in the kernels' order, with the spectrum rows in the
    digit-transposed order (row k1 N2 + k2 holds column frequency k1 + N1 k2)."""
    Ny, Nx = mp.shape
    assert Ny == N1 * N2
    Wy = lambda e: np.exp(-2j * np.pi * np.asarray(e) / Ny)
    h = prof.shape[0] // 2
    # map forward: rows, column pass A (length N1 over rows n1 N2 + n2, twiddle W^(n2 k1)),
    # column pass B (length N2 over the block of k1)
    R = np.fft.rfft(mp, axis=1)
    spec = np.empty_like(R)
    for n2 in range(N2):
        a = np.fft.fft(R[n2::N2], axis=0)  # rows n1 N2 + n2, n1 < N1 -> k1
        spec[n2::N2] = a * Wy(n2 * np.arange(N1))[:, None]
    for k1 in range(N1):
        spec[k1 * N2:(k1 + 1) * N2] = np.fft.fft(spec[k1 * N2:(k1 + 1) * N2], axis=0)
    # P0: the profile's 2h rows
    kx = np.fft.rfft(_profile_rows(prof, Ny, Nx), axis=1)
    out = np.empty_like(spec)
    W1 = lambda e: np.exp(-2j * np.pi * np.asarray(e) / N1)
    for kk in range(N1):
        # P1, profile column sub-pass A at k1 = kk restricted to the non-zero rows
        a = np.zeros((N2, kx.shape[1]), complex)
        if h <= N2:  # the kernels' two-term form: low row n2 < h (weight 1), high row n2 >= N2 - h
            for n2 in range(N2):
                if n2 < h:
                    a[n2] += kx[n2]
                if n2 >= N2 - h:
                    a[n2] += kx[n2 - (N2 - h) + h] * W1((N1 - 1) * kk)
        else:
            for j in range(2 * h):
                r = j if j < h else Ny - 2 * h + j  # kernel row
                a[r % N2] += kx[j] * W1((r // N2) * kk)
        a *= Wy(np.arange(N2) * kk)[:, None]
        K = np.fft.fft(a, axis=0)  # k2
        P = K * spec[kk * N2:(kk + 1) * N2] / (Nx * Ny)
        out[kk * N2:(kk + 1) * N2] = np.fft.ifft(P, axis=0) * N2 * np.conj(Wy(np.arange(N2) * kk))[:, None]
    # P2: inverse column pass A (length N1 over k1 -> n1) per n2; P3: inverse rows
    col = np.empty_like(out)
    for n2 in range(N2):
        col[n2::N2] = np.fft.ifft(out[n2::N2], axis=0) * N1
    return np.fft.irfft(col, n=Nx, axis=1) * Nx


@pytest.mark.parametrize("N", [6, 22])  # h = 3 <= N2 (two-term form) and h = 11 > N2 (general)
def test_fused_convolution_decomposition_matches_oracle(N):
    import oracle
    N1, N2, Nx = 4, 10, 24
    rng = np.random.default_rng(N)
    mp = rng.lognormal(0.0, 0.5, (N1 * N2, Nx))
    prof = rng.random((N, N))
    prof /= prof.sum()
    got = fused_convolution(mp, prof, N1, N2)
    ref = oracle.conv_fft(mp, prof)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)
