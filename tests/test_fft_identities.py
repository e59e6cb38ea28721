"""The transform identities the spectral kernels rely on, checked in numpy
(CPU): the half-shifted decimation-in-time FFT with tangent-form twiddles
(fft.cuh's butterflies and table layout restated), the half-shifted
four-step split, and the mirror-pair identities of the real-transform pack
and unpack steps."""
import numpy as np
import pytest


def _tangent(t, N, code=None):
    w = np.exp(-2j * np.pi * (t % N) / N)
    vx = [w.real, -w.imag, -w.real, w.imag]
    vy = [w.imag, w.real, -w.imag, -w.real]
    if code is None:
        code = int(np.argmax(vx))
    return code, vx[code], vy[code] / vx[code]


def _rot(z, code):   # R z for R = 1, -i, -1, i
    x, y = (z.imag, z.real) if code & 1 else (z.real, z.imag)
    if code >> 1:
        x = -x
    if code in (1, 2):
        y = -y
    return complex(x, y)


def _tanmul(z, code, tau):
    v = _rot(z, code)
    return complex(v.real - tau * v.imag, v.imag + tau * v.real)


def _bitrev(v, L):
    return int(format(v, f"0{L}b")[::-1], 2) if L else 0


def _dit(xin, logM, sigma):
    """Radix-4 DIT over bit-reversed input, one radix-2 pass for odd log2 M,
    twiddles w^(j + sigma/2) in tangent form (sigma = 0: the plain transform;
    the first pass then has unit twiddles)."""
    m = 1 if sigma == 0 else 2
    M = 1 << logM
    x = [xin[_bitrev(i, logM)] for i in range(M)]
    s = 0
    while s + 1 < logM:
        h = 1 << s
        for b in range(M >> 2):
            j = b & (h - 1)
            i = ((b >> s) << (s + 2)) + j
            a, bq, c, d = x[i], x[i + h], x[i + 2 * h], x[i + 3 * h]
            t = m * j + sigma
            c1, r1, t1 = _tangent(t, m * 4 * h)
            c2, r2, t2 = _tangent(2 * t, m * 4 * h)
            c3, r3, t3 = _tangent(3 * t, m * 4 * h)
            uc, ub, ud = _tanmul(c, c1, t1), _tanmul(bq, c2, t2), _tanmul(d, c3, t3)
            rho = r3 / r1
            s0, d0 = a + r2 * ub, a - r2 * ub
            e, f = uc + rho * ud, uc - rho * ud
            x[i], x[i + 2 * h] = s0 + r1 * e, s0 - r1 * e
            x[i + h], x[i + 3 * h] = d0 - 1j * r1 * f, d0 + 1j * r1 * f
        s += 2
    if s < logM:
        h = 1 << s
        for b in range(M >> 1):
            j = b & (h - 1)
            i = ((b >> s) << (s + 1)) + j
            c, r, tau = _tangent(m * j + sigma, m * 2 * h)
            u = _tanmul(x[i + h], c, tau)
            x[i], x[i + h] = x[i] + r * u, x[i] - r * u
    return np.array(x)


@pytest.mark.parametrize("logM", [1, 2, 3, 6, 7])
@pytest.mark.parametrize("sigma", [0, 1, -1])
def test_half_shifted_dit(logM, sigma):
    M = 1 << logM
    z = np.random.default_rng(logM).standard_normal((M, 2)) @ np.array([1, 1j])
    ref = np.fft.fft(z * np.exp(-1j * np.pi * sigma * np.arange(M) / M))
    assert np.max(np.abs(_dit(z, logM, sigma) - ref)) < 1e-13 * np.max(np.abs(ref))


@pytest.mark.parametrize("logM", [9, 10])
@pytest.mark.parametrize("sigma", [1, -1])
def test_half_shifted_four_step(logM, sigma):
    """Columns n1 -> k1 half-shifted, twiddles W_M^(n2 (k1 + sigma/2)) (table
    index n2 (2 k1 + sigma) mod 2M), plain rows, output X[k1 + M1 k2]."""
    M = 1 << logM
    logM1 = (logM + 1) // 2
    M1, M2 = 1 << logM1, 1 << (logM - logM1)
    x = np.random.default_rng(logM).standard_normal((M, 2)) @ np.array([1, 1j])
    ref = np.fft.fft(x * np.exp(-1j * np.pi * sigma * np.arange(M) / M))
    X = x.reshape(M1, M2)
    k1 = np.arange(M1)
    C = np.exp(-2j * np.pi * np.outer(k1 + sigma / 2, np.arange(M1)) / M1) @ X
    t = np.outer(2 * k1 + sigma, np.arange(M2)) % (2 * M)
    R = np.fft.fft(C * np.exp(-2j * np.pi * t / (2 * M)), axis=1)
    out = np.empty(M, complex)
    for a in range(M1):
        out[a + M1 * np.arange(M2)] = R[a]
    assert np.max(np.abs(out - ref)) < 1e-12 * np.max(np.abs(ref))


def test_tan_code_rule():
    """The tangent copy of the plain table takes R from the index: the
    quarter turn nearest the angle, so |tau| <= 1 and r >= 1/sqrt 2."""
    logTW = 10
    N = 1 << logTW
    for t in range(N):
        code = ((8 * t + N - 1) >> (logTW + 1)) & 3
        _, r, tau = _tangent(t, N, code)
        assert abs(tau) <= 1 + 1e-15 and r >= np.sqrt(0.5) - 1e-15


def test_mirror_pair_unpack_and_pack():
    """Unpack: G[f] = (Ev + w Od)/2, G[h - f] = conj(Ev - w Od)/2 for the real
    transform of g from the half-size complex one of g[2t] + i g[2t+1].
    Pack: the inverse input of bin h - f is conj(E) + i conj(O) of bin f's."""
    N = 64
    h = N // 2
    g = np.random.default_rng(3).standard_normal(N)
    W = np.fft.fft(g[0::2] + 1j * g[1::2])
    G = np.fft.fft(g)
    for f in range(h // 2 + 1):
        Ev = W[f] + np.conj(W[(h - f) % h])
        Od = -1j * (W[f] - np.conj(W[(h - f) % h]))
        w = np.exp(-2j * np.pi * f / N)
        assert abs((Ev + w * Od) / 2 - G[f]) < 1e-12
        assert abs(np.conj(Ev - w * Od) / 2 - G[h - f]) < 1e-12
    C = np.fft.fft(np.random.default_rng(4).standard_normal(N))   # a real spectrum
    def U(f):
        E = C[f] + np.conj(C[h - f])
        O = (C[f] - np.conj(C[h - f])) * np.exp(2j * np.pi * f / N)
        return E, O
    for f in range(1, h // 2 + 1):
        E, O = U(f)
        Ec, Oc = U(h - f)
        assert abs((Ec + 1j * Oc) - (np.conj(E) + 1j * np.conj(O))) < 1e-12
