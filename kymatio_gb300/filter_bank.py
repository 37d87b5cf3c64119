"""Host-side construction of the Fourier-domain filter banks.

2-D: Morlet wavelets and the Gaussian low-pass of
kymatio/scattering2d/filter_bank.py:5-175.  Each filter is the sum of 5x5
periodic images of a (rotated, slanted) Gabor built in space, accumulated
in complex64 as the reference does, moved to Fourier with a complex64 FFT,
real part kept, then cropped to coarser resolutions by the masked alias sum
of periodize_filter_fft (accumulated block by block in the reference's
order, so the float32 values match the reference bit for bit).

1-D: Morlet/Gauss filters built in Fourier (kymatio/scattering1d/
filter_bank.py:51-102) on the Anden generator's (xi, sigma) pairs
(:254-311), with alias-summed lower resolutions (:322-404), plus the
padding/border logic of ScatteringBase1D.build (kymatio/scattering1d/
frontend/base_frontend.py:37-98).

Banks are cached per geometry for the life of the process.
"""
import functools
import math

import numpy as np
import scipy.fft

# ---------------------------------------------------------------------------
# 2-D
# ---------------------------------------------------------------------------


def _gabor_2d(M, N, sigma, theta, xi, slant=1.0):
    c, s = np.cos(theta), np.sin(theta)
    R = np.array([[c, -s], [s, c]], np.float32)
    Rinv = np.array([[c, s], [-s, c]], np.float32)
    curv = R @ (np.array([[1, 0], [0, slant * slant]]) @ Rinv) / (2 * sigma * sigma)
    cxx, cxy, cyy = curv[0, 0], curv[0, 1] + curv[1, 0], curv[1, 1]
    out = np.zeros((M, N), np.complex64)
    base_x = np.arange(M)[:, None]
    base_y = np.arange(N)[None, :]
    for ex in (-2, -1, 0, 1, 2):
        xx = np.broadcast_to(base_x + ex * M, (M, N))
        for ey in (-2, -1, 0, 1, 2):
            yy = np.broadcast_to(base_y + ey * N, (M, N))
            out += np.exp(-(cxx * (xx * xx) + cxy * (xx * yy) + cyy * (yy * yy))
                          + 1.j * (xx * xi * np.cos(theta) + yy * xi * np.sin(theta)))
    out /= (2 * 3.1415 * sigma * sigma / slant)
    return out


def _morlet_2d(M, N, sigma, theta, xi, slant):
    g = _gabor_2d(M, N, sigma, theta, xi, slant)
    e = _gabor_2d(M, N, sigma, theta, 0, slant)
    return g - (np.sum(g) / np.sum(e)) * e


def _crop_2d(h, res):
    """Masked alias sum to resolution 2^-res (periodize_filter_fft)."""
    M, N = h.shape
    k = 2 ** res
    keep = np.ones((M, N), np.float32)
    sx, lx = int(M * 2 ** (-res - 1)), int(M * (1 - 2 ** (-res)))
    sy, ly = int(N * 2 ** (-res - 1)), int(N * (1 - 2 ** (-res)))
    keep[sx:sx + lx, :] = 0
    keep[:, sy:sy + ly] = 0
    h = h * keep
    mr, nr = M // k, N // k
    out = np.zeros((mr, nr), h.dtype)
    blocks = h.reshape(k, mr, k, nr)
    for i in range(k):
        for j in range(k):
            out += blocks[i, :, j, :]
    return out


@functools.lru_cache(maxsize=16)
def filter_bank_2d(M, N, J, L=8):
    """Returns (phi_levels, psi) with psi a tuple of dicts {j, theta, levels}."""
    psi = []
    for j in range(J):
        for t in range(L):
            w = _morlet_2d(M, N, 0.8 * 2 ** j, (int(L - L / 2 - 1) - t) * np.pi / L,
                           3.0 / 4.0 * np.pi / 2 ** j, 4.0 / L)
            wf = np.real(scipy.fft.fft2(w))
            nlev = min(j + 1, max(J - 1, 1))
            psi.append({'j': j, 'theta': t, 'levels': tuple(_crop_2d(wf, r) for r in range(nlev))})
    pf = np.real(scipy.fft.fft2(_gabor_2d(M, N, 0.8 * 2 ** (J - 1), 0, 0)))
    phi = tuple(_crop_2d(pf, r) for r in range(J))
    for lv in phi:
        lv.setflags(write=False)
    for p in psi:
        for lv in p['levels']:
            lv.setflags(write=False)
    return phi, tuple(psi)


def filter_bank_2d_device(M, N, J, L=8, device=None):
    """The bank of filter_bank_2d built on a CUDA device (kym_s2d_filter_bank:
    FP64 Gabor sums, DFT and alias crops on the GPU, rounded once to
    float32), in milliseconds instead of the host build's seconds at large
    sizes.  Returns (phi_levels, psi) like filter_bank_2d, with float32 CUDA
    tensors; the values agree with the reference's complex64 build to float32
    rounding, not bit for bit."""
    import torch
    from . import _lib
    lib = _lib.load()
    dev = torch.device('cuda', torch.cuda.current_device()) if device is None else torch.device(device)
    n = lib.kym_s2d_filter_bank_floats(M, N, J, L)
    if n <= 0:
        raise ValueError('unsupported filter-bank geometry %r' % ((M, N, J, L),))
    with torch.cuda.device(dev):
        out = torch.empty(int(n), dtype=torch.float32, device=dev)
        wsb = lib.kym_s2d_filter_bank_workspace_bytes(M, N, J, L)
        ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
        _lib.check(lib.kym_s2d_filter_bank(M, N, J, L, out.data_ptr(), n, ws.data_ptr(), wsb,
                                           torch.cuda.current_stream(dev).cuda_stream), 'kym_s2d_filter_bank')
        torch.cuda.current_stream(dev).synchronize()  # the workspace is released on return
    off = 0

    def take(lev):
        nonlocal off
        m, k = M >> lev, N >> lev
        t = out[off:off + m * k].view(m, k)
        off += m * k
        return t
    phi = tuple(take(r) for r in range(J))
    psi = []
    for j in range(J):
        for t in range(L):
            nlev = min(j + 1, max(J - 1, 1))
            psi.append({'j': j, 'theta': t, 'levels': tuple(take(r) for r in range(nlev))})
    assert off == n
    return phi, tuple(psi)


def padded_size_2d(M, N, J):
    """kymatio/scattering2d/utils.py:4-24."""
    return ((M + 2 ** J) // 2 ** J + 1) * 2 ** J, ((N + 2 ** J) // 2 ** J + 1) * 2 ** J


# ---------------------------------------------------------------------------
# 1-D
# ---------------------------------------------------------------------------

R_PSI = math.sqrt(0.5)
SIGMA0 = 0.1
ALPHA = 5.


def _periods(sigma, eps=1e-7):
    return int(math.ceil(math.sqrt(-2 * sigma ** 2 * math.log(eps)) + 1))


def morlet_1d(N, xi, sigma):
    """Fourier-domain Morlet (xi > 0) or Gaussian (xi falsy), L1-normalised."""
    P = min(_periods(sigma), 5)
    f = np.arange((1 - P) * N, P * N, dtype=float) / float(N)
    fl = np.fft.fftfreq(N) if P == 1 else f
    low = np.exp(-(fl ** 2) / (2 * sigma ** 2)).reshape(2 * P - 1, -1).mean(axis=0)
    if xi:
        gab = np.exp(-(f - xi) ** 2 / (2 * sigma ** 2)).reshape(2 * P - 1, -1).mean(axis=0)
        h = gab - (gab[0] / low[0]) * low
    else:
        h = low
    return h / np.abs(scipy.fft.ifft(h)).sum()


def _sigma_psi(xi, Q, r=R_PSI):
    f = 1. / math.pow(2, 1. / Q)
    return xi * (1 - f) / (1 + f) / math.sqrt(2 * math.log(1. / r))


def _max_subsampling(xi, sigma):
    return int(math.floor(-math.log2(min(abs(xi) + ALPHA * sigma, 0.5))) - 1)


def anden_pairs(J, Q):
    """(xi, sigma) pairs of the Anden/ScatNet generator."""
    pairs = []
    xi = max(1. / (1. + math.pow(2., 3. / Q)), 0.35)
    sigma = _sigma_psi(xi, Q)
    smin = SIGMA0 / 2 ** J
    if sigma <= smin:
        xi = sigma
    else:
        pairs.append((xi, sigma))
        step = math.pow(2, 1 / Q)
        while sigma > smin * step:
            xi /= step
            sigma /= step
            pairs.append((xi, sigma))
    elbow = xi
    for _ in range(Q - 1):
        xi -= 1 / Q * elbow
        pairs.append((xi, smin))
    return pairs


def temporal_support(h_f, criterion_amplitude=1e-3):
    h = scipy.fft.ifft(h_f, axis=1)
    half = h.shape[1] // 2
    resid = np.cumsum(np.abs(h)[:, :half][:, ::-1], axis=1)[:, ::-1]
    ok = np.max(resid, axis=0) <= criterion_amplitude
    if np.any(ok):
        return int(np.argmax(ok) + 1)
    return half


@functools.lru_cache(maxsize=16)
def filter_bank_1d(N_padded, J, Q, T):
    """Returns (phi, psi1, psi2): dicts with levels (float64 arrays), xi, sigma, j."""
    log2_T = math.floor(math.log2(T))
    banks = []
    max_j = prev_J = 0
    for q in Q:
        bank = []
        for xi, sigma in anden_pairs(J, q):
            lv0 = morlet_1d(N_padded, xi, sigma)
            j = _max_subsampling(xi, sigma)
            levels = [lv0] + [lv0.reshape(2 ** l, -1).sum(axis=0)
                              for l in range(1, min(prev_J, j, 1 + log2_T))]
            bank.append({'levels': tuple(levels), 'xi': xi, 'sigma': sigma, 'j': j})
            max_j = max(j, max_j)
        prev_J = max_j
        banks.append(tuple(bank))
    sl = SIGMA0 / T
    p0 = morlet_1d(N_padded, None, sl)
    phi = {'levels': tuple([p0] + [p0.reshape(2 ** l, -1).sum(axis=0)
                                   for l in range(1, max(prev_J, 1 + log2_T))]),
           'xi': 0, 'sigma': sl, 'j': log2_T, 'N': N_padded}
    return (phi,) + tuple(banks)


@functools.lru_cache(maxsize=16)
def filter_bank_fr(N_fr, J_fr, Q_fr, F):
    """Frequency-axis filters of joint time-frequency scattering
    (kymatio/scattering1d/frontend/base_frontend.py:570-579): returns
    (phi_F, psis) where phi_F averages over F first-order channels and psis
    is [phi_{2^J_fr}] followed by the Anden wavelets of (J_fr, Q_fr) with
    positive center frequency, then the same wavelets mirrored to negative
    frequency (the "spin" down; kymatio/scattering1d/filter_bank.py:314-319).
    Levels are alias sums, as for the time filters."""
    def lowpass(T, n_levels):
        sigma = SIGMA0 / T
        p0 = morlet_1d(N_fr, None, sigma)
        levels = [p0] + [p0.reshape(2 ** l, -1).sum(axis=0) for l in range(1, n_levels)]
        return {'levels': tuple(levels), 'xi': 0, 'sigma': sigma, 'j': int(math.floor(math.log2(T))), 'N': N_fr}

    phi_F = lowpass(F, max(0, 1 + int(math.floor(math.log2(F)))))
    pairs = anden_pairs(J_fr, Q_fr)
    psis, max_j = [], 0
    for xi, sigma in pairs + [(-xi, sigma) for xi, sigma in pairs]:
        j = _max_subsampling(xi, sigma)
        psis.append({'levels': (morlet_1d(N_fr, xi, sigma),), 'xi': xi, 'sigma': sigma, 'j': j})
        max_j = max(max_j, j)
    phi_J = lowpass(2 ** J_fr, max(max_j, 1 + J_fr))
    return phi_F, (phi_J,) + tuple(psis)


def geometry_1d(J, N_input, T):
    """Padding of ScatteringBase1D.build: (N_padded, pad_left, pad_right)."""
    phi_f = morlet_1d(N_input, None, SIGMA0 / T)
    min_to_pad = 3 * temporal_support(phi_f.reshape(1, -1), criterion_amplitude=1e-3)
    J_max = int(np.floor(np.log2(3 * N_input - 2)))
    J_pad = min(int(np.ceil(np.log2(N_input + 2 * min_to_pad))), J_max)
    N_padded = 2 ** J_pad
    to_add = N_padded - N_input
    left = to_add // 2
    right = to_add - left
    if max(left, right) >= N_input:
        raise ValueError('Too large padding value, will lead to NaN errors')
    return N_padded, left, right


def border_indices(log2_T, J, i0, i1):
    start, end = {0: i0}, {0: i1}
    for j in range(1, max(log2_T, J) + 1):
        start[j] = start[j - 1] // 2 + start[j - 1] % 2
        end[j] = end[j - 1] // 2 + end[j - 1] % 2
    return start, end


# ---------------------------------------------------------------------------
# Separable low-pass factors (tensor-core form)
# ---------------------------------------------------------------------------

def separable_lowpass(phi_level, out_r0, out_nr, out_c0, out_nc, ks_r, ks_c):
    """Factors T_r (out_nr x m_r), T_c (out_nc x m_c) with

        unpad(Re IFFT2_s(fold_ks(FFT2_m(U) * phi_level))) = T_r U T_c^T

    for real U.  phi_level (real, m_r x m_c) is the periodised Gaussian of the
    bank, a rank-one outer product u v^T up to float32 rounding (FP64 SVD);
    T_r[p, x] = h_u[((p + out_r0) ks_r - x) mod m_r] with h_u = IFFT(u).
    Returns (T_r, T_c, relative residual of the rank-one fit)."""
    f = np.asarray(phi_level, np.float64)
    U, s, Vt = np.linalg.svd(f)
    u, v = U[:, 0] * np.sqrt(s[0]), Vt[0] * np.sqrt(s[0])
    if u.sum() < 0:
        u, v = -u, -v
    resid = float(np.linalg.norm(f - np.outer(u, v)) / np.linalg.norm(f))
    hu, hv = np.fft.ifft(u).real, np.fft.ifft(v).real
    mr, mc = f.shape
    P = np.arange(out_r0, out_r0 + out_nr)[:, None]
    Q = np.arange(out_c0, out_c0 + out_nc)[:, None]
    Tr = hu[(P * ks_r - np.arange(mr)[None, :]) % mr]
    Tc = hv[(Q * ks_c - np.arange(mc)[None, :]) % mc]
    return Tr, Tc, resid
