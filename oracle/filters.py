"""Oracle restatement of kymatio's filter banks (test infrastructure only).

2-D: kymatio/scattering2d/filter_bank.py:5-175 -- Morlet wavelets and the
Gaussian low-pass built in space as sums of 5x5 periodic Gabor images in
complex64, transformed with scipy.fft.fft2, real part kept, then cropped to
coarser resolutions by a masked alias sum.  The dtypes (float32 rotation
matrices, complex64 accumulation, float32 crops) follow the reference so
that the bank is reproduced value for value.

1-D: kymatio/scattering1d/filter_bank.py:6-404 -- Morlet/Gauss filters built
directly in Fourier with P-period folding, the Anden (ScatNet) generator of
(xi, sigma) pairs, and alias-summed lower resolutions.
"""
import math

import numpy as np
import scipy.fft


# --------------------------------------------------------------------------
# 2-D bank
# --------------------------------------------------------------------------

def gabor_2d(M, N, sigma, theta, xi, slant=1.0, offset=0):
    """kymatio/scattering2d/filter_bank.py:132-175 (complex64 accumulation)."""
    c, s = np.cos(theta), np.sin(theta)
    rot = np.array([[c, -s], [s, c]], np.float32)
    rot_inv = np.array([[c, s], [-s, c]], np.float32)
    dmat = np.array([[1, 0], [0, slant * slant]])
    curv = np.dot(rot, np.dot(dmat, rot_inv)) / (2 * sigma * sigma)
    acc = np.zeros((M, N), np.complex64)
    for ex in (-2, -1, 0, 1, 2):
        for ey in (-2, -1, 0, 1, 2):
            xx, yy = np.mgrid[offset + ex * M:offset + M + ex * M,
                              offset + ey * N:offset + N + ey * N]
            arg = (-(curv[0, 0] * xx * xx + (curv[0, 1] + curv[1, 0]) * xx * yy
                     + curv[1, 1] * yy * yy)
                   + 1j * (xx * xi * np.cos(theta) + yy * xi * np.sin(theta)))
            acc += np.exp(arg)
    acc /= (2 * 3.1415 * sigma * sigma / slant)
    return acc


def morlet_2d(M, N, sigma, theta, xi, slant=0.5, offset=0):
    """kymatio/scattering2d/filter_bank.py:94-129: Gabor minus K x envelope."""
    wave = gabor_2d(M, N, sigma, theta, xi, slant, offset)
    env = gabor_2d(M, N, sigma, theta, 0, slant, offset)
    kappa = np.sum(wave) / np.sum(env)
    return wave - kappa * env


def periodize_filter_fft(h, res):
    """kymatio/scattering2d/filter_bank.py:56-91.

    Zero the band of frequencies that does not survive the crop, then sum the
    2^res x 2^res aliases.  The block loop adds in the same (i outer, j inner)
    order as the reference's per-element loop, so float32 sums match.
    """
    M, N = h.shape
    k = 2 ** res
    mask = np.ones(h.shape, np.float32)
    len_x, start_x = int(M * (1 - 2 ** (-res))), int(M * 2 ** (-res - 1))
    len_y, start_y = int(N * (1 - 2 ** (-res))), int(N * 2 ** (-res - 1))
    mask[start_x:start_x + len_x, :] = 0
    mask[:, start_y:start_y + len_y] = 0
    h = np.multiply(h, mask)
    mc, nc = int(M / k), int(N / k)
    crop = np.zeros((M // k, N // k), h.dtype)
    for i in range(k):
        for j in range(k):
            crop += h[i * mc:i * mc + M // k, j * nc:j * nc + N // k]
    return crop


def filter_bank_2d(M, N, J, L=8):
    """kymatio/scattering2d/filter_bank.py:5-53.

    Returns {'phi': {'levels', 'j'}, 'psi': [{'levels', 'j', 'theta'}]} with
    float32 Fourier-domain filters (the imaginary part is dropped).
    """
    psi = []
    for j in range(J):
        for theta in range(L):
            wav = morlet_2d(M, N, 0.8 * 2 ** j, (int(L - L / 2 - 1) - theta) * np.pi / L,
                            3.0 / 4.0 * np.pi / 2 ** j, 4.0 / L)
            wav_f = np.real(scipy.fft.fft2(wav))
            levels = [periodize_filter_fft(wav_f, r) for r in range(min(j + 1, max(J - 1, 1)))]
            psi.append({'levels': levels, 'j': j, 'theta': theta})
    phi_f = np.real(scipy.fft.fft2(gabor_2d(M, N, 0.8 * 2 ** (J - 1), 0, 0)))
    phi = {'levels': [periodize_filter_fft(phi_f, r) for r in range(J)], 'j': J}
    return {'phi': phi, 'psi': psi}


def compute_padding_2d(M, N, J):
    """kymatio/scattering2d/utils.py:4-24."""
    return ((M + 2 ** J) // 2 ** J + 1) * 2 ** J, ((N + 2 ** J) // 2 ** J + 1) * 2 ** J


# --------------------------------------------------------------------------
# 1-D bank
# --------------------------------------------------------------------------

def adaptive_choice_P(sigma, eps=1e-7):
    """kymatio/scattering1d/filter_bank.py:6-48."""
    return int(math.ceil(math.sqrt(-2 * sigma ** 2 * math.log(eps)) + 1))


def morlet_1d(N, xi, sigma):
    """kymatio/scattering1d/filter_bank.py:51-98 (float64, L1-normalised)."""
    P = min(adaptive_choice_P(sigma), 5)
    freqs = np.arange((1 - P) * N, P * N, dtype=float) / float(N)
    freqs_low = np.fft.fftfreq(N) if P == 1 else freqs
    low = np.exp(-(freqs_low ** 2) / (2 * sigma ** 2)).reshape(2 * P - 1, -1).mean(axis=0)
    if xi:
        gab = np.exp(-(freqs - xi) ** 2 / (2 * sigma ** 2)).reshape(2 * P - 1, -1).mean(axis=0)
        h = gab - (gab[0] / low[0]) * low
    else:
        h = low
    h /= np.abs(scipy.fft.ifft(h)).sum()
    return h


def gauss_1d(N, sigma):
    """kymatio/scattering1d/filter_bank.py:101-102."""
    return morlet_1d(N, None, sigma)


def compute_sigma_psi(xi, Q, r=math.sqrt(0.5)):
    """kymatio/scattering1d/filter_bank.py:105-139."""
    f = 1. / math.pow(2, 1. / Q)
    return xi * (1 - f) / (1 + f) / math.sqrt(2 * math.log(1. / r))


def compute_temporal_support(h_f, criterion_amplitude=1e-3):
    """kymatio/scattering1d/filter_bank.py:142-196."""
    h = scipy.fft.ifft(h_f, axis=1)
    half = h.shape[1] // 2
    resid = np.fliplr(np.cumsum(np.fliplr(np.abs(h)[:, :half]), axis=1))
    ok = np.max(resid, axis=0) <= criterion_amplitude
    if np.any(ok):
        return int(np.min(np.where(ok)[0]) + 1)
    return half


def get_max_dyadic_subsampling(xi, sigma, alpha, **unused):
    """kymatio/scattering1d/filter_bank.py:199-233."""
    upper = min(abs(xi) + alpha * sigma, 0.5)
    return int(math.floor(-math.log2(upper)) - 1)


def compute_xi_max(Q):
    """kymatio/scattering1d/filter_bank.py:236-251."""
    return max(1. / (1. + math.pow(2., 3. / Q)), 0.35)


def anden_generator(J, Q, sigma0, r_psi, **unused):
    """kymatio/scattering1d/filter_bank.py:254-311: (xi, sigma) pairs."""
    out = []
    xi = compute_xi_max(Q)
    sigma = compute_sigma_psi(xi, Q, r=r_psi)
    sigma_min = sigma0 / 2 ** J
    if sigma <= sigma_min:
        xi = sigma
    else:
        out.append((xi, sigma))
        while sigma > sigma_min * math.pow(2, 1 / Q):
            xi /= math.pow(2, 1 / Q)
            sigma /= math.pow(2, 1 / Q)
            out.append((xi, sigma))
    elbow = xi
    for _ in range(Q - 1):
        xi -= 1 / Q * elbow
        out.append((xi, sigma_min))
    return out


def scattering_filter_factory_1d(N, J, Q, T, alpha=5., r_psi=math.sqrt(0.5), sigma0=0.1):
    """kymatio/scattering1d/filter_bank.py:322-404 with np.sum level reduction
    (kymatio/scattering1d/frontend/base_frontend.py:35)."""
    log2_T = math.floor(math.log2(T))
    max_j, previous_J = 0, 0
    banks = []
    for q in Q:
        bank = []
        for xi, sigma in anden_generator(J, q, sigma0=sigma0, r_psi=r_psi):
            levels = [morlet_1d(N, xi, sigma)]
            j = get_max_dyadic_subsampling(xi, sigma, alpha)
            for level in range(1, min(previous_J, j, 1 + log2_T)):
                levels.append(levels[0].reshape(2 ** level, -1).sum(axis=0))
            bank.append({'levels': levels, 'xi': xi, 'sigma': sigma, 'j': j})
            max_j = max(j, max_j)
        previous_J = max_j
        banks.append(bank)
    sigma_low = sigma0 / T
    levels = [gauss_1d(N, sigma_low)]
    for level in range(1, max(previous_J, 1 + log2_T)):
        levels.append(levels[0].reshape(2 ** level, -1).sum(axis=0))
    phi = {'levels': levels, 'xi': 0, 'sigma': sigma_low, 'j': log2_T, 'N': N}
    return (phi, *banks)
