"""Precision budget of the stored order-1 modulus U1 (oracle only, CPU).

The order-2 paths read U1 (as its spectrum) after the order-1 pass.  Storing
it in FP16 with a per-channel (per image and path) scale, as a bandwidth
saving, costs about 1e-4 relative L2 on S2 at 256x256 J=3, twice the 5e-5
budget of the tensor-core form; rounding it to FP32 costs about 1e-8.  This
is why the engine keeps U1's spectrum in FP32 (it stays L2-resident between
the two passes, so FP16 would save little HBM traffic anyway)."""
import numpy as np

from conftest import rel_l2
from oracle.scattering2d import (Scattering2D, cdgmm, ifft, irfft, modulus, pad, rfft,
                                 subsample_fourier, unpad)


def _grf(seed):
    """One 256x256 Gaussian random field rescaled to [0, 1] (sigma 2.5 px)."""
    import scipy.ndimage
    w = np.random.default_rng(seed).standard_normal((256, 256))
    f = scipy.ndimage.gaussian_filter(w, 2.5, mode='wrap')
    return ((f - f.min()) / (f.max() - f.min()))[None]


def _round(a, dtype):
    s = np.max(np.abs(a), axis=(-2, -1), keepdims=True) / 16384.0
    return (a / s).astype(dtype).astype(np.float64) * s


def _order2(x, store):
    S = Scattering2D(3, (256, 256))
    U0 = rfft(pad(x, S.pad_size))
    out = []
    for p1 in S.psi:
        j1 = p1['j']
        U1c = cdgmm(U0, p1['levels'][0])
        if j1 > 0:
            U1c = subsample_fourier(U1c, 2 ** j1)
        U1c = rfft(store(modulus(ifft(U1c))))
        for p2 in S.psi:
            j2 = p2['j']
            if j2 <= j1:
                continue
            U2 = subsample_fourier(cdgmm(U1c, p2['levels'][j1]), 2 ** (j2 - j1))
            U2 = rfft(modulus(ifft(U2)))
            out.append(unpad(irfft(subsample_fourier(cdgmm(U2, S.phi['levels'][j2]), 2 ** (3 - j2)))))
    return np.stack(out, -3)


def test_fp16_u1_exceeds_the_tensor_core_budget():
    x = _grf(2)
    ref = _order2(x, lambda u: u)
    e16 = rel_l2(_order2(x, lambda u: _round(u, np.float16)), ref)
    e32 = rel_l2(_order2(x, lambda u: _round(u, np.float32)), ref)
    assert e16 > 5e-5, e16
    assert e32 < 1e-6, e32
