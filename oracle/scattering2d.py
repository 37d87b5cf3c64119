"""Oracle restatement of kymatio's 2-D scattering (test infrastructure only).

Follows the numpy backend (kymatio/scattering2d/backend/numpy_backend.py,
kymatio/backend/numpy_backend.py) and the depth-first cascade of
kymatio/scattering2d/core/scattering2d.py:1-88.  With float64 input every op
runs in FP64 (scipy.fft on complex128) against the float32 filter bank, which
is the FP64 oracle the GPU path is graded against.
"""
import numpy as np
import scipy.fft

from .filters import compute_padding_2d, filter_bank_2d


# ---- op surface (kymatio/scattering2d/backend/numpy_backend.py) ----------

def pad(x, pad_size):
    """numpy_backend.py:3-25: reflect pad [top, bottom, left, right]."""
    return np.pad(x, ((0, 0), (pad_size[0], pad_size[1]), (pad_size[2], pad_size[3])),
                  mode='reflect')


def unpad(x):
    """numpy_backend.py:31-45: drop one sample on every side."""
    return x[..., 1:-1, 1:-1]


def subsample_fourier(x, k):
    """numpy_backend.py:48-76: periodise (mean of k x k aliases)."""
    y = x.reshape(-1, k, x.shape[1] // k, k, x.shape[2] // k)
    return y.mean(axis=(1, 3))


def rfft(x):
    """numpy_backend.py:86-88."""
    return scipy.fft.fft2(x)


def ifft(x):
    """numpy_backend.py:95-99."""
    return scipy.fft.ifft2(x)


def irfft(x):
    """numpy_backend.py:90-93."""
    return scipy.fft.ifft2(x).real


def cdgmm(a, b):
    """kymatio/backend/numpy_backend.py:64-95 (real filter, broadcast)."""
    return a * b


def modulus(x):
    """kymatio/backend/numpy_backend.py:45-62."""
    return np.abs(x)


# ---- cascade (kymatio/scattering2d/core/scattering2d.py:1-88) -------------

def scattering2d_core(x, pad_fn, J, phi, psi, max_order, out_type='array'):
    """Depth-first cascade; returns (B, C, m, n) array or a list of dicts."""
    U_r = pad_fn(x)
    U_0_c = rfft(U_r)
    out0, out1, out2 = [], [], []
    s0 = unpad(irfft(subsample_fourier(cdgmm(U_0_c, phi['levels'][0]), 2 ** J)))
    out0.append({'coef': s0, 'j': (), 'n': (), 'theta': ()})
    for n1, p1 in enumerate(psi):
        j1, t1 = p1['j'], p1['theta']
        U_1_c = cdgmm(U_0_c, p1['levels'][0])
        if j1 > 0:
            U_1_c = subsample_fourier(U_1_c, 2 ** j1)
        U_1_c = rfft(modulus(ifft(U_1_c)))
        s1 = unpad(irfft(subsample_fourier(cdgmm(U_1_c, phi['levels'][j1]), 2 ** (J - j1))))
        out1.append({'coef': s1, 'j': (j1,), 'n': (n1,), 'theta': (t1,)})
        if max_order < 2:
            continue
        for n2, p2 in enumerate(psi):
            j2, t2 = p2['j'], p2['theta']
            if j2 <= j1:
                continue
            U_2_c = subsample_fourier(cdgmm(U_1_c, p2['levels'][j1]), 2 ** (j2 - j1))
            U_2_c = rfft(modulus(ifft(U_2_c)))
            s2 = unpad(irfft(subsample_fourier(cdgmm(U_2_c, phi['levels'][j2]), 2 ** (J - j2))))
            out2.append({'coef': s2, 'j': (j1, j2), 'n': (n1, n2), 'theta': (t1, t2)})
    out = out0 + out1 + out2
    if out_type == 'array':
        return np.stack([o['coef'] for o in out], axis=-3)
    return out


class Scattering2D:
    """Oracle counterpart of ScatteringNumPy2D
    (kymatio/scattering2d/frontend/numpy_frontend.py:6-58 and
    kymatio/scattering2d/frontend/base_frontend.py:19-36)."""

    def __init__(self, J, shape, L=8, max_order=2, pre_pad=False, out_type='array'):
        M, N = shape
        if 2 ** J > M or 2 ** J > N:
            raise RuntimeError('The smallest dimension should be larger than 2^J.')
        self.J, self.L, self.shape = J, L, (M, N)
        self.max_order, self.pre_pad, self.out_type = max_order, pre_pad, out_type
        self.M_padded, self.N_padded = compute_padding_2d(M, N, J)
        self.pad_size = [(self.M_padded - M) // 2, (self.M_padded - M + 1) // 2,
                         (self.N_padded - N) // 2, (self.N_padded - N + 1) // 2]
        bank = filter_bank_2d(self.M_padded, self.N_padded, J, L)
        self.phi, self.psi = bank['phi'], bank['psi']

    def __call__(self, x):
        x = np.asarray(x)
        batch_shape = x.shape[:-2]
        xb = x.reshape((-1,) + x.shape[-2:])
        pad_fn = (lambda v: v) if self.pre_pad else (lambda v: pad(v, self.pad_size))
        S = scattering2d_core(xb, pad_fn, self.J, self.phi, self.psi, self.max_order,
                              self.out_type)
        if self.out_type == 'array':
            return S.reshape(batch_shape + S.shape[-3:])
        for o in S:
            o['coef'] = o['coef'].reshape(batch_shape + o['coef'].shape[-2:])
        return S


def order_slices(J, L, max_order=2):
    """Channel ranges of orders 0, 1, 2 in the stacked output."""
    c1 = J * L
    c2 = L * L * J * (J - 1) // 2 if max_order >= 2 else 0
    return slice(0, 1), slice(1, 1 + c1), slice(1 + c1, 1 + c1 + c2)
