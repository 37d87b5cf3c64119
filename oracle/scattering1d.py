"""Oracle restatement of kymatio's 1-D scattering (test infrastructure only).

Follows kymatio/scattering1d/frontend/base_frontend.py:37-155 (padding,
border indices, pad -> cascade -> unpad -> sort -> stack),
kymatio/scattering1d/core/scattering1d.py:2-107 (the cascade) and the numpy
backend kymatio/scattering1d/backend/numpy_backend.py (np.fft.fft forward,
scipy.fft.ifft inverse, mean periodisation).  Filters stay float64, as the
reference numpy frontend keeps them; ``filters_dtype=np.float32`` reproduces
the torch frontend's float32 cast (kymatio/scattering1d/frontend/torch_frontend.py:38-52).
"""
import math

import numpy as np
import scipy.fft

from .filters import compute_temporal_support, gauss_1d, scattering_filter_factory_1d


def parse_T(T, J, N_input):
    """kymatio/scattering1d/utils.py:75-107."""
    if T is None:
        return 2 ** J, 'local'
    if T == 'global':
        return 2 ** J, 'global'
    if T > N_input:
        raise ValueError('The support {} of the low-pass filter cannot exceed input length'.format(T))
    if T == 0:
        return 2 ** J, False
    if T < 1:
        raise ValueError('T must be ==0 or >=1 (got {})'.format(T))
    return T, 'local'


def compute_border_indices(log2_T, J, i0, i1):
    """kymatio/scattering1d/utils.py:4-38."""
    ind_start, ind_end = {0: i0}, {0: i1}
    for j in range(1, max(log2_T, J) + 1):
        ind_start[j] = ind_start[j - 1] // 2 + ind_start[j - 1] % 2
        ind_end[j] = ind_end[j - 1] // 2 + ind_end[j - 1] % 2
    return ind_start, ind_end


def compute_padding_1d(N, N_input):
    """kymatio/scattering1d/utils.py:40-66."""
    to_add = N - N_input
    left = to_add // 2
    return left, to_add - left


def subsample_fourier(x, k):
    """numpy_backend.py:6-32 (1-D)."""
    return x.reshape(x.shape[:-1] + (k, x.shape[-1] // k)).mean(axis=-2)


def scattering1d_core(U_0, filters, log2_stride, average_local):
    """kymatio/scattering1d/core/scattering1d.py:2-107 as a list of paths."""
    out = []
    U_0_hat = np.fft.fft(U_0)
    phi = filters[0]
    if average_local:
        S_0 = scipy.fft.ifft(subsample_fourier(U_0_hat * phi['levels'][0], 2 ** log2_stride)).real
        out.append({'coef': S_0, 'j': (), 'n': ()})
    else:
        out.append({'coef': U_0, 'j': (), 'n': ()})
    psi1 = filters[1]
    for n1, p1 in enumerate(psi1):
        j1 = p1['j']
        k1 = min(j1, log2_stride) if average_local else j1
        U_1_c = scipy.fft.ifft(subsample_fourier(U_0_hat * p1['levels'][0], 2 ** k1))
        U_1_m = np.abs(U_1_c)
        if average_local or len(filters) > 2:
            U_1_hat = np.fft.fft(U_1_m)
        if average_local:
            k1_J = max(log2_stride - k1, 0)
            S_1 = scipy.fft.ifft(subsample_fourier(U_1_hat * phi['levels'][k1], 2 ** k1_J)).real
            out.append({'coef': S_1, 'j': (j1,), 'n': (n1,)})
        else:
            out.append({'coef': U_1_m, 'j': (j1,), 'n': (n1,)})
        if len(filters) > 2:
            for n2, p2 in enumerate(filters[2]):
                j2 = p2['j']
                if j2 <= j1:
                    continue
                sub2 = min(j2, log2_stride) if average_local else j2
                k2 = max(sub2 - k1, 0)
                U_2_c = scipy.fft.ifft(subsample_fourier(U_1_hat * p2['levels'][k1], 2 ** k2))
                U_2_m = np.abs(U_2_c)
                if average_local:
                    U_2_hat = np.fft.fft(U_2_m)
                    k2_T = max(log2_stride - sub2, 0)
                    S_2 = scipy.fft.ifft(subsample_fourier(U_2_hat * phi['levels'][k1 + k2],
                                                           2 ** k2_T)).real
                    out.append({'coef': S_2, 'j': (j1, j2), 'n': (n1, n2)})
                else:
                    out.append({'coef': U_2_m, 'j': (j1, j2), 'n': (n1, n2)})
    return out


class Scattering1D:
    """Oracle counterpart of ScatteringNumPy1D / ScatteringBase1D
    (kymatio/scattering1d/frontend/base_frontend.py:16-155)."""

    def __init__(self, J, shape, Q=1, T=None, stride=None, max_order=2,
                 oversampling=0, out_type='array', filters_dtype=None):
        self.J, self.max_order, self.out_type = J, max_order, out_type
        self.oversampling = oversampling
        N_input = shape if isinstance(shape, int) else shape[0]
        self.N_input = N_input
        self.Q = (Q, 1) if isinstance(Q, int) else (tuple(Q) + (1,) if len(Q) == 1 else tuple(Q))
        self.T, self.average = parse_T(T, J, N_input)
        self.log2_T = int(math.floor(math.log2(self.T)))
        if oversampling > 0:
            stride = 2 ** (self.log2_T - oversampling)
        self.log2_stride = self.log2_T if stride is None else int(math.log2(stride))
        phi_f = gauss_1d(N_input, 0.1 / self.T)
        min_to_pad = 3 * compute_temporal_support(phi_f.reshape(1, -1), criterion_amplitude=1e-3)
        J_max_support = int(np.floor(np.log2(3 * N_input - 2)))
        J_pad = min(int(np.ceil(np.log2(N_input + 2 * min_to_pad))), J_max_support)
        self.N_padded = 2 ** J_pad
        self.pad_left, self.pad_right = compute_padding_1d(self.N_padded, N_input)
        self.ind_start, self.ind_end = compute_border_indices(
            self.log2_T, J, self.pad_left, self.pad_left + N_input)
        banks = scattering_filter_factory_1d(self.N_padded, J, self.Q, self.T)
        if filters_dtype is not None:
            for bank in (banks[0],) + tuple(p for b in banks[1:] for p in b):
                bank['levels'] = [lv.astype(filters_dtype) for lv in bank['levels']]
        self.phi_f, self.psi1_f, self.psi2_f = banks

    def __call__(self, x):
        x = np.asarray(x)
        batch_shape = x.shape[:-1]
        U0 = x.reshape((-1, 1, x.shape[-1]))
        U0 = np.pad(U0, ((0, 0), (0, 0), (self.pad_left, self.pad_right)), mode='reflect')
        filters = [self.phi_f, self.psi1_f, self.psi2_f][:1 + self.max_order]
        paths = scattering1d_core(U0, filters, self.log2_stride, self.average == 'local')
        S = {} if self.out_type == 'dict' else []
        for p in paths:
            p['order'] = len(p['n'])
            if self.average == 'local':
                res = self.log2_stride
            elif p['order'] > 0:
                res = max(p['j'][-1] - self.oversampling, 0)
            else:
                res = 0
            if self.average == 'global':
                c = p['coef'].sum(axis=-1, keepdims=True)
            else:
                c = p['coef'][..., self.ind_start[res]:self.ind_end[res]]
            p['coef'] = c.reshape(batch_shape + c.shape[-1:])
            if self.out_type == 'dict':
                S[p['n']] = p['coef']
            else:
                S.append(p)
        if self.out_type == 'dict':
            return S
        S.sort(key=lambda p: (p['order'], p['n']))
        if self.out_type == 'array':
            return np.stack([p['coef'] for p in S], axis=-2)
        return S
