"""Joint time-frequency scattering (JTFS) over the GB300 op surface.

``TimeFrequencyScattering`` is a drop-in for kymatio's
``TimeFrequencyScatteringTorch`` (kymatio/scattering1d/frontend/
torch_frontend.py:86-155 with the base frontend
kymatio/scattering1d/frontend/base_frontend.py:524-764): the same
constructor arguments, registered buffers ``tensor{n}`` (the time filters of
``Scattering1D``, then the frequential low-pass phi_F, then the frequential
filters psi_fr), output formats ('time' or 'joint'; out_type 'array',
'list' or 'dict') and ``meta()``.

The transform is computed op by op, as the reference's torch backend does,
by the generators below (a restatement of
kymatio/scattering1d/core/timefrequency_scattering.py:4-444) over
``backend1d``: every FFT, wavelet product, periodisation and modulus runs one
of this package's CUDA kernels; the frequency-axis moves (zero padding,
time/frequency transposition, unpadding, splitting) are tensor views and
copies, as in kymatio/scattering1d/backend/torch_backend.py:150-223.
"""
import math
import numbers
from collections import Counter

import numpy as np
import torch

from .filter_bank import filter_bank_fr
from .scattering1d import Scattering1D, _parse_T


# ---------------------------------------------------------------------------
# The cascade (generators of paths, each a dict with 'coef' and indices)
# ---------------------------------------------------------------------------

def time_scattering_widthfirst(U_0, B, filters, log2_stride, average_local):
    """Zeroth order, then every first-order path averaged in time and stacked
    over n1 (S1), then for each second-order wavelet n2 the complex Y2 of all
    n1 with j1 < j2 stacked over n1 (the n2 loop outside: width first).
    kymatio/scattering1d/core/timefrequency_scattering.py:84-189."""
    phi, psi1, psi2 = filters
    U_0_hat = B.rfft(U_0)
    if average_local:
        S_0 = B.irfft(B.subsample_fourier(B.cdgmm(U_0_hat, phi['levels'][0]), 2 ** log2_stride))
        yield {'coef': S_0, 'j': (), 'n': ()}
    else:
        yield {'coef': U_0, 'j': (), 'n': ()}

    first = []  # (j1, k1, FFT of U1) of every first-order path
    S_1 = []
    for p1 in psi1:
        j1 = p1['j']
        k1 = min(j1, log2_stride) if average_local else j1
        U_1 = B.modulus(B.ifft(B.subsample_fourier(B.cdgmm(U_0_hat, p1['levels'][0]), 2 ** k1)))
        U_1_hat = B.rfft(U_1)
        first.append((j1, k1, U_1_hat))
        S_1.append(B.irfft(B.subsample_fourier(B.cdgmm(U_1_hat, phi['levels'][k1]), 2 ** (log2_stride - k1))))
    # n1 is a stacked axis here: the placeholder -1 stands for it
    yield {'coef': B.stack(S_1, 2), 'j': (-1,), 'n': (-1,), 'n1_max': len(S_1)}

    for n2, p2 in enumerate(psi2):
        j2 = p2['j']
        Y_2 = []
        for j1, k1, U_1_hat in first:
            if j2 <= j1:
                continue
            k2 = min(j2 - k1, log2_stride) if average_local else j2 - k1
            Y_2.append(B.ifft(B.subsample_fourier(B.cdgmm(U_1_hat, p2['levels'][k1]), 2 ** k2)))
        if Y_2:
            yield {'coef': B.stack(Y_2, 2), 'j': (-1, j2), 'n': (-1, n2), 'n1_max': len(Y_2)}


def frequency_scattering(X, B, filters_fr, log2_stride_fr, average_local_fr, spinned):
    """Wavelet transform along n1 of a stacked path X (zero-padded to the
    frequential size): every frequential filter for complex input (spin up
    and down), only those with xi >= 0 for real input (S1).
    kymatio/scattering1d/core/timefrequency_scattering.py:192-275."""
    phi_F, psis = filters_fr
    X_T = B.swap_time_frequency(X['coef'])
    X_pad = B.pad_frequency(X_T, phi_F['N'] - X['n1_max'])
    if spinned:
        X_hat = B.cfft(X_pad)
        bank = psis
    else:
        X_hat = B.rfft(X_pad)
        bank = [p for p in psis if p['xi'] >= 0]
    for n_fr, psi in enumerate(bank):
        j_fr = psi['j']
        k_fr = min(j_fr, log2_stride_fr) if average_local_fr else j_fr
        Y = B.ifft(B.subsample_fourier(B.cdgmm(X_hat, psi['levels'][0]), 2 ** k_fr))
        path = dict(X)
        path.update(coef=B.swap_time_frequency(Y), n=X['n'][1:] + (n_fr,), j_fr=(j_fr,), n_fr=(n_fr,),
                    n1_stride=2 ** j_fr, spin=np.sign(psi['xi']))
        yield path


def joint_timefrequency_scattering(U_0, B, filters, log2_stride, average_local, filters_fr, log2_stride_fr,
                                   average_local_fr):
    """Zeroth order, the frequential scattering of S1, then of every Y2.
    kymatio/scattering1d/core/timefrequency_scattering.py:4-81."""
    time_gen = time_scattering_widthfirst(U_0, B, filters, log2_stride, average_local)
    yield next(time_gen)
    S_1 = next(time_gen)
    yield from frequency_scattering(S_1, B, filters_fr, log2_stride_fr, average_local_fr, spinned=False)
    for Y_2 in time_gen:
        yield from frequency_scattering(Y_2, B, filters_fr, log2_stride_fr, average_local_fr, spinned=True)


def time_averaging(U_2, B, phi, log2_stride):
    """Low-pass in time of a second-order path at its resolution j2.
    kymatio/scattering1d/core/timefrequency_scattering.py:278-315."""
    k_in = U_2['j'][-1]
    S = B.irfft(B.subsample_fourier(B.cdgmm(B.rfft(U_2['coef']), phi['levels'][k_in]), 2 ** (log2_stride - k_in)))
    path = dict(U_2)
    path['coef'] = S
    return path


def frequency_averaging(U_2, B, phi_F, log2_stride_fr, average_fr):
    """Low-pass (or sum) along n1.
    kymatio/scattering1d/core/timefrequency_scattering.py:318-373."""
    path = dict(U_2)
    if not average_fr:
        path['n1_stride'] = 2 ** max(U_2['j_fr'][-1], 0)
        return path
    U_T = B.swap_time_frequency(U_2['coef'])
    if average_fr == 'global':
        S_T = B.average_global(U_T)
        path['n1_stride'] = U_2['n1_max']
    else:
        k_in = min(U_2['j_fr'][-1], phi_F['j'])
        S_T = B.irfft(B.subsample_fourier(B.cdgmm(B.rfft(U_T), phi_F['levels'][k_in]), 2 ** (log2_stride_fr - k_in)))
        path['n1_stride'] = 2 ** log2_stride_fr
    path['coef'] = B.swap_time_frequency(S_T)
    return path


def time_formatting(path, B):
    """One path per retained n1 ('time' format); n becomes (n1,) + n.
    kymatio/scattering1d/core/timefrequency_scattering.py:376-392."""
    n1s = list(range(0, path['n1_max'], path['n1_stride']))
    coefs = [None] * len(n1s) if path['coef'] is None else B.split_frequency_axis(path['coef'])
    for n1, coef in zip(n1s, coefs):
        out = {k: v for k, v in path.items() if k not in ('n1_max', 'n1_stride')}
        out.update(coef=coef, order=len(path['n']) - 1, n=(n1,) + path['n'])
        yield out


def jtfs_average_and_format(U_gen, B, phi, log2_stride, average, phi_F, log2_stride_fr, average_fr, out_type,
                            format):
    """Modulus, averaging in time and frequency, unpadding and splitting.
    kymatio/scattering1d/core/timefrequency_scattering.py:395-444."""
    path = next(U_gen)
    if average == 'global':
        path['coef'] = B.average_global(path['coef'])
    yield dict(path, order=0)
    for path in U_gen:
        path['coef'] = B.modulus(path['coef'])
        if average == 'global':
            path['coef'] = B.average_global(path['coef'])
        elif average == 'local' and len(path['n']) > 1:
            path = time_averaging(path, B, phi, log2_stride)
        # a spin-0 path was filtered by the frequential low-pass already
        if average_fr and path['spin'] != 0:
            path = frequency_averaging(path, B, phi_F, log2_stride_fr, average_fr)
        if not (out_type == 'array' and format == 'joint'):
            path['coef'] = B.unpad_frequency(path['coef'], path['n1_max'], path['n1_stride'])
        if format == 'joint':
            yield dict(path, order=len(path['n']))
        else:
            yield from time_formatting(path, B)


class _NoData:
    """Runs the generators without data (for ``meta``): every op returns None."""

    def __getattr__(self, name):
        return lambda *args, **kwargs: None


# ---------------------------------------------------------------------------
# Frontend
# ---------------------------------------------------------------------------

class TimeFrequencyScattering(Scattering1D):
    """Joint time-frequency scattering (kymatio.torch.TimeFrequencyScattering)."""

    def __init__(self, J, J_fr, Q, shape, T=None, stride=None, Q_fr=1, F=None, stride_fr=None, out_type='array',
                 format='time', backend='torch', graph=False):
        super().__init__(J, shape, Q=Q, T=T, stride=stride, max_order=2, oversampling=None, out_type=out_type,
                         backend=backend)
        # graph=True: an array-output forward without autograd replays one CUDA
        # graph per input shape (its thousands of small launches become one)
        self.graph = graph
        self._graphs = {}
        self.J_fr = J_fr
        self._F = F
        self.oversampling_fr = 0
        self._stride_fr = stride_fr
        self.format = format
        # kymatio/scattering1d/frontend/base_frontend.py:539-568
        if np.any(np.array(Q_fr) < 1):
            raise ValueError('Q_fr must be >= 1, got {}'.format(Q_fr))
        if isinstance(Q_fr, int):
            Q_fr = (Q_fr,)
        elif isinstance(Q_fr, tuple):
            if len(Q_fr) != 1:
                raise NotImplementedError('Q_fr must be an integer or 1-tuple. Time-frequency scattering '
                                          'beyond order 2 is not implemented.')
        else:
            raise ValueError('Q_fr must be an integer or 1-tuple.')
        self.Q_fr = Q_fr
        min_to_pad_fr = 8 * min(self.F, 2 ** self.J_fr)
        N_input_fr = (self.J + 1) * self.Q[0]
        K_fr = max(self.J_fr - self.oversampling_fr, 0)
        self._N_padded_fr = (N_input_fr + min_to_pad_fr) // (2 ** K_fr) * (2 ** K_fr)
        phi_F, psis = filter_bank_fr(self._N_padded_fr, self.J_fr, self.Q_fr[0], self.F)
        assert all(abs(p['xi']) < 0.5 / (2 ** p['j']) for p in psis[1:])
        self.phi_fr_f = {k: v for k, v in phi_F.items() if k != 'levels'}
        self.psis_fr_f = [{k: v for k, v in p.items() if k != 'levels'} for p in psis]
        n = self._n_filters
        self._nlev_fr = {'phi': len(phi_F['levels']), 'psi': [len(p['levels']) for p in psis]}
        for f in (phi_F,) + tuple(psis):
            for lv in f['levels']:
                self.register_buffer('tensor' + str(n), torch.from_numpy(lv).float().view(-1, 1))
                n += 1
        self._n_filters_fr = n - self._n_filters

    # -- reference properties (base_frontend.py:722-764) ---------------------------
    @property
    def average_fr(self):
        return _parse_T(self._F, self.J_fr, (self.J + 1) * self.Q[0], 'F')[1]

    @property
    def F(self):
        return _parse_T(self._F, self.J_fr, (self.J + 1) * self.Q[0], 'F')[0]

    @property
    def log2_F(self):
        return int(math.floor(math.log2(self.F)))

    @property
    def log2_stride_fr(self):
        if self._stride_fr is None:
            return self.log2_F
        if not isinstance(self._stride_fr, numbers.Integral):
            raise ValueError('stride_fr must be integer. Got: {}'.format(self._stride_fr))
        l2 = math.log2(self._stride_fr)
        if math.floor(l2) != math.ceil(l2):
            raise ValueError('stride_fr must be a power of two. Got: {}'.format(self._stride_fr))
        if self.average_fr in [False, 'global']:
            raise ValueError('stride_fr={} is incompatible with F={}.'.format(self._stride_fr, self._F))
        return int(l2)

    @property
    def stride_fr(self):
        return 2 ** self.log2_stride_fr

    @property
    def filters_fr(self):
        """(phi_F, [phi_{2^J_fr}] + psis) with the registered device tensors as levels."""
        n = self._n_filters
        out = []
        for meta, nl in zip([self.phi_fr_f] + self.psis_fr_f, [self._nlev_fr['phi']] + self._nlev_fr['psi']):
            d = dict(meta)
            d['levels'] = [getattr(self, 'tensor%d' % (n + i)) for i in range(nl)]
            n += nl
            out.append(d)
        return out[0], out[1:]

    def _check_runtime_args_fr(self):
        """base_frontend.py:223-230 and 700-720."""
        if self.out_type not in ('array', 'dict', 'list'):
            raise ValueError("out_type must be one of 'array', 'dict', or 'list'. Got: {}".format(self.out_type))
        if not self.average and self.out_type == 'array':
            raise ValueError("Cannot convert to out_type='array' with T=0. Please set out_type to 'dict' or 'list'.")
        if self.format == 'joint' and (not self.average_fr) and self.out_type == 'array':
            raise ValueError("Cannot convert to format='joint' with out_type='array' and F=0. Either set "
                             "format='time', out_type='dict', or out_type='list'.")
        if self.oversampling_fr < 0:
            raise ValueError('oversampling_fr must be nonnegative. Got: {}'.format(self.oversampling_fr))
        if not isinstance(self.oversampling_fr, numbers.Integral):
            raise ValueError('oversampling_fr must be integer. Got: {}'.format(self.oversampling_fr))
        if self.format not in ['time', 'joint']:
            raise ValueError("format must be 'time' or 'joint'. Got: {}".format(self.format))

    # -- forward ------------------------------------------------------------------------
    def scattering(self, x):
        """kymatio/scattering1d/frontend/base_frontend.py:581-648."""
        from .backend import backend1d
        self._check_runtime_args_fr()
        if len(x.shape) < 1:
            raise ValueError('Input tensor x should have at least one axis, got {}'.format(len(x.shape)))
        if not x.is_cuda:
            raise TypeError('The input must be a CUDA tensor: the GB300 scattering engine runs on CUDA only.')
        if x.dtype != torch.float32:
            raise TypeError('The input must be float32 (got %s).' % x.dtype)
        if self.graph and self.out_type == 'array' and not (torch.is_grad_enabled() and x.requires_grad):
            return self._jtfs_graphed(x, backend1d)
        return self._jtfs(x, backend1d)

    def _jtfs_graphed(self, x, B):
        """The same forward replayed from a CUDA graph captured on first use
        for this input shape and format (after an eager warm-up that creates
        every plan and device table); the result is copied out of the graph's
        buffers, so it stays valid across calls."""
        key = (tuple(x.shape), str(x.device), self.format)
        ent = self._graphs.get(key)
        if ent is None:
            static_x = x.detach().contiguous().clone()
            with torch.no_grad():
                self._jtfs(static_x, B)
                torch.cuda.synchronize(x.device)
                g = torch.cuda.CUDAGraph()
                cap = torch.cuda.Stream(x.device)
                cap.wait_stream(torch.cuda.current_stream(x.device))
                with torch.cuda.graph(g, stream=cap):
                    static_out = self._jtfs(static_x, B)
            ent = self._graphs[key] = (g, static_x, static_out)
        g, static_x, static_out = ent
        static_x.copy_(x)
        g.replay()
        return static_out.clone()

    def _apply(self, fn, *args, **kwargs):
        self._graphs = {}  # the captured graphs hold the old buffers' addresses
        return super()._apply(fn, *args, **kwargs)

    def _jtfs(self, x, B):
        """The transform over the op surface B (the CUDA ops in the module)."""
        batch_shape = tuple(x.shape[:-1])
        signal_shape = tuple(x.shape[-1:])
        U_0 = B.pad(B.reshape_input(x.contiguous(), signal_shape), pad_left=self.pad_left, pad_right=self.pad_right)
        filters = self._op_filters()
        filters_fr = self.filters_fr
        U_gen = joint_timefrequency_scattering(U_0, B, filters, self.log2_stride, self.average == 'local',
                                               filters_fr, self.log2_stride_fr, self.average_fr == 'local')
        S_gen = jtfs_average_and_format(U_gen, B, filters[0], self.log2_stride, self.average, filters_fr[0],
                                        self.log2_stride_fr, self.average_fr, self.out_type, self.format)
        path = next(S_gen)
        if self.average != 'global':
            res = self.log2_stride if self.average else 0
            path['coef'] = B.unpad(path['coef'], self.ind_start[res], self.ind_end[res])
        path['coef'] = B.reshape_output(path['coef'], batch_shape, n_kept_dims=1)
        S = [path]
        for path in S_gen:
            if self.average != 'global':
                # un-averaged second order sits at resolution j2; everything else at log2_stride
                res = max(path['j'][-1], 0) if (not self.average and len(path['n']) > 1) else max(self.log2_stride, 0)
                path['coef'] = B.unpad(path['coef'], self.ind_start[res], self.ind_end[res])
            path['coef'] = B.reshape_output(path['coef'], batch_shape, n_kept_dims=1 + (self.format == 'joint'))
            S.append(path)
        if self.format == 'joint' and self.out_type == 'array':
            return B.stack([p['coef'] for p in S[1:]], dim=-3)
        if self.format == 'time' and self.out_type == 'array':
            return B.stack([p['coef'] for p in S], dim=-2)
        if self.out_type == 'dict':
            return {p['n']: p['coef'] for p in S}
        return S

    # -- metadata -----------------------------------------------------------------------
    def _path_table(self):
        """The output paths of the cascade, in output order, without data: the
        generators run over a backend whose ops return None, and each path's
        dict keeps its indices (n, n_fr, j, and the stacked n1 axis
        n1_max / n1_stride in the 'joint' format)."""
        nd = _NoData()

        def blank(meta, n_levels):
            return dict(meta, levels=[None] * n_levels)

        filters = [blank(self.phi_f, self._nlev['phi']),
                   [blank(p, nl) for p, nl in zip(self.psi1_f, self._nlev['psi1'])],
                   [blank(p, nl) for p, nl in zip(self.psi2_f, self._nlev['psi2'])]]
        filters_fr = (blank(self.phi_fr_f, self._nlev_fr['phi']),
                      [blank(p, nl) for p, nl in zip(self.psis_fr_f, self._nlev_fr['psi'])])
        U_gen = joint_timefrequency_scattering(None, nd, filters, self.log2_stride, self.average == 'local',
                                               filters_fr, self.log2_stride_fr, self.average_fr == 'local')
        S_gen = jtfs_average_and_format(U_gen, nd, filters[0], self.log2_stride, self.average, filters_fr[0],
                                        self.log2_stride_fr, self.average_fr, self.out_type, self.format)
        return sorted(S_gen, key=lambda p: (len(p['n']), p['n']))

    def meta(self):
        """Description of every output path, with the fields of kymatio's
        TimeFrequencyScattering.meta (kymatio/scattering1d/frontend/
        base_frontend.py:650-698): 'key' (every path's n), and per row
        'n' = (n1, n2) -- the time-wavelet indices, n1 a range over the
        stacked first-order axis in the 'joint' format, NaN where a path has
        no such wavelet --, 'n_fr', 'order' (the number of time wavelets),
        the time filters' 'xi' / 'sigma' / 'j' (two columns), the frequential
        filter's 'xi_fr' / 'sigma_fr' / 'j_fr' and its 'spin'.  One row per
        path of the path table, except the zeroth order in the 'joint'
        format's array output, which holds no such row."""
        paths = self._path_table()
        rows = [p for p in paths if p['n'] or not (self.format == 'joint' and self.out_type == 'array')]
        nan = np.nan

        def indices(p):
            # (n1, n2, n_fr) of a row; None where the path has no such filter
            if not p['j']:
                return None, None, None
            n1 = range(0, p['n1_max'], p['n1_stride']) if 'n1_max' in p else p['n'][0]
            n2 = p['n'][-2] if len(p['j']) == 2 else None
            return n1, n2, p['n_fr'][0]

        table = [indices(p) for p in rows]

        def field(bank, i, name):
            return bank[i][name] if isinstance(i, (int, np.integer)) else nan

        meta = {'key': [p['n'] for p in paths],
                'n': np.array([[nan if v is None else v for v in t[:2]] for t in table], dtype=object),
                'n_fr': np.array([nan if t[2] is None else t[2] for t in table], dtype=float),
                'order': np.array([len(p['j']) for p in rows])}
        for name in ('xi', 'sigma', 'j'):
            meta[name] = np.array([[field(self.psi1_f, t[0], name), field(self.psi2_f, t[1], name)]
                                   for t in table], dtype=float).reshape(len(table), 2)
            meta[name + '_fr'] = np.array([field(self.psis_fr_f, t[2], name) for t in table], dtype=float)
        meta['spin'] = np.sign(meta['xi_fr'])
        return meta

    def output_size(self, detail=False):
        """kymatio/scattering1d/frontend/base_frontend.py:204-221, over this meta()."""
        meta = self.meta()
        if detail:
            return tuple(Counter(meta['order']).values())
        return len(meta['key'])
