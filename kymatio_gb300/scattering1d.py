"""Scattering1D: drop-in for kymatio's ScatteringTorch1D on one GB300.

Constructor, build-time geometry (padding to a power of two, reflect pad,
border indices; kymatio/scattering1d/frontend/base_frontend.py:37-98),
registered buffers (``tensor0..tensorK`` of shape (n, 1), phi levels then
psi1 then psi2 levels; kymatio/scattering1d/frontend/torch_frontend.py:
30-56), ``meta()``/``output_size()`` (:157-221), argument parsing (Q, T,
stride, oversampling) and output formats ('array', 'list', 'dict') follow
the reference.  With local averaging (T a number or None) the transform runs
as one fused CUDA cascade (kym_s1d_forward).
"""
import math
import numbers
from collections import Counter
from warnings import warn

import numpy as np
import torch
import torch.nn as nn

from . import _autograd, _lib
from .filter_bank import border_indices, filter_bank_1d, geometry_1d
from .scattering2d import _Plan


def _parse_T(T, J, N_input, T_alias='T'):
    """kymatio/scattering1d/utils.py:71-108 (T_alias 'F' for the frequential
    low-pass of time-frequency scattering)."""
    if T is None:
        return 2 ** J, 'local'
    if T == 'global':
        return 2 ** J, 'global'
    if T > N_input:
        raise ValueError("The support {} of the low-pass filter cannot exceed input length (got {} > {}). "
                         "For large averaging size, consider passing {}='global'.".format(T_alias, T, N_input,
                                                                                         T_alias))
    if T == 0:
        return 2 ** J, False
    if T < 1:
        raise ValueError('{} must be ==0 or >=1 (got {})'.format(T_alias, T))
    return T, 'local'


class Scattering1D(nn.Module):
    """1-D scattering transform with Morlet wavelets (kymatio.torch.Scattering1D)."""

    def __init__(self, J, shape, Q=1, T=None, stride=None, max_order=2, oversampling=0, out_type='array',
                 backend='torch'):
        super().__init__()
        self.frontend_name = 'torch'
        if backend is not None and not isinstance(backend, str) and \
                not str(getattr(backend, 'name', '')).startswith('torch'):
            raise ImportError('The backend ' + str(getattr(backend, 'name', backend)) +
                              ' is not supported by the frontend torch.')
        self.backend = backend
        self.J, self._Q, self._T, self._stride = J, Q, T, stride
        self.max_order, self.out_type, self._oversampling = max_order, out_type, oversampling
        if isinstance(shape, numbers.Integral):
            shape = (shape,)
        elif isinstance(shape, tuple):
            if len(shape) > 1:
                raise ValueError('If shape is specified as a tuple, it must have exactly one element. '
                                 'Got: {}'.format(shape))
        else:
            raise ValueError('shape must be an integer or a 1-tuple. Got: {}'.format(shape))
        self.shape = shape
        N_input = shape[0]
        if self._oversampling is None:
            pass
        elif self._oversampling < 0:
            raise ValueError('oversampling must be nonnegative. Got: {}'.format(self._oversampling))
        elif not isinstance(self._oversampling, numbers.Integral):
            raise ValueError('oversampling must be integer. Got: {}'.format(self._oversampling))
        elif self._oversampling > 0:
            warn('oversampling is deprecated in and will be removed in v0.5.Pass stride = 2**(J-oversampling) '
                 'or stride = 2**(log2(T)-oversampling) to retain current behavior.', DeprecationWarning)
            if self._stride not in [None, 2 ** (self.log2_T - self._oversampling - 1)]:
                raise ValueError('oversampling={} and stride={}are incompatible'.format(
                    self._oversampling, self._stride))
            self._stride = 2 ** (self.log2_T - self._oversampling)
        self._N_padded, self.pad_left, self.pad_right = geometry_1d(J, N_input, self.T)
        self.ind_start, self.ind_end = border_indices(self.log2_T, J, self.pad_left, self.pad_left + N_input)
        phi, psi1, psi2 = filter_bank_1d(self._N_padded, J, self.Q, self.T)
        self._check_filterbanks(psi1, psi2)
        self.phi_f = {k: v for k, v in phi.items() if k != 'levels'}
        self.psi1_f = [{k: v for k, v in p.items() if k != 'levels'} for p in psi1]
        self.psi2_f = [{k: v for k, v in p.items() if k != 'levels'} for p in psi2]
        n = 0
        for lv in phi['levels']:
            self.register_buffer('tensor' + str(n), torch.from_numpy(lv).float().view(-1, 1))
            n += 1
        self._nlev = {'phi': len(phi['levels']), 'psi1': [], 'psi2': []}
        for key, bank in (('psi1', psi1), ('psi2', psi2)):
            for p in bank:
                self._nlev[key].append(len(p['levels']))
                for lv in p['levels']:
                    self.register_buffer('tensor' + str(n), torch.from_numpy(lv).float().view(-1, 1))
                    n += 1
        self._n_filters = n
        self._plan = None
        self._ptr_cache = (None, None)

    @staticmethod
    def _check_filterbanks(psi1s, psi2s):
        """kymatio/frontend/base_frontend.py:17-30."""
        assert all((p['xi'] < 0.5 / (2 ** p['j'])) for p in psi1s)
        for p1 in psi1s:
            for p2 in psi2s:
                if p1['j'] < p2['j']:
                    assert p1['xi'] > p2['xi']

    # -- reference properties --------------------------------------------------
    @property
    def average(self):
        return _parse_T(self._T, self.J, self.shape[0])[1]

    @property
    def T(self):
        return _parse_T(self._T, self.J, self.shape[0])[0]

    @property
    def log2_T(self):
        return int(math.floor(math.log2(self.T)))

    @property
    def Q(self):
        if np.any(np.array(self._Q) < 1):
            raise ValueError('Q must always be >= 1, got {}'.format(self._Q))
        if isinstance(self._Q, int):
            return (self._Q, 1)
        if isinstance(self._Q, tuple):
            if len(self._Q) == 1:
                return self._Q + (1,)
            if len(self._Q) == 2:
                return self._Q
            raise NotImplementedError('Q must be an integer, 1-tuple or 2-tuple. Scattering transforms beyond '
                                      'order 2 are not implemented. Got: {}'.format(self._Q))
        raise ValueError('Q must be an integer or a tuple')

    @property
    def log2_stride(self):
        if self._stride is None:
            return self.log2_T
        if not isinstance(self._stride, numbers.Integral):
            raise ValueError('stride must be integer. Got: {}'.format(self._stride))
        l2 = math.log2(self._stride)
        if math.floor(l2) != math.ceil(l2):
            raise ValueError('stride must be a power of two. Got: {}'.format(self._stride))
        if self.average in [False, 'global']:
            raise ValueError('stride={} is incompatible with T={}.'.format(self._stride, self._T))
        return int(l2)

    @property
    def stride(self):
        return 2 ** self.log2_stride

    @property
    def oversampling(self):
        warn('The attribute oversampling is deprecated and will be removed in v0.5. Pass stride = '
             '2**(J-oversampling) or stride = 2**(log2(T)-oversampling) to retain current behavior.',
             DeprecationWarning)
        return self._oversampling

    def _paths(self):
        """Path keys in output order (sorted by (order, n))."""
        keys = [()]
        keys += [(n1,) for n1 in range(len(self.psi1_f))]
        if self.max_order >= 2:
            keys += [(n1, n2) for n1, p1 in enumerate(self.psi1_f) for n2, p2 in enumerate(self.psi2_f)
                     if p2['j'] > p1['j']]
        return keys

    def meta(self):
        """kymatio/scattering1d/frontend/base_frontend.py:157-202."""
        keys = self._paths()
        meta = {'order': np.array([len(k) for k in keys]), 'key': keys}
        meta['n'] = np.stack([np.append(k, (np.nan,) * (self.max_order - len(k))) for k in keys])
        banks = (self.psi1_f, self.psi2_f)[:self.max_order]
        for field in ['xi', 'sigma', 'j']:
            meta[field] = meta['n'] * np.nan
            for order, bank in enumerate(banks):
                for n, p in enumerate(bank):
                    meta[field][meta['n'][:, order] == n, order] = p[field]
        return meta

    def output_size(self, detail=False):
        if detail:
            return tuple(Counter(self.meta()['order']).values())
        return len(self._paths())

    # -- plan ---------------------------------------------------------------------
    def _get_plan(self):
        if self._plan is None:
            lib = _lib.load()
            h = _lib._vp()
            l2s = self.log2_stride
            j1 = [p['j'] for p in self.psi1_f]
            j2 = [p['j'] for p in self.psi2_f]
            _lib.check(lib.kym_s1d_plan_create(
                self._N_padded, self.shape[0], self.pad_left, l2s, self.max_order,
                len(j1), _lib.int_array(j1), _lib.int_array(self._nlev['psi1']),
                len(j2), _lib.int_array(j2), _lib.int_array(self._nlev['psi2']), self._nlev['phi'],
                self.ind_start[l2s], self.ind_end[l2s], _lib.ctypes.byref(h)), 'kym_s1d_plan_create')
            self._plan = _Plan(lib, h.value, lib.kym_s1d_plan_destroy)
            v = [_lib.ctypes.c_int() for _ in range(3)]
            _lib.check(lib.kym_s1d_plan_info(self._plan.h, *[_lib.ctypes.byref(i) for i in v]), 'kym_s1d_plan_info')
            self._channels, self._out_len = v[0].value, v[1].value
            if v[2].value != self._n_filters or self._channels != len(self._paths()):
                raise RuntimeError('filter bank layout mismatch')
        return self._plan

    def set_chunk(self, chunk):
        _lib.check(_lib.load().kym_s1d_set_chunk(self._get_plan().h, int(chunk)), 'kym_s1d_set_chunk')

    def _filter_ptrs(self):
        bufs = [getattr(self, 'tensor' + str(i)) for i in range(self._n_filters)]
        key = tuple(b.data_ptr() for b in bufs)
        if self._ptr_cache[0] != key:
            for b in bufs:
                if not b.is_cuda or b.dtype != torch.float32 or not b.is_contiguous():
                    raise TypeError('The filters must be contiguous float32 CUDA tensors; call .cuda() on the '
                                    'module (the GB300 engine runs on CUDA only).')
            self._ptr_cache = (key, _lib.ptr_array(list(key)))
        return self._ptr_cache[1]

    # -- forward ------------------------------------------------------------------
    def forward(self, x):
        if x is None:
            raise TypeError('The input should be not empty.')
        if torch.is_tensor(x) and not x.is_contiguous():
            raise RuntimeError('Tensors must be contiguous.')
        return self.scattering(x)

    def scattering(self, x):
        if self.out_type not in ('array', 'dict', 'list'):
            raise ValueError("out_type must be one of 'array', 'dict', or 'list'. Got: {}".format(self.out_type))
        if not self.average and self.out_type == 'array':
            raise ValueError("Cannot convert to out_type='array' with T=0. Please set out_type to 'dict' or 'list'.")
        if len(x.shape) < 1:
            raise ValueError('Input tensor x should have at least one axis, got {}'.format(len(x.shape)))
        if not x.is_cuda:
            raise TypeError('The input must be a CUDA tensor: the GB300 scattering engine runs on CUDA only.')
        if x.dtype != torch.float32:
            raise TypeError('The input must be float32 (got %s).' % x.dtype)
        if self.average != 'local':
            return self._scattering_unaveraged(x)
        batch_shape = x.shape[:-1]
        xb = x.reshape((-1, x.shape[-1]))
        # the autograd node only when a gradient can flow (it costs host time per call)
        if torch.is_grad_enabled() and xb.requires_grad:
            S = _autograd.CascadeFn.apply(xb, self)
        else:
            S = self._forward_raw(xb)
        S = S.reshape(tuple(batch_shape) + tuple(S.shape[-2:]))
        if self.out_type == 'array':
            return S
        keys = self._paths()
        if self.out_type == 'dict':
            return {k: S[..., c, :] for c, k in enumerate(keys)}
        out = []
        for c, k in enumerate(keys):
            j = tuple(self.psi1_f[k[0]]['j'] if i == 0 else self.psi2_f[k[1]]['j'] for i in range(len(k)))
            out.append({'coef': S[..., c, :], 'j': j, 'n': k, 'order': len(k)})
        return out

    def _op_filters(self):
        """The registered buffers as the filter dicts of the op-level cascade:
        [phi, psi1 bank, psi2 bank] with 'levels' the device tensors."""
        n = 0
        phi = dict(self.phi_f)
        phi['levels'] = [getattr(self, 'tensor%d' % (n + i)) for i in range(self._nlev['phi'])]
        n += self._nlev['phi']
        banks = []
        for key, meta in (('psi1', self.psi1_f), ('psi2', self.psi2_f)):
            bank = []
            for p, nl in zip(meta, self._nlev[key]):
                d = dict(p)
                d['levels'] = [getattr(self, 'tensor%d' % (n + i)) for i in range(nl)]
                n += nl
                bank.append(d)
            banks.append(bank)
        return [phi] + banks

    def _scattering_unaveraged(self, x):
        """T=0 (no averaging) and T='global' (sum over time), run op by op on
        this package's CUDA op surface (``backend1d``): the reference frontend
        kymatio/scattering1d/frontend/base_frontend.py:108-155 over the core
        kymatio/scattering1d/core/scattering1d.py:2-107 with average_local
        False.  Gradients flow through the ops' autograd rules."""
        from . import core
        from .backend import backend1d as B
        batch_shape = tuple(x.shape[:-1])
        signal_shape = tuple(x.shape[-1:])
        U_0 = B.pad(B.reshape_input(x.contiguous(), signal_shape), pad_left=self.pad_left, pad_right=self.pad_right)
        filters = self._op_filters()[:1 + self.max_order]
        S = {} if self.out_type == 'dict' else []
        for path in core.scattering1d(U_0, B, filters, self.J, False):
            path['order'] = len(path['n'])
            res = max(path['j'][-1] - self._oversampling, 0) if path['order'] > 0 else 0
            if self.average == 'global':
                coef = B.average_global(path['coef'])
            else:
                coef = B.unpad(path['coef'], self.ind_start[res], self.ind_end[res])
            path['coef'] = B.reshape_output(coef, batch_shape, n_kept_dims=1)
            if self.out_type == 'dict':
                S[path['n']] = path['coef']
            else:
                S.append(path)
        if self.out_type == 'dict':
            return S
        S.sort(key=lambda p: (p['order'], p['n']))
        if self.out_type == 'array':
            return B.stack([p['coef'] for p in S], dim=-2)
        return S

    def _forward_raw(self, x):
        plan = self._get_plan()
        lib = _lib.load()
        B = x.shape[0]
        out = torch.empty((B, self._channels, self._out_len), dtype=torch.float32, device=x.device)
        if B == 0:
            return out
        with torch.cuda.device(x.device):
            ptrs = self._filter_ptrs()
            ws_bytes = lib.kym_s1d_workspace_bytes(plan.h, B)
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=x.device)
            stream = torch.cuda.current_stream(x.device).cuda_stream
            _lib.check(lib.kym_s1d_forward(plan.h, x.data_ptr(), out.data_ptr(), B, ptrs, self._n_filters,
                                           ws.data_ptr(), ws_bytes, stream), 'kym_s1d_forward')
        return out

    # -- saved-activation form (autograd) -----------------------------------
    #: bytes of saved modulus inputs above which the backward recomputes them
    activation_budget = _autograd.DEFAULT_ACTIVATION_BUDGET

    def _saved_bytes(self, B):
        return _lib.load().kym_s1d_saved_bytes(self._get_plan().h, B)

    def _forward_save_raw(self, x):
        """Forward that also keeps every path's modulus input."""
        return _autograd.forward_save(_lib.load(), 's1d', self, self._get_plan(), x,
                                      (x.shape[0], self._channels, self._out_len))

    def _backward_saved_raw(self, saved, grad, x_shape):
        return _autograd.backward_saved(_lib.load(), 's1d', self, self._get_plan(), saved, grad, x_shape)

    def _backward_raw(self, x, grad):
        """grad_x = J^T grad through kym_s1d_backward (hand-written adjoints)."""
        plan = self._get_plan()
        lib = _lib.load()
        B = x.shape[0]
        gx = torch.empty_like(x)
        if B == 0:
            return gx
        with torch.cuda.device(x.device):
            ptrs = self._filter_ptrs()
            ws_bytes = lib.kym_s1d_backward_workspace_bytes(plan.h, B)
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=x.device)
            stream = torch.cuda.current_stream(x.device).cuda_stream
            _lib.check(lib.kym_s1d_backward(plan.h, x.data_ptr(), grad.data_ptr(), gx.data_ptr(), B, ptrs,
                                            self._n_filters, ws.data_ptr(), ws_bytes, stream), 'kym_s1d_backward')
        return gx
