"""Scattering2D: drop-in for kymatio's ScatteringTorch2D on one GB300.

Constructor, registered buffers (``tensor0..tensorK``, shape (m, n, 1), in
the order of kymatio/scattering2d/frontend/torch_frontend.py:28-43), input
validation and error messages (:72-111, kymatio/frontend/torch_frontend.py:
13-18, kymatio/backend/torch_backend.py:102-107) and output layout
(S0, S1 over n1, S2 over (n1, n2) with j2 > j1, n1-major; or a list of
dicts with 'coef', 'j', 'n', 'theta') follow the reference.  The transform
itself is one fused CUDA cascade (kym_s2d_forward) on the tensor's device
and torch's current stream; CPU tensors are rejected, there is no fallback.
"""
import contextlib

import torch
import torch.nn as nn

from . import _autograd, _lib
from .filter_bank import filter_bank_2d, filter_bank_2d_device, padded_size_2d, separable_lowpass


class Scattering2D(nn.Module):
    """2-D scattering transform (Mallat) with Morlet wavelets.

    Parameters follow kymatio.torch.Scattering2D: J (log2 scale), shape (M, N),
    L (orientations, default 8), max_order (1 or 2), pre_pad (input already
    padded to the padded size), backend, out_type ('array' or 'list').

    backend='torch' (default) runs the plain FP32 cascade.  backend='torch_tc'
    selects the tensor-core split-precision form: paths without children
    compute their low-pass branch as a separable product on tcgen05 (BF16
    hi/lo operands, FP32 accumulation); ``tensor_cores`` toggles it later.

    filters='host' (default) builds the filter bank on the host, bit for bit
    the reference's; filters='device' builds it on the current CUDA device
    (FP64, rounded to float32: equal to float32 rounding) and registers the
    buffers there, which takes milliseconds instead of seconds at large sizes.
    """

    def __init__(self, J, shape, L=8, max_order=2, pre_pad=False, backend='torch', out_type='array', filters='host'):
        super().__init__()
        self.frontend_name = 'torch'
        if backend is not None and not isinstance(backend, str) and \
                not str(getattr(backend, 'name', '')).startswith('torch'):
            raise ImportError('The backend ' + str(getattr(backend, 'name', backend)) +
                              ' is not supported by the frontend torch.')
        self.backend = backend
        self.J, self.L, self.max_order = int(J), int(L), int(max_order)
        self.pre_pad, self.out_type = pre_pad, out_type
        self.shape = tuple(int(s) for s in shape)
        M, N = self.shape
        if 2 ** self.J > M or 2 ** self.J > N:
            raise RuntimeError('The smallest dimension should be larger than 2^J.')
        self._M_padded, self._N_padded = padded_size_2d(M, N, self.J)
        self.pad_size = [(self._M_padded - M) // 2, (self._M_padded - M + 1) // 2,
                         (self._N_padded - N) // 2, (self._N_padded - N + 1) // 2]
        if filters == 'device':
            phi, psi = filter_bank_2d_device(self._M_padded, self._N_padded, self.J, self.L)
            as_buffer = lambda lv: lv.clone().unsqueeze(-1)  # noqa: E731
        elif filters == 'host':
            phi, psi = filter_bank_2d(self._M_padded, self._N_padded, self.J, self.L)
            as_buffer = lambda lv: torch.from_numpy(lv.copy()).unsqueeze(-1)  # noqa: E731
        else:
            raise ValueError("filters must be 'host' or 'device'")
        self.phi = {'levels': list(phi), 'j': self.J}
        self.psi = [{'levels': list(p['levels']), 'j': p['j'], 'theta': p['theta']} for p in psi]
        n = 0
        for lv in self.phi['levels']:
            self.register_buffer('tensor' + str(n), as_buffer(lv))
            n += 1
        for p in self.psi:
            for lv in p['levels']:
                self.register_buffer('tensor' + str(n), as_buffer(lv))
                n += 1
        self._n_filters = n
        self._plan = None
        self._ptr_cache = (None, None)
        self._lp_cache = (None, None, None)
        self._meta = self._path_meta()
        self.tensor_cores = isinstance(backend, str) and backend in ('torch_tc', 'torch_split')
        # separable factors of every low-pass level (non-persistent: derived from tensor{j})
        s_r, s_c = self._M_padded // 2 ** self.J, self._N_padded // 2 ** self.J
        for j, lv in enumerate(self.phi['levels']):
            dev = lv.device if torch.is_tensor(lv) else torch.device('cpu')
            lvh = lv.cpu().numpy() if torch.is_tensor(lv) else lv
            Tr, Tc, _ = separable_lowpass(lvh, 1, s_r - 2, 1, s_c - 2, 2 ** (self.J - j), 2 ** (self.J - j))
            self.register_buffer('lowpass_r' + str(j), torch.from_numpy(Tr.astype('float32')).to(dev),
                                 persistent=False)
            self.register_buffer('lowpass_c' + str(j), torch.from_numpy(Tc.astype('float32')).to(dev),
                                 persistent=False)
        self.register_buffer('_tc_status', torch.zeros(1, dtype=torch.int32, device=self.tensor0.device),
                             persistent=False)

    # -- plan ---------------------------------------------------------------
    def _get_plan(self):
        if self._plan is None:
            lib = _lib.load()
            h = _lib._vp()
            _lib.check(lib.kym_s2d_plan_create(self.shape[0], self.shape[1], self.J, self.L, self.max_order,
                                               int(bool(self.pre_pad)), _lib.ctypes.byref(h)),
                       'kym_s2d_plan_create')
            self._plan = _Plan(lib, h.value, lib.kym_s2d_plan_destroy)
            ints = [_lib.ctypes.c_int() for _ in range(6)]
            _lib.check(lib.kym_s2d_plan_info(self._plan.h, *[_lib.ctypes.byref(i) for i in ints]),
                       'kym_s2d_plan_info')
            self._channels, self._out_hw = ints[2].value, (ints[3].value, ints[4].value)
            if ints[5].value != self._n_filters:
                raise RuntimeError('filter bank layout mismatch')
        return self._plan

    def set_chunk(self, chunk):
        """Images per order-2 pass (autotuned); bounds the workspace."""
        _lib.check(_lib.load().kym_s2d_set_chunk(self._get_plan().h, int(chunk)), 'kym_s2d_set_chunk')

    def _path_meta(self):
        meta = [{'j': (), 'n': (), 'theta': ()}]
        for n1, p in enumerate(self.psi):
            meta.append({'j': (p['j'],), 'n': (n1,), 'theta': (p['theta'],)})
        if self.max_order >= 2:
            for n1, p1 in enumerate(self.psi):
                for n2, p2 in enumerate(self.psi):
                    if p2['j'] > p1['j']:
                        meta.append({'j': (p1['j'], p2['j']), 'n': (n1, n2), 'theta': (p1['theta'], p2['theta'])})
        return meta

    def _filter_ptrs(self):
        # the table is rebuilt whenever any buffer's address changed (.to(),
        # reassignment, a swapped .data); the names are formatted once
        names = self.__dict__.get('_filter_names')
        if names is None or len(names) != self._n_filters:
            names = self.__dict__['_filter_names'] = ['tensor' + str(i) for i in range(self._n_filters)]
        bufs = self._buffers
        key = tuple(bufs[n].data_ptr() for n in names)
        if self._ptr_cache[0] == key:
            return self._ptr_cache[1]
        bufs = [getattr(self, n) for n in names]
        if self._ptr_cache[0] != key:
            for b in bufs:
                if not b.is_cuda or b.dtype != torch.float32 or not b.is_contiguous():
                    raise TypeError('The filters must be contiguous float32 CUDA tensors; call .cuda() on the '
                                    'module (the GB300 engine runs on CUDA only).')
            self._ptr_cache = (key, _lib.ptr_array(list(key)))
        return self._ptr_cache[1]

    # -- forward ------------------------------------------------------------
    def forward(self, x):
        if x is None:
            raise TypeError('The input should be not empty.')
        if torch.is_tensor(x) and not x.is_contiguous():
            raise RuntimeError('Tensors must be contiguous.')
        return self.scattering(x)

    def scattering(self, input):
        if not torch.is_tensor(input):
            raise TypeError('The input should be a PyTorch Tensor.')
        if len(input.shape) < 2:
            raise RuntimeError('Input tensor must have at least two dimensions.')
        if not input.is_contiguous():
            raise RuntimeError('Tensor must be contiguous.')
        if (input.shape[-1] != self.shape[-1] or input.shape[-2] != self.shape[-2]) and not self.pre_pad:
            raise RuntimeError('Tensor must be of spatial size (%i,%i).' % (self.shape[0], self.shape[1]))
        if (input.shape[-1] != self._N_padded or input.shape[-2] != self._M_padded) and self.pre_pad:
            raise RuntimeError('Padded tensor must be of spatial size (%i,%i).' % (self._M_padded, self._N_padded))
        if self.out_type not in ('array', 'list'):
            raise RuntimeError("The out_type must be one of 'array' or 'list'.")
        if not input.is_cuda:
            raise TypeError('The input must be a CUDA tensor: the GB300 scattering engine runs on CUDA only.')
        if input.dtype != torch.float32:
            raise TypeError('The input must be float32 (got %s).' % input.dtype)
        batch_shape = input.shape[:-2]
        x = input.reshape((-1,) + tuple(input.shape[-2:]))
        # the autograd node only when a gradient can flow (it costs host time per call)
        if torch.is_grad_enabled() and x.requires_grad:
            S = _autograd.CascadeFn.apply(x, self)
        else:
            S = self._forward_raw(x)
        S = S.reshape(tuple(batch_shape) + tuple(S.shape[-3:]))
        if self.out_type == 'array':
            return S
        return [dict(m, coef=S[..., c, :, :]) for c, m in enumerate(self._meta)]

    def _lowpass_ptrs(self):
        r = [getattr(self, 'lowpass_r' + str(j)) for j in range(self.J)]
        c = [getattr(self, 'lowpass_c' + str(j)) for j in range(self.J)]
        key = tuple(t.data_ptr() for t in r + c)
        if self._lp_cache[0] != key:
            for t in r + c:
                if not t.is_cuda or t.dtype != torch.float32 or not t.is_contiguous():
                    raise TypeError('The low-pass factors must be contiguous float32 CUDA tensors.')
            self._lp_cache = (key, _lib.ptr_array([t.data_ptr() for t in r]), _lib.ptr_array([t.data_ptr() for t in c]))
        return self._lp_cache[1], self._lp_cache[2]

    def tensor_core_status(self, reset=True):
        """Non-zero when a tensor-core completion wait ran out (outputs are NaN then)."""
        v = int(self._tc_status.item())
        if reset:
            self._tc_status.zero_()
        return v

    def _forward_raw(self, x):
        """(B, M, N) float32 CUDA -> (B, C, m, n) through kym_s2d_forward (or
        kym_s2d_forward_tc with tensor_cores)."""
        plan = self._get_plan()
        lib = _lib.load()
        B = x.shape[0]
        out = torch.empty((B, self._channels) + self._out_hw, dtype=torch.float32, device=x.device)
        if B == 0:
            return out
        with _on_device(x.device):
            ptrs = self._filter_ptrs()
            ws_bytes = lib.kym_s2d_workspace_bytes(plan.h, B)
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=x.device)
            stream = torch.cuda.current_stream(x.device).cuda_stream
            if self.tensor_cores:
                lr, lc = self._lowpass_ptrs()
                _lib.check(lib.kym_s2d_forward_tc(plan.h, x.data_ptr(), out.data_ptr(), B, ptrs, self._n_filters,
                                                  lr, lc, self.J, ws.data_ptr(), ws_bytes,
                                                  self._tc_status.data_ptr(), stream, None, 0),
                           'kym_s2d_forward_tc')
            else:
                _lib.check(lib.kym_s2d_forward(plan.h, x.data_ptr(), out.data_ptr(), B, ptrs, self._n_filters,
                                               ws.data_ptr(), ws_bytes, stream), 'kym_s2d_forward')
        return out

    def forward_host(self, x, out=None, parts=1, sync=True):
        """End-to-end forward between host tensors: x a CPU float32 tensor
        (..., M, N), returns (..., C, m, n) on the host (in ``out``, or a new
        page-locked tensor).  The input goes to the module's device in
        ``parts`` slices and each launch group's channels come back as soon as
        the group has finished (kym_s2d_forward_host), so the transfers
        overlap the cascade; page-locked inputs (``x.pin_memory()``) overlap
        best.  Tensor-core form when ``tensor_cores``.  With ``sync=False`` the
        call returns once the work is queued on the current stream:
        synchronise before reading the result; calls queued back to back
        alternate between two device staging buffers kept by the module (for
        the last batch size), so a call's input copy overlaps the previous
        call's cascade."""
        if not torch.is_tensor(x) or x.is_cuda or x.dtype != torch.float32 or not x.is_contiguous():
            raise TypeError('forward_host takes a contiguous float32 CPU tensor.')
        hw = (self._M_padded, self._N_padded) if self.pre_pad else self.shape
        if len(x.shape) < 2 or tuple(x.shape[-2:]) != hw:
            raise RuntimeError('Tensor must be of spatial size (%i,%i).' % hw)
        dev = self.tensor0.device
        if dev.type != 'cuda':
            raise TypeError('The module must be on a CUDA device: the GB300 scattering engine runs on CUDA only.')
        plan, lib = self._get_plan(), _lib.load()
        xb = x.reshape((-1,) + hw)
        B = xb.shape[0]
        shape = tuple(x.shape[:-2]) + (self._channels,) + self._out_hw
        if out is None:
            out = torch.empty(shape, dtype=torch.float32, pin_memory=True)
        elif out.is_cuda or out.dtype != torch.float32 or not out.is_contiguous() or tuple(out.shape) != shape:
            raise TypeError('out must be a contiguous float32 CPU tensor of shape %s.' % (shape,))
        if B == 0:
            return out
        with torch.cuda.device(dev):
            ring = self.__dict__.get('_host_ring')
            if ring is None or ring['key'] != (B, dev):
                # two staging slots: (device input, device output, event after the last call using them)
                ring = self.__dict__['_host_ring'] = {
                    'key': (B, dev), 'turn': 0,
                    'slots': [[torch.empty((B,) + hw, dtype=torch.float32, device=dev),
                               torch.empty((B, self._channels) + self._out_hw, dtype=torch.float32, device=dev),
                               None] for _ in range(2)]}
            slot = ring['slots'][ring['turn']]
            ring['turn'] ^= 1
            x_dev, out_dev, free = slot
            ws_bytes = lib.kym_s2d_workspace_bytes(plan.h, B)
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=dev)
            cur = torch.cuda.current_stream(dev)
            lr = lc = status = None
            if self.tensor_cores:
                lr, lc = self._lowpass_ptrs()
                status = self._tc_status.data_ptr()
            _lib.check(lib.kym_s2d_forward_host(plan.h, xb.data_ptr(), out.data_ptr(), B, self._filter_ptrs(),
                                                self._n_filters, lr, lc, self.J, status, x_dev.data_ptr(),
                                                out_dev.data_ptr(), ws.data_ptr(), ws_bytes, int(parts),
                                                free.cuda_event if free is not None else None, cur.cuda_stream),
                       'kym_s2d_forward_host')
            if free is None:
                free = slot[2] = torch.cuda.Event()
            free.record(cur)
            if sync:
                cur.synchronize()
        return out

    def group_times(self, x, steps=3):
        """CUDA-event time (ms) of every launch group of the cascade in one
        forward of x, averaged over ``steps`` forwards (profiling, autotuning)."""
        import ctypes
        plan, lib = self._get_plan(), _lib.load()
        ng = lib.kym_s2d_group_count(plan.h)
        gms = (ctypes.c_float * ng)()
        B = x.shape[0]
        acc = [0.0] * ng
        with torch.cuda.device(x.device):
            out = torch.empty((B, self._channels) + self._out_hw, dtype=torch.float32, device=x.device)
            ptrs = self._filter_ptrs()
            ws_bytes = lib.kym_s2d_workspace_bytes(plan.h, B)
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=x.device)
            stream = torch.cuda.current_stream(x.device).cuda_stream
            for _ in range(steps):
                if self.tensor_cores:
                    lr, lc = self._lowpass_ptrs()
                    _lib.check(lib.kym_s2d_forward_tc(plan.h, x.data_ptr(), out.data_ptr(), B, ptrs, self._n_filters,
                                                      lr, lc, self.J, ws.data_ptr(), ws_bytes,
                                                      self._tc_status.data_ptr(), stream, gms, ng),
                               'kym_s2d_forward_tc')
                else:
                    _lib.check(lib.kym_s2d_forward_timed(plan.h, x.data_ptr(), out.data_ptr(), B, ptrs,
                                                         self._n_filters, ws.data_ptr(), ws_bytes, stream, gms, ng),
                               'kym_s2d_forward_timed')
                acc = [a + gms[i] for i, a in enumerate(acc)]
        return [a / steps for a in acc]

    def set_group_tensor_cores(self, mask):
        """In the tensor-core form, run launch group g in its tensor-core kernel
        when mask[g] is true, else in the plain FP32 kernel (more precise, so
        within the form's bar); the autotuner picks the mask by timing."""
        plan, lib = self._get_plan(), _lib.load()
        for g, on in enumerate(mask):
            if lib.kym_s2d_set_group_tc(plan.h, g, int(bool(on))) < 0:
                raise ValueError('no launch group %d' % g)

    def _backward_raw(self, x, grad):
        """grad_x = J^T grad through kym_s2d_backward (hand-written adjoints)."""
        plan = self._get_plan()
        lib = _lib.load()
        B = x.shape[0]
        gx = torch.empty_like(x)
        if B == 0:
            return gx
        with torch.cuda.device(x.device):
            ptrs = self._filter_ptrs()
            ws_bytes = lib.kym_s2d_backward_workspace_bytes(plan.h, B)
            ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=x.device)
            stream = torch.cuda.current_stream(x.device).cuda_stream
            _lib.check(lib.kym_s2d_backward(plan.h, x.data_ptr(), grad.data_ptr(), gx.data_ptr(), B, ptrs,
                                            self._n_filters, ws.data_ptr(), ws_bytes, stream), 'kym_s2d_backward')
        return gx

    # -- saved-activation form (autograd) -----------------------------------
    #: bytes of saved modulus inputs above which the backward recomputes them
    activation_budget = _autograd.DEFAULT_ACTIVATION_BUDGET

    def _saved_bytes(self, B):
        return _lib.load().kym_s2d_saved_bytes(self._get_plan().h, B)

    def _forward_save_raw(self, x):
        """Plain FP32 forward that also keeps every path's modulus input."""
        plan = self._get_plan()
        return _autograd.forward_save(_lib.load(), 's2d', self, plan, x,
                                      (x.shape[0], self._channels) + self._out_hw)

    def _backward_saved_raw(self, saved, grad, x_shape):
        return _autograd.backward_saved(_lib.load(), 's2d', self, self._get_plan(), saved, grad, x_shape)

    def extra_repr(self):
        return 'J={}, shape={}, L={}, max_order={}, pre_pad={}, out_type={!r}'.format(
            self.J, self.shape, self.L, self.max_order, self.pre_pad, self.out_type)


def _on_device(device):
    """torch.cuda.device(device), skipped when it is already current."""
    if device.index is None or device.index == torch.cuda.current_device():
        return contextlib.nullcontext()
    return torch.cuda.device(device)


class _Plan:
    """Owns a C plan handle."""

    def __init__(self, lib, h, destroy):
        self.h, self._destroy = h, destroy

    def __del__(self):
        try:
            self._destroy(self.h)
        except Exception:
            pass
