"""The reference backend operator surface on GB300 kernels.

``backend2d`` and ``backend1d`` are drop-ins for kymatio's
``TorchBackend2D`` (kymatio/scattering2d/backend/torch_backend.py:89-183) and
``TorchBackend1D`` (kymatio/scattering1d/backend/torch_backend.py:126-226),
with the checks and error messages of ``TorchBackend``
(kymatio/backend/torch_backend.py:99-232).  Their ``name`` starts with
'torch', so the reference frontends accept them:

    kymatio.Scattering2D(J, shape, frontend='torch', backend=backend2d)

Every arithmetic op (pad, FFTs, cdgmm, modulus, periodisation) runs one of
this package's CUDA kernels through the C ABI (kym_op_*), with a hand-written
adjoint for autograd; unpad and stack are views/copies as in the reference.
Only float32 CUDA tensors are accepted.
"""
import torch
from torch.autograd import Function

from . import _lib


def _stream(t):
    return torch.cuda.current_stream(t.device).cuda_stream


def _require_cuda_f32(x):
    if not x.is_cuda:
        raise TypeError('The input must be a CUDA tensor: the GB300 backend runs on CUDA only.')
    if x.dtype != torch.float32:
        raise TypeError('The GB300 backend computes in float32 (got %s).' % x.dtype)


def _batch(shape, n_trailing):
    b = 1
    for s in shape[:len(shape) - n_trailing]:
        b *= s
    return b


def _fft(x, in_real, out_real, inverse, scale, M, N):
    """Batched 2-D (M > 1) or 1-D (M == 1) DFT over the trailing image dims."""
    lib = _lib.load()
    batch = _batch(x.shape, 3 if M > 1 else 2)
    out = torch.empty(x.shape[:-1] + ((1,) if out_real else (2,)), dtype=torch.float32, device=x.device)
    with torch.cuda.device(x.device):
        _lib.check(lib.kym_op_fft2(x.data_ptr(), out.data_ptr(), batch, M, N, int(in_real), int(out_real),
                                   int(inverse), float(scale), _stream(x)), 'kym_op_fft2')
    return out


class _FFTFn(Function):
    """y = scale * T(x), T the unnormalised DFT (inverse: conjugate direction).
    Adjoint: the conjugate direction with the same scale (real parts where
    the input was real)."""

    @staticmethod
    def forward(ctx, x, in_real, out_real, inverse, scale, M, N):
        ctx.cfg = (in_real, out_real, inverse, scale, M, N)
        return _fft(x, in_real, out_real, inverse, scale, M, N)

    @staticmethod
    def backward(ctx, g):
        in_real, out_real, inverse, scale, M, N = ctx.cfg
        g = g.contiguous()
        if out_real:
            g = torch.cat([g, torch.zeros_like(g)], dim=-1)
        return _fft(g, False, in_real, not inverse, scale, M, N), None, None, None, None, None, None


def _image_dims(x, oned):
    if oned:
        return 1, x.shape[-2]
    return x.shape[-3], x.shape[-2]


class _ModulusFn(Function):
    @staticmethod
    def forward(ctx, x):
        ctx.save_for_backward(x)
        y = torch.empty(x.shape[:-1], dtype=torch.float32, device=x.device)
        with torch.cuda.device(x.device):
            _lib.check(_lib.load().kym_op_modulus(x.data_ptr(), y.data_ptr(), y.numel(), _stream(x)), 'kym_op_modulus')
        return y

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        g = g.contiguous()
        gx = torch.empty_like(x)
        with torch.cuda.device(x.device):
            _lib.check(_lib.load().kym_op_modulus_backward(x.data_ptr(), g.data_ptr(), gx.data_ptr(), g.numel(),
                                                           _stream(x)), 'kym_op_modulus_backward')
        return gx


class _SubsampleFn(Function):
    @staticmethod
    def forward(ctx, x, kr, kc, M, N):
        ctx.cfg = (kr, kc, M, N)
        batch = _batch(x.shape, 3 if M > 1 else 2)
        y = torch.empty(x.shape[:-3] + (M // kr, N // kc, 2) if M > 1 else x.shape[:-2] + (N // kc, 2),
                        dtype=torch.float32, device=x.device)
        with torch.cuda.device(x.device):
            _lib.check(_lib.load().kym_op_subsample(x.data_ptr(), y.data_ptr(), batch, M, N, kr, kc, _stream(x)),
                       'kym_op_subsample')
        return y

    @staticmethod
    def backward(ctx, g):
        kr, kc, M, N = ctx.cfg
        g = g.contiguous()
        batch = _batch(g.shape, 3 if M > 1 else 2)
        gx = torch.empty(g.shape[:-3] + (M, N, 2) if M > 1 else g.shape[:-2] + (N, 2), dtype=torch.float32,
                         device=g.device)
        with torch.cuda.device(g.device):
            _lib.check(_lib.load().kym_op_subsample_adjoint(g.data_ptr(), gx.data_ptr(), batch, M, N, kr, kc,
                                                            _stream(g)), 'kym_op_subsample_adjoint')
        return gx, None, None, None, None


class _PadFn(Function):
    @staticmethod
    def forward(ctx, x, top, bottom, left, right):
        M, N = x.shape[-2], x.shape[-1]
        ctx.cfg = (M, N, top, bottom, left, right)
        batch = _batch(x.shape, 2)
        y = torch.empty(x.shape[:-2] + (M + top + bottom, N + left + right), dtype=torch.float32, device=x.device)
        with torch.cuda.device(x.device):
            _lib.check(_lib.load().kym_op_reflect_pad(x.data_ptr(), y.data_ptr(), batch, M, N, top, bottom, left,
                                                      right, _stream(x)), 'kym_op_reflect_pad')
        return y

    @staticmethod
    def backward(ctx, g):
        M, N, top, bottom, left, right = ctx.cfg
        g = g.contiguous()
        batch = _batch(g.shape, 2)
        gx = torch.empty(g.shape[:-2] + (M, N), dtype=torch.float32, device=g.device)
        with torch.cuda.device(g.device):
            _lib.check(_lib.load().kym_op_reflect_pad_adjoint(g.data_ptr(), gx.data_ptr(), batch, M, N, top, bottom,
                                                              left, right, _stream(g)), 'kym_op_reflect_pad_adjoint')
        return gx, None, None, None, None


class _CdgmmFn(Function):
    @staticmethod
    def forward(ctx, A, B):
        complex_b = B.shape[-1] == 2
        ctx.save_for_backward(B)
        ctx.complex_b = complex_b
        n = B.numel() // (2 if complex_b else 1)
        batch = A.numel() // (2 * n)
        C = torch.empty_like(A)
        with torch.cuda.device(A.device):
            _lib.check(_lib.load().kym_op_cdgmm(A.data_ptr(), B.data_ptr(), C.data_ptr(), batch, n, int(complex_b),
                                                _stream(A)), 'kym_op_cdgmm')
        return C

    @staticmethod
    def backward(ctx, g):
        (B,) = ctx.saved_tensors
        g = g.contiguous()
        Bc = B
        if ctx.complex_b:
            Bc = torch.stack([B[..., 0], -B[..., 1]], dim=-1).contiguous()  # conjugate filter
        return _CdgmmFn.apply(g, Bc), None


class TorchGB300Backend:
    """Checks and shared ops (kymatio/backend/torch_backend.py:99-232)."""
    name = 'torch_gb300'

    @classmethod
    def input_checks(cls, x):
        if x is None:
            raise TypeError('The input should be not empty.')
        cls.contiguous_check(x)

    @classmethod
    def complex_check(cls, x):
        if not cls._is_complex(x):
            raise TypeError('The input should be complex (i.e. last dimension is 2).')

    @classmethod
    def real_check(cls, x):
        if not cls._is_real(x):
            raise TypeError('The input should be real.')

    @classmethod
    def complex_contiguous_check(cls, x):
        cls.complex_check(x)
        cls.contiguous_check(x)

    @staticmethod
    def contiguous_check(x):
        if not x.is_contiguous():
            raise RuntimeError('Tensors must be contiguous.')

    @staticmethod
    def _is_complex(x):
        return x.shape[-1] == 2

    @staticmethod
    def _is_real(x):
        return x.shape[-1] == 1

    @classmethod
    def modulus(cls, x):
        cls.complex_contiguous_check(x)
        _require_cuda_f32(x)
        return _ModulusFn.apply(x)[..., None]

    @staticmethod
    def stack(arrays, dim=2):
        return torch.stack(arrays, dim=dim)

    @classmethod
    def cdgmm(cls, A, B):
        if not cls._is_real(B):
            cls.complex_contiguous_check(B)
        else:
            cls.contiguous_check(B)
        cls.complex_contiguous_check(A)
        if A.shape[-len(B.shape):-1] != B.shape[:-1]:
            raise RuntimeError('The filters are not compatible for multiplication.')
        if A.dtype is not B.dtype:
            raise TypeError('Input and filter must be of the same dtype.')
        if B.device.type == 'cuda':
            if A.device.type == 'cuda':
                if A.device.index != B.device.index:
                    raise TypeError('Input and filter must be on the same GPU.')
            else:
                raise TypeError('Input must be on GPU.')
        if B.device.type == 'cpu':
            if A.device.type == 'cuda':
                raise TypeError('Input must be on CPU.')
        _require_cuda_f32(A)
        return _CdgmmFn.apply(A, B)

    @staticmethod
    def reshape_input(x, signal_shape):
        return x.reshape((-1, 1) + signal_shape)

    @staticmethod
    def reshape_output(S, batch_shape, n_kept_dims):
        return S.reshape(batch_shape + S.shape[-n_kept_dims:])

    @staticmethod
    def shape(x):
        return x.shape


class Pad:
    """Reflect padding to the scattering size, with a trailing real dim
    (kymatio/scattering2d/backend/torch_backend.py:19-86)."""

    def __init__(self, pad_size, input_size):
        self.pad_size = list(pad_size)
        self.input_size = input_size

    def __call__(self, x):
        _require_cuda_f32(x)
        x = x.contiguous()
        t, b, l, r = self.pad_size
        return _PadFn.apply(x, t, b, l, r)[..., None]


class TorchGB300Backend2D(TorchGB300Backend):
    Pad = Pad

    @classmethod
    def subsample_fourier(cls, x, k):
        cls.contiguous_check(x)
        cls.complex_check(x)
        _require_cuda_f32(x)
        M, N = x.shape[-3], x.shape[-2]
        return _SubsampleFn.apply(x, k, k, M, N)

    @classmethod
    def rfft(cls, x):
        cls.contiguous_check(x)
        cls.real_check(x)
        _require_cuda_f32(x)
        M, N = _image_dims(x, False)
        return _FFTFn.apply(x, True, False, False, 1.0, M, N)

    @classmethod
    def irfft(cls, x):
        cls.contiguous_check(x)
        cls.complex_check(x)
        _require_cuda_f32(x)
        M, N = _image_dims(x, False)
        return _FFTFn.apply(x, False, True, True, 1.0 / (M * N), M, N)

    @classmethod
    def ifft(cls, x):
        cls.contiguous_check(x)
        cls.complex_check(x)
        _require_cuda_f32(x)
        M, N = _image_dims(x, False)
        return _FFTFn.apply(x, False, False, True, 1.0 / (M * N), M, N)

    @staticmethod
    def unpad(in_):
        in_ = in_[..., 1:-1, 1:-1, :]
        return in_.reshape(in_.shape[:-1])

    @staticmethod
    def stack(arrays):
        return TorchGB300Backend.stack(arrays, -3)


class TorchGB300Backend1D(TorchGB300Backend):
    @classmethod
    def subsample_fourier(cls, x, k):
        cls.complex_check(x)
        _require_cuda_f32(x)
        x = x.contiguous()
        return _SubsampleFn.apply(x, 1, k, 1, x.shape[-2])

    @staticmethod
    def pad(x, pad_left, pad_right, mode='reflect'):
        if mode != 'constant':
            if (pad_left >= x.shape[-1]) or (pad_right >= x.shape[-1]):
                raise ValueError('Indefinite padding size (larger than tensor).')
        if mode != 'reflect':
            raise NotImplementedError('the GB300 backend pads in reflect mode')
        _require_cuda_f32(x)
        return _PadFn.apply(x.contiguous(), 0, 0, pad_left, pad_right)[..., None]

    @staticmethod
    def unpad(x, i0, i1):
        x = x.reshape(x.shape[:-1])
        return x[..., i0:i1]

    @classmethod
    def cfft(cls, x):
        cls.contiguous_check(x)
        cls.complex_check(x)
        _require_cuda_f32(x)
        return _FFTFn.apply(x, False, False, False, 1.0, 1, x.shape[-2])

    @classmethod
    def rfft(cls, x):
        cls.contiguous_check(x)
        cls.real_check(x)
        _require_cuda_f32(x)
        return _FFTFn.apply(x, True, False, False, 1.0, 1, x.shape[-2])

    @classmethod
    def irfft(cls, x):
        cls.contiguous_check(x)
        cls.complex_check(x)
        _require_cuda_f32(x)
        return _FFTFn.apply(x, False, True, True, 1.0 / x.shape[-2], 1, x.shape[-2])

    @classmethod
    def ifft(cls, x):
        cls.contiguous_check(x)
        cls.complex_check(x)
        _require_cuda_f32(x)
        return _FFTFn.apply(x, False, False, True, 1.0 / x.shape[-2], 1, x.shape[-2])

    @classmethod
    def average_global(cls, x):
        cls.contiguous_check(x)
        cls.real_check(x)
        return torch.sum(x, axis=-2, keepdims=True)

    # -- frequency-axis moves of time-frequency scattering
    #    (kymatio/scattering1d/backend/torch_backend.py:150-223): views and copies
    @classmethod
    def pad_frequency(cls, x, padding):
        """One-sided zero padding of the frequency axis (dim -2) to lower frequencies."""
        return torch.nn.functional.pad(x, (0, 0, 0, padding), mode='constant', value=0)

    @classmethod
    def swap_time_frequency(cls, x):
        """(..., frequency, time, 1|2) <-> (..., time, frequency, 1|2), contiguous."""
        return torch.transpose(x, dim0=-2, dim1=-3).contiguous()

    @staticmethod
    def unpad_frequency(x, n1_max, n1_stride):
        """Keep the 1 + n1_max // n1_stride first frequency bins (dim 2)."""
        return x[:, :, :1 + (n1_max // n1_stride), :]

    @staticmethod
    def split_frequency_axis(x):
        """One tensor per frequency bin (dim -3), each of size 1 there."""
        return torch.split(x, 1, dim=-3)


backend2d = TorchGB300Backend2D
backend1d = TorchGB300Backend1D
