"""Joint time-frequency scattering against the reference's FP64 outputs
(tests/golden/ref_jtfs.npz, from kymatio's numpy TimeFrequencyScattering).

On CPU the cascade of kymatio_gb300.jtfs runs over a float64 test double of
the op surface (torch CPU), which pins the restated algorithm, the frequency
filter bank, the formats and meta(); on the GPU the module runs over the
CUDA op surface."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2

torch = pytest.importorskip('torch')

_D = np.load(os.path.join(GOLDEN, 'ref_jtfs.npz'))
CASES = json.loads(str(_D['meta']))


def _kwargs(case):
    kw = dict(case['kwargs'])
    for k in ('Q', 'Q_fr'):
        if isinstance(kw.get(k), list):
            kw[k] = tuple(kw[k])
    return kw


class CpuOps:
    """Float64 test double of the 1-D op surface on CPU tensors: trailing dim
    2 is complex, 1 is real; transforms run along dim -2."""

    @staticmethod
    def _z(x):
        return torch.view_as_complex(x.contiguous())

    @classmethod
    def rfft(cls, x):
        return torch.view_as_real(torch.fft.fft(x[..., 0].to(torch.complex128), dim=-1))

    @classmethod
    def cfft(cls, x):
        return torch.view_as_real(torch.fft.fft(cls._z(x), dim=-1))

    @classmethod
    def ifft(cls, x):
        return torch.view_as_real(torch.fft.ifft(cls._z(x), dim=-1))

    @classmethod
    def irfft(cls, x):
        return torch.fft.ifft(cls._z(x), dim=-1).real[..., None]

    @staticmethod
    def cdgmm(A, B):
        return A * B.to(A.dtype)

    @staticmethod
    def modulus(x):
        return torch.sqrt(x[..., 0] ** 2 + x[..., 1] ** 2)[..., None]

    @staticmethod
    def subsample_fourier(x, k):
        n = x.shape[-2]
        return x.reshape(x.shape[:-2] + (k, n // k, 2)).mean(dim=-3)

    @staticmethod
    def pad(x, pad_left, pad_right):
        return torch.nn.functional.pad(x, (pad_left, pad_right), mode='reflect')[..., None]

    @staticmethod
    def unpad(x, i0, i1):
        return x.reshape(x.shape[:-1])[..., i0:i1]

    @staticmethod
    def stack(arrays, dim=2):
        return torch.stack(arrays, dim=dim)

    @staticmethod
    def average_global(x):
        return x.sum(dim=-2, keepdim=True)

    @staticmethod
    def pad_frequency(x, padding):
        return torch.nn.functional.pad(x, (0, 0, 0, padding))

    @staticmethod
    def swap_time_frequency(x):
        return x.transpose(-2, -3).contiguous()

    @staticmethod
    def unpad_frequency(x, n1_max, n1_stride):
        return x[:, :, :1 + n1_max // n1_stride, :]

    @staticmethod
    def split_frequency_axis(x):
        return torch.split(x, 1, dim=-3)

    @staticmethod
    def reshape_input(x, signal_shape):
        return x.reshape((-1, 1) + tuple(signal_shape))

    @staticmethod
    def reshape_output(S, batch_shape, n_kept_dims):
        return S.reshape(tuple(batch_shape) + tuple(S.shape[-n_kept_dims:]))


def _check(name, out, tol):
    if isinstance(out, (list, dict)):
        items = out.items() if isinstance(out, dict) else ((p['n'], p['coef']) for p in out)
        got = {tuple(k): v for k, v in items}
        keys = sorted(k.split('/S/')[1] for k in _D.files if k.startswith(name + '/S/'))
        assert len(got) == len(keys)
        for key in keys:
            n = tuple(int(v) for v in key.split(',')) if key else ()
            ref = _D[name + '/S/' + key]
            g = got[n].detach().cpu().numpy()
            assert g.shape == ref.shape, (n, g.shape, ref.shape)
            assert rel_l2(g, ref) <= tol, (n, rel_l2(g, ref))
    else:
        ref = _D[name + '/S']
        g = out.detach().cpu().numpy()
        assert g.shape == ref.shape, (g.shape, ref.shape)
        assert rel_l2(g, ref) <= tol, rel_l2(g, ref)


@pytest.mark.parametrize('case', CASES, ids=lambda c: c['name'])
def test_jtfs_cascade_on_cpu_double(case):
    from kymatio_gb300.jtfs import TimeFrequencyScattering
    S = TimeFrequencyScattering(**_kwargs(case))
    x = torch.from_numpy(_D[case['name'] + '/x']).double()
    _check(case['name'], S._jtfs(x, CpuOps), 1e-6)  # float32 filters, float64 arithmetic


@pytest.mark.parametrize('case', CASES, ids=lambda c: c['name'])
def test_jtfs_meta(case):
    from kymatio_gb300.jtfs import TimeFrequencyScattering
    S = TimeFrequencyScattering(**_kwargs(case))
    m = S.meta()
    name = case['name']
    assert [list(k) for k in m['key']] == json.loads(str(_D[name + '/meta/key']))
    for field in ('order', 'n_fr', 'spin', 'xi_fr', 'sigma_fr', 'j_fr', 'xi', 'sigma', 'j'):
        np.testing.assert_allclose(np.asarray(m[field], dtype=np.float64), _D[name + '/meta/' + field],
                                   rtol=1e-12, atol=0, equal_nan=True, err_msg=field)

    def n_json(v):  # a range as its list, NaN as null, an index as int
        if isinstance(v, range):
            return list(v)
        if isinstance(v, float) and v != v:
            return None
        return int(v)
    assert [[n_json(v) for v in row] for row in m['n']] == json.loads(str(_D[name + '/meta/n']))
    assert S.output_size() == len(m['key'])


def test_jtfs_argument_errors():
    from kymatio_gb300.jtfs import TimeFrequencyScattering
    with pytest.raises(ValueError, match='Q_fr must be >= 1'):
        TimeFrequencyScattering(J=4, J_fr=2, Q=2, shape=256, Q_fr=0)
    with pytest.raises(NotImplementedError, match='Q_fr must be an integer or 1-tuple'):
        TimeFrequencyScattering(J=4, J_fr=2, Q=2, shape=256, Q_fr=(1, 1))
    S = TimeFrequencyScattering(J=4, J_fr=2, Q=2, shape=256, F=0, format='joint')
    with pytest.raises(ValueError, match="Cannot convert to format='joint'"):
        S._check_runtime_args_fr()
    with pytest.raises(ValueError, match='The support F of the low-pass filter'):
        TimeFrequencyScattering(J=4, J_fr=2, Q=2, shape=256, F=1000).F


@pytest.mark.gpu
@pytest.mark.parametrize('case', CASES, ids=lambda c: c['name'])
def test_jtfs_on_gpu(case):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300.jtfs import TimeFrequencyScattering
    dev = torch.device('cuda:0')
    S = TimeFrequencyScattering(**_kwargs(case)).to(dev)
    x = torch.from_numpy(_D[case['name'] + '/x']).to(dev)
    _check(case['name'], S(x), 1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize('case', [c for c in CASES if c['kwargs'].get('out_type', 'array') == 'array'],
                         ids=lambda c: c['name'])
def test_jtfs_graph_replay(case):
    """graph=True replays a CUDA graph of the whole forward: the reference's
    outputs on the golden input, then the eager forward on new data, twice."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300.jtfs import TimeFrequencyScattering
    dev = torch.device('cuda:0')
    S = TimeFrequencyScattering(**_kwargs(case), graph=True).to(dev)
    x = torch.from_numpy(_D[case['name'] + '/x']).to(dev)
    out = S(x)
    assert len(S._graphs) == 1
    _check(case['name'], out, 1e-5)
    for _ in range(2):
        x2 = torch.rand_like(x)
        got = S(x2)
        S.graph = False
        ref = S(x2)
        S.graph = True
        assert torch.equal(got, ref)
    assert torch.equal(out, S(x))  # earlier results are copies, not the graph's buffers


GRAD_CASES = [c for c in CASES if c['name'] + '/gx' in _D.files]


@pytest.mark.parametrize('case', GRAD_CASES, ids=lambda c: c['name'])
def test_jtfs_gradient_on_cpu_double(case):
    """d<g, S(x)>/dx through the restated cascade (torch autograd over the
    float64 double) against the reference torch frontend's gradient."""
    from kymatio_gb300.jtfs import TimeFrequencyScattering
    name = case['name']
    S = TimeFrequencyScattering(**_kwargs(case))
    x = torch.from_numpy(_D[name + '/x']).double().requires_grad_()
    S._jtfs(x, CpuOps).backward(torch.from_numpy(_D[name + '/g']).double())
    assert rel_l2(x.grad.numpy(), _D[name + '/gx']) <= 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize('case', GRAD_CASES, ids=lambda c: c['name'])
def test_jtfs_gradient_on_gpu(case):
    """The same gradient through the CUDA ops' adjoints (FFTs, wavelet
    products, periodisation, modulus, reflect padding)."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300.jtfs import TimeFrequencyScattering
    dev = torch.device('cuda:0')
    name = case['name']
    S = TimeFrequencyScattering(**_kwargs(case)).to(dev)
    x = torch.from_numpy(_D[name + '/x']).to(dev).requires_grad_()
    S(x).backward(torch.from_numpy(_D[name + '/g']).to(dev))
    assert rel_l2(x.grad.cpu().numpy(), _D[name + '/gx']) <= 1e-5
