"""The backend operator surface (kymatio_gb300.backend) on GPU: the reference's
op known-answer tests (tests/scattering2d/test_torch_backend_2d.py,
tests/scattering1d/test_torch_backend_1d.py) re-targeted at the CUDA ops, and
the reference cascade driven op by op through them."""
import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def dev():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    return torch.device('cuda:0')


def test_pad_and_unpad(dev):
    from kymatio_gb300.backend import backend2d as B
    pad = B.Pad((2, 2, 2, 2), (4, 4))
    x = torch.randn(1, 4, 4, device=dev)
    z = pad(x)
    assert z.shape == (1, 8, 8, 1)
    assert torch.allclose(z[0, 2, 2], x[0, 0, 0])
    assert torch.allclose(z[0, 1, 0], x[0, 1, 2])
    assert torch.allclose(z[0, 1, 1], x[0, 1, 1])
    assert torch.allclose(z[0, 1, 2], x[0, 1, 0])
    assert torch.allclose(z[0, 1, 3], x[0, 1, 1])
    # pad equal to the input size (the reference's special case)
    x = torch.randn(2, 4, 4, device=dev)
    z = B.Pad((4, 4, 4, 4), (4, 4))(x)
    ref = np.pad(x.cpu().numpy(), ((0, 0), (4, 4), (4, 4)), mode='reflect')
    assert np.allclose(z[..., 0].cpu().numpy(), ref)
    y = B.unpad(torch.randn(4, 4, 1, device=dev))
    assert y.shape == (2, 2)


def test_modulus_and_gradient(dev):
    from kymatio_gb300.backend import backend2d as B
    x = torch.rand(100, 10, 4, 2, device=dev)
    y = B.modulus(x)
    assert torch.allclose(y[..., 0], (x[..., 0] ** 2 + x[..., 1] ** 2).sqrt())
    x = torch.randn(10, 2, device=dev)
    x[3] = 0
    x.requires_grad_()
    y = B.modulus(x)
    g = torch.rand_like(y)
    y.backward(g)
    expect = x.detach() * g / y.detach()
    expect[3] = 0
    assert torch.allclose(x.grad, expect)
    with pytest.raises(TypeError) as e:
        B.modulus(torch.randn(3, 3, device=dev))
    assert 'complex' in e.value.args[0]


def test_subsample_fourier(dev):
    from kymatio_gb300.backend import backend2d as B
    x = torch.randn(3, 2, 16, 16, 2, device=dev)
    for k in (1, 2, 4, 8):
        y = B.subsample_fourier(x, k)
        xn = x.cpu().numpy()
        m = 16 // k
        ref = np.zeros(xn.shape[:-3] + (m, m, 2))
        for a in range(k):
            for b in range(k):
                ref += xn[..., a * m:(a + 1) * m, b * m:(b + 1) * m, :]
        assert np.allclose(y.cpu().numpy(), ref / k ** 2, atol=1e-6)


def test_cdgmm(dev):
    from kymatio_gb300.backend import backend2d as B
    x = torch.randn(3, 4, 5, 6, 2, device=dev)
    f = torch.randn(5, 6, 1, device=dev)
    assert torch.allclose(B.cdgmm(x, f), x * f)
    fc = torch.randn(5, 6, 2, device=dev)
    z = B.cdgmm(x, fc)
    ref = torch.stack([x[..., 0] * fc[..., 0] - x[..., 1] * fc[..., 1],
                       x[..., 0] * fc[..., 1] + x[..., 1] * fc[..., 0]], dim=-1)
    assert torch.allclose(z, ref, atol=1e-6)
    with pytest.raises(RuntimeError) as e:
        B.cdgmm(x, torch.randn(5, 7, 1, device=dev))
    assert 'not compatible' in e.value.args[0]
    with pytest.raises(TypeError) as e:
        B.cdgmm(x, f.double())
    assert 'same dtype' in e.value.args[0]
    with pytest.raises(TypeError) as e:
        B.cdgmm(x.cpu(), f)
    assert 'Input must be on GPU' in e.value.args[0]


def test_fft_kat_and_round_trips(dev):
    # 4x4 DFT by its definition (tests/scattering2d/test_torch_backend_2d.py:284-320)
    from kymatio_gb300.backend import backend2d as B
    x = np.random.default_rng(1).random((4, 4))
    I, Jj, K, L = np.meshgrid(np.arange(4), np.arange(4), np.arange(4), np.arange(4), indexing='ij')
    coef = np.exp(-2 * np.pi * 1j * (K * I / 4 + L * Jj / 4))
    y = np.zeros((4, 4), complex)
    for k in range(4):
        for l in range(4):
            y[k, l] = (x * coef[..., k, l]).sum()
    xt = torch.from_numpy(x.astype(np.float32))[..., None].to(dev)
    z = B.rfft(xt)
    assert np.allclose(z.cpu().numpy(), np.stack([y.real, y.imag], -1), atol=1e-5)
    assert torch.allclose(B.irfft(z), xt, atol=1e-6)
    assert torch.allclose(B.ifft(z)[..., :1], xt, atol=1e-6)
    for shape in ((3, 40, 40), (2, 272, 272), (5, 34, 17)):
        a = torch.randn(shape + (2,), device=dev)
        f = B.ifft(a)
        ref = np.fft.ifft2(a[..., 0].cpu().numpy() + 1j * a[..., 1].cpu().numpy())
        assert rel_l2(f[..., 0].cpu().numpy() + 1j * f[..., 1].cpu().numpy(), ref) < 1e-6
    with pytest.raises(TypeError) as e:
        B.rfft(torch.randn(4, 4, 2, device=dev))
    assert 'real' in e.value.args[0]
    with pytest.raises(TypeError) as e:
        B.ifft(torch.randn(4, 4, 1, device=dev))
    assert 'complex' in e.value.args[0]
    with pytest.raises(RuntimeError) as e:
        B.rfft(torch.randn(4, 4, 1, device=dev)[::2, ::2])
    assert 'must be contiguous' in e.value.args[0]


@pytest.mark.parametrize('n,batch', [(64, 3000), (17, 700), (100, 51), (2048, 9), (4096, 5), (16384, 3)])
def test_fft_1d_batches(dev, n, batch):
    """Batches of 1-D lines through kym_op_fft2 (M = 1): short lines many per
    CTA, long lines one per CTA; forward complex, inverse to real."""
    from kymatio_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(n + batch)
    a = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    at = torch.from_numpy(np.stack([a.real, a.imag], -1)).to(dev)
    out = torch.empty_like(at)
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.kym_op_fft2(at.data_ptr(), out.data_ptr(), batch, 1, n, 0, 0, 0, 1.0, st), 'fft')
    got = out[..., 0].cpu().numpy() + 1j * out[..., 1].cpu().numpy()
    assert rel_l2(got, np.fft.fft(a.astype(np.complex128), axis=-1)) < 1e-6
    real = torch.empty((batch, n), device=dev)
    _lib.check(lib.kym_op_fft2(out.data_ptr(), real.data_ptr(), batch, 1, n, 0, 1, 1, 1.0 / n, st), 'ifft')
    assert rel_l2(real.cpu().numpy(), a.real) < 1e-6


def test_stack(dev):
    from kymatio_gb300.backend import backend2d as B
    x, y, z = (torch.randn(3, 6, 6, device=dev) for _ in range(3))
    w = B.stack((x, y, z))
    assert w.shape == (3, 3, 6, 6)
    assert torch.equal(w[:, 1], y)


def test_op_level_cascade_2d_vs_oracle(dev):
    """The reference cascade driven op by op through backend2d."""
    from kymatio_gb300 import Scattering2D
    from kymatio_gb300 import core
    from kymatio_gb300.backend import backend2d as B
    from oracle.scattering2d import Scattering2D as Oracle, order_slices
    x = np.random.default_rng(2).random((3, 32, 32)).astype(np.float32)
    S = Scattering2D(2, (32, 32)).to(dev)
    phi = {'levels': [getattr(S, 'tensor%d' % i) for i in range(2)], 'j': 2}
    n = 2
    psi = []
    for p in S.psi:
        lv = []
        for _ in p['levels']:
            lv.append(getattr(S, 'tensor%d' % n))
            n += 1
        psi.append({'levels': lv, 'j': p['j'], 'theta': p['theta']})
    pad = B.Pad(S.pad_size, [32, 32])
    xt = torch.from_numpy(x).to(dev)
    out = core.scattering2d(xt, pad, B.unpad, B, 2, 8, phi, psi, 2).cpu().numpy()
    ref = Oracle(2, (32, 32))(x.astype(np.float64))
    for sl in order_slices(2, 8, 2):
        assert rel_l2(out[:, sl], ref[:, sl]) <= 1e-5
    # autograd through the op surface agrees with the fused backward
    xg = xt.clone().requires_grad_()
    g = torch.randn(3, 81, 8, 8, device=dev)
    core.scattering2d(xg, pad, B.unpad, B, 2, 8, phi, psi, 2).backward(g)
    xf = xt.clone().requires_grad_()
    S(xf).backward(g)
    assert rel_l2(xg.grad.cpu().numpy(), xf.grad.cpu().numpy()) <= 1e-5


def test_op_level_cascade_1d_vs_oracle(dev):
    from kymatio_gb300 import core
    from kymatio_gb300.backend import backend1d as B
    from kymatio_gb300.scattering1d import Scattering1D
    from oracle.scattering1d import Scattering1D as Oracle
    x = np.random.default_rng(3).standard_normal((2, 1024)).astype(np.float32)
    S = Scattering1D(5, 1024, Q=4).to(dev)
    n = 0
    phi = dict(S.phi_f)
    phi['levels'] = []
    for _ in range(S._nlev['phi']):
        phi['levels'].append(getattr(S, 'tensor%d' % n))
        n += 1
    banks = []
    for key, meta in (('psi1', S.psi1_f), ('psi2', S.psi2_f)):
        bank = []
        for p, nl in zip(meta, S._nlev[key]):
            d = dict(p)
            d['levels'] = [getattr(S, 'tensor%d' % (n + i)) for i in range(nl)]
            n += nl
            bank.append(d)
        banks.append(bank)
    U0 = B.pad(torch.from_numpy(x).to(dev).reshape(-1, 1, 1024), S.pad_left, S.pad_right)
    paths = sorted(core.scattering1d(U0, B, [phi] + banks, S.log2_stride, True),
                   key=lambda p: (len(p['n']), p['n']))  # the frontend's ordering
    res = S.log2_stride
    out = torch.stack([B.unpad(p['coef'], S.ind_start[res], S.ind_end[res]) for p in paths], dim=-2)
    ref = Oracle(5, 1024, Q=4)(x.astype(np.float64))
    assert rel_l2(out.reshape(ref.shape).cpu().numpy(), ref) <= 1e-5
