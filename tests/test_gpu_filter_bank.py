"""The device build of the 2-D filter bank (kym_s2d_filter_bank, FP64 on the
GPU rounded to float32) against the host build, which matches the
reference's buffers bit for bit (kymatio/scattering2d/filter_bank.py:5-175),
and the transform computed with it against the FP64 oracle."""
import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('M,N,J,L', [(40, 40, 2, 8), (160, 160, 4, 8), (272, 272, 3, 8), (48, 80, 3, 6)])
def test_device_bank_matches_host_bank(M, N, J, L):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300.filter_bank import filter_bank_2d, filter_bank_2d_device
    phi_h, psi_h = filter_bank_2d(M, N, J, L)
    phi_d, psi_d = filter_bank_2d_device(M, N, J, L)
    pairs = list(zip(phi_h, phi_d))
    for ph, pd in zip(psi_h, psi_d):
        assert (ph['j'], ph['theta']) == (pd['j'], pd['theta'])
        pairs += list(zip(ph['levels'], pd['levels']))
    assert len(pairs) == J + sum(min(j + 1, max(J - 1, 1)) for j in range(J)) * L
    for h, d in pairs:
        d = d.cpu().numpy()
        assert h.shape == d.shape and d.dtype == np.float32
        # float32 rounding of the same filter: the reference accumulates in complex64
        assert np.abs(d - h).max() <= 2e-6 * np.abs(h).max(), np.abs(d - h).max() / np.abs(h).max()


@pytest.mark.parametrize('J,side,B', [(2, 32, 8), (3, 256, 2)])
def test_transform_with_device_bank(J, side, B):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300 import Scattering2D
    from oracle.scattering2d import Scattering2D as Oracle, order_slices
    dev = torch.device('cuda:0')
    x = np.random.default_rng(J + side).random((B, side, side)).astype(np.float32)
    S = Scattering2D(J, (side, side), filters='device')
    assert S.tensor0.is_cuda
    out = S(torch.from_numpy(x).to(dev)).cpu().numpy()
    ref = Oracle(J, (side, side))(x.astype(np.float64))
    for k, sl in enumerate(order_slices(J, 8, 2)):
        e = rel_l2(out[:, sl], ref[:, sl])
        assert e <= 1e-5, 'order %d relL2 %.3e' % (k, e)
    # the same module in the tensor-core form (separable factors derived on the device)
    S.tensor_cores = True
    out_tc = S(torch.from_numpy(x).to(dev)).cpu().numpy()
    for k, sl in enumerate(order_slices(J, 8, 2)):
        assert rel_l2(out_tc[:, sl], ref[:, sl]) <= 5e-5
