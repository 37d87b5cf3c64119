"""The benchmark's own inputs, asserted: Scattering2D J=3, L=8 at 256x256 on
the seed-2 Gaussian random fields (white N(0,1) smoothed by sigma U[1,4] px,
rescaled to [0,1]), batch 64 in one call.  The first and the last image (the
last one lands in the last sub-launch of the line-split groups) are checked
per order against the FP64 oracle: the plain FP32 path at 1e-5, the
split-precision tensor-core form (and its DFT-GEMM variant of the 68x68
groups) at 5e-5."""
import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu

TOL_PLAIN = 1e-5
TOL_TC = 5e-5


@pytest.fixture(scope='module')
def grf64():
    from bench import grf_batch
    from oracle.scattering2d import Scattering2D as Oracle
    x = grf_batch(64, seed=2)
    ref = Oracle(3, (256, 256))(x[[0, 63]].astype(np.float64))
    return x, ref


def _check(out, ref, tol):
    from oracle.scattering2d import order_slices
    for k, sl in enumerate(order_slices(3, 8, 2)):
        e = rel_l2(out[:, sl], ref[:, sl])
        assert e <= tol, 'order %d relL2 %.3e > %.0e' % (k, e, tol)


@pytest.mark.parametrize('form', ['plain', 'tc', 'tc_dft'])
def test_grf_batch64_vs_fp64_oracle(grf64, form):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300 import Scattering2D, _lib
    lib = _lib.load()
    x, ref = grf64
    dev = torch.device('cuda:0')
    S = Scattering2D(3, (256, 256), backend='torch_tc' if form != 'plain' else 'torch').to(dev)
    prev = lib.kym_set_tc_dft(1 if form == 'tc_dft' else 0)
    try:
        out = S(torch.from_numpy(x).to(dev))
        torch.cuda.synchronize()
    finally:
        lib.kym_set_tc_dft(prev)
    if form != 'plain':
        assert S.tensor_core_status() == 0
    assert out.shape == (64, 217, 32, 32)
    _check(out[[0, 63]].cpu().numpy(), ref, TOL_PLAIN if form == 'plain' else TOL_TC)
