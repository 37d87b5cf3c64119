"""Hand-written backward (kym_s2d_backward / kym_s1d_backward) against the
reference torch backend's autograd gradient (float64, captured in
tests/golden/ref_grads.npz) and against FP64 central finite differences of
the oracle.  Tolerance: relative L2 <= 1e-5."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu

D = np.load(os.path.join(GOLDEN, 'ref_grads.npz'))
META = json.loads(str(D['meta']))


def _cuda():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    return torch.device('cuda:0')


def _grad(S, x, g, dev):
    xt = torch.from_numpy(x).to(dev).requires_grad_()
    y = S(xt)
    y.backward(torch.from_numpy(g).to(dev))
    return xt.grad.cpu().numpy()


@pytest.mark.parametrize('case', META['g2'], ids=lambda c: c['name'])
def test_2d_grad_vs_reference_autograd(case):
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    S = Scattering2D(case['J'], tuple(case['shape']), max_order=case['max_order'],
                     pre_pad=case['pre_pad']).to(dev)
    n = case['name']
    gx = _grad(S, D[n + '/x'], D[n + '/g'], dev)
    assert gx.shape == D[n + '/gx'].shape
    assert rel_l2(gx, D[n + '/gx']) <= 1e-5


@pytest.mark.parametrize('case', META['g1'], ids=lambda c: c['name'])
def test_1d_grad_vs_reference_autograd(case):
    dev = _cuda()
    from kymatio_gb300.scattering1d import Scattering1D
    kw = dict(case['kwargs'])
    if isinstance(kw.get('Q'), list):
        kw['Q'] = tuple(kw['Q'])
    S = Scattering1D(**kw).to(dev)
    n = case['name']
    gx = _grad(S, D[n + '/x'], D[n + '/g'], dev)
    assert rel_l2(gx, D[n + '/gx']) <= 1e-5


def test_2d_grad_vs_fp64_finite_differences():
    """32x32, J=2: 64 random pixels, h=1e-6 central differences of <g, S(x)>
    on the FP64 oracle vs the GPU backward."""
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    from oracle.scattering2d import Scattering2D as Oracle
    from test_oracle_golden import fd_grad_2d
    rng = np.random.default_rng(3)
    x = rng.random((1, 32, 32)).astype(np.float32)
    S = Scattering2D(2, (32, 32)).to(dev)
    g = rng.standard_normal((1, 81, 8, 8)).astype(np.float32)
    gx = _grad(S, x, g, dev)
    pix = [(0, int(rng.integers(32)), int(rng.integers(32))) for _ in range(64)]
    fd = fd_grad_2d(Oracle(2, (32, 32)), x.astype(np.float64), g.astype(np.float64), pix)
    got = np.array([gx[p] for p in pix])
    assert rel_l2(got, fd) <= 1e-5


def test_backward_chunking_and_recompute_invisible():
    """The backward recomputes parent spectra chunk by chunk; chunk sizes
    (the memory budget) must not change the gradient."""
    dev = _cuda()
    from kymatio_gb300 import Scattering2D, _lib
    S = Scattering2D(3, (64, 64)).to(dev)
    x = torch.rand(5, 64, 64, device=dev)
    g = torch.randn(5, 217, 8, 8, device=dev)
    a = S._backward_raw(x, g)
    lib = _lib.load()
    lib.kym_s2d_set_backward_chunk(S._get_plan().h, 2)
    b = S._backward_raw(x, g)
    assert torch.allclose(a, b, rtol=0, atol=0)


def test_cfg4_fwd_bwd_batch32():
    """128x128, J=4, batch 32 (U[0,1) seed 3, upstream N(0,1)): forward +
    backward run and the gradient of one image matches a batch-of-one run."""
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    rng = np.random.default_rng(3)
    x = rng.random((32, 128, 128)).astype(np.float32)
    g = rng.standard_normal((32, 417, 8, 8)).astype(np.float32)
    S = Scattering2D(4, (128, 128)).to(dev)
    gx = _grad(S, x, g, dev)
    gx1 = _grad(S, x[5:6], g[5:6], dev)
    assert rel_l2(gx[5:6], gx1) <= 1e-6
    assert np.isfinite(gx).all()
