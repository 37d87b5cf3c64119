"""The reference's own frontends and cascade cores driving this package's
CUDA op surface (the backend-object boundary): ``kymatio.Scattering2D`` /
``kymatio.Scattering1D`` with ``frontend='torch', backend=backend2d/1d`` run
kymatio/scattering2d/core/scattering2d.py and
kymatio/scattering1d/core/scattering1d.py op by op on CUDA tensors, every op
one of this package's kernels.  Checked with the reference's own allclose
against its golden files (tests/scattering2d/test_torch_scattering2d.py:45-77,
tests/scattering1d/test_torch_scattering1d.py:84-112).

The reference is looked up in $KYMATIO_REFERENCE (a checkout), else in
baseline/_ref (its pip install into this repository)."""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


def _reference_kymatio():
    cands = [os.environ.get('KYMATIO_REFERENCE', ''), os.path.join(ROOT, 'baseline', '_ref')]
    for c in cands:
        if c and os.path.isfile(os.path.join(c, 'kymatio', '__init__.py')):
            dont = sys.dont_write_bytecode
            sys.dont_write_bytecode = True
            sys.path.insert(0, c)
            try:
                import kymatio
                from kymatio.scattering1d.frontend import torch_frontend as _f1  # noqa: F401
                from kymatio.scattering2d.frontend import torch_frontend as _f2  # noqa: F401
                return kymatio
            finally:
                sys.path.remove(c)
                sys.dont_write_bytecode = dont
    pytest.skip('the reference (kymatio) is not installed: set KYMATIO_REFERENCE or install it into baseline/_ref')


def test_reference_frontend_2d_over_cuda_ops():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    kymatio = _reference_kymatio()
    from kymatio_gb300.backend import backend2d
    dev = torch.device('cuda:0')
    data = np.load(os.path.join(GOLDEN, 'ref_test_data_2d.npz'))
    x = torch.from_numpy(data['x']).to(dev)
    S = torch.from_numpy(data['Sx']).to(dev)
    J, pre_pad = int(data['J']), bool(data['pre_pad'])
    M, N = x.shape[2], x.shape[3]
    sc = kymatio.Scattering2D(J, shape=(M, N), pre_pad=pre_pad, backend=backend2d, frontend='torch').to(dev)
    assert sc.backend is backend2d
    Sg = sc(x)
    assert Sg.is_cuda and Sg.shape == S.shape
    assert torch.allclose(Sg, S)
    sc1 = kymatio.Scattering2D(J, shape=(M, N), pre_pad=pre_pad, max_order=1, backend=backend2d,
                               frontend='torch').to(dev)
    S1x = sc1(x)
    assert torch.allclose(S1x, S[..., :S1x.shape[-3], :, :])


def test_reference_frontend_1d_over_cuda_ops():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    kymatio = _reference_kymatio()
    from kymatio_gb300.backend import backend1d
    dev = torch.device('cuda:0')
    data = np.load(os.path.join(GOLDEN, 'ref_test_data_1d.npz'))
    x = torch.from_numpy(data['x']).to(dev)
    J, Q = int(data['J']), int(data['Q'])
    Sx0 = torch.from_numpy(data['Sx']).to(dev)
    sc = kymatio.Scattering1D(J, x.shape[-1], Q, backend=backend1d, frontend='torch').to(dev)
    assert sc.backend is backend1d
    Sx = sc(x)
    assert Sx.is_cuda and Sx.shape == Sx0.shape
    assert torch.allclose(Sx, Sx0)


def test_reference_frontend_2d_gradient_over_cuda_ops():
    """Autograd through the reference core over the CUDA ops (each op's
    adjoint kernel) against the reference's own torch backend on the CPU."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    kymatio = _reference_kymatio()
    from kymatio_gb300.backend import backend2d
    dev = torch.device('cuda:0')
    rng = np.random.default_rng(7)
    x0 = rng.random((2, 32, 32)).astype(np.float32)
    g = torch.from_numpy(rng.standard_normal((2, 81, 8, 8)).astype(np.float32))
    ref = kymatio.Scattering2D(2, shape=(32, 32), frontend='torch').double()
    xr = torch.from_numpy(x0.astype(np.float64)).requires_grad_()
    ref(xr).backward(g.double())
    sc = kymatio.Scattering2D(2, shape=(32, 32), backend=backend2d, frontend='torch').to(dev)
    xg = torch.from_numpy(x0).to(dev).requires_grad_()
    sc(xg).backward(g.to(dev))
    a, b = xg.grad.double().cpu().numpy(), xr.grad.numpy()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-5
