"""Hand-written backward against the reference torch backend's autograd
gradient (float64, captured in tests/golden/ref_grads.npz) and against FP64
central finite differences of the oracle, in both policies: the saved form
(kym_*_forward_save + kym_*_backward_saved, the default under the activation
budget) and the recompute form (kym_*_backward, budget 0).  Tolerance:
relative L2 <= 1e-5."""
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


POLICIES = ['saved', 'recompute']


def _policy(S, policy):
    S.activation_budget = 0 if policy == 'recompute' else 4 << 30
    return S


@pytest.mark.parametrize('policy', POLICIES)
@pytest.mark.parametrize('case', META['g2'], ids=lambda c: c['name'])
def test_2d_grad_vs_reference_autograd(case, policy):
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    S = _policy(Scattering2D(case['J'], tuple(case['shape']), max_order=case['max_order'],
                             pre_pad=case['pre_pad']).to(dev), policy)
    n = case['name']
    gx = _grad(S, D[n + '/x'], D[n + '/g'], dev)
    assert gx.shape == D[n + '/gx'].shape
    assert rel_l2(gx, D[n + '/gx']) <= 1e-5


@pytest.mark.parametrize('policy', POLICIES)
@pytest.mark.parametrize('case', META['g1'], ids=lambda c: c['name'])
def test_1d_grad_vs_reference_autograd(case, policy):
    dev = _cuda()
    from kymatio_gb300.scattering1d import Scattering1D
    kw = dict(case['kwargs'])
    if isinstance(kw.get('Q'), list):
        kw['Q'] = tuple(kw['Q'])
    S = _policy(Scattering1D(**kw).to(dev), policy)
    n = case['name']
    gx = _grad(S, D[n + '/x'], D[n + '/g'], dev)
    assert rel_l2(gx, D[n + '/gx']) <= 1e-5


@pytest.mark.parametrize('policy', POLICIES)
def test_2d_grad_vs_fp64_finite_differences(policy):
    """32x32, J=2: 64 random pixels, h=1e-6 central differences of <g, S(x)>
    on the FP64 oracle vs the GPU backward."""
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    from oracle.scattering2d import Scattering2D as Oracle
    from test_oracle_golden import fd_grad_2d
    rng = np.random.default_rng(3)
    x = rng.random((1, 32, 32)).astype(np.float32)
    S = _policy(Scattering2D(2, (32, 32)).to(dev), policy)
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


def test_budget_selects_policy_and_forms_agree():
    """The autograd node saves the modulus inputs while batch x saved bytes
    stays within activation_budget and recomputes above it; both forms give
    the same gradient, and the saved forward gives the plain output."""
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    torch.manual_seed(0)
    S = Scattering2D(3, (64, 64)).to(dev)
    x = torch.rand(6, 64, 64, device=dev)
    g = torch.randn(6, 217, 8, 8, device=dev)
    need = S._saved_bytes(6)
    assert need == 6 * S._saved_bytes(1) > 0
    calls = []
    for budget in (need, need - 1):
        S.activation_budget = budget
        orig = (S._backward_saved_raw, S._backward_raw)
        S._backward_saved_raw = lambda *a, o=orig[0]: calls.append('saved') or o(*a)
        S._backward_raw = lambda *a, o=orig[1]: calls.append('recompute') or o(*a)
        xt = x.clone().requires_grad_()
        y = S(xt)
        y.backward(g)
        del S._backward_saved_raw, S._backward_raw
        if budget == need:
            gs, ys = xt.grad.clone(), y.detach().clone()
        else:
            gr = xt.grad.clone()
    assert calls == ['saved', 'recompute']
    with torch.no_grad():
        y0 = S(x)
    assert torch.equal(ys, y0)
    assert rel_l2(gs.cpu().numpy(), gr.cpu().numpy()) <= 1e-6


def test_saved_form_1d_cfg2_shape():
    """1-D saved form at the 8192-sample, J=6, Q=(8,1), T=64 workload: the
    gradient of one signal matches a batch-of-one recompute run."""
    dev = _cuda()
    from kymatio_gb300.scattering1d import Scattering1D
    S = Scattering1D(6, 8192, Q=(8, 1), T=64).to(dev)
    rng = np.random.default_rng(1)
    x = torch.from_numpy(rng.standard_normal((4, 8192)).astype(np.float32)).to(dev)
    y = S(x)
    g = torch.from_numpy(rng.standard_normal(tuple(y.shape)).astype(np.float32)).to(dev)
    xt = x.clone().requires_grad_()
    S(xt).backward(g)
    S.activation_budget = 0
    x1 = x[2:3].clone().requires_grad_()
    S(x1).backward(g[2:3])
    assert rel_l2(xt.grad[2:3].cpu().numpy(), x1.grad.cpu().numpy()) <= 1e-6
