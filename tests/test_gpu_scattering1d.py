"""GPU parity of the fused 1-D cascade against the reference golden vectors and
the FP64 oracle (relative L2 <= 1e-5 per order)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


def _cuda():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    return torch.device('cuda:0')


def _check_orders(out, ref, order, tol=1e-5):
    for k in (0, 1, 2):
        sel = order == k
        if sel.any():
            e = rel_l2(out[..., sel, :], ref[..., sel, :])
            assert e <= tol, 'order %d relL2 %.3e' % (k, e)


def test_reference_golden_file():
    # tests/scattering1d/test_torch_scattering1d.py:82-114
    dev = _cuda()
    from kymatio_gb300.scattering1d import Scattering1D
    d = np.load(os.path.join(GOLDEN, 'ref_test_data_1d.npz'))
    x = torch.from_numpy(d['x']).to(dev)
    S = Scattering1D(int(d['J']), x.shape[-1], int(d['Q'])).to(dev)
    Sx = S(x)
    Sx0 = torch.from_numpy(d['Sx']).to(dev)
    assert Sx.shape == Sx0.shape
    assert torch.allclose(Sx, Sx0, rtol=1e-5, atol=1e-6)
    _check_orders(Sx.cpu().numpy(), d['Sx'], S.meta()['order'])


CASES = json.loads(str(np.load(os.path.join(GOLDEN, 'ref_cases_1d.npz'))['meta']))


@pytest.mark.parametrize('case', CASES, ids=lambda c: c['name'])
def test_reference_cases(case):
    dev = _cuda()
    from kymatio_gb300.scattering1d import Scattering1D
    d = np.load(os.path.join(GOLDEN, 'ref_cases_1d.npz'))
    kw = dict(case['kwargs'])
    if isinstance(kw.get('Q'), list):
        kw['Q'] = tuple(kw['Q'])
    S = Scattering1D(**kw).to(dev)
    x = torch.from_numpy(d[case['name'] + '/x']).to(dev)
    if S.average is False:
        # T=0: un-averaged paths U at their own resolutions, keyed by n
        out = S(x)
        assert isinstance(out, list) and len(out) == S.output_size()
        for p in out:
            ref = d[case['name'] + '/S/' + ','.join(str(n) for n in p['n'])]
            got = p['coef'].cpu().numpy()
            assert got.shape == ref.shape, (p['n'], got.shape, ref.shape)
            assert rel_l2(got, ref) <= 1e-5, (p['n'], rel_l2(got, ref))
        return
    out = S(x).cpu().numpy()
    ref = d[case['name'] + '/S']
    assert out.shape == ref.shape
    _check_orders(out, ref, S.meta()['order'])


def test_cfg2_shape_vs_fp64_oracle():
    """J=6, Q=(8,1), T=64, N=8192: white noise plus a linear chirp (seed 1)."""
    dev = _cuda()
    from kymatio_gb300.scattering1d import Scattering1D
    from oracle.scattering1d import Scattering1D as Oracle
    rng = np.random.default_rng(1)
    B, N = 8, 8192
    x = rng.standard_normal((B, N))
    t = np.arange(N)
    f0 = rng.uniform(0.01, 0.1, B)[:, None]
    f1 = rng.uniform(0.1, 0.4, B)[:, None]
    x = (x + np.cos(2 * np.pi * (f0 * t + (f1 - f0) * t ** 2 / (2 * N)))).astype(np.float32)
    S = Scattering1D(6, N, Q=(8, 1), T=64).to(dev)
    out = S(torch.from_numpy(x).to(dev)).cpu().numpy()
    ref = Oracle(6, N, Q=(8, 1), T=64)(x.astype(np.float64))
    assert out.shape == ref.shape == (B, 126, 128)
    _check_orders(out, ref, S.meta()['order'])


def test_formats_and_meta():
    dev = _cuda()
    from kymatio_gb300.scattering1d import Scattering1D
    from oracle.scattering1d import Scattering1D as Oracle
    x = np.random.default_rng(4).standard_normal((2, 3, 1024)).astype(np.float32)
    kw = dict(J=5, shape=1024, Q=4)
    ref = Oracle(**kw, out_type='list')(x.astype(np.float64))
    S = Scattering1D(**kw, out_type='list').to(dev)
    out = S(torch.from_numpy(x).to(dev))
    assert len(out) == len(ref) == S.output_size()
    for a, b in zip(out, ref):
        assert a['n'] == b['n'] and a['j'] == b['j'] and a['order'] == b['order']
        assert rel_l2(a['coef'].cpu().numpy(), b['coef']) <= 1e-5
    Sd = Scattering1D(**kw, out_type='dict').to(dev)
    od = Sd(torch.from_numpy(x).to(dev))
    for b in ref:
        assert rel_l2(od[b['n']].cpu().numpy(), b['coef']) <= 1e-5
    meta = S.meta()
    assert len(meta['key']) == S.output_size()
    assert tuple(np.bincount(meta['order'])) == S.output_size(detail=True)


def test_batch_shapes_and_errors():
    dev = _cuda()
    from kymatio_gb300.scattering1d import Scattering1D
    S = Scattering1D(4, 256, Q=2).to(dev)
    a = S(torch.randn(256, device=dev))
    for shp in ((1, 256), (2, 3, 256)):
        b = S(torch.randn(shp, device=dev))
        assert b.shape == shp[:-1] + a.shape
    with pytest.raises(TypeError):
        S(None)
    with pytest.raises(TypeError):
        S(torch.randn(256))
    with pytest.raises(ValueError):
        Scattering1D(4, 256, out_type='bad').to(dev)(torch.randn(256, device=dev))
