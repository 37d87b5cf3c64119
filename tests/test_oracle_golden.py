"""Pins the CPU oracle against the reference's own golden vectors and
against reference outputs captured by tests/golden/make_golden.py."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle.filters import filter_bank_2d
from oracle.scattering1d import Scattering1D
from oracle.scattering2d import Scattering2D


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_reference_golden_2d():
    # tests/scattering2d/test_torch_scattering2d.py:45-77 (allclose, rtol 1e-5)
    d = _load('ref_test_data_2d.npz')
    x, Sx, J = d['x'], d['Sx'], int(d['J'])
    S = Scattering2D(J, x.shape[-2:], pre_pad=bool(d['pre_pad']))
    out = S(x)
    assert out.shape == Sx.shape
    assert np.allclose(out, Sx, rtol=1e-5, atol=1e-8)
    S1 = Scattering2D(J, x.shape[-2:], max_order=1)(x)
    assert np.allclose(S1, Sx[..., :S1.shape[-3], :, :], rtol=1e-5, atol=1e-8)


def test_reference_golden_1d():
    # tests/scattering1d/test_torch_scattering1d.py:82-114
    d = _load('ref_test_data_1d.npz')
    S = Scattering1D(int(d['J']), d['x'].shape[-1], int(d['Q']))
    out = S(d['x'])
    assert out.shape == d['Sx'].shape
    assert np.allclose(out, d['Sx'], rtol=1e-5, atol=1e-8)


CASES2 = json.loads(str(_load('ref_cases_2d.npz')['meta']))


@pytest.mark.parametrize('case', [c for c in CASES2 if c['name'] != 'j3_256'], ids=lambda c: c['name'])
def test_reference_cases_2d(case):
    d = _load('ref_cases_2d.npz')
    x, ref = d[case['name'] + '/x'], d[case['name'] + '/S']
    S = Scattering2D(case['J'], tuple(case['shape']), L=case['L'], max_order=case['max_order'],
                     pre_pad=case['pre_pad'])
    out = S(x.astype(np.float64))
    assert out.shape == ref.shape
    assert np.abs(out - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


CASES1 = json.loads(str(_load('ref_cases_1d.npz')['meta']))


@pytest.mark.parametrize('case', CASES1, ids=lambda c: c['name'])
def test_reference_cases_1d(case):
    d = _load('ref_cases_1d.npz')
    kw = dict(case['kwargs'])
    if isinstance(kw.get('Q'), list):
        kw['Q'] = tuple(kw['Q'])
    x = d[case['name'] + '/x']
    out = Scattering1D(**kw)(x.astype(np.float64))
    if isinstance(out, list):
        for p in out:
            ref = d[case['name'] + '/S/' + ','.join(map(str, p['n']))]
            assert np.abs(p['coef'] - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())
    else:
        ref = d[case['name'] + '/S']
        assert out.shape == ref.shape
        assert np.abs(out - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())


def test_reference_bank_2d():
    d = _load('ref_bank_2d.npz')
    bank = filter_bank_2d(40, 40, 2, 8)
    for r, lv in enumerate(bank['phi']['levels']):
        assert np.array_equal(lv, d['phi/%d' % r])
    for n, p in enumerate(bank['psi']):
        for r, lv in enumerate(p['levels']):
            assert np.array_equal(lv, d['psi/%d/%d' % (n, r)])


def test_oracle_subsample_kat():
    # tests/scattering2d/test_torch_backend_2d.py:107-167: explicit alias sum / k^2
    from oracle.scattering2d import subsample_fourier
    rng = np.random.default_rng(0)
    x = rng.standard_normal((3, 16, 16)) + 1j * rng.standard_normal((3, 16, 16))
    for k in (1, 2, 4, 8):
        y = subsample_fourier(x, k)
        m = 16 // k
        z = np.zeros((3, m, m), complex)
        for a in range(k):
            for b in range(k):
                z += x[:, a * m:(a + 1) * m, b * m:(b + 1) * m]
        assert np.allclose(y, z / k ** 2)


def fd_grad_2d(oracle, x, g, pixels, h=1e-6):
    """Central differences of <g, S(x)> in FP64 at the given pixel indices."""
    out = []
    for (b, i, j) in pixels:
        xp = x.copy()
        xm = x.copy()
        xp[b, i, j] += h
        xm[b, i, j] -= h
        out.append((np.sum(g * oracle(xp)) - np.sum(g * oracle(xm))) / (2 * h))
    return np.array(out)


def test_oracle_fd_matches_reference_autograd():
    """FP64 central differences through the oracle reproduce the reference
    torch autograd gradient (pins the finite-difference check used on GPU)."""
    d = _load('ref_grads.npz')
    x = d['g2_j2_32/x'].astype(np.float64)
    g = d['g2_j2_32/g'].astype(np.float64)
    gx = d['g2_j2_32/gx']
    S = Scattering2D(2, (32, 32))
    rng = np.random.default_rng(9)
    pix = [(int(rng.integers(2)), int(rng.integers(32)), int(rng.integers(32))) for _ in range(6)]
    fd = fd_grad_2d(S, x, g, pix)
    ref = np.array([gx[p] for p in pix])
    assert np.abs(fd - ref).max() <= 1e-6 * max(1.0, np.abs(ref).max())
