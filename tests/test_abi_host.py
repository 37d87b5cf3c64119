"""Host-side checks of the C ABI library (no GPU needed): it loads, it exports
every entry point include/kymatio_gb300.h declares, and its plans reproduce
the reference geometry."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def _declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, 'include')):
        if f.endswith('.h'):
            src = open(os.path.join(ROOT, 'include', f)).read()
            src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
            names |= set(re.findall(r'\b(kym_\w+)\s*\(', src))
    return names


@pytest.fixture(scope='module')
def lib():
    from kymatio_gb300 import _lib
    return _lib.load(build_if_missing=True)


def test_exports_every_declared_symbol(lib):
    from kymatio_gb300 import _lib
    declared = _declared()
    assert declared, 'no declarations found'
    for name in declared:
        assert hasattr(lib, name), name
    assert declared == set(_lib.SIGNATURES), declared ^ set(_lib.SIGNATURES)


@pytest.mark.parametrize('M,N,J,L,mo,pp', [(256, 256, 3, 8, 2, 0), (32, 32, 2, 8, 2, 0), (128, 128, 4, 8, 2, 0),
                                          (37, 32, 5, 8, 2, 0), (31, 31, 1, 8, 1, 0), (64, 48, 3, 8, 2, 1),
                                          (24, 24, 2, 4, 2, 0), (256, 256, 4, 8, 2, 0)])
def test_plan_geometry_2d(lib, M, N, J, L, mo, pp):
    from oracle.scattering2d import Scattering2D as O
    from kymatio_gb300 import _lib
    h = _lib._vp()
    assert lib.kym_s2d_plan_create(M, N, J, L, mo, pp, ctypes.byref(h)) == 0
    v = [ctypes.c_int() for _ in range(6)]
    assert lib.kym_s2d_plan_info(h, *[ctypes.byref(i) for i in v]) == 0
    Mp, Np, C, orr, occ, nf = [i.value for i in v]
    o = O.__new__(O)
    from oracle.filters import compute_padding_2d
    assert (Mp, Np) == compute_padding_2d(M, N, J)
    c2 = L * L * J * (J - 1) // 2 if mo == 2 else 0
    assert C == 1 + J * L + c2
    assert (orr, occ) == (Mp // 2 ** J - 2, Np // 2 ** J - 2)
    assert nf == J + L * sum(min(j + 1, max(J - 1, 1)) for j in range(J))
    r, c = ctypes.c_int(), ctypes.c_int()
    assert lib.kym_s2d_filter_shape(h, 0, ctypes.byref(r), ctypes.byref(c)) == 0 and (r.value, c.value) == (Mp, Np)
    assert lib.kym_s2d_filter_shape(h, nf, ctypes.byref(r), ctypes.byref(c)) != 0
    assert lib.kym_s2d_workspace_bytes(h, 4) > 0
    assert lib.kym_s2d_plan_destroy(h) == 0


def test_plan_rejects_bad_geometry(lib):
    from kymatio_gb300 import _lib
    h = _lib._vp()
    assert lib.kym_s2d_plan_create(10, 10, 10, 8, 2, 0, ctypes.byref(h)) == _lib.KYM_ERR_INVALID
    assert lib.kym_s2d_plan_create(0, 10, 1, 8, 2, 0, ctypes.byref(h)) == _lib.KYM_ERR_INVALID
    assert lib.kym_s2d_plan_create(32, 32, 2, 8, 3, 0, ctypes.byref(h)) == _lib.KYM_ERR_INVALID
    assert lib.kym_s2d_forward(None, None, None, 0, None, 0, None, 0, None) == _lib.KYM_ERR_INVALID


def test_host_switches_and_argument_checks(lib):
    """Host-side logic of the per-group tensor-core switch, the side-lane
    switch, the launch counts and the host-buffer forward's argument checks
    (no device work: every call here returns before touching CUDA)."""
    from kymatio_gb300 import _lib
    h = _lib._vp()
    assert lib.kym_s2d_plan_create(256, 256, 3, 8, 2, 0, ctypes.byref(h)) == 0
    ng = lib.kym_s2d_group_count(h)
    assert ng == 7
    assert lib.kym_s2d_set_group_tc(h, -1, 0) == -1 and lib.kym_s2d_set_group_tc(h, ng, 0) == -1
    tc = [g for g in range(ng) if lib.kym_s2d_group_uses_tc(h, g) > 0]
    assert tc, 'no tensor-core group at 256x256 J=3'
    g = tc[0]
    assert lib.kym_s2d_set_group_tc(h, g, 0) == 1
    assert lib.kym_s2d_group_uses_tc(h, g) == 0 and lib.kym_s2d_group_kernels(h, g, 1) == 1
    assert lib.kym_s2d_set_group_tc(h, g, 1) == 0 and lib.kym_s2d_group_uses_tc(h, g) > 0
    prev = lib.kym_set_side_lane(0)
    assert lib.kym_set_side_lane(prev) == 0
    # the 272x272 line-split groups: the input stage in one sub-launch (3
    # kernels); order 1 j1=0 in five sub-launches of 3 line passes, then one
    # low-pass launch
    assert lib.kym_s2d_group_launches(h, 0, 64, 1) == 3
    assert lib.kym_s2d_group_launches(h, 1, 64, 1) == 3 * 5 + 1
    buf = ctypes.create_string_buffer(64)
    p = ctypes.cast(buf, _lib._vp)
    ptrs = (_lib._vp * 1)(p)
    args = dict(x_host=p, out_host=p, x_dev=p, out_dev=p)

    def fwd(parts=1, lowpass=None, status=None, **kw):
        a = dict(args, **kw)
        return lib.kym_s2d_forward_host(h, a['x_host'], a['out_host'], 1, ptrs, 1, lowpass, lowpass, 1, status,
                                        a['x_dev'], a['out_dev'], p, 64, parts, None, None)
    for bad in ('x_host', 'out_host', 'x_dev', 'out_dev'):
        assert fwd(**{bad: None}) == _lib.KYM_ERR_INVALID
    assert fwd(parts=0) == _lib.KYM_ERR_INVALID
    assert fwd(lowpass=ptrs) == _lib.KYM_ERR_INVALID  # tensor-core form without a status word
    assert lib.kym_s2d_plan_destroy(h) == 0


@pytest.mark.parametrize('side,J,lanes', [
    # groups: input stage, order 1 by j1, then order 2 by (j1, j2)
    (256, 3, [0, 0, 1, 0, 0, 0, 1]),
    (128, 4, [0, 0, 1, 1, 0, 0, 0, 0, 1, 1, 1]),
    (32, 2, [0, 0, 0, 0]),
])
def test_launch_lanes(lib, side, J, lanes):
    """The heaviest order-1 scale and its order-2 groups stay on the caller's
    stream; the other order-1 scales with children and their order-2 groups
    go to the side lane; childless order-1 scales stay on the caller's stream.
    Every order-2 group shares its parents' lane (they run in stream order)."""
    from kymatio_gb300 import _lib
    h = _lib._vp()
    assert lib.kym_s2d_plan_create(side, side, J, 8, 2, 0, ctypes.byref(h)) == 0
    ng = lib.kym_s2d_group_count(h)
    got = [lib.kym_s2d_group_lane(h, g) for g in range(ng)]
    assert got == lanes
    assert lib.kym_s2d_group_lane(h, ng) == -1
    info = []
    for g in range(ng):
        v = [ctypes.c_int() for _ in range(6)]
        assert lib.kym_s2d_group_info(h, g, *[ctypes.byref(i) for i in v]) == 0
        info.append((v[0].value, v[2].value, v[4].value))  # level, rows, fold
    # an order-2 group of parent resolution rows * fold reads the order-1 group of that size
    order1 = {rows: g for g, (lvl, rows, fold) in enumerate(info) if lvl == 1}
    for g, (lvl, rows, fold) in enumerate(info):
        if lvl == 2:
            assert got[g] == got[order1[rows * fold]]
    assert lib.kym_s2d_plan_destroy(h) == 0


def test_product_bank_matches_reference():
    from kymatio_gb300.filter_bank import filter_bank_2d
    d = np.load(os.path.join(GOLDEN, 'ref_bank_2d.npz'))
    phi, psi = filter_bank_2d(40, 40, 2, 8)
    for r, lv in enumerate(phi):
        assert np.array_equal(lv, d['phi/%d' % r])
    for n, p in enumerate(psi):
        for r, lv in enumerate(p['levels']):
            assert np.array_equal(lv, d['psi/%d/%d' % (n, r)])


def test_product_bank_checksums_272():
    from kymatio_gb300.filter_bank import filter_bank_2d
    d = np.load(os.path.join(GOLDEN, 'ref_bank_2d.npz'))['big272/checksums']
    phi, psi = filter_bank_2d(272, 272, 3, 8)
    levels = list(phi) + [lv for p in psi for lv in p['levels']]
    got = np.array([[lv.sum(dtype=np.float64), (lv.astype(np.float64) ** 2).sum(), lv[0, 0], lv[3, 5]]
                    for lv in levels])
    assert got.shape == d.shape
    assert np.array_equal(got, d)


@pytest.mark.parametrize('M,J', [(256, 3), (32, 2), (128, 4), (64, 3)])
def test_separable_lowpass_identity(M, J):
    """T_r U T_c^T reproduces unpad(Re IFFT2(fold(FFT2(U) phi))) in FP64 for
    every low-pass level, and phi is rank one to float32 rounding."""
    from kymatio_gb300.filter_bank import filter_bank_2d, padded_size_2d, separable_lowpass
    Mp, Np = padded_size_2d(M, M, J)
    phi, _ = filter_bank_2d(Mp, Np, J, 8)
    s = Mp // 2 ** J
    rng = np.random.default_rng(J)
    for j, lv in enumerate(phi):
        m = Mp >> j
        ks = m // s
        Tr, Tc, resid = separable_lowpass(lv, 1, s - 2, 1, s - 2, ks, ks)
        assert resid < 1e-6
        U = rng.random((m, m))
        Z = np.fft.fft2(U) * lv
        B = Z.reshape(ks, s, ks, s).mean(axis=(0, 2))
        ref = np.fft.ifft2(B).real[1:-1, 1:-1]
        got = Tr @ U @ Tc.T
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-6


def test_reference_frontend_accepts_backend_objects():
    """The reference frontends accept the GB300 backend objects (name check of
    kymatio/frontend/base_frontend.py:47-50); runs when the reference is
    installed in baseline/_ref or KYMATIO_REFERENCE points at a checkout."""
    import sys
    cands = [os.environ.get('KYMATIO_REFERENCE', ''), os.path.join(ROOT, 'baseline', '_ref')]
    ref = next((c for c in cands if c and os.path.isfile(os.path.join(c, 'kymatio', '__init__.py'))), None)
    if ref is None:
        pytest.skip('the reference is not installed')
    dont = sys.dont_write_bytecode
    sys.dont_write_bytecode = True
    sys.path.insert(0, ref)
    try:
        from kymatio.scattering2d.frontend.torch_frontend import ScatteringTorch2D
        from kymatio.scattering1d.frontend.torch_frontend import ScatteringTorch1D
    finally:
        sys.path.remove(ref)
        sys.dont_write_bytecode = dont
    from kymatio_gb300.backend import backend1d, backend2d
    S2 = ScatteringTorch2D(2, (32, 32), backend=backend2d)
    assert S2.backend is backend2d
    S1 = ScatteringTorch1D(4, 256, backend=backend1d)
    assert S1.backend is backend1d
