"""The allocation-free 2-D forward (kym_s2d_forward_noalloc) against the
ordinary one (kym_s2d_forward), through the C ABI.

kym_s2d_forward_noalloc is for callers that cannot allocate device memory
(a fixed pool reserved up front, a host application that forbids allocation
after start-up): its workspace is a static array inside the library.  This
file sorts last so that a failure here cannot hide the other tests.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


def _setup(J, side, batch, seed, L=8):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300 import Scattering2D, _lib
    lib = _lib.load()
    dev = torch.device('cuda:0')
    S = Scattering2D(J, (side, side), L=L).to(dev)
    plan = S._get_plan()
    x = torch.from_numpy(np.random.default_rng(seed).random((batch, side, side)).astype(np.float32)).to(dev)
    return lib, _lib, S, plan, x, dev


def _forward_ref(lib, _lib, S, plan, x):
    B = x.shape[0]
    out = torch.empty((B, S._channels) + S._out_hw, device=x.device)
    ws_bytes = lib.kym_s2d_workspace_bytes(plan.h, B)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=x.device)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.kym_s2d_forward(plan.h, x.data_ptr(), out.data_ptr(), B, S._filter_ptrs(), S._n_filters,
                                   ws.data_ptr(), ws_bytes, stream), 'kym_s2d_forward')
    return out


def _forward_noalloc(lib, _lib, S, plan, x):
    B = x.shape[0]
    out = torch.full((B, S._channels) + S._out_hw, float('nan'), device=x.device)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.kym_s2d_forward_noalloc(plan.h, x.data_ptr(), out.data_ptr(), B, S._filter_ptrs(),
                                           S._n_filters, stream), 'kym_s2d_forward_noalloc')
    return out


@pytest.mark.parametrize('J,side,batch', [(3, 256, 9), (2, 32, 40)])
def test_noalloc_matches_forward_twice(J, side, batch):
    lib, _lib, S, plan, x, dev = _setup(J, side, batch, seed=21)
    ref = _forward_ref(lib, _lib, S, plan, x)
    # two calls in a row: the second runs on a scratch array holding the first's contents
    for _ in range(2):
        got = _forward_noalloc(lib, _lib, S, plan, x)
        torch.cuda.synchronize()
        assert torch.isfinite(got).all()
        assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-5
    # a different input through the same array
    x2 = torch.rand_like(x)
    assert rel_l2(_forward_noalloc(lib, _lib, S, plan, x2).cpu().numpy(),
                  _forward_ref(lib, _lib, S, plan, x2).cpu().numpy()) <= 1e-5


def test_noalloc_one_image_per_chunk():
    """320x320, J=3, L=16: one image's input and parent spectra take 19 MB,
    so the 32 MiB scratch holds a single image and the batch of 3 runs as
    three chunks of one, each chunk's input stage reusing the same region."""
    lib, _lib, S, plan, x, dev = _setup(3, 320, 3, seed=23, L=16)
    per_image = lib.kym_s2d_workspace_bytes(plan.h, 1)
    assert (16 << 20) < per_image < (31 << 20), per_image
    ref = _forward_ref(lib, _lib, S, plan, x)
    for _ in range(2):
        got = _forward_noalloc(lib, _lib, S, plan, x)
        torch.cuda.synchronize()
        assert torch.isfinite(got).all()
        assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-5


def test_noalloc_rejects_oversized_geometry():
    """416x416, J=4, L=16 needs more than the static scratch for one image;
    the entry point refuses before launching anything."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300 import _lib
    lib = _lib.load()
    torch.cuda.init()
    h = _lib._vp()
    assert lib.kym_s2d_plan_create(416, 416, 4, 16, 2, 0, ctypes.byref(h)) == 0
    try:
        per_image = lib.kym_s2d_workspace_bytes(h, 1)
        assert per_image > (32 << 20), per_image  # checked on the host before the call
        nf = ctypes.c_int()
        lib.kym_s2d_plan_info(h, None, None, None, None, None, ctypes.byref(nf))
        dummy = _lib.ptr_array([16] * nf.value)  # never dereferenced: the size check comes first
        rc = lib.kym_s2d_forward_noalloc(h, 16, 16, 1, dummy, nf.value, None)
        assert rc == _lib.KYM_ERR_WORKSPACE
        assert b'static scratch' in lib.kym_last_error()
    finally:
        lib.kym_s2d_plan_destroy(h)
