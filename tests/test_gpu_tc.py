"""tcgen05 split-precision GEMM self-test: bf16 hi/lo operands, FP32
accumulation in tensor memory, against an FP64 product."""
import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('M,N,K', [(128, 32, 144), (100, 16, 68), (77, 64, 256), (128, 48, 40)])
def test_tc_split_gemm(M, N, K):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300 import _lib
    lib = _lib.load()
    dev = torch.device('cuda:0')
    rng = np.random.default_rng(M * 7 + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    a, b = torch.from_numpy(A).to(dev), torch.from_numpy(B).to(dev)
    d = torch.full((M, N), float('nan'), device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    _lib.check(lib.kym_tc_selftest(a.data_ptr(), b.data_ptr(), d.data_ptr(), M, N, K, status.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream), 'kym_tc_selftest')
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    got = d.cpu().numpy()
    assert np.isfinite(got).all()
    # three-product bf16 split keeps ~16 mantissa bits per product
    assert rel_l2(got, ref) < 2e-5, rel_l2(got, ref)


TOL_TC = 5e-5  # split-precision form, relative L2 per order vs the FP64 oracle


@pytest.mark.parametrize('J,side,B', [(3, 256, 2), (2, 32, 16), (4, 128, 4), (3, 64, 4), (4, 256, 1)])
def test_tc_form_vs_fp64_oracle(J, side, B):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300 import Scattering2D, _lib
    from oracle.scattering2d import Scattering2D as Oracle, order_slices
    dev = torch.device('cuda:0')
    x = np.random.default_rng(J * 100 + side).random((B, side, side)).astype(np.float32)
    ref = Oracle(J, (side, side))(x.astype(np.float64))
    S = Scattering2D(J, (side, side), backend='torch_tc').to(dev)
    plan = S._get_plan()
    lib = _lib.load()
    used = [lib.kym_s2d_group_uses_tc(plan.h, g) for g in range(lib.kym_s2d_group_count(plan.h))]
    assert any(u >= 1 for u in used), used
    out = S(torch.from_numpy(x).to(dev)).cpu().numpy()
    assert S.tensor_core_status() == 0
    for k, sl in enumerate(order_slices(J, 8, 2)):
        e = rel_l2(out[:, sl], ref[:, sl])
        assert e <= TOL_TC, 'order %d relL2 %.3e' % (k, e)


def test_dft_gemm_form_256_J3():
    """The 68x68 childless groups of 256x256 J=3 in the DFT-GEMM form (inverse
    DFT and low-pass as split-precision tcgen05 GEMMs): per-order relative L2
    against the FP64 oracle, and against the low-pass-only tensor-core form.
    Three images give 192 tasks per order-2 group, more than one per CTA of
    the persistent grid."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300 import Scattering2D, _lib
    from oracle.scattering2d import Scattering2D as Oracle, order_slices
    lib = _lib.load()
    dev = torch.device('cuda:0')
    x = np.random.default_rng(68).random((3, 256, 256)).astype(np.float32)
    S = Scattering2D(3, (256, 256), backend='torch_tc').to(dev)
    plan = S._get_plan()
    xd = torch.from_numpy(x).to(dev)
    prev = lib.kym_set_tc_dft(1)
    try:
        used = [lib.kym_s2d_group_uses_tc(plan.h, g) for g in range(lib.kym_s2d_group_count(plan.h))]
        assert used.count(2) == 3, used
        out_dft = S(xd).cpu().numpy()
        assert S.tensor_core_status() == 0
        lib.kym_set_tc_dft(0)
        out_lp = S(xd).cpu().numpy()
    finally:
        lib.kym_set_tc_dft(prev)
    ref = Oracle(3, (256, 256))(x.astype(np.float64))
    for k, sl in enumerate(order_slices(3, 8, 2)):
        e = rel_l2(out_dft[:, sl], ref[:, sl])
        assert e <= TOL_TC, 'order %d relL2 %.3e' % (k, e)
        assert rel_l2(out_dft[:, sl], out_lp[:, sl]) <= TOL_TC
