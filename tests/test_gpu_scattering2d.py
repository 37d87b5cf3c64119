"""GPU parity of the fused 2-D cascade against the reference golden vectors and
the FP64 oracle.  Tolerance: relative L2 <= 1e-5 per scattering order (plain
FP32 path), and the reference test's own allclose on its golden file."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu

TOL = 1e-5


def _cuda():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    return torch.device('cuda:0')


def _orders(J, L, max_order):
    from oracle.scattering2d import order_slices
    return order_slices(J, L, max_order)


def _check_orders(out, ref, J, L, max_order, tol=TOL):
    for k, sl in enumerate(_orders(J, L, max_order)):
        if sl.stop > sl.start:
            e = rel_l2(out[..., sl, :, :], ref[..., sl, :, :])
            assert e <= tol, 'order %d relL2 %.3e' % (k, e)


def test_reference_golden_file():
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    d = np.load(os.path.join(GOLDEN, 'ref_test_data_2d.npz'))
    x = torch.from_numpy(d['x']).to(dev)
    S = torch.from_numpy(d['Sx']).to(dev)
    J = int(d['J'])
    sc = Scattering2D(J, shape=tuple(x.shape[-2:]), pre_pad=bool(d['pre_pad'])).to(dev)
    Sg = sc(x)
    assert Sg.shape == S.shape
    assert torch.allclose(Sg, S, rtol=1e-5, atol=1e-6)
    _check_orders(Sg.cpu().numpy(), d['Sx'], J, 8, 2)
    sc1 = Scattering2D(J, shape=tuple(x.shape[-2:]), max_order=1).to(dev)
    S1 = sc1(x)
    assert torch.allclose(S1, S[..., :S1.shape[-3], :, :], rtol=1e-5, atol=1e-6)


CASES = json.loads(str(np.load(os.path.join(GOLDEN, 'ref_cases_2d.npz'))['meta']))


@pytest.mark.parametrize('case', CASES, ids=lambda c: c['name'])
def test_reference_cases(case):
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    d = np.load(os.path.join(GOLDEN, 'ref_cases_2d.npz'))
    x, ref = d[case['name'] + '/x'], d[case['name'] + '/S']
    sc = Scattering2D(case['J'], tuple(case['shape']), L=case['L'], max_order=case['max_order'],
                      pre_pad=case['pre_pad']).to(dev)
    out = sc(torch.from_numpy(x).to(dev)).cpu().numpy()
    assert out.shape == ref.shape
    _check_orders(out, ref, case['J'], case['L'], case['max_order'])


def test_cfg1_batch128_vs_fp64_oracle():
    """32x32, J=2, L=8, batch 128, U[0,1) from seed 0."""
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    from oracle.scattering2d import Scattering2D as Oracle
    x = np.random.default_rng(0).random((128, 32, 32)).astype(np.float32)
    ref = Oracle(2, (32, 32))(x.astype(np.float64))
    out = Scattering2D(2, (32, 32)).to(dev)(torch.from_numpy(x).to(dev)).cpu().numpy()
    _check_orders(out, ref, 2, 8, 2)


def test_cfg3_shape_vs_fp64_oracle():
    """256x256, J=3, L=8 (the padded size 272 runs as line-split passes)."""
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    from oracle.scattering2d import Scattering2D as Oracle
    x = np.random.default_rng(7).random((2, 256, 256)).astype(np.float32)
    ref = Oracle(3, (256, 256))(x.astype(np.float64))
    out = Scattering2D(3, (256, 256)).to(dev)(torch.from_numpy(x).to(dev)).cpu().numpy()
    _check_orders(out, ref, 3, 8, 2)


def test_line_split_sub_launches():
    """256x256, J=3 with 16 images: the line-split 272x272 passes run in two
    sub-launches (as many images as keep their slots within 64 MiB of L2,
    then the rest).  The last image, in the second sub-launch, matches the
    FP64 oracle in both forms, and the batch equals the same images run one
    at a time."""
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    from oracle.scattering2d import Scattering2D as Oracle
    x = np.random.default_rng(16).random((16, 256, 256)).astype(np.float32)
    ref = Oracle(3, (256, 256))(x[[0, 15]].astype(np.float64))
    S = Scattering2D(3, (256, 256)).to(dev)
    xd = torch.from_numpy(x).to(dev)
    out = S(xd)
    _check_orders(out[[0, 15]].cpu().numpy(), ref, 3, 8, 2)
    S.set_chunk(1)
    assert torch.equal(out, S(xd))
    S.set_chunk(16)
    S.tensor_cores = True
    _check_orders(S(xd)[[0, 15]].cpu().numpy(), ref, 3, 8, 2, tol=5e-5)
    assert S.tensor_core_status() == 0


def test_chunking_is_invisible():
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    x = torch.rand(7, 64, 64, device=dev)
    sc = Scattering2D(3, (64, 64)).to(dev)
    a = sc(x)
    sc.set_chunk(2)
    b = sc(x)
    sc.set_chunk(1)
    c = sc(x)
    assert torch.equal(a, b) and torch.equal(a, c)


def test_batch_shape_agnostic():
    # tests/scattering2d/test_torch_scattering2d.py:91-136
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    S = Scattering2D(3, (32, 32), 8).to(dev)
    with pytest.raises(RuntimeError) as e:
        S(torch.zeros((), device=dev))
    assert 'at least two' in e.value.args[0]
    with pytest.raises(RuntimeError) as e:
        S(torch.zeros((32,), device=dev))
    assert 'at least two' in e.value.args[0]
    Sx = S(torch.zeros((32, 32), device=dev))
    assert Sx.shape == (217, 4, 4)
    for shp in ((1, 32, 32), (2, 32, 32), (2, 2, 32, 32), (2, 2, 2, 32, 32)):
        Sx = S(torch.zeros(shp, device=dev))
        assert Sx.shape == shp[:-2] + (217, 4, 4)
    assert S(torch.zeros((0, 32, 32), device=dev)).shape == (0, 217, 4, 4)


def test_errors():
    # tests/scattering2d/test_torch_scattering2d.py:138-177
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    S = Scattering2D(3, (32, 32)).to(dev)
    with pytest.raises(TypeError) as e:
        S(None)
    assert 'input should be' in e.value.args[0]
    y = torch.randn(4, 4, device=dev)[::2, ::2]
    with pytest.raises(RuntimeError) as e:
        S(y)
    assert 'must be contiguous' in e.value.args[0]
    with pytest.raises(RuntimeError) as e:
        S(torch.randn(31, 31, device=dev))
    assert 'Tensor must be of spatial size' in e.value.args[0]
    Sp = Scattering2D(3, (32, 32), pre_pad=True).to(dev)
    with pytest.raises(RuntimeError) as e:
        Sp(torch.randn(31, 31, device=dev))
    assert 'Padded tensor must be of spatial size' in e.value.args[0]
    with pytest.raises(TypeError) as e:
        S(torch.randn(32, 32))
    assert 'CUDA' in e.value.args[0]
    x = torch.randn(8, 8, device=dev)
    S2 = Scattering2D(2, (8, 8)).to(dev)
    assert S2(x).device == x.device


def test_out_type_list():
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    from oracle.scattering2d import Scattering2D as Oracle
    x = np.random.default_rng(3).random((2, 32, 32)).astype(np.float32)
    ref = Oracle(2, (32, 32), out_type='list')(x.astype(np.float64))
    out = Scattering2D(2, (32, 32), out_type='list').to(dev)(torch.from_numpy(x).to(dev))
    assert len(out) == len(ref)
    for a, b in zip(out, ref):
        assert a['j'] == b['j'] and a['n'] == b['n'] and a['theta'] == b['theta']
        assert a['coef'].shape == b['coef'].shape
        assert rel_l2(a['coef'].cpu().numpy(), b['coef']) <= 1e-5


def test_input_size_agnostic():
    # tests/scattering2d/test_torch_scattering2d.py:179-222 (sizes 31/32/33,
    # J in 1/2/4, J=5 with 32x32 and 37x32 -> 1x1 outputs)
    dev = _cuda()
    from kymatio_gb300 import Scattering2D
    from oracle.scattering2d import Scattering2D as Oracle
    rng = np.random.default_rng(11)
    for N in (31, 32, 33):
        for J in (1, 2, 4):
            x = rng.random((2, N, N)).astype(np.float32)
            out = Scattering2D(J, (N, N)).to(dev)(torch.from_numpy(x).to(dev)).cpu().numpy()
            ref = Oracle(J, (N, N))(x.astype(np.float64))
            _check_orders(out, ref, J, 8, 2)
            sp = Scattering2D(J, (N, N), pre_pad=True).to(dev)
            xp = rng.random((2, sp._M_padded, sp._N_padded)).astype(np.float32)
            out = sp(torch.from_numpy(xp).to(dev)).cpu().numpy()
            ref = Oracle(J, (N, N), pre_pad=True)(xp.astype(np.float64))
            _check_orders(out, ref, J, 8, 2)
    for shape in ((32, 32), (37, 32)):
        x = torch.zeros((3, 3) + shape, device=dev)
        S = Scattering2D(5, shape).to(dev)(x)
        assert S.shape[-2:] == (1, 1)


@pytest.mark.parametrize('J,side', [(2, 32), (3, 64), (3, 256), (4, 128)])
def test_specialised_and_runtime_kernels_agree(J, side):
    """The compile-time specialised variants and the runtime-planned kernel
    compute the same transform (both checked against the FP64 oracle)."""
    dev = _cuda()
    from kymatio_gb300 import Scattering2D, _lib
    from oracle.scattering2d import Scattering2D as Oracle
    lib = _lib.load()
    x = np.random.default_rng(5).random((2, side, side)).astype(np.float32)
    ref = Oracle(J, (side, side))(x.astype(np.float64))
    outs = []
    for spec in (1, 0):
        prev = lib.kym_set_specialized(spec)
        try:
            sc = Scattering2D(J, (side, side)).to(dev)
            outs.append(sc(torch.from_numpy(x).to(dev)).cpu().numpy())
        finally:
            lib.kym_set_specialized(prev)
    for o in outs:
        _check_orders(o, ref, J, 8, 2)
    assert rel_l2(outs[0], outs[1]) < 2e-6
