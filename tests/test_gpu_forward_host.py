"""Scattering2D.forward_host / kym_s2d_forward_host: host buffers in and out,
transfers overlapped with the cascade.  Every image's result is the one the
device-tensor forward gives (same kernels, same per-image arithmetic), for
any number of input slices, chunking and either form."""
import numpy as np
import pytest

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def dev():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    return torch.device('cuda:0')


@pytest.mark.parametrize('tc', [False, True])
@pytest.mark.parametrize('parts,chunk', [(1, None), (2, None), (3, 2), (9, 4)])
def test_matches_device_forward(dev, tc, parts, chunk):
    from kymatio_gb300 import Scattering2D
    S = Scattering2D(3, (64, 64)).to(dev)
    S.tensor_cores = tc
    if chunk:
        S.set_chunk(chunk)
    x = torch.from_numpy(np.random.default_rng(parts).random((5, 64, 64)).astype(np.float32))
    ref = S(x.to(dev)).cpu()
    got = S.forward_host(x.pin_memory(), parts=parts)
    assert got.shape == ref.shape and torch.equal(got, ref)
    # pageable buffers, caller-provided output, batch dims kept
    out = torch.full((5, 1) + tuple(ref.shape[1:]), float('nan'))
    S.forward_host(x.reshape(5, 1, 64, 64), out=out, parts=parts)
    assert torch.equal(out[:, 0], ref)
    if tc:
        assert S.tensor_core_status() == 0


def test_headline_size_async_steps(dev):
    """256x256 J=3 (line-split input stage and order-1 group), several steps
    queued without synchronising, each into its own output: the calls
    alternate between the module's two staging buffers, each input copy
    overlapping the previous call's cascade."""
    from kymatio_gb300 import Scattering2D
    S = Scattering2D(3, (256, 256)).to(dev)
    S.tensor_cores = True
    xs = [torch.from_numpy(np.random.default_rng(10 + i).random((3, 256, 256)).astype(np.float32)).pin_memory()
          for i in range(5)]
    outs = [S.forward_host(x, parts=2, sync=False) for x in xs]
    torch.cuda.synchronize()
    for x, o in zip(xs, outs):
        assert torch.equal(o, S(x.to(dev)).cpu())


def test_errors(dev):
    from kymatio_gb300 import Scattering2D
    S = Scattering2D(2, (32, 32)).to(dev)
    with pytest.raises(TypeError):
        S.forward_host(torch.zeros(2, 32, 32, device=dev))
    with pytest.raises(TypeError):
        S.forward_host(torch.zeros(2, 32, 32, dtype=torch.float64))
    with pytest.raises(RuntimeError):
        S.forward_host(torch.zeros(2, 32, 31))
    with pytest.raises(TypeError):
        S.forward_host(torch.zeros(2, 32, 32), out=torch.zeros(2, 3))
    assert S.forward_host(torch.zeros(0, 32, 32)).shape[0] == 0


@pytest.mark.parametrize('J,side,chunk', [(3, 256, None), (4, 128, 3)])
def test_side_lane_identical(dev, J, side, chunk):
    """The side lane (independent group chains on a second stream) changes
    nothing in the results, in either form, with several chunks too."""
    from kymatio_gb300 import Scattering2D, _lib
    lib = _lib.load()
    S = Scattering2D(J, (side, side)).to(dev)
    if chunk:
        S.set_chunk(chunk)
    x = torch.from_numpy(np.random.default_rng(J).random((7, side, side)).astype(np.float32)).to(dev)
    for tc in (False, True):
        S.tensor_cores = tc
        prev = lib.kym_set_side_lane(0)
        try:
            one = S(x)
            lib.kym_set_side_lane(1)
            two = S(x)
            torch.cuda.synchronize()
        finally:
            lib.kym_set_side_lane(prev)
        assert torch.equal(one, two)
