"""The shared-fold line-split form of the childless groups (order 2 and the
last order-1 scale at 256x256, J=3): a rows pass folds each parent and
wavelet row once for the whole group into per-path slots, column passes
finish each path.  Checked per order against the FP64 oracle, against the
fused per-path kernels (kym_set_shared_fold(0)), in the plain and the
tensor-core (separable low-pass) forms, over a batch that needs several
sub-launches."""
import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


def _run(x, form, shared):
    from kymatio_gb300 import Scattering2D, _lib
    lib = _lib.load()
    dev = torch.device('cuda:0')
    prev = lib.kym_set_shared_fold(1 if shared else 0)
    try:
        S = Scattering2D(3, (256, 256), backend='torch_tc' if form == 'tc' else 'torch').to(dev)
        out = S(torch.from_numpy(x).to(dev))
        torch.cuda.synchronize()
        plan = S._get_plan()
        kern = [lib.kym_s2d_group_kernels(plan.h, g, 1 if form == 'tc' else 0)
                for g in range(lib.kym_s2d_group_count(plan.h))]
        if form == 'tc':
            assert S.tensor_core_status() == 0
    finally:
        lib.kym_set_shared_fold(prev)
    return out.cpu().numpy(), kern


@pytest.mark.parametrize('form', ['plain', 'tc'])
def test_shared_fold_256_J3(form):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from oracle.scattering2d import Scattering2D as Oracle, order_slices
    # 13 images: the 136x136 group runs in two sub-launches (7 + 6 images)
    x = np.random.default_rng(31).random((13, 256, 256)).astype(np.float32)
    got, kern = _run(x, form, True)
    fused, kern0 = _run(x, form, False)
    # groups: input, order 1 (j1 = 0, 1, 2), order 2 ((0,1), (0,2), (1,2))
    want = 3 if form == 'tc' else 4
    assert kern[3] == want and kern[4:] == [want] * 3, kern
    assert kern0[4] in (1,), kern0
    pick = [0, 6, 7, 12]
    ref = Oracle(3, (256, 256))(x[pick].astype(np.float64))
    tol = 1e-5 if form == 'plain' else 5e-5
    for k, sl in enumerate(order_slices(3, 8, 2)):
        e = rel_l2(got[pick][:, sl], ref[:, sl])
        assert e <= tol, 'order %d relL2 %.3e' % (k, e)
    assert rel_l2(got, fused) <= (2e-6 if form == 'plain' else 5e-5)
