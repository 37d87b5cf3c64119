"""Mixed-size batches (kymatio_gb300.batching): one CUDA graph over size
groups on separate streams gives the same coefficients as per-size modules."""
import numpy as np
import pytest

from conftest import rel_l2

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu


def test_mixed_batch_graph_matches_per_size(tmp_path, monkeypatch):
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    monkeypatch.setenv('KYMATIO_GB300_CACHE', str(tmp_path))
    from kymatio_gb300 import Scattering2D
    from kymatio_gb300.batching import MixedScattering2D, default_J
    dev = torch.device('cuda:0')
    rng = np.random.default_rng(4)
    sides = rng.choice([32, 64, 128, 256], size=24)
    imgs = [torch.from_numpy(rng.random((s, s)).astype(np.float32)).to(dev) for s in sides]
    M = MixedScattering2D([32, 64, 128, 256], graph=True, tune=True).to(dev)
    for rep in range(2):  # capture, then replay with new data
        if rep:
            imgs = [torch.rand_like(im) for im in imgs]
        out = M(imgs)
        torch.cuda.synchronize()
        for im, o in zip(imgs, out):
            s = im.shape[-1]
            ref = Scattering2D(default_J(s), (s, s)).to(dev)(im[None])[0]
            assert o.shape == ref.shape
            assert rel_l2(o.cpu().numpy(), ref.cpu().numpy()) <= 1e-6
    assert (tmp_path / 'autotune.json').exists()


def test_mixed_batch_tensor_cores():
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300.batching import MixedScattering2D, default_J
    from oracle.scattering2d import Scattering2D as Oracle
    dev = torch.device('cuda:0')
    rng = np.random.default_rng(5)
    imgs = [torch.from_numpy(rng.random((s, s)).astype(np.float32)).to(dev) for s in (32, 64, 128, 64)]
    M = MixedScattering2D([32, 64, 128], tensor_cores=True).to(dev)
    out = M(imgs)
    for im, o in zip(imgs, out):
        s = im.shape[-1]
        ref = Oracle(default_J(s), (s, s))(im.cpu().numpy()[None].astype(np.float64))[0]
        assert rel_l2(o.cpu().numpy(), ref) <= 5e-5


def test_mixed_batch_outputs_not_aliased():
    """Results a caller holds survive the next replay of the same graph."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from kymatio_gb300.batching import MixedScattering2D
    dev = torch.device('cuda:0')
    M = MixedScattering2D([32, 64]).to(dev)
    xs = {32: torch.rand(3, 32, 32, device=dev), 64: torch.rand(2, 64, 64, device=dev)}
    first = M.forward_grouped(xs)
    keep = {s: o.clone() for s, o in first.items()}
    M.forward_grouped({s: torch.rand_like(x) for s, x in xs.items()})
    torch.cuda.synchronize()
    for s in xs:
        assert torch.equal(first[s], keep[s])


def test_autotune_picks_a_form_per_group(tmp_path, monkeypatch):
    """In the tensor-core form the autotuner may keep launch groups in their
    plain kernels (more precise); either way the results meet the tensor-core
    bar and the choice is cached."""
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    monkeypatch.setenv('KYMATIO_GB300_CACHE', str(tmp_path))
    import json
    from kymatio_gb300.batching import MixedScattering2D, default_J
    from oracle.scattering2d import Scattering2D as Oracle
    dev = torch.device('cuda:0')
    rng = np.random.default_rng(6)
    xs = {s: torch.from_numpy(rng.random((3, s, s)).astype(np.float32)).to(dev) for s in (32, 128)}
    M = MixedScattering2D(list(xs), tensor_cores=True, tune=True).to(dev)
    out = M.forward_grouped(xs)
    entries = json.load(open(tmp_path / 'autotune.json'))
    assert all('tc_groups' in v for v in entries.values()) and len(entries) == 2
    for s, m in M.mods.items():
        plan = m._get_plan()
        from kymatio_gb300 import _lib
        lib = _lib.load()
        used = [lib.kym_s2d_group_uses_tc(plan.h, g) > 0 for g in range(lib.kym_s2d_group_count(plan.h))]
        mask = entries[[k for k in entries if k.startswith('%sx%s/' % (s, s))][0]]['tc_groups']
        assert all(u <= bool(b) for u, b in zip(used, mask))
    for s, x in xs.items():
        ref = Oracle(default_J(s), (s, s))(x.cpu().numpy().astype(np.float64))
        assert rel_l2(out[s].cpu().numpy(), ref) <= 5e-5
